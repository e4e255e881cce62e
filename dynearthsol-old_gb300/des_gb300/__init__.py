"""Python host side of the GB300 DynEarthSol3D time-step library.

The product is the C-ABI library libdes_gb300.so (include/des_gpu.h); this
package loads it with ctypes and offers the reference's loop functions with
their names (update_stress, update_force, ...) on a device-resident state.
There is no CPU path: every compute call goes to the CUDA library, and loading
fails loudly when the library is missing.
"""
import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi
from .abi import State, check
from .build import LIB, build

_lib = None

FUNCTIONS = ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
             "update_stress", "NMD_stress", "update_force", "update_velocity", "apply_vbcs",
             "update_coordinate", "compute_volume", "compute_mass", "compute_shape_fn",
             "update_mesh", "rotate_stress"]


def lib():
    """Load libdes_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        raise RuntimeError(f"{LIB} is missing: run des_gb300.build.build() first")
    L = C.CDLL(str(LIB))
    P = C.POINTER
    L.des_box_sizes.argtypes = [P(abi.BoxSpec), P(C.c_int), P(C.c_int), P(C.c_int)]
    L.des_box_fill.argtypes = [P(abi.BoxSpec), P(C.c_double), P(C.c_int), P(C.c_int), P(C.c_int)]
    L.des_markers_layered.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_int), C.c_int,
                                      C.c_double, C.c_int, P(C.c_int), P(C.c_double),
                                      C.c_ulonglong, P(C.c_int)]
    L.des_temperature_linear.argtypes = [C.c_int, P(C.c_double), C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_ulonglong, P(C.c_double)]
    L.des_topology_build.argtypes = [P(abi.MeshView), P(P(abi.Topology))]
    L.des_topology_free.argtypes = [P(abi.Topology)]
    L.des_topology_free.restype = None
    L.des_boundary_normals.argtypes = [P(abi.Topology), P(C.c_int), P(C.c_double), P(abi.Params)]
    L.des_gpu_create.argtypes = [P(abi.MeshView), P(abi.Params), C.c_int, P(C.c_void_p)]
    L.des_gpu_destroy.argtypes = [C.c_void_p]
    L.des_gpu_set_params.argtypes = [C.c_void_p, P(abi.Params)]
    L.des_gpu_set_elemmarkers.argtypes = [C.c_void_p, P(C.c_int)]
    L.des_gpu_remesh.argtypes = [C.c_void_p, P(abi.MeshView), P(abi.StateView), C.c_int]
    L.des_gpu_upload.argtypes = [C.c_void_p, P(abi.StateView), C.c_uint]
    L.des_gpu_download.argtypes = [C.c_void_p, P(abi.StateView), C.c_uint]
    L.des_gpu_init_fields.argtypes = [C.c_void_p]
    L.des_gpu_step.argtypes = [C.c_void_p, C.c_int, P(abi.StepReport)]
    L.des_gpu_step_host.argtypes = [C.c_void_p, P(abi.StateView), C.c_uint, C.c_int,
                                    P(abi.StepReport)]
    L.des_gpu_report.argtypes = [C.c_void_p, P(abi.StepReport)]
    for f in FUNCTIONS:
        getattr(L, "des_gpu_" + f).argtypes = [C.c_void_p]
    L.des_gpu_compute_dt.argtypes = [C.c_void_p, P(C.c_double)]
    L.des_gpu_download_support.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int)]
    L.des_gpu_error_string.argtypes = [C.c_int]
    L.des_gpu_error_string.restype = C.c_char_p
    L.des_gpu_device_bytes.argtypes = [C.c_void_p]
    L.des_gpu_device_bytes.restype = C.c_longlong
    L.des_gpu_kernels_per_step.argtypes = [C.c_void_p]
    L.des_gpu_softf64_check.argtypes = [C.c_int, C.c_longlong, C.c_ulonglong, P(C.c_ulonglong)]
    L.des_gpu_time_steps.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
    L.des_gpu_profile_steps.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
    L.des_host_register.argtypes = [C.c_void_p, C.c_longlong]
    L.des_host_unregister.argtypes = [C.c_void_p]
    L.des_abi_sizes.argtypes = [P(C.c_longlong)]
    L.des_abi_sizes.restype = None
    L.des_compute_dt_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         P(abi.DtInputs), C.c_void_p, C.c_void_p, C.c_void_p]
    fp = P(C.c_float)
    L.des_mlp_forward.argtypes = [P(abi.Mlp), fp, C.c_longlong, fp]
    L.des_mlp_loss_grad.argtypes = [P(abi.Mlp), fp, fp, C.c_longlong, P(C.c_double), P(abi.Mlp)]
    L.des_mlp_train.argtypes = [P(abi.Mlp), fp, fp, C.c_longlong, C.c_int, C.c_int, C.c_float,
                                C.c_ulonglong, fp]
    L.des_gpu_log_returns.argtypes = [C.c_void_p, C.c_int, fp, C.c_longlong, P(C.c_longlong)]
    L.des_gpu_set_closure.argtypes = [C.c_void_p, P(abi.Mlp)]
    L.des_gpu_bad_mesh_quality.argtypes = [C.c_void_p, P(abi.RemeshCheck), P(C.c_int), P(C.c_int),
                                           P(C.c_double)]
    L.des_gpu_elem_quality.argtypes = [C.c_void_p, P(C.c_double)]
    L.des_write_save.argtypes = [C.c_char_p, P(abi.MeshView), P(abi.Params), P(C.c_uint),
                                 P(abi.StateView), P(abi.SaveAverages), P(abi.MarkerSet), C.c_int]
    L.des_write_checkpoint.argtypes = [C.c_char_p, P(abi.MeshView), C.c_double, C.c_double, P(C.c_double),
                                       P(abi.MarkerSet), C.c_int]
    L.des_gpu_set_averaging.argtypes = [C.c_void_p, C.c_int]
    L.des_gpu_output_snapshot.argtypes = [C.c_void_p, C.c_uint]
    L.des_gpu_output_fetch.argtypes = [C.c_void_p, P(abi.StateView)]
    L.des_gpu_output_wait.argtypes = [C.c_void_p, P(abi.StateView)]
    L.des_gpu_download_averages.argtypes = [C.c_void_p] + [P(C.c_double)] * 5
    _lib = L
    return L


def _ck(rc, what):
    if rc != abi.DES_OK:
        msg = lib().des_gpu_error_string(rc).decode()
        raise RuntimeError(f"{what}: error {rc} ({msg})")


class Topology:
    """bcflag, support lists, bnodes, bfacets as built by the library."""

    def __init__(self, mesh):
        import numpy as np
        L = lib()
        ptr = C.POINTER(abi.Topology)()
        mv = mesh.view()
        _ck(L.des_topology_build(C.byref(mv), C.byref(ptr)), "des_topology_build")
        t = ptr.contents
        N, E = mesh.nnode, mesh.nelem
        self.bcflag = np.ctypeslib.as_array(t.bcflag, (N,)).copy()
        self.support_offsets = np.ctypeslib.as_array(t.support_offsets, (N + 1,)).copy()
        self.support_elems = np.ctypeslib.as_array(t.support_elems, (4 * E,)).copy()
        self.support_slots = np.ctypeslib.as_array(t.support_slots, (4 * E,)).copy()
        self.bnodes = [np.ctypeslib.as_array(t.bnodes[b], (t.bnodes_count[b],)).copy()
                       if t.bnodes_count[b] else np.zeros(0, np.int32) for b in range(abi.DES_NBDRY)]
        self.bfacets = [np.ctypeslib.as_array(t.bfacets[b], (t.bfacets_count[b], 2)).copy()
                        if t.bfacets_count[b] else np.zeros((0, 2), np.int32)
                        for b in range(abi.DES_NBDRY)]
        self._ptr = ptr

    def boundary_normals(self, mesh, coord, params):
        _ck(lib().des_boundary_normals(self._ptr, abi.iptr(mesh.connectivity), abi.dptr(coord),
                                       C.byref(params)), "des_boundary_normals")

    def __del__(self):
        try:
            lib().des_topology_free(self._ptr)
        except Exception:
            pass


class Device:
    """A device-resident DynEarthSol3D state on one GPU."""

    def __init__(self, mesh, params, device=0):
        self.L = lib()
        self.mesh, self.params = mesh, params
        self.h = C.c_void_p()
        self._mv = mesh.view()
        _ck(self.L.des_gpu_create(C.byref(self._mv), C.byref(params), device, C.byref(self.h)),
            "des_gpu_create")

    def close(self):
        if self.h:
            self.L.des_gpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self.params = params
        _ck(self.L.des_gpu_set_params(self.h, C.byref(params)), "des_gpu_set_params")

    def set_elemmarkers(self, elemmarkers):
        """New marker counts [nelem][nmat] for the same mesh (after a phase change)."""
        em = np.ascontiguousarray(elemmarkers, dtype=np.int32)
        if em.shape != (self.mesh.nelem, self.mesh.nmat):
            raise ValueError(f"elemmarkers has shape {em.shape}")
        _ck(self.L.des_gpu_set_elemmarkers(self.h, abi.iptr(em)), "des_gpu_set_elemmarkers")

    def remesh(self, mesh, state, reset_bottom_coord0=False):
        """The device half of remesh: `mesh` is the new mesh (with the
        remapped marker counts), `state` its interpolated fields."""
        mv = mesh.view()
        v = state.view()
        _ck(self.L.des_gpu_remesh(self.h, C.byref(mv), C.byref(v), int(bool(reset_bottom_coord0))),
            "des_gpu_remesh")
        self.mesh, self._mv = mesh, mv

    def upload(self, state, mask=abi.F_ALL):
        v = state.view()
        _ck(self.L.des_gpu_upload(self.h, C.byref(v), mask), "des_gpu_upload")

    def download(self, state, mask=abi.F_ALL):
        v = state.view()
        _ck(self.L.des_gpu_download(self.h, C.byref(v), mask), "des_gpu_download")
        state.sync_scalars(v)
        return state

    def init_fields(self):
        _ck(self.L.des_gpu_init_fields(self.h), "des_gpu_init_fields")

    def step(self, nsteps=1, report=True):
        r = abi.StepReport()
        _ck(self.L.des_gpu_step(self.h, nsteps, C.byref(r) if report else None), "des_gpu_step")
        return r

    def step_host(self, state, nsteps=1, mask=abi.F_STEP_STATE):
        r = abi.StepReport()
        v = state.view()
        _ck(self.L.des_gpu_step_host(self.h, C.byref(v), mask, nsteps, C.byref(r)),
            "des_gpu_step_host")
        state.sync_scalars(v)
        return r

    def report(self):
        r = abi.StepReport()
        _ck(self.L.des_gpu_report(self.h, C.byref(r)), "des_gpu_report")
        return r

    def call(self, name):
        if name == "compute_dt":
            dt = C.c_double()
            _ck(self.L.des_gpu_compute_dt(self.h, C.byref(dt)), "des_gpu_compute_dt")
            return dt.value
        _ck(getattr(self.L, "des_gpu_" + name)(self.h), "des_gpu_" + name)

    def time_steps(self, nsteps):
        ms = C.c_double()
        _ck(self.L.des_gpu_time_steps(self.h, nsteps, C.byref(ms)), "des_gpu_time_steps")
        return ms.value

    def profile_steps(self, nsteps):
        ms = (C.c_double * 6)()
        _ck(self.L.des_gpu_profile_steps(self.h, nsteps, ms), "des_gpu_profile_steps")
        return list(ms)

    def log_returns(self, nsteps, capacity):
        """Runs nsteps FP64 steps and returns the shear-return records
        (float32 [n][24]) and how many returns there were in total."""
        rec = np.zeros((capacity, abi.RET_RECORD), np.float32)
        n = C.c_longlong()
        _ck(lib().des_gpu_log_returns(self.h, nsteps, rec.ctypes.data_as(C.POINTER(C.c_float)),
                                      capacity, C.byref(n)), "des_gpu_log_returns")
        return rec[:min(n.value, capacity)], n.value

    def support(self):
        """The device's support lists: (offsets, elements, slots) as des_topology holds them."""
        N, E = self.mesh.nnode, self.mesh.nelem
        off = np.zeros(N + 1, np.int32)
        el = np.zeros(4 * E, np.int32)
        sl = np.zeros(4 * E, np.int32)
        _ck(self.L.des_gpu_download_support(self.h, abi.iptr(off), abi.iptr(el), abi.iptr(sl)),
            "des_gpu_download_support")
        return off, el, sl

    def bad_mesh_quality(self, check):
        """(code, index, cube root of the worst quality) of bad_mesh_quality."""
        code, index, q = C.c_int(), C.c_int(-1), C.c_double()
        _ck(self.L.des_gpu_bad_mesh_quality(self.h, C.byref(check), C.byref(code), C.byref(index),
                                            C.byref(q)), "des_gpu_bad_mesh_quality")
        return code.value, index.value, q.value

    def elem_quality(self):
        q = np.zeros(self.mesh.nelem)
        _ck(self.L.des_gpu_elem_quality(self.h, abi.dptr(q)), "des_gpu_elem_quality")
        return q

    OUTPUT_FIELDS = (abi.F_COORD | abi.F_VEL | abi.F_FORCE | abi.F_TEMPERATURE | abi.F_VOLUME |
                     abi.F_STRESS | abi.F_STRAIN | abi.F_STRAIN_RATE | abi.F_PLSTRAIN | abi.F_COORD0)

    def output_snapshot(self, mask=None):
        """Copy the output fields on the device (step stream)."""
        _ck(self.L.des_gpu_output_snapshot(self.h, self.OUTPUT_FIELDS if mask is None else mask),
            "des_gpu_output_snapshot")

    def output_fetch(self, state):
        """Start the snapshot's copy into state's arrays (page-locked for
        overlap); the arrays must stay alive until output_wait."""
        self._fetch_view = state.view()
        _ck(self.L.des_gpu_output_fetch(self.h, C.byref(self._fetch_view)), "des_gpu_output_fetch")

    def output_wait(self, state):
        v = self._fetch_view
        _ck(self.L.des_gpu_output_wait(self.h, C.byref(v)), "des_gpu_output_wait")
        state.sync_scalars(v)
        return state

    def set_averaging(self, interval):
        """Output::average_fields after every step (0 stops it)."""
        _ck(self.L.des_gpu_set_averaging(self.h, interval), "des_gpu_set_averaging")

    def download_averages(self, interval):
        """The device's averaging state as an abi.SaveAverages (with the
        numpy arrays it points into kept alive on the object)."""
        N, E = self.mesh.nnode, self.mesh.nelem
        arr = dict(coord0=np.zeros((N, 3)), strain0=np.zeros((E, 6)), stress_sum=np.zeros((E, 6)),
                   dpls_sum=np.zeros(E))
        t0 = C.c_double()
        _ck(self.L.des_gpu_download_averages(self.h, *(abi.dptr(arr[k]) for k in
                                                      ("coord0", "strain0", "stress_sum", "dpls_sum")),
                                             C.byref(t0)), "des_gpu_download_averages")
        return save_averages(arr["coord0"], arr["strain0"], arr["stress_sum"], arr["dpls_sum"],
                             t0.value, interval)

    def set_closure(self, net):
        """Installs an abi.Mlp as the learned closure (None removes it)."""
        _ck(lib().des_gpu_set_closure(self.h, C.byref(net) if net is not None else None),
            "des_gpu_set_closure")

    @property
    def kernels_per_step(self):
        return self.L.des_gpu_kernels_per_step(self.h)

    @property
    def device_bytes(self):
        return self.L.des_gpu_device_bytes(self.h)


def save_averages(coord0, strain0, stress_sum, dpls_sum, time0, interval):
    """An abi.SaveAverages over numpy arrays (kept alive on it)."""
    a = abi.SaveAverages()
    a._keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (coord0, strain0, stress_sum, dpls_sum)]
    a.coord0, a.strain0, a.stress_sum, a.dpls_sum = (abi.dptr(x) for x in a._keep)
    a.time0 = time0
    a.interval = interval
    return a


def marker_sets(sets):
    """A ctypes array of des_marker_set from (name, eta [n][4], elem, mattype,
    id, last_id) tuples; the numpy arrays it points into ride along on it."""
    if not sets:
        return None, 0
    arr = (abi.MarkerSet * len(sets))()
    keep = []
    for k, (name, eta, elem, mattype, ids, last_id) in enumerate(sets):
        eta = np.ascontiguousarray(eta, dtype=np.float64).reshape(-1, 4)
        cols = [np.ascontiguousarray(a, dtype=np.int32) for a in (elem, mattype, ids)]
        if any(c.ndim != 1 or c.size != len(eta) for c in cols):
            raise ValueError(f"marker set {name}: eta, elem, mattype and id differ in length")
        keep += [eta] + cols
        arr[k] = abi.MarkerSet(str(name).encode(), len(eta), int(last_id), abi.dptr(eta), abi.iptr(cols[0]),
                               abi.iptr(cols[1]), abi.iptr(cols[2]))
    arr._keep = keep
    return arr, len(sets)


def write_save(path, mesh, params, bcflag, state, averages=None, markers=None):
    """The .save file of one output frame (des_write_save); markers: marker
    sets as (name, eta, elem, mattype, id, last_id), written as with
    sim.has_marker_output on."""
    v = state.view()
    mv = mesh.view()
    b = np.ascontiguousarray(bcflag, dtype=np.uint32)
    sets, n = marker_sets(markers)
    _ck(lib().des_write_save(str(path).encode(), C.byref(mv), C.byref(params), abi.uptr(b), C.byref(v),
                             C.byref(averages) if averages is not None else None, sets, n),
        "des_write_save")


def write_checkpoint(path, mesh, state, compensation_pressure, markers=None):
    """The .chkpt file of a frame (des_write_checkpoint), with its marker sets."""
    mv = mesh.view()
    sets, n = marker_sets(markers)
    _ck(lib().des_write_checkpoint(str(path).encode(), C.byref(mv), state.time, compensation_pressure,
                                   abi.dptr(state.volume_old), sets, n), "des_write_checkpoint")


def softf64_check(n, seed=20261203, device=0):
    """Mismatches of the integer-pipe FP64 arithmetic against the device's
    FP64 unit over n seeded operands per kind: [multiply, any bits; multiply,
    near 1; conversion to FP32, any bits; conversion, FP32 range; 0 + x;
    2 x; x / 2; x / 6; x / 3; x / 4]."""
    out = (C.c_ulonglong * 10)()
    _ck(lib().des_gpu_softf64_check(device, n, seed, out), "des_gpu_softf64_check")
    return list(out)


def pin(state):
    """Page-lock every array of a host State (for asynchronous copies)."""
    L = lib()
    for n in State.ARRAYS:
        a = getattr(state, n)
        _ck(L.des_host_register(a.ctypes.data, a.nbytes), "des_host_register")


def unpin(state):
    L = lib()
    for n in State.ARRAYS:
        L.des_host_unregister(getattr(state, n).ctypes.data)


def setup_case(cfg, params=None):
    """Mesh, params (with boundary normals), initial T and plastic strain."""
    from . import workload as W
    L = lib()
    mesh = W.Mesh(cfg, L)
    T, pls = W.initial_inputs(cfg, mesh, L)
    p = params if params is not None else W.make_params(cfg)
    topo = Topology(mesh)
    topo.boundary_normals(mesh, mesh.coord, p)
    return mesh, p, T, pls, topo
