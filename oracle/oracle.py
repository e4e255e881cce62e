"""TEST INFRASTRUCTURE -- ctypes wrappers of the two CPU checkers.

  PortOracle  oracle/des_oracle.cpp, a restatement of the reference hot path
              (built here and on any host by build_oracle())
  RefOracle   the reference's own functions, compiled from its sources by
              oracle/ref.mk into oracle/_ref/libdesref.so (only where the
              reference tree is present)

Both offer the same calls on an abi.State; only tests/, __graft_entry__.smoke()
and bench.py's CPU baseline use them.
"""
import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ORACLE = Path(__file__).resolve().parent
ROOT = ORACLE.parent
sys.path.insert(0, str(ROOT / "dynearthsol-old_gb300"))
from des_gb300 import abi  # noqa: E402

PORT_LIB = ORACLE / "_build" / "libdes_oracle.so"
REF_LIB = ORACLE / "_ref" / "libdesref.so"
# the reference checkout the CPU checkers read (DES_REFERENCE overrides the
# build container's location; where neither exists the checks that need it skip)
REF_SRC = Path(os.environ.get("DES_REFERENCE", "/root/reference"))

FUNCTIONS = ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
             "update_stress", "NMD_stress", "update_force", "update_velocity", "apply_vbcs",
             "update_coordinate", "compute_volume", "compute_mass", "compute_shape_fn",
             "update_mesh", "rotate_stress"]


def build_oracle(force=False):
    (ORACLE / "_build").mkdir(exist_ok=True)
    srcs = [ORACLE / "des_oracle.cpp", ORACLE / "des_oracle_eig.cpp"]
    deps = srcs + [ORACLE / "des_oracle.h", ROOT / "include" / "des_gpu.h"]
    if force or not PORT_LIB.exists() or any(d.stat().st_mtime > PORT_LIB.stat().st_mtime
                                             for d in deps):
        cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-o", str(PORT_LIB)] + [str(x) for x in srcs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("oracle build failed\n" + r.stderr)
    return PORT_LIB


def build_ref(jobs=8):
    """Compile the reference's sources (only where the reference tree exists)."""
    if not (REF_SRC / "rheology.cxx").exists():
        return None
    cmd = ["make", "-s", "-f", str(ORACLE / "ref.mk"), f"REF={REF_SRC}", f"-j{jobs}"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(ROOT))
    if r.returncode:
        raise RuntimeError("reference build failed\n" + r.stderr[-4000:])
    return REF_LIB


class _Base:
    def __init__(self, mesh, params):
        self.mesh, self.params = mesh, params


class PortOracle(_Base):
    _L = None

    @classmethod
    def lib(cls):
        if cls._L is None:
            build_oracle()
            L = C.CDLL(str(PORT_LIB))
            P = C.POINTER
            L.dso_create.argtypes = [P(abi.MeshView), P(abi.Params), P(C.c_void_p)]
            L.dso_destroy.argtypes = [C.c_void_p]
            L.dso_destroy.restype = None
            L.dso_set_params.argtypes = [C.c_void_p, P(abi.Params)]
            L.dso_set_elemmarkers.argtypes = [C.c_void_p, P(C.c_int)]
            L.dso_init_fields.argtypes = [C.c_void_p, P(abi.StateView)]
            L.dso_step.argtypes = [C.c_void_p, P(abi.StateView), C.c_int]
            L.dso_compute_dt.argtypes = [C.c_void_p, P(abi.StateView), P(C.c_double)]
            L.dso_elem_quality.argtypes = [C.c_void_p, P(abi.StateView), P(C.c_double)]
            L.dso_elem_quality.restype = None
            L.dso_bad_mesh_quality.argtypes = [C.c_void_p, P(abi.StateView), P(abi.RemeshCheck),
                                               P(C.c_int), P(C.c_int), P(C.c_double)]
            L.dso_bad_mesh_quality.restype = None
            for f in FUNCTIONS:
                getattr(L, "dso_" + f).argtypes = [C.c_void_p, P(abi.StateView)]
            L.dso_bcflag.argtypes = [C.c_void_p, P(C.c_uint)]
            L.dso_support.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int)]
            L.dso_bnodes.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int)]
            L.dso_bfacets.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int)]
            L.dso_boundary_normals.argtypes = [C.c_void_p, P(C.c_double), P(abi.Params)]
            L.dso_dsyevh3.argtypes = [P(C.c_double)] * 3
            L.dso_principal_stresses3.argtypes = [P(C.c_double)] * 3
            L.dso_principal_stresses3.restype = None
            L.dso_elasto_plastic.argtypes = [C.c_double] * 7 + [P(C.c_double), P(C.c_double),
                                                                P(C.c_double), P(C.c_int)]
            L.dso_elasto_plastic.restype = None
            cls._L = L
        return cls._L

    def __init__(self, mesh, params):
        super().__init__(mesh, params)
        self.L = self.lib()
        self.h = C.c_void_p()
        self._mv = mesh.view()
        rc = self.L.dso_create(C.byref(self._mv), C.byref(params), C.byref(self.h))
        if rc:
            raise RuntimeError(f"dso_create failed {rc}")

    def __del__(self):
        if getattr(self, "h", None):
            self.L.dso_destroy(self.h)

    def set_params(self, params):
        self.params = params
        self.L.dso_set_params(self.h, C.byref(params))

    def set_elemmarkers(self, elemmarkers):
        self._em = np.ascontiguousarray(elemmarkers, dtype=np.int32)
        rc = self.L.dso_set_elemmarkers(self.h, abi.iptr(self._em))
        if rc:
            raise RuntimeError(f"dso_set_elemmarkers failed {rc}")

    def boundary_normals(self, coord, params):
        rc = self.L.dso_boundary_normals(self.h, abi.dptr(coord), C.byref(params))
        if rc:
            raise RuntimeError(f"boundary normals failed {rc}")

    def init_fields(self, state):
        v = state.view()
        rc = self.L.dso_init_fields(self.h, C.byref(v))
        state.sync_scalars(v)
        if rc:
            raise RuntimeError(f"dso_init_fields failed {rc}")

    def call(self, name, state):
        v = state.view()
        if name == "compute_dt":
            dt = C.c_double()
            rc = self.L.dso_compute_dt(self.h, C.byref(v), C.byref(dt))
            if rc:
                raise RuntimeError(f"compute_dt failed {rc}")
            return dt.value
        rc = getattr(self.L, "dso_" + name)(self.h, C.byref(v))
        state.sync_scalars(v)
        if rc:
            raise RuntimeError(f"dso_{name} failed {rc}")

    def step(self, state, n=1):
        v = state.view()
        rc = self.L.dso_step(self.h, C.byref(v), n)
        state.sync_scalars(v)
        if rc:
            raise RuntimeError(f"dso_step failed {rc}")

    def elem_quality(self, state):
        """elem_quality of every element (geometry.cxx:472-509)."""
        v = state.view()
        q = np.zeros(state.volume.shape[0])
        self.L.dso_elem_quality(self.h, C.byref(v), abi.dptr(q))
        return q

    def bad_mesh_quality(self, state, check):
        """(code, index, cube root of the worst quality) of remeshing.cxx:1893-1960."""
        v = state.view()
        code, index, q = C.c_int(), C.c_int(-1), C.c_double()
        self.L.dso_bad_mesh_quality(self.h, C.byref(v), C.byref(check), C.byref(code), C.byref(index),
                                    C.byref(q))
        return code.value, index.value, q.value

    def bcflag(self):
        a = np.zeros(self.mesh.nnode, np.uint32)
        self.L.dso_bcflag(self.h, abi.uptr(a))
        return a

    def support(self):
        off = np.zeros(self.mesh.nnode + 1, np.int32)
        el = np.zeros(4 * self.mesh.nelem, np.int32)
        self.L.dso_support(self.h, abi.iptr(off), abi.iptr(el))
        return off, el

    def bnodes(self, b):
        n = C.c_int()
        self.L.dso_bnodes(self.h, b, C.byref(n), None)
        a = np.zeros(n.value, np.int32)
        self.L.dso_bnodes(self.h, b, C.byref(n), abi.iptr(a))
        return a

    def bfacets(self, b):
        n = C.c_int()
        self.L.dso_bfacets(self.h, b, C.byref(n), None)
        a = np.zeros((n.value, 2), np.int32)
        self.L.dso_bfacets(self.h, b, C.byref(n), abi.iptr(a))
        return a


class RefOracle(_Base):
    """The reference's own functions (oracle/_ref/libdesref.so)."""
    _L = None

    @classmethod
    def available(cls):
        return REF_LIB.exists()

    @classmethod
    def lib(cls):
        if cls._L is None:
            if not REF_LIB.exists():
                raise RuntimeError("oracle/_ref/libdesref.so is not built")
            L = C.CDLL(str(REF_LIB))
            P = C.POINTER
            L.dsr_create.argtypes = [P(abi.MeshView), P(abi.Params), P(C.c_void_p)]
            L.dsr_set_state.argtypes = [C.c_void_p, P(abi.StateView), C.c_uint]
            L.dsr_get_state.argtypes = [C.c_void_p, P(abi.StateView), C.c_uint]
            L.dsr_init_fields.argtypes = [C.c_void_p, P(abi.StateView)]
            L.dsr_step.argtypes = [C.c_void_p, C.c_int]
            L.dsr_compute_dt.argtypes = [C.c_void_p]
            L.dsr_compute_dt.restype = C.c_double
            L.dsr_set_elemmarkers.argtypes = [C.c_void_p, P(C.c_int)]
            L.dsr_inherit.argtypes = [C.c_void_p, C.c_void_p]
            L.dsr_max_vbc_val.argtypes = [C.c_void_p]
            L.dsr_max_vbc_val.restype = C.c_double
            L.dsr_compensation_pressure.argtypes = [C.c_void_p]
            L.dsr_compensation_pressure.restype = C.c_double
            for f in FUNCTIONS:
                getattr(L, "dsr_" + f).argtypes = [C.c_void_p]
            L.dsr_bcflag.argtypes = [C.c_void_p, P(C.c_uint)]
            L.dsr_support.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int)]
            L.dsr_bnodes.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int)]
            L.dsr_bfacets.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int)]
            L.dsr_normals.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
            L.dsr_dsyevh3.argtypes = [P(C.c_double)] * 3
            L.dsr_output_begin.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int]
            L.dsr_output_write.argtypes = [C.c_void_p, C.c_int]
            L.dsr_output_checkpoint.argtypes = [C.c_void_p]
            L.dsr_add_markers.argtypes = [C.c_void_p, C.c_char_p, C.c_int, P(C.c_double), P(C.c_int),
                                          P(C.c_int), C.c_int]
            L.dsr_elem_quality.argtypes = [C.c_void_p, P(C.c_double)]
            L.dsr_worst_elem_quality.argtypes = [C.c_void_p, P(C.c_int)]
            L.dsr_worst_elem_quality.restype = C.c_double
            cls._L = L
        return cls._L

    def __init__(self, mesh, params):
        super().__init__(mesh, params)
        self.L = self.lib()
        self.h = C.c_void_p()
        self._mv = mesh.view()
        rc = self.L.dsr_create(C.byref(self._mv), C.byref(params), C.byref(self.h))
        if rc:
            raise RuntimeError(f"dsr_create failed {rc}")

    def init_fields(self, state):
        v = state.view()
        self.L.dsr_init_fields(self.h, C.byref(v))
        state.sync_scalars(v)

    def set_elemmarkers(self, elemmarkers):
        em = np.ascontiguousarray(elemmarkers, dtype=np.int32)
        self.L.dsr_set_elemmarkers(self.h, abi.iptr(em))

    def inherit(self, other):
        """Boundary normals, edge vectors and compensation pressure of `other`
        (what remesh keeps across a new mesh)."""
        self.L.dsr_inherit(self.h, other.h)

    def _in(self, state):
        v = state.view()
        self.L.dsr_set_state(self.h, C.byref(v), abi.F_ALL)

    def _out(self, state):
        v = state.view()
        self.L.dsr_get_state(self.h, C.byref(v), abi.F_ALL)
        state.sync_scalars(v)

    def call(self, name, state):
        self._in(state)
        if name == "compute_dt":
            return self.L.dsr_compute_dt(self.h)
        getattr(self.L, "dsr_" + name)(self.h)
        self._out(state)

    def step(self, state, n=1):
        self._in(state)
        self.L.dsr_step(self.h, n)
        self._out(state)

    def bcflag(self):
        a = np.zeros(self.mesh.nnode, np.uint32)
        self.L.dsr_bcflag(self.h, abi.uptr(a))
        return a

    def support(self):
        off = np.zeros(self.mesh.nnode + 1, np.int32)
        el = np.zeros(4 * self.mesh.nelem, np.int32)
        self.L.dsr_support(self.h, abi.iptr(off), abi.iptr(el))
        return off, el

    def bnodes(self, b):
        n = C.c_int()
        self.L.dsr_bnodes(self.h, b, C.byref(n), None)
        a = np.zeros(n.value, np.int32)
        self.L.dsr_bnodes(self.h, b, C.byref(n), abi.iptr(a))
        return a

    def bfacets(self, b):
        n = C.c_int()
        self.L.dsr_bfacets(self.h, b, C.byref(n), None)
        a = np.zeros((n.value, 2), np.int32)
        self.L.dsr_bfacets(self.h, b, C.byref(n), abi.iptr(a))
        return a

    def add_markers(self, name, eta, elem, mattype, marker_output=True):
        """A marker set in var.markersets from the reference's own
        MarkerSet::append_marker (ids 0..n-1); with marker_output the next
        output_begin writes marker sets into .save files."""
        self._mk = [np.ascontiguousarray(eta, np.float64).reshape(-1, 4),
                    np.ascontiguousarray(elem, np.int32), np.ascontiguousarray(mattype, np.int32)]
        self.L.dsr_add_markers(self.h, str(name).encode(), len(self._mk[1]), abi.dptr(self._mk[0]),
                               abi.iptr(self._mk[1]), abi.iptr(self._mk[2]), int(marker_output))

    def output_begin(self, modelname, frame=0, averaged=False, interval=1):
        """The reference's Output for `modelname` (averaging in every later
        step when averaged)."""
        self.L.dsr_output_begin(self.h, str(modelname).encode(), frame, int(averaged), interval)

    def output_write(self, state, exact=False):
        """Output::write (write_exact) of `state`: <modelname>.save.<frame>."""
        self._in(state)
        rc = self.L.dsr_output_write(self.h, int(exact))
        if rc:
            raise RuntimeError("output not set up")

    def output_checkpoint(self, state):
        """Output::write_checkpoint of `state`: <modelname>.chkpt.<frame>."""
        self._in(state)
        if self.L.dsr_output_checkpoint(self.h):
            raise RuntimeError("output not set up")

    def compensation_pressure(self):
        return self.L.dsr_compensation_pressure(self.h)

    def elem_quality(self, state):
        """The reference's elem_quality of every element, and its
        worst_elem_quality (value, index)."""
        self._in(state)
        q = np.zeros(state.volume.shape[0])
        self.L.dsr_elem_quality(self.h, abi.dptr(q))
        w = C.c_int()
        qw = self.L.dsr_worst_elem_quality(self.h, C.byref(w))
        return q, qw, w.value

    def normals(self):
        bn = np.zeros((10, 3))
        ev = np.zeros((10, 10, 3))
        self.L.dsr_normals(self.h, abi.dptr(bn), abi.dptr(ev))
        return bn, ev


def dsyevh3(a, which="port"):
    """Eigen-decomposition of a 3x3 symmetric matrix (upper part of a)."""
    a = np.ascontiguousarray(a, np.float64).reshape(9)
    q = np.zeros(9)
    w = np.zeros(3)
    L = PortOracle.lib() if which == "port" else RefOracle.lib()
    fn = L.dso_dsyevh3 if which == "port" else L.dsr_dsyevh3
    rc = fn(abi.dptr(a), abi.dptr(q), abi.dptr(w))
    return rc, q.reshape(3, 3), w


class Averages:
    """Output::average_fields (output.cxx:227-267) restated over AoS states:
    call update(state) after every step."""

    def __init__(self, interval):
        self.interval = interval
        self.coord0 = self.strain0 = self.stress_sum = self.dpls_sum = None
        self.time0 = 0.0

    def update(self, s):
        if s.steps % self.interval == 1:
            self.time0 = s.time
            self.coord0 = s.coord.copy()
            self.strain0 = s.strain.copy()
            self.stress_sum = s.stress.copy()
            self.dpls_sum = s.delta_plstrain.copy()
        else:
            self.stress_sum += s.stress
            self.dpls_sum += s.delta_plstrain
