"""des_compute_dt_noalloc against the handle's des_gpu_compute_dt and the oracle.

The no-alloc entry point serves callers that cannot let a library call
cudaMalloc: they own all device memory (their own pool or budget), or must
not trigger the device-wide synchronisation cudaMalloc/cudaFree can cause.
It takes device arrays the caller already holds and keeps its scratch in a
fixed array inside the library.  Cases: the quasi-static thermal path on the
default stream; the dynamic dt_elastic branch (bulkm(0)/rho(0)) without
thermal diffusion, with a per-element shear modulus, on a side stream; a
37,500-block grid (config 2); dt <= 0 reported in the status word.  Every
case makes two calls in a row.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import Case, phase_config

MAX_ELEMS = 256 * 65536


def matv(mv, m):
    """Material m's value of a property vector: a vector of one value holds
    for every material (matprops.cxx:509-520)."""
    return mv.v[m] if mv.len > 1 else mv.v[0]


def harmonic(mv, em):
    """MatProps harmonic_mean over each element's marker counts
    (matprops.cxx:450-461); a one-value vector is that value."""
    if mv.len == 1:
        return np.full(em.shape[0], mv.v[0])
    r = np.zeros(em.shape[0])
    for m in range(em.shape[1]):
        r += em[:, m].astype(np.float64) / mv.v[m]
    return em.sum(axis=1).astype(np.float64) / r


def rho_of(p, mesh, T, e):
    """MatProps::rho(e) (matprops.cxx:707-728) in the reference's order."""
    t = 0.0
    for i in range(4):
        t += T[mesh.connectivity[e, i]]
    t /= 4
    tc = t - 273.0
    r, n = 0.0, 0
    for m in range(mesh.nmat):
        r += matv(p.rho0, m) * (1 - matv(p.alpha, m) * tc) * int(mesh.elemmarkers[e, m])
        n += int(mesh.elemmarkers[e, m])
    return r / n


def dt_inputs(p, mesh, state):
    return abi.DtInputs(visc_min=p.visc_min, therm_diff_max=p.therm_diff_max,
                        max_vbc_val=p.max_vbc_val, inertial_scaling=p.inertial_scaling,
                        dt_fraction=p.dt_fraction, fixed_dt=p.fixed_dt,
                        shear_modulus=p.shear_modulus.v[0],
                        bulkm0=float(harmonic(p.bulk_modulus, mesh.elemmarkers[:1])[0]),
                        rho0=rho_of(p, mesh, state.temperature, 0),
                        is_quasi_static=p.is_quasi_static,
                        has_thermal_diffusion=p.has_thermal_diffusion)


def noalloc(L, torch, mesh, state, inp, shearm=None, stream=None):
    """One call through the C ABI on device copies of the state's arrays;
    returns (rc, dt, status)."""
    conn = torch.from_numpy(mesh.connectivity).cuda()
    coord = torch.from_numpy(state.coord).cuda()
    vol = torch.from_numpy(state.volume).cuda()
    sh = torch.from_numpy(shearm).cuda() if shearm is not None else None
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    st = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.des_compute_dt_noalloc(mesh.nelem, coord.data_ptr(), conn.data_ptr(), vol.data_ptr(),
                                  sh.data_ptr() if sh is not None else None, C.byref(inp),
                                  out.data_ptr(), st.data_ptr(),
                                  stream.cuda_stream if stream is not None else None)
    torch.cuda.synchronize()
    return rc, float(out.item()), int(st.item())


def handle_dt(c, s):
    dev = c.device()
    dev.upload(s, abi.F_ALL)
    want = dev.call("compute_dt")      # the existing entry point (des_gpu_compute_dt)
    dev.close()
    return want


@pytest.mark.gpu
def test_noalloc_dt_equals_handle_dt_on_two_calls_in_a_row(gpu):
    """Quasi-static, thermal diffusion, one material (shearm NULL), default stream."""
    torch = pytest.importorskip("torch")
    L = D.lib()
    c = Case(W.CONFIGS["1"])
    for nsteps in (3, 17):          # two consecutive calls on different states
        s = c.state_after(nsteps)
        want = handle_dt(c, s)
        rc, got, status = noalloc(L, torch, c.mesh, s, dt_inputs(c.params, c.mesh, s))
        assert rc == abi.DES_OK and status == abi.DES_OK
        assert got == want, (nsteps, got, want)
        assert got == c.oracle.call("compute_dt", s.copy())


@pytest.mark.gpu
@pytest.mark.parametrize("visc_min", [1e7, 1e20], ids=["dt_maxwell_wins", "dt_elastic_wins"])
def test_noalloc_dynamic_no_diffusion_per_element_shearm_side_stream(gpu, visc_min):
    """The dynamic dt_elastic branch (0.5 minl / sqrt(bulkm(0)/rho(0))), no
    thermal diffusion, and a per-element shear modulus from three materials
    (harmonic means over the marker counts), on a side stream.  With
    visc_min 1e7 the per-element dt_maxwell sets dt (and a NULL shearm would
    give another dt); with 1e20 the dynamic dt_elastic does."""
    torch = pytest.importorskip("torch")
    L = D.lib()
    cfg = phase_config()
    cfg.extra = dict(cfg.extra, params=dict(is_quasi_static=0, has_thermal_diffusion=0,
                                            visc_min=visc_min))
    c = Case(cfg)
    p = c.params
    shearm = harmonic(p.shear_modulus, c.mesh.elemmarkers)
    assert len(np.unique(shearm)) > 1
    side = torch.cuda.Stream()
    for nsteps in (2, 9):
        s = c.state_after(nsteps)
        want = handle_dt(c, s)
        inp = dt_inputs(p, c.mesh, s)
        rc, got, status = noalloc(L, torch, c.mesh, s, inp, shearm, side)
        assert rc == abi.DES_OK and status == abi.DES_OK
        assert got == want, (nsteps, got, want)
        assert got == c.oracle.call("compute_dt", s.copy())
        if visc_min < 1e10:
            _, uniform, _ = noalloc(L, torch, c.mesh, s, inp, None, side)
            assert uniform != got


@pytest.mark.gpu
def test_noalloc_large_grid_config2(gpu):
    """Config 2 (9.6M tets): 37,500 blocks of partial minima in the fixed
    array, on the initial state and after 12 device steps."""
    torch = pytest.importorskip("torch")
    L = D.lib()
    c = Case(W.CONFIGS["2"])
    dev = c.device()
    s = W.new_state(c.mesh, c.T, c.pls)
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    for nsteps in (0, 12):
        if nsteps:
            dev.step(nsteps)
        st = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
        want = dev.call("compute_dt")
        rc, got, status = noalloc(L, torch, c.mesh, st, dt_inputs(c.params, c.mesh, st))
        assert rc == abi.DES_OK and status == abi.DES_OK
        assert got == want, (nsteps, got, want)
    dev.close()
    assert got == c.oracle.call("compute_dt", st.copy())


@pytest.mark.gpu
def test_noalloc_status_reports_dt_not_positive(gpu):
    """dt <= 0 (compute_dt's exit 11) comes back as DES_ERR_DT in the status
    word, and the next call with good inputs clears it; a fixed dt is
    returned unchecked with DES_OK."""
    torch = pytest.importorskip("torch")
    L = D.lib()
    c = Case(W.CONFIGS["1"])
    s = c.state_after(1)
    inp = dt_inputs(c.params, c.mesh, s)
    inp.dt_fraction = 0.0
    rc, got, status = noalloc(L, torch, c.mesh, s, inp)
    assert rc == abi.DES_OK and got == 0.0 and status == abi.DES_ERR_DT
    inp = dt_inputs(c.params, c.mesh, s)
    rc, got, status = noalloc(L, torch, c.mesh, s, inp)
    assert rc == abi.DES_OK and status == abi.DES_OK and got == c.oracle.call("compute_dt", s.copy())
    inp.fixed_dt = 1.5e7
    rc, got, status = noalloc(L, torch, c.mesh, s, inp)
    assert rc == abi.DES_OK and status == abi.DES_OK and got == 1.5e7


@pytest.mark.gpu
def test_noalloc_rejects_sizes_above_its_limit(gpu):
    L = D.lib()
    inp = abi.DtInputs(max_vbc_val=1.0, dt_fraction=1.0, shear_modulus=1.0, visc_min=1.0,
                       therm_diff_max=1.0, inertial_scaling=1.0, is_quasi_static=1)
    dummy = C.c_double()
    big = (C.c_int * 4)()
    rc = L.des_compute_dt_noalloc(MAX_ELEMS + 1, C.addressof(dummy), C.addressof(big),
                                  C.addressof(dummy), None, C.byref(inp), C.addressof(dummy), None,
                                  None)
    assert rc == abi.DES_ERR_SIZE
