"""The fused, graph-captured time step against the oracle's loop body
(dynearthsol.cxx:358-394)."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import Case, plastic_config, evp_config, layered_config, rel_l2, diff_fields, COMPARED

_cases = {}


def case(name):
    if name not in _cases:
        cfg = {"c1": W.CONFIGS["1"], "tiny": W.CONFIGS["tiny"], "plastic": plastic_config(),
               "evp": evp_config(), "layered": layered_config()}[name]
        _cases[name] = Case(cfg)
    return _cases[name]


def run_gpu(c, state, nsteps, chunks=1):
    dev = c.device()
    dev.upload(state, abi.F_ALL)
    for _ in range(chunks):
        rep = dev.step(nsteps // chunks)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    return got, rep


@pytest.mark.gpu
def test_config1_2000_steps_bit_identical(gpu):
    """Config 1 (9,600 tets) for the full 2,000 steps: every field equal."""
    c = case("c1")
    s0 = c.initial_state()
    want = s0.copy()
    c.oracle.step(want, 2000)
    got, rep = run_gpu(c, s0, 2000, chunks=4)
    assert rep.status == 0
    assert got.steps == want.steps == 2000 and got.dt == want.dt and got.time == want.time
    bad = diff_fields(got, want)
    assert not bad, {f: rel_l2(getattr(got, f), getattr(want, f)) for f in bad}


# Per-step bar from an identical input state.  Elasto-plastic without
# yielding: every bit equal.  With yielding, CUDA's atan2/sincos in the
# eigen-solver differ from the host libm by an ulp, and the return map
# amplifies that in elements whose trial stress has two close principal
# values; the strict CPU restatement and the reference's own build (3x3-C
# with -ffast-math) differ by up to 3e-11 on the same states, so stress,
# strain and plastic strain are held to 5e-12 there and everything else to
# 1e-12.  EVP uses CUDA's pow/exp for the viscosity: 1e-12.
ONE_STEP_TOL = {"tiny": 0.0, "plastic": 5e-12, "evp": 1e-12, "layered": 1e-12}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny", "plastic", "evp", "layered"])
def test_one_step_from_the_same_state(gpu, name):
    c = case(name)
    tol = ONE_STEP_TOL[name]
    for k in [0, 5, 40]:
        s0 = c.state_after(k)
        want = s0.copy()
        c.oracle.step(want, 1)
        got, rep = run_gpu(c, s0, 1)
        for f in COMPARED:
            t = tol if f in ("stress", "strain", "plstrain", "delta_plstrain", "dpressure") else min(tol, 1e-12)
            assert rel_l2(getattr(got, f), getattr(want, f)) <= t, (k, f, rel_l2(getattr(got, f), getattr(want, f)))
        for f in ["vel", "temperature"]:
            assert rel_l2(getattr(got, f), getattr(want, f)) <= 1e-12
        assert got.dt == want.dt and got.steps == want.steps


# After 200 steps: elasto-plastic bit-identical; EVP accumulates the per-step
# ulp differences of pow/exp in the viscosity (measured 1.2e-9 for velocity
# on the 3-layer box), held to 1e-8.
MULTI_TOL = {"tiny": 0.0, "evp": 1e-8, "layered": 1e-8}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny", "evp", "layered"])
def test_multi_step(gpu, name):
    c = case(name)
    s0 = c.initial_state()
    want = s0.copy()
    c.oracle.step(want, 200)
    got, rep = run_gpu(c, s0, 200, chunks=2)
    for f in ["vel", "stress", "temperature"]:
        assert rel_l2(getattr(got, f), getattr(want, f)) <= MULTI_TOL[name], (f, rel_l2(getattr(got, f), getattr(want, f)))


@pytest.mark.gpu
def test_fused_step_equals_per_function_sequence(gpu):
    """The six fused passes and the per-function kernels give identical bits."""
    c = case("plastic")
    s0 = c.state_after(30)
    a, _ = run_gpu(c, s0, 1)
    dev = c.device()
    dev.upload(s0, abi.F_ALL)
    s = abi.State(c.mesh.nnode, c.mesh.nelem)
    # the loop body through the per-function entry points
    dev.download(s, abi.F_SCALARS)
    s.steps += 1
    s.time += s.dt
    dev.upload(s, abi.F_SCALARS)
    for fn in ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
               "update_stress", "NMD_stress", "update_force", "update_velocity", "apply_vbcs",
               "update_mesh", "rotate_stress"]:
        dev.call(fn)
    b = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    bad = diff_fields(a, b, [f for f in COMPARED if f not in ("ntmp",)])
    assert not bad, bad


@pytest.mark.gpu
def test_step_host_round_trip(gpu):
    """des_gpu_step_host (host buffers in and out) equals upload/step/download."""
    c = case("tiny")
    s0 = c.state_after(3)
    a, _ = run_gpu(c, s0, 2)
    dev = c.device()
    b = s0.copy()
    dev.step_host(b, 2, abi.F_ALL)
    dev.close()
    assert not diff_fields(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_FP32])
@pytest.mark.parametrize("nsteps", [1, 4])
def test_step_host_overlapped_downloads(gpu, precision, nsteps):
    """The fields finished before the last pass download on the second stream
    while that pass runs in element chunks, each chunk's rows downloading
    while the next computes; with one step, the stress pass's element inputs
    also come up chunk by chunk on their own stream while it runs on the
    chunks already landed.  Every field and dt equal upload/step/download,
    with the loop-state mask and page-locked host arrays, and with the output
    averaging switched on (it runs after the last pass)."""
    c = case("plastic")
    s0 = c.state_after(10 - nsteps)     # the last step forms dt (E-A runs in chunks there)
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = precision
    want = []
    for avg in (0, 5):
        # the same upload (and derived geometry) as des_gpu_step_host, then
        # the steps as graphs and a plain download
        dev = D.Device(c.mesh, p, device=0)
        dev.set_averaging(avg)
        dev.step_host(s0.copy(), 0, abi.F_STEP_STATE)
        dev.step(nsteps)
        want.append(dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL))
        dev.close()
    for avg, pinned in ((0, False), (0, True), (5, True)):
        dev = D.Device(c.mesh, p, device=0)
        dev.set_averaging(avg)
        b = s0.copy()
        if pinned:
            D.pin(b)
        rep = dev.step_host(b, nsteps, abi.F_STEP_STATE)
        if pinned:
            D.unpin(b)
        dev.close()
        w = want[1 if avg else 0]
        assert rep.status == 0 and rep.steps == s0.steps + nsteps
        assert not diff_fields(b, w, COMPARED), (avg, pinned)
        assert (b.time, b.dt, b.steps) == (w.time, w.dt, w.steps)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_FP32])
def test_page_locked_host_buffers(gpu, precision):
    """Page-locked host arrays are read and written in place by the layout
    kernels (no staging copy); the results equal the staged path bit for bit."""
    c = case("plastic")
    s0 = c.state_after(3)
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = precision
    out = []
    for pinned in (False, True):
        dev = D.Device(c.mesh, p, device=0)
        b = s0.copy()
        if pinned:
            D.pin(b)
        dev.step_host(b, 3, abi.F_ALL)
        if pinned:
            D.unpin(b)
        dev.close()
        out.append(b)
    assert not diff_fields(out[0], out[1], COMPARED)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_FP32])
def test_nonfinite_coordinates_stop_the_step(gpu, precision):
    """A NaN velocity reaches the coordinates; the step reports it with the
    reference's exit code 11 (output.cxx:195-208) instead of running on."""
    c = case("tiny")
    s = c.state_after(2)
    s.vel[3, 1] = np.nan
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = precision
    dev = D.Device(c.mesh, p, device=0)
    dev.upload(s, abi.F_ALL)
    with pytest.raises(RuntimeError, match="error 11"):
        dev.step(1)
    assert dev.report().status & abi.DES_STATUS_NONFINITE
    dev.close()
