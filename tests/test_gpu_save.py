"""Output::average_fields on the device and the .save file written from the
device state, against the oracle pipeline (byte for byte on config 1, where
the device loop is bit-identical to the oracle's)."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import Case, rel_l2
from oracle.oracle import Averages

pytestmark = pytest.mark.gpu


def test_device_averages_and_save_file(gpu, tmp_path):
    c = Case(W.CONFIGS["1"])
    interval, nsteps = 10, 34
    s0 = c.initial_state()
    dev = c.device()
    dev.upload(s0, abi.F_ALL)
    dev.set_averaging(interval)
    dev.step(nsteps)
    s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    a = dev.download_averages(interval)
    dev.close()
    avg = Averages(interval)
    so = s0.copy()
    for _ in range(nsteps):
        c.oracle.step(so, 1)
        avg.update(so)
    got = {k: np.ctypeslib.as_array(getattr(a, k), shape=avg_shape)
           for k, avg_shape in (("coord0", avg.coord0.shape), ("strain0", avg.strain0.shape),
                                ("stress_sum", avg.stress_sum.shape), ("dpls_sum", avg.dpls_sum.shape))}
    assert np.array_equal(got["coord0"], avg.coord0) and np.array_equal(got["strain0"], avg.strain0)
    assert np.array_equal(got["stress_sum"], avg.stress_sum) and np.array_equal(got["dpls_sum"], avg.dpls_sum)
    assert a.time0 == avg.time0
    D.write_save(tmp_path / "gpu.save", c.mesh, c.params, c.oracle.bcflag(), s, a)
    D.write_save(tmp_path / "oracle.save", c.mesh, c.params, c.oracle.bcflag(), so,
                 D.save_averages(avg.coord0, avg.strain0, avg.stress_sum, avg.dpls_sum, avg.time0, interval))
    assert (tmp_path / "gpu.save").read_bytes() == (tmp_path / "oracle.save").read_bytes()


def test_fp32_form_averages(gpu):
    c = Case(W.CONFIGS["1"])
    interval, nsteps = 10, 25
    s0 = c.initial_state()
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = abi.PREC_FP32
    dev = D.Device(c.mesh, p, device=0)
    dev.upload(s0, abi.F_ALL)
    dev.set_averaging(interval)
    dev.step(nsteps)
    a = dev.download_averages(interval)
    dev.close()
    avg = Averages(interval)
    so = s0.copy()
    for _ in range(nsteps):
        c.oracle.step(so, 1)
        avg.update(so)
    ss = np.ctypeslib.as_array(a.stress_sum, shape=avg.stress_sum.shape)
    assert rel_l2(ss, avg.stress_sum) < 1e-5
    assert a.time0 == avg.time0


@pytest.mark.parametrize("pinned", [False, True])
def test_output_snapshot_overlaps_the_steps(gpu, pinned):
    """A snapshot after 5 steps, fetched while 5 more steps run, holds the
    state after 5 steps; the stepping is not disturbed."""
    c = Case(W.CONFIGS["1"])
    s0 = c.initial_state()
    dev = c.device()
    dev.upload(s0, abi.F_ALL)
    dev.step(5)
    host = abi.State(c.mesh.nnode, c.mesh.nelem)
    if pinned:
        D.pin(host)
    dev.output_snapshot()
    dev.output_fetch(host)
    dev.step(5)
    dev.output_wait(host)
    after10 = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    if pinned:
        D.unpin(host)
    dev.close()
    want5 = s0.copy()
    c.oracle.step(want5, 5)
    want10 = want5.copy()
    c.oracle.step(want10, 5)
    for f in ("coord", "vel", "force", "temperature", "volume", "volume_old", "stress", "strain",
              "strain_rate", "plstrain", "delta_plstrain", "coord0"):
        assert np.array_equal(getattr(host, f), getattr(want5, f)), f
        if f != "coord0":
            assert np.array_equal(getattr(after10, f), getattr(want10, f)), f
    assert (host.steps, host.time, host.dt) == (want5.steps, want5.time, want5.dt)
