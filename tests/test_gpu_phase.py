"""Material bookkeeping on the device: marker counts changed between steps
(phase_changes, phasechanges.cxx:232-258, every 10 steps before compute_dt,
dynearthsol.cxx:382-393) through des_gpu_set_elemmarkers, against the oracle
given the same counts."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import Case, phase_config, phase_change, diff_fields, rel_l2

pytestmark = pytest.mark.gpu


def case():
    return Case(phase_config())


def fresh_device(c, params=None):
    dev = D.Device(c.mesh, params or c.params, device=0)
    s = W.new_state(c.mesh, c.T, c.pls)
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    return dev


def test_phase_changes_every_10_steps_bit_identical():
    c = case()
    want = c.initial_state()
    dev = fresh_device(c)
    em = c.mesh.elemmarkers.copy()
    nmix = [len(np.unique(em, axis=0))]
    for _ in range(3):
        c.oracle.step(want, 10)
        dev.step(10)
        em2 = phase_change(c.mesh, want, em)
        assert (em2 != em).any()
        em = em2
        nmix.append(len(np.unique(em, axis=0)))
        c.oracle.set_elemmarkers(em)
        want.dt = c.oracle.call("compute_dt", want)
        dev.set_elemmarkers(em)
        assert dev.call("compute_dt") == want.dt
    assert max(nmix) > nmix[0]          # new mixes appeared
    c.oracle.step(want, 25)
    rep = dev.step(25)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    assert rep.status == 0
    assert not diff_fields(got, want)
    assert (got.time, got.dt, got.steps) == (want.time, want.dt, want.steps)


def test_rejected_counts_leave_the_device_unchanged():
    c = case()
    want = c.initial_state()
    dev = fresh_device(c)
    em = c.mesh.elemmarkers.copy()
    empty = em.copy()
    empty[5] = 0                                   # an element without markers
    negative = em.copy()
    negative[7] = [5, -1, 0]
    many = em.copy()
    many[:, 0] = np.arange(c.mesh.nelem) % 300 + 1  # 300 distinct count vectors
    for bad, code in ((empty, abi.DES_ERR_TOPOLOGY), (negative, abi.DES_ERR_TOPOLOGY),
                      (many, abi.DES_ERR_SIZE)):
        with pytest.raises(RuntimeError, match=f"error {code}"):
            dev.set_elemmarkers(bad)
    with pytest.raises(ValueError):
        dev.set_elemmarkers(em[:, :2])
    c.oracle.step(want, 20)
    dev.step(20)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    assert not diff_fields(got, want)


def test_fp32_form_one_step_after_a_phase_change():
    """The FP32 form's terms prepared for the next step (conductivity,
    reference density in the FP64 force part) follow the new counts."""
    c = case()
    s0 = c.state_after(10)
    em = phase_change(c.mesh, s0, c.mesh.elemmarkers)
    c.oracle.set_elemmarkers(em)
    want = s0.copy()
    want.dt = c.oracle.call("compute_dt", want)
    c.oracle.step(want, 1)
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = abi.PREC_FP32
    errs = {}
    for label, markers in (("set", em), ("stale", None)):
        dev = D.Device(c.mesh, p, device=0)
        dev.upload(s0, abi.F_ALL)
        if markers is not None:
            dev.set_elemmarkers(markers)
        dt = dev.call("compute_dt")
        dev.step(1)
        got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
        dev.close()
        errs[label] = {f: rel_l2(getattr(got, f), getattr(want, f))
                       for f in ["vel", "force", "stress", "temperature"]}
        if markers is not None:
            assert dt == pytest.approx(want.dt, rel=1e-14)
    # bars of the layered FP32 one-step test; the stale tables miss them
    assert errs["set"]["force"] <= 1e-5 and errs["set"]["stress"] <= 1e-5, errs
    assert errs["set"]["vel"] <= 1e-3 and errs["set"]["temperature"] <= 1e-12, errs
    assert errs["stale"]["force"] > 10 * errs["set"]["force"], errs


def test_closure_keeps_its_material():
    """A closure was trained on one mix: counts that change it are refused,
    the same counts are accepted."""
    from des_gb300 import closure
    c = Case(W.CONFIGS["tiny"])
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = abi.PREC_FP32
    dev = D.Device(c.mesh, p, device=0)
    net = closure.new_net(3, tol=1e-3)
    dev.set_closure(net)
    em = c.mesh.elemmarkers.copy()
    dev.set_elemmarkers(em)
    em[0, 0] += 1
    with pytest.raises(RuntimeError, match=f"error {abi.DES_ERR_UNSUPPORTED}"):
        dev.set_elemmarkers(em)
    dev.set_closure(None)
    dev.set_elemmarkers(em)
    dev.close()
