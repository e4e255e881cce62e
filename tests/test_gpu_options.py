"""The option matrix on the GPU: the rheologies, damping options, fixed dt,
dynamic mode, missing thermal diffusion or gravity, velocity boundary types,
material count and mesh size the five workloads leave out (the variants of
tests/helpers.py, each pinned to the reference's own functions on the CPU),
against the oracle."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import (Case, COMPARED, LOOP, OPTION_TRANSCENDENTAL, OPTION_VARIANTS, diff_fields,
                     rel_l2)

pytestmark = pytest.mark.gpu

NAMES = sorted(OPTION_VARIANTS)
_cases = {}


def case(name):
    if name not in _cases:
        _cases[name] = Case(OPTION_VARIANTS[name])
    return _cases[name]


def worst(got, want, fields=COMPARED):
    return max(rel_l2(getattr(got, f), getattr(want, f)) for f in fields)


@pytest.mark.parametrize("name", NAMES)
def test_fused_steps_from_init(name):
    """init() and 50 fused steps: every field bit-identical (pow/exp
    variants: 1e-10, CUDA's viscosity against the host libm's)."""
    c = case(name)
    want = c.initial_state()
    dev = c.device()
    s = W.new_state(c.mesh, c.T, c.pls)
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    got0 = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    rep = dev.step(50)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    assert not diff_fields(got0, want) and got0.dt == want.dt
    c.oracle.step(want, 50)
    assert rep.status == 0 and got.steps == want.steps == 50
    if name in OPTION_TRANSCENDENTAL:
        assert worst(got, want) <= 1e-10, {f: rel_l2(getattr(got, f), getattr(want, f)) for f in COMPARED}
        assert got.dt == pytest.approx(want.dt, rel=1e-12)
    else:
        bad = diff_fields(got, want)
        assert not bad, {f: rel_l2(getattr(got, f), getattr(want, f)) for f in bad}
        assert (got.time, got.dt) == (want.time, want.dt)


@pytest.mark.parametrize("name", NAMES)
def test_every_function_from_a_loop_state(name):
    """Each per-function entry point on the state 7 steps into the run, in
    loop order, against the oracle's function."""
    c = case(name)
    for fn in LOOP:
        if fn == "update_temperature" and not c.params.has_thermal_diffusion:
            continue
        s = c.state_before(fn, 7)
        want = s.copy()
        c.oracle.call(fn, want)
        dev = c.device()
        dev.upload(s, abi.F_ALL)
        dev.call(fn)
        got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
        dev.close()
        fields = [f for f in COMPARED if f != "ntmp"]
        if name in OPTION_TRANSCENDENTAL and fn == "update_stress":
            assert worst(got, want, fields) <= 1e-12, fn
        else:
            bad = diff_fields(got, want, fields)
            assert not bad, (fn, {f: rel_l2(getattr(got, f), getattr(want, f)) for f in bad})


@pytest.mark.parametrize("name", NAMES)
def test_fp32_form_one_step(name):
    """The FP32 form, one step from the same state 10 steps into the run:
    stress and force within 1e-5 of the FP64 oracle, temperature within
    1e-12 (velocity: 1e-3, it is a difference of near-balanced forces)."""
    c = case(name)
    s0 = c.state_after(10)
    want = s0.copy()
    c.oracle.step(want, 1)
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = abi.PREC_FP32
    dev = D.Device(c.mesh, p, device=0)
    dev.upload(s0, abi.F_ALL)
    rep = dev.step(1)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    errs = {f: rel_l2(getattr(got, f), getattr(want, f)) for f in ["vel", "force", "stress", "temperature"]}
    assert rep.status == 0
    assert errs["stress"] <= 1e-5 and errs["force"] <= 1e-5, errs
    assert errs["vel"] <= 1e-3 and errs["temperature"] <= 1e-12, errs
