"""Config 2 at its full size (200x200x40 hexes x 6 = 9.6M tets): the fused
FP64 step from init() is bit-identical to the oracle's loop, every field."""
import pytest

from des_gb300 import abi, workload as W
from helpers import Case, diff_fields, COMPARED

pytestmark = pytest.mark.gpu


def test_config2_fused_steps_bit_identical(gpu):
    c = Case(W.CONFIGS["2"])
    s = c.initial_state()
    dev = c.device()
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    dev.step(3)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    c.oracle.step(s, 3)
    assert not diff_fields(got, s, [f for f in COMPARED if f != "ntmp"])
    assert (got.steps, got.time, got.dt) == (s.steps, s.time, s.dt)


def test_config2_fp32_2000_steps_within_1e4_of_fp64():
    """The FP32 form against the FP64 form on config 2 at full size for 2,000
    steps, with the smooth damping (option 2) under which the loop is not
    chaotic: velocity and stress within 1e-4 (measured: 4e-6 and 4e-8)."""
    import numpy as np
    import des_gb300 as D
    from helpers import rel_l2
    base = W.CONFIGS["2"]
    d = dict(base.__dict__)
    d["extra"] = dict(base.extra, params=dict(base.extra.get("params", {}), damping_option=2))
    c = Case(W.Config(**d))
    got = {}
    for prec in (abi.PREC_FP64, abi.PREC_FP32):
        p = abi.Params.from_buffer_copy(c.params)
        p.precision = prec
        dev = D.Device(c.mesh, p, device=0)
        s = W.new_state(c.mesh, c.T, c.pls)
        dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
        dev.init_fields()
        rep = dev.step(2000)
        got[prec] = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
        dev.close()
        assert rep.status == 0
    a, b = got[abi.PREC_FP32], got[abi.PREC_FP64]
    errs = {f: rel_l2(getattr(a, f), getattr(b, f)) for f in ("vel", "stress", "temperature")}
    assert errs["vel"] <= 1e-4 and errs["stress"] <= 1e-4 and errs["temperature"] <= 1e-8, errs
