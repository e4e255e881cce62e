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
