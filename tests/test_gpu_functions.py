"""Each per-function entry point of the CUDA library against the oracle's
function on the same loop-consistent input state.

Bit-exact for every function whose arithmetic has no transcendental call.
update_stress on yielding elements goes through CUDA's atan2/sin/cos in the
eigen-solver (and sin/tan where the friction angle weakens); there the bar is
relative L2 <= 1e-12 per call for stress, strain and plastic strain."""
import numpy as np
import pytest

from des_gb300 import abi
from helpers import Case, plastic_config, evp_config, layered_config, rel_l2, diff_fields
from des_gb300 import workload as W

FUNCS = ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
         "update_stress", "NMD_stress", "update_force", "update_velocity", "apply_vbcs",
         "update_coordinate", "compute_volume", "compute_mass", "compute_shape_fn",
         "rotate_stress"]

_cases = {}


def case(name):
    if name not in _cases:
        cfg = {"c1": W.CONFIGS["1"], "plastic": plastic_config(), "evp": evp_config(),
               "layered": layered_config()}[name]
        _cases[name] = Case(cfg)
    return _cases[name]


STEPS = {"c1": 7, "plastic": 60, "evp": 12, "layered": 12}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "plastic", "evp", "layered"])
@pytest.mark.parametrize("fn", FUNCS)
def test_function_matches_oracle(gpu, name, fn):
    c = case(name)
    s0 = c.state_before(fn, STEPS[name])
    want = s0.copy()
    c.oracle.call(fn, want)
    dev = c.device()
    dev.upload(s0, abi.F_ALL)
    dev.call(fn)
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    bad = diff_fields(got, want)
    if fn == "update_stress" and name != "c1":
        # eigen-solver / pow / exp: CUDA's libm vs the host's
        for f in ["stress", "strain", "strain_rate", "plstrain", "delta_plstrain", "dpressure"]:
            assert rel_l2(getattr(got, f), getattr(want, f)) <= 1e-12, (f, rel_l2(getattr(got, f), getattr(want, f)))
        bad = [f for f in bad if f not in ("stress", "plstrain", "delta_plstrain", "dpressure")]
    assert not bad, {f: float(np.abs(getattr(got, f) - getattr(want, f)).max()) for f in bad}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "plastic", "evp"])
def test_compute_dt_matches_oracle(gpu, name):
    c = case(name)
    s0 = c.state_after(STEPS[name])
    dt_want = c.oracle.call("compute_dt", s0.copy())
    dev = c.device()
    dev.upload(s0, abi.F_ALL)
    dt_got = dev.call("compute_dt")
    dev.close()
    assert dt_got == dt_want


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "plastic", "evp", "layered"])
def test_init_fields_matches_oracle(gpu, name):
    c = case(name)
    want = c.initial_state()
    dev = c.device()
    s = W.new_state(c.mesh, c.T, c.pls)
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    got = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    assert not diff_fields(got, want, ["coord", "vel", "temperature", "mass", "tmass",
                                       "volume_n", "volume", "volume_old", "stress", "strain",
                                       "plstrain", "shpdx", "shpdy", "shpdz"])
    assert got.dt == want.dt and got.steps == 0 and got.time == 0
