"""The oracle's numpy restatement of the seeded workloads (oracle/workload_np.py,
which the CPU arm of the benchmark builds its case with) gives the same mesh,
markers, temperatures, plastic strain and parameters, boundary normals
included, as the product's generator (csrc/workload.cpp)."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import workload as W
from helpers import OPTION_VARIANTS
from oracle import workload_np as WN

CASES = {
    "tiny": W.CONFIGS["tiny"],
    "config1": W.CONFIGS["1"],
    "config2_shape_32x28x8": W.scaled(W.CONFIGS["2"], 32, 28, 8),
    "config3_noise_12x10x6": W.scaled(W.CONFIGS["3"], 12, 10, 6),
    "config5_layers_14x12x10": W.scaled(W.CONFIGS["5"], 14, 12, 10),
    "inclined": OPTION_VARIANTS["inclined_1"],
}


@pytest.mark.parametrize("name", list(CASES))
def test_numpy_workload_equals_product_generator(name):
    cfg = CASES[name]
    mesh, p, T, pls, topo = D.setup_case(cfg)
    m2, p2, T2, pls2, o = WN.setup_case(cfg)
    for f in ("coord", "connectivity", "segment", "segflag", "elemmarkers"):
        a, b = getattr(mesh, f), getattr(m2, f)
        assert a.shape == b.shape and a.dtype == b.dtype, f
        assert np.array_equal(a, b), f
    assert np.array_equal(T, T2) and np.array_equal(pls, pls2)
    assert bytes(p) == bytes(p2)            # boundary normals and edge vectors included
    assert np.array_equal(o.bcflag(), topo.bcflag)


def test_counter_prng_known_values():
    """splitmix64 (Steele, Lea & Flood 2014): the finaliser applied to the
    golden-gamma sequence from state 0 gives the published first outputs."""
    gamma = 0x9E3779B97F4A7C15
    out = [int(WN._mix64(np.array((gamma * k) % 2**64, np.uint64))) for k in range(3)]
    assert out == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
