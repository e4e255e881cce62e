"""The CUDA path against the golden fixtures written by the reference's own
functions: bit-identical where no eigen-solve or transcendental is involved."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from des_gb300 import abi, workload as W
from helpers import Case, plastic_config, evp_config, rel_l2
from test_golden import FIELDS, load, assert_state

G = Path(__file__).resolve().parent / "golden"


def gpu_from_init(c):
    dev = c.device()
    s = W.new_state(c.mesh, c.T, c.pls)
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    return dev


@pytest.mark.gpu
def test_gpu_tiny_box_matches_reference_bit_for_bit(gpu):
    z = np.load(G / "tiny_states.npz")
    c = Case(W.CONFIGS["tiny"])
    dev = gpu_from_init(c)
    s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    assert_state(s, z, "init")
    done = 0
    for n in (1, 10, 50):
        dev.step(n - done)
        done = n
        s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
        assert_state(s, z, f"step{n}")
    dev.close()


@pytest.mark.gpu
def test_gpu_config1_2000_steps_hashes_equal_reference(gpu):
    want = json.loads((G / "config1_hashes.json").read_text())
    c = Case(W.CONFIGS["1"])
    dev = gpu_from_init(c)
    for key, n in (("init", 0), ("step100", 100), ("step2000", 1900)):
        if n:
            dev.step(n)
        s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
        for f in FIELDS:
            h = hashlib.sha256(np.ascontiguousarray(getattr(s, f)).tobytes()).hexdigest()
            assert h == want[key][f], (key, f)
        assert [s.time, s.dt, s.steps] == want[key]["scalars"]
    dev.close()


@pytest.mark.gpu
def test_gpu_evp_box_20_steps(gpu):
    z = np.load(G / "evp_states.npz")
    c = Case(evp_config())
    dev = gpu_from_init(c)
    dev.step(20)
    s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    for f in FIELDS:
        assert rel_l2(getattr(s, f), z[f"step20/{f}"]) <= 1e-10, f


@pytest.mark.gpu
def test_gpu_yielding_step_from_reference_state(gpu):
    z = np.load(G / "plastic_states.npz")
    c = Case(plastic_config())
    s0 = load(abi.State(c.mesh.nnode, c.mesh.nelem), z, "step30")
    dev = c.device()
    dev.upload(s0, abi.F_ALL)
    dev.step(1)
    s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    dev.close()
    for f in FIELDS:
        assert rel_l2(getattr(s, f), z[f"step31/{f}"]) <= 1e-10, f
