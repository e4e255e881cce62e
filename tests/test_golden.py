"""The CPU oracle against golden fixtures written by the reference's own
functions (tests/golden/make_golden.py).  These pin the oracle wherever it runs,
including hosts without the reference tree."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from des_gb300 import abi, workload as W
from helpers import Case, plastic_config, evp_config, rel_l2
from oracle.oracle import dsyevh3

G = Path(__file__).resolve().parent / "golden"
FIELDS = ["coord", "vel", "force", "temperature", "mass", "tmass", "volume_n", "ntmp", "volume",
          "volume_old", "edvoldt", "plstrain", "delta_plstrain", "dpressure", "stress", "strain",
          "strain_rate", "shpdx", "shpdy", "shpdz"]


def load(state, z, prefix):
    for f in FIELDS:
        getattr(state, f)[...] = z[f"{prefix}/{f}"]
    state.time, state.dt, state.steps = z[f"{prefix}/scalars"]
    state.steps = int(state.steps)
    return state


def assert_state(s, z, prefix, tol=0.0):
    for f in FIELDS:
        want = z[f"{prefix}/{f}"]
        got = getattr(s, f)
        if tol == 0.0:
            assert np.array_equal(got, want), (prefix, f, float(np.abs(got - want).max()))
        else:
            assert rel_l2(got, want) <= tol, (prefix, f, rel_l2(got, want))
    assert (s.time, s.dt, s.steps) == tuple(z[f"{prefix}/scalars"])


def test_tiny_box_init_and_steps_bit_exact():
    z = np.load(G / "tiny_states.npz")
    c = Case(W.CONFIGS["tiny"])
    s = c.initial_state()
    assert_state(s, z, "init")
    done = 0
    for n in (1, 10, 50):
        c.oracle.step(s, n - done)
        done = n
        assert_state(s, z, f"step{n}")


def test_evp_box_bit_exact():
    z = np.load(G / "evp_states.npz")
    c = Case(evp_config())
    s = c.initial_state()
    assert_state(s, z, "init")
    c.oracle.step(s, 20)
    assert_state(s, z, "step20")


def test_yielding_box_one_step_from_reference_state():
    """The reference's 3x3-C is built with -ffast-math; the strict restatement
    matches it to 1e-10 relative on a yielding state (per step)."""
    z = np.load(G / "plastic_states.npz")
    c = Case(plastic_config())
    s = load(abi.State(c.mesh.nnode, c.mesh.nelem), z, "step30")
    c.oracle.step(s, 1)
    for f in FIELDS:
        assert rel_l2(getattr(s, f), z[f"step31/{f}"]) <= 1e-10, f
    s = load(abi.State(c.mesh.nnode, c.mesh.nelem), z, "before_stress")
    c.oracle.call("update_stress", s)
    assert rel_l2(s.stress, z["after_stress/stress"]) <= 1e-10
    assert rel_l2(s.plstrain, z["after_stress/plstrain"]) <= 1e-10
    assert np.array_equal(s.strain, z["after_stress/strain"])
    assert np.array_equal(s.strain_rate, z["after_stress/strain_rate"])
    # the same elements yield
    assert np.array_equal(s.delta_plstrain > 0, z["after_stress/delta_plstrain"] > 0)


def test_config1_hashes_after_2000_steps():
    """Config 1 (9,600 tets): SHA-256 of every field equals the reference's
    after init, 100 and 2,000 steps."""
    want = json.loads((G / "config1_hashes.json").read_text())
    c = Case(W.CONFIGS["1"])
    s = c.initial_state()
    for key, n in (("init", 0), ("step100", 100), ("step2000", 1900)):
        if n:
            c.oracle.step(s, n)
        for f in FIELDS:
            h = hashlib.sha256(np.ascontiguousarray(getattr(s, f)).tobytes()).hexdigest()
            assert h == want[key][f], (key, f)
        assert [s.time, s.dt, s.steps] == want[key]["scalars"]


def test_eigen_kat():
    """dsyevh3 restated, against the reference's output on the matrices of
    tests.cxx:82-88 and 136-142 and 200 seeded ones.  The reference's Cardano
    branch is itself inaccurate for nearly isotropic matrices (its eigenvalues
    lose about half the digits of the deviatoric part there), so agreement is
    judged relative to the reference's own reconstruction error; the two
    tests.cxx matrices are well conditioned and reconstruct to 1e-12 (the checks
    of tests.cxx:79-127: V diag(w) V^T = A, V orthonormal)."""
    z = np.load(G / "eigen_kat.npz")
    for i, (a, q_ref, w_ref) in enumerate(zip(z["A"], z["Q"], z["w"])):
        rc, q, w = dsyevh3(a)
        full = np.triu(a) + np.triu(a, 1).T
        scale = np.abs(w_ref).max()
        err_ref = np.abs(q_ref @ np.diag(w_ref) @ q_ref.T - full).max() / scale
        err = np.abs(q @ np.diag(w) @ q.T - full).max() / scale
        if i < 2:
            assert err <= 1e-12 and np.abs(q.T @ q - np.eye(3)).max() <= 1e-12
        assert err <= max(1e-12, 10 * err_ref), (i, err, err_ref)
        assert np.abs(w - w_ref).max() / scale <= max(1e-12, 10 * err_ref), i
