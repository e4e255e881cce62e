"""Writes the golden fixtures of tests/test_golden.py from the reference's own
functions (oracle/_ref/libdesref.so, built from the reference sources by
oracle/ref.mk).  Run in a tree where the reference exists:

    python tests/golden/make_golden.py

Fixtures (all small):
  tiny_states.npz     144-tet box (config-2 physics): full state after init and
                      after 1, 10 and 50 steps
  plastic_states.npz  540-tet yielding box: state after 30 steps and after one
                      more step, and update_stress alone from the loop state
  evp_states.npz      540-tet elasto-visco-plastic box: state after init and 20 steps
  config1_hashes.json SHA-256 of every field of config 1 (9,600 tets) after
                      init, 100 and 2,000 steps
  eigen_kat.npz       dsyevh3 on the matrices of the reference's tests.cxx:82-88
                      and 136-142 and on 200 seeded symmetric matrices
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "dynearthsol-old_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import des_gb300 as D                     # noqa: E402
from des_gb300 import abi, workload as W  # noqa: E402
from oracle import oracle as O            # noqa: E402
from helpers import plastic_config, evp_config, LOOP, MESH_PARTS  # noqa: E402

FIELDS = ["coord", "vel", "force", "temperature", "mass", "tmass", "volume_n", "ntmp", "volume",
          "volume_old", "edvoldt", "plstrain", "delta_plstrain", "dpressure", "stress", "strain",
          "strain_rate", "shpdx", "shpdy", "shpdz"]


def pack(prefix, s, out):
    for f in FIELDS:
        out[f"{prefix}/{f}"] = getattr(s, f).copy()
    out[f"{prefix}/scalars"] = np.array([s.time, s.dt, s.steps], dtype=np.float64)


def field_hashes(s):
    h = {f: hashlib.sha256(np.ascontiguousarray(getattr(s, f)).tobytes()).hexdigest() for f in FIELDS}
    h["scalars"] = [s.time, s.dt, s.steps]
    return h


def ref_case(cfg):
    D.build()
    O.build_ref()
    mesh, p, T, pls, _ = D.setup_case(cfg)
    r = O.RefOracle(mesh, p)
    s = W.new_state(mesh, T, pls)
    r.init_fields(s)
    return mesh, p, r, s


def main():
    out = {}
    mesh, p, r, s = ref_case(W.CONFIGS["tiny"])
    pack("init", s, out)
    done = 0
    for n in (1, 10, 50):
        r.step(s, n - done)
        done = n
        pack(f"step{n}", s, out)
    np.savez_compressed(HERE / "tiny_states.npz", **out)

    out = {}
    mesh, p, r, s = ref_case(plastic_config())
    r.step(s, 30)
    pack("step30", s, out)
    s1 = s.copy()
    r.step(s1, 1)
    pack("step31", s1, out)
    # update_stress alone from the state the loop hands it at step 31
    si = s.copy()
    si.steps += 1
    si.time += si.dt
    for f in ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt"]:
        r.call(f, si)
    pack("before_stress", si, out)
    r.call("update_stress", si)
    pack("after_stress", si, out)
    np.savez_compressed(HERE / "plastic_states.npz", **out)

    out = {}
    mesh, p, r, s = ref_case(evp_config())
    pack("init", s, out)
    r.step(s, 20)
    pack("step20", s, out)
    np.savez_compressed(HERE / "evp_states.npz", **out)

    hashes = {}
    mesh, p, r, s = ref_case(W.CONFIGS["1"])
    hashes["init"] = field_hashes(s)
    r.step(s, 100)
    hashes["step100"] = field_hashes(s)
    r.step(s, 1900)
    hashes["step2000"] = field_hashes(s)
    (HERE / "config1_hashes.json").write_text(json.dumps(hashes, indent=1))

    mats = [np.array([[3e4, 2, 4], [0, -1, 2], [0, 0, 3]], float),      # tests.cxx:82-88
            np.array([[3e4, 2, 4], [0, -1e-5, 8], [0, 0, 3]], float)]   # tests.cxx:136-142
    rng = np.random.default_rng(20260101)
    for i in range(200):
        a = rng.normal(size=(3, 3)) * 10 ** rng.uniform(0, 8)
        a = a + a.T
        if i % 3 == 0:
            a += np.eye(3) * rng.normal() * 1e8
        mats.append(np.triu(a))
    A = np.array(mats)
    Q = np.zeros_like(A)
    Wv = np.zeros((len(A), 3))
    for i, a in enumerate(A):
        _, Q[i], Wv[i] = O.dsyevh3(a, "ref")
    np.savez_compressed(HERE / "eigen_kat.npz", A=A, Q=Q, w=Wv)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
