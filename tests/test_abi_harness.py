"""The C ABI called from compiled C (tests/abi_harness.c), not through ctypes:
config 1 built, initialised and stepped 2,000 times by a plain C program
linked against libdes_gb300.so; every field after init, 100 and 2,000 steps
hashes to the reference's own (tests/golden/config1_hashes.json)."""
import hashlib
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import workload as W
from test_golden import FIELDS

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
NODE3, NODE1 = {"coord", "vel", "force"}, {"temperature", "mass", "tmass", "volume_n", "ntmp"}
ELEM6, ELEM4 = {"stress", "strain", "strain_rate"}, {"shpdx", "shpdy", "shpdz"}


def build_harness(tmp):
    exe = tmp / "abi_harness"
    lib = D.build()
    cmd = ["gcc", "-std=c99", "-O2", str(HERE / "abi_harness.c"), f"-I{ROOT / 'include'}",
           f"-L{lib.parent}", "-ldes_gb300", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_harness_compiles_and_links(tmp_path):
    assert build_harness(tmp_path).exists()


@pytest.mark.gpu
def test_c_caller_config1_2000_steps_hashes_equal_reference(gpu, tmp_path):
    exe = build_harness(tmp_path)
    cfg = W.CONFIGS["1"]
    mesh, p, T, pls, _ = D.setup_case(cfg)
    pfile, out = tmp_path / "params.bin", tmp_path / "fields.bin"
    pfile.write_bytes(bytes(W.make_params(cfg)))       # boundary normals are the harness's own
    args = [str(exe), str(pfile), str(cfg.nx), str(cfg.ny), str(cfg.nz), repr(cfg.xlength),
            repr(cfg.ylength), repr(cfg.zlength), repr(cfg.jitter), str(cfg.mesh_seed), "273.0",
            repr(273.0 + cfg.t_bottom_c), str(out)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.float64)
    N, E = mesh.nnode, mesh.nelem
    size = {f: (3 * N if f in NODE3 else N if f in NODE1 else 6 * E if f in ELEM6
                else 4 * E if f in ELEM4 else E) for f in FIELDS}
    want = json.loads((HERE / "golden" / "config1_hashes.json").read_text())
    pos = 0
    for key in ("init", "step100", "step2000"):
        for f in FIELDS:
            a = raw[pos:pos + size[f]]
            pos += size[f]
            assert hashlib.sha256(a.tobytes()).hexdigest() == want[key][f], (key, f)
        assert list(raw[pos:pos + 3]) == want[key]["scalars"], key
        pos += 3
    assert pos == raw.size
