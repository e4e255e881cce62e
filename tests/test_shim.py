"""The drop-in shim compiles against the reference's own headers."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = Path("/root/reference")


@pytest.mark.skipif(not (REF / "parameters.hpp").exists(), reason="reference headers absent")
def test_shim_compiles_against_reference_headers():
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-DTHREED", f"-I{REF}", f"-I{ROOT / 'include'}",
           f"-I{ROOT / 'dynearthsol-old_gb300' / 'shim'}",
           str(ROOT / "dynearthsol-old_gb300" / "shim" / "des_shim.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
