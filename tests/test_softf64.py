"""The integer-pipe FP64 multiply, FP64 -> FP32 conversion, 0 + x, 2 x, x / 2,
x / 6, x / 3 and x / 4 the step kernels use in place of FP64 unit instructions
(dynearthsol-old_gb300/csrc/des_softf64.cuh), bit for bit against IEEE
arithmetic: against the host's on every operand kind (zeros, subnormals,
infinities, NaN, ties, overflow and underflow thresholds), and against the
GPU's own FP64 unit."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "dynearthsol-old_gb300" / "csrc"
BUILD = ROOT / "dynearthsol-old_gb300" / "_build"


def test_host_bit_identical_to_ieee():
    BUILD.mkdir(exist_ok=True)
    exe = BUILD / "softf64_check"
    src = ROOT / "tests" / "softf64_check.cpp"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", f"-I{CSRC}",
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "4000000"], capture_output=True, text=True, timeout=600)
    lines = [l for l in r.stdout.splitlines() if "mismatches" in l]
    assert len(lines) == 42, r.stdout
    assert r.returncode == 0 and all(l.endswith(" 0 mismatches") for l in lines), r.stdout


@pytest.mark.gpu
def test_device_bit_identical_to_the_fp64_unit(gpu):
    import des_gb300 as D
    bad = D.softf64_check(1 << 28)
    assert bad == [0] * 10, bad
