"""The drop-in shims against the reference's own code: both compile against
its headers, and the reference program -- its unchanged dynearthsol.cxx and
every other source -- links with its hot-path functions taken from the shim
(dynearthsol-old_gb300/shim/link_reference.mk), each call in the loop body
binding to the shim's definition.  Runs where the reference tree is present."""
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SHIM = ROOT / "dynearthsol-old_gb300" / "shim"
sys.path.insert(0, str(ROOT))
from oracle.oracle import REF_SRC as REF  # noqa: E402

pytestmark = pytest.mark.skipif(not (REF / "parameters.hpp").exists(), reason="reference tree absent")

# what dynearthsol.cxx:358-394 calls on the hot path (update_mesh's parts included)
LOOP_CALLS = ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
              "update_stress", "NMD_stress", "update_force", "update_velocity", "apply_vbcs",
              "update_coordinate", "compute_volume", "compute_mass", "compute_shape_fn",
              "rotate_stress", "compute_dt"]


@pytest.mark.parametrize("src", ["des_shim.cpp", "des_shim_functions.cpp"])
def test_shim_compiles_against_reference_headers(src):
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-DTHREED", f"-I{REF}", f"-I{ROOT / 'include'}",
           f"-I{SHIM}", str(SHIM / src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_program_links_with_the_hot_path_from_the_shim(tmp_path):
    # boost (program_options) is absent here: get_input_parameters comes from
    # a stub, every other object from the reference's sources
    stub = tmp_path / "input_stub.cpp"
    stub.write_text("#include <cstdlib>\nstruct Param;\n"
                    "void get_input_parameters(const char *, Param &) { std::exit(2); }\n")
    subprocess.run(["g++", "-c", "-fPIC", str(stub), "-o", str(tmp_path / "input_stub.o")], check=True)
    out = ROOT / "dynearthsol-old_gb300" / "_build" / "ref_link"
    exe = out / "dynearthsol3d_gpu"
    if exe.exists():
        exe.unlink()
    cmd = ["make", "-s", "-f", str(SHIM / "link_reference.mk"), f"REF={REF}", f"OUT={out}",
           f"INPUT_OBJ={tmp_path / 'input_stub.o'}", f"LINK_EXTRA=-Wl,-Map={tmp_path / 'map.txt'}",
           "-j8"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-3000:]

    syms = (out / "shim_symbols.txt").read_text().split()
    def plain(s):                       # _Z<length><name><parameters>
        n = re.match(r"_Z(\d+)", s)
        return s[n.end():n.end() + int(n.group(1))]

    names = {plain(s) for s in syms}
    assert names == set(LOOP_CALLS)

    # the loop body calls them (undefined in the reference's dynearthsol.o) ...
    undef = subprocess.run(["nm", "-u", str(out / "weak" / "dynearthsol.o")], capture_output=True,
                           text=True, check=True).stdout
    for fn in ["update_temperature", "update_strain_rate", "update_stress", "NMD_stress",
               "update_force", "compute_dt", "rotate_stress", "compute_volume"]:
        assert any(re.search(rf"_Z\d+{fn}R", ln) for ln in undef.splitlines()), fn

    # ... and in the program every one of them is the shim's definition
    text = (tmp_path / "map.txt").read_text()
    m = re.search(r"^ \.text\s+0x([0-9a-f]+)\s+0x([0-9a-f]+)\s+\S*des_shim_functions\.o$", text, re.M)
    assert m, "des_shim_functions.o has no .text in the link map"
    lo, hi = int(m.group(1), 16), int(m.group(1), 16) + int(m.group(2), 16)
    table = subprocess.run(["nm", str(exe)], capture_output=True, text=True, check=True).stdout
    addr = {ln.split()[2]: int(ln.split()[0], 16) for ln in table.splitlines()
            if len(ln.split()) == 3 and ln.split()[1] == "T"}
    for s in syms:
        assert lo <= addr[s] < hi, s

    # the program starts (the loader finds libdes_gb300.so) and prints its usage
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert "Usage" in r.stdout
