"""The C-ABI library loads without a GPU and exports every declared symbol."""
import ctypes as C
import re
from pathlib import Path

import des_gb300 as D
from des_gb300 import abi

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(des_[a-zA-Z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    L = D.lib()
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_sizes_match_the_header():
    L = D.lib()
    out = (C.c_longlong * 5)()
    L.des_abi_sizes(out)
    mine = [C.sizeof(abi.Params), C.sizeof(abi.MeshView), C.sizeof(abi.StateView),
            C.sizeof(abi.Topology), C.sizeof(abi.StepReport)]
    assert list(out) == mine


def test_error_strings():
    L = D.lib()
    for code in [0, 1, 2, 3, 4, 5, 6, 11, 12, 99]:
        assert L.des_gpu_error_string(code)


def test_create_rejects_bad_arguments_without_touching_the_gpu():
    L = D.lib()
    h = C.c_void_p()
    assert L.des_gpu_create(None, None, 0, C.byref(h)) == abi.DES_ERR_ARG
