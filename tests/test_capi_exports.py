"""libmcg.so loads without a GPU and exports every entry point that
include/*.h declares."""
import ctypes
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(REPO, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(inc, f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        m = re.search(r'extern "C" \{(.*)\}', txt, re.S)
        if not m:
            continue
        for name in re.findall(r"\b(mcg_\w+)\s*\(", m.group(1)):
            names.add(name)
    return sorted(names)


def test_library_exports_all_declared():
    import marching_cube_gb300 as m
    lib = ctypes.CDLL(m.library_path())
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    import marching_cube_gb300 as m
    lib = m._lib
    assert lib.mcg_status_string(0) == b"ok"
    assert lib.mcg_status_string(2) == b"output capacity exceeded"
    assert lib.mcg_version() >= 100


def test_create_without_device_fails_cleanly():
    import torch
    import marching_cube_gb300 as m
    if torch.cuda.is_available():
        return
    h = ctypes.c_void_p()
    st = m._lib.mcg_create(ctypes.byref(h), 0)
    assert st in (m.MCG_ERR_CUDA, m.MCG_ERR_INVALID_ARG)
    assert not h.value


def test_rle_bound_and_header_host_only():
    import marching_cube_gb300 as m
    assert m._lib.mcg_rle_bound(4, 4, 4) == 40 + 4 * (4 + 6 * 16)
    assert m._lib.mcg_rle_bound(0, 4, 4) == 0
    import pytest
    with pytest.raises(m.MCGError):
        m.rle_header(b"NOT_A_VOLUME_TAG" + bytes(24))
