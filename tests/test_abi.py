"""The C ABI: the library loads and exports every entry point include/gbk.h declares."""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gbk.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbk_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from deformetrica_code_gb300 import _lib
    lib = _lib.load()
    declared = declared_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes signatures cover exactly the declared ABI
    assert sorted(_lib.SIGNATURES) == declared


def test_nm_exports_match_header():
    import subprocess
    from deformetrica_code_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r"\sT\s(gbk_[a-z0-9_]+)$", out, flags=re.M)))
    assert exported == declared_symbols()


def test_create_without_device_fails_cleanly():
    """No GPU here: gbk_create reports GBK_ERR_CUDA instead of crashing."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    from deformetrica_code_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.gbk_create(0, ctypes.byref(h))
    assert rc == _lib.GBK_ERR_CUDA
    assert not h.value
    assert b"device" in lib.gbk_last_error(None)


def test_null_context_is_an_argument_error():
    from deformetrica_code_gb300 import _lib
    lib = _lib.load()
    assert lib.gbk_set_mode(None, 0) == _lib.GBK_ERR_ARG
    assert lib.gbk_convolve(None, 3, 3, None, 0, None, None, 0, 1.0, None) == _lib.GBK_ERR_ARG
