"""The C-ABI library loads and exports every entry point of
include/spd_gb300.h (CPU: no compute call)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:int|const char\*)\s+(spd_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    assert "spd_create" in names and "spd_step" in names and len(names) >= 12


def test_library_exports_every_declared_symbol():
    from spd_gb300 import _lib
    from spd_gb300.build import build
    build()
    for path in (_lib.LIB_PATH, _lib.LIB_PATH_FMA):
        lib = ctypes.CDLL(path)
        missing = [n for n in declared() if not hasattr(lib, n)]
        assert not missing, (path, missing)
    assert set(_lib.EXPORTS) <= set(declared())


def test_version_string():
    from spd_gb300 import _lib
    lib = _lib.load()
    assert b"sm_103a" in lib.spd_version()


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from spd_gb300 import SDADER_Simulator
    from spd_gb300._lib import SpdError
    with pytest.raises(SpdError):
        SDADER_Simulator(N=(4,), p=1, verbose=False)
