"""CPU checks of the drop-in boundary: the C-ABI library loads and exports
every entry point include/ima_gpu.h declares (no device calls)."""
import ctypes
import os
import re

import pytest

from ima2p_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "ima_gpu.h")).read()
    return sorted(set(re.findall(r"\b(ima_(?:gpu|mt19937|ti|ug_rng)_\w+)\s*\(", txt)))


def test_header_and_wrapper_agree():
    assert declared() == sorted(api.EXPORTS)


def test_library_exports_every_symbol():
    if not os.path.exists(api.LIB_PATH):
        pytest.skip("library not built here")
    lib = ctypes.CDLL(api.LIB_PATH)
    missing = [s for s in declared() if not hasattr(lib, s)]
    assert not missing, missing


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(api.ImaError):
        api._lib = None
        api.load_library(str(tmp_path / "nope.so"))
    api._lib = None
