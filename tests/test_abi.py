"""The C-ABI library loads and exports every entry point the header declares (CPU only)."""
from __future__ import annotations

import ctypes
import glob
import os
import re

import pytest

from conftest import REPO


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(pa_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("pa_create", "pa_destroy", "pa_align_batch", "pa_align_batch_device", "pa_status_string"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built_lib):
    from pairwise_aligner_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def declared_arity():
    """name -> number of parameters of every prototype in include/*.h."""
    out = {}
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for name, args in re.findall(r"\b(pa_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
            args = args.strip()
            out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_python_binding_argument_counts_match_the_header(built_lib):
    from pairwise_aligner_gb300 import _lib
    arity = declared_arity()
    assert len(arity) >= 20
    wrong = {n: (k, len(_lib.SIGNATURES[n][0])) for n, k in arity.items() if len(_lib.SIGNATURES[n][0]) != k}
    assert not wrong, wrong


def test_status_strings_and_version(built_lib):
    from pairwise_aligner_gb300 import _lib
    lib = _lib.load()
    assert lib.pa_abi_version() == 2
    assert lib.pa_status_string(0) == b"ok"
    for code in range(1, 9):
        assert lib.pa_status_string(code) not in (b"", b"unknown status")


def test_struct_layouts_match_header(built_lib):
    from pairwise_aligner_gb300 import _lib
    assert ctypes.sizeof(_lib.PaResult) == 16
    assert ctypes.sizeof(_lib.PaConfig) == 32
    assert ctypes.sizeof(_lib.PaStats) == 8 * 14
    assert ctypes.sizeof(_lib.PaBandOptions) == 32


def test_create_without_gpu_reports_no_device(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pairwise_aligner_gb300 import _lib
    lib = _lib.load()
    ptr = ctypes.c_void_p()
    assert lib.pa_create(ctypes.byref(ptr), 0, None) == 7      # PA_ERR_NO_DEVICE, no crash
    assert not ptr
    assert lib.pa_destroy(None) == 0


def test_missing_library_fails_loudly(tmp_path):
    from pairwise_aligner_gb300 import _lib
    with pytest.raises(OSError):
        _lib.load(str(tmp_path / "absent.so"))
