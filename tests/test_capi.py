"""The C-ABI library loads and exports every entry point include/gbsym.h
declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re
import subprocess

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "gbsym.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbsym_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from sympiler_gb300 import _lib
    path = _lib.LIB_PATH
    assert os.path.exists(path), "libgbsym.so not built"
    L = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from sympiler_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == _declared()


def test_library_has_no_cuda_runtime_dependency():
    from sympiler_gb300 import _lib
    out = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "libcudart" not in out


def test_status_strings_without_gpu():
    from sympiler_gb300 import _lib
    L = _lib.lib()
    assert L.gbsym_status_string(0) == b"ok"
    assert b"schedule" in L.gbsym_status_string(_lib.ERR_BAD_SCHEDULE)
    assert L.gbsym_last_error() == 0
