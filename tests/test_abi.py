"""The C-ABI library builds for sm_103a, loads without a GPU and exports every entry point that
include/cvf.h declares; argument checks fail with CVF_EINVAL before any CUDA call."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "cvf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cvf_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_version_string(engine_lib):
    assert b"sm_103a" in engine_lib.cvf_version()


@pytest.mark.parametrize("field,value,msg", [
    ("L", 7, b"even"),
    ("L", 2, b"even"),
    ("L", 712, b"too large"),       # 6 L^3 > 2^31 - 1
    ("L", 1200000, b"too large"),   # 6 L^3 would overflow a signed 64-bit product of ints
    ("L", 2147483646, b"too large"),
    ("flag_chessboard", 2, b"Flag_chessboard"),
    ("start", 3, b"Flag_config"),
    ("T", 0.0, b"T must"),
])
def test_invalid_params_rejected_without_gpu(engine_lib, field, value, msg):
    from cvfbulkwater_gb300 import abi
    p = abi.Params(16, 0.8, 0.45, 1, 6.0, 0, 1, 0, 0, 0)
    setattr(p, field, value)
    h = C.c_void_p()
    rc = engine_lib.cvf_create(C.byref(p), C.byref(h))
    assert rc == -1
    assert msg in engine_lib.cvf_last_error_string()
    assert not h.value


def test_package_fails_loudly_without_library(tmp_path, monkeypatch):
    from cvfbulkwater_gb300 import abi
    monkeypatch.setattr(abi, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(abi, "_lib", None)
    with pytest.raises(FileNotFoundError):
        abi.lib()
