"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/bm4dof.h; host-only calls work without a device."""
import ctypes
import os
import re

from helpers import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "bm4dof.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bm4dof_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol(gpulib):
    lib = ctypes.CDLL(gpulib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(gpulib.EXPORTS) == names


def test_version_and_error_without_device(gpulib):
    assert "sm_103a" in gpulib.version()
    lib = gpulib.load()
    assert lib.bm4dof_last_error() is not None


def test_no_cpu_fallback_when_library_missing(tmp_path):
    import importlib
    import bm4dof
    mod = importlib.reload(bm4dof)
    mod._lib = None
    try:
        mod.load(str(tmp_path / "missing.so"))
    except OSError as e:
        assert "missing" in str(e)
    else:
        raise AssertionError("loading a missing library must fail")
    finally:
        mod._lib = None
