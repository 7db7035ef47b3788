"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/bm4dof.h; host-only calls work without a device."""
import ctypes
import os
import re

import numpy as np

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


def test_stream_getters_refuse_null_handles(gpulib):
    """bm4dof_get_stream / bm4dof_trainer_get_stream check their arguments
    before touching a device."""
    lib = gpulib.load()
    out = ctypes.c_void_p()
    assert lib.bm4dof_get_stream(None, ctypes.byref(out)) == 1
    assert lib.bm4dof_trainer_get_stream(None, ctypes.byref(out)) == 1
    assert b"null" in lib.bm4dof_last_error()


def test_host_outputs_are_written_in_place(gpulib):
    """runNlBayes on host arrays writes a caller's writable C-contiguous
    float32 basic/final in place (pinned buffers stay the copy targets) and
    copies anything else."""
    shape = (2, 1, 4, 5)
    a = np.zeros(shape, np.float32)
    assert gpulib._out_array(a, shape) is a
    for other in (np.zeros(shape, np.float64), np.zeros((2, 1, 5, 4), np.float32).transpose(0, 1, 3, 2),
                  np.zeros((2, 20), np.float32)):
        b = gpulib._out_array(other, shape)
        assert b is not other and b.dtype == np.float32 and b.shape == shape
    ro = np.zeros(shape, np.float32)
    ro.setflags(write=False)
    assert gpulib._out_array(ro, shape) is not ro


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


def test_flag_values_match_the_header(gpulib):
    """The Python binding's run flags are the header's #define values."""
    import pyoracle
    text = open(os.path.join(ROOT, "include", "bm4dof.h")).read()
    flags = {m.group(1): int(m.group(2), 16) for m in re.finditer(r"#define BM4DOF_([A-Z0-9_]+)\s+0x([0-9a-fA-F]+)u", text)}
    for name in ("DEVICE_POINTERS", "KEEP_GROUPS", "MIXED_PRECISION", "LEARNED", "VBM3D_SEARCH"):
        assert getattr(gpulib, name) == flags[name], name
    assert pyoracle.VBM3D_SEARCH == flags["VBM3D_SEARCH"]


def test_cli_params_take_the_predictive_search_options(gpulib, oracle):
    """bm4dof.cli_params resolves -wxf/-npf/-dsub/-t like the reference's VBM3D_SEARCH build."""
    from helpers import resolve_params
    kw = dict(px1=4, np1=16, wxf1=7, wxf2=3, npf1=3, npf2=4, dsub1=2.5, dsub2=0.0, t1=40.0, t2=12.0)
    a = gpulib.cli_params((40, 36, 6, 1), 20.0, **kw)
    b = resolve_params(oracle, (40, 36, 6, 1), 20.0, **kw)
    for pa, pb in zip(a, b):
        for f, _ in gpulib.Params._fields_:
            assert getattr(pa, f) == getattr(pb, f), f
