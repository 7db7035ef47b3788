"""Python binding of libbm4dof_gpu.so, mirroring the reference's VideoNLB API.

The names follow src/core/nldct.h (initializeNlbParameters, setSizeSearchWindow,
setSizePatch, setNSimilarPatches, printNlbParameters, runNlBayes) so that code
written against the reference reads the same.  Videos are numpy arrays or
torch tensors of shape (frames, channels, height, width), float32 -- the
reference's planar layout.  CUDA tensors are passed to the library as device
pointers (no host round trip); everything else goes through host memory.

The library is the GPU implementation: there is no CPU fallback.  Importing
this module fails loudly when libbm4dof_gpu.so has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbm4dof_gpu.so")

DEVICE_POINTERS = 0x1
KEEP_GROUPS = 0x2
MIXED_PRECISION = 0x4

DCT, BIOR1_5 = 0, 1
RGB, YUV = 0, 1

STATUS = {
    0: "OK", 1: "ERR_ARGUMENT", 2: "ERR_CHANNELS", 3: "ERR_FWD_FLOW", 4: "ERR_BWD_FLOW",
    5: "ERR_NO_STEP", 6: "ERR_BASIC_SIZE", 7: "ERR_BIOR_SIZE", 8: "ERR_UNSUPPORTED",
    9: "ERR_CUDA", 10: "ERR_NO_MEMORY", 11: "ERR_TIMEOUT", 12: "ERR_NO_DEVICE",
}

# every entry point declared in include/bm4dof.h
EXPORTS = [
    "bm4dof_initialize_params", "bm4dof_set_size_search_window", "bm4dof_set_size_patch",
    "bm4dof_set_n_similar_patches", "bm4dof_format_params", "bm4dof_print_params",
    "bm4dof_last_error", "bm4dof_version", "bm4dof_create", "bm4dof_destroy", "bm4dof_run",
    "bm4dof_get_groups", "bm4dof_last_timings", "bm4dof_search_groups_noalloc",
]


class BM4DOFError(RuntimeError):
    """A failed library call; .status is the bm4dof_status name, str() the message
    (the reference's std::runtime_error text where it has one)."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code
        self.status = STATUS.get(code, str(code))


class Params(C.Structure):
    """bm4dof_params, field for field VideoNLB::nlbParams (src/core/nldct.h:55-82)."""
    _fields_ = [
        ("sigma", C.c_float), ("sizePatch", C.c_uint), ("sizePatchTime", C.c_uint),
        ("nSimilarPatches", C.c_uint), ("sizeSearchWindow", C.c_uint),
        ("sizeSearchTimeRangeFwd", C.c_uint), ("sizeSearchTimeRangeBwd", C.c_uint),
        ("boundary", C.c_uint), ("offSet", C.c_uint), ("offSetTime", C.c_uint),
        ("beta", C.c_float), ("betaMean", C.c_float), ("tau", C.c_float),
        ("orderInvariance", C.c_int), ("isFirstStep", C.c_int), ("doPasteBoost", C.c_int),
        ("verbose", C.c_int), ("colorSpace", C.c_int), ("transform", C.c_int),
        ("sizeSearchWindowPred", C.c_uint), ("nSimilarPatchesPred", C.c_uint),
        ("dsub", C.c_float), ("agg_window", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class VideoSize(C.Structure):
    _fields_ = [("width", C.c_uint), ("height", C.c_uint), ("frames", C.c_uint), ("channels", C.c_uint)]


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (once).  Raises OSError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with `python bm4d-of_gb300/build.py`")
    L = C.CDLL(path)
    L.bm4dof_initialize_params.argtypes = [C.POINTER(Params), C.c_uint, C.c_float, C.POINTER(VideoSize), C.c_int]
    L.bm4dof_initialize_params.restype = None
    L.bm4dof_set_size_search_window.argtypes = [C.POINTER(Params), C.c_uint]
    L.bm4dof_set_size_search_window.restype = None
    L.bm4dof_set_size_patch.argtypes = [C.POINTER(Params), C.POINTER(VideoSize), C.c_uint]
    L.bm4dof_set_size_patch.restype = None
    L.bm4dof_set_n_similar_patches.argtypes = [C.POINTER(Params), C.c_uint]
    L.bm4dof_set_n_similar_patches.restype = None
    L.bm4dof_format_params.argtypes = [C.POINTER(Params), C.c_char_p, C.c_size_t]
    L.bm4dof_format_params.restype = C.c_int
    L.bm4dof_print_params.argtypes = [C.POINTER(Params)]
    L.bm4dof_print_params.restype = None
    L.bm4dof_last_error.restype = C.c_char_p
    L.bm4dof_version.restype = C.c_char_p
    L.bm4dof_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    L.bm4dof_create.restype = C.c_int
    L.bm4dof_destroy.argtypes = [C.c_void_p]
    L.bm4dof_destroy.restype = None
    L.bm4dof_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint,
                             C.c_uint, C.c_void_p, C.c_void_p, C.POINTER(Params), C.POINTER(Params),
                             C.c_uint, C.c_uint, C.POINTER(C.c_float)]
    L.bm4dof_run.restype = C.c_int
    L.bm4dof_get_groups.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                    C.POINTER(C.c_uint), C.c_uint, C.c_size_t, C.POINTER(C.c_size_t)]
    L.bm4dof_get_groups.restype = C.c_int
    L.bm4dof_last_timings.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint)]
    L.bm4dof_last_timings.restype = C.c_int
    L.bm4dof_search_groups_noalloc.argtypes = [C.c_void_p] * 3 + [C.c_uint] * 4 + [
        C.POINTER(Params), C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_size_t,
        C.POINTER(C.c_size_t), C.c_void_p]
    L.bm4dof_search_groups_noalloc.restype = C.c_int
    _lib = L
    return L


def _check(code):
    if code != 0:
        raise BM4DOFError(code, load().bm4dof_last_error().decode())


# ---- parameter resolution: VideoNLB's setters ------------------------------

def initializeNlbParameters(step, sigma, size, verbose=False):
    """size = (width, height, frames, channels)."""
    p = Params()
    load().bm4dof_initialize_params(C.byref(p), step, sigma, C.byref(VideoSize(*size)), int(verbose))
    return p


def setSizeSearchWindow(p, wx):
    load().bm4dof_set_size_search_window(C.byref(p), wx)


def setSizePatch(p, size, px):
    load().bm4dof_set_size_patch(C.byref(p), C.byref(VideoSize(*size)), px)


def setNSimilarPatches(p, n):
    load().bm4dof_set_n_similar_patches(C.byref(p), n)


def formatNlbParameters(p) -> str:
    buf = C.create_string_buffer(4096)
    load().bm4dof_format_params(C.byref(p), buf, 4096)
    return buf.value.decode()


def printNlbParameters(p):
    load().bm4dof_print_params(C.byref(p))


def version() -> str:
    return load().bm4dof_version().decode()


# ---- device context ----------------------------------------------------------

def _is_cuda_tensor(x):
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


class Context:
    """A device context (one CUDA device, one stream) -- wraps bm4dof_create."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        _check(load().bm4dof_create(C.byref(self._h), device))
        self.device = device

    def close(self):
        if self._h:
            load().bm4dof_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def runNlBayes(self, noisy, fflow, bflow, p1, p2, basic=None, nparts=2, keep_groups=False,
                   final=None, mixed=False):
        """VideoNLB::runNlBayes.  Returns (basic, final, (ratio1, ratio2)).

        With CUDA tensors the inputs stay on the device and basic/final are
        CUDA tensors (pass preallocated ones to avoid allocation)."""
        flags = (KEEP_GROUPS if keep_groups else 0) | (MIXED_PRECISION if mixed else 0)
        if _is_cuda_tensor(noisy):
            import torch
            F, Cc, H, W = noisy.shape
            noisy = noisy.contiguous()
            if basic is None:
                basic = torch.empty_like(noisy)
            if final is None:
                final = torch.empty_like(noisy)
            ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
            ff = fflow.contiguous() if fflow is not None else None
            bf = bflow.contiguous() if bflow is not None else None
            args = (ptr(noisy), ptr(ff), ptr(bf), W, H, Cc, F, ptr(basic), ptr(final))
            flags |= DEVICE_POINTERS
        else:
            noisy = np.ascontiguousarray(noisy, np.float32)
            F, Cc, H, W = noisy.shape
            ff = None if fflow is None else np.ascontiguousarray(fflow, np.float32)
            bf = None if bflow is None else np.ascontiguousarray(bflow, np.float32)
            basic = np.zeros_like(noisy) if basic is None else np.array(basic, np.float32, copy=True)
            if final is None:
                final = np.zeros_like(noisy)
            ptr = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
            args = (ptr(noisy), ptr(ff), ptr(bf), W, H, Cc, F, ptr(basic), ptr(final))
        ratios = (C.c_float * 2)()
        _check(load().bm4dof_run(self._h, *args, C.byref(p1), C.byref(p2), nparts, flags, ratios))
        return basic, final, (ratios[0], ratios[1])

    def groups(self, step, tile, stride=32):
        """Neighbour lists of the last keep_groups run: dict(ref, nsimp, index)."""
        L = load()
        n = C.c_size_t()
        _check(L.bm4dof_get_groups(self._h, step, tile, None, None, None, stride, 0, C.byref(n)))
        cnt = n.value
        ref = np.zeros(cnt, np.uint32)
        ns = np.zeros(cnt, np.uint32)
        idx = np.zeros(cnt * stride, np.uint32)
        up = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint))
        _check(L.bm4dof_get_groups(self._h, step, tile, up(ref), up(ns), up(idx), stride, cnt, C.byref(n)))
        return {"ref": ref, "nsimp": ns, "index": idx.reshape(cnt, stride)}

    def timings(self):
        """(ms_search, ms_filter, ms_aggregation, ms_other, ms_total), kernel launches."""
        ms = (C.c_float * 5)()
        n = C.c_uint()
        _check(load().bm4dof_last_timings(self._h, ms, C.byref(n)))
        return tuple(ms), n.value


_default = None


def runNlBayes(noisy, fflow, bflow, p1, p2, basic=None, nparts=2, **kw):
    """Module-level VideoNLB::runNlBayes on device 0."""
    global _default
    if _default is None:
        _default = Context(0)
    return _default.runNlBayes(noisy, fflow, bflow, p1, p2, basic=basic, nparts=nparts, **kw)
