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

import contextlib
import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbm4dof_gpu.so")

DEVICE_POINTERS = 0x1
KEEP_GROUPS = 0x2
MIXED_PRECISION = 0x4
LEARNED = 0x8
VBM3D_SEARCH = 0x10   # the predictive search of the reference's VBM3D_SEARCH build
MIXED_CERTIFIED = 0x20   # mixed precision with the exact path's neighbour lists
GAIN_PARAMS = 99136   # floats in a gain-network parameter blob

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
    "bm4dof_last_error", "bm4dof_version", "bm4dof_create", "bm4dof_destroy", "bm4dof_get_stream", "bm4dof_run",
    "bm4dof_process",
    "bm4dof_set_memory_limit", "bm4dof_plan",
    "bm4dof_get_groups", "bm4dof_last_timings", "bm4dof_search_groups_noalloc",
    "bm4dof_set_gain_network", "bm4dof_learned_stats", "bm4dof_mixed_stats", "bm4dof_tc_selftest", "bm4dof_fp32_mix_rate",
    "bm4dof_gain_samples",
    "bm4dof_trainer_create", "bm4dof_trainer_destroy", "bm4dof_trainer_get_stream", "bm4dof_trainer_params",
    "bm4dof_trainer_state",
    "bm4dof_trainer_grad",
    "bm4dof_trainer_step", "bm4dof_trainer_predict", "bm4dof_run_batched", "bm4dof_autotune",
    "bm4dof_tvl1_default_params", "bm4dof_tvl1_pairs", "bm4dof_tvl1_video",
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


class Crop(C.Structure):
    """bm4dof_crop: the fields of VideoUtils::CropPosition that processNlBayes reads."""
    _fields_ = [("origin_x", C.c_int), ("origin_y", C.c_int), ("origin_t", C.c_int),
                ("ending_x", C.c_int), ("ending_y", C.c_int), ("ending_t", C.c_int),
                ("source_sz", VideoSize)]


def make_crop(origin, ending, source):
    """origin/ending (x, y, t); source (width, height, frames, channels)."""
    return Crop(*origin, *ending, VideoSize(*source))


class Sequence(C.Structure):
    """bm4dof_sequence: one sequence of a batched run (device pointers)."""
    _fields_ = [
        ("noisy", C.c_void_p), ("fflow", C.c_void_p), ("bflow", C.c_void_p),
        ("width", C.c_uint), ("height", C.c_uint), ("channels", C.c_uint), ("frames", C.c_uint),
        ("basic", C.c_void_p), ("final_", C.c_void_p), ("params1", Params), ("params2", Params),
        ("nparts", C.c_uint), ("ratios", C.c_float * 2),
    ]


class Tuning(C.Structure):
    """bm4dof_tuning: launch shape of a batched run."""
    _fields_ = [("branches", C.c_uint), ("slot_mb", C.c_uint), ("search_ctas", C.c_uint),
                ("search_strip", C.c_uint), ("gather_depth", C.c_uint)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tvl1Params(C.Structure):
    """bm4dof_tvl1_params (lib/tvl1flow's arguments)."""
    _fields_ = [("tau", C.c_float), ("lambda_", C.c_float), ("theta", C.c_float), ("nscales", C.c_int),
                ("fscale", C.c_int), ("zfactor", C.c_float), ("warps", C.c_int), ("epsilon", C.c_float)]


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
    L.bm4dof_get_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    L.bm4dof_get_stream.restype = C.c_int
    L.bm4dof_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint,
                             C.c_uint, C.c_void_p, C.c_void_p, C.POINTER(Params), C.POINTER(Params),
                             C.c_uint, C.c_uint, C.POINTER(C.c_float)]
    L.bm4dof_run.restype = C.c_int
    L.bm4dof_process.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint,
                                 C.c_uint, C.c_void_p, C.c_void_p, C.POINTER(Params), C.POINTER(Crop), C.c_uint,
                                 C.POINTER(C.c_uint)]
    L.bm4dof_process.restype = C.c_int
    L.bm4dof_set_memory_limit.argtypes = [C.c_void_p, C.c_size_t]
    L.bm4dof_set_memory_limit.restype = C.c_int
    L.bm4dof_plan.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.POINTER(Params), C.POINTER(Crop), C.c_int,
                              C.c_void_p, C.c_uint, C.c_void_p, C.c_size_t, C.POINTER(C.c_uint),
                              C.POINTER(C.c_size_t)]
    L.bm4dof_plan.restype = C.c_int
    L.bm4dof_get_groups.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                    C.POINTER(C.c_uint), C.c_uint, C.c_size_t, C.POINTER(C.c_size_t)]
    L.bm4dof_get_groups.restype = C.c_int
    L.bm4dof_last_timings.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint)]
    L.bm4dof_last_timings.restype = C.c_int
    L.bm4dof_search_groups_noalloc.argtypes = [C.c_void_p] * 3 + [C.c_uint] * 4 + [
        C.POINTER(Params), C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_size_t,
        C.POINTER(C.c_size_t), C.c_void_p]
    L.bm4dof_search_groups_noalloc.restype = C.c_int
    L.bm4dof_run_batched.argtypes = [C.c_void_p, C.POINTER(Sequence), C.c_uint, C.c_uint, C.POINTER(Tuning)]
    L.bm4dof_run_batched.restype = C.c_int
    L.bm4dof_autotune.argtypes = [C.c_void_p, C.POINTER(Sequence), C.c_uint, C.c_uint, C.c_uint,
                                  C.POINTER(Tuning), C.POINTER(C.c_float), C.c_uint, C.POINTER(C.c_uint)]
    L.bm4dof_autotune.restype = C.c_int
    L.bm4dof_tvl1_default_params.argtypes = [C.POINTER(Tvl1Params)]
    L.bm4dof_tvl1_default_params.restype = None
    L.bm4dof_tvl1_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint,
                                    C.POINTER(Tvl1Params), C.c_void_p, C.c_uint]
    L.bm4dof_tvl1_pairs.restype = C.c_int
    L.bm4dof_tvl1_video.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.POINTER(Tvl1Params),
                                    C.c_void_p, C.c_void_p, C.c_uint]
    L.bm4dof_tvl1_video.restype = C.c_int
    L.bm4dof_set_gain_network.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_float]
    L.bm4dof_set_gain_network.restype = C.c_int
    L.bm4dof_learned_stats.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]
    L.bm4dof_learned_stats.restype = C.c_int
    L.bm4dof_mixed_stats.argtypes = [C.c_void_p] + [C.POINTER(C.c_ulonglong)] * 3
    L.bm4dof_mixed_stats.restype = C.c_int
    L.bm4dof_tc_selftest.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.bm4dof_tc_selftest.restype = C.c_int
    L.bm4dof_fp32_mix_rate.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.bm4dof_fp32_mix_rate.restype = C.c_int
    L.bm4dof_gain_samples.argtypes = [C.c_void_p] * 5 + [C.c_uint] * 3 + [
        C.POINTER(Params), C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
        C.POINTER(C.c_size_t)]
    L.bm4dof_gain_samples.restype = C.c_int
    L.bm4dof_trainer_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_uint, C.c_uint]
    L.bm4dof_trainer_create.restype = C.c_int
    L.bm4dof_trainer_destroy.argtypes = [C.c_void_p]
    L.bm4dof_trainer_destroy.restype = None
    L.bm4dof_trainer_get_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    L.bm4dof_trainer_get_stream.restype = C.c_int
    L.bm4dof_trainer_params.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    L.bm4dof_trainer_params.restype = C.c_int
    L.bm4dof_trainer_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                       C.POINTER(C.c_ulonglong), C.c_int]
    L.bm4dof_trainer_state.restype = C.c_int
    L.bm4dof_trainer_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p,
                                      C.POINTER(C.c_float)]
    L.bm4dof_trainer_grad.restype = C.c_int
    L.bm4dof_trainer_step.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_float, C.c_float,
                                      C.POINTER(C.c_float)]
    L.bm4dof_trainer_step.restype = C.c_int
    L.bm4dof_trainer_predict.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p]
    L.bm4dof_trainer_predict.restype = C.c_int
    _lib = L
    return L


def _out_array(a, shape):
    """a itself when it is a writable C-contiguous float32 array of `shape`,
    else a float32 copy of it (returned to the caller, as the outputs are)."""
    if isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and \
            a.flags["WRITEABLE"] and a.shape == tuple(shape):
        return a
    return np.array(a, np.float32, copy=True).reshape(shape)


def _mixed_flags(mixed):
    """mixed=True: the mixed-precision form; mixed="certified": the same with
    the exact path's neighbour lists (BM4DOF_MIXED_CERTIFIED)."""
    if mixed == "certified":
        return MIXED_PRECISION | MIXED_CERTIFIED
    return MIXED_PRECISION if mixed else 0


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


def cli_params(size, sigma, px1=-1, px2=-1, pt1=1, pt2=1, wx1=-1, wx2=-1, np1=-1, np2=-1, b1=-1.0,
               b2=-1.0, bm1=-1.0, bm2=-1.0, no_step1=False, no_step2=False, order_inv=False, verbose=False,
               wxf1=-1, wxf2=-1, npf1=-1, npf2=-1, dsub1=-1.0, dsub2=-1.0, t1=-1.0, t2=-1.0):
    """Parameters of both steps as the reference CLI resolves them from its
    flags (src/main_vnlb.cpp:206-246; -t1/-t2 only apply under VBM3D_SEARCH,
    -wt1/-wt2 never).  size = (width, height, frames, channels); -1 = flag
    not given.  wxf*/npf*/dsub*/t* are the options of the VBM3D_SEARCH build
    (main_vnlb.cpp:227-236), for runs with vbm3d=True."""
    p1 = initializeNlbParameters(1, sigma, size, verbose)
    p2 = initializeNlbParameters(2, sigma, size, verbose)
    if wx1 >= 0: setSizeSearchWindow(p1, wx1)
    if wx2 >= 0: setSizeSearchWindow(p2, wx2)
    if px1 >= 0: setSizePatch(p1, size, px1)
    if px2 >= 0: setSizePatch(p2, size, px2)
    if np1 >= 0: setNSimilarPatches(p1, np1)
    if np2 >= 0: setNSimilarPatches(p2, np2)
    if b1 >= 0: p1.beta = b1; p1.betaMean = b1
    if b2 >= 0: p2.beta = b2; p2.betaMean = b2
    if bm1 >= 0: p1.betaMean = bm1
    if bm2 >= 0: p2.betaMean = bm2
    if pt1 >= 0: p1.sizePatchTime = pt1
    if pt2 >= 0: p2.sizePatchTime = pt2
    if no_step1: p1.offSet = 1
    if no_step2: p2.offSet = 1
    if wxf1 >= 0: p1.sizeSearchWindowPred = wxf1
    if wxf2 >= 0: p2.sizeSearchWindowPred = wxf2
    if npf1 >= 0: p1.nSimilarPatchesPred = npf1
    if npf2 >= 0: p2.nSimilarPatchesPred = npf2
    if dsub1 >= 0: p1.dsub = dsub1
    if dsub2 >= 0: p2.dsub = dsub2
    if t1 >= 0: p1.tau = t1
    if t2 >= 0: p2.tau = t2
    if order_inv:
        p1.orderInvariance = 1
        p2.orderInvariance = 1
    return p1, p2


# ---- device context ----------------------------------------------------------

def _is_cuda_tensor(x):
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


@contextlib.contextmanager
def _stream_order(get_stream, handle, device):
    """Orders the library's own stream (bm4dof_get_stream,
    bm4dof_trainer_get_stream) after torch's current stream on entry, and
    torch's current stream after it on exit, so that CUDA tensors torch has
    just written are complete before the library reads them, and memory that
    torch frees after the call is not reused while the library still reads
    it.  Neither side waits on the host."""
    import torch
    s = C.c_void_p()
    _check(get_stream(handle, C.byref(s)))
    cur = torch.cuda.current_stream(device)
    lib = torch.cuda.ExternalStream(s.value, device=device)
    lib.wait_stream(cur)
    try:
        yield
    finally:
        cur.wait_stream(lib)


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

    def _ordered(self):
        return _stream_order(load().bm4dof_get_stream, self._h, self.device)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def runNlBayes(self, noisy, fflow, bflow, p1, p2, basic=None, nparts=2, keep_groups=False,
                   final=None, mixed=False, learned=False, vbm3d=False):
        """VideoNLB::runNlBayes.  Returns (basic, final, (ratio1, ratio2)).

        vbm3d=True searches neighbours like the reference built with
        VBM3D_SEARCH (predictive search along the best matches of each frame).

        With CUDA tensors the inputs stay on the device and basic/final are
        CUDA tensors (pass preallocated ones to avoid allocation).
        learned=True runs the learned form (no step-1 pass; the gain network
        installed by set_gain_network, or none)."""
        flags = (KEEP_GROUPS if keep_groups else 0) | _mixed_flags(mixed)
        flags |= (LEARNED if learned else 0) | (VBM3D_SEARCH if vbm3d else 0)
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
            # basic is in/out as the reference's Video<float>& basic: the
            # caller's array is written in place when it can take float32 data
            # (so pinned host buffers stay the copy targets), else a copy is
            basic = np.zeros_like(noisy) if basic is None else _out_array(basic, noisy.shape)
            final = np.zeros_like(noisy) if final is None else _out_array(final, noisy.shape)
            ptr = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
            args = (ptr(noisy), ptr(ff), ptr(bf), W, H, Cc, F, ptr(basic), ptr(final))
        ratios = (C.c_float * 2)()
        if flags & DEVICE_POINTERS:
            with self._ordered():
                _check(load().bm4dof_run(self._h, *args, C.byref(p1), C.byref(p2), nparts, flags, ratios))
        else:
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

    @staticmethod
    def _sequences(items):
        """items: dicts with CUDA tensors noisy, fflow, bflow (or None), basic,
        final (F, C, H, W) and params p1, p2 (and optional nparts)."""
        arr = (Sequence * len(items))()
        for q, it in zip(arr, items):
            F, Cc, H, W = it["noisy"].shape
            ptr = lambda t: t.data_ptr() if t is not None else None
            q.noisy, q.fflow, q.bflow = ptr(it["noisy"]), ptr(it.get("fflow")), ptr(it.get("bflow"))
            q.width, q.height, q.channels, q.frames = W, H, Cc, F
            q.basic, q.final_ = ptr(it["basic"]), ptr(it["final"])
            q.params1, q.params2 = it["p1"], it["p2"]
            q.nparts = it.get("nparts", 2)
        return arr

    def run_batched(self, items, mixed=False, learned=False, tuning=None, vbm3d=False):
        """Denoise many sequences with one CUDA graph (bm4dof_run_batched).
        Returns the per-sequence ratios."""
        arr = self._sequences(items)
        flags = _mixed_flags(mixed) | (LEARNED if learned else 0) | (VBM3D_SEARCH if vbm3d else 0)
        t = None
        if tuning is not None:
            t = Tuning(**tuning) if isinstance(tuning, dict) else tuning
        with self._ordered():
            _check(load().bm4dof_run_batched(self._h, arr, len(items), flags,
                                             C.byref(t) if t is not None else None))
        return [(q.ratios[0], q.ratios[1]) for q in arr]

    def autotune(self, items, sample=16, mixed=False, learned=False, vbm3d=False):
        """(best tuning dict, table of (branches, slot_mb, search_ctas, search_strip,
        gather_depth, ms))."""
        arr = self._sequences(items)
        flags = _mixed_flags(mixed) | (LEARNED if learned else 0) | (VBM3D_SEARCH if vbm3d else 0)
        best = Tuning()
        table = (C.c_float * (6 * 32))()
        rows = C.c_uint()
        with self._ordered():
            _check(load().bm4dof_autotune(self._h, arr, len(items), sample, flags, C.byref(best), table, 32,
                                          C.byref(rows)))
        tab = [tuple(table[6 * i:6 * i + 6]) for i in range(min(rows.value, 32))]
        return best.as_dict(), tab

    def set_gain_network(self, params=None, kappa=0.0):
        """Install the gain network (float blob of GAIN_PARAMS values) for
        learned runs; None runs the learned form without it."""
        if params is None:
            _check(load().bm4dof_set_gain_network(self._h, None, 0, kappa))
            return
        a = np.ascontiguousarray(params, np.float32).ravel()
        _check(load().bm4dof_set_gain_network(self._h, C.c_void_p(a.ctypes.data), a.size, kappa))

    def learned_stats(self):
        """(groups, fallback groups) of the last learned run."""
        g, f = C.c_ulonglong(), C.c_ulonglong()
        _check(load().bm4dof_learned_stats(self._h, C.byref(g), C.byref(f)))
        return g.value, f.value

    def mixed_stats(self):
        """(groups searched through the tensor-core pre-screen, groups of those
        given the exact search, groups kept with an uncertified re-rank) of the
        last mixed-precision run."""
        g, e, u = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
        _check(load().bm4dof_mixed_stats(self._h, C.byref(g), C.byref(e), C.byref(u)))
        return g.value, e.value, u.value

    def gain_samples(self, noisy, basic, fflow, bflow, p2, nparts=2):
        """Training pairs of the gain network for one grey video (CUDA
        tensors (F, 1, H, W)): returns (features [n, 65], targets [n, 64]) as
        CUDA tensors, the groups the filter processes only."""
        import torch
        F, Cc, H, W = noisy.shape
        dev = noisy.device
        L = load()
        n = C.c_size_t()
        cap = 1
        while True:
            feat = torch.empty((cap, 65), dtype=torch.float32, device=dev)
            tgt = torch.empty((cap, 64), dtype=torch.float32, device=dev)
            valid = torch.empty((cap,), dtype=torch.uint8, device=dev)
            ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
            nz, bs = noisy.contiguous(), basic.contiguous()
            with self._ordered():
                code = L.bm4dof_gain_samples(self._h, ptr(nz), ptr(bs), ptr(fflow), ptr(bflow), W, H, F,
                                             C.byref(p2), nparts, DEVICE_POINTERS, ptr(feat), ptr(tgt),
                                             ptr(valid), cap, C.byref(n))
            if code == 1 and n.value > cap:
                cap = n.value
                continue
            _check(code)
            break
        keep = valid[: n.value].bool()
        return feat[: n.value][keep], tgt[: n.value][keep]

    def set_memory_limit(self, nbytes):
        """Cap on the device memory this context holds (0: none)."""
        _check(load().bm4dof_set_memory_limit(self._h, int(nbytes)))

    def processNlBayes(self, noisy, fflow, bflow, params, crop=None, basic=None, mixed=False, vbm3d=False,
                       keep_groups=False):
        """VideoNLB::processNlBayes: the step params.isFirstStep names, over one
        video (numpy (F, C, H, W)) cut from a source as crop (make_crop) says.
        Step 2 reads basic.  Returns (basic, final, groups)."""
        flags = (KEEP_GROUPS if keep_groups else 0) | _mixed_flags(mixed)
        flags |= VBM3D_SEARCH if vbm3d else 0
        noisy = np.ascontiguousarray(noisy, np.float32)
        F, Cc, H, W = noisy.shape
        ff = None if fflow is None else np.ascontiguousarray(fflow, np.float32)
        bf = None if bflow is None else np.ascontiguousarray(bflow, np.float32)
        b = np.zeros_like(noisy) if basic is None else np.array(basic, np.float32, copy=True)
        fin = np.zeros_like(noisy)
        ptr = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
        groups = C.c_uint()
        _check(load().bm4dof_process(self._h, ptr(noisy), ptr(ff), ptr(bf), W, H, Cc, F, ptr(b), ptr(fin),
                                     C.byref(params), None if crop is None else C.byref(crop), flags,
                                     C.byref(groups)))
        return b, fin, groups.value

    @staticmethod
    def tvl1_params(**kw):
        """bm4dof_tvl1_params with the tvl1flow-seq.sh defaults, overridden by kw."""
        p = Tvl1Params()
        load().bm4dof_tvl1_default_params(C.byref(p))
        for k, v in kw.items():
            setattr(p, "lambda_" if k == "lambda" else k, v)
        return p

    def tvl1_pairs(self, I0, I1, params=None):
        """TV-L1 flow of frame pairs (numpy [n, H, W] or [H, W] float32):
        returns [n, 2, H, W] (u, v)."""
        a = np.ascontiguousarray(I0, np.float32)
        b = np.ascontiguousarray(I1, np.float32)
        single = a.ndim == 2
        if single:
            a, b = a[None], b[None]
        n, H, W = a.shape
        uv = np.zeros((n, 2, H, W), np.float32)
        p = params or self.tvl1_params()
        _check(load().bm4dof_tvl1_pairs(self._h, C.c_void_p(a.ctypes.data), C.c_void_p(b.ctypes.data), W, H, n,
                                        C.byref(p), C.c_void_p(uv.ctypes.data), 0))
        return uv[0] if single else uv

    def tvl1_video(self, video, params=None):
        """Forward and backward flows (F, 2, H, W) of a grey video (F, 1, H, W)
        or (F, H, W), in the layout runNlBayes takes."""
        v = np.ascontiguousarray(video, np.float32)
        if v.ndim == 4:
            v = np.ascontiguousarray(v[:, 0])
        F, H, W = v.shape
        ff = np.zeros((F, 2, H, W), np.float32)
        bf = np.zeros((F, 2, H, W), np.float32)
        p = params or self.tvl1_params()
        _check(load().bm4dof_tvl1_video(self._h, C.c_void_p(v.ctypes.data), W, H, F, C.byref(p),
                                        C.c_void_p(ff.ctypes.data), C.c_void_p(bf.ctypes.data), 0))
        return ff, bf

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


def tc_selftest(a, b):
    """D = a @ b.T through tcgen05.mma (bm4dof_tc_selftest): a [128, 64] and
    b [256, 64] float16 CUDA tensors; returns D [128, 256] float32."""
    import torch
    a = a.contiguous()
    b = b.contiguous()
    d = torch.empty((128, 256), dtype=torch.float32, device=a.device)
    stream = torch.cuda.current_stream(a.device).cuda_stream
    _check(load().bm4dof_tc_selftest(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                     C.c_void_p(d.data_ptr()), C.c_void_p(stream)))
    return d


def fp32_mix_rate(device=0):
    """Measured FP32 rate (tera-operations/s, 3 per patch element) of the exact
    search's instruction mix (bm4dof_fp32_mix_rate) and one launch's ms."""
    t, ms = C.c_float(), C.c_float()
    _check(load().bm4dof_fp32_mix_rate(device, C.byref(t), C.byref(ms)))
    return t.value, ms.value


def plan(W, H, F, params, nparts=2, crop=None, process=False):
    """The reference-patch grid (bm4dof_plan, host only): a list of tiles, each
    {"box": (ox, oy, w, h), "xs": [...], "ys": [...], "fs": [...]} with
    tile-local positions."""
    nt, nc = C.c_uint(), C.c_size_t()
    cr = None if crop is None else C.byref(crop)
    _check(load().bm4dof_plan(W, H, F, nparts, C.byref(params), cr, int(process), None, 0, None, 0,
                              C.byref(nt), C.byref(nc)))
    tiles = np.zeros(7 * nt.value, np.int32)
    coords = np.zeros(max(nc.value, 1), np.int32)
    _check(load().bm4dof_plan(W, H, F, nparts, C.byref(params), cr, int(process),
                              C.c_void_p(tiles.ctypes.data), nt.value, C.c_void_p(coords.ctypes.data), nc.value,
                              C.byref(nt), C.byref(nc)))
    out, o = [], 0
    for i in range(nt.value):
        ox, oy, w, h, nx, ny, nf = (int(v) for v in tiles[7 * i:7 * i + 7])
        xs = coords[o:o + nx].tolist(); o += nx
        ys = coords[o:o + ny].tolist(); o += ny
        fs = coords[o:o + nf].tolist(); o += nf
        out.append({"box": (ox, oy, w, h), "xs": xs, "ys": ys, "fs": fs})
    return out


def processNlBayes(noisy, fflow, bflow, params, crop=None, basic=None, **kw):
    """Module-level VideoNLB::processNlBayes on device 0."""
    global _default
    if _default is None:
        _default = Context(0)
    return _default.processNlBayes(noisy, fflow, bflow, params, crop=crop, basic=basic, **kw)


class Trainer:
    """GPU training of the gain network (bm4dof_trainer_*): BF16 forward and
    backward with FP32 accumulation, AdamW on FP32 master weights.  Features
    and targets are CUDA float tensors [n, 65] and [n, 64], n <= batch."""

    def __init__(self, batch=8192, device=0, seed=0):
        self._h = C.c_void_p()
        _check(load().bm4dof_trainer_create(C.byref(self._h), device, batch, seed))
        self.batch = batch
        self.device = device

    def _ordered(self):
        return _stream_order(load().bm4dof_trainer_get_stream, self._h, self.device)

    def close(self):
        if self._h:
            load().bm4dof_trainer_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        a = np.zeros(GAIN_PARAMS, np.float32)
        _check(load().bm4dof_trainer_params(self._h, C.c_void_p(a.ctypes.data), a.size, 0))
        return a

    def set_params(self, a):
        a = np.ascontiguousarray(a, np.float32).ravel()
        _check(load().bm4dof_trainer_params(self._h, C.c_void_p(a.ctypes.data), a.size, 1))

    def state(self):
        """AdamW state: (first moment, second moment, steps taken)."""
        m1, m2 = np.zeros(GAIN_PARAMS, np.float32), np.zeros(GAIN_PARAMS, np.float32)
        steps = C.c_ulonglong()
        _check(load().bm4dof_trainer_state(self._h, C.c_void_p(m1.ctypes.data), C.c_void_p(m2.ctypes.data),
                                           GAIN_PARAMS, C.byref(steps), 0))
        return m1, m2, steps.value

    def set_state(self, m1, m2, steps):
        m1 = np.ascontiguousarray(m1, np.float32).ravel()
        m2 = np.ascontiguousarray(m2, np.float32).ravel()
        n = C.c_ulonglong(int(steps))
        _check(load().bm4dof_trainer_state(self._h, C.c_void_p(m1.ctypes.data), C.c_void_p(m2.ctypes.data),
                                           m1.size, C.byref(n), 1))

    def checkpoint(self, path, meta=None, best=None):
        """Parameters and AdamW state to a host file (save_checkpoint), with
        the caller's run record and best-epoch parameters when given."""
        save_checkpoint(path, self.params(), *self.state(), batch=self.batch, meta=meta, best=best)

    def restore(self, path):
        """Parameters and AdamW state from a file written by checkpoint: the
        next step is the one an uninterrupted run would have taken."""
        ck = load_checkpoint(path)
        self.set_params(ck["params"])
        self.set_state(ck["moment1"], ck["moment2"], ck["steps"])
        return ck

    def grad(self, feat, target):
        g = np.zeros(GAIN_PARAMS, np.float32)
        loss = C.c_float()
        with self._ordered():
            _check(load().bm4dof_trainer_grad(self._h, C.c_void_p(feat.data_ptr()), C.c_void_p(target.data_ptr()),
                                              feat.shape[0], C.c_void_p(g.ctypes.data), C.byref(loss)))
        return g, loss.value

    def step(self, feat, target, lr=1e-3, weight_decay=1e-4, want_loss=True):
        """One AdamW step; returns the batch loss (before the update) when
        want_loss, else None (no host synchronisation)."""
        loss = C.c_float()
        with self._ordered():
            _check(load().bm4dof_trainer_step(self._h, C.c_void_p(feat.data_ptr()), C.c_void_p(target.data_ptr()),
                                              feat.shape[0], lr, weight_decay,
                                              C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def predict(self, feat):
        import torch
        out = torch.empty((feat.shape[0], 64), dtype=torch.float32, device=feat.device)
        with self._ordered():
            _check(load().bm4dof_trainer_predict(self._h, C.c_void_p(feat.data_ptr()), feat.shape[0],
                                                 C.c_void_p(out.data_ptr())))
        return out


CHECKPOINT_VERSION = 2


def save_checkpoint(path, params, moment1, moment2, steps, batch=0, meta=None, best=None):
    """Gain-network training checkpoint: FP32 parameters, AdamW moments (laid
    out like the parameters) and step count in one .npz file, optionally with
    the training run's record (meta: a JSON-serialisable dict) and the
    parameters of its best epoch.  The file is written beside its final name
    and renamed over it, so a reader finds either the previous checkpoint or
    this one, never a mixture or a partial file."""
    arrs = [np.ascontiguousarray(a, np.float32).ravel() for a in (params, moment1, moment2)]
    if best is not None:
        arrs.append(np.ascontiguousarray(best, np.float32).ravel())
    if any(a.size != GAIN_PARAMS for a in arrs):
        raise ValueError(f"checkpoint blobs hold {GAIN_PARAMS} floats each")
    extra = {}
    if meta is not None:
        extra["meta"] = np.array(json.dumps(meta))
    if best is not None:
        extra["best"] = arrs[3]
    path = os.fspath(path)
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        np.savez(f, version=np.array(CHECKPOINT_VERSION), params=arrs[0], moment1=arrs[1], moment2=arrs[2],
                 steps=np.array(int(steps), np.uint64), batch=np.array(int(batch), np.uint64), **extra)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def load_checkpoint(path):
    """A checkpoint as a dict: params, moment1, moment2, steps, batch, and
    meta / best (None when the file holds none)."""
    with np.load(path) as z:
        if int(z["version"]) != CHECKPOINT_VERSION:
            raise ValueError(f"{path}: checkpoint version {int(z['version'])}, expected {CHECKPOINT_VERSION}")
        ck = {k: z[k].copy() for k in ("params", "moment1", "moment2")}
        ck["steps"], ck["batch"] = int(z["steps"]), int(z["batch"])
        ck["meta"] = json.loads(str(z["meta"])) if "meta" in z.files else None
        ck["best"] = z["best"].copy() if "best" in z.files else None
    if any(ck[k].size != GAIN_PARAMS for k in ("params", "moment1", "moment2")) or \
            (ck["best"] is not None and ck["best"].size != GAIN_PARAMS):
        raise ValueError(f"{path}: checkpoint blobs hold {GAIN_PARAMS} floats each")
    return ck


def split_params(a):
    """Views of a parameter blob: (W1[65,256], b1, W2[256,256], b2, W3[256,64], b3)."""
    a = np.asarray(a, np.float32).ravel()
    shapes = [(65, 256), (256,), (256, 256), (256,), (256, 64), (64,)]
    out, o = [], 0
    for sh in shapes:
        n = int(np.prod(sh))
        out.append(a[o:o + n].reshape(sh))
        o += n
    assert o == GAIN_PARAMS
    return out
