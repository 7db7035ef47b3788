"""ctypes bindings of the CPU oracle (libbm4dof_oracle.so) and of the reference
built from its own sources (_ref/libbm4dof_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libbm4dof_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libbm4dof_ref.so")
# the reference built with its VBM3D_SEARCH switch (predictive patch search)
REF_VBM3D_SO = os.path.join(HERE, "_ref", "libbm4dof_ref_vbm3d.so")
VBM3D_SEARCH = 0x10   # BM4DOF_VBM3D_SEARCH of include/bm4dof.h


class Params(C.Structure):
    """Layout of bm4dof_params (include/bm4dof.h), a mirror of VideoNLB::nlbParams."""
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
    """Layout of bm4dof_crop (include/bm4dof.h): the fields of
    VideoUtils::CropPosition that processNlBayes reads."""
    _fields_ = [("origin_x", C.c_int), ("origin_y", C.c_int), ("origin_t", C.c_int),
                ("ending_x", C.c_int), ("ending_y", C.c_int), ("ending_t", C.c_int),
                ("source_sz", VideoSize)]


def make_crop(origin, ending, source):
    """origin/ending (x, y, t), source (width, height, frames, channels)."""
    return Crop(*origin, *ending, VideoSize(*source))


def _process(fn, noisy, fflow, bflow, prm, crop, basic, *extra):
    """Shared by Oracle.processNlBayes and Reference.processNlBayes: one step of
    processNlBayes; returns (basic, final, groups)."""
    noisy = np.ascontiguousarray(noisy, np.float32)
    F, Cc, H, W = noisy.shape
    fflow = None if fflow is None else np.ascontiguousarray(fflow, np.float32)
    bflow = None if bflow is None else np.ascontiguousarray(bflow, np.float32)
    b = np.zeros_like(noisy) if basic is None else np.array(basic, np.float32, copy=True)
    fin = np.zeros_like(noisy)
    groups = C.c_uint()
    err = C.create_string_buffer(512)
    rc = fn(_fp(noisy), _fp(fflow), _fp(bflow), W, H, Cc, F, _fp(b), _fp(fin), C.byref(prm),
            None if crop is None else C.byref(crop), *extra, C.byref(groups), err, 512)
    if rc:
        raise RuntimeError(err.value.decode())
    return b, fin, groups.value


class Trace(C.Structure):
    _fields_ = [("cap", C.c_uint), ("stride", C.c_uint),
                ("step", C.POINTER(C.c_uint)), ("tile", C.POINTER(C.c_uint)),
                ("ref", C.POINTER(C.c_uint)), ("nsimp", C.POINTER(C.c_uint)),
                ("index", C.POINTER(C.c_uint)), ("count", C.c_uint)]


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def ref_root() -> str | None:
    """The reference's source tree: the REF_ROOT environment variable (no
    default), or None when it is unset or holds no reference sources."""
    root = os.environ.get("REF_ROOT")
    return root if root and os.path.isfile(os.path.join(root, "src", "core", "nldct.cpp")) else None


def build(ref_root_dir: str | None = None) -> None:
    """Compile the oracle, and the reference when its source tree is given
    (argument or REF_ROOT)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    root = ref_root_dir or ref_root()
    if root and os.path.isfile(os.path.join(root, "src", "core", "nldct.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={root}"], check=True)


class _Lib:
    prefix = ""

    def __init__(self, path):
        self.lib = C.CDLL(path)
        p = self.prefix
        L = self.lib
        for name in ("initialize_params",):
            f = getattr(L, p + name)
            f.argtypes = [C.POINTER(Params), C.c_uint, C.c_float, C.POINTER(VideoSize), C.c_int]
            f.restype = None
        getattr(L, p + "set_size_search_window").argtypes = [C.POINTER(Params), C.c_uint]
        getattr(L, p + "set_size_patch").argtypes = [C.POINTER(Params), C.POINTER(VideoSize), C.c_uint]
        getattr(L, p + "set_n_similar_patches").argtypes = [C.POINTER(Params), C.c_uint]
        getattr(L, p + "format_params").argtypes = [C.POINTER(Params), C.c_char_p, C.c_size_t]
        getattr(L, p + "format_params").restype = C.c_int

    # -- parameter resolution mirrors VideoNLB's setters -------------------
    def initializeNlbParameters(self, step, sigma, size, verbose=False, betaMean=0.0):
        prm = Params()
        prm.betaMean = betaMean
        vs = VideoSize(*size)
        getattr(self.lib, self.prefix + "initialize_params")(C.byref(prm), step, sigma, C.byref(vs), int(verbose))
        return prm

    def setSizeSearchWindow(self, prm, wx):
        getattr(self.lib, self.prefix + "set_size_search_window")(C.byref(prm), wx)

    def setSizePatch(self, prm, size, px):
        vs = VideoSize(*size)
        getattr(self.lib, self.prefix + "set_size_patch")(C.byref(prm), C.byref(vs), px)

    def setNSimilarPatches(self, prm, n):
        getattr(self.lib, self.prefix + "set_n_similar_patches")(C.byref(prm), n)

    def formatNlbParameters(self, prm):
        buf = C.create_string_buffer(4096)
        getattr(self.lib, self.prefix + "format_params")(C.byref(prm), buf, 4096)
        return buf.value.decode()


class Oracle(_Lib):
    prefix = "oracle_"

    def __init__(self, path=ORACLE_SO):
        super().__init__(path)
        L = self.lib
        L.oracle_run.restype = C.c_int
        L.oracle_run.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint] * 4 + [C.POINTER(C.c_float)] * 2 + \
            [C.POINTER(Params)] * 2 + [C.c_uint, C.c_uint, C.POINTER(C.c_float), C.POINTER(Trace), C.c_char_p, C.c_size_t]
        L.oracle_run_ex.restype = C.c_int
        L.oracle_run_ex.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint] * 4 + [C.POINTER(C.c_float)] * 2 + \
            [C.POINTER(Params)] * 2 + [C.c_uint] * 3 + [C.POINTER(C.c_float), C.POINTER(Trace), C.c_char_p, C.c_size_t]
        L.oracle_basis.argtypes = [C.c_int, C.c_uint, C.c_uint, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oracle_window.argtypes = [C.c_int, C.c_uint, C.c_uint, C.POINTER(C.c_float)]
        L.oracle_tile_crops.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_int, C.POINTER(C.c_int)]
        L.oracle_tile_crops.restype = C.c_int
        L.oracle_determine_factor.argtypes = [C.c_uint, C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
        L.oracle_color_transform.argtypes = [C.POINTER(C.c_float), C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_int]
        L.oracle_process.restype = C.c_int
        L.oracle_process.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint] * 4 + [C.POINTER(C.c_float)] * 2 + \
            [C.POINTER(Params), C.POINTER(Crop), C.c_uint, C.POINTER(C.c_uint), C.c_char_p, C.c_size_t]

    def processNlBayes(self, noisy, fflow, bflow, prm, crop=None, basic=None, vbm3d=False):
        """VideoNLB::processNlBayes: the step prm.isFirstStep names, over one
        video cut from a source as crop says.  Returns (basic, final, groups)."""
        return _process(self.lib.oracle_process, noisy, fflow, bflow, prm, crop, basic,
                        VBM3D_SEARCH if vbm3d else 0)

    def runNlBayes(self, noisy, fflow, bflow, p1, p2, basic=None, nparts=2, nthreads=1,
                   trace_cap=0, trace_stride=16, vbm3d=False):
        """noisy: (F, C, H, W) float32.  Returns (basic, final, ratios[, trace]).
        vbm3d: the predictive search of the reference's VBM3D_SEARCH build."""
        noisy = np.ascontiguousarray(noisy, np.float32)
        F, Cc, H, W = noisy.shape
        fflow = None if fflow is None else np.ascontiguousarray(fflow, np.float32)
        bflow = None if bflow is None else np.ascontiguousarray(bflow, np.float32)
        b = np.zeros_like(noisy) if basic is None else np.array(basic, np.float32, copy=True)
        fin = np.zeros_like(noisy)
        ratios = (C.c_float * 2)()
        err = C.create_string_buffer(512)
        tr = None
        arrays = None
        if trace_cap:
            arrays = {k: np.zeros(trace_cap, np.uint32) for k in ("step", "tile", "ref", "nsimp")}
            arrays["index"] = np.zeros(trace_cap * trace_stride, np.uint32)
            up = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint))
            tr = Trace(trace_cap, trace_stride, up(arrays["step"]), up(arrays["tile"]), up(arrays["ref"]),
                       up(arrays["nsimp"]), up(arrays["index"]), 0)
        rc = self.lib.oracle_run_ex(_fp(noisy), _fp(fflow), _fp(bflow), W, H, Cc, F, _fp(b), _fp(fin),
                                    C.byref(p1), C.byref(p2), nparts, nthreads, VBM3D_SEARCH if vbm3d else 0,
                                    ratios, C.byref(tr) if tr is not None else None, err, 512)
        if rc:
            raise RuntimeError(err.value.decode())
        out = (b, fin, (ratios[0], ratios[1]))
        if tr is not None:
            n = min(tr.count, trace_cap)
            t = {k: v[:n] for k, v in arrays.items() if k != "index"}
            t["index"] = arrays["index"][: n * trace_stride].reshape(n, trace_stride)
            t["count"] = tr.count
            out = out + (t,)
        return out

    def basis(self, transform, px, pt):
        n = px * px * pt
        b = np.zeros(n * n, np.float32)
        bi = np.zeros(n * n, np.float32)
        if self.lib.oracle_basis(transform, px, pt, _fp(b), _fp(bi)):
            raise ValueError("bior1.5 needs px == 8")
        return b.reshape(n, n), bi.reshape(n, n)

    def window(self, agg, px, pt):
        w = np.zeros(px * px * pt, np.float32)
        self.lib.oracle_window(int(agg), px, pt, _fp(w))
        return w

    def tile_crops(self, W, H, nparts, boundary):
        boxes = np.zeros(4 * nparts, np.int32)
        n = self.lib.oracle_tile_crops(W, H, nparts, boundary, boxes.ctypes.data_as(C.POINTER(C.c_int)))
        return boxes[: 4 * n].reshape(n, 4)

    def determine_factor(self, n):
        a, b = C.c_uint(), C.c_uint()
        self.lib.oracle_determine_factor(n, C.byref(a), C.byref(b))
        return a.value, b.value

    def color_transform(self, v, forward):
        v = np.array(v, np.float32, copy=True)
        F, Cc, H, W = v.shape
        self.lib.oracle_color_transform(_fp(v), W, H, Cc, F, int(forward))
        return v


class Reference(_Lib):
    """The reference's own VideoNLB code, compiled from its sources."""
    prefix = "ref_"

    def __init__(self, path=REF_SO):
        super().__init__(path)
        L = self.lib
        L.ref_run.restype = C.c_int
        L.ref_run.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint] * 4 + [C.POINTER(C.c_float)] * 2 + \
            [C.POINTER(Params)] * 2 + [C.c_uint, C.POINTER(C.c_float), C.c_char_p, C.c_size_t]
        L.ref_search.restype = C.c_uint
        L.ref_search.argtypes = [C.c_uint] + [C.POINTER(C.c_float)] * 4 + [C.c_uint] * 4 + \
            [C.POINTER(Params), C.c_uint, C.POINTER(C.c_uint)]
        L.ref_process.restype = C.c_int
        L.ref_process.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint] * 4 + [C.POINTER(C.c_float)] * 2 + \
            [C.POINTER(Params), C.POINTER(Crop), C.POINTER(C.c_uint), C.c_char_p, C.c_size_t]

    def processNlBayes(self, noisy, fflow, bflow, prm, crop=None, basic=None):
        """The reference's own VideoNLB::processNlBayes.  Returns (basic, final, groups)."""
        return _process(self.lib.ref_process, noisy, fflow, bflow, prm, crop, basic)

    @staticmethod
    def available(path=REF_SO):
        return os.path.isfile(path)

    def runNlBayes(self, noisy, fflow, bflow, p1, p2, basic=None, nthreads=1):
        noisy = np.ascontiguousarray(noisy, np.float32)
        F, Cc, H, W = noisy.shape
        fflow = None if fflow is None else np.ascontiguousarray(fflow, np.float32)
        bflow = None if bflow is None else np.ascontiguousarray(bflow, np.float32)
        b = np.zeros_like(noisy) if basic is None else np.array(basic, np.float32, copy=True)
        fin = np.zeros_like(noisy)
        ratios = (C.c_float * 2)()
        err = C.create_string_buffer(512)
        rc = self.lib.ref_run(_fp(noisy), _fp(fflow), _fp(bflow), W, H, Cc, F, _fp(b), _fp(fin),
                              C.byref(p1), C.byref(p2), nthreads, ratios, err, 512)
        if rc:
            raise RuntimeError(err.value.decode())
        return b, fin, (ratios[0], ratios[1])

    def search(self, step, noisy, basic, fflow, bflow, prm, pidx, cap=64):
        noisy = np.ascontiguousarray(noisy, np.float32)
        F, Cc, H, W = noisy.shape
        idx = np.zeros(cap, np.uint32)
        n = self.lib.ref_search(step, _fp(noisy), _fp(None if basic is None else np.ascontiguousarray(basic, np.float32)),
                                _fp(None if fflow is None else np.ascontiguousarray(fflow, np.float32)),
                                _fp(None if bflow is None else np.ascontiguousarray(bflow, np.float32)),
                                W, H, Cc, F, C.byref(prm), pidx, idx.ctypes.data_as(C.POINTER(C.c_uint)))
        return idx[:n].copy()
