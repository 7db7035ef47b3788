"""The C++ layer for the reference's callers (include/bm4dof_videonlb.hpp):
VideoNLB's parameter functions and runNlBayes over the C ABI, templates over
the caller's own types.  A small driver (tests/videonlb_layer.cpp) is built
with stand-in types and, where the reference's sources are present, with the
reference's own nlbParams / VideoSize / Video<float>, linked to the
reference's code: there the layer's resolved parameters and the messages it
throws on bad input (nldct.cpp:276-342) are compared with the reference's in
the same process.  On the GPU, a run through the layer equals the library's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import ROOT, video_case

DRIVER = os.path.join(ROOT, "tests", "videonlb_layer.cpp")
LIBDIR = os.path.join(ROOT, "bm4d-of_gb300", "lib")
ORACLE = os.path.join(ROOT, "oracle")

ERRORS = [
    "two channels: VideoNLB::runNlBayes: Wrong number of channels. Must be 1, 3 or 4.",
    "forward flow of the wrong length: VideoNLB::runNlBayes: Wrong size of fwd optical flow.",
    "backward flow of the wrong length: VideoNLB::runNlBayes: Wrong size of bwd optical flow.",
    "forward flow with one channel: VideoNLB::runNlBayes: Wrong size of fwd optical flow.",
    "no step: VideoNLB::runNlBayes: Both patch sizes are zero.",
    "step 2 with a basic of another size: VideoNLB::runNlBayes: sizes of noisy and basic videos don't match",
]


def _compile(out, extra):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    cmd = [cxx, "-std=c++11", "-O1", "-ffp-contract=off", "-w", *extra[0], DRIVER, "-o", str(out), *extra[1],
           "-L" + LIBDIR, "-lbm4dof_gpu", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


@pytest.fixture(scope="module")
def layer(gpulib, tmp_path_factory):
    return _compile(tmp_path_factory.mktemp("layer") / "videonlb_layer", ([], []))


@pytest.fixture(scope="module")
def layer_ref(gpulib, reference, tmp_path_factory):
    import __graft_entry__
    import pyoracle
    root = __graft_entry__.reference_tree()
    if root is None:
        pytest.skip("REF_ROOT (the reference's source tree) not set")
    inc = ["-fopenmp", "-I" + os.path.join(ORACLE, "ref_stubs"), "-I" + os.path.join(root, "src", "core"),
           "-I" + os.path.join(root, "src", "utils"), "-DWITH_REFERENCE_TYPES"]
    libs = [pyoracle.REF_SO, "-Wl,-rpath," + os.path.dirname(pyoracle.REF_SO)]
    return _compile(tmp_path_factory.mktemp("layer_ref") / "videonlb_layer_ref", (inc, libs))


def run(exe, *args):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=120)


def test_layer_header_compiles_without_warnings(gpulib, tmp_path):
    # the header is included into callers' builds: C++11 and warning-free
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    for std in ("-std=c++11", "-std=c++17"):
        r = subprocess.run([cxx, std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", DRIVER],
                           capture_output=True, text=True)
        assert r.returncode == 0, (std, r.stderr)


def test_layer_conversion_round_trip(layer):
    r = run(layer, "roundtrip")
    assert r.returncode == 0 and r.stdout.strip() == "roundtrip ok"


def test_layer_parameters_match_the_c_abi(layer, gpulib):
    r = run(layer, "params")
    assert r.returncode == 0, r.stderr
    cases = [((256, 256, 1, 1), 20.0, 1, 0, 0, 0), ((256, 256, 1, 1), 45.0, 2, 0, 0, 0),
             ((854, 480, 20, 1), 20.0, 1, 0, 0, 0), ((854, 480, 20, 1), 20.0, 2, 21, 4, 16),
             ((64, 48, 8, 3), 30.0, 1, 15, 5, 24), ((64, 48, 8, 3), 10.0, 2, 9, 6, 0),
             ((32, 32, 1, 3), 50.0, 1, 0, 8, 8)]
    want = ""
    for size, sigma, step, wx, px, np_ in cases:
        p = gpulib.initializeNlbParameters(step, sigma, size)
        if wx:
            gpulib.setSizeSearchWindow(p, wx)
        if px:
            gpulib.setSizePatch(p, size, px)
        if np_:
            gpulib.setNSimilarPatches(p, np_)
        want += gpulib.formatNlbParameters(p)
    assert r.stdout == want


def test_layer_errors(layer):
    r = run(layer, "errors")
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == ERRORS


def test_layer_with_the_reference_types(layer_ref, layer):
    # the reference's own types compile against the layer; its parameter
    # functions and its errors agree with the layer's (checked in the driver)
    r = run(layer_ref, "params")
    assert r.returncode == 0, r.stderr
    assert r.stdout == run(layer, "params").stdout
    r = run(layer_ref, "errors")
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == ERRORS


def test_layer_without_a_device(layer, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    noisy = np.zeros((2, 1, 12, 16), np.float32)
    noisy.tofile(tmp_path / "n.raw")
    r = run(layer, "run", 16, 12, 1, 2, 20, 2, tmp_path / "n.raw", tmp_path / "b.raw", tmp_path / "f.raw")
    assert r.returncode == 1 and "bm4dof_create: no CUDA device" in r.stderr


@pytest.mark.gpu
def test_gpu_layer_run_equals_the_library(layer, gpulib, gpuctx, tmp_path):
    W, H, F, sigma = 48, 40, 4, 20.0
    clean, nz, _, _ = video_case(W, H, F, sigma=sigma, seed=23)
    noisy = np.ascontiguousarray(nz, np.float32)           # (F, C, H, W): the reference's planar layout
    noisy.tofile(tmp_path / "n.raw")
    r = run(layer, "run", W, H, 1, F, sigma, 4, tmp_path / "n.raw", tmp_path / "b.raw", tmp_path / "f.raw")
    assert r.returncode == 0, r.stderr
    basic = np.fromfile(tmp_path / "b.raw", np.float32).reshape(noisy.shape)
    final = np.fromfile(tmp_path / "f.raw", np.float32).reshape(noisy.shape)
    size = (W, H, F, 1)
    p1 = gpulib.initializeNlbParameters(1, sigma, size)
    p2 = gpulib.initializeNlbParameters(2, sigma, size)
    b, f, ratios = gpuctx.runNlBayes(noisy, None, None, p1, p2, nparts=4)
    assert np.array_equal(basic, b) and np.array_equal(final, f)
    assert [float(x) for x in r.stdout.split()] == pytest.approx([float(x) for x in ratios], abs=1e-5)


def test_layer_tile_count_follows_openmp(layer):
    # 2 x omp_get_max_threads() as the reference (nldct.cpp:318-323): from
    # OMP_NUM_THREADS when set, else the CPUs the process may run on (libgomp
    # counts its affinity mask, not the online CPUs)
    env = {k: v for k, v in os.environ.items() if k != "OMP_NUM_THREADS"}
    r = subprocess.run([layer, "tiles"], capture_output=True, text=True, env=dict(env, OMP_NUM_THREADS="3"))
    assert r.stdout.strip() == "6"
    r = subprocess.run([layer, "tiles"], capture_output=True, text=True, env=dict(env, OMP_NUM_THREADS="4,2"))
    assert r.stdout.strip() == "8"
    r = subprocess.run([layer, "tiles"], capture_output=True, text=True, env=env)
    assert r.stdout.strip() == str(2 * len(os.sched_getaffinity(0)))
    taskset = shutil.which("taskset")
    if taskset:
        cpu = sorted(os.sched_getaffinity(0))[0]
        r = subprocess.run([taskset, "-c", str(cpu), layer, "tiles"], capture_output=True, text=True, env=env)
        assert r.returncode == 0, r.stderr
        assert r.stdout.strip() == "2"


def test_layer_process_refuses_sizes_it_cannot_read(layer):
    r = run(layer, "process_errors")
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == [
        "flows: bm4dof_process: the flows' size differs from the video's",
        "basic: bm4dof_process: the basic estimate's size differs from the video's",
    ]


@pytest.mark.gpu
def test_gpu_layer_process_equals_the_library(layer, gpulib, gpuctx, tmp_path):
    W, H, F, sigma = 40, 36, 4, 20.0
    clean, nz, _, _ = video_case(W, H, F, sigma=sigma, seed=27)
    noisy = np.ascontiguousarray(nz, np.float32)
    noisy.tofile(tmp_path / "n.raw")
    crop = ((6, 0, 0), (46, 36, 4), (60, 50, 4))    # borders on the left, the right and the bottom
    r = run(layer, "process", W, H, 1, F, sigma, tmp_path / "n.raw", tmp_path / "b.raw", tmp_path / "f.raw",
            *crop[0], *crop[1], *crop[2])
    assert r.returncode == 0, r.stderr
    basic = np.fromfile(tmp_path / "b.raw", np.float32).reshape(noisy.shape)
    final = np.fromfile(tmp_path / "f.raw", np.float32).reshape(noisy.shape)
    size = (W, H, F, 1)
    p1 = gpulib.initializeNlbParameters(1, sigma, size)
    p2 = gpulib.initializeNlbParameters(2, sigma, size)
    c = gpulib.make_crop(crop[0], crop[1], (*crop[2], 1))
    b, _, g1 = gpuctx.processNlBayes(noisy, None, None, p1, c)
    _, f, g2 = gpuctx.processNlBayes(noisy, None, None, p2, c, basic=b)
    assert np.array_equal(basic, b) and np.array_equal(final, f)
    assert [int(x) for x in r.stdout.split()] == [g1, g2]
