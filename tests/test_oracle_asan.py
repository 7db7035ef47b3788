"""The oracle restatement under AddressSanitizer and UBSan: every mode it
restates (colour, tiles, no flow, order invariance, the paste trick, the
predictive search) runs on small videos without a memory error.  Test
infrastructure checking test infrastructure: the GPU library is not involved."""
import os
import shutil
import subprocess

import pytest

from helpers import ROOT


def test_oracle_is_clean_under_sanitizers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "asan_check"
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-ffp-contract=off", os.path.join(ROOT, "oracle", "asan_check.cpp"),
           os.path.join(ROOT, "oracle", "bm4dof_oracle.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("sanitizer runtime not available: " + r.stderr[-200:])
    assert r.returncode == 0, r.stderr[-2000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert r.stdout.count("rc 0") == 8, r.stdout
