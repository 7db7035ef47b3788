"""Frame files of the command line (bm4d-of_gb300/csrc/frames.cpp), checked on
the CPU through a small converter built from the same source: baseline TIFF in
every sample layout the reference's scripts may hand it (8/16/32-bit integer
and 32-bit float, 1 or 3 samples, interleaved or planar, several strips,
either byte order), the float TIFF it writes, PFM, the grey rule for three
equal channels, and the optical-flow tool's reader (iio_read_image_float:
colour reduced to grey in the file's sample type) and flow writer."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from helpers import ROOT


@pytest.fixture(scope="module")
def convert(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("frames") / "frames_convert"
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-ffp-contract=off", os.path.join(ROOT, "tests", "frames_convert.cpp"),
                        os.path.join(ROOT, "bm4d-of_gb300", "csrc", "frames.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def write_tiff(path, planar, dtype, little=True, interleaved=True, rows_per_strip=None):
    """Minimal baseline TIFF writer for the test: planar (C, H, W) samples."""
    C, H, W = planar.shape
    e = "<" if little else ">"
    dt = np.dtype(dtype).newbyteorder(e)
    data = planar.transpose(1, 2, 0) if interleaved else planar
    rps = rows_per_strip or H
    strips = []
    planes = [data] if interleaved else [data[k] for k in range(C)]
    for pl in planes:
        for y0 in range(0, H, rps):
            strips.append(np.ascontiguousarray(pl[y0:y0 + rps], dtype=dt).tobytes())
    bits = dt.itemsize * 8
    fmt = 3 if np.dtype(dtype).kind == "f" else 1
    entries = [(256, 4, [W]), (257, 4, [H]), (258, 3, [bits] * C), (259, 3, [1]),
               (262, 3, [2 if C == 3 else 1]), (273, 4, None), (277, 3, [C]), (278, 4, [rps]),
               (279, 4, [len(s) for s in strips]), (284, 3, [1 if interleaved else 2]), (339, 3, [fmt] * C)]
    head = 8
    ifd_size = 2 + 12 * len(entries) + 4
    extra = bytearray()
    extra_base = head + ifd_size
    data_base = extra_base + 4096
    offs, o = [], data_base
    for s in strips:
        offs.append(o)
        o += len(s)
    entries[5] = (273, 4, offs)
    ifd = struct.pack(e + "H", len(entries))
    for tag, typ, vals in entries:
        sz = 2 if typ == 3 else 4
        raw = b"".join(struct.pack(e + ("H" if typ == 3 else "I"), v) for v in vals)
        if len(raw) <= 4:
            ifd += struct.pack(e + "HHI", tag, typ, len(vals)) + raw.ljust(4, b"\0")
        else:
            ifd += struct.pack(e + "HHII", tag, typ, len(vals), extra_base + len(extra))
            extra += raw
    ifd += struct.pack(e + "I", 0)
    assert len(extra) <= 4096
    with open(path, "wb") as f:
        f.write((b"II" if little else b"MM") + struct.pack(e + "HI", 42, head))
        f.write(ifd)
        f.write(bytes(extra).ljust(4096, b"\0"))
        for s in strips:
            f.write(s)


def read_pfm(path):
    with open(path, "rb") as f:
        tag = f.readline().strip()
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        c = 3 if tag == b"PF" else 1
        a = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4").reshape(h, w, c)[::-1]
    return np.ascontiguousarray(a.transpose(2, 0, 1))


def read_float_tiff(path):
    """The float TIFF the command line writes: little endian, interleaved, one strip."""
    b = open(path, "rb").read()
    assert b[:4] == b"II*\0"
    ifd = struct.unpack_from("<I", b, 4)[0]
    n = struct.unpack_from("<H", b, ifd)[0]
    tags = {}
    for i in range(n):
        tag, typ, cnt, val = struct.unpack_from("<HHII", b, ifd + 2 + 12 * i)
        if typ == 3 and cnt == 1:
            val &= 0xFFFF
        tags[tag] = (typ, cnt, val)
    W, H, C = tags[256][2], tags[257][2], tags[277][2]
    assert tags[259][2] == 1 and tags[284][2] == 1
    off = tags[273][2]
    return np.frombuffer(b, "<f4", count=W * H * C, offset=off).reshape(H, W, C).transpose(2, 0, 1)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.float32])
@pytest.mark.parametrize("little", [True, False])
@pytest.mark.parametrize("channels,interleaved", [(1, True), (3, True), (3, False)])
def test_tiff_read(convert, tmp_path, dtype, little, channels, interleaved):
    rng = np.random.default_rng(1)
    hi = 255 if dtype == np.uint8 else 4000
    img = rng.integers(0, hi, size=(channels, 13, 17)).astype(dtype)
    if dtype == np.float32:
        img = (img + rng.uniform(-0.5, 0.5, size=img.shape)).astype(np.float32)
    src, dst = tmp_path / "a.tif", tmp_path / "a.pfm"
    write_tiff(src, img, dtype, little=little, interleaved=interleaved, rows_per_strip=5)
    r = subprocess.run([convert, str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == ["17", "13", str(channels)]
    assert np.array_equal(read_pfm(dst), img.astype(np.float32))


@pytest.mark.parametrize("channels", [1, 3, 4])
def test_float_tiff_written_and_read_back(convert, tmp_path, channels):
    rng = np.random.default_rng(2)
    img = rng.normal(100, 60, size=(channels, 9, 11)).astype(np.float32)
    a, b, c = tmp_path / "a.tif", tmp_path / "b.tif", tmp_path / "c.tif"
    write_tiff(a, img, np.float32)
    assert subprocess.run([convert, str(a), str(b)]).returncode == 0      # our writer
    assert np.array_equal(read_float_tiff(b), img)
    assert subprocess.run([convert, str(b), str(c)]).returncode == 0      # our reader of our writer
    assert open(b, "rb").read() == open(c, "rb").read()


def test_equal_channels_read_as_grey(convert, tmp_path):
    g = np.arange(35, dtype=np.float32).reshape(1, 5, 7)
    src, dst = tmp_path / "rgb.tif", tmp_path / "g.pfm"
    write_tiff(src, np.repeat(g, 3, axis=0), np.float32)
    r = subprocess.run([convert, str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split() == ["7", "5", "1"]
    assert np.array_equal(read_pfm(dst), g)


def test_rejects_compressed_and_missing(convert, tmp_path):
    img = np.zeros((1, 4, 4), np.float32)
    src = tmp_path / "z.tif"
    write_tiff(src, img, np.float32)
    b = bytearray(open(src, "rb").read())
    n = struct.unpack_from("<H", b, 8)[0]
    for i in range(n):
        if struct.unpack_from("<H", b, 10 + 12 * i)[0] == 259:
            struct.pack_into("<H", b, 10 + 12 * i + 8, 5)    # LZW
    open(src, "wb").write(bytes(b))
    assert subprocess.run([convert, str(src), str(tmp_path / "o.pfm")]).returncode == 3
    assert subprocess.run([convert, str(tmp_path / "missing.tif"), str(tmp_path / "o.pfm")]).returncode == 3


def iio_grey(planar, dtype):
    """iio_hacky_uncolorize(a) (lib/iio/iio.c:935-1006): .299 r + .587 g + .114 b
    in double, stored in the sample type (integers truncate), then float."""
    r, g, b = (planar[k].astype(np.float64) for k in range(3))
    return ((.299 * r + .587 * g) + .114 * b).astype(dtype).astype(np.float32)


@pytest.mark.parametrize("dtype,channels", [(np.uint8, 3), (np.uint16, 3), (np.float32, 3),
                                            (np.uint8, 4), (np.float32, 4)])
def test_flow_tool_reads_colour_as_grey(convert, tmp_path, dtype, channels):
    rng = np.random.default_rng(3)
    hi = 256 if dtype == np.uint8 else 4000
    img = rng.integers(0, hi, size=(channels, 11, 15)).astype(dtype)
    img[:3, 0, :4] = hi - 1                      # white: the sum of the weights rounds below 1
    if dtype == np.float32:
        img = (img + rng.uniform(-0.5, 0.5, size=img.shape)).astype(np.float32)
    src, dst = tmp_path / "c.tif", tmp_path / "g.pfm"
    write_tiff(src, img, dtype, interleaved=channels == 3)
    r = subprocess.run([convert, "-grey", str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["15", "11", "1"]
    want = iio_grey(img, dtype)
    assert np.array_equal(read_pfm(dst)[0], want)
    if dtype != np.float32:
        # truncation, not rounding: some pixels land one below the rounded value
        exact = .299 * img[0].astype(np.float64) + .587 * img[1] + .114 * img[2]
        assert np.all(want <= np.round(exact)) and np.any(want < np.round(exact))


def test_flow_tool_reader_keeps_grey_and_refuses_the_rest(convert, tmp_path):
    g = np.arange(20, dtype=np.float32).reshape(1, 4, 5) * 3.5
    src, dst = tmp_path / "g.tif", tmp_path / "g.pfm"
    write_tiff(src, g, np.float32)
    assert subprocess.run([convert, "-grey", str(src), str(dst)], capture_output=True).returncode == 0
    assert np.array_equal(read_pfm(dst), g)
    for dtype, channels, why in [(np.uint32, 3, "uncolorize type not supported"),
                                 (np.uint16, 4, "uncolorize type not supported"),
                                 (np.float32, 2, "non-scalarizable image")]:
        write_tiff(src, np.ones((channels, 4, 5), dtype), dtype)
        r = subprocess.run([convert, "-grey", str(src), str(dst)], capture_output=True, text=True)
        assert r.returncode == 3 and why in r.stderr, (dtype, channels, r.stderr)
    r = subprocess.run([convert, "-grey", str(tmp_path / "missing.pfm"), str(dst)], capture_output=True, text=True)
    assert r.returncode == 3 and "could not read image" in r.stderr


def test_flow_written_as_flo_or_tiff(convert, tmp_path):
    rng = np.random.default_rng(4)
    uv = rng.normal(0, 3, size=(2, 6, 9)).astype(np.float32)
    src = tmp_path / "in.flo"
    with open(src, "wb") as f:
        f.write(struct.pack("<fii", 202021.25, 9, 6))
        f.write(np.ascontiguousarray(uv.transpose(1, 2, 0), "<f4").tobytes())
    for name in ["out.flo", "out.other"]:        # any name but .tif/.tiff is .flo
        dst = tmp_path / name
        assert subprocess.run([convert, "-flow", str(src), str(dst)], capture_output=True).returncode == 0
        assert open(dst, "rb").read() == open(src, "rb").read()
    dst = tmp_path / "out.tif"
    assert subprocess.run([convert, "-flow", str(src), str(dst)], capture_output=True).returncode == 0
    assert np.array_equal(read_float_tiff(dst), uv)


def test_corrupt_files_are_refused(convert, tmp_path):
    # host-side fault injection: truncated data, a wrong magic number and
    # headers that promise more samples than the file holds are read errors,
    # never an allocation of the promised size or a crash
    dst = str(tmp_path / "o.pfm")
    cases = {
        "short.flo": struct.pack("<fii", 202021.25, 4, 3) + bytes(4 * 2 * 11),
        "magic.flo": struct.pack("<fii", 1.0, 4, 3) + bytes(4 * 2 * 12),
        "huge.flo": struct.pack("<fii", 202021.25, 1 << 30, 1 << 30) + bytes(64),
        "short.pfm": b"Pf\n4 3\n-1.0\n" + bytes(4 * 11),
        "huge.pfm": b"PF\n1073741824 1073741824\n-1.0\n" + bytes(64),
        "empty.pfm": b"",
    }
    for name, data in cases.items():
        (tmp_path / name).write_bytes(data)
        r = subprocess.run([convert, str(tmp_path / name), dst], capture_output=True, text=True)
        assert r.returncode == 3, (name, r.returncode, r.stderr)
    # a TIFF whose width and height promise far more samples than its strip
    src = tmp_path / "huge.tif"
    write_tiff(src, np.zeros((1, 4, 4), np.float32), np.float32)
    b = bytearray(open(src, "rb").read())
    n = struct.unpack_from("<H", b, 8)[0]
    for i in range(n):
        tag = struct.unpack_from("<H", b, 10 + 12 * i)[0]
        if tag in (256, 257):
            struct.pack_into("<I", b, 10 + 12 * i + 8, 1 << 30)
    open(src, "wb").write(bytes(b))
    r = subprocess.run([convert, str(src), dst], capture_output=True, text=True)
    assert r.returncode == 3, r.stderr
