"""Depth-plane image output on the host: the oracle's TransientImage::save
restatement against the reference's own image code (Image.h, compiled from
its sources), and the PNG writer (decoded here with zlib)."""
import struct
import zlib

import numpy as np
import pytest

from oracle import image_harness, numpy_ref

CASES = [  # (width, height, (out_w, out_h), stride, offset)
    (64, 64, (256, 256), 200, 17),    # confocal depth planes: 64^2 scan, 200 depths
    (16, 16, (64, 64), 5, 4),         # exhaustive: 4 x side
    (7, 5, (13, 9), 3, 1),            # ragged, odd ratios
    (32, 32, (32, 32), 1, 0),         # no resize
    (5, 9, (2, 2), 1, 0),             # downscale to the smallest resized image
]


def _slice(width, height, stride, offset, seed):
    rng = np.random.default_rng(seed)
    n = offset + (width * height - 1) * stride + 1
    s = rng.random(n, dtype=np.float32)
    s[::7] = 0.0
    s[::11] = 1.0
    return s


@pytest.mark.skipif(not image_harness.available(), reason="reference image harness not built")
@pytest.mark.parametrize("w,h,size,stride,offset", CASES)
def test_oracle_matches_reference_image_code(w, h, size, stride, offset):
    s = _slice(w, h, stride, offset, seed=w * 100 + h)
    np.testing.assert_array_equal(numpy_ref.transient_image(s, w, h, size, stride, offset),
                                  image_harness.transient_image(s, w, h, size, stride, offset))


@pytest.mark.skipif(not image_harness.available(), reason="reference image harness not built")
def test_oracle_normalize_matches_reference_on_a_plain_slice():
    s = _slice(24, 20, 1, 0, seed=3) * np.float32(7.5)
    np.testing.assert_array_equal(numpy_ref.transient_image(s, 24, 20, (96, 80), normalize=True),
                                  image_harness.transient_image(s, 24, 20, (96, 80), normalize=True))


def test_resized_alpha_follows_the_reference_rounding():
    """The reference interpolates the alpha channel too; FP32 weights that sum
    just below 1 truncate 255 to 254 at some pixels."""
    img = numpy_ref.transient_image(np.ones(64 * 64, np.float32), 64, 64, (256, 256))
    assert set(np.unique(img[..., 3])) <= {254, 255}
    assert img[0, 0, 3] == 255


def _decode_png(data: bytes) -> np.ndarray:
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == crc
        if typ == b"IHDR":
            w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", body)
            assert (depth, ctype, comp, filt, inter) == (8, 6, 0, 0, 0)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    row = w * 4
    assert len(raw) == h * (row + 1)
    out = np.zeros((h, row), np.uint8)
    for y in range(h):
        f, line = raw[y * (row + 1)], np.frombuffer(raw, np.uint8, row, y * (row + 1) + 1).astype(np.int32)
        prev = out[y - 1].astype(np.int32) if y else np.zeros(row, np.int32)
        if f == 0:
            out[y] = line
        elif f == 1:
            cur = line.copy()
            for i in range(4, row):
                cur[i] = (cur[i] + cur[i - 4]) & 0xFF
            out[y] = cur
        elif f == 2:
            out[y] = (line + prev) & 0xFF
        else:
            raise AssertionError(f"unexpected filter {f}")
    return out.reshape(h, w, 4)


@pytest.mark.parametrize("kind", ["depth_plane", "noise", "flat", "tiny"])
def test_png_writer_round_trip(tmp_path, built, kind):
    from fasterbackprojection_gb300.api import write_png

    rng = np.random.default_rng(5)
    if kind == "depth_plane":
        img = numpy_ref.transient_image(_slice(64, 64, 1, 0, 9), 64, 64, (256, 256))
    elif kind == "noise":
        img = rng.integers(0, 256, (37, 53, 4), dtype=np.uint8)
    elif kind == "flat":
        img = np.full((300, 200, 4), 77, np.uint8)
    else:
        img = np.array([[[1, 2, 3, 4]]], np.uint8)
    p = tmp_path / "x.png"
    write_png(str(p), img)
    data = p.read_bytes()
    np.testing.assert_array_equal(_decode_png(data), img)
    if kind == "flat":
        assert len(data) < img.nbytes // 50  # the LZ77 stage works


def test_png_writer_reports_io_errors(tmp_path, built):
    from fasterbackprojection_gb300 import FbpError
    from fasterbackprojection_gb300.api import write_png

    with pytest.raises(FbpError):
        write_png(str(tmp_path / "missing_dir" / "x.png"), np.zeros((2, 2, 4), np.uint8))


def test_depth_image_size_rule():
    from fasterbackprojection_gb300.api import depth_image_size

    assert depth_image_size(64) == (256, 256)
    assert depth_image_size(100) == (200, 200)
    assert depth_image_size(256) == (256, 256)
    assert depth_image_size(300) == (300, 300)
    assert depth_image_size(16, exhaustive=True) == (64, 64)


def test_png_writer_rejects_oversized_images(tmp_path, built):
    """Above 1 GiB of filtered rows the writer refuses before reading pixels."""
    import ctypes

    from fasterbackprojection_gb300 import _lib

    buf = np.zeros(16, np.uint8)
    rc = _lib.load().fbp_write_png(str(tmp_path / "x.png").encode(), buf.ctypes.data_as(ctypes.c_void_p), 40000,
                                   40000)
    assert rc == _lib.FBP_ERR_UNSUPPORTED
    assert not (tmp_path / "x.png").exists()
