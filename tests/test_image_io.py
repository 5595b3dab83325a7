"""Image output (dl_image_write, host only): PNG as the reference's
Bitmap::savePNG (sRGB, x255, clamp, truncation), uncompressed OpenEXR with
float R, G, B as Bitmap::saveEXR, PFM.  Each file is parsed back here with
an independent reader and compared with the image written."""
import struct
import zlib

import numpy as np
import pytest

from drawlab_gb300 import abi, api


def sample_image(h=37, w=53, seed=0):
    rng = np.random.default_rng(seed)
    img = rng.uniform(0.0, 1.3, (h, w, 3)).astype(np.float32)
    img[0, 0] = (0.0, 0.001, 0.0031308)      # the linear segment and its end
    img[0, 1] = (-0.5, 2.0, np.nan)            # clamped low, clamped high, NaN
    img[0, 2] = (1.0, 0.5, 1e-8)
    return img


def expected_png_bytes(img):
    """Color3f::toSRGB (include/core/bitmap/color.h:76-87) and the clamp /
    truncation of Bitmap::savePNG, in float32."""
    v = img.astype(np.float32)
    with np.errstate(invalid="ignore"):
        lin = np.float32(12.92) * v
        powed = np.float32(1.055) * np.power(np.maximum(v, np.float32(0)), np.float32(1.0 / 2.4)).astype(
            np.float32) - np.float32(0.055)
        s = np.where(v <= np.float32(0.0031308), lin, powed).astype(np.float32)
        x = np.float32(255) * s
        x = np.where(np.isnan(x), 0, np.clip(x, 0, 255))
    return x.astype(np.uint8)


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF, typ
        chunks.append((typ, body))
        pos += 12 + n
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 2, 0, 0, 0)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def read_exr(path):
    data = open(path, "rb").read()
    magic, version = struct.unpack("<II", data[:8])
    assert magic == 20000630 and version == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        name = data[pos:e].decode()
        e2 = data.index(b"\0", e + 1)
        typ = data[e + 1:e2].decode()
        (size,) = struct.unpack("<I", data[e2 + 1:e2 + 5])
        attrs[name] = (typ, data[e2 + 5:e2 + 5 + size])
        pos = e2 + 5 + size
    pos += 1
    for k in ("channels", "compression", "dataWindow", "displayWindow", "lineOrder", "pixelAspectRatio",
              "screenWindowCenter", "screenWindowWidth"):
        assert k in attrs, k
    assert attrs["compression"][1] == b"\0"
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack("<%dQ" % h, data[pos:pos + 8 * h])
    out = np.empty((h, w, 3), np.float32)
    for y, off in enumerate(offsets):
        ly, size = struct.unpack("<ii", data[off:off + 8])
        assert ly == y and size == 12 * w
        line = np.frombuffer(data[off + 8:off + 8 + size], "<f4").reshape(3, w)  # B, G, R
        out[y] = line[::-1].T
    return out


def read_pfm(path):
    data = open(path, "rb").read()
    head = data.split(b"\n", 3)
    assert head[0] == b"PF"
    w, h = map(int, head[1].split())
    assert float(head[2]) < 0
    return np.frombuffer(head[3], "<f4").reshape(h, w, 3)[::-1]


def test_png_matches_the_reference_conversion(tmp_path):
    img = sample_image()
    api.write_image(tmp_path / "a.png", img)
    got = read_png(tmp_path / "a.png").astype(np.int32)
    want = expected_png_bytes(img).astype(np.int32)
    # float pow may differ by an ulp from numpy's: a byte at most, rarely
    assert np.abs(got - want).max() <= 1
    assert np.mean(got == want) > 0.999
    # clamped low, clamped high, NaN -> 0; 1.0 -> 254: (1 + 0.055) - 0.055
    # rounds below 1 in float and the cast truncates, as in the reference
    assert tuple(got[0, 1]) == (0, 255, 0) and tuple(got[0, 2][:2]) == (254, 187)


def test_png_spans_several_deflate_blocks(tmp_path):
    img = sample_image(h=200, w=160, seed=3)   # > 64 KiB of scanlines
    api.write_image(tmp_path / "b.png", img)
    assert read_png(tmp_path / "b.png").shape == (200, 160, 3)


def test_exr_and_pfm_round_trip_exactly(tmp_path):
    img = sample_image()
    api.write_image(tmp_path / "a.exr", img)
    api.write_image(tmp_path / "a.pfm", img)
    np.testing.assert_array_equal(read_exr(tmp_path / "a.exr"), img)
    np.testing.assert_array_equal(read_pfm(tmp_path / "a.pfm"), img)


def test_image_write_errors(tmp_path):
    img = sample_image(4, 4)
    with pytest.raises(api.DrawlabError) as e:
        api.write_image(tmp_path / "missing_dir" / "a.png", img)
    assert e.value.status == abi.DL_ERR_IO
    with pytest.raises(ValueError):
        api.write_image(tmp_path / "a.bmp", img)
    with pytest.raises(api.DrawlabError) as e:
        api.write_image(tmp_path / "a.png", img, fmt=7)
    assert e.value.status == abi.DL_ERR_INVALID_ARG
