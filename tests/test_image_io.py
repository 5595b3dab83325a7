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


# ------------------------------------------------------------ reading
def png_bytes(pixels, ctype, filters, palette=None, level=9):
    """A PNG made here (Python's zlib: dynamic / fixed Huffman blocks) with
    the given per-row filter types applied to `pixels` (h, w, channels uint8)."""
    h, w = pixels.shape[:2]
    ch = pixels.shape[2]
    raw = bytearray()
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        cur = pixels[y].reshape(-1).astype(np.int32)
        f = filters[y % len(filters)]
        out = np.empty_like(cur)
        for i in range(len(cur)):
            a = cur[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[i] = (cur[i] - pred) & 0xFF
        raw += bytes([f]) + out.astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if palette is not None:
        data += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    z = zlib.compress(bytes(raw), level)
    data += chunk(b"IDAT", z[: len(z) // 2]) + chunk(b"IDAT", z[len(z) // 2:])   # split over two chunks
    return data + chunk(b"IEND", b"")


@pytest.mark.parametrize("ctype,ch", [(2, 3), (6, 4), (0, 1), (4, 2)])
def test_png_reader_decodes_every_filter(tmp_path, ctype, ch):
    rng = np.random.default_rng(ctype)
    h, w = 23, 31
    px = rng.integers(0, 256, (h, w, ch)).astype(np.uint8)
    px[5:15, 3:20] = 200                     # runs: back-references in the deflate stream
    for level in (0, 1, 9):                  # stored, fixed and dynamic Huffman blocks
        p = tmp_path / ("t%d_%d.png" % (ctype, level))
        p.write_bytes(png_bytes(px, ctype, [0, 1, 2, 3, 4], level=level))
        img = api.read_image(p)
        want = px[..., :3] if ch >= 3 else np.repeat(px[..., :1], 3, axis=2)
        np.testing.assert_array_equal(img, want.astype(np.float32) / np.float32(255))


def test_png_reader_palette_and_own_writer(tmp_path):
    rng = np.random.default_rng(4)
    pal = rng.integers(0, 256, (16, 3))
    idx = rng.integers(0, 16, (9, 12, 1)).astype(np.uint8)
    (tmp_path / "p.png").write_bytes(png_bytes(idx, 3, [4, 2], palette=pal))
    np.testing.assert_array_equal(api.read_image(tmp_path / "p.png"), pal[idx[..., 0]].astype(np.float32) / 255)
    img = sample_image()
    api.write_image(tmp_path / "own.png", img)
    np.testing.assert_array_equal(api.read_image(tmp_path / "own.png"),
                                  expected_png_bytes(img).astype(np.float32) / np.float32(255))


def test_pfm_reader_round_trip_and_errors(tmp_path):
    img = sample_image()
    api.write_image(tmp_path / "a.pfm", img)
    np.testing.assert_array_equal(api.read_image(tmp_path / "a.pfm"), img)
    (tmp_path / "bad.png").write_bytes(b"\x89PNG\r\n\x1a\n" + b"\0" * 20)
    with pytest.raises(api.DrawlabError) as e:
        api.read_image(tmp_path / "bad.png")
    assert e.value.status == abi.DL_ERR_PARSE
    with pytest.raises(api.DrawlabError) as e:
        api.read_image(tmp_path / "a.jpg")
    assert e.value.status == abi.DL_ERR_UNSUPPORTED
