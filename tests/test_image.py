"""Image files of a frame (PPM, PNG, PFM) and the oracle's supersampling
postprocess, on the CPU."""
import struct
import zlib

import numpy as np

import vrg


def _frame(rng, h=37, w=53):
    bgra = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    bgra[..., 3] = 255
    return bgra


def test_ppm_round_trip(vrglib, tmp_path):
    img = _frame(np.random.default_rng(1))
    p = tmp_path / "f.ppm"
    vrg.write_image(str(p), img)
    data = p.read_bytes()
    head, rest = data.split(b"\n", 3)[:3], data.split(b"\n", 3)[3]
    assert head[0] == b"P6" and head[1] == b"53 37" and head[2] == b"255"
    rgb = np.frombuffer(rest, np.uint8).reshape(37, 53, 3)
    assert np.array_equal(rgb, img[..., 2::-1])


def test_png_round_trip(vrglib, tmp_path):
    img = _frame(np.random.default_rng(2), h=300, w=257)  # several stored deflate blocks
    p = tmp_path / "f.png"
    vrg.write_image(str(p), img)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    off, idat, w, h = 8, b"", None, None
    while off < len(data):
        (n,) = struct.unpack(">I", data[off:off + 4])
        typ = data[off + 4:off + 8]
        body = data[off + 8:off + 8 + n]
        (crc,) = struct.unpack(">I", data[off + 8 + n:off + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
            assert body[8:] == bytes([8, 2, 0, 0, 0])
        elif typ == b"IDAT":
            idat += body
        off += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 3 * w)
    assert (raw[:, 0] == 0).all()
    assert np.array_equal(raw[:, 1:].reshape(h, w, 3), img[..., 2::-1])


def test_pfm_round_trip(vrglib, tmp_path):
    rgb = np.random.default_rng(3).normal(size=(19, 23, 3)).astype(np.float32)
    p = tmp_path / "f.pfm"
    vrg.write_image(str(p), rgb)
    data = p.read_bytes()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"PF" and parts[1] == b"23 19" and parts[2] == b"-1.0"
    got = np.frombuffer(parts[3], "<f4").reshape(19, 23, 3)[::-1]
    assert np.array_equal(got.view(np.uint32), rgb.view(np.uint32))


def test_write_rejects_bad_arguments(vrglib, tmp_path):
    lib = vrg.load_library()
    img = np.zeros((4, 4, 4), np.uint8)
    assert lib.vrg_image_write_ppm(str(tmp_path / "x.ppm").encode(), vrg._ptr(img), 0, 4) == vrg.ERR_INVALID_ARGUMENT
    assert lib.vrg_image_write_png(b"/nonexistent-dir/x.png", vrg._ptr(img), 4, 4) == vrg.ERR_INVALID_ARGUMENT


def test_oracle_postprocess_scaled_matches_restatement(orc):
    """postprocess.rs:39-88: rows outer, columns inner, summed from 0 in f32,
    divided by float(s*s), u8(bgr * 255) saturating."""
    rng = np.random.default_rng(4)
    for s in (1, 2, 3):
        view = (rng.random((6 * s, 10 * s, 3)) * 1.3 - 0.1).astype(np.float32)
        img, out = orc.postprocess_scaled(view, s)
        c = np.zeros((6, 10, 3), np.float32)
        for sy in range(s):
            for sx in range(s):
                c = (c + view[sy::s, sx::s]).astype(np.float32)
        c = (c / np.float32(s * s)).astype(np.float32)
        assert np.array_equal(out.view(np.uint32), c.view(np.uint32))
        v = c * np.float32(255.0)
        u8 = np.where(v > 0, np.minimum(v, 255.0), 0).astype(np.int32).astype(np.uint8)
        assert np.array_equal(img[..., 0], u8[..., 2]) and np.array_equal(img[..., 2], u8[..., 0])
        assert (img[..., 3] == 255).all()
