"""FITS snapshots in the reference's buffer image layout (host only)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "hydro-cl-lua_gb300"))

import snapshot  # noqa: E402


def _coded(grid):
    """A ghost-inclusive AoS-6 array whose values encode (ch, i, j, k)."""
    w, h, d = grid
    k, j, i = np.meshgrid(np.arange(d), np.arange(h), np.arange(w), indexing="ij")
    full = np.zeros((d, h, w, 6))
    for ch in range(6):
        full[..., ch] = ch * 1e6 + i + 100 * j + 10000 * k
    return full.reshape(-1, 6)


def test_image_order_is_the_references():
    """getIndex(ch, i, j, k) = i + width * (k + depth * (j + height * ch))
    (gridsolver.lua:1431) is the flat position of (ch, i, j, k) in the image."""
    grid = (7, 5, 3)
    w, h, d = grid
    img = snapshot.to_image(_coded(grid), grid).reshape(-1)
    for ch, i, j, k in ((0, 0, 0, 0), (2, 6, 1, 2), (5, 3, 4, 1), (1, 1, 0, 2)):
        assert img[i + w * (k + d * (j + h * ch))] == ch * 1e6 + i + 100 * j + 10000 * k
    np.testing.assert_array_equal(snapshot.from_image(snapshot.to_image(_coded(grid), grid), grid), _coded(grid))


def test_fits_round_trip_and_header(tmp_path):
    grid = (12, 9, 1)
    full = _coded(grid) + np.pi
    path = str(tmp_path / "UBuf.fits")
    snapshot.write_fits(path, snapshot.to_image(full, grid), {"HCTIME": 0.125, "HCDIM": 2})
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0
    assert raw[:30] == b"SIMPLE  =                    T"
    img, hdr = snapshot.read_fits(path)
    assert (hdr["BITPIX"], hdr["NAXIS"], hdr["NAXIS1"], hdr["NAXIS2"], hdr["NAXIS3"]) == (-64, 3, 12, 9, 6)
    assert hdr["HCTIME"] == 0.125 and hdr["HCDIM"] == 2
    np.testing.assert_array_equal(snapshot.from_image(img.reshape(6, 9, 1, 12), grid), full)
    # big-endian doubles right after the header block
    first = np.frombuffer(raw, dtype=">f8", count=1, offset=2880)[0]
    assert first == full[0, 0]


def test_png_round_trip(tmp_path):
    img = np.random.default_rng(3).integers(0, 256, size=(5, 7, 4), dtype=np.uint8)
    p = snapshot.write_png(str(tmp_path / "v.png"), img)
    with open(p, "rb") as f:
        assert f.read(8) == b"\x89PNG\r\n\x1a\n"
    np.testing.assert_array_equal(snapshot.read_png(p), img)
