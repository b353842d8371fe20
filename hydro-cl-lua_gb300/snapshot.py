"""Snapshots of a solver's state as FITS files, and restarts from them.

hydro-cl-lua saves each solver buffer as a FITS image (GridSolver:saveBuffer,
hydro/solver/gridsolver.lua:1410-1459; GridSolver:save, :1467-1472): the
buffer holds every cell of the grid, ghosts included, with `channels` reals
per cell; the image is (width * depth) x height x channels with the channel
as the slowest axis and, within a channel, x fastest, then z, then y
(getIndex(ch, i, j, k) = i + width * (k + depth * (j + height * ch))).  The
state buffer UBuf has 6 channels: rho, m.x, m.y, m.z, ETotal, ePot.

This module writes the same image as a standard FITS primary array
(BITPIX -64 for doubles, big-endian, 2880-byte records) with NAXIS1 =
width * depth, NAXIS2 = height, NAXIS3 = channels, and keeps the solve's time
in the header (HCTIME) so a run can resume from the file.  `save` / `restore`
work with every precision form of the library: the state goes through the
ghost-inclusive state I/O of the C ABI.
"""
import os
import struct
import zlib

import numpy as np

BLOCK = 2880
CHANNELS = 6


def _card(key, value, comment=""):
    if isinstance(value, bool):
        v = "T" if value else "F"
        s = "%-8s= %20s" % (key, v)
    elif isinstance(value, int):
        s = "%-8s= %20d" % (key, value)
    elif isinstance(value, float):
        s = "%-8s= %20s" % (key, repr(float(value)).upper())
    else:
        s = "%-8s= '%-8s'" % (key, str(value).replace("'", "''"))
    if comment:
        s += " / " + comment
    if len(s) > 80:
        raise ValueError("FITS card too long: %r" % s)
    return s.ljust(80)


def to_image(full, grid):
    """The reference's image order of a ghost-inclusive AoS-6 array.

    full: (cells, 6) in x-fastest cell order; grid: (width, height, depth)
    including ghosts (1 on unused axes).  Returns (channels, height, depth,
    width), i.e. C order of [ch][j][k][i]."""
    w, h, d = grid
    a = np.asarray(full, dtype=np.float64).reshape(d, h, w, CHANNELS)      # [k][j][i][ch]
    return np.ascontiguousarray(np.transpose(a, (3, 1, 0, 2)))            # [ch][j][k][i]


def from_image(img, grid):
    w, h, d = grid
    a = np.asarray(img, dtype=np.float64).reshape(CHANNELS, h, d, w)      # [ch][j][k][i]
    return np.ascontiguousarray(np.transpose(a, (2, 1, 3, 0))).reshape(-1, CHANNELS)


def write_fits(path, img, extra=None):
    """A FITS primary array from img[ch][j][k][i] (float64)."""
    ch, h, d, w = img.shape
    cards = [_card("SIMPLE", True, "conforms to FITS"), _card("BITPIX", -64, "IEEE double"),
             _card("NAXIS", 3), _card("NAXIS1", w * d, "width * depth"), _card("NAXIS2", h, "height"),
             _card("NAXIS3", ch, "channels")]
    for k, v in (extra or {}).items():
        cards.append(_card(k, v))
    cards.append("END".ljust(80))
    header = "".join(cards).encode("ascii")
    header += b" " * (-len(header) % BLOCK)
    data = np.asarray(img, dtype=">f8").tobytes()
    data += b"\0" * (-len(data) % BLOCK)
    with open(path, "wb") as f:
        f.write(header)
        f.write(data)


def read_fits(path):
    """(image [NAXIS3][NAXIS2][NAXIS1] as float64, header dict)."""
    with open(path, "rb") as f:
        raw = f.read()
    hdr = {}
    off = 0
    while True:
        rec = raw[off:off + BLOCK]
        if len(rec) < BLOCK:
            raise ValueError("truncated FITS header")
        off += BLOCK
        done = False
        for i in range(0, BLOCK, 80):
            card = rec[i:i + 80].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] != "= ":
                continue
            val = card[10:].split(" / ")[0].strip()
            if val.startswith("'"):
                hdr[key] = val.strip("'").rstrip()
            elif val in ("T", "F"):
                hdr[key] = val == "T"
            else:
                try:
                    hdr[key] = int(val)
                except ValueError:
                    hdr[key] = float(val.replace("D", "E"))
        if done:
            break
    bitpix = hdr["BITPIX"]
    dtype = {-64: ">f8", -32: ">f4"}[bitpix]
    dims = [hdr["NAXIS%d" % (k + 1)] for k in range(hdr["NAXIS"])]
    n = int(np.prod(dims))
    img = np.frombuffer(raw, dtype=dtype, count=n, offset=off).astype(np.float64)
    return img.reshape(dims[::-1]), hdr


def grid_of(desc):
    """(width, height, depth) of the reference's grid, ghosts included."""
    return tuple(desc.n[k] + 4 if k < desc.dim else 1 for k in range(3))


def save(solver, prefix=None):
    """GridSolver:save for the state buffer: writes <prefix>_UBuf.fits (or
    UBuf.fits) and returns its path."""
    full = solver.getState(withGhosts=True)
    grid = grid_of(solver.desc)
    path = (prefix + "_" if prefix else "") + "UBuf.fits"
    write_fits(path, to_image(full, grid), {"HCTIME": float(solver.t), "HCDIM": int(solver.desc.dim)})
    return path


def restore(solver, path):
    """Loads a UBuf written by `save` (or by the reference) into `solver`,
    which must have the same grid; restores the time when the file has it."""
    img, hdr = read_fits(path)
    grid = grid_of(solver.desc)
    w, h, d = grid
    if img.shape != (CHANNELS, h, w * d):
        raise ValueError("%s holds a %s image; this solver's grid needs %s" % (
            os.path.basename(path), img.shape, (CHANNELS, h, w * d)))
    solver.setState(from_image(img.reshape(CHANNELS, h, d, w), grid), withGhosts=True)
    if "HCTIME" in hdr:
        solver.t = float(hdr["HCTIME"])
    return hdr


def write_png(path, rgba):
    """Writes an RGBA8 image from the library's views (row 0 at the bottom, as
    glReadPixels returns it) as a PNG file, top row first."""
    img = np.ascontiguousarray(np.asarray(rgba, dtype=np.uint8)[::-1])
    h, w, c = img.shape
    if c != 4:
        raise ValueError("expected an RGBA image")
    raw = b"".join(b"\0" + img[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
    return path


def read_png(path):
    """Reads a PNG written by write_png back into the library's row order."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    off, idat, w, h = 8, b"", 0, 0
    while off < len(data):
        n, = struct.unpack(">I", data[off:off + 4])
        tag = data[off + 4:off + 8]
        body = data[off + 8:off + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if depth != 8 or ctype != 6:
                raise ValueError("only 8-bit RGBA PNG files are read")
        elif tag == b"IDAT":
            idat += body
        off += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(h, 1 + 4 * w)
    if rows[:, 0].any():
        raise ValueError("filtered PNG rows are not read")
    return np.ascontiguousarray(rows[:, 1:].reshape(h, w, 4)[::-1])
