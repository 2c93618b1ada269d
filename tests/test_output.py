"""Headless output (blit replacement): PFM round trip and PNG structure."""
import struct
import zlib

import numpy as np

from nbounce_gb300 import output


def test_pfm_round_trip(tmp_path):
    img = np.random.default_rng(0).random((7, 5, 4)).astype(np.float32) * 100
    p = tmp_path / "a.pfm"
    output.write_pfm(p, img)
    back = output.read_pfm(p)
    assert np.array_equal(back, img[..., :3])


def test_png_is_valid_and_bottom_up(tmp_path):
    img = np.zeros((4, 3, 4), np.float32)
    img[0] = 10.0  # texture row 0 = bottom of the picture
    p = tmp_path / "a.png"
    output.write_png(p, img)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (3, 4)
    idat = data[data.index(b"IDAT") + 4:]
    raw = zlib.decompress(idat[: idat.index(b"IEND") - 8])
    rows = [raw[i * (1 + 3 * w) + 1:(i + 1) * (1 + 3 * w)] for i in range(h)]
    assert max(rows[-1]) > 200 and max(rows[0]) == 0
