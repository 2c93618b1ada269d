"""Headless image output replacing the reference's blit to the swapchain.

The reference shows its RGBA32F accumulation texture with a full-screen triangle
(``src/pathtracing/blit.wgsl:26-38``) whose texture coordinate (0, 0) is the bottom-left of the
screen, so texture row 0 is the bottom row of the picture.  ``write_pfm`` stores the HDR
image losslessly (PFM rows run bottom to top, so row 0 is written first, as displayed);
``write_png`` writes an 8-bit preview (Reinhard tonemap, sRGB-like 1/2.2 gamma) with row 0
at the bottom.
"""
import struct
import zlib

import numpy as np


def write_pfm(path, rgba):
    img = np.asarray(rgba, np.float32)
    h, w = img.shape[:2]
    rgb = np.ascontiguousarray(img[..., :3], dtype="<f4")
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode("ascii"))
        f.write(rgb.tobytes())


def read_pfm(path):
    with open(path, "rb") as f:
        tag = f.readline().strip()
        if tag not in (b"PF", b"Pf"):
            raise ValueError("not a PFM file")
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        ch = 3 if tag == b"PF" else 1
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4", count=w * h * ch)
    return data.reshape(h, w, ch).astype(np.float32)


def tonemap(rgba, exposure=1.0):
    x = np.clip(np.asarray(rgba, np.float32)[..., :3] * exposure, 0.0, None)
    x = x / (1.0 + x)
    return (np.clip(x, 0.0, 1.0) ** (1.0 / 2.2) * 255.0 + 0.5).astype(np.uint8)


def write_png(path, rgba, exposure=1.0):
    rgb = tonemap(rgba, exposure)[::-1]  # row 0 at the bottom, as the blit shows it
    h, w = rgb.shape[:2]
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag, payload):
        return struct.pack(">I", len(payload)) + tag + payload + struct.pack(">I", zlib.crc32(tag + payload) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
