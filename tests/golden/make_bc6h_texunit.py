"""Golden BC6H vectors decoded by the GPU's texture unit (needs a GPU and nvcc).

    python tests/golden/make_bc6h_texunit.py [out.npz]

Writes ``bc6h_texunit.npz`` (default: beside this file): seeded 16-byte BC6H blocks - for each
of the 14 modes a set of random blocks with that mode's bits, plus blocks of fully random bits
(which include the reserved modes) - and the half-float bits of their texels as the texture
unit decodes them, for BC6H_UF16 and BC6H_SF16.  ``build_texunit`` compiles the helper
``bc6h_texunit.cu``; the GPU tests use it to decode fresh blocks.
"""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MODE_VALUES = [(0b00, 2), (0b01, 2), (0b00010, 5), (0b00110, 5), (0b01010, 5), (0b01110, 5), (0b10010, 5),
               (0b10110, 5), (0b11010, 5), (0b11110, 5), (0b00011, 5), (0b00111, 5), (0b01011, 5), (0b01111, 5)]


def build_texunit(out_dir=None):
    """Compiles bc6h_texunit.cu for sm_103a; returns the decode function
    (blocks, width, height, signed) -> (height, width, 4) float32."""
    out_dir = out_dir or tempfile.mkdtemp(prefix="bc6h_texunit_")
    so = os.path.join(out_dir, "libbc6h_texunit.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler", "-fPIC",
                    "-o", so, os.path.join(HERE, "bc6h_texunit.cu")], check=True)
    lib = C.CDLL(so)
    fn = lib.texunit_bc6h_decode
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_char_p, C.c_int]
    fn.restype = C.c_int

    def decode(blocks, width, height, signed=False):
        b = np.ascontiguousarray(blocks, dtype=np.uint8)
        assert b.size == (width // 4) * (height // 4) * 16
        out = np.empty((height, width, 4), np.float32)
        err = C.create_string_buffer(512)
        if fn(b.ctypes.data_as(C.c_void_p), width, height, 1 if signed else 0, out.ctypes.data_as(C.c_void_p),
              err, 512) != 0:
            raise RuntimeError(err.value.decode())
        return out

    return decode


def make_blocks(seed=2024, per_mode=48, n_random=96):
    """(n, 16) uint8 blocks: per_mode random blocks for each mode, then n_random random blocks."""
    rng = np.random.default_rng(seed)
    out = []
    for value, bits in MODE_VALUES:
        b = rng.integers(0, 256, size=(per_mode, 16), dtype=np.uint8)
        mask = (1 << bits) - 1
        b[:, 0] = (b[:, 0] & np.uint8(0xFF ^ mask)) | np.uint8(value)
        out.append(b)
    out.append(rng.integers(0, 256, size=(n_random, 16), dtype=np.uint8))
    return np.concatenate(out)


def texels_to_block_halves(img, n):
    """(4, 4 n, 4) texels of n blocks laid out in a row -> (n, 16, 3) half-float bits."""
    t = img[:, :, :3].reshape(4, n, 4, 3).transpose(1, 0, 2, 3).reshape(n, 16, 3)
    return t.astype(np.float16).view(np.uint16)


def main(path):
    decode = build_texunit()
    blocks = make_blocks()
    n = blocks.shape[0]
    res = {"blocks": blocks}
    for name, signed in (("uf16", False), ("sf16", True)):
        img = decode(blocks, 4 * n, 4, signed)
        res[name] = texels_to_block_halves(img, n)
        res[name + "_alpha"] = img[:, :, 3].copy()
    np.savez_compressed(path, **res)
    print(f"wrote {path}: {n} blocks")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "bc6h_texunit.npz"))
