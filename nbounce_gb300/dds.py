"""DDS cube-map ingest for the environment (EnvMap::load, envmap.rs:12-17;
Texture::create_cubemap, texture.rs:89-144).

The reference reads a DDS file whose DX10 header names DXGI BC6H_UF16, forces its array size
to 6 (texture.rs:95-96) and uploads the six layers (+X, -X, +Y, -Y, +Z, -Z, each with its mip
chain) as a cube texture, which the pass samples at mip 0 (pathtracing.wgsl:168).

``EnvMap.from_dds`` hands the file to the library (``nb_env_create_dds``), which parses it and
decodes BC6H on the device.  This module reads and writes the same files from Python:
``read_cube_dds`` returns mip 0 of the six faces as RGBA32F (BC6H_UF16 / BC6H_SF16 through the
library's device decoder, R16G16B16A16_FLOAT / R32G32B32A32_FLOAT directly, also under the
legacy D3DFMT codes 113 / 116 with the cube-map caps bit); ``write_cube_dds`` and
``write_cube_dds_bc6h`` write DX10 cube files.

DDS layout (Microsoft's DDS programming guide): "DDS " magic, a 124-byte DDS_HEADER (size,
flags, height, width, pitch, depth, mip count, 11 reserved words, a 32-byte DDS_PIXELFORMAT,
caps 1-4, reserved), then for FourCC "DX10" a 20-byte DDS_HEADER_DXT10 (dxgiFormat,
resourceDimension, miscFlag - 0x4 for a cube -, arraySize, miscFlags2), then each array
layer's mip chain in turn.
"""
import ctypes as C
import struct

import numpy as np

DXGI_R32G32B32A32_FLOAT = 2
DXGI_R16G16B16A16_FLOAT = 10
DXGI_BC6H_UF16 = 95
DXGI_BC6H_SF16 = 96
_DXGI_NAMES = {DXGI_R32G32B32A32_FLOAT: "R32G32B32A32_FLOAT", DXGI_R16G16B16A16_FLOAT: "R16G16B16A16_FLOAT",
               DXGI_BC6H_UF16: "BC6H_UF16", DXGI_BC6H_SF16: "BC6H_SF16"}
_D3DFMT_A16B16G16R16F = 113
_D3DFMT_A32B32G32R32F = 116
_DDSCAPS2_CUBEMAP = 0x200
_DDS_RESOURCE_MISC_TEXTURECUBE = 0x4
_DDPF_FOURCC = 0x4
_MAX_FACE = 32768


def _bytes(data):
    if isinstance(data, (bytes, bytearray, memoryview)):
        return memoryview(data)
    with open(data, "rb") as f:
        return memoryview(f.read())


def _level_bytes(dxgi, w, h):
    if dxgi in (DXGI_BC6H_UF16, DXGI_BC6H_SF16):
        return ((w + 3) // 4) * ((h + 3) // 4) * 16
    return w * h * (16 if dxgi == DXGI_R32G32B32A32_FLOAT else 8)


def _block_bytes(blocks):
    """The bytes of BC6H blocks given as bytes or as an array of any integer type (its memory
    taken as it is, not converted element by element)."""
    if isinstance(blocks, np.ndarray):
        return np.ascontiguousarray(blocks).reshape(-1).view(np.uint8)
    return np.frombuffer(bytes(blocks), np.uint8)


def parse_cube_dds(data):
    """The format (a DXGI code), face size and mip-0 bytes of the six faces of a cube-map DDS
    file (bytes or a path), accepting what ``nb_env_create_dds`` accepts."""
    buf = _bytes(data)
    if len(buf) < 128 or bytes(buf[:4]) != b"DDS ":
        raise ValueError("not a DDS file")
    (size, flags, height, width, pitch, depth, mips) = struct.unpack_from("<7I", buf, 4)
    if size != 124:
        raise ValueError(f"DDS header size {size} != 124")
    pf_flags, fourcc = struct.unpack_from("<I4s", buf, 80)
    caps2 = struct.unpack_from("<I", buf, 112)[0]
    offset = 128
    if (pf_flags & _DDPF_FOURCC) and fourcc == b"DX10":
        if len(buf) < 148:
            raise ValueError("DDS file truncated in its DX10 header")
        dxgi = struct.unpack_from("<I", buf, 128)[0]
        offset = 148
        if dxgi not in _DXGI_NAMES:
            raise NotImplementedError(f"DDS DXGI format {dxgi} is not supported")
        # six array layers whatever the header says, as texture.rs:95-96 forces them
    elif pf_flags & _DDPF_FOURCC:
        code = struct.unpack("<I", fourcc)[0]
        if code == _D3DFMT_A16B16G16R16F:
            dxgi = DXGI_R16G16B16A16_FLOAT
        elif code == _D3DFMT_A32B32G32R32F:
            dxgi = DXGI_R32G32B32A32_FLOAT
        else:
            raise NotImplementedError(f"DDS FourCC {fourcc!r} is not supported")
        if not caps2 & _DDSCAPS2_CUBEMAP:
            raise ValueError("DDS file is not a cube map")
    else:
        raise NotImplementedError("DDS file without a FourCC pixel format is not supported")
    if width == 0 or width != height or width > _MAX_FACE:
        raise ValueError(f"cube faces must be square, 1 to {_MAX_FACE} texels ({width} x {height})")
    mips = max(1, mips)
    if mips > 32:
        raise ValueError(f"DDS mip count {mips}")
    chain = sum(_level_bytes(dxgi, max(1, width >> m), max(1, height >> m)) for m in range(mips))
    need = offset + 6 * chain
    if len(buf) < need:
        raise ValueError(f"DDS file truncated: {len(buf)} bytes, {need} expected")
    level0 = _level_bytes(dxgi, width, height)
    faces = [bytes(buf[offset + f * chain:offset + f * chain + level0]) for f in range(6)]
    return {"format": dxgi, "format_name": _DXGI_NAMES[dxgi], "size": width, "faces": faces}


def decode_bc6h(blocks, width, height, layers=1, signed=False):
    """BC6H blocks ((layers, ceil(h/4), ceil(w/4), 16) bytes, or the same bytes flat) decoded by
    the library on the device into (layers, height, width, 4) float32 (alpha 1)."""
    from . import _lib as L
    src = _block_bytes(blocks)
    need = ((width + 3) // 4) * ((height + 3) // 4) * layers * 16
    if src.size != need:
        raise ValueError(f"{src.size} bytes of BC6H blocks, {need} expected for {layers} x {width} x {height}")
    out = np.empty((layers, height, width, 4), np.float32)
    L.check(L.lib().nb_bc6h_decode(src.ctypes.data_as(C.c_void_p), int(width), int(height), int(layers),
                                   1 if signed else 0, out.ctypes.data_as(C.c_void_p)))
    return out


def read_cube_dds(data):
    """Mip 0 of the six faces of a cube-map DDS file (bytes or a path) as (6, n, n, 4) float32.
    BC6H files are decoded by the library on the device."""
    d = parse_cube_dds(data)
    n, fmt = d["size"], d["format"]
    if fmt in (DXGI_BC6H_UF16, DXGI_BC6H_SF16):
        return decode_bc6h(b"".join(d["faces"]), n, n, 6, signed=fmt == DXGI_BC6H_SF16)
    dtype = np.float16 if fmt == DXGI_R16G16B16A16_FLOAT else np.float32
    return np.stack([np.frombuffer(f, dtype=dtype).reshape(n, n, 4).astype(np.float32) for f in d["faces"]])


def _dx10_header(n, dxgi, pitch, mips):
    header = bytearray(148)
    header[:4] = b"DDS "
    struct.pack_into("<7I", header, 4, 124, 0x1 | 0x2 | 0x4 | 0x1000 | 0x20000, n, n, pitch, 0, mips)
    struct.pack_into("<2I4s", header, 76, 32, _DDPF_FOURCC, b"DX10")
    struct.pack_into("<2I", header, 108, 0x1000 | 0x8 | 0x400000, _DDSCAPS2_CUBEMAP | 0xFC00)
    struct.pack_into("<5I", header, 128, dxgi, 3, _DDS_RESOURCE_MISC_TEXTURECUBE, 1, 0)
    return header


def _finish(out, path):
    if path is not None:
        with open(path, "wb") as fh:
            fh.write(out)
    return out


def write_cube_dds(faces, path=None, half=True, mips=1):
    """A DX10 cube-map DDS file of (6, n, n, 4) faces (R16G16B16A16_FLOAT or R32G32B32A32_FLOAT;
    mip levels past 0 are box-filtered).  Returns the bytes, also written to path if given."""
    faces = np.asarray(faces, np.float32)
    n = faces.shape[1]
    dtype = np.float16 if half else np.float32
    header = _dx10_header(n, DXGI_R16G16B16A16_FLOAT if half else DXGI_R32G32B32A32_FLOAT,
                          n * 4 * np.dtype(dtype).itemsize, mips)
    body = []
    for f in range(6):
        level = faces[f]
        for m in range(mips):
            body.append(level.astype(dtype).tobytes())
            if level.shape[0] > 1:
                level = level.reshape(level.shape[0] // 2, 2, level.shape[1] // 2, 2, 4).mean(axis=(1, 3))
    return _finish(bytes(header) + b"".join(body), path)


def write_cube_dds_bc6h(blocks, n, signed=False, path=None, mip_blocks=None):
    """A DX10 BC6H_UF16 (or BC6H_SF16) cube-map DDS file from the six faces' mip-0 blocks
    ((6, ceil(n/4), ceil(n/4), 16) bytes).  mip_blocks, if given, lists per face the bytes of
    the further mip levels, written after each face's level 0.  Returns the bytes, also written
    to path if given."""
    b = _block_bytes(blocks).reshape(6, -1)
    per_face = ((n + 3) // 4) ** 2 * 16
    if b.shape[1] != per_face:
        raise ValueError(f"{b.shape[1]} bytes per face, {per_face} expected for n = {n}")
    mips = 1 + (len(mip_blocks[0]) if mip_blocks else 0)
    header = _dx10_header(n, DXGI_BC6H_SF16 if signed else DXGI_BC6H_UF16, per_face, mips)
    body = []
    for f in range(6):
        body.append(b[f].tobytes())
        if mip_blocks:
            body.extend(bytes(x) for x in mip_blocks[f])
    return _finish(bytes(header) + b"".join(body), path)
