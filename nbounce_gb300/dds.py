"""DDS cube-map ingest for the environment (EnvMap::load, envmap.rs:12; Texture::create_cubemap,
texture.rs:89-144).

The reference reads a DDS file with a DX10 header holding a BC6H_UF16 cube map and uploads the
six faces (array layers +X, -X, +Y, -Y, +Z, -Z, mip chain after each face) as a cube texture.
This reader returns mip 0 of each face as RGBA32F, the layout ``EnvMap(cube=...)`` takes, for
uncompressed half- and single-precision RGBA files (DXGI R16G16B16A16_FLOAT / R32G32B32A32_FLOAT,
or the legacy D3DFMT codes 113 / 116).  Block-compressed BC6H data is not decoded here: such a
file raises NotImplementedError naming its format, to be converted to RGBA16F / RGBA32F first.

DDS layout (Microsoft's DDS programming guide): "DDS " magic, a 124-byte DDS_HEADER (size,
flags, height, width, pitch, depth, mip count, 11 reserved words, a 32-byte DDS_PIXELFORMAT,
caps 1-4, reserved), then for FourCC "DX10" a 20-byte DDS_HEADER_DXT10 (dxgiFormat,
resourceDimension, miscFlag - 0x4 for a cube -, arraySize, miscFlags2).
"""
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


def read_cube_dds(data):
    """Mip 0 of the six faces of a cube-map DDS file (bytes or a path) as (6, n, n, 4) float32."""
    if not isinstance(data, (bytes, bytearray, memoryview)):
        with open(data, "rb") as f:
            data = f.read()
    buf = memoryview(data)
    if len(buf) < 128 or bytes(buf[:4]) != b"DDS ":
        raise ValueError("not a DDS file")
    (size, flags, height, width, pitch, depth, mips) = struct.unpack_from("<7I", buf, 4)
    if size != 124:
        raise ValueError(f"DDS header size {size} != 124")
    pf_size, pf_flags, fourcc = struct.unpack_from("<2I4s", buf, 76)
    caps2 = struct.unpack_from("<I", buf, 112)[0]
    offset = 128
    cube = bool(caps2 & _DDSCAPS2_CUBEMAP)
    if (pf_flags & _DDPF_FOURCC) and fourcc == b"DX10":
        dxgi, dim, misc, array_size, _ = struct.unpack_from("<5I", buf, 128)
        offset = 148
        cube = cube or bool(misc & _DDS_RESOURCE_MISC_TEXTURECUBE)
        if dxgi in (DXGI_BC6H_UF16, DXGI_BC6H_SF16):
            raise NotImplementedError(f"DDS format {_DXGI_NAMES[dxgi]} (block-compressed) is not decoded; "
                                      "convert the cube map to R16G16B16A16_FLOAT or R32G32B32A32_FLOAT")
        if dxgi == DXGI_R16G16B16A16_FLOAT:
            dtype = np.float16
        elif dxgi == DXGI_R32G32B32A32_FLOAT:
            dtype = np.float32
        else:
            raise NotImplementedError(f"DDS DXGI format {dxgi} is not supported")
    elif pf_flags & _DDPF_FOURCC:
        code = struct.unpack("<I", fourcc)[0]
        if code == _D3DFMT_A16B16G16R16F:
            dtype = np.float16
        elif code == _D3DFMT_A32B32G32R32F:
            dtype = np.float32
        else:
            raise NotImplementedError(f"DDS FourCC {fourcc!r} is not supported")
    else:
        raise NotImplementedError("uncompressed DDS without a float FourCC is not supported")
    if not cube:
        raise ValueError("DDS file is not a cube map")
    if width != height:
        raise ValueError(f"cube faces must be square ({width} x {height})")
    mips = max(1, mips)
    item = np.dtype(dtype).itemsize * 4
    chain = sum(max(1, width >> m) * max(1, height >> m) for m in range(mips)) * item
    need = offset + 6 * chain
    if len(buf) < need:
        raise ValueError(f"DDS file truncated: {len(buf)} bytes, {need} expected")
    faces = np.empty((6, height, width, 4), np.float32)
    for f in range(6):
        start = offset + f * chain
        faces[f] = np.frombuffer(buf[start:start + width * height * item], dtype=dtype).reshape(height, width, 4)
    return faces


def write_cube_dds(faces, path=None, half=True, mips=1):
    """A DX10 cube-map DDS file of (6, n, n, 4) faces (R16G16B16A16_FLOAT or R32G32B32A32_FLOAT;
    mip levels past 0 are box-filtered).  Returns the bytes, also written to path if given."""
    faces = np.asarray(faces, np.float32)
    n = faces.shape[1]
    dtype = np.float16 if half else np.float32
    header = bytearray(148)
    header[:4] = b"DDS "
    struct.pack_into("<7I", header, 4, 124, 0x1 | 0x2 | 0x4 | 0x1000 | 0x20000, n, n,
                     n * 4 * np.dtype(dtype).itemsize, 0, mips)
    struct.pack_into("<2I4s", header, 76, 32, _DDPF_FOURCC, b"DX10")
    struct.pack_into("<2I", header, 108, 0x1000 | 0x8 | 0x400000, _DDSCAPS2_CUBEMAP | 0xFC00)
    struct.pack_into("<5I", header, 128, DXGI_R16G16B16A16_FLOAT if half else DXGI_R32G32B32A32_FLOAT, 3,
                     _DDS_RESOURCE_MISC_TEXTURECUBE, 1, 0)
    body = []
    for f in range(6):
        level = faces[f]
        for m in range(mips):
            body.append(level.astype(dtype).tobytes())
            if level.shape[0] > 1:
                level = level.reshape(level.shape[0] // 2, 2, level.shape[1] // 2, 2, 4).mean(axis=(1, 3))
    out = bytes(header) + b"".join(body)
    if path is not None:
        with open(path, "wb") as fh:
            fh.write(out)
    return out
