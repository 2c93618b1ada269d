"""DDS cube-map ingest (envmap.rs:12, texture.rs:89-144): header parsing, face order and mip 0,
half and single precision, and the errors for what is not decoded."""
import struct

import numpy as np
import pytest

from nbounce_gb300 import dds, scenes


def faces(n, seed=1):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.0, 8.0, (6, n, n, 4)).astype(np.float32)
    f[..., 3] = 1.0
    return f


@pytest.mark.parametrize("half,mips", [(True, 1), (False, 1), (True, 4), (False, 6)])
def test_roundtrip_returns_mip0_of_each_face(half, mips, tmp_path):
    src = faces(32)
    path = tmp_path / "sky.dds"
    dds.write_cube_dds(src, path, half=half, mips=mips)
    got = dds.read_cube_dds(str(path))
    want = src.astype(np.float16).astype(np.float32) if half else src
    np.testing.assert_array_equal(got, want)
    assert got.shape == (6, 32, 32, 4) and got.dtype == np.float32


def test_face_order_is_the_layer_order():
    src = np.zeros((6, 4, 4, 4), np.float32)
    src[..., 0] = np.arange(6)[:, None, None]
    got = dds.read_cube_dds(dds.write_cube_dds(src, half=False, mips=3))
    np.testing.assert_array_equal(got[:, 0, 0, 0], np.arange(6))


def test_bc6h_and_non_cube_files_are_rejected():
    data = bytearray(dds.write_cube_dds(faces(8), half=True))
    bc6h = bytearray(data)
    struct.pack_into("<I", bc6h, 128, dds.DXGI_BC6H_UF16)
    with pytest.raises(NotImplementedError, match="BC6H_UF16"):
        dds.read_cube_dds(bytes(bc6h))
    flat = bytearray(data)
    struct.pack_into("<I", flat, 112, 0)        # caps2 without the cube bit
    struct.pack_into("<I", flat, 136, 0)        # misc flag without TEXTURECUBE
    with pytest.raises(ValueError, match="not a cube"):
        dds.read_cube_dds(bytes(flat))
    with pytest.raises(ValueError, match="truncated"):
        dds.read_cube_dds(bytes(data[:-16]))
    with pytest.raises(ValueError, match="not a DDS"):
        dds.read_cube_dds(b"PNG" + bytes(200))


def test_sky_through_dds_keeps_the_cube():
    cube = scenes.cube_from_equirect(scenes.sky_envmap(2, 128, 64, sun_radiance=50.0), 16)
    got = dds.read_cube_dds(dds.write_cube_dds(cube, half=False))
    np.testing.assert_array_equal(got, cube)
