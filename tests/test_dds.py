"""DDS cube-map ingest (envmap.rs:12, texture.rs:89-144): header parsing, face order and mip 0,
half and single precision, BC6H files, and the errors for malformed files - in Python and in
the library's own parser (nb_env_create_dds), which rejects them without a GPU."""
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


def legacy_cube(src, cube_bit=True):
    """A legacy (non-DX10) RGBA16F cube file: D3DFMT 113 as the FourCC."""
    n = src.shape[1]
    header = bytearray(128)
    header[:4] = b"DDS "
    struct.pack_into("<7I", header, 4, 124, 0x1 | 0x2 | 0x4 | 0x1000, n, n, n * 8, 0, 1)
    struct.pack_into("<2II", header, 76, 32, 0x4, 113)
    struct.pack_into("<2I", header, 108, 0x1000 | 0x8, (0x200 | 0xFC00) if cube_bit else 0)
    return bytes(header) + src.astype(np.float16).tobytes()


def test_dx10_files_are_six_layers_whatever_the_cube_flags_say():
    """texture.rs:95-96 forces the array size of the reference's DX10 file to 6."""
    src = faces(8)
    flat = bytearray(dds.write_cube_dds(src, half=False))
    struct.pack_into("<I", flat, 112, 0)        # caps2 without the cube bit
    struct.pack_into("<I", flat, 136, 0)        # misc flag without TEXTURECUBE
    struct.pack_into("<I", flat, 140, 1)        # array size 1
    np.testing.assert_array_equal(dds.read_cube_dds(bytes(flat)), src)


def test_legacy_fourcc_files_need_the_cube_bit():
    src = faces(4)
    np.testing.assert_array_equal(dds.read_cube_dds(legacy_cube(src)), src.astype(np.float16).astype(np.float32))
    with pytest.raises(ValueError, match="not a cube"):
        dds.read_cube_dds(legacy_cube(src, cube_bit=False))


def malformed_files():
    data = bytearray(dds.write_cube_dds(faces(8), half=True))
    unsupported = bytearray(data)
    struct.pack_into("<I", unsupported, 128, 28)  # R8G8B8A8_UNORM
    wide = bytearray(data)
    struct.pack_into("<I", wide, 16, 16)          # width 16, height 8
    return {"truncated": bytes(data[:-16]), "not a DDS": b"PNG" + bytes(200),
            "unsupported": bytes(unsupported), "square": bytes(wide),
            "legacy flat": legacy_cube(faces(4), cube_bit=False), "short": b"DDS " + bytes(60)}


def test_malformed_files_are_rejected():
    bad = malformed_files()
    with pytest.raises(ValueError, match="truncated"):
        dds.read_cube_dds(bad["truncated"])
    with pytest.raises(ValueError, match="not a DDS"):
        dds.read_cube_dds(bad["not a DDS"])
    with pytest.raises(NotImplementedError, match="DXGI format 28"):
        dds.read_cube_dds(bad["unsupported"])
    with pytest.raises(ValueError, match="square"):
        dds.read_cube_dds(bad["square"])


def test_library_rejects_malformed_files_before_touching_the_device():
    """nb_env_create_dds parses the file first: every malformed file is NB_ERR_INVALID_ARG,
    with or without a GPU; a well-formed one gets as far as the device check."""
    import ctypes as C

    from nbounce_gb300 import _lib as L
    lib = L.lib()
    for name, data in malformed_files().items():
        h = C.c_void_p()
        assert lib.nb_env_create_dds(data, len(data), C.byref(h)) == L.NB_ERR_INVALID_ARG, name
        assert not h.value
    h = C.c_void_p()
    assert lib.nb_env_create_dds(None, 0, C.byref(h)) == L.NB_ERR_INVALID_ARG
    good = dds.write_cube_dds_bc6h(np.zeros((6, 2, 2, 16), np.uint8), 8)
    st = lib.nb_env_create_dds(good, len(good), C.byref(h))
    assert st in (L.NB_OK, L.NB_ERR_NO_DEVICE), st
    if st == L.NB_OK:
        lib.nb_env_destroy(h)


@pytest.mark.parametrize("n,mips", [(16, 1), (16, 5), (10, 3), (4, 1)])
def test_bc6h_files_give_mip0_blocks_of_each_face(n, mips):
    rng = np.random.default_rng(n * 10 + mips)
    nb_ = (n + 3) // 4
    blocks = rng.integers(0, 256, size=(6, nb_, nb_, 16), dtype=np.uint8)
    extra = [[rng.integers(0, 256, size=16 * (((max(1, n >> m)) + 3) // 4) ** 2, dtype=np.uint8).tobytes()
              for m in range(1, mips)] for _ in range(6)] if mips > 1 else None
    data = dds.write_cube_dds_bc6h(blocks, n, signed=(n == 10), mip_blocks=extra)
    d = dds.parse_cube_dds(data)
    assert d["size"] == n and d["format_name"] == ("BC6H_SF16" if n == 10 else "BC6H_UF16")
    for f in range(6):
        assert d["faces"][f] == blocks[f].tobytes()


def test_sky_through_dds_keeps_the_cube():
    cube = scenes.cube_from_equirect(scenes.sky_envmap(2, 128, 64, sun_radiance=50.0), 16)
    got = dds.read_cube_dds(dds.write_cube_dds(cube, half=False))
    np.testing.assert_array_equal(got, cube)


def test_bc6h_writer_takes_block_arrays_of_any_integer_type():
    rng = np.random.default_rng(3)
    blocks = rng.integers(0, 256, size=(6, 2, 2, 16), dtype=np.uint8)
    want = dds.write_cube_dds_bc6h(blocks, 8)
    assert dds.write_cube_dds_bc6h(blocks.view(np.uint32), 8) == want
    assert dds.write_cube_dds_bc6h(blocks.view(np.uint64).reshape(6, -1), 8) == want


def test_bc6h_decode_rejects_bad_arguments_before_touching_the_device():
    import ctypes as C

    from nbounce_gb300 import _lib as L
    lib = L.lib()
    blk = np.zeros(16, np.uint8)
    out = np.zeros(64, np.float32)
    p_in, p_out = blk.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)
    assert lib.nb_bc6h_decode(p_in, 4, 4, 1, 2, p_out) == L.NB_ERR_INVALID_ARG          # is_signed
    assert lib.nb_bc6h_decode(None, 4, 4, 1, 0, p_out) == L.NB_ERR_INVALID_ARG          # NULL blocks
    assert lib.nb_bc6h_decode(p_in, 70000, 4, 1, 0, p_out) == L.NB_ERR_INVALID_ARG      # width
    assert lib.nb_bc6h_decode(p_in, 4, 4, 1 << 20, 0, p_out) == L.NB_ERR_INVALID_ARG    # layers
    assert lib.nb_bc6h_decode(p_in, 0, 4, 1, 0, p_out) == L.NB_OK                       # nothing to do
