"""The CPU oracle's BC6H decoder (oracle/bc6h.cpp): known answers worked out by hand from the
published format, and the texture unit's own decode of seeded blocks of every mode
(tests/golden/bc6h_texunit.npz, made on a GB300 by tests/golden/make_bc6h_texunit.py)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bc6h_texunit.npz")


def pack(fields):
    """A block from (value, bit count) fields laid out from bit 0 upward."""
    v, pos = 0, 0
    for val, n in fields:
        v |= (val & ((1 << n) - 1)) << pos
        pos += n
    assert pos <= 128
    return np.frombuffer(v.to_bytes(16, "little"), np.uint8)


def test_mode11_explicit_endpoints():
    # 10-bit endpoint 1023 unquantises to 0xFFFF and finishes as 0x7BFF (65504); 512 as
    # ((512 << 16) + 0x8000) >> 10 = 32800 -> (32800 * 31) >> 6 = 0x3E0F
    top = pack([(0b00011, 5)] + [(1023, 10)] * 6 + [(0, 63)])
    assert np.all(O.bc6h_decode_blocks(top) == 0x7BFF)
    mid = pack([(0b00011, 5), (512, 10), (0, 10), (0, 10), (0, 10), (0, 10), (0, 10), (0, 63)])
    h = O.bc6h_decode_blocks(mid)[0]
    assert np.all(h[:, 0] == 0x3E0F) and np.all(h[:, 1:] == 0)
    img = O.bc6h_decode(mid, 4, 4)
    assert np.all(img[0, :, :, 0] == np.float32(1.5146484375)) and np.all(img[0, :, :, 3] == 1.0)


def test_mode12_delta_endpoint_and_the_high_base_bit():
    # base 1024 (bit 10 stored after rx), delta -1 -> endpoint 1023; unquantised 32784 / 32752,
    # finished 0x3E07 / 0x3DF8; texel 0 has index 0 (3 bits), the others index 15 (weight 64)
    fields = [(0b00111, 5), (0, 10), (0, 10), (0, 10)]
    for _ in range(3):
        fields += [(0x1FF, 9), (1, 1)]
    fields += [(0, 3)] + [(15, 4)] * 15
    h = O.bc6h_decode_blocks(pack(fields))[0]
    assert np.all(h[0] == 0x3E07) and np.all(h[1:] == 0x3DF8)


def test_reserved_modes_decode_to_zero():
    for mode in (0b10011, 0b10111, 0b11011, 0b11111):
        blk = pack([(mode, 5), ((1 << 123) - 1, 123)])
        assert np.all(O.bc6h_decode_blocks(blk) == 0)
        assert np.all(O.bc6h_decode(blk, 4, 4)[0, :, :, :3] == 0)


def test_signed_finish_keeps_the_sign():
    # mode 11 signed, 10-bit endpoints: red 0x200 is -512 and green 0x1FF is 511, both at or
    # past 2^9 - 1, so they unquantise to -0x7FFF / 0x7FFF and finish as 0x8000 | 0x7BFF / 0x7BFF;
    # blue 0x100 = 256 unquantises to ((256 << 15) + 0x4000) >> 9 = 16416 -> (16416 * 31) >> 5
    blk = pack([(0b00011, 5), (0x200, 10), (0x1FF, 10), (0x100, 10), (0, 10), (0, 10), (0, 10), (0, 63)])
    h = O.bc6h_decode_blocks(blk, signed=True)[0]
    assert h[0, 0] == 0xFBFF and h[0, 1] == 0x7BFF and h[0, 2] == (16416 * 31) >> 5


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="texture-unit fixture not generated")
@pytest.mark.parametrize("fmt", ["uf16", "sf16"])
def test_oracle_matches_the_texture_unit(fmt):
    g = np.load(GOLDEN)
    got = O.bc6h_decode_blocks(g["blocks"], signed=fmt == "sf16")
    want = g[fmt]
    same = np.all(got == want, axis=-1)
    bad = np.argwhere(~same)
    assert bad.size == 0, f"{len(bad)} texels differ, first at block {bad[0][0]}: {got[bad[0][0]]} vs {want[bad[0][0]]}"
    # BC6H has no alpha: CUDA's texture path fills it with 0 (the stored *_alpha), graphics
    # APIs with 1 as the decoders here do; the pass reads the environment's RGB only.
    assert np.all(g[fmt + "_alpha"] == 0.0)


def test_block_arrays_of_any_integer_type_are_read_as_bytes():
    blk = pack([(0b00011, 5), (512, 10), (0, 10), (0, 10), (0, 10), (0, 10), (0, 10), (0, 63)])
    want = O.bc6h_decode_blocks(blk)
    for dt in (np.uint16, np.uint32, np.uint64):
        assert np.array_equal(O.bc6h_decode_blocks(blk.view(dt)), want)
        assert np.array_equal(O.bc6h_decode(blk.view(dt), 4, 4), O.bc6h_decode(blk, 4, 4))
    with pytest.raises(ValueError, match="expected"):
        O.bc6h_decode(blk, 8, 4)
