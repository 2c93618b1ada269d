"""BC6H environments on the GPU: the library's device decoder against the CPU oracle
(bit-exact) and against the texture unit's own BC6H decode (the decoder the reference's
textureSampleLevel uses, pathtracing.wgsl:168); DDS cube maps through nb_env_create_dds
rendering like the oracle with the oracle's decode of the same blocks."""
import importlib.util
import os

import numpy as np
import pytest
import torch

import nbounce_gb300 as nb
from nbounce_gb300 import dds, scenes
from oracle import oracle as O

from test_gpu_render import EXACT_FRAC, REL_MSE, gpu_render, rel_mse

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden_module():
    spec = importlib.util.spec_from_file_location("make_bc6h_texunit",
                                                  os.path.join(HERE, "golden", "make_bc6h_texunit.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def texunit(tmp_path_factory):
    return _golden_module().build_texunit(str(tmp_path_factory.mktemp("texunit")))


def _blocks(seed, n):
    return _golden_module().make_blocks(seed=seed, per_mode=max(1, n // 16), n_random=n - 14 * max(1, n // 16))


@pytest.mark.parametrize("signed", [False, True])
def test_device_decoder_matches_oracle_bit_exact(signed):
    blocks = _blocks(7, 4096)  # 64 x 64 blocks: a 256 x 256 image
    img = dds.decode_bc6h(blocks, 256, 256, 1, signed=signed)
    ref = O.bc6h_decode(blocks, 256, 256, 1, signed=signed)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("signed", [False, True])
def test_device_decoder_matches_texture_unit(texunit, signed):
    blocks = _blocks(11, 2048)
    n = blocks.shape[0]
    hw = texunit(blocks, 4 * n, 4, signed)
    ours = dds.decode_bc6h(blocks, 4 * n, 4, 1, signed=signed)[0]
    same = np.all(hw[:, :, :3].view(np.uint32) == ours[:, :, :3].view(np.uint32), axis=-1)
    bad = np.argwhere(~same)
    assert bad.size == 0, (f"{len(bad)} of {same.size} texels differ; first block {bad[0][1] // 4}: "
                           f"{blocks[bad[0][1] // 4].tolist()} hw {hw[bad[0][0], bad[0][1]]} "
                           f"ours {ours[bad[0][0], bad[0][1]]}")


def test_partial_edge_blocks_and_layers_match_oracle():
    """Sizes off the 4-texel grid decode the covering blocks and keep the texels inside."""
    w, h, layers = 13, 10, 3
    n = ((w + 3) // 4) * ((h + 3) // 4) * layers
    blocks = _blocks(3, n)[:n]
    img = dds.decode_bc6h(blocks, w, h, layers)
    ref = O.bc6h_decode(blocks, w, h, layers)
    assert img.shape == (layers, h, w, 4)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))


def smooth_cube_blocks(n, rng):
    """Mode-11 blocks (two explicit 10-bit endpoints, 4-bit indices) of a sky-like cube map:
    moderate values with a bright patch, so renders stay in a sensible range."""
    nb_ = (n + 3) // 4
    out = np.zeros((6, nb_, nb_, 16), np.uint8)
    for f in range(6):
        for by in range(nb_):
            for bx in range(nb_):
                base = 200 + 40 * f + 3 * (bx + by)
                e0 = [base, base + 20, base + 60]
                e1 = [min(1023, c + int(rng.integers(0, 200))) for c in e0]
                if f == 2 and bx == 1 and by == 1:
                    e1 = [1022, 1000, 900]
                v = 0b00011
                pos = 5
                for c in e0 + e1:
                    v |= c << pos
                    pos += 10
                for t in range(16):
                    bits = 3 if t == 0 else 4
                    v |= int(rng.integers(0, 1 << bits)) << pos
                    pos += bits
                out[f, by, bx] = np.frombuffer(v.to_bytes(16, "little"), np.uint8)
    return out


def test_dds_bc6h_environment_renders_like_oracle():
    """nb_env_create_dds on a BC6H_UF16 cube file (the reference's format): misses sample the
    decoded cube exactly as the oracle samples its own decode of the same blocks."""
    rng = np.random.default_rng(5)
    n = 24
    blocks = smooth_cube_blocks(n, rng)
    data = dds.write_cube_dds_bc6h(blocks, n)
    cube = O.bc6h_decode(blocks, n, n, 6)
    assert np.array_equal(dds.read_cube_dds(data).view(np.uint32), cube.view(np.uint32))
    desc = scenes.spheres_scene(width=40, height=40, spp=2, bounces=4)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    img, _, status, _ = gpu_render(desc, desc.spp, env=nb.EnvMap.from_dds(data))
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env_cube=cube)
    assert status == 0
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE


def test_dds_mip_chain_and_float_formats_give_the_same_environment():
    """Only mip 0 of each face is read, at the per-face stride of the whole chain; RGBA16F and
    RGBA32F files of the decoded faces give the same environment as the BC6H file."""
    rng = np.random.default_rng(9)
    n = 16
    blocks = smooth_cube_blocks(n, rng)
    mips = [[rng.integers(0, 256, size=16 * max(1, (n >> m) // 4) ** 2, dtype=np.uint8).tobytes()
             for m in range(1, 5)] for _ in range(6)]
    plain = dds.read_cube_dds(dds.write_cube_dds_bc6h(blocks, n))
    chained = dds.read_cube_dds(dds.write_cube_dds_bc6h(blocks, n, mip_blocks=mips))
    assert np.array_equal(plain, chained)
    desc = scenes.spheres_scene(width=32, height=32, spp=1, bounces=3)
    imgs = []
    for data in (dds.write_cube_dds_bc6h(blocks, n, mip_blocks=mips), dds.write_cube_dds(plain, half=True),
                 dds.write_cube_dds(plain, half=False)):
        img, _, status, _ = gpu_render(desc, desc.spp, env=nb.EnvMap.from_dds(data))
        assert status == 0
        imgs.append(img)
    assert np.array_equal(imgs[0], imgs[1]) and np.array_equal(imgs[0], imgs[2])


def test_dds_environment_importance_sampling_matches_its_texels():
    """The NEE tables of a DDS environment are built from the decoded texels: the same uniform
    numbers give bit-identical directions and densities as a cube built from the oracle's
    decode of the same blocks."""
    rng = np.random.default_rng(13)
    n = 16
    blocks = smooth_cube_blocks(n, rng)
    data = dds.write_cube_dds_bc6h(blocks, n)
    u = torch.rand(4096, 2, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    outs = []
    for env in (nb.EnvMap.from_dds(data), nb.EnvMap(cube=O.bc6h_decode(blocks, n, n, 6))):
        out = torch.empty(4096, 4, device="cuda")
        env.sample(u, 4096, out)
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
