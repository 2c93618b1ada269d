"""Makes the binary64 truth images that relMSE is judged against.

Each image is the oracle's binary64 render (oracle/nb_oracle.cpp, precision 64: every path
computed in binary64, samples averaged in binary64) at 16,384 samples per pixel, Sobol-Burley
rows 1..16,384, with the reference's Russian roulette (contribution factor 4):

  spheres_256       the 64-icosphere workload: 256 x 256 full frame, 6 bounces, constant sky
  instanced_1080p   the 1920 x 1080 benchmark frame (16 meshes, 1024 instances, 2048 x 1024 sky,
                    8 bounces): 24 tiles of 32 x 32 pixels, one centred in each cell of a 6 x 4
                    grid (scenes.stratified_tiles)
  instanced_cache   the same scene from the radiance-cache workload's last camera
                    (scenes.cache_camera), same tiles

Usage: python tests/golden/make_truth.py [--threads N] [--spp 16384] [--only NAME ...]
Writes tests/golden/truth_<name>.npz with the image (tiles), the tile list, the samples, the
command, the host's core count, the seconds taken and the scene's fingerprint.  The full set
takes about 15 minutes on 8 x86 cores.
"""
import argparse
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from nbounce_gb300 import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    def spheres():
        d = scenes.spheres_scene(width=256, height=256, spp=16, bounces=6)
        return d, d.clip_to_world, [(0, 0, 256, 256)]

    def instanced():
        d = scenes.instanced_scene()
        return d, d.clip_to_world, scenes.stratified_tiles(d.width, d.height, size=32)

    def instanced_cache():
        d = scenes.instanced_scene()
        return d, scenes.cache_camera(d.width, d.height)[1], scenes.stratified_tiles(d.width, d.height, size=32)

    return {"spheres_256": spheres, "instanced_1080p": instanced, "instanced_cache": instanced_cache}


def make(name, spp, threads):
    desc, c2w, tiles = cases()[name]()
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    sobol = O.sobol_table(spp, 17)
    t0 = time.perf_counter()
    imgs, rays = [], 0
    for (x0, y0, w, h) in tiles:
        img, r, _, _ = osc.render(c2w, desc.width, desc.height, sobol, 1, spp, bounces=desc.bounces,
                                  env=desc.env_color, env_texels=desc.env_texels, region=(x0, y0, w, h),
                                  precision=64, threads=threads)
        imgs.append(img[..., :3].copy())
        rays += r
    secs = time.perf_counter() - t0
    out = os.path.join(HERE, f"truth_{name}.npz")
    fp = scenes.scene_fingerprint(desc)
    np.savez_compressed(out, rgb=np.stack(imgs).astype(np.float32), tiles=np.array(tiles, np.int32), spp=spp,
                        width=desc.width, height=desc.height, bounces=desc.bounces,
                        clip_to_world=np.asarray(c2w, np.float32), rays=rays, seconds=secs, cores=threads,
                        host=platform.machine(), precision=64,
                        command=f"python tests/golden/make_truth.py --only {name} --spp {spp} --threads {threads}",
                        fingerprint=np.array([fp["triangles"], fp["instances"], fp["pos_sum"], fp["l2w_sum"]]))
    print(f"{name}: {len(tiles)} tile(s), {rays} rays in {secs:.0f} s on {threads} threads -> {out}", flush=True)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    p.add_argument("--spp", type=int, default=16384)
    p.add_argument("--only", nargs="*", default=None)
    a = p.parse_args()
    for name in (a.only or list(cases())):
        make(name, a.spp, a.threads)


if __name__ == "__main__":
    main()
