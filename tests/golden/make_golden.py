"""Writes tests/golden/oracle_golden.npz: regression fixtures of the CPU oracle.

The reference ships no golden vectors; these pin the oracle's own outputs bit for bit
(Sobol table rows, closest hits of a seeded soup, a small image of the 64-sphere scene) so
that a change to the oracle is caught.  The Sobol direction-number fixture next to it is
made by nbounce_gb300/csrc/gen_sobol_directions.py from SciPy.
Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nbounce_gb300 import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    out = {"sobol32": O.sobol_table(32, 17)}
    desc = scenes.soup_scene(2000, seed=21)
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    hf, hu, _ = osc.trace(scenes.incoherent_rays(4000, seed=22))
    out["soup_hits_f"], out["soup_hits_u"] = hf, hu
    sph = scenes.spheres_scene(width=24, height=24)
    osc = O.OracleScene(sph.vertices, sph.indices, sph.primitives(), dedup=True)
    img, rays, _, _ = osc.render(sph.clip_to_world, 24, 24, O.sobol_table(1024, 17), 1, 4, bounces=6,
                                 env=sph.env_color)
    out["spheres24_4spp"], out["spheres24_rays"] = img, np.array(rays)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "oracle_golden.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
