"""Cube-map environment (NB_ENV_CUBE): the oracle's lookup, pinned against an independent
numpy statement of the standard cube-map face table (scenes.cube_directions).

The reference samples a cube texture at mip 0 with a linear clamp-to-edge sampler
(pathtracing.wgsl:168, texture.rs:89-144); the faces are its layer order +X, -X, +Y, -Y, +Z, -Z.
"""
import numpy as np

from nbounce_gb300 import scenes
from oracle import oracle as O


def index_faces(n):
    faces = np.ones((6, n, n, 4), np.float32)
    f, y, x = np.meshgrid(np.arange(6), np.arange(n), np.arange(n), indexing="ij")
    faces[..., 0], faces[..., 1], faces[..., 2] = f, y, x
    return faces


def test_texel_centres_return_their_texel():
    for n in (1, 4, 7, 16):
        faces = index_faces(n)
        d = scenes.cube_directions(n).reshape(-1, 3)
        for precision in (32, 64):
            out = O.env_lookup(d, cube=faces, precision=precision)
            np.testing.assert_allclose(out, faces[..., :3].reshape(-1, 3), atol=1e-4)


def test_axes_hit_face_centres_and_ties_go_to_x_then_y():
    n = 4
    faces = index_faces(n)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    out = O.env_lookup(axes, cube=faces)
    np.testing.assert_array_equal(out[:, 0], np.arange(6))
    np.testing.assert_array_equal(out[:, 1:], np.full((6, 2), 1.5, np.float32))
    ties = np.array([[1, 1, 0], [-1, 0, 1], [0, 1, 1], [0, -1, -1], [1, 1, 1], [-2, 2, -2]], np.float32)
    np.testing.assert_array_equal(O.env_lookup(ties, cube=faces)[:, 0], [0, 1, 2, 3, 0, 1])


def test_face_orientation_follows_the_cube_table():
    """On +X, s = -z / x and t = -y / x: +z moves toward column 0, +y toward row 0; on +Y,
    s = x / y and t = z / y; on -Z, s = -x / |z| and t = -y / |z|."""
    n = 8
    faces = index_faces(n)
    probe = np.array([[1, 0, 0.9], [1, 0.9, 0], [0.9, 1, 0], [0, 1, 0.9], [0.9, 0, -1], [0, -0.9, -1]], np.float32)
    out = O.env_lookup(probe, cube=faces)
    np.testing.assert_array_equal(out[:, 0], [0, 0, 2, 2, 5, 5])
    assert out[0, 2] < 1.0 and out[1, 1] < 1.0           # +X: column 0 side, row 0 side
    assert out[2, 2] > n - 2 and out[3, 1] > n - 2        # +Y: s = x, t = z
    assert out[4, 2] < 1.0 and out[5, 1] > n - 2          # -Z: s = -x, t = -y


def test_edges_clamp_within_the_face_and_bad_directions_are_black():
    n = 4
    faces = index_faces(n)
    edge = np.array([[1, -0.999, 0.999]], np.float32)   # +X, s and t near -1 ... +1 corner
    out = O.env_lookup(edge, cube=faces)
    assert out[0, 0] == 0 and out[0, 1] == n - 1 and out[0, 2] == 0
    bad = np.array([[np.nan, 0, 1], [0, 0, 0], [1, np.nan, 0]], np.float32)
    np.testing.assert_array_equal(O.env_lookup(bad, cube=faces), np.zeros((3, 3), np.float32))


def test_cube_from_equirect_samples_the_same_sky():
    sky = scenes.sky_envmap(5, 256, 128, sun_radiance=1.0)
    cube = scenes.cube_from_equirect(sky, 32)
    d = scenes.cube_directions(32).reshape(-1, 3).astype(np.float32)
    a = O.env_lookup(d, cube=cube)
    b = O.env_lookup(d, texels=sky)
    # nearest texel against bilinear of the same smooth field
    assert np.median(np.abs(a - b) / (np.abs(b) + 1e-3)) < 0.05


def test_oversized_environments_are_rejected_before_touching_the_device():
    import ctypes as C

    from nbounce_gb300 import _lib as L
    texel = np.zeros(4, np.float32)
    for kind, w, h in ((L.NB_ENV_EQUIRECT, 40000, 2), (L.NB_ENV_CUBE, 40000, 40000), (L.NB_ENV_EQUIRECT, 2, 1 << 31)):
        d = L.NbEnvDesc()
        d.kind, d.width, d.height = kind, w, h
        d.texels = texel.ctypes.data
        h_ = C.c_void_p()
        assert L.lib().nb_env_create(C.byref(d), C.byref(h_)) == L.NB_ERR_INVALID_ARG
        assert not h_.value
