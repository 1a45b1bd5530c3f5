"""Known-answer tests of the CPU oracle, derived by hand from the reference's
shader maths (the reference ships no tests or golden vectors of its own)."""
import math

import numpy as np
import pytest

from tests.helpers import emissive_material, quad_z, tri_scene


# ----------------------------------------------------------- mipmap.comp ----
def test_uniform_opaque_grid_mips_equal_input(oracle):
    """alpha_blend(f, b) with f.a = 1 returns f; the mean of equal values is
    the value: every level of every map equals level 0 (mipmap.comp:40-98)."""
    n = 16
    p = oracle.Params(grid_res=n)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    l0[...] = (37, 200, 91, 255)
    ch = oracle.mipmap(p, l0)
    for lvl in range(1, p.levels):
        for m in range(6):
            assert (oracle.chain_level(ch, n, lvl, m) == (37, 200, 91, 255)).all()


@pytest.mark.parametrize("n", [8])
def test_front_to_back_pairs(oracle, n):
    """N=2 corner: x=1 texels opaque red, x=0 opaque green.  The -x map sees
    the x-offset-1 child in front (mipmap.comp:59-63) -> red; +x -> green;
    the y and z maps blend each colour with itself and average 2+2 ->
    127.5 -> 128 (round to nearest, ties up)."""
    p = oracle.Params(grid_res=n)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    l0[0:2, 0:2, 1] = (255, 0, 0, 255)
    l0[0:2, 0:2, 0] = (0, 255, 0, 255)
    ch = oracle.mipmap(p, l0)
    got = [tuple(oracle.chain_level(ch, n, 1, m)[0, 0, 0]) for m in range(6)]
    assert got[0] == (255, 0, 0, 255)
    assert got[1] == (0, 255, 0, 255)
    for m in range(2, 6):
        assert got[m] == (128, 128, 0, 255)


def test_semi_transparent_front(oracle):
    """front (255,0,0,128), back (0,0,255,255): R = 1, B = (1-128/255)*1 =
    0.498 -> 127, A = 128/255 + 127/255 = 1 -> 255."""
    n = 8
    p = oracle.Params(grid_res=n)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    l0[0:2, 0:2, 1] = (255, 0, 0, 128)
    l0[0:2, 0:2, 0] = (0, 0, 255, 255)
    ch = oracle.mipmap(p, l0)
    assert tuple(oracle.chain_level(ch, n, 1, 0)[0, 0, 0]) == (255, 0, 127, 255)


def test_iso_mip_box_mean(oracle):
    n = 8
    p = oracle.Params(grid_res=n, mip_mode=oracle.MIP_ISO)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    l0[0, 0, 0] = (255, 8, 4, 255)
    ch = oracle.mipmap(p, l0)
    # 255/8 = 31.875 -> 32, 8/8 = 1, 4/8 = 0.5 -> 1 (ties up)
    assert tuple(oracle.chain_level(ch, n, 1, 0)[0, 0, 0]) == (32, 1, 1, 32)


# ----------------------------------------------------------- GL sampling ----
def test_texture_lod_texel_centre_and_lerp(oracle):
    n = 8
    p = oracle.Params(grid_res=n)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    l0[3, 2, 1] = (255, 0, 0, 255)
    ch = oracle.mipmap(p, l0)
    u = [(1 + 0.5) / n, (2 + 0.5) / n, (3 + 0.5) / n]
    np.testing.assert_allclose(oracle.texture_lod(p, l0, ch, 0, u, 0.0), [1, 0, 0, 1], atol=1e-12)
    # half a texel along x: two texels blended 50/50
    u2 = [(1 + 1.0) / n, u[1], u[2]]
    np.testing.assert_allclose(oracle.texture_lod(p, l0, ch, 0, u2, 0.0), [0.5, 0, 0, 0.5], atol=1e-12)
    # lod 0.5 blends level 0 and level 1 equally
    t0 = oracle.texture_lod(p, l0, ch, 0, u, 0.0)
    t1 = oracle.texture_lod(p, l0, ch, 0, u, 1.0)
    np.testing.assert_allclose(oracle.texture_lod(p, l0, ch, 0, u, 0.5), 0.5 * (t0 + t1), atol=1e-12)
    # outside the texture: border colour 0
    np.testing.assert_allclose(oracle.texture_lod(p, l0, ch, 0, [-0.5, 0.5, 0.5], 0.0), 0.0, atol=1e-12)


def _steps_to(n, aperture, max_dist):
    vs = 1.0 / n
    dist = 3 * vs
    diam = dist * aperture
    k = 0
    while dist < max_dist:
        dist += max(diam / 2, vs)
        diam = dist * aperture
        k += 1
    return k


def test_cone_through_empty_space(oracle):
    """Empty grid: the cone accumulates nothing and marches until max_dist
    with steps max(diam/2, 1/N) (voxel_cone_tracing.frag:88-119)."""
    n = 32
    p = oracle.Params(grid_res=n)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    ch = oracle.mipmap(p, l0)
    rgba, steps = oracle.trace_cone(p, l0, ch, [0.5, 0.5, 0.5], [0.3, -0.2, 0.9], 0.55785173935, 1.73205080757)
    np.testing.assert_array_equal(rgba, 0.0)
    assert steps == _steps_to(n, 0.55785173935, 1.73205080757)


def test_cone_into_opaque_wall(oracle):
    """Uniformly opaque grid: the first sample has alpha = |d|_1 >= 1, so the
    march stops after one step with colour = |d|_1 * texel."""
    n = 16
    p = oracle.Params(grid_res=n)
    l0 = np.zeros((n, n, n, 4), np.uint8)
    l0[...] = (255, 255, 255, 255)
    ch = oracle.mipmap(p, l0)
    d = np.array([0.6, 0.0, 0.8])
    rgba, steps = oracle.trace_cone(p, l0, ch, [0.5, 0.5, 0.5], d, 0.1, 1.7)
    assert steps == 1
    np.testing.assert_allclose(rgba, np.abs(d).sum(), rtol=1e-12)


# ------------------------------------------------------ voxelize (REF) ------
def test_axis_aligned_slab_ref(oracle):
    """A quad covering the whole grid at the centre depth of voxel slab k:
    each voxel column gets exactly its 2x2 samples (top-left rule on the
    shared diagonal), all in slab k; colour = emission (no lights)."""
    n = 16
    k = 5
    z = (k + 0.5) * 2 / n - 1
    s = tri_scene(quad_z(z), material=emissive_material((0.2, 0.4, 0.6)))
    p = oracle.Params(grid_res=n)
    l0, cnt, rej = oracle.voxelize(s, p)
    assert rej == 0
    assert (cnt[k] == 4).all()
    assert cnt.sum() == 4 * n * n
    assert (l0[k] == (51, 102, 153, 255)).all()
    assert (l0[np.arange(n) != k] == 0).all()


def test_degenerate_dominant_axis_dropped_ref(oracle):
    """|n| = (1,0,1): both strict tests of voxelize.geom:40-47 fail, the y
    projection is chosen and the triangle projects to a line -> no samples.
    The conservative mode still voxelizes it."""
    n = 16
    tri = [[(-0.5, -0.5, 0.5), (0.5, -0.5, -0.5), (0.0, 0.5, 0.0)]]
    s = tri_scene(tri)
    l0, cnt, _ = oracle.voxelize(s, oracle.Params(grid_res=n))
    assert cnt.sum() == 0
    _, cnt2, _ = oracle.voxelize(s, oracle.Params(grid_res=n, vox_mode=oracle.VOX_CONSERVATIVE))
    assert cnt2.sum() > 0


def test_truncation_quirk_low_face(oracle):
    """int(N*(0.5c+0.5)) truncates toward 0: depth a quarter voxel below the
    grid still lands in slab 0 (voxelize.frag:157); depth exactly +1 maps to
    index N and is dropped."""
    n = 16
    s = tri_scene(quad_z(-1.0 - 0.25 * 2 / n))
    _, cnt, _ = oracle.voxelize(s, oracle.Params(grid_res=n))
    assert (cnt[0] == 4).all() and cnt.sum() == 4 * n * n
    s2 = tri_scene(quad_z(1.0))
    _, cnt2, _ = oracle.voxelize(s2, oracle.Params(grid_res=n))
    assert cnt2.sum() == 0


def test_running_average_is_mean(oracle):
    """Two overlapping coplanar quads of different emission: every voxel is
    the mean of its 8 contributions, rounded once."""
    n = 8
    z = (2 + 0.5) * 2 / n - 1
    tris = quad_z(z) + quad_z(z)
    s = tri_scene(tris, material=emissive_material((0.0, 1.0, 0.5)))
    _, cnt, _ = oracle.voxelize(s, oracle.Params(grid_res=n))
    assert (cnt[2] == 8).all()


def test_light_attenuation_value(oracle):
    """One light straight above a floor quad: colour = diffuse * cos *
    1/(1+d^2) (voxelize.frag:128-139) at the sample points."""
    n = 8
    k = 3
    z = (k + 0.5) * 2 / n - 1
    mat = emissive_material(emission=(0, 0, 0), diffuse=(1.0, 1.0, 1.0))
    s = tri_scene(quad_z(z), material=mat, lights=[((0.0, 0.0, z + 1.0), (1, 1, 1), 1.0)])
    l0, cnt, _ = oracle.voxelize(s, oracle.Params(grid_res=n))
    # voxel column (i, j): 4 samples at ((2i+a+0.5)/n - 1, ...)
    i = j = 3
    vals = []
    for a in (0, 1):
        for b in (0, 1):
            x = (2 * i + a + 0.5) / n - 1
            y = (2 * j + b + 0.5) / n - 1
            d2 = x * x + y * y + 1.0
            vals.append((1.0 / math.sqrt(d2)) / (1.0 + d2))
    want = math.floor(np.mean(vals) * 255 + 0.5)
    assert int(l0[k, j, i, 0]) == want


# ------------------------------------------------- voxelize (conservative) --
def test_conservative_small_triangle_one_voxel(oracle):
    n = 8
    c = lambda i: (i + 0.5) * 2 / n - 1  # noqa: E731
    h = 0.2 * 2 / n
    tri = [[(c(3) - h, c(4) - h, c(5)), (c(3) + h, c(4) - h, c(5)), (c(3), c(4) + h, c(5))]]
    _, cnt, _ = oracle.voxelize(tri_scene(tri), oracle.Params(grid_res=n, vox_mode=oracle.VOX_CONSERVATIVE))
    assert cnt.sum() == 1 and cnt[5, 4, 3] == 1


def test_conservative_touching_face_counts_both(oracle):
    """Closed boxes: a triangle lying exactly on the face between slabs 3 and
    4 overlaps both."""
    n = 8
    z = 4 * 2 / n - 1
    _, cnt, _ = oracle.voxelize(tri_scene(quad_z(z, -0.5, 0.5)),
                                oracle.Params(grid_res=n, vox_mode=oracle.VOX_CONSERVATIVE))
    assert cnt[3].sum() > 0 and cnt[4].sum() > 0 and cnt[3].sum() == cnt[4].sum()


# ------------------------------------------------------------- G-buffer -----
def test_gbuffer_full_screen_quad(oracle):
    """Identity camera: a quad on NDC [-1,1]^2 at z=0 covers every pixel once
    and the interpolated world position is the pixel centre."""
    w, h = 32, 16
    s = tri_scene(quad_z(0.0))
    gb = oracle.gbuffer(s, oracle.Params(grid_res=8, width=w, height=h))
    assert (gb["tri_id"] != 0xffffffff).all()
    xs = (np.arange(w) + 0.5) * 2 / w - 1
    ys = (np.arange(h) + 0.5) * 2 / h - 1
    np.testing.assert_allclose(gb["pos"][..., 0], np.broadcast_to(xs, (h, w)), atol=1e-6)
    np.testing.assert_allclose(gb["pos"][..., 1], np.broadcast_to(ys[:, None], (h, w)), atol=1e-6)


def test_gbuffer_depth_test_nearest_wins(oracle):
    """Two full-screen quads; GL_LESS keeps the nearer (smaller z_window)."""
    s = tri_scene(quad_z(0.5) + quad_z(-0.5))
    gb = oracle.gbuffer(s, oracle.Params(grid_res=8, width=8, height=8))
    assert set(np.unique(gb["tri_id"])) <= {2, 3}
    s2 = tri_scene(quad_z(-0.5) + quad_z(0.5))
    gb2 = oracle.gbuffer(s2, oracle.Params(grid_res=8, width=8, height=8))
    assert set(np.unique(gb2["tri_id"])) <= {0, 1}


def test_frame_background_is_clear_colour(oracle):
    s = tri_scene([[(5, 5, 5), (6, 5, 5), (5, 6, 5)]])
    p = oracle.Params(grid_res=8, width=8, height=8)
    r = oracle.render(s, p)
    np.testing.assert_allclose(r["frame"], np.broadcast_to([0.15, 0.25, 0.25, 1.0], (8, 8, 4)), atol=1e-7)
