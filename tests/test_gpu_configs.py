"""Parity of two workloads at the sizes they are stated at, against the FP64
oracle, stage by stage.

Small plain method: the closed box room (10 triangles) + 2 rotated cuboids
(24 triangles), one point light, 64^3 RGBA8 grid with 7 isotropic mip
levels, 256x256 frame, six 60-degree diffuse cones + 1 specular cone (+ the
shadow cone of the light), FP32 march.

Precision: 512^3 grid, RGBA16F maps with radiance clamped to [0, 16], the
exact conservative (SAT) voxelizer, 1,997,514 triangles (room + 4 displaced
icospheres + 32 cuboids), 1920x1080 frame, 9 diffuse + 1 specular + 1 shadow
cone, FP32 march.

Tolerances (stated per output):
  voxel contribution counts / occupancy ....... bit-exact (whole grid)
  level 0, RGBA8 .............................. |d| <= 1 LSB of the FP64 mean
  level 0, half ............................... |d| <= 1 half ulp of the FP64
                                                mean for >= 99.99% of the
                                                occupied voxels, <= 2 half ulp
                                                everywhere (FP32 shading at
                                                the closest point of sliver
                                                triangles moves a few means by
                                                more than half an ulp)
  mips, RGBA8 (from the GPU's level 0) ........ bit-exact
  mip level k+1, half (from the GPU's level k)  |d| <= 1 half ulp + 1e-6
  visible triangle id ......................... bit-exact
  radiance, FP32 software filtering (EXACT) ... PSNR >= 60 dB (RGBA8); max
                                                |d| <= 2e-3 x peak (half)
  radiance, texture-unit filtering ............ PSNR >= 40 dB
  whole small frame vs the oracle's own
  voxelize -> mip -> G-buffer -> trace (EXACT)  PSNR >= 50 dB
The precision frame's radiance is compared on every 64th pixel row (17 rows,
32,640 pixels); everything else on the whole grid / frame.
"""
import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu


def _gb64(gb):
    return dict(tri_id=gb["tri_id"], pos=gb["pos"].astype(np.float64), nrm=gb["nrm"].astype(np.float64),
                mat=gb["mat"])


def _render(vct, scene, w, h, n, **cfg):
    cfg.setdefault("keep_counts", 1)
    cfg.setdefault("keep_float_frame", 1)
    r = vct.Renderer(w, h, grid_res=n, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    r.synchronize()
    return r


# ------------------------------------------------------ small plain method --
SW, SH, SN = 256, 256, 64
SMALL = dict(mip_mode=1, cone_set=1)  # isotropic mips, six 60-degree cones


@pytest.fixture(scope="module")
def small():
    s = scenes.scene_small(width=SW, height=SH)
    assert s.n_tris == 34
    return s


@pytest.fixture(scope="module")
def small_params(oracle):
    return oracle.Params(grid_res=SN, width=SW, height=SH, mip_mode=oracle.MIP_ISO, cone_set=oracle.CONES_SIX60)


@pytest.fixture(scope="module")
def small_hw(vct, small):
    return _render(vct, small, SW, SH, SN, **SMALL)


@pytest.fixture(scope="module")
def small_exact(vct, small):
    return _render(vct, small, SW, SH, SN, sampler=vct.SAMPLER_EXACT, **SMALL)


def _iso_chain(r, n, levels):
    from oracle import oracle as O
    ch = np.zeros((1, O.chain_texels(n, levels), 4), np.uint8)
    off = 0
    for lvl in range(1, levels):
        s = n >> lvl
        ch[0, off:off + s ** 3] = r.read_voxels(lvl, 0).reshape(-1, 4)
        off += s ** 3
    return ch


def test_small_stated_size_voxels_and_mips(oracle, small, small_params, small_hw):
    r = small_hw
    n, levels = r.grid()
    assert (n, levels) == (SN, 7)
    l0, cnt, rej = oracle.voxelize(small, small_params)
    assert rej == 0
    np.testing.assert_array_equal(r.read_voxel_counts(), cnt)
    d = np.abs(r.read_voxels(0).astype(int) - l0.astype(int))
    print(f"small: {int((cnt > 0).sum())} occupied voxels, level 0 max|d| {d.max()} LSB, "
          f"identical {100 * (d == 0).mean():.4f}%")
    assert d.max() <= 1
    np.testing.assert_array_equal(_iso_chain(r, n, levels), oracle.mipmap(small_params, r.read_voxels(0)))


def test_small_stated_size_gbuffer(oracle, small, small_params, small_hw):
    g = small_hw.read_gbuffer()
    o = oracle.gbuffer(small, small_params)
    np.testing.assert_array_equal(g["tri_id"], o["tri_id"])
    assert (o["tri_id"] != 0xffffffff).mean() > 0.9


@pytest.mark.parametrize("sampler", ["exact", "hw"])
def test_small_stated_size_radiance(oracle, small, small_params, small_hw, small_exact, sampler):
    """Oracle trace from the GPU's own maps and G-buffer: isolates the six-cone
    tracer over the whole 256x256 frame."""
    r = small_exact if sampler == "exact" else small_hw
    n, levels = r.grid()
    ref = oracle.trace(small, small_params, r.read_voxels(0), _iso_chain(r, n, levels), _gb64(r.read_gbuffer()))
    got = r.read_frame(1)
    q = psnr(np.clip(got, 0, 1), np.clip(ref, 0, 1))
    print(f"small {sampler}: PSNR {q:.1f} dB, max|d| {np.abs(got - ref).max():.3e}")
    assert q >= (60.0 if sampler == "exact" else 40.0)


def test_small_stated_size_end_to_end(oracle, small, small_params, small_exact):
    """The GPU frame against the oracle's own voxelize -> mip -> G-buffer ->
    trace (nothing shared but the scene)."""
    ref = oracle.render(small, small_params)["frame"]
    got = small_exact.read_frame(1)
    q = psnr(np.clip(got, 0, 1), np.clip(ref, 0, 1))
    print(f"small end to end: PSNR {q:.1f} dB")
    assert q >= 50.0


# --------------------------------------------------------------- precision --
PW, PH, PN, ROWS = 1920, 1080, 512, 64
RMAX = scenes.HDR_RADIANCE_MAX


@pytest.fixture(scope="module")
def hdr():
    s = scenes.scene_hdr(width=PW, height=PH)
    assert s.n_tris == 1_997_514
    return s


@pytest.fixture(scope="module")
def hdr_frames(vct, hdr):
    cfg = dict(storage=vct.STORAGE_RGBA16F, radiance_max=RMAX, vox_mode=vct.VOX_CONSERVATIVE)
    hw = _render(vct, hdr, PW, PH, PN, **cfg)
    ex = _render(vct, hdr, PW, PH, PN, sampler=vct.SAMPLER_EXACT, keep_counts=0, **cfg)
    yield hw, ex
    hw.close()
    ex.close()


def _half_ulp(ref):
    return np.spacing(np.abs(ref).astype(np.float16)).astype(np.float64)


def test_precision_full_size_voxelize(oracle, hdr, hdr_frames):
    r = hdr_frames[0]
    ref, cnt, rej = oracle.voxelize_hdr(hdr, oracle.Params(grid_res=PN, vox_mode=oracle.VOX_CONSERVATIVE,
                                                           radiance_max=RMAX))
    assert rej == 0
    np.testing.assert_array_equal(r.read_voxel_counts(), cnt)
    got = r.read_voxels(0)
    worst_ulp, worst_abs, n_hdr, over = 0.0, 0.0, 0, 0
    for z in range(0, PN, 64):  # slabs: keeps the FP64 copies small
        g = got[z:z + 64].astype(np.float64)
        o = ref[z:z + 64].astype(np.float64)
        d = np.abs(g - o)
        ulps = d / _half_ulp(o)
        worst_abs = max(worst_abs, float(d.max()))
        worst_ulp = max(worst_ulp, float(ulps.max()))
        over += int((ulps > 1.0).any(axis=-1).sum())
        n_hdr += int((o[..., :3] > 1.0).sum())
    occupied = int((cnt > 0).sum())
    print(f"precision level 0: {occupied} occupied voxels, {int(cnt.sum())} contributions, max|d| {worst_abs:.3e}, "
          f"worst {worst_ulp:.3f} half ulp, {over} voxels above 1 half ulp, {n_hdr} channels > 1")
    assert n_hdr > 1000
    assert over <= 1e-4 * occupied
    assert worst_ulp <= 2.0


def test_precision_full_size_mips(oracle, hdr_frames):
    """Every level k+1 against the FP64 reduction of the GPU's level k."""
    r = hdr_frames[0]
    n, levels = r.grid()
    worst = []
    src = r.read_voxels(0).astype(np.float32)
    for lvl in range(1, levels):
        ref = oracle.mip_level_f(src, 0)
        got = np.stack([r.read_voxels(lvl, m) for m in range(6)]).astype(np.float32)
        tol = _half_ulp(ref) + 1e-6
        ratio = float((np.abs(got.astype(np.float64) - ref) / tol).max())
        worst.append(round(ratio, 3))
        assert ratio <= 1.0, f"level {lvl}"
        src = got
    print(f"precision mips: worst |d| / (1 half ulp + 1e-6) per level {worst}")


def _chains_f(r, n, levels):
    from oracle import oracle as O
    ch = np.zeros((6, O.chain_texels(n, levels), 4), np.float32)
    off = 0
    for lvl in range(1, levels):
        s = n >> lvl
        for m in range(6):
            ch[m, off:off + s ** 3] = r.read_voxels(lvl, m).astype(np.float32).reshape(-1, 4)
        off += s ** 3
    return ch


@pytest.mark.parametrize("sampler", ["exact", "hw"])
def test_precision_full_size_radiance_rows(oracle, hdr, hdr_frames, sampler):
    r = hdr_frames[1] if sampler == "exact" else hdr_frames[0]
    n, levels = r.grid()
    p = oracle.Params(grid_res=n, width=PW, height=PH, radiance_max=RMAX)
    ref = oracle.trace_hdr(hdr, p, r.read_voxels(0).astype(np.float32), _chains_f(r, n, levels),
                           _gb64(r.read_gbuffer()), row_stride=ROWS)[::ROWS]
    got = r.read_frame(1)[::ROWS]
    peak = float(ref[..., :3].max())
    d = np.abs(got - ref)[..., :3]
    q = psnr(got[..., :3], ref[..., :3], peak=peak)
    print(f"precision {sampler}: {ref.shape[0]} rows, peak {peak:.2f}, PSNR {q:.1f} dB, max|d| {d.max():.3e}")
    assert peak > 1.0
    if sampler == "exact":
        assert d.max() <= 2e-3 * peak
    else:
        assert q >= 40.0
