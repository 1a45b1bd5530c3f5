"""vct_voxelize_noalloc -- the voxelizer for callers that cannot allocate
device memory (applications that own every device allocation through their
own heaps and keep cudaMalloc / cudaFree out of their frame loop).  Called
through the C ABI with caller-owned device buffers (made with torch here),
twice in a row, and compared with level 0 of the renderer's own frame
(vct_render + vct_read_voxels): same kernels, same fixed-point averaging,
so the texels must be identical (the parity tests allow 1 LSB against the
FP64 oracle; between two GPU paths of the same rule nothing less than
equality is expected).

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import numpy as np
import pytest

from voxel_cone_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu

N = 64


def _device_scene(torch, R, scene, pad=0):
    """Device copies of the scene's meshes and materials.  pad > 0 appends
    that many spare vertices to every vertex buffer and spare records to the
    material buffer (beyond the counts passed to the call), so that a test of
    an out-of-range id cannot read outside a device allocation even if the
    library's clamp were missing."""
    keep = []
    meshes = []
    for mesh, model in zip(scene.meshes, scene.models):
        vv = np.ascontiguousarray(mesh.verts, np.float32)
        if pad:
            vv = np.concatenate([vv, np.repeat(vv[:1], pad, axis=0)])
        v = torch.from_numpy(vv).cuda()
        ix = torch.from_numpy(np.ascontiguousarray(mesh.indices, np.uint32).view(np.int32)).cuda()
        tm = torch.from_numpy(np.ascontiguousarray(mesh.tri_material(), np.uint32).view(np.int32)).cuda()
        keep += [v, ix, tm]
        m = R.DeviceMesh()
        m.verts, m.indices, m.tri_material = v.data_ptr(), ix.data_ptr(), tm.data_ptr()
        m.n_verts, m.n_tris = mesh.verts.shape[0], mesh.n_tris
        m.model[:] = [float(x) for x in np.asarray(model, np.float32)]
        meshes.append(m)
    mats_h = np.ascontiguousarray(scene.materials)
    if pad:
        mats_h = np.concatenate([mats_h, np.repeat(mats_h[:1], pad)])
    mats = torch.from_numpy(np.frombuffer(mats_h.tobytes(), np.uint8).copy()).cuda()
    keep.append(mats)
    return meshes, mats, keep


def _renderer_level0(R, scene, n, mode=0):
    r = R.Renderer(32, 32, grid_res=n, vox_mode=mode)
    ids = R.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    R.queue_scene(r, scene, ids)
    r.render()
    want = r.read_voxels(0)
    r.close()
    return want


@pytest.mark.parametrize("mode", [0, 1], ids=["ref_raster2x", "conservative"])
def test_noalloc_voxelize_matches_renderer(vct, mode):
    torch = pytest.importorskip("torch")
    scene = scenes.scene_small(width=32, height=32)
    r = vct.Renderer(32, 32, grid_res=N, vox_mode=mode)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    vct.queue_scene(r, scene, ids)
    r.render()
    want = r.read_voxels(0)
    assert want[..., 3].astype(bool).sum() > 1000

    meshes, mats, keep = _device_scene(torch, vct, scene)
    out = torch.empty(N * N * N * 4, dtype=torch.uint8, device="cuda")
    for call in range(2):
        out.fill_(0xAB if call else 0x00)  # the call must overwrite every texel
        torch.cuda.synchronize()
        vct.voxelize_noalloc(meshes, mats.data_ptr(), scene.materials.shape[0], scene.lights, scene.cube_size, N,
                             mode, out.data_ptr())
        got = out.cpu().numpy().reshape(N, N, N, 4)
        d = np.abs(got.astype(int) - want.astype(int))
        assert d.max() <= 1, (call, d.max())
        np.testing.assert_array_equal(got, want)
    del keep


def test_noalloc_rejects_sizes_beyond_its_limits(vct):
    torch = pytest.importorskip("torch")
    scene = scenes.scene_small(width=32, height=32)
    meshes, mats, keep = _device_scene(torch, vct, scene)
    out = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(vct.VCTError) as e:
        vct.voxelize_noalloc(meshes, mats.data_ptr(), scene.materials.shape[0], scene.lights, scene.cube_size, 512,
                             0, out.data_ptr())
    assert e.value.status == 1 and "256" in str(e.value)
    with pytest.raises(vct.VCTError) as e:
        vct.voxelize_noalloc(meshes * 33, mats.data_ptr(), scene.materials.shape[0], scene.lights,
                             scene.cube_size, N, 0, out.data_ptr())
    assert e.value.status == 1 and "64" in str(e.value)
    del keep


def test_noalloc_rejects_more_lights_than_it_shades(vct):
    torch = pytest.importorskip("torch")
    scene = scenes.scene_small(width=32, height=32)
    meshes, mats, keep = _device_scene(torch, vct, scene)
    out = torch.empty(N * N * N * 4, dtype=torch.uint8, device="cuda")
    lights = np.repeat(scene.lights[:1], 11)
    with pytest.raises(vct.VCTError) as e:
        vct.voxelize_noalloc(meshes, mats.data_ptr(), scene.materials.shape[0], lights, scene.cube_size, N, 0,
                             out.data_ptr())
    assert e.value.status == 1 and "10" in str(e.value)
    del keep


@pytest.mark.parametrize("what", ["material", "index"])
def test_noalloc_out_of_range_ids_fail_after_the_call(vct, what):
    """A material id >= n_materials or a vertex index >= n_verts in the
    caller's device arrays: the kernels clamp it, the call fails with
    VCT_ERR_INVALID_VALUE, and the next call with valid ids is exact again.
    The device buffers are padded, so the test reads nothing outside them
    even without the clamp."""
    torch = pytest.importorskip("torch")
    scene = scenes.scene_small(width=32, height=32)
    want = _renderer_level0(vct, scene, N)
    meshes, mats, keep = _device_scene(torch, vct, scene, pad=4)
    n_mat = scene.materials.shape[0]
    k = 1  # the mesh after the room
    tm, ix = keep[3 * k + 2], keep[3 * k + 1]
    saved = (tm.clone(), ix.clone())
    if what == "material":
        tm[5] = n_mat
    else:
        ix[7] = meshes[k].n_verts
    out = torch.empty(N * N * N * 4, dtype=torch.uint8, device="cuda")
    with pytest.raises(vct.VCTError) as e:
        vct.voxelize_noalloc(meshes, mats.data_ptr(), n_mat, scene.lights, scene.cube_size, N, 0, out.data_ptr())
    assert e.value.status == 1 and "out of range" in str(e.value)
    tm.copy_(saved[0])
    ix.copy_(saved[1])
    vct.voxelize_noalloc(meshes, mats.data_ptr(), n_mat, scene.lights, scene.cube_size, N, 0, out.data_ptr())
    np.testing.assert_array_equal(out.cpu().numpy().reshape(N, N, N, 4), want)
    del keep


def test_noalloc_pair_overflow_fails_then_recovers(vct):
    """4096 grid-wide quads at 256^3 need about 4.3 M (triangle, brick)
    pairs, twice the fixed list: the binning keeps its writes inside the
    list, the brick pass reads only the stored part, and the call fails
    with VCT_ERR_INVALID_VALUE.  A following valid call is exact."""
    torch = pytest.importorskip("torch")
    from tests import helpers
    n = 256
    zs = np.linspace(-0.95, 0.95, 4096)
    tris = np.array([t for z in zs for t in helpers.quad_z(float(z), -0.999, 0.999)], np.float32)
    big = helpers.tri_scene(tris, lights=[((0.0, 0.0, 0.5),)])
    meshes, mats, keep = _device_scene(torch, vct, big)
    out = torch.empty(n * n * n * 4, dtype=torch.uint8, device="cuda")
    with pytest.raises(vct.VCTError) as e:
        vct.voxelize_noalloc(meshes, mats.data_ptr(), big.materials.shape[0], big.lights, big.cube_size, n, 0,
                             out.data_ptr())
    assert e.value.status == 1 and "pairs" in str(e.value)
    del keep
    scene = scenes.scene_small(width=32, height=32)
    want = _renderer_level0(vct, scene, n)
    meshes, mats, keep = _device_scene(torch, vct, scene)
    vct.voxelize_noalloc(meshes, mats.data_ptr(), scene.materials.shape[0], scene.lights, scene.cube_size, n, 0,
                         out.data_ptr())
    np.testing.assert_array_equal(out.cpu().numpy().reshape(n, n, n, 4), want)
    del keep
