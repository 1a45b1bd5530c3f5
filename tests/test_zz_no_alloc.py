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


def _device_scene(torch, R, scene):
    keep = []
    meshes = []
    for mesh, model in zip(scene.meshes, scene.models):
        v = torch.from_numpy(np.ascontiguousarray(mesh.verts, np.float32)).cuda()
        ix = torch.from_numpy(np.ascontiguousarray(mesh.indices, np.uint32).view(np.int32)).cuda()
        tm = torch.from_numpy(np.ascontiguousarray(mesh.tri_material(), np.uint32).view(np.int32)).cuda()
        keep += [v, ix, tm]
        m = R.DeviceMesh()
        m.verts, m.indices, m.tri_material = v.data_ptr(), ix.data_ptr(), tm.data_ptr()
        m.n_verts, m.n_tris = mesh.verts.shape[0], mesh.n_tris
        m.model[:] = [float(x) for x in np.asarray(model, np.float32)]
        meshes.append(m)
    mats = torch.from_numpy(np.frombuffer(np.ascontiguousarray(scene.materials).tobytes(), np.uint8).copy()).cuda()
    keep.append(mats)
    return meshes, mats, keep


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
