"""Frames after a model moved: every voxel map level, and the frame, equal a
fresh renderer's that only ever saw the new pose, bit for bit.

The brick kernel skips the stores of a brick that is empty in this frame
and was empty in the last one (its texels, levels 1-3 and occupancy bytes
are zero already); these cases check that the bricks a model leaves are
cleared, that switching to light injection and back rewrites every brick,
and that a renderer whose counts are kept still matches."""
import numpy as np
import pytest

from voxel_cone_tracing_gb300 import scenes

W, H, N = 96, 64, 64


@pytest.fixture(scope="module")
def small():
    return scenes.scene_small(width=W, height=H)


def _renderer(vct, scene, **cfg):
    r = vct.Renderer(W, H, grid_res=N, **cfg)
    ids = vct.load_scene(r, scene)
    r.set_voxel_view_dir(7, 0.0)
    return r, ids


def _frame(r, scene, ids):
    for mid in ids:
        r.queue_model(mid)
    for l in scene.lights:
        r.queue_point_light(l)
    r.render()
    return r.read_frame().copy()


def _maps(r):
    out = [r.read_voxels(0, 0)]
    lv = 1
    while (N >> lv) >= 1:
        out += [r.read_voxels(lv, d) for d in range(6)]
        lv += 1
    return out


def _assert_same(r, fresh, f, ff):
    np.testing.assert_array_equal(f, ff)
    for k, (a, b) in enumerate(zip(_maps(r), _maps(fresh))):
        np.testing.assert_array_equal(a, b, err_msg=f"map {k}")


POSE_B = scenes.trs(translate=(0.3, 0.2, 0.25), scale=(0.2, 0.2, 0.2))


@pytest.mark.gpu
@pytest.mark.parametrize("keep_counts", [0, 1])
def test_gpu_moved_model_equals_fresh(vct, small, keep_counts):
    r, ids = _renderer(vct, small, keep_counts=keep_counts)
    _frame(r, small, ids)
    _frame(r, small, ids)
    r.set_model_transform(ids[1], POSE_B)
    f = _frame(r, small, ids)
    fresh, fids = _renderer(vct, small, keep_counts=keep_counts)
    fresh.set_model_transform(fids[1], POSE_B)
    _assert_same(r, fresh, f, _frame(fresh, small, fids))


@pytest.mark.gpu
def test_gpu_injection_round_trip_equals_fresh(vct, small):
    r, ids = _renderer(vct, small)
    _frame(r, small, ids)
    r.set_light_injection(True)
    r.set_model_transform(ids[1], POSE_B)
    _frame(r, small, ids)
    r.set_light_injection(False)
    f = _frame(r, small, ids)
    fresh, fids = _renderer(vct, small)
    fresh.set_model_transform(fids[1], POSE_B)
    _assert_same(r, fresh, f, _frame(fresh, small, fids))


@pytest.mark.gpu
def test_gpu_model_removed_clears_its_bricks(vct, small):
    r, ids = _renderer(vct, small)
    _frame(r, small, ids)
    r.queue_model(ids[0])  # this frame without the second model
    for l in small.lights:
        r.queue_point_light(l)
    r.render()
    f = r.read_frame().copy()
    fresh, fids = _renderer(vct, small)
    fresh.queue_model(fids[0])
    for l in small.lights:
        fresh.queue_point_light(l)
    fresh.render()
    _assert_same(r, fresh, f, fresh.read_frame().copy())
