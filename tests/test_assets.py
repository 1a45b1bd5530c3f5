"""The reference's own demo assets through the OBJ/MTL loader and the headless
demo, checked against an independent parse (tests/objparse.py) and the CPU
oracle.

Assets: tests/assets/CornellBox-Glossy.{obj,mtl} are the reference's files
(Williams College, released into the public domain, as their header says).
The demo's second model, assets/suzanne.obj, states no licence, so the demo
test writes a stand-in of the same form (triangles with v/vt/vn corners, a
`usemtl` naming no library, a smoothing group): a seeded bumpy icosphere.

Tolerances:
  loader vs independent parse: materials, dimensions, voxel counts and the
    RGBA8 frame identical (same triangles, same draw objects);
  loader's voxel counts vs the oracle's on the independent parse: bit-exact;
  demo's default frame (800x600, 128^3, grid size 3, ceiling light at
    (0, 1.4, 0), main.cpp:85-121) vs oracle.render on the independent parse:
    PSNR >= 50 dB with FP32 software filtering, >= 40 dB with the texture
    unit (the end-to-end tolerances of tests/test_gpu_parity.py).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests import objparse
from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
BOX = os.path.join(HERE, "assets", "CornellBox-Glossy.obj")
W, H, N = 800, 600, 128  # main.cpp:28-29, renderer.cpp:146


def test_cornell_box_independent_parse():
    m = objparse.parse_obj(BOX, material_base=1)
    assert m.indices.shape[0] == 1112          # every face of the file is a triangle
    assert m.material_names == ["sphere", "shortBox", "floor", "ceiling", "backWall", "leftWall", "rightWall",
                                "light"]
    assert m.shapes == 8 and m.draw_objs.shape[0] == 8
    assert m.draw_objs["count"].sum() == 3 * 1112
    light = m.materials[7]
    assert tuple(light["emission"][:3]) == (10.0, 10.0, 10.0)
    assert m.materials[0]["shininess"] == 32.0 and m.materials[0]["dissolve"] == 1.0
    # the reference's arithmetic (max starts at 0, z compared with min.y)
    np.testing.assert_allclose(m.dimensions, (2.02, 1.5901, 1.21), rtol=1e-5)


def _object_obj(path, seed=7, subdiv=3):
    """A stand-in of suzanne.obj's form: unit icosphere subdivided `subdiv`
    times with seeded bumps, triangles with v/vt/vn corners, a usemtl naming
    no material library (so its triangles take material 0 until
    set_model_material)."""
    t = (1 + 5 ** 0.5) / 2
    p = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t), (t, 0, -1),
         (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    p = [np.array(q, np.float64) / np.linalg.norm(q) for q in p]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7),
         (9, 8, 1)]
    for _ in range(subdiv):
        cache, g = {}, []

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                q = p[a] + p[b]
                p.append(q / np.linalg.norm(q))
                cache[k] = len(p) - 1
            return cache[k]
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            g += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = g
    rng = np.random.default_rng(seed)
    v = np.array(p) * (1.0 + 0.08 * rng.standard_normal(len(p)))[:, None]
    uv = rng.random((len(p), 2))
    lines = ["# generated stand-in for the demo's dynamic object"]
    lines += [f"v {a:.6f} {b:.6f} {c:.6f}" for a, b, c in v]
    lines += [f"vt {a:.6f} {b:.6f}" for a, b in uv]
    lines += [f"vn {a:.6f} {b:.6f} {c:.6f}" for a, b, c in np.array(p)]
    lines += ["usemtl Material_ray.png", "s 1"]
    lines += ["f " + " ".join(f"{i + 1}/{i + 1}/{i + 1}" for i in tri) for tri in f]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def _demo_material():
    m = np.zeros((), scenes.MATERIAL_DTYPE)  # main.cpp:88-97
    m["ambient"], m["diffuse"], m["specular"], m["transmittance"] = 1.0, 0.0, 1.0, 1.0
    m["emission"] = (0.0, 0.0, 0.25)
    m["shininess"], m["ior"], m["dissolve"], m["illum"] = 1000.0, 5.0, 0.1, 4
    return m


def _demo_camera():
    """Camera(glm::vec3(0, .9, 3), 0, -90) with glm::perspective(45, ...) (45
    taken as radians, as glm does), main.cpp:107-108 -- built here in FP64."""
    eye = np.array([0.0, 0.9, 3.0])
    f = np.array([np.cos(np.radians(-90.0)), 0.0, np.sin(np.radians(-90.0))])
    return scenes.look_at(eye, eye + f), scenes.perspective(45.0, W / H, 0.1, 100.0)


def _material_fields(m):
    return {k: np.asarray(m[k], np.float64).ravel()[:3] if np.asarray(m[k]).size > 1 else float(m[k])
            for k in ("ambient", "diffuse", "specular", "transmittance", "emission", "shininess", "ior", "dissolve",
                      "illum")}


@pytest.mark.gpu
def test_cornell_box_loader_matches_independent_parse(vct, oracle):
    ref = objparse.parse_obj(BOX, material_base=1)
    view, proj = _demo_camera()
    light = scenes.point_light((0.0, 1.4, 0.0))
    frames, counts = [], []
    for use_loader in (True, False):
        r = vct.Renderer(W, H, grid_res=N, keep_counts=1)
        if use_loader:
            mid = r.load_model(BOX)
            assert mid != vct.INVALID_ID
            for k in range(8):
                got, want = _material_fields(r.get_material(1 + k)), _material_fields(ref.materials[k])
                for key in want:
                    np.testing.assert_allclose(got[key], want[key], rtol=0, atol=0, err_msg=f"{k} {key}")
            np.testing.assert_array_equal(r.get_model_dimensions(mid), ref.dimensions)
        else:
            for k in range(8):
                assert r.add_material(ref.materials[k]) == 1 + k
            mid = r.load_mesh(ref.verts, ref.indices, ref.draw_objs)
        r.set_grid_size(3.0)
        r.set_camera_transform(view, proj)
        r.set_voxel_view_dir(7, 0.0)
        r.queue_model(mid)
        r.queue_point_light(light)
        r.render()
        frames.append(r.read_frame().copy())
        counts.append(r.read_voxel_counts())
        r.close()
    np.testing.assert_array_equal(counts[0], counts[1])
    np.testing.assert_array_equal(frames[0], frames[1])
    mats = np.concatenate([np.array([scenes.default_material()], scenes.MATERIAL_DTYPE), ref.materials])
    scene = scenes.Scene([ref.mesh()], [scenes.mat_identity()], mats, np.array([light], scenes.LIGHT_DTYPE),
                         view, proj, 3.0, name="cornell")
    _, cnt, rej = oracle.voxelize(scene, oracle.Params(grid_res=N))
    assert rej == 0
    np.testing.assert_array_equal(counts[0], cnt)


@pytest.mark.gpu
@pytest.mark.parametrize("sampler", ["exact", "hw"])
def test_demo_default_frame_against_oracle(vct, oracle, tmp_path, sampler):
    from voxel_cone_tracing_gb300 import build
    demo = build.build_demo()
    d = str(tmp_path)
    for ext in ("obj", "mtl"):
        shutil.copy(os.path.join(HERE, "assets", f"CornellBox-Glossy.{ext}"), d)
    _object_obj(os.path.join(d, "suzanne.obj"))
    out, dump = os.path.join(d, "frame"), os.path.join(d, "matrices.txt")
    r = subprocess.run([demo, "--assets", d, "--out", out, "--frames", "1", "--sampler", sampler, "--dump-matrices",
                        dump], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    with open(out + "_0000.ppm", "rb") as f:
        head = [f.readline() for _ in range(3)]
        assert head[0].strip() == b"P6" and head[1].split() == [b"800", b"600"]
        got = np.frombuffer(f.read(), np.uint8).reshape(H, W, 3)[::-1]  # PPM rows run top-down
    mats = np.loadtxt(dump, dtype=np.float32).reshape(-1, 48)[0]
    view, proj, model = mats[:16], mats[16:32], mats[32:48]

    box = objparse.parse_obj(os.path.join(d, "CornellBox-Glossy.obj"), material_base=1)
    obj = objparse.parse_obj(os.path.join(d, "suzanne.obj"), material_base=9)
    assert len(obj.materials) == 0 and (obj.draw_objs["material"] == 0).all()
    obj.draw_objs["material"] = 9  # set_model_material(dynamic_object_material_id, dynamic_object)
    table = np.concatenate([np.array([scenes.default_material()], scenes.MATERIAL_DTYPE), box.materials,
                            np.array([_demo_material()], scenes.MATERIAL_DTYPE)])
    scene = scenes.Scene([box.mesh(), obj.mesh()], [scenes.mat_identity(), model], table,
                         np.array([scenes.point_light((0.0, 1.4, 0.0))], scenes.LIGHT_DTYPE), view, proj, 3.0,
                         name="demo")
    ref = oracle.render(scene, oracle.Params(grid_res=N, width=W, height=H))["frame"]
    q = psnr(got / 255.0, np.clip(ref[..., :3], 0, 1))
    lsb = np.abs(got.astype(int) - np.round(np.clip(ref[..., :3], 0, 1) * 255).astype(int)).max(axis=2)
    print(f"demo frame ({sampler}) vs oracle: PSNR {q:.1f} dB, {100 * (lsb <= 1).mean():.2f}% of pixels within 1 LSB")
    assert q >= (50.0 if sampler == "exact" else 40.0)
