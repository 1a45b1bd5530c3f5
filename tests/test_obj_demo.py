"""The OBJ/MTL loader (Renderer::load_model) and the headless demo driver
(the stand-in for src/main.cpp).

GPU tests: an OBJ file renders exactly like the same triangles given to
load_mesh; the demo's frames match the same calls made from Python on the
same files (PSNR >= 40 dB: its camera matrices are computed in C++ FP32,
here in FP64 rounded to FP32).  CPU tests: the demo builds and rejects bad
arguments before touching a device.
"""
import math
import os
import subprocess

import numpy as np
import pytest

from tests.helpers import psnr
from voxel_cone_tracing_gb300 import scenes

BOX_MTL = """newmtl white
Kd 0.73 0.73 0.73
Ka 1 1 1
Ns 10
illum 2
newmtl red
Kd 0.63 0.06 0.04
Ns 10
illum 2
newmtl green
Kd 0.15 0.48 0.09
Ns 10
illum 2
"""

# x in [-1, 1], y in [0, 2], z in [-1, 1]; quads (fan-triangulated by the
# loader), normals facing the inside.
BOX_V = [(-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1), (-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)]
BOX_FACES = [  # (material, normal, corner indices)
    ("white", (0, 1, 0), (0, 1, 2, 3)),
    ("white", (0, -1, 0), (4, 7, 6, 5)),
    ("white", (0, 0, 1), (0, 4, 5, 1)),
    ("red", (1, 0, 0), (0, 3, 7, 4)),
    ("green", (-1, 0, 0), (1, 5, 6, 2)),
]


def _write_box(d):
    with open(os.path.join(d, "box.mtl"), "w") as f:
        f.write(BOX_MTL)
    lines = ["mtllib box.mtl", "o box"] + [f"v {x} {y} {z}" for x, y, z in BOX_V]
    for k, (_, n, _) in enumerate(BOX_FACES):
        lines.append("vn %g %g %g" % n)
    cur = None
    for k, (mat, _, c) in enumerate(BOX_FACES):
        if mat != cur:
            lines.append(f"usemtl {mat}")
            cur = mat
        lines.append("f " + " ".join(f"{i + 1}//{k + 1}" for i in c))
    path = os.path.join(d, "CornellBox-Glossy.obj")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def _write_object(d):
    t = (1 + 5 ** 0.5) / 2
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7),
         (9, 8, 1)]
    lines = [f"v {a:.7f} {b:.7f} {c:.7f}" for a, b, c in v] + [f"vn {a:.7f} {b:.7f} {c:.7f}" for a, b, c in v]
    lines += ["f " + " ".join(f"{i + 1}//{i + 1}" for i in tri) for tri in f]
    path = os.path.join(d, "suzanne.obj")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


def _box_arrays():
    """The triangles of the box OBJ in the loader's order (per face: fan
    (0,1,2), (0,2,3)), one draw object per run of equal materials."""
    verts, idx, runs = [], [], []
    for k, (mat, n, c) in enumerate(BOX_FACES):
        base = len(verts)
        for i in c:
            verts.append(list(BOX_V[i]) + list(n) + [0.0, 0.0])
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    mats = [m for m, _, _ in BOX_FACES]
    start = 0
    for k in range(1, len(mats) + 1):
        if k == len(mats) or mats[k] != mats[start]:
            runs.append((6 * start, 6 * (k - start), {"white": 1, "red": 2, "green": 3}[mats[start]]))
            start = k
    return (np.array(verts, np.float32), np.array(idx, np.uint32).reshape(-1, 3),
            np.array(runs, scenes.DRAWOBJ_DTYPE))


def _look_at(eye, center, up):
    f = np.subtract(center, eye, dtype=np.float64)
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m.T.reshape(-1).astype(np.float32)  # column-major


def _perspective(fovy, aspect, n, f):
    t = math.tan(fovy / 2)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = 1 / (aspect * t), 1 / t
    m[2, 2], m[2, 3], m[3, 2] = -(f + n) / (f - n), -2 * f * n / (f - n), -1
    return m.T.reshape(-1).astype(np.float32)


def _demo_material():
    m = np.zeros((), scenes.MATERIAL_DTYPE)  # src/main.cpp:88-97
    m["ambient"], m["diffuse"], m["specular"], m["transmittance"] = 1.0, 0.0, 1.0, 1.0
    m["emission"] = (0.0, 0.0, 0.25)
    m["shininess"], m["ior"], m["dissolve"], m["illum"] = 1000.0, 5.0, 0.1, 4
    return m


def _read_ppm(path):
    with open(path, "rb") as f:
        data = f.read()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P6"
    w, h = map(int, parts[1].split())
    assert parts[2] == b"255"
    return np.frombuffer(parts[3], np.uint8).reshape(h, w, 3)


@pytest.fixture(scope="module")
def demo_bin():
    from voxel_cone_tracing_gb300 import build
    build.build()
    return build.build_demo()


def test_demo_rejects_bad_arguments(demo_bin):
    r = subprocess.run([demo_bin, "--no-such-flag"], capture_output=True, text=True)
    assert r.returncode == 2
    assert "unknown argument" in r.stderr


@pytest.mark.gpu
def test_obj_renders_like_load_mesh(vct, tmp_path):
    path = _write_box(str(tmp_path))
    v, i, runs = _box_arrays()
    frames = []
    for use_obj in (True, False):
        r = vct.Renderer(96, 72, grid_res=32)
        if use_obj:
            mid = r.load_model(path)
            assert mid != vct.INVALID_ID
            np.testing.assert_allclose(r.get_material(2)["diffuse"][:3], (0.63, 0.06, 0.04), rtol=1e-6)
            d = r.get_model_dimensions(mid)
            assert d[0] == pytest.approx(2.0) and d[1] == pytest.approx(2.0)
        else:
            for name in ("white", "red", "green"):
                m = np.zeros((), scenes.MATERIAL_DTYPE)
                m["diffuse"][:3] = {"white": 0.73, "red": (0.63, 0.06, 0.04), "green": (0.15, 0.48, 0.09)}[name]
                m["ambient"][:3] = 1.0 if name == "white" else 0.0
                m["shininess"], m["ior"], m["dissolve"], m["illum"] = 10.0, 1.0, 1.0, 2
                r.add_material(m)
            mid = r.load_mesh(v, i, runs)
        r.set_grid_size(3.0)
        r.set_camera_transform(_look_at(np.array([0, 0.9, 3.0]), np.array([0, 0.9, 2.0]), (0, 1, 0)),
                               _perspective(45.0, 96 / 72, 0.1, 100.0))
        r.set_voxel_view_dir(7, 0.0)
        r.queue_model(mid)
        r.queue_point_light(scenes.point_light((0, 1.4, 0)))
        r.render()
        frames.append(r.read_frame().copy())
    np.testing.assert_array_equal(frames[0], frames[1])


@pytest.mark.gpu
def test_demo_frames_match_python_driver(vct, demo_bin, tmp_path):
    d = str(tmp_path)
    _write_box(d)
    _write_object(d)
    w, h, n = 160, 120, 64
    out = os.path.join(d, "frame")
    r = subprocess.run([demo_bin, "--assets", d, "--out", out, "--frames", "2", "--width", str(w), "--height",
                        str(h), "--grid", str(n), "--rotate", "0.5"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    f0, f1 = _read_ppm(out + "_0000.ppm"), _read_ppm(out + "_0001.ppm")
    assert f0.shape == (h, w, 3)
    assert (f0 != f1).any()  # the object turned

    rr = vct.Renderer(w, h, grid_res=n)
    box = rr.load_model(os.path.join(d, "CornellBox-Glossy.obj"))
    obj = rr.load_model(os.path.join(d, "suzanne.obj"))
    rr.set_model_material(rr.add_material(_demo_material()), obj)
    rr.set_grid_size(3.0)
    eye = np.array([0.0, 0.9, 3.0])
    yaw = math.radians(-90.0)
    rr.set_camera_transform(_look_at(eye, eye + np.array([math.cos(yaw), 0.0, math.sin(yaw)]), (0, 1, 0)),
                            _perspective(45.0, w / h, 0.1, 100.0))
    rr.set_voxel_view_dir(7, 0.0)
    model = np.eye(4)
    model[:3, :3] *= 0.3
    model[:3, 3] = (0.0, 1.1, -0.5)
    rr.set_model_transform(obj, model.T.reshape(-1).astype(np.float32))
    rr.set_model_transform(box, np.eye(4, dtype=np.float32).reshape(-1))
    rr.queue_model(box)
    rr.queue_model(obj)
    rr.queue_point_light(scenes.point_light((0, 1.4, 0)))
    rr.render()
    ref = rr.read_frame()[::-1, :, :3]  # row 0 = bottom; PPM rows run top-down
    q = psnr(f0 / 255.0, ref / 255.0)
    close = (np.abs(f0.astype(int) - ref.astype(int)).max(axis=2) <= 2).mean()
    print(f"demo vs Python driver: PSNR {q:.1f} dB, {100 * close:.2f}% of pixels within 2 LSB")
    assert q >= 40.0
    assert close >= 0.99
