"""bench.py's reference arm without a GPU: the JSON line it prints (its
timing stubbed, so the test takes no CPU frame), that ranks other than 0
exit without work under torchrun, and the timed FP32 frame of the CPU
restatement on a small scene."""
import json
import os
import sys
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def _run(bench, monkeypatch, argv, env=None):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    for k, v in (env or {}).items():
        monkeypatch.setenv(k, v)
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    return bench.main()


def test_reference_line(monkeypatch, capsys):
    bench = _bench()
    calls = []

    def frame(scene, threads, row_stride=1):  # -> (vox + mip + trace, per-stage ms)
        calls.append((threads, row_stride))
        n = len(calls)
        return 10.0 + n, [1.0, 2.0, 3.0, 7.0 + n]

    monkeypatch.setattr(bench, "cpu_frame_ms", frame)
    monkeypatch.setattr(bench, "_scene", lambda: SimpleNamespace(n_tris=499290))
    assert _run(bench, monkeypatch, ["--impl", "reference", "--steps", "2", "--warmup", "3"]) == 0
    out = capsys.readouterr().out.strip().splitlines()
    assert len(out) == 1, out
    line = json.loads(out[0])
    cores = os.cpu_count() or 1
    # three warm-up frames on every 64th row, then two whole frames, all host threads
    assert calls == [(cores, bench.CPU_WARMUP_ROW_STRIDE)] * 3 + [(cores, 1)] * 2
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] == 14.5                       # mean of the timed frames (14, 15)
    assert line["ms_per_step"] == 17.5                 # with the G-buffer raster
    assert line["stages_ms"] == {"voxelize": 1.0, "mipmap": 2.0, "gbuffer": 3.0, "trace": 11.5}
    assert (line["n_gpus"], line["steps"], line["warmup"]) == (1, 2, 3)
    assert line["higher_is_better"] is False and line["scaling"] == "weak" and line["vs_baseline"] is None
    assert line["dtype"] == "f32" and line["data"] == "synthetic" and line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["value"] == 14.5 and cb["unit"] == bench.UNIT and cb["cores"] == cores and cb["kind"] == "port"
    assert cb["sample"]
    assert line["e2e"] == {"value": 14.5, "unit": bench.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_other_ranks_exit_without_work(monkeypatch, capsys):
    bench = _bench()

    def frame(*a, **k):
        raise AssertionError("rank 1 timed a frame")

    monkeypatch.setattr(bench, "cpu_frame_ms", frame)
    monkeypatch.setattr(bench, "_scene", frame)
    env = {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}
    assert _run(bench, monkeypatch, ["--impl", "reference", "--gpus", "2", "--steps", "1"], env) == 0
    assert capsys.readouterr().out == ""


def test_timed_frame_small_scene(oracle):
    """The FP32 restatement the arm times: four stage times, the trace over
    every row_stride-th row."""
    from voxel_cone_tracing_gb300 import scenes
    s = scenes.scene_small(width=64, height=48)
    p = oracle.Params(grid_res=32, width=64, height=48, threads=2)
    for stride in (1, 16):
        ms = oracle.time_frame(s, p, stride)
        assert ms.shape == (4,) and np.all(np.isfinite(ms)) and np.all(ms >= 0.0)
        assert ms[0] > 0.0 and ms[3] > 0.0
