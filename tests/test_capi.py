"""The C-ABI library: builds, loads and exports every entry point that
include/vct.h declares; host-side error behaviour that needs no GPU."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "vct.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vct_[a-z0-9_]+)\s*\(", src)))


def test_header_declarations_match_binding(vct):
    assert _declared() == sorted(vct.EXPORTS)


def test_library_exports_every_declared_symbol(vct):
    lib = vct.lib()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", vct.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(vct_[a-z0-9_]+)\b", out))
    assert set(_declared()) <= exported


def test_library_is_sm103a_build(vct):
    """The shipped kernels are compiled for sm_103a only (no PTX JIT fallback)."""
    from voxel_cone_tracing_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_config_default_matches_reference(vct):
    c = vct.default_config()
    assert c.grid_res == 128  # set_grid_resolution(128), renderer.cpp:146
    assert c.mip_mode == vct.MIP_ANISO and c.vox_mode == vct.VOX_REF_RASTER2X


def test_status_strings(vct):
    assert vct.lib().vct_status_string(0) == b"ok"
    assert vct.lib().vct_status_string(2) == b"invalid id"


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_no_device_is_reported_not_faked(vct):
    """Without a GPU the engine refuses to run (there is no CPU fallback)."""
    with pytest.raises(vct.VCTError) as e:
        vct.Renderer(16, 16)
    assert e.value.status == 7
    with pytest.raises(vct.VCTError):
        vct.create_tex_3d(8, 8, 8, 1)


def test_bad_config_rejected_before_device(vct):
    with pytest.raises(vct.VCTError) as e:
        vct.Renderer(16, 16, grid_res=100)
    assert e.value.status == 1
    with pytest.raises(vct.VCTError) as e:
        vct.Renderer(0, 16)
    assert e.value.status == 1
    with pytest.raises(vct.VCTError) as e:
        vct.Renderer(16, 16, mip_mode=vct.MIP_BOTH + 1)
    assert e.value.status == 1
    # every switch of vct_config is 0 or 1
    for field in ("shadow_from_maps", "full_march", "overlap_raster", "far_share", "trace_tile_rows"):
        with pytest.raises(vct.VCTError) as e:
            vct.Renderer(16, 16, **{field: 2})
        assert e.value.status == 1, field


def test_config_defaults_of_the_engine_switches(vct):
    """The engine's own switches default to the fastest path: alpha-only
    shadow chains, cone exit and empty-space skip on (all exact), one stream,
    and shared far fields of the diffuse cones for the texture-unit sampler."""
    c = vct.default_config()
    assert (c.shadow_from_maps, c.full_march, c.overlap_raster, c.far_share) == (0, 0, 0, 1)
    assert c.trace_tile_rows == 0  # 16-row tiles
    assert list(c.reserved) == [0, 0]


def test_cpp_facade_header_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "vct_renderer.hpp"\nint main(){ vct::mat4 m = vct::mat4::identity(); (void)m; return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
