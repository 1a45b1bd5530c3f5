"""The oracle against its committed golden fixtures (tests/golden/*.npz,
made by tests/golden/make_golden.py): voxel maps, counts and visible
triangle ids bit-exact, radiance to 1e-6."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("name", ["small_ref_aniso", "small_sat_iso_six", "sphere_ref_aniso"])
def test_oracle_matches_golden(oracle, name):
    from tests.golden import make_golden
    gold = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    out = make_golden.compute(name)
    for k in ("level0", "counts", "chains", "tri_id"):
        np.testing.assert_array_equal(out[k], gold[k], err_msg=k)
    np.testing.assert_allclose(out["frame"], gold["frame"], atol=1e-6, rtol=0)
    assert gold["counts"].sum() > 0
