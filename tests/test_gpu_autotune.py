"""The plane-stage autotuner picks tiles that compute the same step."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("grid,prec", [((64, 32, 32), 0), ((192, 96, 96), 0), ((96, 48, 48), 1)])
def test_autotune_keeps_the_step(grid, prec):
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(*grid, rez=4000.0))
    st0 = sb.seed_state(p, 9)
    ref = sb.ShearBox(p, precision=prec)
    a = copy_state(st0)
    tr_a, _ = ref.cross(a, 5)
    box = sb.ShearBox(p, precision=prec)
    box.set_state(st0)
    choice = box.autotune()
    assert choice["p1_cols"] in (4, 8) and choice["p3_cols"] in (4, 8) and choice["p2_threads"] >= 64
    b = copy_state(st0)
    tr_b, _ = box.cross(b, 5)
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < 1e-13, k
    np.testing.assert_allclose(tr_b, tr_a, rtol=1e-11, atol=1e-300)
