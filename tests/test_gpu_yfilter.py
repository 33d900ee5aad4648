"""GPU parity of the step with the compact y-filter (iydealiasing = 3) against
the CPU oracle, alone and with the LES model."""
import pytest

from conftest import box_params, copy_state, rel_l2
from test_gpu_step import _field_errors, _run_both, _trace_error

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("grid,kw", [((64, 32, 32), {"fixed_dt": 0.005}),
                                     ((96, 48, 48), {}),
                                     ((64, 32, 32), {"les": 1, "cs": 0.1})])
def test_filtered_step(grid, kw):
    pp = box_params(*grid, rez=4000.0, ydeal=3, **kw)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < 1e-12, err
    assert _trace_error(tr_g, tr_o) < 1e-10


def test_filtered_twenty_steps():
    pp = box_params(64, 32, 32, rez=4000.0, ydeal=3)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 20)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < 1e-10, err
    assert _trace_error(tr_g, tr_o) < 1e-10


def test_filtered_mixed_against_fp64():
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=4000.0, ydeal=3)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 4)
    out = {}
    for prec in (sb.SB_FP64, sb.SB_MIXED):
        st = copy_state(st0)
        sb.ShearBox(p, precision=prec).cross(st, 20)
        out[prec] = st
    err = max(rel_l2(out[sb.SB_MIXED][k], out[sb.SB_FP64][k]) for k in ("vor", "phi"))
    assert err < 1e-5, err
