"""Transform lengths beyond the benchmark configurations: powers of two (128,
256), 5 x 2^k (80, 160, 320, with a radix-5 first stage) and mgalz = 384 (plane
stage 3 with 4 columns per block), in x and z, against
the oracle (whose mixed-radix FFT covers them): the step (FP64 one step and ten
steps, the FP32-mixed form), the LES stages (their x and z transforms) and the
physical fields (the x transform of convh5's fields)."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2
from test_gpu_step import ONE_STEP, TRACE_TOL, _field_errors, _run_both, _trace_error

pytestmark = pytest.mark.gpu

GRIDS = [(80, 32, 80), (128, 64, 128), (160, 48, 160), (256, 32, 256), (320, 32, 160),
         (128, 48, 80), (192, 32, 384)]


@pytest.mark.parametrize("grid", GRIDS)
def test_one_step(grid):
    pp = box_params(*grid, rez=2000.0, cfl=0.5)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL


@pytest.mark.parametrize("grid", [(128, 64, 128), (160, 48, 160)])
def test_ten_steps(grid):
    pp = box_params(*grid, rez=2000.0, fixed_dt=0.004)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 10)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < 1e-11, err
    assert status.steps_done == 10


@pytest.mark.parametrize("grid", [(128, 64, 128), (160, 48, 80)])
def test_mixed_close_to_fp64(grid):
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(*grid, rez=2000.0))
    st0 = sb.seed_state(p, 6)
    a, b = copy_state(st0), copy_state(st0)
    sb.ShearBox(p).cross(a, 10)
    sb.ShearBox(p, precision=sb.SB_MIXED).cross(b, 10)
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < 1e-5, k


@pytest.mark.parametrize("grid", [(128, 48, 128), (160, 48, 80), (96, 32, 384)])
def test_les_one_step(grid):
    pp = box_params(*grid, rez=4000.0, les=1, les_visc=1, cs=0.1)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err


def test_physical_fields():
    import oracle
    import shear_nnf_gb300 as sb
    kw = box_params(160, 32, 80, 2000.0)
    p = sb.make_params(**kw)
    st = sb.seed_state(p, 5)
    names = sb.ShearBox.PHYSICAL
    ref = dict(zip(names, oracle.Oracle(**kw).physical(st, 0x7FF)))
    box = sb.ShearBox(p)
    box.set_state(st)
    got = box.physical(0)
    for k in names:
        err = np.linalg.norm(got[k] - ref[k]) / max(np.linalg.norm(ref[k]), 1e-300)
        assert err < 1e-12, (k, err)


def test_temperature_refused_beyond_256_in_z():
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(96, 32, 384, rez=2000.0, temperature=1, fkappa=0.01))
    with pytest.raises(sb.ShearBoxError):
        sb.ShearBox(p)


@pytest.mark.parametrize("implicit", [0, 1])
def test_shortest_lines(implicit):
    """my = 16, the shortest y line (two segments of six banded rows), in
    both integrators, ten steps against the oracle."""
    import oracle
    import shear_nnf_gb300 as sb
    pp = box_params(32, 16, 32, rez=1000.0, fixed_dt=0.005)
    p = sb.make_params(**pp, implicit_visc=implicit)
    st0 = sb.seed_state(p, 8)
    a, b = copy_state(st0), copy_state(st0)
    oracle.Oracle(**pp, implicit_visc=implicit).cross(a, 10)
    box = sb.ShearBox(p)
    box.set_line_segments(2)
    box.cross(b, 10)
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < 1e-11, k


def test_longest_lines():
    """my = 448, the longest y line: the fused block does not fit in shared
    memory, so the split y-line kernels run (and the semi-implicit branch,
    which needs the fused block, is refused)."""
    import shear_nnf_gb300 as sb
    pp = box_params(32, 448, 32, rez=1000.0, fixed_dt=0.002)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert sb.ShearBox(sb.make_params(**pp)).tuning()["line_form"] == "split"
    with pytest.raises(sb.ShearBoxError):
        sb.ShearBox(sb.make_params(**pp, implicit_visc=1))
