"""GPU parity of the full RK3 step against the CPU oracle, through the C-ABI.

Tolerances are the FP64 drop-in bar: relative L2 of vor, phi, u00, w00 below
1e-12 after one step and below 1e-9 after 100 steps; UNER traces to 1e-10."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2

pytestmark = pytest.mark.gpu

ONE_STEP = 1e-12
MANY_STEPS = 1e-9
TRACE_TOL = 1e-10


def _run_both(pp, nstep, seed=3, k0=4.0):
    import oracle
    import shear_nnf_gb300 as sb
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, seed, k0=k0)
    st_o = copy_state(st0)
    o = oracle.Oracle(**pp)
    tr_o, istop_o = o.cross(st_o, nstep)
    box = sb.ShearBox(p)
    st_g = copy_state(st0)
    tr_g, status = box.cross(st_g, nstep)
    return st_o, tr_o, st_g, tr_g, status


def _field_errors(st_o, st_g):
    return {k: rel_l2(st_g[k], st_o[k]) for k in ("vor", "phi", "u00", "w00")}


def _trace_error(tr_g, tr_o):
    assert tr_g.shape == tr_o.shape
    cols = [q for q in range(tr_o.shape[1]) if np.abs(tr_o[:, q]).max() > 0]
    return max(float(np.max(np.abs(tr_g[:, q] - tr_o[:, q]) / np.maximum(np.abs(tr_o[:, q]), 1e-300)))
               for q in cols)


@pytest.mark.parametrize("grid", [(64, 32, 32), (96, 48, 48)])
def test_one_step_fixed_dt(grid):
    pp = box_params(*grid, rez=1000.0, fixed_dt=0.005)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 1 and status.istop == 0
    assert abs(st_g["time"] - st_o["time"]) < 1e-15


def test_one_step_cfl_192():
    pp = box_params(192, 96, 96, rez=4000.0, cfl=0.5)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL


def test_hundred_steps_64():
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 100)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < MANY_STEPS, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 100


def test_hundred_steps_benchmark_box():
    """The benchmark configuration itself (192x96x96, Re_z 4000, CFL 0.5, the
    seed of the bench): the drop-in bar after 100 steps, with every record of
    the UNER trace."""
    pp = box_params(192, 96, 96, rez=4000.0, cfl=0.5)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 100, seed=3)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < MANY_STEPS, err
    assert tr_g.shape[0] == 100
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 100 and status.istop == 0
    assert abs(st_g["time"] - st_o["time"]) < 1e-12 * st_o["time"]


def test_twenty_steps_largest_grid():
    """384x192x192 without LES (Re_z 20000, k0 6), 20 CFL steps."""
    pp = box_params(384, 192, 192, rez=20000.0, cfl=0.5)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 20, seed=6, k0=6.0)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < MANY_STEPS, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 20


@pytest.mark.parametrize("les", [0, 1])
def test_one_step_largest_grid(les):
    # the largest transform lengths (x 384, z 192) and my = 192, with and
    # without the LES stage
    pp = box_params(384, 192, 192, rez=20000.0, cfl=0.5, les=les, cs=0.1)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1, k0=6.0)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
