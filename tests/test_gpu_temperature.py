"""GPU parity of the temperature variant crosst (itemperature = 1) against the
CPU oracle through the C-ABI: FP64 one-step and twenty-step runs with and
without shear, with the Smagorinsky stage (molecular terms kept or dropped),
the y filter and y dealiasing (which leave tb alone), the rest-state known
answer, the FP32-mixed form against FP64, a batch against single boxes, and
the largest grid.  Tolerances as for cross: relative L2 below
1e-12 after one step, statistics records to 1e-10."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2
from test_gpu_step import _trace_error
from test_temperature_oracle import REST, _rest_state, _rk3

pytestmark = pytest.mark.gpu

KEYS = ("vor", "phi", "u00", "w00", "tb", "tb00")
LZ = 2 * np.pi


def _temp(grid, rez, pr=0.7, bym=1.0, gbeta=0.5, **kw):
    return box_params(*grid, rez=rez, temperature=1, fkappa=LZ ** 2 / rez / pr, bym=bym,
                      gbeta=gbeta, **kw)


def _run_both(pp, nstep, seed=7, k0=4.0, precision=0):
    import oracle
    import shear_nnf_gb300 as sb
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, seed, k0=k0)
    st_o = copy_state(st0)
    tr_o, _ = oracle.Oracle(**pp).cross(st_o, nstep)
    box = sb.ShearBox(p, precision=precision)
    st_g = copy_state(st0)
    tr_g, status = box.cross(st_g, nstep)
    return st_o, tr_o, st_g, tr_g, status


def _errors(st_o, st_g):
    return {k: rel_l2(st_g[k], st_o[k]) for k in KEYS}


@pytest.mark.parametrize("grid,kw", [((64, 32, 32), {}),
                                     ((64, 32, 32), {"s": 0.0, "fixed_dt": 0.01}),
                                     ((96, 48, 48), {"bym": -0.5, "gbeta": 2.0}),
                                     ((64, 32, 32), {"les": 1, "les_visc": 1, "cs": 0.1}),
                                     ((64, 32, 32), {"les": 1, "les_visc": 0, "cs": 0.1}),
                                     ((64, 32, 32), {"ydeal": 3}),
                                     ((64, 32, 32), {"ydeal": 2})])
def test_temperature_one_step(grid, kw):
    pp = _temp(grid, 4000.0, **kw)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _errors(st_o, st_g)
    assert max(err.values()) < 1e-12, err
    assert tr_g.shape == tr_o.shape == (1, 29)
    assert _trace_error(tr_g, tr_o) < 1e-10
    assert status.steps_done == 1


def test_temperature_twenty_steps():
    pp = _temp((64, 32, 32), 4000.0)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 20)
    err = _errors(st_o, st_g)
    assert max(err.values()) < 1e-10, err
    assert _trace_error(tr_g, tr_o) < 1e-10
    assert status.steps_done == 20


def test_temperature_stop_from_second_step():
    pp = _temp((64, 32, 32), 4000.0, etime=1e-3)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 4)
    assert len(tr_g) == len(tr_o) == 1
    assert status.steps_done == 1 and status.istop == 1
    assert max(_errors(st_o, st_g).values()) < 1e-12


def test_rest_known_answer_gpu():
    import oracle
    import shear_nnf_gb300 as sb
    kappa, gbeta, dt, n = 0.01, 0.7, 0.05, 6
    pp = dict(REST, fixed_dt=dt, fkappa=kappa, gbeta=gbeta)
    o = oracle.Oracle(**pp)
    amp = 1e-7
    st = _rest_state(o, amp, 0.0)
    tr, _ = sb.ShearBox(sb.make_params(**pp)).cross(st, n)
    k2 = pp["alp"] ** 2
    A = np.array([[-kappa * k2, 0.0], [-gbeta * k2, -k2 / pp["Re"]]])
    T_n, phi_n = _rk3(dt * A, n) @ np.array([amp, 0.0])
    np.testing.assert_allclose(st["tb"][0, 1, :], T_n, rtol=1e-9, atol=0)
    np.testing.assert_allclose(st["phi"][0, 1, :], phi_n, rtol=1e-7, atol=0)
    assert tr[0, 24] == pytest.approx(2 * amp, rel=1e-12)
    assert tr[0, 25] == pytest.approx(np.sqrt(2) * amp, rel=1e-12)


def test_temperature_mixed_against_fp64():
    import shear_nnf_gb300 as sb
    pp = _temp((96, 48, 48), 4000.0)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 7)
    a, b = copy_state(st0), copy_state(st0)
    sb.ShearBox(p).cross(a, 20)
    sb.ShearBox(p, precision=sb.SB_MIXED).cross(b, 20)
    err = {k: rel_l2(b[k], a[k]) for k in KEYS}
    assert max(err.values()) < 1e-4, err


def test_temperature_batch_matches_single():
    import shear_nnf_gb300 as sb
    pp = _temp((64, 32, 32), 4000.0)
    p = sb.make_params(**pp)
    states = [sb.seed_state(p, s) for s in (1, 2, 3)]
    box = sb.ShearBox(p, batch=3)
    for m, st in enumerate(states):
        box.set_state(st, m)
    box.step(5)
    for m, st in enumerate(states):
        one = copy_state(st)
        sb.ShearBox(p).cross(one, 5)
        got = box.get_state(m)
        for k in KEYS:
            assert np.array_equal(got[k], one[k]), (m, k)


def test_temperature_largest_grid():
    pp = _temp((384, 192, 192), 20000.0)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1, k0=6.0)
    err = _errors(st_o, st_g)
    assert max(err.values()) < 1e-12, err
    assert _trace_error(tr_g, tr_o) < 1e-10


def test_temperature_autotune_and_physical():
    import shear_nnf_gb300 as sb
    pp = _temp((192, 96, 96), 4000.0)
    p = sb.make_params(**pp)
    st = sb.seed_state(p, 7)
    box = sb.ShearBox(p)
    box.set_state(st)
    choice = box.autotune()
    assert choice["p3_cols"] in (4, 8)
    box.set_state(st)
    box.step(2)
    a = box.get_state()
    ref = copy_state(st)
    sb.ShearBox(p).cross(ref, 2)
    assert max(rel_l2(a[k], ref[k]) for k in KEYS) < 1e-13
    f = box.physical(fields=("u", "Q"))
    assert np.all(np.isfinite(f["u"])) and np.all(np.isfinite(f["Q"]))
