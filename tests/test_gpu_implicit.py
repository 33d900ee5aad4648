"""GPU parity of the semi-implicit viscous branch (implicit_visc = 1, the
reference's explicit = 0, cross.f90:797-989, and crosst's with the scalar,
crosst.f90:916-1195) against the oracle: the drop-in bar of the explicit step
(1e-12 after one step, 1e-9 after 100, traces to 1e-10), for every y-line
tile, with the CFL rule and past the explicit viscous limit, in batches and
in the FP32-mixed form."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2
from test_gpu_step import MANY_STEPS, ONE_STEP, TRACE_TOL, _field_errors, _trace_error

pytestmark = pytest.mark.gpu


def _run_both(pp, nstep, seed=3, nseg=None, k0=4.0):
    import oracle
    import shear_nnf_gb300 as sb
    p = sb.make_params(**pp, implicit_visc=1)
    st0 = sb.seed_state(p, seed, k0=k0)
    st_o = copy_state(st0)
    tr_o, _ = oracle.Oracle(**pp, implicit_visc=1).cross(st_o, nstep)
    box = sb.ShearBox(p)
    assert box.tuning()["line_form"] == "implicit"
    if nseg:
        box.set_line_segments(nseg)
    st_g = copy_state(st0)
    tr_g, status = box.cross(st_g, nstep)
    return st_o, tr_o, st_g, tr_g, status


@pytest.mark.parametrize("grid", [(64, 32, 32), (96, 48, 48)])
def test_one_step(grid):
    pp = box_params(*grid, rez=1000.0, fixed_dt=0.005)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 1


@pytest.mark.parametrize("nseg", [1, 2, 3])
def test_hundred_steps_cfl(nseg):
    """100 CFL steps at 64x32x32 with 1, 2 or 3 warps per line solve."""
    pp = box_params(64, 32, 32, rez=1000.0, cfl=0.5)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 100, nseg=nseg)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < MANY_STEPS, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 100


def test_one_step_192():
    pp = box_params(192, 96, 96, rez=4000.0, cfl=0.5)
    st_o, tr_o, st_g, tr_g, _ = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < ONE_STEP, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL


def test_beyond_the_explicit_viscous_limit():
    """A low Reynolds number and a step 20 times the explicit viscous limit:
    the semi-implicit branch stays bounded and on the oracle."""
    pp = box_params(64, 32, 32, rez=20.0, fixed_dt=0.05, keep_laminar=1)
    st_o, tr_o, st_g, tr_g, _ = _run_both(pp, 40)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < MANY_STEPS, err
    assert all(np.all(np.isfinite(st_g[k])) for k in ("vor", "phi"))


def test_batch_members_match_single_runs():
    """Three boxes with their own Reynolds numbers (their own dtr1 and
    factor tables) equal the single-box runs."""
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, cfl=0.5)
    p = sb.make_params(**pp, implicit_visc=1)
    lz = 2 * np.pi
    res = [500.0, 1000.0, 2000.0]
    sts = [sb.seed_state(p, 20 + m) for m in range(3)]
    box = sb.ShearBox(p, batch=3)
    for m in range(3):
        box.set_state(sts[m], m)
        box.set_re(m, res[m] / lz ** 2)
    box.step(10)
    for m in range(3):
        single = sb.ShearBox(sb.make_params(**dict(pp, Re=res[m] / lz ** 2), implicit_visc=1))
        single.set_state(sts[m])
        single.step(10)
        a, b = box.get_state(m), single.get_state(0)
        for k in ("vor", "phi", "u00", "w00"):
            assert rel_l2(a[k], b[k]) < 1e-13, (m, k)


def test_mixed_form_close_to_fp64():
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, cfl=0.5)
    p = sb.make_params(**pp, implicit_visc=1)
    st0 = sb.seed_state(p, 5)
    out = []
    for prec in (0, 1):
        s = copy_state(st0)
        sb.ShearBox(p, precision=prec).cross(s, 20)
        out.append(s)
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(out[1][k], out[0][k]) < 1e-5, k


def test_refused_combinations():
    import shear_nnf_gb300 as sb
    for kw in ({"les": 1}, {"temperature": 1, "fkappa": 0.0}, {"ydeal": 3}):
        p = sb.make_params(**box_params(64, 32, 32, rez=1000.0, **kw), implicit_visc=1)
        with pytest.raises(sb.ShearBoxError):
            sb.ShearBox(p)


# ---- crosst's semi-implicit branch (the scalar on a third pipeline)

def _run_both_t(pp, nstep, seed=7, nseg=None, precision=0):
    import oracle
    import shear_nnf_gb300 as sb
    p = sb.make_params(**pp, implicit_visc=1)
    st0 = sb.seed_state(p, seed)
    st_o = copy_state(st0)
    tr_o, _ = oracle.Oracle(**pp, implicit_visc=1).cross(st_o, nstep)
    box = sb.ShearBox(p, precision=precision)
    if nseg:
        box.set_line_segments(nseg)
    st_g = copy_state(st0)
    tr_g, status = box.cross(st_g, nstep)
    return st_o, tr_o, st_g, tr_g, status


@pytest.mark.parametrize("grid,kw", [((64, 32, 32), {}),
                                     ((64, 32, 32), {"s": 0.0, "fixed_dt": 0.01}),
                                     ((96, 48, 48), {"bym": -0.5, "gbeta": 2.0})])
def test_crosst_one_step(grid, kw):
    from test_gpu_temperature import KEYS, _temp
    pp = _temp(grid, 4000.0, **kw)
    st_o, tr_o, st_g, tr_g, status = _run_both_t(pp, 1)
    err = {k: rel_l2(st_g[k], st_o[k]) for k in KEYS}
    assert max(err.values()) < ONE_STEP, err
    assert tr_g.shape == tr_o.shape == (1, 29)
    assert _trace_error(tr_g, tr_o) < TRACE_TOL


@pytest.mark.parametrize("nseg", [1, 2])
def test_crosst_fifty_steps(nseg):
    from test_gpu_temperature import KEYS, _temp
    pp = _temp((64, 32, 32), 4000.0)
    st_o, tr_o, st_g, tr_g, status = _run_both_t(pp, 50, nseg=nseg)
    err = {k: rel_l2(st_g[k], st_o[k]) for k in KEYS}
    assert max(err.values()) < MANY_STEPS, err
    assert _trace_error(tr_g, tr_o) < TRACE_TOL
    assert status.steps_done == 50


def test_crosst_rest_known_answer_gpu():
    """The rest-state recurrence of tests/test_oracle_implicit.py on the GPU:
    semi-implicit diffusion of tb, explicit buoyancy into phi."""
    import oracle
    import shear_nnf_gb300 as sb
    from test_oracle_implicit import _rest_scalar_recurrence
    from test_temperature_oracle import BASE, REST, _rest_state
    kappa, gbeta, dt, n = 0.05, 0.7, 0.2, 6
    pp = dict(REST, fixed_dt=dt, fkappa=kappa, gbeta=gbeta)
    o = oracle.Oracle(**pp, implicit_visc=1)
    p = sb.make_params(**pp, implicit_visc=1)
    # the line alone (a mean profile would couple to it through v dtb00/dy)
    st = _rest_state(o, 1e-7, 0.0)
    sb.ShearBox(p).cross(st, n)
    k2 = BASE["alp"] ** 2
    T_n, phi_n = _rest_scalar_recurrence(1e-7, 0.0, n, dt, kappa, 1.0 / BASE["Re"], k2, gbeta)
    np.testing.assert_allclose(st["tb"][0, 1, :], T_n, rtol=1e-11, atol=0)
    np.testing.assert_allclose(st["phi"][0, 1, :], phi_n, rtol=1e-9, atol=0)
    # the mean profile alone
    from test_oracle_implicit import _gain
    st = _rest_state(o, 0.0, 0.3)
    tb00_0 = st["tb00"].copy()
    sb.ShearBox(p).cross(st, n)
    lam = kappa * o.derivyc(tb00_0, iord=2)[0] / tb00_0[0]
    np.testing.assert_allclose(st["tb00"], _gain(lam, dt) ** n * tb00_0, rtol=1e-10, atol=1e-14)


def test_crosst_mixed_close_to_fp64():
    import shear_nnf_gb300 as sb
    from test_gpu_temperature import KEYS, _temp
    pp = _temp((64, 32, 32), 4000.0)
    p = sb.make_params(**pp, implicit_visc=1)
    st0 = sb.seed_state(p, 7)
    out = []
    for prec in (0, 1):
        s = copy_state(st0)
        sb.ShearBox(p, precision=prec).cross(s, 20)
        out.append(s)
    err = {k: rel_l2(out[1][k], out[0][k]) for k in KEYS}
    assert max(err.values()) < 1e-4, err


def test_crosst_batch_members_match_single_runs():
    """Three crosst boxes with their own Reynolds numbers on the
    three-pipeline line kernel equal the single-box runs."""
    import shear_nnf_gb300 as sb
    from test_gpu_temperature import KEYS, _temp
    pp = _temp((64, 32, 32), 4000.0)
    p = sb.make_params(**pp, implicit_visc=1)
    lz = 2 * np.pi
    res = [2000.0, 4000.0, 8000.0]
    sts = [sb.seed_state(p, 30 + m) for m in range(3)]
    box = sb.ShearBox(p, batch=3)
    for m in range(3):
        box.set_state(sts[m], m)
        box.set_re(m, res[m] / lz ** 2)
    box.step(8)
    for m in range(3):
        single = sb.ShearBox(sb.make_params(**dict(pp, Re=res[m] / lz ** 2), implicit_visc=1))
        single.set_state(sts[m])
        single.step(8)
        a, b = box.get_state(m), single.get_state(0)
        for k in KEYS:
            assert rel_l2(a[k], b[k]) < 1e-13, (m, k)


@pytest.mark.parametrize("temperature", [0, 1])
def test_autotune_keeps_the_implicit_step(temperature):
    import shear_nnf_gb300 as sb
    from test_gpu_temperature import _temp
    pp = _temp((64, 32, 32), 4000.0) if temperature else box_params(64, 32, 32, rez=4000.0)
    p = sb.make_params(**pp, implicit_visc=1)
    st0 = sb.seed_state(p, 12)
    ref = sb.ShearBox(p)
    a = copy_state(st0)
    ref.cross(a, 5)
    box = sb.ShearBox(p)
    box.set_state(st0)
    choice = box.autotune()
    assert choice["line_form"] == "implicit"
    b = copy_state(st0)
    box.cross(b, 5)
    tol = 1e-13 if choice["line_segments"] == ref.tuning()["line_segments"] else 1e-11
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < tol, k
