"""FP32-mixed precision form against FP64.

FFTs, the nonlinear product and the RK3 arithmetic run in FP32; the compact
y-solves, the Helmholtz solve and the phase factors in FP64.  Tolerance: the
target of the precision form, relative L2 error of the fields at or below 1e-5
against FP64 after 100 steps (1e-6 after one step)."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2

pytestmark = pytest.mark.gpu
FIELDS = ("vor", "phi", "u00", "w00")


def _mixed(pp, nstep, seed=3):
    import shear_nnf_gb300 as sb
    p = sb.make_params(**pp)
    st = sb.seed_state(p, seed)
    box = sb.ShearBox(p, precision=sb.SB_MIXED)
    s = copy_state(st)
    tr, status = box.cross(s, nstep)
    return st, s, tr, status


def test_mixed_one_and_hundred_steps_vs_oracle_64():
    import oracle
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005)
    for nstep, tol in ((1, 1e-6), (100, 1e-5)):
        st0, sm, trm, status = _mixed(pp, nstep)
        so = copy_state(st0)
        tro, _ = oracle.Oracle(**pp).cross(so, nstep)
        err = {k: rel_l2(sm[k], so[k]) for k in FIELDS}
        assert max(err.values()) < tol, (nstep, err)
        assert status.steps_done == nstep
        for q in range(2, 12):  # UNER columns, scaled by each column's magnitude
            scale = np.abs(tro[:, q]).max()
            assert np.abs(trm[:, q] - tro[:, q]).max() <= 1e-5 * scale, q


def test_mixed_vs_fp64_192_hundred_steps():
    """The 192x96x96 configuration (Re_z = 4000, CFL = 0.5): mixed against the
    FP64 GPU path, which the oracle pins."""
    import shear_nnf_gb300 as sb
    pp = box_params(192, 96, 96, rez=4000.0, cfl=0.5)
    p = sb.make_params(**pp)
    st = sb.seed_state(p, 3)
    a = copy_state(st)
    b = copy_state(st)
    sb.ShearBox(p).cross(a, 100)
    sb.ShearBox(p, precision=sb.SB_MIXED).cross(b, 100)
    err = {k: rel_l2(b[k], a[k]) for k in FIELDS}
    assert max(err.values()) < 1e-5, err
    assert abs(a["time"] - b["time"]) / a["time"] < 1e-5


def test_mixed_batch_members_independent():
    """Boxes of one batch evolve independently: member results equal single-box runs."""
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005)
    p = sb.make_params(**pp)
    states = [sb.seed_state(p, 10 + m) for m in range(3)]
    box = sb.ShearBox(p, batch=3, precision=sb.SB_MIXED)
    for m, st in enumerate(states):
        box.set_state(st, m)
    box.step(5)
    for m, st in enumerate(states):
        single = copy_state(st)
        sb.ShearBox(p, precision=sb.SB_MIXED).cross(single, 5)
        got = box.get_state(m)
        for k in FIELDS:
            assert np.array_equal(got[k], single[k]), (m, k)
