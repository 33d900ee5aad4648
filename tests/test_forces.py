"""Body forces of cross (iadd_force, cross.f90:610-624; crosst.f90:680-693):
1 / 2 add the one- / two-pair streamwise-roll force to hv(kx=0, kz=1)
(add_force, operators.f90:1-40), -1 the inertial force xforce to the mean
streamwise forcing rf0u.  Known answers on the oracle: with the fluid at rest,
a vanishing viscosity and a small force, phi(kx=0, kz=1) grows as t F(y) and
u00 as t xforce (an RK3 step integrates a constant right-hand side exactly).
GPU: the step against the oracle with each force on, and with the temperature."""
import numpy as np
import pytest

import oracle
import shear_nnf_gb300 as sb
from conftest import box_params, copy_state, rel_l2


def _roll(y, amp, gam, which):
    w = 1.0 - y * y
    if which == 1:
        return -0.5 * amp * (-4.0 * (1.0 - 3.0 * y * y) - gam * gam * w * w)
    return 0.5 * amp * (4.0 * y * (-3.0 + 5.0 * y * y) - y * w * w * gam * gam)


def _rest(o, my, u0=None):
    z = np.zeros((o.mz, o.nkx, my), np.complex128)
    return {"vor": z.copy(), "phi": z.copy(), "u00": np.zeros(my) if u0 is None else u0.copy(),
            "w00": np.zeros(my), "time": 0.0, "xoffb": 0.0, "xofft": 0.0}


@pytest.mark.parametrize("which", [1, 2])
def test_roll_force_known_answer(which):
    amp, dt, n = 1e-9, 0.02, 4
    pp = box_params(32, 32, 32, rez=1e15 * (2 * np.pi) ** 2, fixed_dt=dt, keep_laminar=1,
                    s=0.0, force=which, force_roll=amp)
    o = oracle.Oracle(**pp)
    my, Ly = pp["my"], pp["Ly"]
    y = np.arange(my) * (Ly / my) - 0.5 * Ly
    st = _rest(o, my)
    o.cross(st, n)
    F = _roll(y, amp, pp["gam"], which)
    np.testing.assert_allclose(st["phi"][1, 0, :].real, n * dt * F, rtol=1e-7,
                               atol=1e-6 * np.abs(n * dt * F).max())
    others = st["phi"].copy()
    others[1, 0, :] = 0.0
    assert np.abs(others).max() <= 1e-6 * np.abs(F).max() * n * dt


def test_xforce_known_answer():
    dt, n, xf = 0.02, 5, 0.3
    pp = box_params(32, 32, 32, rez=1e15 * (2 * np.pi) ** 2, fixed_dt=dt, keep_laminar=1,
                    s=0.0, force=-1, xforce=xf)
    o = oracle.Oracle(**pp)
    my = pp["my"]
    u0 = 0.1 * np.cos(2 * np.pi * np.arange(my) / my)
    st = _rest(o, my, u0)
    o.cross(st, n)
    np.testing.assert_allclose(st["u00"], u0 + n * dt * xf, rtol=1e-12)
    assert np.all(st["w00"] == 0.0)


def test_invalid_force_rejected():
    p = sb.make_params(**box_params(32, 32, 32, rez=1000.0, force=3))
    with pytest.raises(RuntimeError):
        sb.ShearBox(p)


def _gpu_vs_oracle(pp, nstep, seed=5):
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, seed)
    a, b = copy_state(st0), copy_state(st0)
    oracle.Oracle(**pp).cross(a, nstep)
    sb.ShearBox(p).cross(b, nstep)
    keys = ("vor", "phi", "u00", "w00") + (("tb", "tb00") if pp.get("temperature") else ())
    return {k: rel_l2(b[k], a[k]) for k in keys}


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(force=1, force_roll=0.05), dict(force=2, force_roll=0.05),
                                dict(force=-1, xforce=0.02),
                                dict(force=1, force_roll=0.05, damping=1, damp_up=0.5,
                                     damp_aa=0.1)])
def test_gpu_forces_match_oracle(kw):
    pp = box_params(64, 32, 32, rez=4000.0, **kw)
    err = _gpu_vs_oracle(pp, 1)
    assert max(err.values()) < 1e-12, err
    err = _gpu_vs_oracle(pp, 10)
    assert max(err.values()) < 1e-10, err


@pytest.mark.gpu
def test_gpu_forces_crosst():
    lz = 2 * np.pi
    pp = box_params(64, 32, 32, rez=4000.0, temperature=1, fkappa=lz ** 2 / 4000 / 0.7, bym=1.0,
                    gbeta=0.5, force=2, force_roll=0.05)
    err = _gpu_vs_oracle(pp, 1)
    assert max(err.values()) < 1e-12, err
