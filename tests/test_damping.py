"""Window damping of the mean streamwise forcing (iadd_damping = 1,
add_damping, operators.f90:42-84; called by cross.f90:625-626 and
crosst.f90:694-695): rf0u -= damp_up Hw(y) u00 with
Hw = 1 - (1 + tanh(6 (aa - y)/Lz + 3)) (1 + tanh(6 (aa + y)/Lz + 3)) / 4 and
aa = Lz damp_aa.  Known answer on the oracle: with no fluctuations and a
vanishing viscosity every point of u00 decays as the RK3 amplification of
u' = -damp_up Hw(y) u, and w00 is left alone.  GPU: the step against the
oracle with the damping on (FP64 one and twenty steps, crosst, FP32-mixed
against FP64)."""
import numpy as np
import pytest

import oracle
import shear_nnf_gb300 as sb
from conftest import box_params, copy_state, rel_l2

LZ = 2 * np.pi


def _hw(y, aa, lz=LZ):
    return 1.0 - (0.25 * (1.0 + np.tanh(6.0 * (aa - y) / lz + 3.0))) * \
        (1.0 + np.tanh(6.0 * (aa + y) / lz + 3.0))


def test_window_function_shape():
    y = np.linspace(-np.pi / 2, np.pi / 2, 101)
    hw = _hw(y, 0.25 * LZ)
    assert hw.min() >= 0.0 and hw.max() <= 1.0
    assert hw[50] < 1e-3 and np.allclose(hw, hw[::-1], atol=1e-15)


def test_mean_decay_known_answer():
    pp = box_params(32, 32, 32, rez=1e15 * LZ ** 2, fixed_dt=0.02, keep_laminar=1, s=0.0,
                    damping=1, damp_up=0.8, damp_aa=0.05)
    o = oracle.Oracle(**pp)
    my, Ly = pp["my"], pp["Ly"]
    y = np.arange(my) * (Ly / my) - 0.5 * Ly
    z = np.zeros((o.mz, o.nkx, my), np.complex128)
    u0 = 0.3 * np.cos(2 * np.pi * y / Ly) + 0.1
    w0 = 0.2 * np.sin(2 * np.pi * y / Ly)
    st = {"vor": z.copy(), "phi": z.copy(), "u00": u0.copy(), "w00": w0.copy(), "time": 0.0,
          "xoffb": 0.0, "xofft": 0.0}
    n = 5
    o.cross(st, n)
    zz = -0.02 * 0.8 * _hw(y, 0.05 * LZ)
    g = 1 + zz + zz ** 2 / 2 + zz ** 3 / 6
    np.testing.assert_allclose(st["u00"], g ** n * u0, rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(st["w00"], w0, rtol=1e-10, atol=1e-14)
    assert np.abs(st["u00"] - u0).max() > 1e-3  # the damping acted


def test_damping_off_leaves_the_step():
    pp = box_params(32, 32, 32, rez=1000.0, fixed_dt=0.01)
    st = sb.seed_state(sb.make_params(**pp), 4)
    a, b = copy_state(st), copy_state(st)
    oracle.Oracle(**pp).cross(a, 2)
    oracle.Oracle(**dict(pp, damping=0, damp_up=5.0, damp_aa=0.2)).cross(b, 2)
    for k in ("vor", "phi", "u00", "w00"):
        assert np.array_equal(a[k], b[k]), k


def test_invalid_damping_rejected():
    p = sb.make_params(**box_params(32, 32, 32, rez=1000.0, damping=2))
    with pytest.raises(RuntimeError):
        sb.ShearBox(p)


DAMP = dict(damping=1, damp_up=0.5, damp_aa=0.1)


def _gpu_vs_oracle(pp, nstep, seed=3, precision=0):
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, seed)
    a, b = copy_state(st0), copy_state(st0)
    tr_o, _ = oracle.Oracle(**pp).cross(a, nstep)
    tr_g, _ = sb.ShearBox(p, precision=precision).cross(b, nstep)
    keys = ("vor", "phi", "u00", "w00") + (("tb", "tb00") if pp.get("temperature") else ())
    return {k: rel_l2(b[k], a[k]) for k in keys}, tr_o, tr_g


@pytest.mark.gpu
@pytest.mark.parametrize("nstep,tol", [(1, 1e-12), (20, 1e-10)])
def test_gpu_damping_matches_oracle(nstep, tol):
    pp = box_params(64, 32, 32, rez=4000.0, **DAMP)
    err, tr_o, tr_g = _gpu_vs_oracle(pp, nstep)
    assert max(err.values()) < tol, err
    assert np.allclose(tr_g, tr_o, rtol=1e-9, atol=1e-14)


@pytest.mark.gpu
def test_gpu_damping_crosst():
    pp = box_params(64, 32, 32, rez=4000.0, temperature=1, fkappa=LZ ** 2 / 4000 / 0.7, bym=1.0,
                    gbeta=0.5, **DAMP)
    err, _, _ = _gpu_vs_oracle(pp, 1)
    assert max(err.values()) < 1e-12, err


@pytest.mark.gpu
def test_gpu_damping_mixed_against_fp64():
    pp = box_params(96, 48, 48, rez=4000.0, **DAMP)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 7)
    a, b = copy_state(st0), copy_state(st0)
    sb.ShearBox(p).cross(a, 10)
    sb.ShearBox(p, precision=sb.SB_MIXED).cross(b, 10)
    err = {k: rel_l2(b[k], a[k]) for k in ("vor", "phi", "u00", "w00")}
    assert max(err.values()) < 1e-5, err
