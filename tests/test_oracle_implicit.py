"""Known answers for the oracle's semi-implicit viscous branch (explicit = 0,
cross.f90:797-989).  With the nonlinear terms zero (single plane waves,
unidirectional mean flows) the branch is the scalar recurrence
    f_k (1 - beta_k Dt lam) = f_{k-1} (1 + alpha_k Dt lam)
per substep, lam = -nu (k^2 + kappa^2) with kappa^2 the compact scheme's
modified wavenumber of the y profile; the shear case follows the
rapid-distortion solution like the explicit branch; crosst's branch adds the
scalar (semi-implicit diffusion, explicit buoyancy)."""
import numpy as np
import pytest

import oracle
from conftest import box_params
from test_oracle import _single_wave_state

ALPHA = (29 / 96, -3 / 40, 1 / 6)
BETA = (37 / 160, 5 / 24, 1 / 6)


def _gain(lam, dt):
    g = 1.0
    for a, b in zip(ALPHA, BETA):
        g *= (1 + a * dt * lam) / (1 - b * dt * lam)
    return g


def test_coefficients_split_the_rk3_weights():
    """alpha_k + beta_k = gama_k + zeta_{k-1} (the viscous term carries the
    substep's full weight) and the three substeps are second-order accurate."""
    gama, zeta = (8 / 15, 5 / 12, 3 / 4), (0.0, -17 / 60, -5 / 12)
    for k in range(3):
        assert abs(ALPHA[k] + BETA[k] - (gama[k] + zeta[k])) < 1e-15
    # local error O(dt^3): second order
    e1 = abs(_gain(-1.0, 1e-2) - np.exp(-1e-2))
    e2 = abs(_gain(-1.0, 5e-3) - np.exp(-5e-3))
    assert e1 < 0.1 * 1e-6 and 7.0 < e1 / e2 < 9.0


@pytest.mark.parametrize("dt", [0.01, 0.2])
def test_plane_wave_decay(dt):
    """s = 0, a single wave in phi (ky = 0): |phi| follows the implicit gain
    exactly, also at a step far beyond the explicit viscous limit."""
    pp = box_params(64, 32, 32, rez=100.0, fixed_dt=dt, s=0.0, keep_laminar=1)
    o = oracle.Oracle(**pp, implicit_visc=1)
    st, kx, kz = _single_wave_state(o, 2, 1, 1e-3)
    n = 40
    o.cross(st, n)
    k2 = kx * kx + kz * kz
    ratio = np.abs(st["phi"][1, 2, 0]) / (k2 * 1e-3)
    lam = -k2 / pp["Re"]
    assert abs(ratio / _gain(lam, dt) ** n - 1) < 1e-12
    assert np.all(np.isfinite(st["phi"]))


def test_vorticity_line_with_y_profile():
    """s = 0, u = (0, 0, w(x, y)): no nonlinear term; omega_y on the line
    (kx, kz = 0) with a cos(ky y) profile decays with the modified
    wavenumber of the compact d2/dy2."""
    pp = box_params(64, 32, 32, rez=50.0, fixed_dt=0.05, s=0.0, keep_laminar=1)
    o = oracle.Oracle(**pp, implicit_visc=1)
    my = pp["my"]
    y = np.arange(my) * pp["Ly"] / my
    ky = 3 * 2 * np.pi / pp["Ly"]
    prof = np.cos(ky * y) * 1e-3
    kappa2 = -(o.derivyc(prof.astype(complex), iord=2).real / prof)[0]
    assert abs(kappa2 / ky ** 2 - 1) < 0.05  # a modified wavenumber near ky^2
    st = {"vor": np.zeros((o.mz, o.nkx, my), complex), "phi": np.zeros((o.mz, o.nkx, my), complex),
          "u00": np.zeros(my), "w00": np.zeros(my), "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    i0 = 3
    st["vor"][0, i0, :] = prof
    n = 30
    o.cross(st, n)
    kx = 0.5 * i0
    lam = -(kx * kx + kappa2) / pp["Re"]
    np.testing.assert_allclose(st["vor"][0, i0, :].real, prof * _gain(lam, 0.05) ** n,
                               rtol=0, atol=1e-12 * 1e-3)
    assert np.abs(st["vor"][0, i0, :].imag).max() < 1e-17


def test_mean_profile_decay():
    """A unidirectional mean flow u00 = A cos(ky y) (s = 0) decays through the
    real Helmholtz solve of the mean line (lapcdy(u00wk, dtr1), cross.f90:965)."""
    pp = box_params(64, 32, 32, rez=50.0, fixed_dt=0.05, s=0.0, keep_laminar=1)
    o = oracle.Oracle(**pp, implicit_visc=1)
    my = pp["my"]
    y = np.arange(my) * pp["Ly"] / my
    ky = 2 * 2 * np.pi / pp["Ly"]
    u0 = 1e-3 * np.cos(ky * y)
    kappa2 = -(o.derivyc(u0, iord=2) / u0)[0]
    st = {"vor": np.zeros((o.mz, o.nkx, my), complex), "phi": np.zeros((o.mz, o.nkx, my), complex),
          "u00": u0.copy(), "w00": -0.5 * u0, "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    n = 25
    o.cross(st, n)
    g = _gain(-kappa2 / pp["Re"], 0.05) ** n
    np.testing.assert_allclose(st["u00"], u0 * g, rtol=0, atol=1e-12 * 1e-3)
    np.testing.assert_allclose(st["w00"], -0.5 * u0 * g, rtol=0, atol=1e-12 * 1e-3)


def test_rdt_single_wave_implicit():
    """The rapid-distortion known answer of the explicit branch
    (rdtfunc, operators.f90:1516-1562) holds for the semi-implicit branch."""
    pp = box_params(64, 64, 32, rez=1000.0, fixed_dt=0.004)
    o = oracle.Oracle(**pp, implicit_visc=1)
    v0 = 1e-3
    st, kx, kz = _single_wave_state(o, 1, 1, v0)
    o.cross(st, 1000)
    t = st["time"]
    nu = 1.0 / pp["Re"]
    ky = -1.0 * kx * t
    k02 = kx * kx + kz * kz
    du = np.exp(-nu * t * (k02 + (1.0 * t * kx) ** 2 / 3.0))
    shp = np.exp(-1j * kx * st["xofft"])
    v = o.lapcdy(st["phi"][1, 1, :].copy(), k02, shp=shp)
    expected = v0 * k02 / (k02 + ky * ky) * du
    assert np.abs(np.abs(v) / expected - 1).max() < 2e-5


def test_implicit_refused_with_les_or_zero_diffusivity():
    pp = box_params(64, 32, 32, rez=1000.0)
    for kw in ({"les": 1}, {"temperature": 1, "fkappa": 0.0}):
        with pytest.raises(ValueError):
            oracle.Oracle(**pp, **kw, implicit_visc=1)


def test_seeded_turbulence_close_to_explicit():
    """On a seeded turbulent state at a small step the two branches differ by
    the time-discretisation error of the viscous term only."""
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.002)
    st0 = sb.seed_state(sb.make_params(**pp), 3)
    out = []
    for imp in (0, 1):
        o = oracle.Oracle(**pp, implicit_visc=imp)
        st = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in st0.items()}
        o.cross(st, 10)
        out.append(st)
    for k in ("vor", "phi"):
        d = np.linalg.norm(out[0][k] - out[1][k]) / np.linalg.norm(out[0][k])
        assert 1e-12 < d < 1e-4, (k, d)


# ---- crosst's semi-implicit branch (crosst.f90:916-1195)

def _rest_scalar_recurrence(T, P, n, dt, kap, nu, k2, gb):
    """Fluid at rest, one y-constant line (kx, 0): the scalar diffuses
    semi-implicitly (fkappa), the buoyancy -gbeta k^2 T of the substep's start
    drives phi as a nonlinear term (gama/zeta), phi's viscous term is
    semi-implicit."""
    gama, zeta = (8 / 15, 5 / 12, 3 / 4), (-17 / 60, -5 / 12, 0.0)
    lt, lp = -kap * k2, -nu * k2
    for _ in range(n):
        hold = 0.0
        for k in range(3):
            h = -gb * k2 * T
            extra = dt * (gama[k] * h + (zeta[k - 1] * hold if k else 0.0))
            T, P = (T * (1 + ALPHA[k] * dt * lt) / (1 - BETA[k] * dt * lt),
                    (P * (1 + ALPHA[k] * dt * lp) + extra) / (1 - BETA[k] * dt * lp))
            hold = h
    return T, P


def test_rest_scalar_and_buoyancy_implicit():
    """crosst at rest with implicit_visc: the line (kx=1, kz=0) follows the
    semi-implicit recurrence of diffusion and buoyancy, at a step 10 times the
    explicit thermal limit."""
    from test_temperature_oracle import REST, BASE, _rest_state
    kappa, gbeta, dt, n = 0.05, 0.7, 0.2, 6
    o = oracle.Oracle(**dict(REST, fixed_dt=dt, fkappa=kappa, gbeta=gbeta), implicit_visc=1)
    amp = 1e-7
    st = _rest_state(o, amp, 0.0)
    o.cross(st, n)
    k2 = (BASE["alp"] * 1) ** 2
    T_n, phi_n = _rest_scalar_recurrence(amp, 0.0, n, dt, kappa, 1.0 / BASE["Re"], k2, gbeta)
    np.testing.assert_allclose(st["tb"][0, 1, :], T_n, rtol=1e-11, atol=0)
    np.testing.assert_allclose(st["phi"][0, 1, :], phi_n, rtol=1e-9, atol=0)


def test_rest_mean_scalar_implicit():
    """tb00 = A cos(ky y) at rest decays with the implicit gain of fkappa and
    the compact scheme's modified wavenumber (lapcdy(tb00wk, dtr1k),
    crosst.f90:1158-1161)."""
    from test_temperature_oracle import REST, _rest_state
    kappa, dt, n = 0.05, 0.2, 6
    o = oracle.Oracle(**dict(REST, fixed_dt=dt, fkappa=kappa, gbeta=0.7), implicit_visc=1)
    st = _rest_state(o, 0.0, 0.3)
    tb00_0 = st["tb00"].copy()
    o.cross(st, n)
    lam = kappa * o.derivyc(tb00_0, iord=2)[0] / tb00_0[0]
    np.testing.assert_allclose(st["tb00"], _gain(lam, dt) ** n * tb00_0, rtol=1e-10, atol=1e-14)
    assert np.all(st["tb"] == 0.0) and np.all(st["phi"] == 0.0)


def test_crosst_implicit_close_to_explicit():
    """Seeded turbulence with the scalar at a small step: the semi-implicit
    crosst differs from the explicit one by the time-discretisation error of
    the viscous and diffusive terms, except on the (0,0) line of tb, which the
    explicit branch advances with ht(0,0) (crosst.f90:813-826) and the
    semi-implicit one leaves alone (its solves skip (0,0),
    crosst.f90:1094-1104)."""
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.002, temperature=1, fkappa=0.02,
                    bym=1.0, gbeta=0.5)
    st0 = sb.seed_state(sb.make_params(**pp), 3)
    out = []
    for imp in (0, 1):
        o = oracle.Oracle(**pp, implicit_visc=imp)
        st = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in st0.items()}
        o.cross(st, 10)
        out.append(st)
    for st in out:
        assert np.all(np.isfinite(st["tb"]))
    assert np.all(out[1]["tb"][0, 0] == 0.0) and np.abs(out[0]["tb"][0, 0]).max() > 0
    for st in out:
        st["tb"][0, 0] = 0.0
    for k in ("vor", "phi", "tb", "tb00"):
        d = np.linalg.norm(out[0][k] - out[1][k]) / np.linalg.norm(out[0][k])
        assert 1e-12 < d < 1e-5, (k, d)
