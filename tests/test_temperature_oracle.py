"""Temperature variant crosst (crosst.f90:3-1310) in the oracle.

Known answers: with the fluid at rest the scalar diffuses and drives phi
through the buoyancy term, a linear system per Fourier mode whose RK3 solution
is the cubic Taylor polynomial of the step matrix; histt's tbmax and tner of a
single mode; conservation of the mean-profile integral without diffusion; and
crosst with gbeta = 0 leaves the flow exactly as cross does."""
import numpy as np
import pytest

import oracle
import shear_nnf_gb300 as sb

BASE = dict(mgalx=32, my=32, mgalz=32, Re=400.0, alp=0.5, Ly=2.0, gam=1.0, s=1.0, nhist=1)


def _copy(st):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}


def _rest_state(o, amp, mean):
    """Fluid at rest; tb = amp on line (kx=1, kz=0), constant in y; tb00 =
    mean * cos(4 pi y / Ly)."""
    z = np.zeros((o.mz, o.nkx, o.my), np.complex128)
    tb = z.copy()
    tb[0, 1, :] = amp
    y = np.arange(o.my) * (BASE["Ly"] / o.my) - 0.5 * BASE["Ly"]
    tb00 = mean * np.cos(2 * np.pi * 2 * y / BASE["Ly"])
    return {"vor": z.copy(), "phi": z.copy(), "u00": np.zeros(o.my), "w00": np.zeros(o.my),
            "tb": tb, "tb00": tb00, "time": 0.0, "xoffb": 0.0, "xofft": 0.0}


def _rk3(Z, n):
    """Amplification of n explicit RK3 steps of the linear system x' = A x with
    Z = dt A (any three-stage third-order scheme)."""
    I = np.eye(Z.shape[0])
    G = I + Z + Z @ Z / 2 + Z @ Z @ Z / 6
    return np.linalg.matrix_power(G, n)


REST = dict(BASE, s=0.0, keep_laminar=1, temperature=1, bym=0.0)


def test_rest_diffusion_and_buoyancy_known_answer():
    kappa, gbeta, dt, n = 0.01, 0.7, 0.05, 6
    o = oracle.Oracle(**dict(REST, fixed_dt=dt, fkappa=kappa, gbeta=gbeta))
    amp = 1e-7
    st = _rest_state(o, amp, 0.0)
    tr, _ = o.cross(st, n)
    assert len(tr) == n
    nu = 1.0 / BASE["Re"]
    k2 = (BASE["alp"] * 1) ** 2
    # line (kx=1, kz=0): T' = -kappa k2 T, phi' = -gbeta k2 T - nu k2 phi
    # (y-constant lines: d2/dy2 vanishes); the products are O(amp^2)
    A = np.array([[-kappa * k2, 0.0], [-gbeta * k2, -nu * k2]])
    T_n, phi_n = _rk3(dt * A, n) @ np.array([amp, 0.0])
    np.testing.assert_allclose(st["tb"][0, 1, :], T_n, rtol=1e-9, atol=0)
    np.testing.assert_allclose(st["phi"][0, 1, :], phi_n, rtol=1e-7, atol=0)
    # histt of the first record: tbmax = 2 amp, tner(1) = sqrt(2) amp, no fluxes
    assert tr[0, 24] == pytest.approx(2 * amp, rel=1e-12)
    assert tr[0, 25] == pytest.approx(np.sqrt(2) * amp, rel=1e-12)
    assert np.all(tr[0, 26:29] == 0.0)


def test_rest_mean_profile_diffusion_known_answer():
    kappa, dt, n = 0.01, 0.05, 6
    o = oracle.Oracle(**dict(REST, fixed_dt=dt, fkappa=kappa, gbeta=0.7))
    st = _rest_state(o, 0.0, 0.3)
    tb00_0 = st["tb00"].copy()
    tr, _ = o.cross(st, n)
    # tb00' = kappa d2/dy2 tb00: the compact scheme's eigenvalue of the cosine
    lam = o.derivyc(tb00_0, iord=2)[0] / tb00_0[0]
    g = _rk3(np.array([[dt * kappa * lam]]), n)[0, 0]
    np.testing.assert_allclose(st["tb00"], g * tb00_0, rtol=1e-10, atol=1e-13)
    assert np.all(st["tb"] == 0.0) and np.all(st["phi"] == 0.0)
    assert tr[0, 24] == pytest.approx(0.3, rel=1e-12)
    assert tr[0, 25] == pytest.approx(np.sqrt(np.mean(tb00_0**2)), rel=1e-12)


def test_gbeta_zero_leaves_flow_as_cross():
    pt = dict(BASE, temperature=1, fkappa=1 / 400 / 0.7, bym=0.3, gbeta=0.0)
    st = sb.seed_state(sb.make_params(**pt), 3)
    st2 = _copy(st)
    tr1, _ = oracle.Oracle(**pt).cross(st, 4)
    tr0, _ = oracle.Oracle(**BASE).cross(st2, 4)
    for k in ("vor", "phi", "u00", "w00"):
        assert np.array_equal(st[k], st2[k]), k
    assert tr1.shape == (4, oracle.TRACE_LEN_T)
    assert np.array_equal(tr1[:, :24], tr0)
    assert np.all(np.isfinite(tr1[:, 24:])) and np.all(tr1[:, 24] > 0)


def test_mean_integral_conserved_without_diffusion():
    pc = dict(BASE, temperature=1, fkappa=0.0, bym=0.4, gbeta=0.5)
    st = sb.seed_state(sb.make_params(**pc), 4)
    st["tb00"] = st["tb00"] + 1.0
    s0 = st["tb00"].sum()
    oracle.Oracle(**pc).cross(st, 5)
    assert abs(st["tb00"].sum() - s0) < 1e-12 * abs(s0) * 32


def test_bym_drives_scalar_from_v():
    """bym alone (no initial scalar): after the first substep tb = -bym dt
    gamma_1 v on every line but (0,0) -- to first order in the amplitude."""
    prm = dict(BASE, s=0.0, fixed_dt=0.02, keep_laminar=1, temperature=1, fkappa=0.0,
               gbeta=0.0, bym=0.8)
    o = oracle.Oracle(**prm)
    st = sb.seed_state(sb.make_params(**prm), 9, urms=1e-8)
    st["tb"][:] = 0.0
    st["tb00"][:] = 0.0
    phi0 = st["phi"].copy()
    o.cross(st, 1)
    # v of the initial state from phi (lapcdy) on one line, compared with the
    # RK3 integral of -bym v over one step to leading order: -bym dt v
    k, i = 1, 2
    kz = k if k <= o.nz else k - o.mz
    k2 = (BASE["alp"] * i) ** 2 + (BASE["gam"] * kz) ** 2
    v0 = o.lapcdy(phi0[k, i, :], k2)
    np.testing.assert_allclose(st["tb"][k, i, :], -0.8 * 0.02 * v0, rtol=2e-3,
                               atol=1e-3 * np.abs(0.8 * 0.02 * v0).max())


def test_stop_check_from_second_step():
    """crosst tests the stop flag at the start of its second step
    (crosst.f90:259); cross only from its third (cross.f90:221)."""
    pt = dict(BASE, temperature=1, fkappa=1e-3, etime=1e-3)
    st = sb.seed_state(sb.make_params(**pt), 5)
    trt, stop = oracle.Oracle(**pt).cross(st, 4)
    assert st["time"] == pytest.approx(1e-3, abs=1e-15) and stop == 1
    assert len(trt) == 1
    st2 = sb.seed_state(sb.make_params(**BASE), 5)
    tr, _ = oracle.Oracle(**dict(BASE, etime=1e-3)).cross(st2, 4)
    assert len(tr) == 2  # cross runs one more (zero-length) step
