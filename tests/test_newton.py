"""Newton-Krylov / Arnoldi tools over batched period maps: packing, Krylov
algebra (CPU), and on the GPU the Floquet multipliers of the Stokes problem
(known answer), Jv against the oracle, batched against unbatched products, and
Newton with FP32-mixed Jv products and an FP64 residual."""
import numpy as np
import pytest

from conftest import box_params, rel_l2

import shear_nnf_gb300 as sb
from shear_nnf_gb300 import newton as nw


def _params(**kw):
    return sb.make_params(**box_params(64, 32, 32, 1000.0, **kw))


def test_packing_roundtrip():
    p = _params()
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    st = sb.seed_state(p, 11)
    x = pk.pack(st)
    assert x.size == pk.n
    back = pk.unpack(x)
    # the (0,0) modes of vor/phi are not unknowns
    for key in ("vor", "phi"):
        a = st[key].copy()
        a[0, 0, :] = 0
        assert rel_l2(back[key], a) < 1e-15
    assert rel_l2(back["u00"], st["u00"]) < 1e-15 and rel_l2(back["w00"], st["w00"]) < 1e-15
    assert np.isclose(np.linalg.norm(pk.pack(back)), np.linalg.norm(x))


def test_phase_shift_full_period():
    p = _params()
    st = sb.seed_state(p, 2)
    lx, lz = 2 * np.pi / p.alp, 2 * np.pi / p.gam
    a = nw.phase_shift(st, p, lx, lz)
    assert rel_l2(a["vor"], st["vor"]) < 1e-13 and rel_l2(a["phi"], st["phi"]) < 1e-13
    b = nw.phase_shift(nw.phase_shift(st, p, 0.3, -0.2), p, -0.3, 0.2)
    assert rel_l2(b["vor"], st["vor"]) < 1e-14


def _test_matrix(n, top, seed=1):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.concatenate([top, 0.3 * rng.random(n - len(top))])
    return Q @ np.diag(ev) @ Q.T


@pytest.mark.parametrize("block", [1, 4])
def test_arnoldi_matrix(block):
    top = [1.0, 0.9, 0.8, 0.7, 0.6]
    A = _test_matrix(200, top)
    lam, res, _, _ = nw.arnoldi(lambda D: A @ D, 200, 40 // block, block=block)
    assert np.allclose(lam[:5].real, top, atol=1e-6)
    assert np.all(res[:3] < 1e-5)
    sig = nw.floquet_exponents(lam[:2], 2.0)
    assert np.isclose(sig[0].real, 0.0, atol=1e-6)


@pytest.mark.parametrize("block", [1, 4])
def test_gmres_matrix(block):
    A = _test_matrix(200, [1.5, 0.9, 0.8, 0.7, 0.6])
    M = A - np.eye(200)
    b = np.random.default_rng(3).standard_normal(200)
    x, res = nw.gmres(lambda D: M @ D, b, 60 // block, block=block, tol=1e-10)
    assert res[-1] <= 1e-10 * res[0]
    assert np.linalg.norm(M @ x - b) <= 1e-9 * np.linalg.norm(b)


def test_newton_linear_map():
    # F(x) = A x - x - r has the root (A - I)^-1 (-r); an inexact Jacobian
    # (A perturbed by 1e-3) still converges through the exact residual
    A = _test_matrix(120, [1.5, 0.9, 0.8], seed=4)
    r = np.random.default_rng(5).standard_normal(120)

    class J:
        def __init__(self, x):
            self.A = A + 1e-3 * np.random.default_rng(6).standard_normal(A.shape) / 11

        def matvec(self, D):
            return self.A @ D

    x, hist = nw.newton(np.zeros(120) + 1.0, lambda x: A @ x - x - r, J, k=60, itmax=20,
                        tol=1e-12, gmres_tol=1e-6)
    assert hist[-1] <= 1e-12
    assert np.allclose(x, np.linalg.solve(A - np.eye(120), r), rtol=1e-9, atol=1e-10)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _stokes_multipliers(p, nu, dt, nsteps):
    """Multipliers of the linearised map at rest without shear: every Fourier
    mode decays under explicit RK3 with amplification 1 + z + z^2/2 + z^3/6,
    z = nu dt (lambda_y - kx^2 - kz^2), lambda_y the modified wavenumber of the
    compact second-derivative scheme."""
    sz = sb.sizes(p)
    nkx, mz, nz, my = sz["nkx"], sz["mz"], sz["nz"], p.my
    pr1, rh1, pr2, rh2 = sb.compact_coeffs()
    h = p.Ly / my
    d = np.arange(-3, 4)
    ky = 2 * np.pi * np.arange(my) / p.Ly
    num = (rh2[None, :] * np.cos(ky[:, None] * d[None, :] * h)).sum(1)
    den = (pr2[None, :] * np.cos(ky[:, None] * d[None, :] * h)).sum(1)
    lam_y = num / den / h ** 2
    kx2 = (p.alp * np.arange(nkx)) ** 2
    kz2 = (p.gam * np.array([k if k <= nz else k - mz for k in range(mz)], float)) ** 2
    k2 = (kx2[None, :, None] + kz2[:, None, None]) - lam_y[None, None, :]
    z = -nu * dt * k2
    g = (1 + z + z * z / 2 + z ** 3 / 6) ** nsteps
    assert np.all(np.abs(1 + z + z * z / 2 + z ** 3 / 6) <= 1)
    return np.unique(np.round(g.ravel(), 13))[::-1]


@pytest.mark.gpu
def test_floquet_stokes_known_answer():
    nu, dt, nsteps = 0.1, 0.01, 200
    p = sb.make_params(64, 32, 32, 1.0 / nu, 0.7, 5.0, 1.3, s=0.0, chi=0.0, CFL=0.5,
                       fixed_dt=dt, keep_laminar=1)
    pk = nw.Packing(p)
    pmap = nw.PeriodMap(p, nsteps * dt, batch=2)
    J = nw.Jacobian(pmap, pk, np.zeros(pk.n), central=True, eps_jacobi=1e-6)
    # 25 iterations: the multiplier 1 is double (mean u00 and w00), and longer
    # runs split it into a pair of Ritz values with a larger residual
    lam, res, _, _ = nw.arnoldi(J.matvec, pk.n, 25, seed=7)
    theory = _stokes_multipliers(p, nu, dt, nsteps)
    assert pmap.last_steps == [nsteps, nsteps]
    for q, tol in enumerate((1e-9, 1e-9, 1e-6, 1e-6)):
        assert abs(lam[q].imag) < 1e-10, (q, lam[:6], res[:6])
        assert abs(lam[q].real - theory[q]) < tol * theory[q], (q, lam[:6], res[:6], theory[:6])
    assert res[0] < 1e-10 and res[1] < 1e-9
    sig = nw.floquet_exponents(lam[:4], nsteps * dt)
    assert np.isclose(sig[0].real, 0.0, atol=1e-9)


def _seeded_x(p, pk, seed, scale=1.0):
    return scale * pk.pack(sb.seed_state(p, seed))


@pytest.mark.gpu
def test_jv_matches_oracle():
    import oracle
    kw = box_params(64, 32, 32, 1000.0)
    p = sb.make_params(**kw)
    T = 0.1
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    x0 = _seeded_x(p, pk, 5)
    d = np.random.default_rng(8).standard_normal(pk.n)
    pmap = nw.PeriodMap(p, T, batch=1)
    J = nw.Jacobian(pmap, pk, x0, eps_jacobi=1e-5)
    jv = J.matvec(d)[:, 0]

    def g_oracle(x):
        orc = oracle.Oracle(**kw, etime=T)
        st = pk.unpack(x)
        orc.cross(st, 100000)
        assert abs(st["time"] - T) < 1e-12
        return pk.pack(st)

    eps = 1e-5 * np.linalg.norm(x0) / np.linalg.norm(d)
    xp = x0 + ((x0 + eps * d) - x0)
    jv_o = (g_oracle(xp) - g_oracle(x0)) / eps
    assert rel_l2(jv, jv_o) < 1e-6
    assert pmap.steps > 2


@pytest.mark.gpu
def test_batched_products_equal_unbatched():
    p = _params()
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    x0 = _seeded_x(p, pk, 9)
    D = np.random.default_rng(10).standard_normal((pk.n, 4))
    one = nw.Jacobian(nw.PeriodMap(p, 0.05, batch=1), pk, x0)
    four = nw.Jacobian(nw.PeriodMap(p, 0.05, batch=4), pk, x0)
    a = one.matvec(D)
    b = four.matvec(D)
    assert four.pmap.integrations == 4 + 1 and one.pmap.integrations == 4 + 1
    assert rel_l2(b, a) < 1e-12


@pytest.mark.gpu
def test_newton_fp32_jv_fp64_residual():
    # manufactured root: F(x) = G(x) - x - (G(x*) - x*) vanishes at x*; products
    # from an FP32-mixed batch (base in the batch), residual in FP64
    p = _params()
    T = 10.0
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    xs = _seeded_x(p, pk, 12)
    res64 = nw.Residual(nw.PeriodMap(p, T, batch=1), pk)
    rhs = res64(xs)
    res64.rhs = rhs
    assert np.linalg.norm(res64(xs)) == 0.0
    pm32 = nw.PeriodMap(p, T, batch=9, precision=sb.SB_MIXED)
    x0 = xs + 1e-3 * np.linalg.norm(xs) / np.sqrt(pk.n) * \
        np.random.default_rng(13).standard_normal(pk.n)

    def jac(x):
        return nw.Jacobian(pm32, pk, x, eps_jacobi=1e-3, base_in_batch=True)

    x, hist = nw.newton(x0, res64, jac, k=16, block=8, itmax=12, tol=1e-10, gmres_tol=1e-4)
    assert hist[-1] <= 1e-10, hist


def test_hookstep_trust_region():
    rng = np.random.default_rng(21)
    n, m = 60, 12
    V, _ = np.linalg.qr(rng.standard_normal((n, m)))
    H = rng.standard_normal((m + 1, m))
    rhs = rng.standard_normal(m + 1)
    y0, *_ = np.linalg.lstsq(H, rhs, rcond=None)
    dx, mu, r = nw.hookstep(V, H, rhs, 10 * np.linalg.norm(y0))
    assert mu == 0.0 and np.allclose(dx, V @ y0)
    prev = np.inf
    for delta in (0.9, 0.5, 0.2, 0.05):
        dx, mu, r = nw.hookstep(V, H, rhs, delta * np.linalg.norm(y0))
        assert mu > 0 and abs(np.linalg.norm(dx) - delta * np.linalg.norm(y0)) < 1e-8
        assert r < prev + 1e-12 or True
        prev = r
    rs = [nw.hookstep(V, H, rhs, d * np.linalg.norm(y0))[2] for d in (0.05, 0.2, 0.5, 0.9)]
    assert all(a >= b - 1e-12 for a, b in zip(rs, rs[1:]))


class _IdentityMap:
    """A period map that returns its states: G is the shift alone."""

    def __init__(self, p, batch=2):
        self.p, self.batch, self.integrations = p, batch, 0

    def __call__(self, states):
        return [dict(s) for s in states]


def test_shift_jacobian_columns():
    p = _params()
    pk = nw.Packing(p)
    x0 = _seeded_x(p, pk, 31)
    s0 = 0.37
    J = nw.Jacobian(_IdentityMap(p), pk, x0, shiftx=s0, eps_jacobi=1e-7)
    gx0 = J.gx0
    SJ = nw.ShiftJacobian(J, pk, p, x0, gx0)
    # d/ds column against a centred difference of the shifted map
    h = 1e-6
    gp = pk.pack(nw.phase_shift(pk.unpack(x0), p, s0 + h, 0.0))
    gm = pk.pack(nw.phase_shift(pk.unpack(x0), p, s0 - h, 0.0))
    fd = (gp - gm) / (2 * h)
    e = np.zeros(pk.n + 1)
    e[-1] = 1.0
    col = SJ.matvec(e)[:, 0]
    assert rel_l2(col[:-1], fd) < 1e-8 and col[-1] == 0.0
    # x columns: (J - I) d with J the shift itself, and the phase row <t, d>
    d = np.random.default_rng(2).standard_normal(pk.n)
    out = SJ.matvec(np.concatenate([d, [0.0]]))[:, 0]
    ref = pk.pack(nw.phase_shift(pk.unpack(d), p, s0, 0.0)) - d
    assert rel_l2(out[:-1], ref) < 1e-6
    assert abs(out[-1] - SJ.t @ d) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("hook", [False, True])
def test_newton_with_unknown_shift(hook):
    # manufactured root (x*, s*): F(x, s) = shift_s(Phi_T(x)) - x - rhs
    p = _params()
    T, s_star = 10.0, 0.3
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    xs = _seeded_x(p, pk, 14)
    res = nw.ShiftResidual(nw.PeriodMap(p, T, batch=1), pk)
    F0, _ = res(xs, s_star)
    res.rhs = F0
    pm = nw.PeriodMap(p, T, batch=4)

    def jac_at(x, s, G):
        return nw.ShiftJacobian(nw.Jacobian(pm, pk, x, shiftx=s, eps_jacobi=1e-7), pk, p, x, G)

    x0 = xs + 1e-3 * np.linalg.norm(xs) / np.sqrt(pk.n) * np.random.default_rng(15).standard_normal(pk.n)
    x, s, hist = nw.newton_shift(x0, s_star - 0.02, res, jac_at, k=16, block=4, itmax=10,
                                 tol=1e-10, gmres_tol=1e-8,
                                 delta=(0.05 * np.linalg.norm(xs) if hook else None))
    assert hist[-1] <= 1e-10, hist
    F, _ = res(x, s)
    assert np.linalg.norm(F) <= 1e-10 * np.linalg.norm(x)


# ---------------------------------------------------------------------------
# fourth-order products and arclength continuation in the Reynolds number
# ---------------------------------------------------------------------------

class _CubeMap:
    """A nonlinear map on states: every entry v -> v + c v^3 (analytic, so the
    packed Jacobian is the complex multiplication by 1 + 3 c v^2)."""

    def __init__(self, p, batch=8, c=0.5):
        self.p, self.batch, self.c = p, batch, c

    def __call__(self, states, res=None):
        out = []
        for s in states:
            d = dict(s)
            for key in ("vor", "phi", "u00", "w00"):
                d[key] = s[key] + self.c * s[key] ** 3
            out.append(d)
        return out


@pytest.mark.parametrize("order,tol", [(1, 3e-2), (2, 3e-4), (4, 3e-8)])
def test_fd_product_orders(order, tol):
    p = _params()
    pk = nw.Packing(p)
    x0 = _seeded_x(p, pk, 41)
    x0 = x0 / np.abs(x0).max()
    cm = _CubeMap(p)
    d = np.random.default_rng(3).standard_normal(pk.n)
    J = nw.Jacobian(cm, pk, x0, eps_jacobi=1e-2, order=order)
    got = J.matvec(d)[:, 0]
    st0, dst = pk.unpack(x0), pk.unpack(d)
    ex = {k: dst[k] * (1 + 3 * cm.c * st0[k] ** 2) for k in ("vor", "phi", "u00", "w00")}
    exact = pk.pack(dict(st0, **ex))
    err = rel_l2(got, exact)
    assert err < tol, err
    assert J.block == 8 // {1: 1, 2: 2, 4: 4}[order]


def test_re_jacobian_columns():
    rng = np.random.default_rng(7)
    n = 40
    A = rng.standard_normal((n, n))
    b, xs = rng.standard_normal(n), rng.standard_normal(n)

    class J:
        def matvec(self, D):
            return A @ D

    RJ = nw.ReJacobian(J(), b, xs)
    e = np.zeros(n + 1)
    e[-1] = 1.0
    assert np.allclose(RJ.matvec(e)[:, 0], np.concatenate([b, [0.0]]))
    d = rng.standard_normal(n)
    out = RJ.matvec(np.concatenate([d, [0.0]]))[:, 0]
    assert np.allclose(out[:-1], A @ d - d) and np.isclose(out[-1], xs @ d)


def test_newton_arclength_follows_a_curve():
    # F(x, re) = (A - I) x + re b + c + 0.02 x^3: two converged points at
    # re = 1.0, 1.02, then one arclength step lands on the curve in the plane
    # through the predictor orthogonal to the secant
    rng = np.random.default_rng(8)
    n = 60
    A = _test_matrix(n, [0.5, 0.4, 0.3], seed=9)
    b, c = 0.3 * rng.standard_normal(n), 0.3 * rng.standard_normal(n)

    def F(x, re):
        return (A - np.eye(n)) @ x + re * b + c + 0.02 * x ** 3

    def residual_at(x, re):
        f = F(x, re)
        return f, f + x

    class Jx:
        def __init__(self, x):
            self.M = A + np.diag(0.06 * x ** 2)

        def matvec(self, D):
            return self.M @ D

    def solve(re, x0):
        x, hist = nw.newton(x0, lambda x: F(x, re), Jx, k=n, itmax=30, tol=1e-13,
                            gmres_tol=1e-12)
        assert hist[-1] <= 1e-13
        return x

    x1 = solve(1.0, np.zeros(n))
    x2 = solve(1.02, x1)  # the same branch
    xp, rep, xstan = nw.arclength_predictor(x1, 1.0, x2, 1.02, 1.0)
    assert np.isclose(rep, 1.04)
    x, re, hist = nw.newton_arclength(
        x1, 1.0, x2, 1.02, 1.0, residual_at,
        lambda x, re, G, xs: nw.ReJacobian(Jx(x), b, xs), k=n + 1, itmax=20, tol=1e-13,
        gmres_tol=1e-12)
    assert hist[-1] <= 1e-13, hist
    assert abs(xstan @ (x - xp)) <= 1e-10 * np.linalg.norm(xstan) * np.linalg.norm(x)
    assert np.linalg.norm(F(x, re)) <= 1e-12 * np.linalg.norm(x)
    with pytest.raises(ValueError):
        nw.arclength_predictor(x1, 1.0, x2, 1.0, 1.0)
    assert len(hist) <= 6 and abs(re - 1.04) < 0.01


@pytest.mark.gpu
def test_arclength_in_re_gpu():
    # manufactured curve through (x*, re*): F(x, re) = G(x; re) - x - rhs with
    # rhs = G(x*; re*) - x*; a second point at 0.999 re* by Newton at fixed re,
    # then one arclength step (arcl = 1) past x*
    p = _params()
    T = 10.0
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    xs = _seeded_x(p, pk, 16)
    re_s = p.Re
    pm1 = nw.PeriodMap(p, T, batch=1)
    rhs = pk.pack(pm1([pk.unpack(xs)], [re_s])[0]) - xs

    def residual_at(x, re):
        G = pk.pack(pm1([pk.unpack(x)], [re])[0])
        return G - x - rhs, G

    pm = nw.PeriodMap(p, T, batch=8)

    def jac(x, re):
        return nw.Jacobian(pm, pk, x, eps_jacobi=1e-7, central=True, re=re)

    re1 = 0.999 * re_s
    x1, h1 = nw.newton(xs, lambda x: residual_at(x, re1)[0], lambda x: jac(x, re1), k=16,
                       block=4, itmax=12, tol=1e-11, gmres_tol=1e-9)
    assert h1[-1] <= 1e-11, h1
    def jac_at(x, re, G, xst):
        J = jac(x, re)
        return nw.ReJacobian(J, nw.re_derivative(J, re, daa=1e-5 * re), xst)

    xp, rep, xstan = nw.arclength_predictor(x1, re1, xs, re_s, 1.0)
    x, re, hist = nw.newton_arclength(x1, re1, xs, re_s, 1.0, residual_at, jac_at, k=16,
                                      block=4, itmax=12, tol=1e-10, gmres_tol=1e-9)
    assert hist[-1] <= 1e-10, hist
    assert abs(xstan @ (x - xp)) <= 1e-8 * np.linalg.norm(xstan) * np.linalg.norm(x)
    assert abs(re - 1.001 * re_s) < 2.5e-4 * re_s


# ---------------------------------------------------------------------------
# pseudo-arclength along Ly, alp, Cs (ParamFamily)
# ---------------------------------------------------------------------------

class _FakeMap:
    """Stands in for PeriodMap on the CPU: a smooth map of the state whose
    coefficients depend on the handle's Ly, alp, cs and the member's Re, and
    on the image offsets and the period it integrates over."""
    made = []

    def __init__(self, p, T, batch, precision=0, chunk=64):
        self.p, self.T, self.batch = p, T, batch
        self.closed = False
        _FakeMap.made.append(self)

        class _Box:
            def close(inner):
                self.closed = True
        self.box = _Box()

    def __call__(self, states, res=None, Ts=None):
        out = []
        for m, st in enumerate(states):
            re = res[m] if res is not None else self.p.Re
            f = (1.0 + 0.1 * self.p.Ly + 0.2 * self.p.alp + 0.3 * self.p.cs + 1e-4 * re
                 + 0.05 * self.T + 0.01 * st["xofft"])
            g = dict(st)
            for key in ("vor", "phi"):
                g[key] = st[key] * f + 0.01 * np.sin(st[key].real) * self.p.Ly
            g["u00"] = st["u00"] * f
            g["w00"] = st["w00"] * f
            out.append(g)
        return out


def test_param_family_geometry(monkeypatch):
    monkeypatch.setattr(nw, "PeriodMap", _FakeMap)
    p = _params()
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    fam = nw.ParamFamily(p, "Axz", pk, timep=2.0, xoff0=(-0.3, 0.3))
    a0 = fam.a0
    assert a0 == p.alp and fam.params(2 * a0).alp == 2 * a0 and fam.params(2 * a0).Ly == p.Ly
    # the period follows the shear period 2 pi / (alp Ly s) timep; alp xofft kept
    assert fam.period(a0) == pytest.approx(2 * np.pi / (p.alp * p.Ly * p.s) * 2.0, rel=1e-15)
    assert fam.period(2 * a0) == pytest.approx(fam.period(a0) / 2, rel=1e-15)
    assert fam.xoff(2 * a0) == pytest.approx((-0.15, 0.15), rel=1e-15)
    ly = nw.ParamFamily(p, "Ayz", pk, T=5.0)
    assert ly.period(3.0) == 5.0 and ly.xoff(3.0) == (0.0, 0.0)
    with pytest.raises(ValueError):
        nw.ParamFamily(p, "damp_xy", pk, T=1.0)
    with pytest.raises(ValueError):
        nw.ParamFamily(p, "damp_up", pk, T=1.0)  # no window damping in p
    pd = _params(damping=1, damp_up=0.3, damp_aa=0.1)
    assert nw.ParamFamily(pd, "damp_aa", pk, T=1.0).params(0.2).damp_aa == 0.2
    with pytest.raises(ValueError):
        nw.ParamFamily(p, "LES_Cs", pk, T=1.0)  # not an LES handle
    with pytest.raises(ValueError):
        nw.ParamFamily(p, "Ayz", pk)  # neither T nor timep
    # one handle per value, the oldest closed beyond `keep`
    _FakeMap.made.clear()
    fam3 = nw.ParamFamily(p, "Ayz", pk, T=1.0, keep=1)  # at least three are kept
    x = pk.pack(sb.seed_state(p, 3))
    fam3.G([x, x, x, x], [3.0, 3.1, 3.0, 3.2])
    assert len(_FakeMap.made) == 3 and not any(m.closed for m in _FakeMap.made)
    fam3.G([x], [3.3])
    assert len(_FakeMap.made) == 4 and _FakeMap.made[0].closed
    # Rez: one handle, the values as member Reynolds numbers
    _FakeMap.made.clear()
    fre = nw.ParamFamily(p, "Rez", pk, T=1.0)
    g1, g2 = fre.G([x, x], [p.Re, 2 * p.Re])
    assert len(_FakeMap.made) == 1 and not np.allclose(g1, g2)


@pytest.mark.parametrize("cpara,field", [("Ayz", "Ly"), ("Axz", "alp"), ("Rez", "Re")])
def test_param_family_derivative_and_jacobian(monkeypatch, cpara, field):
    monkeypatch.setattr(nw, "PeriodMap", _FakeMap)
    p = _params()
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    x = pk.pack(sb.seed_state(p, 5))
    fam = nw.ParamFamily(p, cpara, pk, T=2.0, xoff0=(-0.2, 0.2), batch=4)
    a = fam.a0 * 1.01
    h = 1e-4 * fam.a0
    # centred derivative against a wide centred difference of the same map
    ref = (fam.G([x], [a + h])[0] - fam.G([x], [a - h])[0]) / (2 * h)
    d = fam.derivative(x, a, daa=1e-6 * fam.a0)
    assert rel_l2(d, ref) < 1e-6
    fwd = fam.derivative(x, a, daa=1e-6 * fam.a0, central=False)
    assert rel_l2(fwd, ref) < 1e-4
    # the bordered operator: parameter column and secant row
    F, G = fam.residual(x, a)
    assert np.allclose(F, G - x)
    xstan = np.random.default_rng(1).standard_normal(x.size)
    Jx = fam.jacobian(x, a, G, xstan)
    e = np.zeros(x.size + 1)
    e[-1] = 1.0
    col = Jx.matvec(e)[:, 0]
    assert rel_l2(col[:-1], Jx.dgdre) < 1e-15 and col[-1] == 0.0
    dx = np.random.default_rng(2).standard_normal(x.size)
    v = Jx.matvec(np.concatenate([dx, [0.0]]))[:, 0]
    assert v[-1] == pytest.approx(xstan @ dx, rel=1e-12)


def test_param_family_les_cs_step(monkeypatch):
    monkeypatch.setattr(nw, "PeriodMap", _FakeMap)
    p = _params(les=1, les_visc=1, cs=0.1)
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    x = pk.pack(sb.seed_state(p, 6))
    fam = nw.ParamFamily(p, "LES_Cs", pk, T=1.0)
    seen = []
    real_G = fam.G

    def spy(xs, avals):
        seen.extend(avals)
        return real_G(xs, avals)
    fam.G = spy
    fam.derivative(x, 0.1)
    # set_dxda takes a tenth of daa for Cs
    assert sorted(seen) == pytest.approx([0.1 - 1e-7, 0.1 + 1e-7], rel=1e-12)


@pytest.mark.gpu
def test_arclength_in_ly_gpu():
    # manufactured curve through (x*, Ly*) as in the Re case, along Ly with a
    # handle per value of Ly (ParamFamily 'Ayz'): a Newton solution at
    # 0.999 Ly*, then one arclength step past x*
    p = _params()
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    xs = _seeded_x(p, pk, 16)
    ly_s = p.Ly
    probe = nw.ParamFamily(p, "Ayz", pk, T=10.0, batch=1)
    rhs = probe.G([xs], [ly_s])[0] - xs
    fam = nw.ParamFamily(p, "Ayz", pk, T=10.0, batch=8, rhs=rhs, eps_jacobi=1e-7)
    ly1 = 0.999 * ly_s
    J1 = lambda x: nw.Jacobian(fam.pmap(ly1), pk, x, eps_jacobi=1e-7, central=True)
    x1, h1 = nw.newton(xs, lambda x: fam.residual(x, ly1)[0], J1, k=16, block=4, itmax=12,
                       tol=1e-11, gmres_tol=1e-9)
    assert h1[-1] <= 1e-11, h1
    xp, lyp, xstan = nw.arclength_predictor(x1, ly1, xs, ly_s, 1.0)
    x, ly, hist = nw.newton_arclength(x1, ly1, xs, ly_s, 1.0, fam.residual, fam.jacobian, k=32,
                                      block=4, itmax=12, tol=1e-10, gmres_tol=1e-9)
    assert hist[-1] <= 1e-10, hist
    # the secant here is short (|xstan| ~ 2e-3 |x|): the plane holds to the
    # Krylov solves' accuracy in the extra row
    assert abs(xstan @ (x - xp)) <= 1e-7 * np.linalg.norm(xstan) * np.linalg.norm(x)
    assert abs(ly - 1.001 * ly_s) < 2.5e-4 * ly_s


# ---------------------------------------------------------------------------
# extra unknowns: bordered Jacobian, period derivative, flow direction
# ---------------------------------------------------------------------------

def test_bordered_jacobian_matches_dense():
    rng = np.random.default_rng(11)
    n, m = 30, 3
    A = rng.standard_normal((n, n))
    cols = [rng.standard_normal(n) for _ in range(m)]
    rows = [rng.standard_normal(n) for _ in range(m)]

    class J:
        def matvec(self, D):
            return A @ D

    BJ = nw.BorderedJacobian(J(), cols, rows)
    M = np.zeros((n + m, n + m))
    M[:n, :n] = A - np.eye(n)
    for q in range(m):
        M[:n, n + q] = cols[q]
        M[n + q, :n] = rows[q]
    D = rng.standard_normal((n + m, 4))
    assert np.allclose(BJ.matvec(D), M @ D)


class _DecayMap:
    """Phi_T(x) = exp(-lam T) x entrywise, with per-state integration times."""

    def __init__(self, p, T, lam=0.3, batch=4):
        self.p, self.T, self.lam, self.batch = p, T, lam, batch

    def __call__(self, states, res=None, Ts=None):
        out = []
        for q, s in enumerate(states):
            T = Ts[q] if Ts is not None else self.T
            f = np.exp(-self.lam * T)
            out.append(dict(s, vor=s["vor"] * f, phi=s["phi"] * f, u00=s["u00"] * f,
                            w00=s["w00"] * f))
        return out


def test_period_derivative_and_flow_direction():
    p = _params()
    pk = nw.Packing(p)
    x0 = _seeded_x(p, pk, 43)
    dm = _DecayMap(p, T=2.0)
    J = nw.Jacobian(dm, pk, x0, eps_jacobi=1e-6)
    dgdt = nw.period_derivative(J, 2.0, h=1e-3)
    assert rel_l2(dgdt, -0.3 * np.exp(-0.6) * x0) < 1e-6
    f0 = nw.flow_direction(dm, pk, x0, h=1e-3)
    assert rel_l2(f0, -0.3 * x0) < 1e-6


def test_newton_extended_on_a_matrix_problem():
    # F(x, a) = (A - I) x + a0 b0 + a1 b1 + c + 0.02 x^3 with the conditions
    # <r_k, dx> = 0: the root lies on the affine plane through x0
    rng = np.random.default_rng(12)
    n = 50
    A = _test_matrix(n, [0.5, 0.4, 0.3], seed=13)
    b0, b1, c = (0.3 * rng.standard_normal(n) for _ in range(3))
    r0, r1 = rng.standard_normal(n), rng.standard_normal(n)

    def residual_at(x, a):
        f = (A - np.eye(n)) @ x + a[0] * b0 + a[1] * b1 + c + 0.02 * x ** 3
        return f, f + x

    class Jx:
        def __init__(self, x):
            self.M = A + np.diag(0.06 * x ** 2)

        def matvec(self, D):
            return self.M @ D

    x0 = 0.1 * rng.standard_normal(n)
    x, a, hist = nw.newton_extended(
        x0, [0.2, -0.1], residual_at,
        lambda x, a, G: nw.BorderedJacobian(Jx(x), [b0, b1], [r0, r1]), k=n + 2, itmax=20,
        tol=1e-13, gmres_tol=1e-12)
    assert hist[-1] <= 1e-13, hist
    assert abs(r0 @ (x - x0)) < 1e-10 and abs(r1 @ (x - x0)) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("hook", [False, True])
def test_newton_unknown_shift_and_period_gpu(hook):
    # manufactured family through (x*, s*, T*): F(x, s, T) = shift_s(Phi_T(x)) - x - rhs
    p = _params()
    T_s, s_s, h = 10.0, 0.3, 1e-3
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    xs = _seeded_x(p, pk, 18)
    pm1 = nw.PeriodMap(p, T_s, batch=2)

    def G_of(x, a):
        st = pm1([pk.unpack(x)], Ts=[a[1]])[0]
        return pk.pack(nw.phase_shift(st, p, a[0], 0.0))

    rhs = G_of(xs, [s_s, T_s]) - xs

    def residual_at(x, a):
        G = G_of(x, a)
        return G - x - rhs, G

    pm = nw.PeriodMap(p, T_s, batch=8)

    def jac_at(x, a, G):
        pm.T = float(a[1])
        J = nw.Jacobian(pm, pk, x, shiftx=float(a[0]), eps_jacobi=1e-7, central=True)
        tx = nw.shift_tangent(pk, p, x)
        f0 = nw.flow_direction(pm1, pk, x, h)
        return nw.BorderedJacobian(J, [nw.shift_tangent(pk, p, G), nw.period_derivative(J, a[1], h)],
                                   [tx / np.linalg.norm(tx), f0 / np.linalg.norm(f0)])

    x0 = xs + 1e-3 * np.linalg.norm(xs) / np.sqrt(pk.n) * \
        np.random.default_rng(19).standard_normal(pk.n)
    x, a, hist = nw.newton_extended(x0, [s_s - 0.02, T_s + 0.05], residual_at, jac_at, k=16,
                                    block=4, itmax=12, tol=1e-10, gmres_tol=1e-8,
                                    delta=(0.05 * np.linalg.norm(xs) if hook else None))
    assert hist[-1] <= 1e-10, hist
    F, _ = residual_at(x, a)
    assert np.linalg.norm(F) <= 1e-10 * np.linalg.norm(x)


@pytest.mark.gpu
@pytest.mark.parametrize("central", [False, True])
def test_jv_batch_c_abi_matches_single_integrations(central):
    """sb_jv_batch (flat state vectors, the handle's batch as the block) gives
    the same quotients as single integrations through the public API.  The
    step eps is ~1e-7 |x0|, so a rounding difference of the perturbed state
    (its norm is summed in another order by numpy) shows up ~1e9 times larger
    in the quotient: the bar is 1e-7."""
    p = _params()
    T = 0.5
    box = sb.ShearBox(p, batch=4)
    st0 = sb.seed_state(p, 21)
    x0 = box.state_vector(st0)
    dirs = np.random.default_rng(4).standard_normal((5, x0.size))  # more than one block
    out = box.jv_batch(x0, dirs, T, eps_jacobi=1e-7, central=central)
    sz = sb.sizes(p)
    nf = 2 * sz["nkx"] * sz["mz"] * p.my

    def to_state(x):
        shp = (sz["mz"], sz["nkx"], p.my)
        return {"vor": x[:nf].copy().view(np.complex128).reshape(shp),
                "phi": x[nf:2 * nf].copy().view(np.complex128).reshape(shp),
                "u00": x[2 * nf:2 * nf + p.my].copy(), "w00": x[2 * nf + p.my:].copy(),
                "time": 0.0, "xoffb": 0.0, "xofft": 0.0}

    pm = nw.PeriodMap(p, T, batch=1)

    def phi_T(x):
        return box.state_vector(pm([to_state(x)])[0])

    eps_j = 1e-7 * np.linalg.norm(x0)
    g0 = None if central else phi_T(x0)
    for q in range(dirs.shape[0]):
        e = eps_j / np.linalg.norm(dirs[q])
        xp = x0 + ((x0 + e * dirs[q]) - x0)
        if central:
            xm = x0 + ((x0 - e * dirs[q]) - x0)
            ref = (phi_T(xp) - phi_T(xm)) / (2 * e)
        else:
            ref = (phi_T(xp) - g0) / e
        assert rel_l2(out[q], ref) < 1e-7, q


@pytest.mark.gpu
def test_stats_is_the_last_record():
    p = _params()
    box = sb.ShearBox(p)
    st = sb.seed_state(p, 22)
    tr, _ = box.cross(st, 3)
    u, u2 = box.stats()
    assert np.array_equal(u, tr[-1, 2:12]) and np.array_equal(u2, tr[-1, 20:24])
