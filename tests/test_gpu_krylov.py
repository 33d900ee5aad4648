"""Device-resident Krylov algebra of the Newton/Arnoldi searches (sb_kspace,
shear_nnf_gb300.krylov) against numpy FP64 and the host tools: inner
products, block updates and transforms to 1e-14, the finite-difference
step and products bit for bit, the packed state against Packing, products
of the device Jacobian against the host Jacobian, GMRES and Arnoldi on the
device against known answers, and a Newton search for a relative periodic
orbit with FP32-mixed batched products and FP64 residuals."""
import numpy as np
import pytest

from conftest import box_params, rel_l2

import shear_nnf_gb300 as sb
from shear_nnf_gb300 import krylov as kr
from shear_nnf_gb300 import newton as nw

pytestmark = pytest.mark.gpu
ALG = 1e-14  # FP64 vector algebra against numpy


def _params(**kw):
    return sb.make_params(**box_params(64, 32, 32, 1000.0, **kw))


def test_kspace_algebra_matches_numpy():
    rng = np.random.default_rng(1)
    n, cols = 100003, 24
    ks = kr.KSpace(n, cols)
    X = rng.standard_normal((cols, n))
    for c in range(cols):
        ks.set(c, X[c])
    # gram over all rows and a row range
    C = ks.gram(0, 5, 8, 7)
    ref = X[0:5] @ X[8:15].T
    assert np.abs(C - ref).max() < ALG * np.abs(ref).max() * 10
    C2 = ks.gram(2, 3, 20, 2, rows=(17, 90001))
    ref2 = X[2:5, 17:90001] @ X[20:22, 17:90001].T
    assert np.abs(C2 - ref2).max() < ALG * np.abs(ref2).max() * 10
    # deterministic: the same call twice gives the same bits
    assert np.array_equal(ks.gram(0, 5, 8, 7), C)
    # update: cols 8..14 += -1 * X[0:5]^T-combination
    M = rng.standard_normal((5, 7))
    ks.update(0, 5, 8, 7, M, -1.0)
    want = X[8:15] - (M.T @ X[0:5])
    got = np.stack([ks.get(8 + b) for b in range(7)])
    assert np.abs(got - want).max() < ALG * np.abs(want).max() * 10
    # transform in place
    T = rng.standard_normal((4, 4))
    ks.transform(16, 4, T)
    want = T.T @ X[16:20]
    got = np.stack([ks.get(16 + b) for b in range(4)])
    assert np.abs(got - want).max() < ALG * np.abs(want).max() * 10
    # combine, perturb (bit for bit against the host formula), fd
    ks.combine(23, [0, 1, 2], [0.5, -2.0, 3.0])
    assert np.abs(ks.get(23) - (0.5 * X[0] - 2.0 * X[1] + 3.0 * X[2])).max() < 1e-13
    e = 1.234e-5
    ks.perturb(22, 3, 4, e)
    assert np.array_equal(ks.get(22), X[3] + ((X[3] + e * X[4]) - X[3]))
    ks.fd(21, 1, [5, 6], 0.37)
    assert np.array_equal(ks.get(21), (X[5] - X[6]) / 0.37)
    ks.fd(21, 2, [5, 6], 0.37)
    assert np.array_equal(ks.get(21), (X[5] - X[6]) / (2 * 0.37))
    ks.set(0, X[0])
    ks.fd(21, 4, [0, 5, 6, 7], 0.37)
    assert np.array_equal(ks.get(21), (8.0 * (X[0] - X[5]) - (X[6] - X[7])) / (12 * 0.37))
    assert abs(ks.norm(7) - np.linalg.norm(X[7])) < 1e-13 * np.linalg.norm(X[7])


def test_packed_state_matches_packing():
    p = _params()
    sca = nw.Packing.reference_scales(p)
    pk = nw.Packing(p, *sca)
    st = sb.seed_state(p, 11)
    for prec in (sb.SB_FP64, sb.SB_MIXED):
        box = sb.ShearBox(p, batch=2, precision=prec)
        assert box.packed_length == pk.n
        ks = kr.KSpace(pk.n, 3)
        box.set_state(st, 1)
        box.get_state_packed(1, ks.col(0), sca)
        box.sync()
        want = pk.pack(box.get_state(1))
        got = ks.get(0)
        assert np.array_equal(got, want) if prec == sb.SB_FP64 else rel_l2(got, want) < 1e-15
        # shifted
        box.get_state_packed(1, ks.col(1), sca, 0.3, -0.2)
        box.sync()
        want = pk.pack(nw.phase_shift(box.get_state(1), p, 0.3, -0.2))
        assert rel_l2(ks.get(1), want) < 1e-14
        # back into member 0 from the device vector: set_conj and (0,0) restored
        x = pk.pack(st)
        ks.set(2, x)
        box.set_state_packed(0, ks.col(2), sca, 1.5, -0.25, 0.25)
        back = box.get_state(0)
        ref = pk.unpack(x, 1.5, -0.25, 0.25)
        tol = 0.0 if prec == sb.SB_FP64 else 1e-7
        for k in ("vor", "phi", "u00", "w00"):
            assert rel_l2(back[k], ref[k]) <= tol, (prec, k)
        assert (back["time"], back["xoffb"], back["xofft"]) == (1.5, -0.25, 0.25)
        # the shift tangent on the device against the host formula
        box.shift_tangent_packed(ks.col(2), ks.col(1), "x")
        box.sync()
        assert rel_l2(ks.get(1), nw.shift_tangent(pk, p, x, "x")) < 1e-15
        box.shift_tangent_packed(ks.col(2), ks.col(1), "z")
        box.sync()
        assert rel_l2(ks.get(1), nw.shift_tangent(pk, p, x, "z")) < 1e-15


@pytest.mark.parametrize("order", [1, 2])
def test_device_products_match_host_products(order):
    """FP64 products through device vectors equal the host tool's products."""
    p = _params()
    sca = nw.Packing.reference_scales(p)
    pk = nw.Packing(p, *sca)
    T = 0.3
    x0 = pk.pack(sb.seed_state(p, 5))
    D = np.random.default_rng(6).standard_normal((pk.n, 3))
    host = nw.Jacobian(nw.PeriodMap(p, T, batch=4), pk, x0, eps_jacobi=1e-6, order=order,
                       shiftx=0.2)
    want = host.matvec(D)
    ks = kr.KSpace(pk.n, 16)
    xc, dc, oc = ks.alloc(1), ks.alloc(3), ks.alloc(3)
    ks.set(xc, x0)
    for q in range(3):
        ks.set(dc + q, D[:, q])
    pm = kr.DevPeriodMap(p, T, batch=4, sca=sca)
    J = kr.DevJacobian(pm, ks, xc, shift=(0.2, 0.0), eps_jacobi=1e-6, order=order)
    J.matvec([dc, dc + 1, dc + 2], [oc, oc + 1, oc + 2])
    got = np.stack([ks.get(oc + q) for q in range(3)], axis=1)
    # the step eps = eps_jacobi |x0| / |d| comes from device norms (fixed-order
    # sums) against numpy's: a last-bit difference of eps moves the
    # representable step h in a few entries, 1e-10 of a product at most
    assert rel_l2(got, want) < 1e-9


@pytest.mark.parametrize("block", [1, 4])
def test_gmres_and_arnoldi_on_device_operator(block):
    """A diagonal operator with a known spectrum: device GMRES solves to
    1e-10 and device Arnoldi finds the leading eigenvalues."""
    n = 5000
    rng = np.random.default_rng(2)
    ev = np.concatenate([[1.0, 0.9, 0.8, 0.7, 0.6], 0.3 * rng.random(n - 5)])
    ks = kr.KSpace(n, 200)

    # the test operators act through the host; the algebra under test (the
    # projections, norms and updates of GMRES and Arnoldi) stays on the device
    def op(cin, cout):
        for a, b in zip(cin, cout):
            ks.set(b, ks.get(a) * ev)

    lam, res, _ = kr.arnoldi_dev(ks, op, 40 // block, block=block, seed=3)
    assert np.allclose(np.sort(lam.real)[::-1][:5], ev[:5], atol=1e-6)
    b = ks.alloc(1)
    bv = rng.standard_normal(n)
    ks.set(b, bv)

    def op2(cin, cout):
        for a, c in zip(cin, cout):
            v = ks.get(a)
            ks.set(c, v * ev - 1.5 * v)

    x, rh, KB = kr.gmres_dev(ks, op2, b, 60 // block, block=block, tol=1e-10)
    xv = ks.get(x)
    assert rh[-1] <= 1e-10 * rh[0]
    assert np.linalg.norm(xv * (ev - 1.5) - bv) <= 1e-9 * np.linalg.norm(bv)
    ks.release(x)
    ks.release(KB.c0, (60 // block + 1) * block)


def test_floquet_stokes_known_answer_on_device():
    """Block Arnoldi with device vectors on the Stokes problem (s = 0): the
    leading multipliers are the exact discrete ones."""
    nu, dt, nsteps = 0.1, 0.01, 200
    p = sb.make_params(64, 32, 32, 1.0 / nu, 0.7, 5.0, 1.3, s=0.0, chi=0.0, CFL=0.5,
                       fixed_dt=dt, keep_laminar=1)
    pk = nw.Packing(p)
    ks = kr.KSpace(pk.n, 64)
    x0 = ks.alloc(1)
    ks.zero(x0)
    pm = kr.DevPeriodMap(p, nsteps * dt, batch=2)
    J = kr.DevJacobian(pm, ks, x0, eps_jacobi=1e-6, order=2)
    lam, res, _ = kr.arnoldi_dev(ks, J.matvec, 25, seed=7)
    from test_newton import _stokes_multipliers
    theory = _stokes_multipliers(p, nu, dt, nsteps)
    for q, tol in enumerate((1e-9, 1e-9, 1e-6, 1e-6)):
        assert abs(lam[q].imag) < 1e-10, (q, lam[:6], res[:6])
        assert abs(lam[q].real - theory[q]) < tol * theory[q], (q, lam[:6], theory[:6])
    assert res[0] < 1e-10


@pytest.mark.parametrize("hook", [False, True])
def test_newton_rpo_fp32_batched_products(hook):
    """Manufactured relative periodic orbit (x*, s*): F(x, s) =
    shift_s(Phi_T(x)) - x - rhs with rhs = F(x*, s*); Newton from a perturbed
    start with FP32-mixed batched products (base in the batch) and FP64
    residuals converges to |F|/|x| <= 1e-10, every vector on the device."""
    p = _params()
    sca = nw.Packing.reference_scales(p)
    pk = nw.Packing(p, *sca)
    T, s_star = 6.0, 0.3
    n = pk.n
    ks = kr.KSpace(n + 1, 400)
    xs = pk.pack(sb.seed_state(p, 14))
    rhs = ks.alloc(1)
    x = ks.alloc(1)
    res64 = kr.DevPeriodMap(p, T, batch=1, sca=sca)
    ks.set(x, xs)
    res64(ks, [x], [rhs], shift=(s_star, 0.0))
    ks.combine(rhs, [rhs, x], [1.0, -1.0], n)
    pert = 1e-3 * np.linalg.norm(xs) / np.sqrt(n) * np.random.default_rng(15).standard_normal(n)
    ks.set(x, np.concatenate([xs + pert, [0.0]]))
    pm32 = kr.DevPeriodMap(p, T, batch=9, precision=sb.SB_MIXED, sca=sca)
    s, hist, stats = kr.newton_rpo(ks, p, x, s_star - 0.01, res64, pm32, rhs=rhs, k=12, block=8,
                                   itmax=12, tol=1e-10, gmres_tol=1e-4, eps_jacobi=1e-3,
                                   base_in_batch=True,
                                   delta=(0.05 * np.linalg.norm(xs) if hook else None))
    assert hist[-1] <= 1e-10, hist
    assert stats["products"] > 0 and pm32.box.batch == 9
    # the roots of F(x, s) = 0 form a curve (n equations, n + 1 unknowns; the
    # phase condition only fixes the steps), so the search lands on a root near
    # (x*, s*) rather than on it: check that root with the host tools
    xv = ks.get(x, 0, n)
    hres = nw.ShiftResidual(nw.PeriodMap(p, T, batch=1), pk, rhs=ks.get(rhs, 0, n))
    F, _ = hres(xv, s)
    assert np.linalg.norm(F) <= 2e-10 * np.linalg.norm(xv)
    assert abs(s - s_star) < 0.05 and rel_l2(xv, xs) < 1e-2
