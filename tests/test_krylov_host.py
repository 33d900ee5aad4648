"""The host logic of the device Newton-Krylov tools (shear_nnf_gb300.krylov)
on the CPU: block Gram-Schmidt, (block) GMRES with its restart directions,
block Arnoldi and the hookstep, run over a numpy stand-in for the device
column store.  The stand-in subclasses KSpace and replaces only the calls
into the library (sb_kspace_*) by their documented arithmetic, so the column
bookkeeping, the row ranges and every algorithm above the column algebra are
the product's own; the device algebra itself is checked against numpy in the
GPU tests."""
import numpy as np
import pytest

from shear_nnf_gb300 import krylov as kr


class HostSpace(kr.KSpace):
    """sb_kspace's column algebra (include/shearbox.h) in numpy FP64."""

    def __init__(self, n, cols):
        self.n, self.cols = int(n), int(cols)
        self.h = None
        self._free = np.ones(self.cols, bool)
        self.V = np.zeros((self.cols, self.n))

    def close(self):
        pass

    def sync(self):
        pass

    def col(self, c):
        if not 0 <= c < self.cols:
            raise kr.ShearBoxError(f"column {c} out of range")
        return 4096 + 8 * self.n * int(c)

    def gram(self, a0, m, b0, p, rows=None):
        r0, r1 = self._rows(rows)
        return self.V[a0:a0 + m, r0:r1] @ self.V[b0:b0 + p, r0:r1].T

    def update(self, a0, m, b0, p, C, alpha=1.0, rows=None):
        r0, r1 = self._rows(rows)
        C = np.asarray(C, np.float64).reshape(m, p)
        assert b0 >= a0 + m or b0 + p <= a0, "ranges must not overlap"
        self.V[b0:b0 + p, r0:r1] += alpha * (C.T @ self.V[a0:a0 + m, r0:r1])

    def transform(self, b0, p, M, rows=None):
        r0, r1 = self._rows(rows)
        M = np.asarray(M, np.float64).reshape(p, p)
        self.V[b0:b0 + p, r0:r1] = M.T @ self.V[b0:b0 + p, r0:r1]

    def combine(self, dst, srcs, coefs, rows=None):
        r0, r1 = self._rows(rows)
        acc = np.zeros(r1 - r0)
        for c, a in zip(srcs, np.asarray(coefs, np.float64).reshape(-1)):
            acc += a * self.V[c, r0:r1]
        self.V[dst, r0:r1] = acc

    def perturb(self, dst, x0, d, e, rows=None):
        r0, r1 = self._rows(rows)
        x = self.V[x0, r0:r1]
        self.V[dst, r0:r1] = x + ((x + e * self.V[d, r0:r1]) - x)

    def set(self, col, vec, off=0):
        v = np.asarray(vec, np.float64).reshape(-1)
        self.V[col, off:off + v.size] = v

    def get(self, col, off=0, length=None):
        length = self.n - off if length is None else int(length)
        return self.V[col, off:off + length].copy()


def _matrix_op(ks, A):
    def op(cin, cout):
        for a, b in zip(cin, cout):
            ks.V[b] = A @ ks.V[a]
    return op


@pytest.mark.parametrize("prev", [0, 3])
def test_block_orthonormalize_factorises_the_block(prev):
    """Columns come out orthonormal (and orthogonal to the `prev` basis
    columns), with input = basis Hprev + Q R."""
    rng = np.random.default_rng(1)
    n, p = 200, 4
    ks = HostSpace(n, 16)
    base = ks.alloc(max(prev, 1))
    if prev:
        Qb, _ = np.linalg.qr(rng.standard_normal((n, prev)))
        ks.V[base:base + prev] = Qb.T
    c0 = ks.alloc(p)
    X = rng.standard_normal((p, n))
    ks.V[c0:c0 + p] = X
    Hprev, R = kr.block_orthonormalize(ks, c0, p, None, prev=prev, base=base)
    Q = ks.V[c0:c0 + p]
    assert np.allclose(Q @ Q.T, np.eye(p), atol=1e-13)
    if prev:
        assert np.abs(ks.V[base:base + prev] @ Q.T).max() < 1e-13
        rebuilt = Hprev.T @ ks.V[base:base + prev] + R.T @ Q
    else:
        rebuilt = R.T @ Q
    assert np.allclose(rebuilt, X, atol=1e-12)
    assert np.allclose(R, np.triu(R))


def test_block_orthonormalize_replaces_a_dependent_column():
    """A column that is a combination of the earlier ones is replaced by a
    unit vector orthogonal to them, with a zero on R's diagonal."""
    rng = np.random.default_rng(2)
    n = 100
    ks = HostSpace(n, 8)
    c0 = ks.alloc(3)
    ks.V[c0] = rng.standard_normal(n)
    ks.V[c0 + 1] = rng.standard_normal(n)
    ks.V[c0 + 2] = 2.0 * ks.V[c0] - 0.5 * ks.V[c0 + 1]
    _, R = kr.block_orthonormalize(ks, c0, 3, None)
    Q = ks.V[c0:c0 + 3]
    assert np.allclose(Q @ Q.T, np.eye(3), atol=1e-12)
    assert R[2, 2] == 0.0 and R[0, 0] > 0 and R[1, 1] > 0


def test_row_ranges_leave_other_rows_alone():
    """Operations on a row range (the packed vector's part of an extended
    column) do not touch the rows outside it."""
    rng = np.random.default_rng(3)
    ks = HostSpace(50, 6)
    c0 = ks.alloc(2)
    ks.V[c0:c0 + 2] = rng.standard_normal((2, 50))
    tail = ks.V[c0:c0 + 2, 40:].copy()
    kr.block_orthonormalize(ks, c0, 2, (0, 40))
    assert np.array_equal(ks.V[c0:c0 + 2, 40:], tail)
    Q = ks.V[c0:c0 + 2, :40]
    assert np.allclose(Q @ Q.T, np.eye(2), atol=1e-13)


@pytest.mark.parametrize("block", [1, 3])
def test_gmres_solves_a_nonsymmetric_system(block):
    """GMRES from x = 0 on a well-conditioned non-normal matrix: the residual
    history decreases and the solution matches numpy's solve."""
    rng = np.random.default_rng(4)
    n = 120
    A = np.eye(n) * 2.0 + 0.3 * rng.standard_normal((n, n)) / np.sqrt(n)
    A[np.triu_indices(n, 1)] *= 1.5
    ks = HostSpace(n, 160)
    b = ks.alloc(1)
    bv = rng.standard_normal(n)
    ks.set(b, bv)
    k = 60 // block
    x, res, KB = kr.gmres_dev(ks, _matrix_op(ks, A), b, k, block=block, tol=1e-12)
    assert res[-1] <= 1e-12 * res[0]
    assert all(r1 <= r0 * (1 + 1e-12) for r0, r1 in zip(res, res[1:]))
    xv = ks.get(x)
    assert np.linalg.norm(A @ xv - bv) <= 1e-11 * np.linalg.norm(bv)
    # the kept basis and Hessenberg matrix satisfy A V_m = V_{m+p} H
    m = KB.m
    Vm = ks.V[KB.c0:KB.c0 + m + block]
    assert np.allclose(A @ Vm[:m].T, Vm.T @ KB.H, atol=1e-10)
    ks.release(x)
    ks.release(KB.c0, (k + 1) * block)
    assert ks._free.sum() == ks.cols - 1


def test_gmres_zero_rhs_and_column_budget():
    ks = HostSpace(30, 20)
    b = ks.alloc(1)
    x, res, KB = kr.gmres_dev(ks, _matrix_op(ks, np.eye(30)), b, 5)
    assert res == [0.0] and np.all(ks.get(x) == 0)
    ks.release(x)
    ks.release(KB.c0, 6)
    with pytest.raises(kr.ShearBoxError):
        kr.gmres_dev(ks, _matrix_op(ks, np.eye(30)), b, 25)


def test_ritz_directions_restart_gmres():
    """Directions written from one solve's Hessenberg matrix are orthonormal
    and lie in that solve's Krylov space; a second block solve started from
    them converges."""
    rng = np.random.default_rng(5)
    n = 150
    ev = np.concatenate([[3.0, 2.6, -2.2], 0.5 + 0.2 * rng.random(n - 3)])
    Qm, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Qm * ev) @ Qm.T
    ks = HostSpace(n, 120)
    b = ks.alloc(1)
    ks.set(b, rng.standard_normal(n))
    x, res, KB = kr.gmres_dev(ks, _matrix_op(ks, A), b, 20)
    d0 = ks.alloc(3)
    q = kr.ritz_directions(KB, 3, d0, shift=0.0)
    assert q == 3
    D = ks.V[d0:d0 + q]
    assert np.allclose(D @ D.T, np.eye(q), atol=1e-12)
    Vm = ks.V[KB.c0:KB.c0 + KB.m]
    assert np.allclose(D.T, Vm.T @ (Vm @ D.T), atol=1e-10)
    ks.release(x)
    ks.release(KB.c0, 21)
    b2 = ks.alloc(1)
    ks.set(b2, rng.standard_normal(n))
    x2, res2, KB2 = kr.gmres_dev(ks, _matrix_op(ks, A), b2, 12, block=4, tol=1e-10,
                                 start=[d0, d0 + 1, d0 + 2])
    assert res2[-1] <= 1e-10 * res2[0]


@pytest.mark.parametrize("block", [1, 4])
def test_arnoldi_finds_the_leading_eigenvalues(block):
    """Block Arnoldi on a normal matrix with five well-separated leading
    eigenvalues (one complex pair): Ritz values to 1e-8 with small residual
    estimates; the basis columns are released."""
    rng = np.random.default_rng(6)
    n = 300
    lead = [1.2, 0.95 + 0.2j, 0.95 - 0.2j, -0.8, 0.7]
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    B = np.diag(np.concatenate([[1.2, 0.0, 0.0, -0.8, 0.7], 0.3 * rng.random(n - 5)]))
    B[1:3, 1:3] = [[0.95, 0.2], [-0.2, 0.95]]
    A = Q @ B @ Q.T
    ks = HostSpace(n, 200)
    lam, res, H = kr.arnoldi_dev(ks, _matrix_op(ks, A), 60 // block, block=block, seed=7)
    assert ks._free.all()
    got = lam[:5]
    for z in lead:
        assert np.min(np.abs(got - z)) < 1e-8, (z, got)
    assert np.all(res[:5] < 1e-6)


def test_hookstep_respects_the_trust_region():
    """Inside the region the step is the least-squares solution; outside it
    lies on the boundary and is the regularised solution for the returned mu."""
    rng = np.random.default_rng(8)
    H = rng.standard_normal((11, 10))
    rhs = rng.standard_normal(11)
    y_ls = np.linalg.lstsq(H, rhs, rcond=None)[0]
    y, mu, pred = kr.hookstep_coeffs(H, rhs, 10 * np.linalg.norm(y_ls))
    assert mu == 0.0 and np.allclose(y, y_ls)
    assert pred == pytest.approx(np.linalg.norm(H @ y_ls - rhs))
    delta = 0.3 * np.linalg.norm(y_ls)
    y, mu, pred = kr.hookstep_coeffs(H, rhs, delta)
    assert mu > 0 and np.linalg.norm(y) == pytest.approx(delta, rel=1e-9)
    y_mu = np.linalg.solve(H.T @ H + mu * np.eye(10), H.T @ rhs)
    assert np.allclose(y, y_mu, atol=1e-10)
    assert pred >= np.linalg.norm(H @ y_ls - rhs)
