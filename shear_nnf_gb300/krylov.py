"""Device-resident Newton-Krylov and Arnoldi over batched period maps.

The reference's periodic-orbit search (newton_shear.f90:183-597 with
gmres_k_shear, gmres_shear.f90:1905-2207) and its Floquet analysis
(arnoldi_shear.f90:222-406) keep their Krylov vectors on MPI rank 0 and do
every inner product, vector update and norm there (dotp, vecadd, norm,
gmres_shear.f90:3680-3919).  Here every vector of a search lives in one
device-resident Krylov space (sb_kspace, FP64 columns): the period map reads
its initial states from columns and writes its final states into columns
(sb_set_state_packed / sb_get_state_packed), the finite-difference products,
the Gram-Schmidt projections and the norms are FP64 kernels on those columns,
and only the small coefficient matrices cross to the host, where the
Hessenberg least-squares problems, the hookstep SVD and the Ritz values are
solved.

Pieces:
  KSpace         the column store with its FP64 vector algebra
  DevPeriodMap   x -> shift(Phi_T(x)) for a block of columns, one batched
                 integration per block (calc_dns_disk3d)
  DevJacobian    finite-difference products J d of order 1, 2 or 4
                 (matvec_dns_disk3d, iuse_hej), a block of directions per
                 batched integration
  ShiftSystem    the bordered operator of the relative periodic orbit with the
                 streamwise shift as unknown (isol_mode 4: the column dG/ds and
                 the phase row), on columns of n + 1 entries
  gmres_dev      (block) GMRES with classical Gram-Schmidt twice across blocks
                 and modified Gram-Schmidt inside a block
  arnoldi_dev    (block) Arnoldi, Ritz values and their residual estimates
  newton_rpo     Newton(-hookstep) for (x, s): FP64 residual, products from
                 any period map (FP32-mixed batches or FP64 one at a time),
                 optionally reusing the Krylov space of earlier iterations
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import SB_FP64, ShearBox, ShearBoxError, _check, _dp, lib


class KSpace:
    """`cols` device vectors of n FP64 entries (sb_kspace)."""

    def __init__(self, n: int, cols: int, stream: int = 0):
        self.n, self.cols = int(n), int(cols)
        h = ctypes.c_void_p()
        _check(lib().sb_kspace_create(self.n, self.cols, ctypes.c_void_p(stream or None),
                                      ctypes.byref(h)))
        self.h = h
        self._free = np.ones(self.cols, bool)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().sb_kspace_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # column allocation: contiguous first-fit ranges
    def alloc(self, k: int) -> int:
        k = int(k)
        run = 0
        for c in range(self.cols):
            run = run + 1 if self._free[c] else 0
            if run == k:
                c0 = c - k + 1
                self._free[c0:c + 1] = False
                return c0
        raise ShearBoxError(f"KSpace: no {k} free contiguous columns of {self.cols}")

    def release(self, c0: int, k: int = 1):
        self._free[int(c0):int(c0) + int(k)] = True

    def col(self, c: int) -> int:
        p = lib().sb_kspace_col(self.h, int(c))
        if not p:
            raise ShearBoxError(f"KSpace: column {c} out of range")
        return int(p)

    def _rows(self, rows):
        if rows is None:
            return 0, self.n
        if isinstance(rows, tuple):
            return int(rows[0]), int(rows[1])
        return 0, int(rows)

    def sync(self):
        _check(lib().sb_kspace_sync(self.h))

    def gram(self, a0: int, m: int, b0: int, p: int, rows=None) -> np.ndarray:
        r0, r1 = self._rows(rows)
        C = np.zeros((m, p))
        _check(lib().sb_kspace_gram(self.h, r0, r1, int(a0), int(m), int(b0), int(p), _dp(C)))
        return C

    def update(self, a0: int, m: int, b0: int, p: int, C, alpha: float = 1.0, rows=None):
        r0, r1 = self._rows(rows)
        C = np.ascontiguousarray(np.asarray(C, np.float64).reshape(m, p))
        _check(lib().sb_kspace_update(self.h, r0, r1, int(a0), int(m), int(b0), int(p), _dp(C),
                                      float(alpha)))

    def transform(self, b0: int, p: int, M, rows=None):
        r0, r1 = self._rows(rows)
        M = np.ascontiguousarray(np.asarray(M, np.float64).reshape(p, p))
        _check(lib().sb_kspace_transform(self.h, r0, r1, int(b0), int(p), _dp(M)))

    def combine(self, dst: int, srcs, coefs, rows=None):
        r0, r1 = self._rows(rows)
        s = (ctypes.c_int * max(len(srcs), 1))(*[int(c) for c in srcs])
        c = np.ascontiguousarray(np.asarray(coefs, np.float64).reshape(-1))
        if c.size == 0:
            c = np.zeros(1)
        _check(lib().sb_kspace_combine(self.h, r0, r1, int(dst), len(srcs), s, _dp(c)))

    def zero(self, dst: int, rows=None):
        self.combine(dst, [], [], rows)

    def copy(self, dst: int, src: int, rows=None):
        self.combine(dst, [src], [1.0], rows)

    def scale(self, dst: int, a: float, rows=None):
        self.combine(dst, [dst], [a], rows)

    def perturb(self, dst: int, x0: int, d: int, e: float, rows=None):
        r0, r1 = self._rows(rows)
        _check(lib().sb_kspace_perturb(self.h, r0, r1, int(dst), int(x0), int(d), float(e)))

    def fd(self, dst: int, order: int, gcols, eps: float, rows=None):
        r0, r1 = self._rows(rows)
        g = (ctypes.c_int * 4)(*([int(c) for c in gcols] + [0] * (4 - len(gcols))))
        _check(lib().sb_kspace_fd(self.h, r0, r1, int(dst), int(order), g, float(eps)))

    def set(self, col: int, vec, off: int = 0):
        v = np.ascontiguousarray(np.asarray(vec, np.float64).reshape(-1))
        _check(lib().sb_kspace_set(self.h, int(col), int(off), v.size, _dp(v)))

    def get(self, col: int, off: int = 0, length: int = None) -> np.ndarray:
        length = self.n - off if length is None else int(length)
        out = np.zeros(length)
        _check(lib().sb_kspace_get(self.h, int(col), int(off), length, _dp(out)))
        return out

    def dot(self, a: int, b: int, rows=None) -> float:
        return float(self.gram(a, 1, b, 1, rows)[0, 0])

    def norm(self, c: int, rows=None) -> float:
        return float(np.sqrt(max(self.dot(c, c, rows), 0.0)))


class DevPeriodMap:
    """x -> shift(Phi_T(x)) on packed columns, the members of one batch
    advanced together (calc_dns_disk3d).  Each member stops on its own end
    time; members beyond the block get their start time as end time and stop
    at once.  sca: the scalings of the packed vector (Packing.reference_scales).
    With autotune the handle's tiles (plane stages, warps per y-line solve)
    are timed on the states of the first call (sb_autotune)."""

    def __init__(self, p, T: float, batch: int, precision: int = SB_FP64, chunk: int = 256,
                 sca=(1.0, 1.0, 1.0), autotune: bool = False):
        self.p, self.T, self.batch, self.chunk = p, float(T), int(batch), int(chunk)
        self.autotune, self.tuning = autotune, None
        self.box = ShearBox(p, batch=self.batch, precision=precision)
        self.sca = np.asarray(sca, np.float64)
        self.n = self.box.packed_length
        self.integrations = 0
        self.steps = 0
        self.seconds = 0.0
        self.last_steps = []

    def __call__(self, ks: KSpace, in_cols, out_cols, time0=0.0, xoff=(0.0, 0.0),
                 shift=(0.0, 0.0), Ts=None, res=None):
        """Integrates the states of columns in_cols over T (or Ts[q]) at the
        Reynolds numbers res[q] (default the parameters'), writing the
        shifted final states into out_cols (which may equal in_cols)."""
        t0 = time.perf_counter()
        in_cols, out_cols = list(in_cols), list(out_cols)
        assert len(in_cols) == len(out_cols)
        box, B = self.box, self.batch
        steps = []
        for q0 in range(0, len(in_cols), B):
            grp = list(range(q0, min(q0 + B, len(in_cols))))
            ks.sync()
            for m in range(B):
                q = grp[m] if m < len(grp) else grp[0]
                box.set_state_packed(m, ks.col(in_cols[q]), self.sca, time0, *xoff)
                if m < len(grp):
                    T = Ts[q] if Ts is not None else self.T
                    box.set_etime(m, time0 + T)
                    box.set_re(m, res[q] if res is not None else self.p.Re)
                else:
                    # padding: an end time just past the start stops it at once
                    box.set_etime(m, time0 + max(1e-12, 1e-15 * abs(time0)))
                    box.set_re(m, self.p.Re)
            if self.autotune and not self.tuning:
                # tiles for this batch, timed on its first states (left as set)
                self.tuning = box.autotune()
            done = [0] * len(grp)
            fin = [False] * len(grp)
            for _ in range(1 << 20):
                box.step(self.chunk)
                for m in range(len(grp)):
                    if fin[m]:
                        continue
                    s = box.status(m)
                    if s.flags & 3 or (s.flags & 4 and not self.p.keep_laminar):
                        raise RuntimeError(f"period map: member {m} stopped (flags {s.flags})")
                    done[m] += s.steps_done
                    fin[m] = bool(s.flags & 8)
                if all(fin):
                    break
            for m, q in enumerate(grp):
                box.get_state_packed(m, ks.col(out_cols[q]), self.sca, *shift)
            box.sync()
            steps += done
        self.last_steps = steps
        self.steps += sum(steps)
        self.integrations += len(in_cols)
        self.seconds += time.perf_counter() - t0


class DevJacobian:
    """Finite-difference products J d of G(x) = shift(Phi_T(x)) at the column
    x0 (matvec_dns_disk3d, gmres_shear.f90:2666-2948): eps = eps_jacobi |x0| /
    |d| over the n state entries, the representable step h = (x0 + eps d) - x0,
    order 1 (G(x0 + h) - G(x0)) / eps, 2 (G(x0 + h) - G(x0 - h)) / (2 eps), or 4
    (8 (G(x0+h) - G(x0-h)) - (G(x0+2h) - G(x0-2h))) / (12 eps).  A block of
    directions is one batched integration; with base_in_batch G(x0) is
    integrated again as the first member of every block (FP32-mixed maps), else
    once (g0 column, computed on first use or given)."""

    def __init__(self, pmap: DevPeriodMap, ks: KSpace, x0: int, time0=0.0, xoff=(0.0, 0.0),
                 shift=(0.0, 0.0), eps_jacobi=1e-7, order=1, base_in_batch=False, g0: int = None,
                 re=None):
        if order not in (1, 2, 4):
            raise ValueError("order must be 1, 2 or 4")
        self.pmap, self.ks, self.x0 = pmap, ks, int(x0)
        self.time0, self.xoff, self.shift = time0, tuple(xoff), tuple(shift)
        self.eps_jacobi, self.order, self.base_in_batch = eps_jacobi, order, base_in_batch
        self.re = re
        self.n = pmap.n
        self._g0 = g0
        self.products = 0

    @property
    def block(self) -> int:
        per = {1: 1, 2: 2, 4: 4}[self.order]
        return (self.pmap.batch - (1 if self.base_in_batch else 0)) // per

    def g0(self) -> int:
        if self._g0 is None and not self.base_in_batch:
            c = self.ks.alloc(1)
            self._run([self.x0], [c])
            self._g0 = c
        return self._g0

    def _run(self, cin, cout):
        res = None if self.re is None else [self.re] * len(cin)
        self.pmap(self.ks, cin, cout, self.time0, self.xoff, self.shift, res=res)

    def matvec(self, dcols, ocols):
        """out column q = J (state part of column dcols[q]); rows n.. of the
        outputs are left as they are."""
        ks, n = self.ks, self.n
        nb = self.block
        if nb < 1:
            raise ValueError("matvec: batch too small for one product")
        xn = ks.norm(self.x0, n)
        eps_j = self.eps_jacobi * (xn if xn > 0 else 1.0)
        steps = {1: (1.0,), 2: (1.0, -1.0), 4: (1.0, -1.0, 2.0, -2.0)}[self.order]
        dcols, ocols = list(dcols), list(ocols)
        for q0 in range(0, len(dcols), nb):
            ds, os_ = dcols[q0:q0 + nb], ocols[q0:q0 + nb]
            nmem = len(ds) * len(steps) + (1 if self.base_in_batch else 0)
            tmp = ks.alloc(nmem)
            cols = list(range(tmp, tmp + nmem))
            base = None
            k = 0
            if self.base_in_batch:
                ks.copy(cols[0], self.x0, n)
                base, k = cols[0], 1
            eps = []
            for d in ds:
                dn = ks.norm(d, n)
                if not dn > 0:
                    raise ValueError("matvec: zero direction")
                e = eps_j / dn
                eps.append(e)
                for f in steps:
                    ks.perturb(cols[k], self.x0, d, f * e, n)
                    k += 1
            self._run(cols, cols)
            if base is None and self.order == 1:
                base = self.g0()
            ns = len(steps)
            off = 1 if self.base_in_batch else 0
            for q, (o, e) in enumerate(zip(os_, eps)):
                g = cols[off + ns * q: off + ns * (q + 1)]
                if self.order == 1:
                    ks.fd(o, 1, [g[0], base], e, n)
                elif self.order == 2:
                    ks.fd(o, 2, [g[0], g[1]], e, n)
                else:
                    ks.fd(o, 4, g, e, n)
            ks.sync()
            ks.release(tmp, nmem)
            self.products += len(ds)


def shift_tangent_dev(ks: KSpace, box: ShearBox, src: int, dst: int, which: str = "x"):
    """d/ds of shift_s(x) at s = 0 on a packed column: -i kx x (or -i kz x),
    the mean profiles zero (the derivative of phase_shift_fou), on the
    device."""
    ks.sync()
    box.shift_tangent_packed(ks.col(src), ks.col(dst), which)
    box.sync()


def block_orthonormalize(ks: KSpace, c0: int, p: int, rows, prev: int = 0, base: int = 0,
                         rng=None):
    """Orthonormalise columns c0..c0+p-1 against columns base..base+prev-1
    (classical Gram-Schmidt, twice) and among themselves (modified
    Gram-Schmidt, twice per column).  Returns (Hprev (prev x p), R (p x p)): the
    projections and the triangular factor.  A column that vanishes
    (linear dependence) is replaced by a random orthonormal one and its R
    column is zero there."""
    Hprev = np.zeros((prev, p))
    if prev > 0:
        for _ in range(2):
            C = ks.gram(base, prev, c0, p, rows)
            ks.update(base, prev, c0, p, C, -1.0, rows)
            Hprev += C
    R = np.zeros((p, p))
    for j in range(p):
        cj = c0 + j
        nrm0 = ks.norm(cj, rows)
        for _ in range(2):
            if j > 0:
                C = ks.gram(c0, j, cj, 1, rows)
                ks.update(c0, j, cj, 1, C, -1.0, rows)
                R[:j, j] += C[:, 0]
        nrm = ks.norm(cj, rows)
        if not nrm > 1e-12 * max(nrm0, 1e-300):
            # dependent: a random direction orthogonal to everything so far
            rng = rng or np.random.default_rng(1234 + j)
            r0, r1 = ks._rows(rows)
            v = np.zeros(ks.n)
            v[r0:r1] = rng.standard_normal(r1 - r0)
            ks.set(cj, v)
            if prev > 0:
                for _ in range(2):
                    C = ks.gram(base, prev, cj, 1, rows)
                    ks.update(base, prev, cj, 1, C, -1.0, rows)
            for _ in range(2):
                if j > 0:
                    C = ks.gram(c0, j, cj, 1, rows)
                    ks.update(c0, j, cj, 1, C, -1.0, rows)
            ks.scale(cj, 1.0 / ks.norm(cj, rows), rows)
            R[j, j] = 0.0
            continue
        R[j, j] = nrm
        ks.scale(cj, 1.0 / nrm, rows)
    return Hprev, R


class KrylovBasis:
    """The basis, Hessenberg matrix and projected right-hand side of a (block)
    GMRES run, kept for the hookstep."""

    def __init__(self, ks, c0, m, H, rhs):
        self.ks, self.c0, self.m, self.H, self.rhs = ks, c0, m, H, rhs

    def combine_into(self, dst: int, y, rows=None):
        self.ks.zero(dst, rows)
        self.ks.update(self.c0, self.m, dst, 1, np.asarray(y).reshape(-1, 1), 1.0, rows)


def gmres_dev(ks: KSpace, op, b: int, k: int, block: int = 1, tol: float = 0.0, rows=None,
              seed: int = 0, basis_cols: int = None, start=None):
    """(Block) GMRES for A x = b from x = 0 on device columns: op(in_cols,
    out_cols) applies A; the first basis vector is b/|b|, with block > 1 the
    other columns of the starting block are the columns `start` (directions
    kept from an earlier solve, e.g. ritz_directions) and then random ones.
    Returns (x column, residual-norm history, KrylovBasis); the caller
    releases the x column and the basis (KrylovBasis.c0, (k + 1) * block
    columns)."""
    p = int(block)
    r0, r1 = ks._rows(rows)
    beta = ks.norm(b, rows)
    ncols = basis_cols or (k + 1) * p
    V = ks.alloc(ncols)
    x = ks.alloc(1)
    ks.zero(x)
    if beta == 0:
        return x, [0.0], KrylovBasis(ks, V, 0, np.zeros((0, 0)), np.zeros(0))
    rng = np.random.default_rng(seed)
    ks.copy(V, b, rows)
    start = list(start or [])[: p - 1]
    for j in range(1, p):
        if j - 1 < len(start):
            ks.copy(V + j, start[j - 1], rows)
            continue
        v = np.zeros(ks.n)
        v[r0:r1] = rng.standard_normal(r1 - r0)
        ks.set(V + j, v)
    _, R0 = block_orthonormalize(ks, V, p, rows)
    H = np.zeros(((k + 1) * p, k * p))
    rhs0 = np.zeros((k + 1) * p)
    rhs0[:p] = R0[:, 0]
    res = [beta]
    y = None
    m = 0
    for it in range(k):
        cur, new = V + it * p, V + (it + 1) * p
        if new + p > V + ncols:
            break
        op(list(range(cur, cur + p)), list(range(new, new + p)))
        Hp, R = block_orthonormalize(ks, new, p, rows, prev=(it + 1) * p, base=V)
        H[: (it + 1) * p, it * p:(it + 1) * p] = Hp
        H[(it + 1) * p:(it + 2) * p, it * p:(it + 1) * p] = R
        m = (it + 1) * p
        Hm = H[: m + p, :m]
        y, *_ = np.linalg.lstsq(Hm, rhs0[: m + p], rcond=None)
        r = float(np.linalg.norm(rhs0[: m + p] - Hm @ y))
        res.append(r)
        if r <= tol * beta:
            break
    if m:
        ks.update(V, m, x, 1, y.reshape(-1, 1), 1.0, rows)
    return x, res, KrylovBasis(ks, V, m, H[: m + p, :m], rhs0[: m + p])


def ritz_directions(KB: KrylovBasis, q: int, dst0: int, rows=None, shift: float = 1.0) -> int:
    """Writes up to q real directions spanning the Ritz vectors of the
    projected operator H_m (KB) whose eigenvalues mu are farthest from -shift
    -- for A = J - I the eigenvalues of J of largest modulus, which GMRES
    resolves last -- into columns dst0.. (complex pairs as their real and
    imaginary parts, orthonormalised in Krylov coordinates).  Returns the
    number written.  The recycling of deflated restarting (GCRO-DR): the next
    solve starts from these directions beside its right-hand side."""
    m = KB.m
    if m == 0 or q <= 0:
        return 0
    Hm = KB.H[:m, :m]
    mu, Y = np.linalg.eig(Hm)
    order = np.argsort(-np.abs(mu + shift))
    cols = []
    for i in order:
        if len(cols) >= q:
            break
        y = Y[:, i]
        if abs(mu[i].imag) > 1e-14 * max(abs(mu[i]), 1e-300):
            if mu[i].imag < 0:
                continue  # the pair is taken once, from its upper member
            cols += [y.real, y.imag]
        else:
            cols.append(y.real)
    Yr = np.stack(cols[:q], axis=1)
    Qy, _ = np.linalg.qr(Yr)
    for j in range(Qy.shape[1]):
        KB.combine_into(dst0 + j, Qy[:, j], rows)
    return Qy.shape[1]


def arnoldi_dev(ks: KSpace, op, k: int, block: int = 1, rows=None, seed: int = 0, start=None):
    """Block Arnoldi (arnoldi_shear.f90:222-330 with block = 1): k iterations of
    `block` products.  Returns Ritz values (largest modulus first), their
    residual estimates |H_{k+1,k} y_k| for unit Ritz vectors y, and H; the
    basis columns are released."""
    p = int(block)
    r0, r1 = ks._rows(rows)
    V = ks.alloc((k + 1) * p)
    rng = np.random.default_rng(seed)
    for j in range(p):
        if start is not None and j < len(start):
            ks.copy(V + j, start[j], rows)
        else:
            v = np.zeros(ks.n)
            v[r0:r1] = rng.standard_normal(r1 - r0)
            ks.set(V + j, v)
    block_orthonormalize(ks, V, p, rows)
    H = np.zeros(((k + 1) * p, k * p))
    for it in range(k):
        cur, new = V + it * p, V + (it + 1) * p
        op(list(range(cur, cur + p)), list(range(new, new + p)))
        Hp, R = block_orthonormalize(ks, new, p, rows, prev=(it + 1) * p, base=V)
        H[: (it + 1) * p, it * p:(it + 1) * p] = Hp
        H[(it + 1) * p:(it + 2) * p, it * p:(it + 1) * p] = R
    ks.release(V, (k + 1) * p)
    Hk = H[: k * p, : k * p]
    lam, Y = np.linalg.eig(Hk)
    Y = Y / np.linalg.norm(Y, axis=0)
    res = np.linalg.norm(H[k * p:, (k - 1) * p:k * p] @ Y[(k - 1) * p:, :], axis=0)
    order = np.argsort(-np.abs(lam))
    return lam[order], res[order], H


def hookstep_coeffs(H: np.ndarray, rhs: np.ndarray, delta: float, iters: int = 200):
    """The trust-region step in Krylov coordinates (hookstep, gmres_shear.f90:
    4200-4419, with the mu iteration of solv_mu, 4064-4198): minimise
    |H y - rhs| subject to |y| <= delta through the SVD of H.  Returns
    (y, mu, predicted residual)."""
    U, s, Wt = np.linalg.svd(H, full_matrices=True)
    m = s.size
    pv = U.T @ rhs

    def q_of(mu):
        return s * pv[:m] / (s ** 2 + mu)

    mu = 0.0
    q = q_of(0.0)
    if np.linalg.norm(q) > delta:
        mu = 1e-3
        for _ in range(iters):
            q = q_of(mu)
            qn = np.linalg.norm(q)
            ph = qn * qn - delta * delta
            phprim = -2.0 * np.sum(q ** 2 / (s ** 2 + mu))
            mu = max(mu - (qn / delta) * (ph / phprim), 0.0)
            if abs(ph) <= 1e-12 * delta * delta:
                break
        q = q_of(mu)
    y = Wt.T @ q
    return y, mu, float(np.linalg.norm(H @ y - rhs))


class ShiftSystem:
    """The relative-periodic-orbit system with the streamwise shift s as the
    extra unknown (isol_mode 4), on columns of n + 1 entries (x, s):
        F(x, s) = shift_s(Phi_T(x)) - x - rhs,   <t, dx> = 0,
    with products [(J - I) dx + dG/ds ds ; <t, dx>], J the finite-difference
    Jacobian of the shifted map at (x0, s0), dG/ds = -i kx G(x0, s0) and
    t = -i kx x0 normalised (the phase condition of newton_shear.f90 with the
    shift, gmres_shear.f90:2900-2934)."""

    def __init__(self, J: DevJacobian, G: int):
        ks, n = J.ks, J.n
        self.J, self.ks, self.n = J, ks, n
        self.dgds = ks.alloc(1)
        self.t = ks.alloc(1)
        box = J.pmap.box
        shift_tangent_dev(ks, box, G, self.dgds, "x")
        shift_tangent_dev(ks, box, J.x0, self.t, "x")
        tn = ks.norm(self.t, n)
        ks.scale(self.t, 1.0 / max(tn, 1e-300), n)

    def release(self):
        self.ks.release(self.dgds)
        self.ks.release(self.t)

    def __call__(self, dcols, ocols):
        ks, n = self.ks, self.n
        self.J.matvec(dcols, ocols)
        for d, o in zip(dcols, ocols):
            ds = float(ks.get(d, n, 1)[0])
            ks.combine(o, [o, d, self.dgds], [1.0, -1.0, ds], n)
            ks.set(o, [ks.dot(self.t, d, n)], n)


def newton_rpo(ks: KSpace, p, x0: int, s0: float, res_map: DevPeriodMap, jac_map: DevPeriodMap,
               rhs: int = None, k: int = 20, block: int = 1, itmax: int = 10, tol: float = 1e-10,
               gmres_tol: float = 1e-3, delta: float = None, eps_jacobi: float = 1e-7,
               order: int = 1, base_in_batch: bool = False, time0: float = 0.0,
               xoff=(0.0, 0.0), log=None, recycle: int = 0):
    """Newton(-hookstep) search for a relative periodic orbit (x, s) with the
    streamwise shift s unknown (newton_shear.f90:183-597, isol_mode 4) on
    device columns of n + 1 entries: residual F = shift_s(Phi_T(x)) - x - rhs
    from the FP64 map res_map, products from jac_map (an FP32-mixed batch or
    the FP64 map itself), GMRES to gmres_tol per step (iterative refinement:
    the FP64 residual of the next iterate corrects what approximate products
    miss).  With delta every step is a hookstep of at most delta in the
    Krylov space, delta halved on a failed step and doubled on a good one
    (newton_shear.f90:446-490).  With recycle = q > 0 each GMRES solve after
    the first starts from the right-hand side and q Ritz directions of the
    previous solve (ritz_directions), so a block of q + 1 products per
    iteration carries the directions the solve needs most.  x0 is a column
    (n + 1 entries, the last ignored); the iterate is written back into it.
    Returns (s, history of |F|/|x|, stats)."""
    n = res_map.n
    N = n + 1
    rows_n = (0, n)
    G = ks.alloc(1)
    F = ks.alloc(1)
    xt = ks.alloc(1)
    stats = {"newton": 0, "gmres_iterations": 0, "products": 0, "residuals": 0,
             "hook_trials": 0}

    def residual(xc, s):
        res_map(ks, [xc], [G], time0, xoff, (s, 0.0))
        stats["residuals"] += 1
        srcs, coefs = [G, xc], [1.0, -1.0]
        if rhs is not None:
            srcs.append(rhs)
            coefs.append(-1.0)
        ks.combine(F, srcs, coefs, rows_n)
        ks.set(F, [0.0], n)
        return ks.norm(F, rows_n) / max(ks.norm(xc, rows_n), 1e-300)

    s = float(s0)
    U = ks.alloc(recycle) if recycle > 0 else None
    nU = 0
    hist = [residual(x0, s)]
    if log:
        log(f"newton 0: |F|/|x| = {hist[-1]:.3e}")
    for it in range(itmax):
        if hist[-1] <= tol:
            break
        J = DevJacobian(jac_map, ks, x0, time0, xoff, (s, 0.0), eps_jacobi=eps_jacobi,
                        order=order, base_in_batch=base_in_batch,
                        g0=(G if (order == 1 and not base_in_batch and jac_map is res_map)
                            else None))
        A = ShiftSystem(J, G)
        ks.scale(F, -1.0, rows_n)  # b = [-F; 0]
        start = list(range(U, U + nU)) if nU else None
        xcol, rh, KB = gmres_dev(ks, A, F, k, block=block, tol=gmres_tol, rows=N, seed=it,
                                 start=start)
        ks.scale(F, -1.0, rows_n)
        if U is not None:
            nU = ritz_directions(KB, min(recycle, block - 1), U, N)
        stats["gmres_iterations"] += len(rh) - 1
        stats["products"] += J.products
        if J._g0 is not None and J._g0 != G:
            ks.release(J._g0)
        A.release()
        stats["newton"] += 1
        if delta is None:
            ds = float(ks.get(xcol, n, 1)[0])
            ks.combine(x0, [x0, xcol], [1.0, 1.0], rows_n)
            s += ds
            hist.append(residual(x0, s))
        else:
            fn0 = hist[-1]
            accepted = False
            for _trial in range(20):
                y, _, _ = hookstep_coeffs(KB.H, KB.rhs, delta)
                KB.combine_into(xcol, y, N)
                ds = float(ks.get(xcol, n, 1)[0])
                ks.combine(xt, [x0, xcol], [1.0, 1.0], rows_n)
                stats["hook_trials"] += 1
                r = residual(xt, s + ds)
                if r < fn0:
                    ks.copy(x0, xt, rows_n)
                    s += ds
                    delta *= 2.0
                    accepted = True
                    hist.append(r)
                    break
                delta *= 0.5
            if not accepted:
                hist.append(residual(x0, s))
        ks.release(xcol)
        ks.release(KB.c0, (k + 1) * block)
        if log:
            log(f"newton {it + 1}: |F|/|x| = {hist[-1]:.3e} after {len(rh) - 1} GMRES "
                f"iterations (residual {rh[-1] / max(rh[0], 1e-300):.1e})")
    ks.release(G)
    ks.release(F)
    ks.release(xt)
    if U is not None:
        ks.release(U, recycle)
    return s, hist, stats
