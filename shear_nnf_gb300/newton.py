"""Newton-Krylov and Arnoldi tools over batched period maps of the shearing box.

Host side of the reference's periodic-orbit search and Floquet analysis, whose
cost is the Jacobian-vector product: each product is one integration of the
box over the period T (matvec_dns_disk3d, gmres_shear.f90:2666-2948, through
calc_dns_disk3d, 2951-3120).  Here every Krylov block of products is one
batched integration on the GPU: the base state and all its perturbations are
members of one ShearBox batch, advanced together by the graph-captured RK3
step.  The vectors are packed as the reference's `throwing`
(gmres_shear.f90:2229-2426, iuse_fou_mode=2); inner products, Gram-Schmidt and
the small Hessenberg problems are FP64 on the host (numpy), a few hundred
kilobytes per vector.

Pieces:
  Packing       state <-> unknown vector (throwing / backthrowing)
  PeriodMap     x -> Phi_T(x) for a batch of states (calc_dns_disk3d)
  Jacobian      forward-difference Jv with the Dennis-Schnabel step
                (matvec_dns_disk3d, iopt_matvec=1, iuse_hej=1), optional x/z
                phase shift (phase_shift_fou, operators.f90:488-544)
  arnoldi       (block) Arnoldi with modified Gram-Schmidt (arnoldi_shear.f90:
                222-330) -> Floquet multipliers and exponents log(lambda)/T
                (arnoldi_shear.f90:371-406)
  gmres         (block) GMRES for J dx = r (gmres_k_shear, gmres_shear.f90:
                1905-2207), least squares on the block Hessenberg
  Residual      F(x) = shift(Phi_T(x)) - x (- rhs) from an FP64 period map
  newton        Newton iteration for shift(Phi_T(x)) - x = 0 at fixed T and
                shifts (newton_shear.f90:183-597)
  hookstep      trust-region step in the Krylov space (gmres_shear.f90:4064-4419)
  ShiftJacobian, newton_shift
                the streamwise shift as an unknown with its phase condition,
                Newton or Newton-hookstep
  re_derivative, ReJacobian, newton_arclength
                pseudo-arclength continuation in the Reynolds number
                (iarclength=1, cpara='Rez': set_arclength, set_dxda and the
                extra row of matvec_dns_disk3d, gmres_shear.f90:1018-1147,
                3169-3316, 2936-2942); the re-perturbed integrations are
                members of the same batch with their own Re
  BorderedJacobian, period_derivative, flow_direction, newton_extended
                any set of extra unknowns with their conditions: streamwise
                and spanwise shifts and the period (isol_mode 4-6), the
                period's column dG/dT and the phase row f(x0) from members
                with their own end times
"""
from __future__ import annotations

import numpy as np

from collections import OrderedDict

from . import SB_FP64, SbParams, ShearBox, sizes


class Packing:
    """Unknown vector of a state, in the order of `throwing` with
    iuse_fou_mode=2: u00/sca_u (my), w00/sca_u (my), then for every y plane j,
    kz index k and real index q over kx (re, im interleaved): omega_y/sca_g and
    phi/sca_p of that entry, skipping the (0,0) mode and the kx=0 entries with
    negative kz (the conjugates of the positive ones; gmres_shear.f90:2356-2362).
    The second field is phi = lap(v) where the reference throws v (iuse_v=1,
    gmres_shear.f90:51): the two differ by a fixed invertible operator per
    mode, so the roots of F and the Floquet multipliers are the same.
    reference_scales() gives the scalings of gmres_shear.f90:411-413."""

    def __init__(self, p, sca_u=1.0, sca_g=1.0, sca_p=1.0):
        sz = sizes(p)
        self.my, self.nkx, self.mz, self.nz = p.my, sz["nkx"], sz["mz"], sz["nz"]
        self.sca = (sca_u, sca_g, sca_p)
        mask = np.ones((self.mz, 2 * self.nkx), bool)
        mask[0, 0:2] = False
        mask[self.nz + 1:, 0:2] = False
        self.mask = mask
        self.nsel = int(mask.sum())
        self.n = 2 * self.my + self.my * self.nsel * 2

    @staticmethod
    def reference_scales(p) -> tuple:
        lz = 2 * np.pi / p.gam
        return (p.s * lz, p.s, p.s * lz)

    def _plane_real(self, f):
        # pencil complex (mz, nkx, my) -> plane real (my, mz, 2 nkx)
        return np.ascontiguousarray(np.transpose(f, (2, 0, 1))).view(np.float64)

    def pack(self, st: dict) -> np.ndarray:
        su, sg, sp = self.sca
        V = self._plane_real(st["vor"])[:, self.mask] / sg
        P = self._plane_real(st["phi"])[:, self.mask] / sp
        body = np.stack([V, P], axis=-1).reshape(-1)
        return np.concatenate([st["u00"] / su, st["w00"] / su, body])

    def unpack(self, x: np.ndarray, time=0.0, xoffb=0.0, xofft=0.0) -> dict:
        su, sg, sp = self.sca
        my, nkx, mz, nz = self.my, self.nkx, self.mz, self.nz
        u00 = x[:my] * su
        w00 = x[my:2 * my] * su
        body = x[2 * my:].reshape(my, self.nsel, 2)
        fields = []
        for c, sca in ((0, sg), (1, sp)):
            pl = np.zeros((my, mz, 2 * nkx))
            pl[:, self.mask] = body[:, :, c] * sca
            cp = pl.view(np.complex128)  # (my, mz, nkx)
            for k in range(nz + 1, mz):  # conjugate symmetry of kx = 0
                cp[:, k, 0] = np.conj(cp[:, mz - k, 0])
            fields.append(np.ascontiguousarray(np.transpose(cp, (1, 2, 0))))
        return {"vor": fields[0], "phi": fields[1], "u00": u00.copy(), "w00": w00.copy(),
                "time": time, "xoffb": xoffb, "xofft": xofft}


def phase_shift(st: dict, p, shiftx: float, shiftz: float) -> dict:
    """phase_shift_fou (operators.f90:488-544): multiply each (kx, kz) mode by
    exp(-i kx shiftx) exp(-i kz shiftz)."""
    if shiftx == 0.0 and shiftz == 0.0:
        return st
    sz = sizes(p)
    nkx, mz, nz = sz["nkx"], sz["mz"], sz["nz"]
    kx = p.alp * np.arange(nkx)
    kz = p.gam * np.array([k if k <= nz else k - mz for k in range(mz)], float)
    f = np.exp(-1j * kx[None, :] * shiftx) * np.exp(-1j * kz[:, None] * shiftz)
    out = dict(st)
    out["vor"] = st["vor"] * f[:, :, None]
    out["phi"] = st["phi"] * f[:, :, None]
    return out


class PeriodMap:
    """x -> Phi_T(x): states integrated from their own time to time + T, all
    members of one batch advanced together (calc_dns_disk3d).  Each member
    stops on its own end time (the clipped last step of cross.f90:1694-1711);
    the batch is stepped in chunks until every member has reached it."""

    def __init__(self, p, T: float, batch: int, precision: int = SB_FP64, chunk: int = 64,
                 autotune: bool = False):
        self.p, self.T, self.batch, self.chunk = p, float(T), int(batch), int(chunk)
        self.autotune, self.tuning = autotune, None
        self.box = ShearBox(p, batch=self.batch, precision=precision)
        self.integrations = 0
        self.steps = 0  # RK3 steps summed over the integrated states
        self.last_steps = []

    def __call__(self, states: list, res: list = None, Ts: list = None) -> list:
        """Integrates the states over T; res gives each state's Reynolds
        number (1/nu), default the parameters' Re, and Ts each state's
        integration time, default T."""
        assert 1 <= len(states) <= self.batch
        box = self.box
        full = list(states) + [states[0]] * (self.batch - len(states))
        for m, st in enumerate(full):
            box.set_state(st, m)
            T = Ts[m] if Ts is not None and m < len(Ts) else self.T
            box.set_etime(m, st["time"] + T)
            box.set_re(m, res[m] if res is not None and m < len(res) else self.p.Re)
        if self.autotune and not self.tuning:
            # tiles for this batch, timed on its first states (left as set)
            self.tuning = box.autotune()
        steps = [0] * len(states)
        fin = [False] * len(states)
        for _ in range(1 << 20):
            # a member already at its end time takes zero-length steps
            box.step(self.chunk)
            for m in range(len(states)):
                if fin[m]:
                    continue
                s = box.status(m)
                if s.flags & 3 or (s.flags & 4 and not self.p.keep_laminar):
                    raise RuntimeError(f"period map: member {m} stopped (flags {s.flags})")
                steps[m] += s.steps_done
                fin[m] = bool(s.flags & 8)
            if all(fin):
                break
        self.last_steps = steps
        self.steps += sum(steps)
        self.integrations += len(states)
        return [box.get_state(m) for m in range(len(states))]


class Jacobian:
    """Finite-difference products J d of the shifted period map
    G(x) = pack(shift(Phi_T(unpack(x)))) at x0 (matvec_dns_disk3d,
    gmres_shear.f90:2666-2948): eps = eps_jacobi |x0| / |d| (gmres_shear.f90:1380,
    2699), the representable step h = (x0 + eps d) - x0 (iuse_hej=1),
    J d = (G(x0 + h) - G(x0)) / eps, or (G(x0 + h) - G(x0 - h)) / (2 eps) with
    central=True or order=2 (iopt_matvec=2), or with order=4 (iopt_matvec=4)
    (8 (G(x0 + h) - G(x0 - h)) - (G(x0 + 2h) - G(x0 - 2h))) / (12 eps).
    Products are evaluated a block at a time: one batched integration per
    block of PeriodMap.batch states.  re sets the Reynolds number of the map
    (default the parameters').

    base_in_batch=True integrates x0 again as the first member of every block
    and differences against that copy, so that the base and the perturbed
    states see the same arithmetic (FP32-mixed boxes)."""

    def __init__(self, pmap: PeriodMap, packing: Packing, x0: np.ndarray, time0=0.0,
                 xoff0=(0.0, 0.0), shiftx=0.0, shiftz=0.0, eps_jacobi=1e-6, central=False,
                 base_in_batch=False, order=None, re=None):
        self.pmap, self.pk, self.x0 = pmap, packing, np.asarray(x0, float)
        self.time0, self.xoff0, self.shift = time0, tuple(xoff0), (shiftx, shiftz)
        self.order = int(order) if order is not None else (2 if central else 1)
        if self.order not in (1, 2, 4):
            raise ValueError("order must be 1, 2 or 4")
        self.central = self.order > 1
        self.eps_jacobi, self.base_in_batch = eps_jacobi, base_in_batch
        self.re = re
        self.products = 0
        self._gx0 = None

    @property
    def gx0(self):
        """G(x0), integrated on first use (the forward-difference base; None
        when the base is integrated in every block)."""
        if self._gx0 is None and not self.base_in_batch:
            self._gx0 = self.G([self.x0])[0]
        return self._gx0

    def G(self, xs: list, res: list = None) -> list:
        """Shifted period maps of the vectors xs (at Reynolds numbers res, by
        default the Jacobian's)."""
        states = [self.pk.unpack(x, self.time0, *self.xoff0) for x in xs]
        if res is None and self.re is not None:
            res = [self.re] * len(xs)
        out = []
        for q in range(0, len(states), self.pmap.batch):
            chunk = states[q:q + self.pmap.batch]
            out += (self.pmap(chunk) if res is None else
                    self.pmap(chunk, res[q:q + self.pmap.batch]))
        return [self.pk.pack(phase_shift(s, self.pmap.p, *self.shift)) for s in out]

    @property
    def block(self) -> int:
        """Products per batched integration."""
        per = {1: 1, 2: 2, 4: 4}[self.order]
        return (self.pmap.batch - (1 if self.base_in_batch else 0)) // per

    def matvec(self, D: np.ndarray) -> np.ndarray:
        D = np.asarray(D, float)
        D = D[:, None] if D.ndim == 1 else D
        nb = self.block
        if nb < 1:
            raise ValueError("matvec: batch too small for one product")
        out = np.zeros_like(D)
        nz = [q for q in range(D.shape[1]) if np.any(D[:, q])]  # J 0 = 0 without integrating
        for q in range(0, len(nz), nb):
            cols = nz[q:q + nb]
            out[:, cols] = self._matvec_block(D[:, cols])
        return out

    def _matvec_block(self, D: np.ndarray) -> np.ndarray:
        xn = np.linalg.norm(self.x0)
        eps_j = self.eps_jacobi * (xn if xn > 0 else 1.0)
        xs, eps = ([self.x0] if self.base_in_batch else []), []
        steps = {1: (1,), 2: (1, -1), 4: (1, -1, 2, -2)}[self.order]
        for q in range(D.shape[1]):
            e = eps_j / np.linalg.norm(D[:, q])
            for f in steps:
                xs.append(self.x0 + ((self.x0 + (f * e) * D[:, q]) - self.x0))
            eps.append(e)
        gs = self.G(xs)
        if self.base_in_batch:
            g0, gs = gs[0], gs[1:]
        self.products += D.shape[1]
        ns = len(steps)
        if self.order == 1:
            if not self.base_in_batch:
                g0 = self.gx0
            cols = [(gs[q] - g0) / eps[q] for q in range(D.shape[1])]
        elif self.order == 2:
            cols = [(gs[2 * q] - gs[2 * q + 1]) / (2 * eps[q]) for q in range(D.shape[1])]
        else:
            cols = [(8.0 * (gs[ns * q] - gs[ns * q + 1]) - (gs[ns * q + 2] - gs[ns * q + 3])) /
                    (12 * eps[q]) for q in range(D.shape[1])]
        return np.stack(cols, axis=1)


class Residual:
    """F(x) = shift(Phi_T(x)) - x - rhs with an FP64 period map (the Newton
    residual of newton_shear.f90:183-300; rhs = 0 there, a manufactured target
    otherwise)."""

    def __init__(self, pmap: PeriodMap, packing: Packing, time0=0.0, xoff0=(0.0, 0.0),
                 shiftx=0.0, shiftz=0.0, rhs=None):
        self.pmap, self.pk = pmap, packing
        self.time0, self.xoff0, self.shift, self.rhs = time0, tuple(xoff0), (shiftx, shiftz), rhs

    def G(self, x: np.ndarray) -> np.ndarray:
        st = self.pmap([self.pk.unpack(x, self.time0, *self.xoff0)])[0]
        return self.pk.pack(phase_shift(st, self.pmap.p, *self.shift))

    def __call__(self, x: np.ndarray) -> np.ndarray:
        F = self.G(x) - x
        return F if self.rhs is None else F - self.rhs


class ShiftResidual:
    """(F, G) at (x, s): G = shift_s(Phi_T(x)) from an FP64 period map and
    F = G - x (- rhs), for newton_shift."""

    def __init__(self, pmap: PeriodMap, packing: Packing, time0=0.0, xoff0=(0.0, 0.0), rhs=None):
        self.pmap, self.pk, self.time0, self.xoff0, self.rhs = pmap, packing, time0, tuple(xoff0), rhs

    def __call__(self, x: np.ndarray, s: float):
        st = self.pmap([self.pk.unpack(x, self.time0, *self.xoff0)])[0]
        G = self.pk.pack(phase_shift(st, self.pmap.p, s, 0.0))
        F = G - x
        return (F if self.rhs is None else F - self.rhs), G


def _orthonormalize(W: np.ndarray, V: list, Hcol: list):
    """Modified Gram-Schmidt of the block W against the blocks of V (twice, for
    robustness), then a QR of the remainder; returns (Q, R) and appends the
    projections to Hcol."""
    for _ in range(2):
        for i, Vi in enumerate(V):
            c = Vi.T @ W
            W = W - Vi @ c
            if len(Hcol) <= i:
                Hcol.append(c)
            else:
                Hcol[i] = Hcol[i] + c
    return np.linalg.qr(W)


def arnoldi(matvec, n: int, k: int, block: int = 1, seed: int = 0, start=None):
    """Block Arnoldi: k iterations of blocks of `block` products.  Returns the
    Ritz values (largest modulus first), their residual estimates
    |H_{k+1,k} y_k| (unit Ritz vectors y), the block Hessenberg matrix and the
    basis.  block=1 is the reference's Arnoldi with modified Gram-Schmidt
    (arnoldi_shear.f90:222-330)."""
    rng = np.random.default_rng(seed)
    Q0 = rng.standard_normal((n, block)) if start is None else np.asarray(start, float).reshape(n, -1)
    Q, _ = np.linalg.qr(Q0)
    V = [Q]
    p = Q.shape[1]
    H = np.zeros(((k + 1) * p, k * p))
    for it in range(k):
        W = matvec(V[-1])
        cols = []
        Qn, R = _orthonormalize(W, V, cols)
        for i, c in enumerate(cols):
            H[i * p:(i + 1) * p, it * p:(it + 1) * p] = c
        H[(it + 1) * p:(it + 2) * p, it * p:(it + 1) * p] = R
        V.append(Qn)
    Hk = H[: k * p, : k * p]
    lam, Y = np.linalg.eig(Hk)
    Y = Y / np.linalg.norm(Y, axis=0)
    res = np.linalg.norm(H[k * p:, (k - 1) * p:k * p] @ Y[(k - 1) * p:, :], axis=0)
    order = np.argsort(-np.abs(lam))
    return lam[order], res[order], H, V


def floquet_exponents(lam: np.ndarray, T: float) -> np.ndarray:
    """sigma = log(lambda) / T (arnoldi_shear.f90:403-406)."""
    return np.log(lam.astype(complex)) / T


def gmres(matvec, b: np.ndarray, k: int, block: int = 1, tol: float = 0.0, seed: int = 0,
          krylov: bool = False):
    """(Block) GMRES for J x = b from x = 0: the first basis vector is b/|b|;
    with block > 1 the other columns of the starting block are random, so every
    iteration applies J to `block` vectors in one batched integration and the
    solution is minimised over a larger space.  Returns (x, residual norms), and
    with krylov=True also (V, H, rhs): the basis, the block Hessenberg matrix
    and the projected right-hand side of the last iteration, for hookstep."""
    n = b.size
    beta = np.linalg.norm(b)
    if beta == 0:
        return np.zeros(n), [0.0]
    rng = np.random.default_rng(seed)
    Q0 = np.concatenate([b[:, None], rng.standard_normal((n, block - 1))], axis=1)
    Q, R0 = np.linalg.qr(Q0)
    V = [Q]
    p = Q.shape[1]
    H = np.zeros(((k + 1) * p, k * p))
    rhs0 = np.zeros((k + 1) * p)
    rhs0[:p] = R0[:, 0]
    res = [beta]
    x = np.zeros(n)
    for it in range(k):
        W = matvec(V[-1])
        cols = []
        Qn, R = _orthonormalize(W, V, cols)
        for i, c in enumerate(cols):
            H[i * p:(i + 1) * p, it * p:(it + 1) * p] = c
        H[(it + 1) * p:(it + 2) * p, it * p:(it + 1) * p] = R
        V.append(Qn)
        m = (it + 1) * p
        Hm = H[: m + p, :m]
        y, *_ = np.linalg.lstsq(Hm, rhs0[: m + p], rcond=None)
        r = np.linalg.norm(rhs0[: m + p] - Hm @ y)
        res.append(r)
        Vm = np.concatenate(V[: it + 1], axis=1)
        x = Vm @ y
        if r <= tol * beta:
            break
    if krylov:
        return x, res, (Vm, Hm, rhs0[: Hm.shape[0]])
    return x, res


def hookstep(V: np.ndarray, H: np.ndarray, rhs: np.ndarray, delta: float, sv_cut: float = 0.0,
             iters: int = 200):
    """Trust-region step in the Krylov space (hookstep, gmres_shear.f90:4200-4419,
    with the mu iteration of solv_mu, 4064-4198): minimise |H y - rhs| subject
    to |y| <= delta through the SVD H = U S W^T: q_i = s_i p_i / (s_i^2 + mu),
    p = U^T rhs, with mu >= 0 chosen so that |q| = delta (mu = 0 when the
    unconstrained step is shorter); singular values with s^2 <= sv_cut are
    dropped.  Returns (dx = V W q, mu, predicted residual |H y - rhs|)."""
    U, s, Wt = np.linalg.svd(H, full_matrices=True)
    m = s.size
    p = U.T @ rhs
    keep = s * s > sv_cut

    def q_of(mu):
        q = np.zeros(m)
        q[keep] = s[keep] * p[:m][keep] / (s[keep] ** 2 + mu)
        return q

    mu = 0.0
    q = q_of(0.0)
    if np.linalg.norm(q) > delta:
        mu = 1e-3
        for _ in range(iters):
            q = q_of(mu)
            qn = np.linalg.norm(q)
            ph = qn * qn - delta * delta
            phprim = -2.0 * np.sum(q[keep] ** 2 / (s[keep] ** 2 + mu))
            step = (qn / delta) * (ph / phprim)
            mu = max(mu - step, 0.0)
            if abs(ph) <= 1e-12 * delta * delta:
                break
        q = q_of(mu)
    y = Wt.T @ q
    return V @ y, mu, float(np.linalg.norm(H @ y - rhs))


def shift_tangent(packing: Packing, p, x: np.ndarray, which: str = "x") -> np.ndarray:
    """d/ds of shift_s(x) at s = 0: -i kx x (or -i kz x), packed."""
    st = packing.unpack(x)
    sz = sizes(p)
    if which == "x":
        fac = -1j * (p.alp * np.arange(sz["nkx"]))[None, :, None]
    else:
        mz, nz = sz["mz"], sz["nz"]
        kz = p.gam * np.array([k if k <= nz else k - mz for k in range(mz)], float)
        fac = -1j * kz[:, None, None]
    out = dict(st)
    out["vor"] = st["vor"] * fac
    out["phi"] = st["phi"] * fac
    out["u00"] = np.zeros_like(st["u00"])
    out["w00"] = np.zeros_like(st["w00"])
    return packing.pack(out)


class ShiftJacobian:
    """Jacobian of the relative-periodic-orbit system with the streamwise shift
    as unknown (the unknowns of newton_shear.f90 with the shift, its phase
    condition orthogonal to the shift direction): for X = (x, s),
        F(x, s) = shift_s(Phi_T(x)) - x - rhs,   <t(x0), dx> = 0,
    products [(J - I) dx + dG/ds ds ; <t, dx>] with J the shifted period map's
    Jacobian at (x0, s0) (a Jacobian built with shiftx = s0), dG/ds = -i kx G(x0)
    and t = -i kx x0 normalised."""

    def __init__(self, J, packing: Packing, p, x0: np.ndarray, gx0: np.ndarray):
        self.J, self.pk, self.p = J, packing, p
        self.dgds = shift_tangent(packing, p, gx0)
        t = shift_tangent(packing, p, x0)
        self.t = t / max(np.linalg.norm(t), 1e-300)
        self.n = x0.size

    def matvec(self, D: np.ndarray) -> np.ndarray:
        D = np.asarray(D, float)
        D = D[:, None] if D.ndim == 1 else D
        dx, ds = D[: self.n], D[self.n]
        out = np.empty_like(D)
        out[: self.n] = self.J.matvec(dx) - dx + self.dgds[:, None] * ds[None, :]
        out[self.n] = self.t @ dx
        return out


def newton_shift(x0: np.ndarray, s0: float, residual_at, jac_at, k: int = 20, block: int = 1,
                 itmax: int = 10, tol: float = 1e-10, gmres_tol: float = 1e-3, delta: float = None):
    """Newton(-hookstep) search for a relative periodic orbit with unknown
    streamwise shift s: residual_at(x, s) returns (F, G) with G the shifted
    period map of x (FP64) and F = G - x (- rhs); jac_at(x, s, G) returns a
    ShiftJacobian.  With delta set, every step is a hookstep of at most delta
    in the Krylov space, delta halved when the residual grows (the step is
    then retaken without new products) and doubled after a good step
    (newton_shear.f90:446-490 restores the previous iterate the same way).
    Returns (x, s, history of |F|/|x|)."""
    x, s = np.asarray(x0, float).copy(), float(s0)
    F, G = residual_at(x, s)
    hist = [np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300)]
    n = x.size
    for _ in range(itmax):
        if hist[-1] <= tol:
            break
        Jx = jac_at(x, s, G)
        b = np.concatenate([-F, [0.0]])
        sol, _, (V, H, rhs) = gmres(Jx.matvec, b, k, block=block, tol=gmres_tol, krylov=True)
        if delta is None:
            X = np.concatenate([x, [s]]) + sol
            x, s = X[:n], X[n]
            F, G = residual_at(x, s)
            hist.append(np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300))
            continue
        fn0 = np.linalg.norm(F)
        for _trial in range(20):
            dX, _, _ = hookstep(V, H, rhs, delta)
            Xn = np.concatenate([x, [s]]) + dX
            Fn, Gn = residual_at(Xn[:n], Xn[n])
            if np.linalg.norm(Fn) < fn0:
                x, s, F, G = Xn[:n], Xn[n], Fn, Gn
                delta *= 2.0
                break
            delta *= 0.5
        hist.append(np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300))
    return x, s, hist


def newton(x0: np.ndarray, residual, jac_factory, k: int = 20, block: int = 1, itmax: int = 10,
           tol: float = 1e-10, gmres_tol: float = 1e-3):
    """Newton iteration for F(x) = 0 with F(x) = G(x) - x (- b): residual(x)
    returns F(x) (FP64 integration); jac_factory(x) returns a Jacobian of G at x,
    whose products may come from FP32-mixed integrations: each step solves
    (J - I) dx = -F with GMRES to gmres_tol and the FP64 residual of the next
    iterate corrects what the approximate Jacobian missed (iterative
    refinement).  Returns (x, history of |F|/|x|)."""
    x = np.asarray(x0, float).copy()
    hist = []
    for _ in range(itmax + 1):
        F = residual(x)
        rel = np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300)
        hist.append(rel)
        if rel <= tol or len(hist) > itmax:
            break
        J = jac_factory(x)
        dx, _ = gmres(lambda D: J.matvec(D) - D, -F, k, block=block, tol=gmres_tol)
        x = x + dx
    return x, hist


def re_derivative(J: Jacobian, re: float, daa: float = 1e-6, central: bool = True,
                  gx0: np.ndarray = None) -> np.ndarray:
    """dG/dre at J.x0 by finite differences in the Reynolds number (1/nu) with
    the absolute step daa (set_dxda, gmres_shear.f90:3169-3316: forward with
    iopt_matvec=1, else centred); the perturbed integrations run as members of
    one batch with their own Re."""
    if central:
        gp, gm = J.G([J.x0, J.x0], [re + daa, re - daa])
        return (gp - gm) / (2.0 * daa)
    if gx0 is None:
        gx0 = J.G([J.x0], [re])[0]
    return (J.G([J.x0], [re + daa])[0] - gx0) / daa


class ReJacobian:
    """Jacobian of the pseudo-arclength system in the Reynolds number
    (iarclength=1, cpara='Rez'): for X = (x, re),
        F(x, re) = G(x; re) - x - rhs,   <xstan, dx> = 0,
    products [(J - I) dx + dG/dre dre ; <xstan, dx>] (matvec_dns_disk3d,
    gmres_shear.f90:2936-2942: the parameter column dxda and the row
    orthogonal to the secant xstan = x0 - xm1; sca_re = 1)."""

    def __init__(self, J, dgdre: np.ndarray, xstan: np.ndarray):
        self.J, self.dgdre, self.xstan = J, np.asarray(dgdre, float), np.asarray(xstan, float)
        self.n = self.xstan.size

    def matvec(self, D: np.ndarray) -> np.ndarray:
        D = np.asarray(D, float)
        D = D[:, None] if D.ndim == 1 else D
        dx, dre = D[: self.n], D[self.n]
        out = np.empty_like(D)
        out[: self.n] = self.J.matvec(dx) - dx + self.dgdre[:, None] * dre[None, :]
        out[self.n] = self.xstan @ dx
        return out


def arclength_predictor(xm1: np.ndarray, rem1: float, x0: np.ndarray, re0: float,
                        arcl: float):
    """set_arclength (gmres_shear.f90:1018-1147) for cpara='Rez': the secant
    xstan = x0 - xm1, ptan = re0 - rem1 and the predicted point
    (x0 + arcl xstan, re0 + arcl ptan).  Returns (x, re, xstan)."""
    xstan = np.asarray(x0, float) - np.asarray(xm1, float)
    ptan = float(re0) - float(rem1)
    if np.linalg.norm(xstan) <= 0.0 or ptan == 0.0:
        raise ValueError("arclength: the two points give no tangent")
    if not arcl > 0.0:
        raise ValueError("arclength: arcl must be positive")
    return np.asarray(x0, float) + arcl * xstan, float(re0) + arcl * ptan, xstan


def newton_arclength(xm1: np.ndarray, rem1: float, x0: np.ndarray, re0: float, arcl: float,
                     residual_at, jac_at, k: int = 20, block: int = 1, itmax: int = 10,
                     tol: float = 1e-10, gmres_tol: float = 1e-3):
    """One pseudo-arclength step along the Reynolds number from the solutions
    (xm1, rem1) and (x0, re0): the predictor of arclength_predictor, then
    Newton corrections (dx, dre) solving [(J - I) dx + dG/dre dre = -F,
    <xstan, dx> = 0] (the right-hand side of the extra row is zero,
    gmres_shear.f90:1283-1285).  residual_at(x, re) returns (F, G) with
    F = G(x; re) - x (- rhs) in FP64; jac_at(x, re, G, xstan) returns a
    ReJacobian.  Returns (x, re, history of |F|/|x|)."""
    x, re, xstan = arclength_predictor(xm1, rem1, x0, re0, arcl)
    F, G = residual_at(x, re)
    hist = [np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300)]
    n = x.size
    for _ in range(itmax):
        if hist[-1] <= tol:
            break
        Jx = jac_at(x, re, G, xstan)
        sol, _ = gmres(Jx.matvec, np.concatenate([-F, [0.0]]), k, block=block, tol=gmres_tol)
        x, re = x + sol[:n], re + sol[n]
        F, G = residual_at(x, re)
        hist.append(np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300))
    return x, re, hist


# pseudo-arclength parameters (cpara, gmres_shear.f90:115-160,922-975) and the
# parameter field each one sets
CPARA_FIELDS = {"Rez": "Re", "Ayz": "Ly", "Axz": "alp", "LES_Cs": "cs", "damp_up": "damp_up",
                "damp_aa": "damp_aa"}


class ParamFamily:
    """Shifted period maps G(x; a) along one pseudo-arclength parameter a
    (cpara): 'Rez' the Reynolds number 1/nu, 'Ayz' Ly, 'Axz' alp, 'LES_Cs' the
    Smagorinsky constant, 'damp_up'/'damp_aa' the window damping's permeability
    and half width.  A value of a geometric, LES or damping parameter gets its own
    handle (the compact-scheme tables, wavenumbers, CFL constants and LES
    filter width follow from it; the last few are kept); 'Rez' integrates all
    values as members of one batch with their own Re.  With timep (shear
    periods per orbit) the period follows 2 pi / (alp Ly s) timep, as set_dxda
    recomputes it for Ayz and Axz (gmres_shear.f90:3204-3221), else T is
    fixed; for Axz the image offsets keep alp xofft (xofft = xofft0 alp0 / alp,
    xoffb = -xofft; gmres_shear.f90:3211-3220).  derivative() is dG/da by
    finite differences with the steps of set_dxda (gmres_shear.f90:3169-3316):
    daa = 1e-6, a tenth of it for LES_Cs, centred unless forward.
    residual(x, a) returns (F, G) with F = G - x (- rhs) and jacobian(x, a, G,
    xstan) the bordered operator, the two callables of newton_arclength."""

    def __init__(self, p, cpara: str, packing: Packing, batch: int = 2,
                 precision: int = SB_FP64, T: float = None, timep: float = None, time0=0.0,
                 xoff0=(0.0, 0.0), shiftx=0.0, shiftz=0.0, rhs=None, chunk: int = 64,
                 eps_jacobi: float = 1e-6, order: int = 2, keep: int = 3):
        if cpara not in CPARA_FIELDS:
            raise ValueError(f"cpara {cpara!r}: one of {sorted(CPARA_FIELDS)}")
        if (T is None) == (timep is None):
            raise ValueError("give the period T or the shear periods timep")
        if cpara == "LES_Cs" and not p.les:
            raise ValueError("cpara LES_Cs needs an LES handle (les = 1)")
        if cpara.startswith("damp_") and not p.damping:
            raise ValueError(f"cpara {cpara} needs the window damping (damping = 1)")
        self.p0 = SbParams.from_buffer_copy(p)
        self.cpara, self.field = cpara, CPARA_FIELDS[cpara]
        self.pk, self.batch, self.precision, self.chunk = packing, int(batch), precision, chunk
        self.T, self.timep = T, timep
        self.time0, self.xoff0, self.shift, self.rhs = time0, tuple(xoff0), (shiftx, shiftz), rhs
        # a Jacobian at a uses the map of a while the derivative adds a +- daa
        self.eps_jacobi, self.order, self.keep = eps_jacobi, order, max(int(keep), 3)
        self._maps = OrderedDict()

    @property
    def a0(self) -> float:
        return float(getattr(self.p0, self.field))

    def params(self, a: float) -> SbParams:
        q = SbParams.from_buffer_copy(self.p0)
        setattr(q, self.field, float(a))
        return q

    def period(self, a: float) -> float:
        if self.timep is None:
            return float(self.T)
        q = self.params(a)
        return 2.0 * np.pi / (q.alp * q.Ly * q.s) * self.timep

    def xoff(self, a: float) -> tuple:
        xb, xt = self.xoff0
        if self.cpara == "Axz":
            xt = xt * self.a0 / float(a)
            xb = -xt
        return xb, xt

    def _key(self, a: float) -> float:
        return self.a0 if self.cpara == "Rez" else float(a)

    def pmap(self, a: float) -> PeriodMap:
        """The period map of parameter value a (one handle per value, the last
        `keep` values kept)."""
        key = self._key(a)
        if key in self._maps:
            self._maps.move_to_end(key)
            return self._maps[key]
        m = PeriodMap(self.params(key), self.period(a), self.batch, self.precision, self.chunk)
        self._maps[key] = m
        while len(self._maps) > self.keep:
            _, old = self._maps.popitem(last=False)
            old.box.close()
        return m

    def G(self, xs: list, avals: list) -> list:
        """Shifted period maps of the vectors xs at the parameter values avals."""
        out = [None] * len(xs)
        groups = OrderedDict()
        for q, a in enumerate(avals):
            groups.setdefault(self._key(a), []).append(q)
        for idx in groups.values():
            a = avals[idx[0]]
            m = self.pmap(a)
            xb, xt = self.xoff(a)
            for c in range(0, len(idx), m.batch):
                part = idx[c:c + m.batch]
                sts = [self.pk.unpack(xs[q], self.time0, xb, xt) for q in part]
                if self.cpara == "Rez":
                    gs = m(sts, [float(avals[q]) for q in part])
                else:
                    gs = m(sts)
                for q, g in zip(part, gs):
                    out[q] = self.pk.pack(phase_shift(g, m.p, *self.shift))
        return out

    def derivative(self, x: np.ndarray, a: float, daa: float = 1e-6, central: bool = True,
                   gx: np.ndarray = None) -> np.ndarray:
        """dG/da at (x, a) (set_dxda)."""
        if self.cpara == "LES_Cs":
            daa = daa / 10.0
        if central:
            gp, gm = self.G([x, x], [a + daa, a - daa])
            return (gp - gm) / (2.0 * daa)
        if gx is None:
            gx = self.G([x], [a])[0]
        return (self.G([x], [a + daa])[0] - gx) / daa

    def residual(self, x: np.ndarray, a: float):
        G = self.G([x], [a])[0]
        F = G - x
        return (F if self.rhs is None else F - self.rhs), G

    def jacobian(self, x: np.ndarray, a: float, G: np.ndarray, xstan: np.ndarray) -> "ReJacobian":
        """[(J - I) dx + dG/da da ; <xstan, dx>] at (x, a): J from the map of
        value a (finite differences of order `order`), dG/da from derivative()
        with the forward base G."""
        m = self.pmap(a)
        xb, xt = self.xoff(a)
        J = Jacobian(m, self.pk, x, self.time0, (xb, xt), *self.shift,
                     eps_jacobi=self.eps_jacobi, order=self.order,
                     re=float(a) if self.cpara == "Rez" else None)
        J._gx0 = G if self.order == 1 else None  # the forward-difference base
        dgda = self.derivative(x, a, central=self.order > 1, gx=G)
        return ReJacobian(J, dgda, xstan)


class BorderedJacobian:
    """Jacobian of the periodic-orbit system with extra unknowns
    (matvec_dns_disk3d, gmres_shear.f90:2900-2942): for X = (x, a_1..a_m),
        [(J - I) dx + sum_k c_k da_k ; <r_k, dx>, k = 1..m]
    with c_k = dG/da_k (shift_tangent of G for the shifts, period_derivative
    for the period, re_derivative for the Reynolds number) and r_k the k-th
    condition (the shift directions of x0 for the shifts, flow_direction of
    x0 for the period: the rows of gmres_shear.f90:2915-2934)."""

    def __init__(self, J, cols: list, rows: list):
        self.J = J
        self.cols = [np.asarray(c, float) for c in cols]
        self.rows = [np.asarray(r, float) for r in rows]
        assert len(self.cols) == len(self.rows)
        self.n = self.cols[0].size if self.cols else None

    def matvec(self, D: np.ndarray) -> np.ndarray:
        D = np.asarray(D, float)
        D = D[:, None] if D.ndim == 1 else D
        m = len(self.cols)
        n = D.shape[0] - m
        dx, da = D[:n], D[n:]
        out = np.empty_like(D)
        out[:n] = self.J.matvec(dx) - dx
        for k in range(m):
            out[:n] += self.cols[k][:, None] * da[k][None, :]
            out[n + k] = self.rows[k] @ dx
        return out


def period_derivative(J: Jacobian, T: float, h: float) -> np.ndarray:
    """dG/dT at J.x0: centred difference of the shifted map over the
    integration times T +- h, two members of one batch with their own end
    times (the dxdt column of matvec_dns_disk3d, gmres_shear.f90:2928-2931)."""
    st = J.pk.unpack(J.x0, J.time0, *J.xoff0)
    gp, gm = J.pmap([st, st], Ts=[T + h, T - h])
    gp = J.pk.pack(phase_shift(gp, J.pmap.p, *J.shift))
    gm = J.pk.pack(phase_shift(gm, J.pmap.p, *J.shift))
    return (gp - gm) / (2.0 * h)


def flow_direction(pmap: PeriodMap, packing: Packing, x: np.ndarray, h: float, time0=0.0,
                   xoff0=(0.0, 0.0)) -> np.ndarray:
    """The time derivative of the flow at x (dxdt0 of the period's phase
    condition <dxdt0, dx> = 0, gmres_shear.f90:2931), as the second-order
    one-sided difference (-3 x + 4 Phi_h(x) - Phi_2h(x)) / (2h) from two
    members with their own end times.  The reference evaluates the right-hand
    side instead (set_dxdt); any direction transverse to the flow fixes the
    phase, so the converged orbit is the same."""
    st = packing.unpack(x, time0, *xoff0)
    a, b = pmap([st, st], Ts=[h, 2.0 * h])
    return (-3.0 * x + 4.0 * packing.pack(a) - packing.pack(b)) / (2.0 * h)


def newton_extended(x0: np.ndarray, a0, residual_at, jac_at, k: int = 20, block: int = 1,
                    itmax: int = 10, tol: float = 1e-10, gmres_tol: float = 1e-3,
                    delta: float = None):
    """Newton(-hookstep) for F(x, a) = 0 with extra unknowns a (shifts,
    period; newton_shear.f90:183-597 with isol_mode 4-6): residual_at(x, a)
    returns (F, G) with G the shifted period map of x over the period in a
    (FP64) and F = G - x (- rhs); jac_at(x, a, G) returns a BorderedJacobian
    with len(a) conditions, whose right-hand sides are zero.  With delta set,
    every step is a Krylov hookstep of at most delta (delta halved on a failed
    step, doubled on a good one).  Returns (x, a, history of |F|/|x|)."""
    x, a = np.asarray(x0, float).copy(), np.atleast_1d(np.asarray(a0, float)).copy()
    m = a.size
    F, G = residual_at(x, a)
    hist = [np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300)]
    n = x.size
    for _ in range(itmax):
        if hist[-1] <= tol:
            break
        Jx = jac_at(x, a, G)
        b = np.concatenate([-F, np.zeros(m)])
        sol, _, (V, H, rhs) = gmres(Jx.matvec, b, k, block=block, tol=gmres_tol, krylov=True)
        if delta is None:
            x, a = x + sol[:n], a + sol[n:]
            F, G = residual_at(x, a)
            hist.append(np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300))
            continue
        fn0 = np.linalg.norm(F)
        for _trial in range(20):
            dX, _, _ = hookstep(V, H, rhs, delta)
            xn, an = x + dX[:n], a + dX[n:]
            Fn, Gn = residual_at(xn, an)
            if np.linalg.norm(Fn) < fn0:
                x, a, F, G = xn, an, Fn, Gn
                delta *= 2.0
                break
            delta *= 0.5
        hist.append(np.linalg.norm(F) / max(np.linalg.norm(x), 1e-300))
    return x, a, hist
