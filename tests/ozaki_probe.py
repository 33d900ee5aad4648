"""Go/no-go probe: the backward z-transform of plane stage 1 as an FP64-accurate
product on the bf16 tensor cores (an Ozaki-type split), measured against the
FP64 FFT stage it would replace.

Plane stage 1 (k_p1) transforms, per y plane, the 63 kz modes of 6 fields x 64
kx columns to 96 z points (c2r in z of fou3D_thread.f:22-55, FFTW backward
convention, unnormalised).  Written as a real matrix product,

    [Yr; Yi] (192 x N) = [[Wr, -Wi]; [Wi, Wr]] (192 x 126) . [Xr; Xi] (126 x N),
    W[n, k] = exp(+2 pi i kz(k) n / 96),  N = 6 * 64 * 96 columns per substep,

it fits the tensor cores.  The split (in the manner of Ozaki, Ogita, Oishi and
Rump's error-free splitting, here with fixed-point digits):
  - every row r of A and column c of X is scaled by a power of two so that
    its largest entry is below 1, then rounded to a 8 s-bit integer;
  - the integers are written in s balanced base-256 digits (|digit| <= 129,
    exact in bf16), A = sum_p D_p 2^(e_r - 8p), X = sum_q E_q 2^(f_c - 8q);
  - every product D_p E_q has integer entries below 126 * 129^2 < 2^21.1,
    exact in FP32 accumulation, and the products of one diagonal p + q = d
    (at most s of them) add up below 2^24, still exact;
  - the leading diagonals d <= 5 are combined exactly in int64 and converted
    once to FP64, the smaller ones added in FP64, and the result scaled: the
    roundings are the 8 s-bit quantisation of A and X and the dropped
    diagonals d > s + 1 (relative to the row and column maxima, about
    2^(-8s) each).
The GEMMs run in cuBLAS (bf16 in, FP32 out); the split and the combination run
as integer tensor operations.  This module is a measurement, not part of the
library: it is run by tests/test_gpu_ozaki.py and standalone for timing:

    python tests/ozaki_probe.py [--digits 7] [--reps 20]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys

import numpy as np

MGALZ, MZ, NZ = 96, 63, 31  # the 192x96x96 grid's z transform
COLS = 6 * 64 * 96           # fields x kx columns x y planes of one substep


def dft_block():
    """The real 192 x 126 form of the backward z-DFT of the 2/3-rule modes."""
    kz = np.array([k if k <= NZ else k - MZ for k in range(MZ)], float)
    n = np.arange(MGALZ)[:, None]
    W = np.exp(2j * np.pi * n * kz[None, :] / MGALZ)
    return np.block([[W.real, -W.imag], [W.imag, W.real]])


def split(A, digits: int, axis: int):
    """Balanced base-256 digits of A scaled per row (axis=1) or column
    (axis=0): returns (list of digit tensors, most significant first, as
    bf16; exponent tensor e with A ~ sum_p D_p 2^(e - 8p))."""
    import torch
    amax = A.abs().amax(dim=axis, keepdim=True)
    _, e = torch.frexp(torch.where(amax > 0, amax, torch.ones_like(amax)))
    e = e.to(torch.int64)
    # |A| < 2^e: an integer below 2^(8 digits - 1) in magnitude, then digits-1
    # balanced base-256 digits and the rest (at most 129) as the leading one
    m = torch.round(torch.ldexp(A, (8 * digits - 1 - e).to(A.dtype))).to(torch.int64)
    out = []
    for _ in range(digits - 1):
        d = ((m + 128) & 255) - 128
        m = (m - d) >> 8
        out.append(d)
    assert int(m.abs().max()) <= 256
    out.append(m)
    return [d.to(torch.float32).to(torch.bfloat16) for d in reversed(out)], e + 1


def mm32(a, b):
    """bf16 x bf16 -> FP32 product (cuBLAS)."""
    import torch
    return torch.mm(a, b, out_dtype=torch.float32)


def ozaki_product(A, X, digits: int, split_A=None):
    """A (M x K) . X (K x N) in FP64 from bf16 digit products."""
    import torch
    DA, eA = split_A if split_A is not None else split(A, digits, 1)
    DX, eX = split(X, digits, 0)
    keep = digits + 1
    lead = min(keep, 5)  # diagonals 2..5 combined exactly in int64 (shifts <= 24 bits)
    hi, lo = None, None
    for d in range(2, keep + 1):
        Z = None
        for p in range(1, d):
            q = d - p
            if p > digits or q > digits:
                continue
            P = mm32(DA[p - 1], DX[q - 1])
            Z = P if Z is None else Z + P
        if d <= lead:
            Zi = Z.to(torch.int64) << (8 * (lead - d))
            hi = Zi if hi is None else hi + Zi
        else:  # below 2^-40 of the leading part: FP64 rounding is far below the quantisation
            Zd = torch.ldexp(Z.to(torch.float64), torch.tensor(-8.0 * (d - lead), dtype=torch.float64,
                                                               device=Z.device))
            lo = Zd if lo is None else lo + Zd
    T = hi.to(torch.float64) if lo is None else hi.to(torch.float64) + lo
    return torch.ldexp(T, (eA + eX - 8 * lead).to(torch.float64))


def columns(seed: int = 3):
    """N realistic z columns: the kz modes of vor and phi of the seeded
    192x96x96 field (and their products by i kz and kx, as the fields of
    plane stage 1 are), [Re; Im] stacked: 126 x COLS FP64."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import shear_nnf_gb300 as sb
    lz = 2 * np.pi
    p = sb.make_params(mgalx=192, my=96, mgalz=96, Re=4000 / lz ** 2, alp=0.5, Ly=lz, gam=1.0)
    st = sb.seed_state(p, seed)
    kz = np.array([k if k <= NZ else k - MZ for k in range(MZ)], float)
    kx = 0.5 * np.arange(64)
    f = [st["vor"], st["phi"], 1j * kz[:, None, None] * st["vor"],
         1j * kx[None, :, None] * st["phi"], 1j * kz[:, None, None] * st["phi"],
         1j * kx[None, :, None] * st["vor"]]
    C = np.concatenate([g.reshape(MZ, -1) for g in f], axis=1)  # (mz, 6 * nkx * my)
    return np.concatenate([C.real, C.imag], axis=0)


def main():
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--digits", type=int, default=7)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--profile", action="store_true",
                    help="two split products only (for an ncu capture of the GEMMs)")
    a = ap.parse_args()
    dev = "cuda"
    A = torch.tensor(dft_block(), device=dev)
    X = torch.tensor(columns(), device=dev)
    if a.profile:
        sA = split(A, a.digits, 1)
        for _ in range(2):
            ozaki_product(A, X, a.digits, sA)
        torch.cuda.synchronize()
        return
    ref = A @ X  # FP64 reference product
    sA = split(A, a.digits, 1)
    Y = ozaki_product(A, X, a.digits, sA)
    err = float((Y - ref).abs().max() / ref.abs().max())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(a.reps):
            fn()
        ev1.record()
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / a.reps * 1e3  # us

    DX, _ = split(X, a.digits, 0)
    pairs = [(p, d - p) for d in range(2, a.digits + 2) for p in range(1, d)
             if p <= a.digits and d - p <= a.digits]
    t_split = timed(lambda: split(X, a.digits, 0))
    t_gemm = timed(lambda: [mm32(sA[0][p - 1], DX[q - 1]) for p, q in pairs])
    t_total = timed(lambda: ozaki_product(A, X, a.digits, sA))
    flops = 2.0 * A.shape[0] * A.shape[1] * X.shape[1] * len(pairs)
    print(json.dumps({"digits": a.digits, "gemms": len(pairs), "columns": X.shape[1],
                      "max_rel_err_vs_fp64_product": err, "split_us": t_split,
                      "gemm_us": t_gemm, "total_us": t_total,
                      "gemm_tflops": flops / (t_gemm * 1e-6) / 1e12}))


if __name__ == "__main__":
    main()
