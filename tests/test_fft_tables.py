"""Twiddle tables of the transforms (host code, sb_fft_twiddles): the factored
FP64 form e^{-2 pi i t/n} = (-i)^q c (1 + i tau) reconstructs the complex table,
keeps c >= cos(pi/4) and |tau| <= 1, and its swap bits and signs follow q; a
numpy model of the device's FP64 stages (radix 3 or 5 first, fused radix-4
and radix-2 pairs, the 2/3-gap radix-3 stage) on these tables equals the DFT
for every supported length.  The device stages themselves are checked by the GPU
parity tests."""
import numpy as np
import pytest

import shear_nnf_gb300 as sb

LENGTHS = (32, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384)
PLANS = {32: [4, 4, 2], 48: [3, 4, 4], 64: [4, 4, 4], 80: [5, 4, 4], 96: [3, 4, 4, 2],
         128: [4, 4, 4, 2], 160: [5, 4, 4, 2], 192: [3, 4, 4, 4], 256: [4, 4, 4, 4],
         320: [5, 4, 4, 4], 384: [3, 4, 4, 4, 2]}


def _factored(n):
    g = sb.fft_twiddles(n, factored=True)
    sw = g[:, 3].copy().view(np.int64)
    return g[:, 0], g[:, 1], g[:, 2], sw


@pytest.mark.parametrize("n", LENGTHS)
def test_factored_table_reconstructs_the_twiddles(n):
    mx, my, tau, sw = _factored(n)
    w = sb.fft_twiddles(n, factored=False)
    t = np.arange(n)
    q = ((8 * t + n) // (2 * n)) % 4
    assert np.array_equal(sw, q & 1)
    c = np.where(q <= 1, mx, -mx)
    assert np.all(c >= np.cos(np.pi / 4) - 1e-15) and np.all(np.abs(tau) <= 1 + 1e-15)
    assert np.array_equal(my, np.where(sw == 1, -mx, mx))
    rec = (-1j) ** q * c * (1 + 1j * tau)
    assert np.abs(rec - w).max() < 1e-15  # a few ulp: tau and the product round
    assert np.abs(w - np.exp(-2j * np.pi * t / n)).max() < 2e-15


def _apply(tab, t, v, sign):
    mx, my, tau, sw = tab
    if sign < 0:
        za, zb, ax, ay = v.real - tau[t] * v.imag, v.imag + tau[t] * v.real, mx[t], my[t]
    else:
        za, zb, ax, ay = v.real + tau[t] * v.imag, v.imag - tau[t] * v.real, my[t], mx[t]
    sx, sy = (zb, za) if sw[t] else (za, zb)
    return ax * sx + 1j * (ay * sy)


def _stage(x, n, ns, r, sign, tab, gap):
    out = np.zeros_like(x)
    nr, step = n // r, n // (ns * r)
    s3 = np.sqrt(3) / 2 * (1 if sign < 0 else -1)
    for j in range(nr):
        v = [x[j + q * nr] for q in range(r)]
        jm = j % ns
        if ns == 1 and r == 3:
            v1 = 0 if gap else v[1]
            t1, d = v1 + v[2], v1 - v[2]
            h = v[0] - 0.5 * t1
            X = [v[0] + t1, h + s3 * (d.imag - 1j * d.real), h - s3 * (d.imag - 1j * d.real)]
        elif ns == 1 and r == 5:
            # the 5-point DFT of butterfly<5> from the symmetric pairs
            c1, c2 = np.cos(2 * np.pi / 5), np.cos(4 * np.pi / 5)
            s1, s2 = np.sin(2 * np.pi / 5), np.sin(4 * np.pi / 5)
            t1, t2, t3, t4 = v[1] + v[4], v[2] + v[3], v[1] - v[4], v[2] - v[3]
            a1, a2 = v[0] + c1 * t1 + c2 * t2, v[0] + c2 * t1 + c1 * t2
            b1, b2 = s1 * t3 + s2 * t4, s2 * t3 - s1 * t4
            sg = -1 if sign < 0 else 1
            X = [v[0] + t1 + t2, a1 + 1j * sg * b1, a2 + 1j * sg * b2, a2 - 1j * sg * b2,
                 a1 - 1j * sg * b1]
        elif ns == 1 and r == 4:
            a0, a1, b0, b1 = v[0] + v[2], v[0] - v[2], v[1] + v[3], v[1] - v[3]
            jb = -1j * b1 if sign < 0 else 1j * b1
            X = [a0 + b0, a1 + jb, a0 - b0, a1 - jb]
        elif r == 4:
            w2v2, w2v3 = _apply(tab, 2 * jm * step, v[2], sign), _apply(tab, 2 * jm * step, v[3], sign)
            a0, a1, e0, e1 = v[0] + w2v2, v[0] - w2v2, v[1] + w2v3, v[1] - w2v3
            p, q = _apply(tab, jm * step, e0, sign), _apply(tab, jm * step, e1, sign)
            jq = -1j * q if sign < 0 else 1j * q
            X = [a0 + p, a1 + jq, a0 - p, a1 - jq]
        else:
            wv = _apply(tab, jm * step, v[1], sign)
            X = [v[0] + wv, v[0] - wv]
        base = (j // ns) * ns * r + jm
        for q in range(r):
            out[base + q * ns] = X[q]
    return out


@pytest.mark.parametrize("n", LENGTHS)
@pytest.mark.parametrize("sign", [-1, 1])
def test_factored_stages_equal_the_dft(n, sign):
    tab = _factored(n)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * n
    for gap in ((False, True) if n % 3 == 0 else (False,)):
        y = x.copy()
        if gap:  # a truncated spectrum: zero middle third
            y[n // 3:2 * n // 3 + 1] = 0
        want = np.fft.fft(y) if sign < 0 else np.fft.ifft(y) * n
        ns = 1
        for r in PLANS[n]:
            y = _stage(y, n, ns, r, sign, tab, gap and ns == 1)
            ns *= r
        assert np.abs(y - want).max() < 1e-14 * np.abs(want).max(), (n, sign, gap)
    assert ref is not None
