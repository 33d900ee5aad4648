"""CPU checks of the oracle: the transforms against numpy's DFT, the compact
schemes against their design conditions (prederiv1/prederiv2), the cyclic
shear-periodic solves against the discrete dispersion relation, and the time
step against the reference's own verification: the rapid-distortion solution
rdtfunc (operators.f90:1516-1562) and viscous decay without shear."""
import numpy as np
import pytest

import oracle
from conftest import box_params, copy_state


@pytest.mark.parametrize("n", [32, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384, 30])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(oracle.fft(x, -1), np.fft.fft(x), atol=1e-12 * n)
    np.testing.assert_allclose(oracle.fft(x, +1), np.fft.ifft(x) * n, atol=1e-12 * n)


def _full_spectrum(o, fou, mgalx, mgalz):
    full = np.zeros((mgalz, mgalx // 2 + 1), complex)
    for k in range(o.mz):
        kg = k if k <= o.nz else k + (mgalz - o.mz)
        full[kg, : o.nkx] = fou[k]
    return full


@pytest.mark.parametrize("grid", [(64, 32), (96, 48), (192, 96), (80, 160), (320, 256),
                                  (128, 384)])
def test_fourxz_matches_numpy(grid):
    """fourxz with fill00/pack00 (fou3D_thread.f:22-161): unnormalised c2r, r2c
    scaled by 1/(mgalx*mgalz), 2/3-rule truncation."""
    mgalx, mgalz = grid
    o = oracle.Oracle(mgalx, 32, mgalz, Re=10.0, alp=0.5, Ly=2 * np.pi, gam=1.0)
    rng = np.random.default_rng(mgalx)
    fou = rng.standard_normal((o.mz, o.nkx)) + 1j * rng.standard_normal((o.mz, o.nkx))
    for k in range(o.nz + 1, o.mz):
        fou[k, 0] = np.conj(fou[o.mz - k, 0])
    fou[0, 0] = fou[0, 0].real
    phys = o.fourxz_c2r(fou)
    ref = np.fft.irfft2(_full_spectrum(o, fou, mgalx, mgalz), s=(mgalz, mgalx)) * (mgalx * mgalz)
    np.testing.assert_allclose(phys[:, :mgalx], ref, atol=1e-12 * np.abs(ref).max())
    assert np.all(phys[:, mgalx:] == 0)
    back = o.fourxz_r2c(phys)
    np.testing.assert_allclose(back, fou, atol=1e-13 * np.abs(fou).max())
    # a physical field with content beyond 2/3 of the grid is truncated, not aliased
    x = np.arange(mgalx) * 2 * np.pi / mgalx
    high = np.cos((o.nkx + 2) * x)[None, :] * np.ones((mgalz, 1))
    ph = np.zeros((mgalz, mgalx + 2))
    ph[:, :mgalx] = high
    assert np.abs(o.fourxz_r2c(ph)).max() < 1e-13


def _mod_wavenumber(pr, rh, kap, second):
    j = np.arange(1, 4)
    den = 1 + 2 * np.sum(pr[4:] * np.cos(np.outer(kap, j)), axis=1)
    if second:
        return -(rh[3] + 2 * np.sum(rh[4:] * np.cos(np.outer(kap, j)), axis=1)) / den
    return 2 * np.sum(rh[4:] * np.sin(np.outer(kap, j)), axis=1) / den


def test_compact_scheme_design_conditions():
    """prederiv1: spectral points kappa = 0.5, 0.9, 0.7 pi; prederiv2: 0.9, 0.5,
    0.7 pi (diffy_shear_hepta.f90:81-88,199-208); plus the Taylor conditions."""
    o = oracle.Oracle(64, 32, 32, Re=10.0, alp=0.5, Ly=2 * np.pi, gam=1.0)
    pr1, rh1, pr2, rh2, dy = o.coeffs()
    rh1h, rh2h = rh1 * dy, rh2 * dy * dy
    kap = np.array([0.5, 0.9, 0.7]) * np.pi
    np.testing.assert_allclose(_mod_wavenumber(pr1, rh1h, kap, False), kap, rtol=1e-13)
    np.testing.assert_allclose(_mod_wavenumber(pr2, rh2h, kap, True), kap ** 2, rtol=1e-13)
    small = np.array([1e-3, 1e-2])
    np.testing.assert_allclose(_mod_wavenumber(pr1, rh1h, small, False), small, rtol=1e-11)
    np.testing.assert_allclose(_mod_wavenumber(pr2, rh2h, small, True), small ** 2, rtol=1e-8)
    assert pr1[3] == 1.0 and pr2[3] == 1.0 and rh1h[3] == 0.0
    np.testing.assert_allclose(pr1[:3], pr1[4:][::-1], rtol=0)
    np.testing.assert_allclose(rh1h[:3], -rh1h[4:][::-1], rtol=0)


@pytest.mark.parametrize("my", [32, 48, 96])
@pytest.mark.parametrize("theta", [0.0, 0.37, -2.5])
def test_derivyc_bloch_waves(my, theta):
    """On a shear-periodic Bloch wave u_j = exp(i k y_j) with u(y+Ly) = shp u(y),
    shp = exp(i k Ly), the cyclic LDL^H solve with the shear tail
    (modChol_addshear + solve7cyclic) returns exactly i k' u and -k''^2 u."""
    Ly = 2 * np.pi
    o = oracle.Oracle(64, my, 32, Re=10.0, alp=0.5, Ly=Ly, gam=1.0)
    pr1, rh1, pr2, rh2, dy = o.coeffs()
    y = np.arange(my) * dy - Ly / 2
    for n in [0, 3, my // 4, my // 3]:
        k = (2 * np.pi * n + theta) / Ly
        shp = np.exp(1j * k * Ly)
        u = np.exp(1j * k * y)
        kap = np.array([k * dy])
        k1 = _mod_wavenumber(pr1, rh1 * dy, kap, False)[0] / dy
        k2 = _mod_wavenumber(pr2, rh2 * dy * dy, kap, True)[0] / dy ** 2
        np.testing.assert_allclose(o.derivyc(u, shp=shp, iord=1), 1j * k1 * u, atol=1e-12 * max(1, abs(k1)))
        np.testing.assert_allclose(o.derivyc(u, shp=shp, iord=2), -k2 * u, atol=1e-12 * max(1, k2))
        for kk in [0.25, 7.0]:
            p = o.lapcdy(u, kk, shp=shp)
            np.testing.assert_allclose(p, u / (-k2 - kk), atol=1e-13 / kk)


def test_real_line_path():
    o = oracle.Oracle(64, 32, 32, Re=10.0, alp=0.5, Ly=2 * np.pi, gam=1.0)
    rng = np.random.default_rng(1)
    ur = rng.standard_normal(32)
    np.testing.assert_allclose(o.derivyc(ur, iord=1), o.derivyc(ur.astype(complex), iord=1).real,
                               atol=1e-14)


def _single_wave_state(o, i0, k0z, v0):
    """getini_rdt2 with k0y = 0 (initcr.f90:1501-1666): v = v0 exp(i(kx x + kz z))
    + c.c.; vor = 0, phi = -(kx^2 + kz^2) v."""
    st = {"vor": np.zeros((o.mz, o.nkx, o.my), complex), "phi": np.zeros((o.mz, o.nkx, o.my), complex),
          "u00": np.zeros(o.my), "w00": np.zeros(o.my), "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    kx, kz = 0.5 * i0, 1.0 * k0z
    st["phi"][k0z, i0, :] = -(kx * kx + kz * kz) * v0
    return st, kx, kz


def test_rdt_single_wave():
    """Rapid-distortion check used to verify the reference (log_changes rev.428-430):
    a single small-amplitude wave tilted by the shear follows rdtfunc
    (operators.f90:1516-1562): v(t) = v0 k0^2/k(t)^2 Du(t), ky(t) = -s kx t."""
    pp = box_params(64, 64, 32, rez=1000.0, fixed_dt=0.004)
    o = oracle.Oracle(**pp)
    v0 = 1e-3
    st, kx, kz = _single_wave_state(o, 1, 1, v0)
    nstep = 1000
    o.cross(st, nstep)
    t = st["time"]
    nu = 1.0 / pp["Re"]
    ky = -1.0 * kx * t
    k02 = kx * kx + kz * kz
    kt2 = k02 + ky * ky
    du = np.exp(-nu * t * (k02 + (1.0 * t * kx) ** 2 / 3.0))
    # v from phi through the Helmholtz solve with the current shear phase
    shp = np.exp(-1j * kx * st["xofft"])
    v = o.lapcdy(st["phi"][1, 1, :].copy(), k02, shp=shp)
    amp = np.abs(v)
    expected = v0 * k02 / kt2 * du
    assert np.abs(amp / expected - 1).max() < 2e-5
    # local wavenumber of the tilted wave
    dphase = np.angle(v[1:] / v[:-1])
    dy = pp["Ly"] / pp["my"]
    np.testing.assert_allclose(np.abs(dphase) / dy, abs(ky), rtol=1e-6)


def test_viscous_decay_without_shear():
    """s = 0: a small single wave decays as exp(-nu k^2 t) under the explicit RK3
    viscous term (laminar decay known answer)."""
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.01, s=0.0)
    o = oracle.Oracle(**pp)
    st, kx, kz = _single_wave_state(o, 2, 1, 1e-3)
    n = 100
    o.cross(st, n)
    k2 = kx * kx + kz * kz
    ratio = np.abs(st["phi"][1, 2, 0]) / (k2 * 1e-3)
    assert abs(ratio / np.exp(-k2 / pp["Re"] * st["time"]) - 1) < 1e-7


def test_cross_trace_and_time():
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005)
    import shear_nnf_gb300 as sb
    st = sb.seed_state(sb.make_params(**pp), 3)
    o = oracle.Oracle(**pp)
    tr, istop = o.cross(st, 5)
    assert istop == 0 and tr.shape == (5, oracle.TRACE_LEN)
    np.testing.assert_allclose(tr[:, 0], 0.005 * np.arange(5), atol=1e-15)
    assert np.all(tr[:, 1] == 0.005)
    assert np.all(np.diff(tr[:, 2]) < 0)  # u_rms decays in the first steps
    assert abs(st["time"] - 0.025) < 1e-15
    # offsets of the shear-periodic images: xofft = s Ly t, xoffb = -xofft
    assert abs(st["xofft"] - 2 * np.pi * 0.025) < 1e-13 and st["xoffb"] == -st["xofft"]


def test_etime_stops_the_run():
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005, etime=0.012)
    import shear_nnf_gb300 as sb
    st = sb.seed_state(sb.make_params(**{k: v for k, v in pp.items() if k != "etime"}), 3)
    o = oracle.Oracle(**pp)
    tr, istop = o.cross(st, 10)
    assert istop == 1
    assert abs(st["time"] - 0.012) < 1e-15
