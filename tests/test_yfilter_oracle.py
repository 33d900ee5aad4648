"""CPU checks of the oracle's compact y-filter (iydealiasing = 3, prefilter /
filterc, filter_shear_hepta.f90:21-148): the transfer function of the fixed
coefficients equals its design points, and shear-periodic Bloch waves are
eigenfunctions with that transfer function."""
import numpy as np
import pytest

import oracle
from conftest import box_params, copy_state

RH = np.array([-0.000179828066167, 0.054442102978149, 0.309968182770373, 0.749052269410218,
               0.987412035368317, 0.749052269410218, 0.309968182770373, 0.054442102978149,
               -0.000179828066167])
PR = np.array([0.053003478448814, 0.315003368623046, 0.738981897704866, 1.0,
               0.738981897704866, 0.315003368623046, 0.053003478448814])


def transfer(kap):
    return (RH * np.cos(kap * np.arange(-4, 5))).sum() / (PR * np.cos(kap * np.arange(-3, 4))).sum()


def test_filter_design_points():
    # the design of the coefficients (the MATLAB notes of prefilter): G(pi) = 0,
    # G(6pi/9) = 0.72, G(8.5pi/9) = 0.001, G(5.5pi/9) = 0.91, G(0) = 1
    for kap, g in ((1.0, 0.0), (6 / 9, 0.72), (8.5 / 9, 0.001), (5.5 / 9, 0.91), (0.0, 1.0)):
        assert abs(transfer(kap * np.pi) - g) < 1e-12


@pytest.mark.parametrize("my", [32, 48])
@pytest.mark.parametrize("theta", [0.0, 0.7, -2.1])
def test_filter_bloch_waves(my, theta):
    o = oracle.Oracle(64, my, 64, Re=100.0, alp=0.5, Ly=2 * np.pi, gam=1.0)
    shp = np.exp(1j * theta)
    j = np.arange(my)
    for n in (0, 3, my // 4, my // 2 - 1, my // 2):
        q = (2 * np.pi * n + theta) / my
        u = np.exp(1j * q * j)
        np.testing.assert_allclose(o.filterc(u, shp), transfer(q) * u, atol=1e-13)
    # real lines (the mean profiles)
    u = np.cos(2 * np.pi * 5 * j / my)
    np.testing.assert_allclose(o.filterc(u), transfer(2 * np.pi * 5 / my) * u, atol=1e-13)


def test_filtered_run_damps_short_y_scales():
    # no shear and small amplitude: y Fourier modes do not couple, so the
    # filter applied at every substep removes the y-Nyquist mode for good
    kw = box_params(32, 16, 32, 1000.0, fixed_dt=0.005, s=0.0, keep_laminar=1)
    o0 = oracle.Oracle(**kw)
    o3 = oracle.Oracle(**kw, ydeal=3)
    rng = np.random.default_rng(1)
    st = {"vor": np.zeros((o0.mz, o0.nkx, 16), complex), "phi": np.zeros((o0.mz, o0.nkx, 16), complex),
          "u00": np.zeros(16), "w00": np.zeros(16), "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    yy = np.arange(16)
    st["vor"][1, 1, :] = 1e-6 * np.exp(1j * np.pi * yy) + 1e-4 * np.exp(1j * 2 * np.pi * yy / 16)
    st["phi"][2, 1, :] = 1e-4 * rng.standard_normal(16)
    a, b = copy_state(st), copy_state(st)
    o0.cross(a, 2)
    o3.cross(b, 2)
    # the Nyquist component in y is removed by the filter, the long wave kept
    nyq = lambda v: abs(np.sum(v * np.exp(-1j * np.pi * yy)))
    assert nyq(b["vor"][1, 1]) < 1e-6 * nyq(a["vor"][1, 1])
    assert abs(np.vdot(b["vor"][1, 1], a["vor"][1, 1])) > 0.9 * np.vdot(a["vor"][1, 1], a["vor"][1, 1]).real
