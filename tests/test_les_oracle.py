"""CPU checks of the oracle's Smagorinsky LES block (cross.f90:1291-1406,
537-608, 639-648): with Cs = 0 it is the DNS step bit for bit, and on single
Fourier modes its eddy-viscosity decay rate matches the analytic value."""
import numpy as np
import pytest

import oracle
from conftest import box_params, copy_state


def _seed(o, seed, amp=0.3):
    """A smooth divergence-free state in pencil layout: random low modes of
    omega_y and phi (conjugate-symmetric kx = 0 column)."""
    rng = np.random.default_rng(seed)
    mz, nkx, my = o.mz, o.nkx, o.my
    st = {}
    for key in ("vor", "phi"):
        a = np.zeros((mz, nkx, my), complex)
        for k in list(range(0, 4)) + list(range(mz - 3, mz)):
            for i in range(0, 4):
                if i == 0 and k == 0:
                    continue
                ky = rng.integers(0, 3)
                yy = np.arange(my) * 2 * np.pi / my
                a[k, i, :] = amp * (rng.standard_normal() + 1j * rng.standard_normal()) * \
                    np.exp(1j * ky * yy)
        for k in range(o.nz + 1, mz):
            a[k, 0, :] = np.conj(a[mz - k, 0, :])
        st[key] = a
    yy = np.arange(my) * 2 * np.pi / my
    st["u00"] = 0.1 * np.sin(yy)
    st["w00"] = 0.05 * np.cos(2 * yy)
    st.update(time=0.0, xoffb=0.0, xofft=0.0)
    return st


def test_les_with_zero_constant_is_the_dns_step():
    kw = box_params(32, 16, 32, 1000.0)
    dns = oracle.Oracle(**kw)
    les = oracle.Oracle(**kw, les=1, les_visc=1, cs=0.0)
    st = _seed(dns, 1)
    a, b = copy_state(st), copy_state(st)
    tra, _ = dns.cross(a, 3)
    trb, _ = les.cross(b, 3)
    for key in ("vor", "phi", "u00", "w00"):
        assert np.array_equal(a[key], b[key]), key
    assert np.array_equal(tra, trb)


def _filter_width(o):
    lx, lz = 2 * np.pi / o.p.alp, 2 * np.pi / o.p.gam
    dx, dy, dz = lx / o.mx, o.p.Ly / o.my, lz / o.mz
    return (dx * dy * dz) ** (1.0 / 3.0)


def _mode_state(o, field, k, i, value):
    st = {"vor": np.zeros((o.mz, o.nkx, o.my), complex), "phi": np.zeros((o.mz, o.nkx, o.my), complex),
          "u00": np.zeros(o.my), "w00": np.zeros(o.my), "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    st[field][k, i, :] = value
    if i == 0:
        st[field][o.mz - k, 0, :] = np.conj(value)
    return st


RATE = 8.0 / (3.0 * np.pi)  # |cos| cos projected on cos: dA/dt = -RATE (Cs D)^2 A^2 k^3


@pytest.mark.parametrize("which", ["u(z)", "v(x)"])
def test_les_single_mode_decay_rate(which):
    """u = A sin(g z) (omega_y equation, rhgc1) or v = A sin(a x) (phi
    equation, rhvc2), no shear, no molecular viscosity: |S| = A k |cos|, the
    stress nu_t S has the fundamental (8/3pi) (Cs D)^2 A^2 k^2, so A decays at
    (8/3pi) (Cs D)^2 A^2 k^3."""
    cs, A, dt = 0.2, 0.1, 1e-5
    o = oracle.Oracle(32, 16, 32, Re=1e6, alp=1.0, Ly=2 * np.pi, gam=1.0, s=0.0, chi=0.0,
                      fixed_dt=dt, keep_laminar=1, les=1, les_visc=0, cs=cs)
    C = (cs * _filter_width(o)) ** 2
    if which == "u(z)":
        g = 1.0
        st = _mode_state(o, "vor", 1, 0, A * g / 2)       # omega_y = A g cos(g z)
        o.cross(st, 1)
        A1 = 2 * st["vor"][1, 0, :].real / g
        k = g
    else:
        a = 1.0
        st = _mode_state(o, "phi", 0, 1, -a * a * A / 2j)  # phi = lap v, v = A sin(a x)
        o.cross(st, 1)
        A1 = (2j * st["phi"][0, 1, :] / (-a * a)).real
        k = a
    rate = (A1 - A) / dt
    expect = -RATE * C * A * A * k ** 3
    np.testing.assert_allclose(rate, expect, rtol=2e-3)


def test_les_dissipates_and_reports_eddy_terms():
    kw = box_params(32, 16, 32, 1000.0)
    dns = oracle.Oracle(**kw)
    les = oracle.Oracle(**kw, les=1, les_visc=1, cs=0.2)
    st = _seed(dns, 2, amp=1.0)
    a, b = copy_state(st), copy_state(st)
    tra, _ = dns.cross(a, 10)
    trb, _ = les.cross(b, 10)
    e_dns = tra[-1, 2] ** 2 + tra[-1, 3] ** 2 + tra[-1, 4] ** 2
    e_les = trb[-1, 2] ** 2 + trb[-1, 3] ** 2 + trb[-1, 4] ** 2
    assert e_les < e_dns
    assert np.all(tra[:, 22:24] == 0.0)
    assert np.all(trb[:, 22] > 0.0) and np.all(trb[:, 23] > 0.0)   # nu_t, eddy dissipation
    # the eddy viscosity enters the viscous CFL number
    assert np.all(trb[:, 13] >= tra[:, 13] * 0.999)
