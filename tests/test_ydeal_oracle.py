"""CPU checks of the oracle's y transforms and y dealiasing (rfty/cfty,
rftdoublew.F / cftdoublew.F; dealiasing_y, operators.f90:352-467):
transform conventions against numpy, and the 2/3 rule in y on the kx = 0
lines and mean profiles (iydealiasing = 1)."""
import numpy as np
import pytest

import oracle
from conftest import box_params, copy_state


def _o(my=48, **kw):
    return oracle.Oracle(64, my, 32, Re=100.0, alp=0.5, Ly=2 * np.pi, gam=1.0, **kw)


@pytest.mark.parametrize("my", [32, 48])
def test_y_transforms_match_numpy(my):
    o = _o(my)
    rng = np.random.default_rng(my)
    u = rng.standard_normal(my)
    p = np.concatenate([u, [0.0, 0.0]])
    f = o.rfty(p, -1)
    ref = np.fft.rfft(u) / my
    np.testing.assert_allclose(f[0::2], ref.real, atol=1e-15)
    np.testing.assert_allclose(f[1::2], ref.imag, atol=1e-15)
    back = o.rfty(f, +1)
    np.testing.assert_allclose(back[:my], u, atol=1e-14)
    assert back[my] == 0.0 and back[my + 1] == 0.0
    z = rng.standard_normal(my) + 1j * rng.standard_normal(my)
    np.testing.assert_allclose(o.cfty(z, -1), np.fft.fft(z) / my, atol=1e-15)
    np.testing.assert_allclose(o.cfty(z, +1), np.fft.ifft(z) * my, atol=1e-13)


def test_ydeal1_removes_the_top_third_in_y():
    my = 48
    kw = box_params(64, my, 32, 1000.0, fixed_dt=1e-9, s=0.0, keep_laminar=1)
    o = oracle.Oracle(**kw, ydeal=1)
    rng = np.random.default_rng(3)
    st = {"vor": np.zeros((o.mz, o.nkx, my), complex), "phi": np.zeros((o.mz, o.nkx, my), complex),
          "u00": rng.standard_normal(my) * 1e-3, "w00": rng.standard_normal(my) * 1e-3,
          "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    for k in (1, 2):
        st["vor"][k, 0] = 1e-3 * (rng.standard_normal(my) + 1j * rng.standard_normal(my))
        st["vor"][o.mz - k, 0] = np.conj(st["vor"][k, 0])
    st["vor"][1, 3] = 1e-3 * (rng.standard_normal(my) + 1j * rng.standard_normal(my))
    b = copy_state(st)
    o.cross(b, 1)
    my23 = 2 * (my // 3)
    ny1 = ((my23 - 1) - 1) // 2
    # kx = 0 lines: y modes ny1 < j < my - ny1 removed; other lines keep them
    spec = np.fft.fft(b["vor"][1, 0])
    assert np.max(np.abs(spec[ny1 + 1: my - ny1])) < 1e-12 * np.max(np.abs(spec))
    spec3 = np.fft.fft(b["vor"][1, 3])
    assert np.max(np.abs(spec3[ny1 + 1: my - ny1])) > 1e-3 * np.max(np.abs(spec3))
    # mean profiles: real modes m >= my23 / 2 removed
    for key in ("u00", "w00"):
        f = np.fft.rfft(b[key])
        assert np.max(np.abs(f[my23 // 2:])) < 1e-12 * np.max(np.abs(f))


def test_ydeal2_runs_with_wrapped_offsets():
    kw = box_params(64, 48, 32, 1000.0, fixed_dt=0.01)
    o = oracle.Oracle(**kw, ydeal=2)
    rng = np.random.default_rng(5)
    st = {"vor": 1e-2 * (rng.standard_normal((o.mz, o.nkx, 48)) + 1j * rng.standard_normal((o.mz, o.nkx, 48))),
          "phi": np.zeros((o.mz, o.nkx, 48), complex), "u00": np.zeros(48), "w00": np.zeros(48),
          "time": 0.0, "xoffb": -5.0 * 4 * np.pi - 1.0, "xofft": 5.0 * 4 * np.pi + 1.0}
    for k in range(o.nz + 1, o.mz):
        st["vor"][k, 0] = np.conj(st["vor"][o.mz - k, 0])
    st["vor"][0, 0] = 0
    o.cross(st, 3)
    lx = 4 * np.pi
    assert abs(st["xoffb"]) < lx and st["xofft"] == -st["xoffb"]
    assert np.all(np.isfinite(st["vor"]))
