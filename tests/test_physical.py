"""Physical fields of the post-processor convh5 (hvhg_uvwp, convh5.f90:650-933):
the oracle on known answers (laminar shear; Q = Qs + Qw for a divergence-free
field), and the GPU against the oracle."""
import numpy as np
import pytest

from conftest import box_params

import oracle
import shear_nnf_gb300 as sb

NAMES = ("u", "v", "w", "ox", "oy", "oz", "Q", "R", "Qs", "Rs", "Qw")


def _state(p, seed):
    st = sb.seed_state(p, seed)
    st.update(xoffb=-0.7, xofft=0.7)
    return st


def test_laminar_shear_known_answer():
    kw = box_params(32, 16, 32, 1000.0)
    o = oracle.Oracle(**kw)
    st = {"vor": np.zeros((o.mz, o.nkx, o.my), complex), "phi": np.zeros((o.mz, o.nkx, o.my), complex),
          "u00": np.zeros(o.my), "w00": np.zeros(o.my), "time": 0.0, "xoffb": 0.0, "xofft": 0.0}
    f = dict(zip(NAMES, o.physical(st, 0x7FF)))
    s = kw["s"]
    y = np.arange(o.my) * kw["Ly"] / o.my - kw["Ly"] / 2
    np.testing.assert_allclose(f["u"], np.broadcast_to(s * y[:, None, None], f["u"].shape), atol=1e-14)
    for k in ("v", "w", "ox", "oy", "Q", "R", "Rs"):
        assert np.abs(f[k]).max() < 1e-14, k
    np.testing.assert_allclose(f["oz"], -s, atol=1e-14)
    np.testing.assert_allclose(f["Qs"], -s * s / 4, atol=1e-14)
    np.testing.assert_allclose(f["Qw"], s * s / 4, atol=1e-14)


def test_q_is_qs_plus_qw():
    kw = box_params(64, 32, 32, 1000.0)
    p = sb.make_params(**kw)
    f = dict(zip(NAMES, oracle.Oracle(**kw).physical(_state(p, 3), 0x7FF)))
    assert np.abs(f["Q"] - f["Qs"] - f["Qw"]).max() < 1e-12 * np.abs(f["Q"]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_gpu_physical_matches_oracle(prec, tol):
    kw = box_params(96, 48, 48, 2000.0)
    p = sb.make_params(**kw)
    st = _state(p, 5)
    ref = dict(zip(NAMES, oracle.Oracle(**kw).physical(st, 0x7FF)))
    box = sb.ShearBox(p, batch=2, precision=prec)
    box.set_state(sb.seed_state(p, 1), 0)
    box.set_state(st, 1)
    got = box.physical(1)
    for k in NAMES:
        err = np.linalg.norm(got[k] - ref[k]) / max(np.linalg.norm(ref[k]), 1e-300)
        assert err < tol, (k, err)
    # the state is left as it was
    back = box.get_state(1)
    assert np.abs(back["vor"] - st["vor"]).max() <= 1e-6 * np.abs(st["vor"]).max()
