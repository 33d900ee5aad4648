"""GPU parity of the Smagorinsky LES step (iuse_LES) against the CPU oracle,
the analytic single-mode eddy-viscosity decay on the GPU, and the FP32-mixed
LES step against FP64."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2
from test_gpu_step import _field_errors, _run_both, _trace_error
from test_les_oracle import RATE, _filter_width, _mode_state

pytestmark = pytest.mark.gpu


def _les(grid, rez, **kw):
    d = dict(les=1, les_visc=1, cs=0.1)
    d.update(kw)
    return box_params(*grid, rez=rez, **d)


@pytest.mark.parametrize("grid,kw", [((64, 32, 32), {}),
                                     ((64, 32, 32), {"fixed_dt": 0.005, "les_visc": 0}),
                                     ((96, 48, 48), {"cs": 0.2})])
def test_les_one_step(grid, kw):
    pp = _les(grid, 4000.0, **kw)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1, k0=6.0)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < 1e-12, err
    assert _trace_error(tr_g, tr_o) < 1e-10
    assert np.all(tr_g[:, 22] > 0) and np.all(tr_g[:, 23] > 0)


def test_les_twenty_steps():
    pp = _les((64, 32, 32), 20000.0)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 20, k0=6.0)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < 1e-10, err
    assert _trace_error(tr_g, tr_o) < 1e-10
    assert status.steps_done == 20


@pytest.mark.parametrize("which", ["u(z)", "v(x)"])
def test_les_single_mode_decay_gpu(which):
    import oracle
    import shear_nnf_gb300 as sb
    cs, A, dt = 0.2, 0.1, 1e-5
    kw = dict(mgalx=32, my=16, mgalz=32, Re=1e6, alp=1.0, Ly=2 * np.pi, gam=1.0, s=0.0, chi=0.0,
              fixed_dt=dt, keep_laminar=1, les=1, les_visc=0, cs=cs)
    o = oracle.Oracle(**kw)
    C = (cs * _filter_width(o)) ** 2
    box = sb.ShearBox(sb.make_params(**kw))
    if which == "u(z)":
        st = _mode_state(o, "vor", 1, 0, A / 2)
        box.cross(st, 1)
        A1 = 2 * st["vor"][1, 0, :].real
    else:
        st = _mode_state(o, "phi", 0, 1, -A / 2j)
        box.cross(st, 1)
        A1 = (2j * st["phi"][0, 1, :] / -1.0).real
    np.testing.assert_allclose((A1 - A) / dt, -RATE * C * A * A, rtol=2e-3)


def test_les_mixed_against_fp64():
    import shear_nnf_gb300 as sb
    pp = _les((64, 32, 32), 20000.0)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 5, k0=6.0)
    out = {}
    for prec in (sb.SB_FP64, sb.SB_MIXED):
        box = sb.ShearBox(p, precision=prec)
        st = copy_state(st0)
        tr, _ = box.cross(st, 20)
        out[prec] = (st, tr)
    err = max(rel_l2(out[sb.SB_MIXED][0][k], out[sb.SB_FP64][0][k]) for k in ("vor", "phi"))
    assert err < 1e-5, err
    a, b = out[sb.SB_MIXED][1], out[sb.SB_FP64][1]
    # velocity variances, Reynolds stress and the eddy-viscosity records
    for q in (2, 3, 4, 22, 23):
        assert np.max(np.abs(a[:, q] - b[:, q]) / np.abs(b[:, q])) < 1e-5, q
    assert np.max(np.abs(a[:, 5] - b[:, 5])) < 1e-5 * np.max(np.abs(b[:, 2:5]) ** 2)


def test_les_batch_member_equals_single():
    import shear_nnf_gb300 as sb
    pp = _les((64, 32, 32), 8000.0)
    p = sb.make_params(**pp)
    states = [sb.seed_state(p, s, k0=6.0) for s in (11, 12, 13)]
    box = sb.ShearBox(p, batch=3)
    for m, st in enumerate(states):
        box.set_state(st, m)
    box.step(5)
    one = sb.ShearBox(p)
    one.set_state(states[1])
    one.step(5)
    a, b = box.get_state(1), one.get_state(0)
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(a[k], b[k]) < 1e-14, k
    assert np.allclose(box.trace(1), one.trace(0), rtol=1e-13, atol=0)
