"""GPU checks of the y-direction operators off the default step path: the y
transforms rfty/cfty and the compact filter as C-ABI operators against numpy
and the oracle, and the step with y dealiasing (iydealiasing 1, 2) against
the oracle."""
import numpy as np
import pytest

from conftest import box_params
from test_gpu_ops import _lines
from test_gpu_step import _field_errors, _run_both, _trace_error

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("my", [32, 48, 80, 96, 128, 160, 192, 256, 320])
def test_op_y_transforms(my):
    import torch
    import shear_nnf_gb300 as sb
    nl = 37
    rng = np.random.default_rng(my)
    z = rng.standard_normal((my, nl)) + 1j * rng.standard_normal((my, nl))
    d = torch.from_numpy(z.copy()).cuda()
    sb.op_cfty(my, d.data_ptr(), nl, -1)
    np.testing.assert_allclose(d.cpu().numpy(), np.fft.fft(z, axis=0) / my, atol=1e-14)
    sb.op_cfty(my, d.data_ptr(), nl, +1)
    np.testing.assert_allclose(d.cpu().numpy(), z, atol=1e-13)
    u = rng.standard_normal((my, nl))
    r = torch.zeros((my + 2, nl), dtype=torch.float64, device="cuda")
    r[:my] = torch.from_numpy(u).cuda()
    sb.op_rfty(my, r.data_ptr(), nl, -1)
    f = r.cpu().numpy()
    ref = np.fft.rfft(u, axis=0) / my
    np.testing.assert_allclose(f[0::2], ref.real, atol=1e-14)
    np.testing.assert_allclose(f[1::2], ref.imag, atol=1e-14)
    sb.op_rfty(my, r.data_ptr(), nl, +1)
    back = r.cpu().numpy()
    np.testing.assert_allclose(back[:my], u, atol=1e-13)
    assert np.all(back[my:] == 0.0)


@pytest.mark.parametrize("my", [32, 48, 96])
def test_op_filterc(my):
    import torch
    import oracle
    import shear_nnf_gb300 as sb
    nl = 41
    u, shp, _ = _lines(nl, my, 3 * my)
    du = torch.from_numpy(u.copy()).cuda()
    dout = torch.zeros_like(du)
    sb.op_filterc(my, du.data_ptr(), dout.data_ptr(), nl, shp)
    got = dout.cpu().numpy()
    o = oracle.Oracle(64, my, 32, Re=10.0, alp=0.5, Ly=2 * np.pi, gam=1.0)
    for line in range(nl):
        ref = o.filterc(u[:, line].copy(), shp[line])
        assert np.abs(got[:, line] - ref).max() < 1e-13 * np.abs(ref).max(), line


@pytest.mark.parametrize("grid,kw", [((64, 32, 32), {"ydeal": 1, "fixed_dt": 0.005}),
                                     ((96, 48, 48), {"ydeal": 1}),
                                     ((64, 32, 32), {"ydeal": 2, "fixed_dt": 0.005}),
                                     ((96, 48, 48), {"ydeal": 2}),
                                     ((64, 80, 32), {"ydeal": 1}),
                                     ((64, 128, 64), {"ydeal": 2})])
def test_ydeal_step(grid, kw):
    pp = box_params(*grid, rez=4000.0, **kw)
    st_o, tr_o, st_g, tr_g, status = _run_both(pp, 1)
    err = _field_errors(st_o, st_g)
    assert max(err.values()) < 1e-12, err
    assert _trace_error(tr_g, tr_o) < 1e-10


@pytest.mark.parametrize("ydeal", [1, 2])
def test_ydeal_ten_steps_wrapped_offsets(ydeal):
    import oracle
    import shear_nnf_gb300 as sb
    from conftest import copy_state, rel_l2
    pp = box_params(64, 32, 32, rez=4000.0, ydeal=ydeal)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 8)
    lx = 2 * np.pi / p.alp
    st0["xoffb"], st0["xofft"] = -(3 * lx + 1.3), 3 * lx + 1.3
    a, b = copy_state(st0), copy_state(st0)
    tr_o, _ = oracle.Oracle(**pp).cross(a, 10)
    tr_g, _ = sb.ShearBox(p).cross(b, 10)
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < 1e-10, k
    assert abs(b["xoffb"] - a["xoffb"]) < 1e-12 * lx
    assert _trace_error(tr_g, tr_o) < 1e-10
