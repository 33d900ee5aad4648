"""GPU parity of the standalone y-operators (derivyc, lapcdy) against the oracle,
line by line, with random shear phases (FP64: relative error below 1e-13)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-13


def _lines(nlines, my, seed):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((my, nlines)) + 1j * rng.standard_normal((my, nlines))
    th = rng.uniform(-np.pi, np.pi, nlines)
    shp = np.exp(1j * th)
    return u, shp, np.conj(shp)


@pytest.mark.parametrize("my", [32, 48, 96])
@pytest.mark.parametrize("iord", [1, 2])
def test_op_derivyc(my, iord):
    import torch
    import oracle
    import shear_nnf_gb300 as sb
    Ly = 2 * np.pi
    nlines = 77
    u, shp, shm = _lines(nlines, my, 10 * my + iord)
    du = torch.from_numpy(u.copy()).cuda()
    dout = torch.zeros_like(du)
    sb.op_derivyc(my, Ly, iord, du.data_ptr(), dout.data_ptr(), nlines, shp, shm)
    got = dout.cpu().numpy()
    o = oracle.Oracle(64, my, 32, Re=10.0, alp=0.5, Ly=Ly, gam=1.0)
    for line in range(nlines):
        ref = o.derivyc(u[:, line].copy(), shp=shp[line], shm=shm[line], iord=iord)
        err = np.abs(got[:, line] - ref).max() / np.abs(ref).max()
        assert err < TOL, (line, err)


@pytest.mark.parametrize("my", [32, 96])
def test_op_lapcdy(my):
    import torch
    import oracle
    import shear_nnf_gb300 as sb
    Ly = 2 * np.pi
    nlines = 50
    u, shp, shm = _lines(nlines, my, 77 + my)
    k2 = np.random.default_rng(my).uniform(0.2, 900.0, nlines)
    du = torch.from_numpy(u.copy()).cuda()
    dout = torch.zeros_like(du)
    sb.op_lapcdy(my, Ly, du.data_ptr(), dout.data_ptr(), nlines, k2, shp, shm)
    got = dout.cpu().numpy()
    o = oracle.Oracle(64, my, 32, Re=10.0, alp=0.5, Ly=Ly, gam=1.0)
    for line in range(nlines):
        ref = o.lapcdy(u[:, line].copy(), k2[line], shp=shp[line], shm=shm[line])
        err = np.abs(got[:, line] - ref).max() / np.abs(ref).max()
        assert err < TOL, (line, err)


def test_op_derivyc_real_line_matches_m1_path():
    """A real line (zero imaginary part, shp = shm = 1) takes the reference's
    m=1 path (diffy_shear_hepta.f90:341-354,408-410)."""
    import torch
    import oracle
    import shear_nnf_gb300 as sb
    my, Ly = 48, 2 * np.pi
    rng = np.random.default_rng(5)
    ur = rng.standard_normal(my)
    du = torch.from_numpy(ur.astype(np.complex128).reshape(my, 1)).cuda()
    dout = torch.zeros_like(du)
    one = np.ones(1, np.complex128)
    sb.op_derivyc(my, Ly, 1, du.data_ptr(), dout.data_ptr(), 1, one, one)
    got = dout.cpu().numpy()[:, 0]
    o = oracle.Oracle(64, my, 32, Re=10.0, alp=0.5, Ly=Ly, gam=1.0)
    ref = o.derivyc(ur, iord=1)
    assert np.abs(got.imag).max() == 0.0
    assert np.abs(got.real - ref).max() / np.abs(ref).max() < TOL
