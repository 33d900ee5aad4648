"""The allocation-free derivyc entry point (sb_op_derivyc_noalloc) against the
allocating one (sb_op_derivyc), through the C-ABI.

Callers that cannot allocate device memory where they need a y-derivative (their
device memory is all in their own pool, or an allocation's possible
synchronisation is not acceptable there) use the no-alloc variant; it must give
the same results.  Two calls in a row with different inputs check that nothing
left in the shared scratch array leaks into the next call.  This file is
collected last so that a run stopping at the first failure has run every other
test before it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-13  # the tolerance of the operator tests


def _case(nlines, my, seed):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((my, nlines)) + 1j * rng.standard_normal((my, nlines))
    shp = np.exp(1j * rng.uniform(-np.pi, np.pi, nlines))
    return u, shp, np.conj(shp)


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    import shear_nnf_gb300 as sb
    Ly = 2 * np.pi
    for call, (nlines, my, iord) in enumerate([(4032, 96, 1), (333, 48, 2)]):
        u, shp, shm = _case(nlines, my, 100 + call)
        du = torch.from_numpy(u).cuda()
        ref = torch.zeros_like(du)
        got = torch.full_like(du, float("nan"))
        sb.op_derivyc(my, Ly, iord, du.data_ptr(), ref.data_ptr(), nlines, shp, shm)
        sb.op_derivyc_noalloc(my, Ly, iord, du.data_ptr(), got.data_ptr(), nlines, shp, shm)
        r = ref.cpu().numpy()
        g = got.cpu().numpy()
        assert np.all(np.isfinite(g))
        err = np.abs(g - r).max() / np.abs(r).max()
        assert err < TOL, (call, err)


def test_noalloc_exact_fit_matches_allocating_entry_point():
    """The largest request the scratch holds: 32768 lines of 16 points fill the
    y-buffer exactly (16 * pad32(2 * 32768) = 2**20 doubles)."""
    import torch
    import shear_nnf_gb300 as sb
    nlines, my = 32768, 16
    assert my * (((2 * nlines + 31) // 32) * 32) == 1 << 20
    u, shp, shm = _case(nlines, my, 7)
    du = torch.from_numpy(u).cuda()
    ref = torch.zeros_like(du)
    got = torch.full_like(du, float("nan"))
    sb.op_derivyc(my, 2 * np.pi, 1, du.data_ptr(), ref.data_ptr(), nlines, shp, shm)
    sb.op_derivyc_noalloc(my, 2 * np.pi, 1, du.data_ptr(), got.data_ptr(), nlines, shp, shm)
    r = ref.cpu().numpy()
    g = got.cpu().numpy()
    assert np.all(np.isfinite(g))
    assert np.abs(g - r).max() / np.abs(r).max() < TOL


@pytest.mark.parametrize("nlines,my", [(32769, 16), (32768, 17)])
def test_noalloc_rejects_one_past_the_limit(nlines, my):
    """One line more than the limit, or one point more per line at the full
    line count, is refused with error 6 before any device work."""
    import torch
    import shear_nnf_gb300 as sb
    du = torch.zeros((1, 1), dtype=torch.complex128, device="cuda")
    one = np.ones(nlines, np.complex128)
    with pytest.raises(sb.ShearBoxError, match="error 6.*exceed the fixed scratch"):
        sb.op_derivyc_noalloc(my, 2 * np.pi, 1, du.data_ptr(), du.data_ptr(), nlines, one, one)


def test_noalloc_rejects_oversized_requests():
    import torch
    import shear_nnf_gb300 as sb
    my, nlines = 512, 4096  # my * 2*nlines = 4 Mi doubles > the 1 Mi scratch
    du = torch.zeros((1, 1), dtype=torch.complex128, device="cuda")
    one = np.ones(nlines, np.complex128)
    with pytest.raises(sb.ShearBoxError, match="exceed the fixed scratch"):
        sb.op_derivyc_noalloc(my, 2 * np.pi, 1, du.data_ptr(), du.data_ptr(), nlines, one, one)
