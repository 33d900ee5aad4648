"""The autotuner (plane-stage tiles and warps per y-line solve) picks tiles
that compute the same step: bit for bit where only plane tiles change, to
the rounding of the segment corrections where the y-line tile changes."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("grid,prec", [((64, 32, 32), 0), ((192, 96, 96), 0), ((96, 48, 48), 1)])
def test_autotune_keeps_the_step(grid, prec):
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(*grid, rez=4000.0))
    st0 = sb.seed_state(p, 9)
    ref = sb.ShearBox(p, precision=prec)
    a = copy_state(st0)
    tr_a, _ = ref.cross(a, 5)
    box = sb.ShearBox(p, precision=prec)
    box.set_state(st0)
    choice = box.autotune()
    assert choice["p1_cols"] in (4, 8) and choice["p3_cols"] in (4, 8) and choice["p2_threads"] >= 64
    assert choice["line_segments"] in (1, 2, 3) and box.tuning() == choice
    b = copy_state(st0)
    tr_b, _ = box.cross(b, 5)
    # FP32 storage rounds the FP64 solves: a last-bit change there can move an
    # FP32 entry by one ulp
    same_lines = choice["line_segments"] == ref.tuning()["line_segments"]
    tol = 1e-13 if (prec == 0 or same_lines) else 1e-6
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < tol, k
    np.testing.assert_allclose(tr_b, tr_a, rtol=1e-11 if tol < 1e-12 else 1e-5, atol=1e-300)


@pytest.mark.parametrize("nseg", [1, 2, 3])
def test_every_line_tile_matches_the_oracle(nseg):
    """1, 2 or 3 warps per y-line solve: one step at 96x48x48 within the
    drop-in bar of the oracle, and 100 steps at 64x32x32."""
    import oracle
    import shear_nnf_gb300 as sb
    for grid, nstep, tol in (((96, 48, 48), 1, 1e-12), ((64, 32, 32), 100, 1e-9)):
        pp = box_params(*grid, rez=1000.0, fixed_dt=0.005)
        p = sb.make_params(**pp)
        st0 = sb.seed_state(p, 4)
        box = sb.ShearBox(p)
        box.set_line_segments(nseg)
        assert box.tuning()["line_segments"] == nseg
        g = copy_state(st0)
        box.cross(g, nstep)
        o = copy_state(st0)
        oracle.Oracle(**pp).cross(o, nstep)
        for k in ("vor", "phi", "u00", "w00"):
            assert rel_l2(g[k], o[k]) < tol, (grid, k)
