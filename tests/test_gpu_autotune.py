"""The autotuner (plane-stage tiles, warps per y-line solve and the y-line
form) picks tiles that compute the same step: bit for bit where only plane
tiles change, to the last bits where the y-line form changes, to the
rounding of the segment corrections where the y-line tile changes."""
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
    assert choice["line_form"] in ("fused", "split")
    b = copy_state(st0)
    tr_b, _ = box.cross(b, 5)
    # FP32 storage rounds the FP64 solves: a last-bit change there can move an
    # FP32 entry by one ulp
    same_lines = all(choice[k] == ref.tuning()[k] for k in ("line_segments", "line_form"))
    tol = 1e-13 if (prec == 0 or same_lines) else 1e-6
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < tol, k
    np.testing.assert_allclose(tr_b, tr_a, rtol=1e-11 if tol < 1e-12 else 1e-5, atol=1e-300)


@pytest.mark.parametrize("form", ["fused", "split"])
@pytest.mark.parametrize("nseg", [1, 2, 3])
def test_every_line_tile_matches_the_oracle(nseg, form):
    """1, 2 or 3 warps per y-line solve, fused or split y-line kernels: one
    step at 96x48x48 within the drop-in bar of the oracle, and 100 steps at
    64x32x32."""
    import oracle
    import shear_nnf_gb300 as sb
    for grid, nstep, tol in (((96, 48, 48), 1, 1e-12), ((64, 32, 32), 100, 1e-9)):
        pp = box_params(*grid, rez=1000.0, fixed_dt=0.005)
        p = sb.make_params(**pp)
        st0 = sb.seed_state(p, 4)
        box = sb.ShearBox(p)
        box.set_line_segments(nseg)
        box.set_line_form(form)
        assert box.tuning()["line_segments"] == nseg and box.tuning()["line_form"] == form
        g = copy_state(st0)
        box.cross(g, nstep)
        o = copy_state(st0)
        oracle.Oracle(**pp).cross(o, nstep)
        for k in ("vor", "phi", "u00", "w00"):
            assert rel_l2(g[k], o[k]) < tol, (grid, k)


@pytest.mark.parametrize("nseg", [1, 2, 3])
@pytest.mark.parametrize("grid,prec,extra", [((192, 96, 96), 0, {}), ((64, 32, 32), 1, {}),
                                             ((64, 32, 32), 0, {"les": 1, "les_visc": 1,
                                                                "cs": 0.1})])
def test_fused_lines_equal_split_lines(nseg, grid, prec, extra):
    """The fused y-line kernel computes the split kernels' step: the same
    operations on the same values (T and S rounded to the storage type as the
    split kernels store them), so FP64 agrees to the last bits (the compiler
    may pair multiplies and adds into FMAs differently in the two kernels)
    and the mixed form to FP32 rounding; with LES too."""
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(*grid, rez=4000.0, **extra))
    st0 = sb.seed_state(p, 11)
    out = {}
    for form in ("split", "fused"):
        box = sb.ShearBox(p, precision=prec)
        box.set_line_segments(nseg)
        box.set_line_form(form)
        s = copy_state(st0)
        tr, _ = box.cross(s, 4)
        out[form] = (s, tr)
    (a, tra), (b, trb) = out["split"], out["fused"]
    for k in ("vor", "phi", "u00", "w00"):
        assert rel_l2(b[k], a[k]) < (1e-13 if prec == 0 else 1e-6), k
    if prec == 0:
        np.testing.assert_allclose(trb, tra, rtol=1e-11, atol=1e-300)


def test_fused_form_refused_where_unavailable():
    """The temperature and y-filter handles run the split kernels only."""
    import shear_nnf_gb300 as sb
    for kw in ({"temperature": 1}, {"ydeal": 3}):
        p = sb.make_params(**box_params(64, 32, 32, rez=1000.0, **kw))
        box = sb.ShearBox(p)
        assert box.tuning()["line_form"] == "split"
        with pytest.raises(sb.ShearBoxError):
            box.set_line_form("fused")
        box.set_line_form("split")


@pytest.mark.parametrize("prec,extra", [(0, {}), (1, {}), (0, {"implicit_visc": 1}),
                                        (0, {"les": 1, "les_visc": 1, "cs": 0.1})])
def test_side_branch_masks_compute_the_same_step(prec, extra):
    """The spectra and the per-box scalars run as concurrent graph branches or
    in order on the main stream (sb_set_side_branch): the same kernels on the
    same inputs, so the state, the trace and the statistics agree bit for
    bit; the autotuner's mask is one of the four."""
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(64, 32, 32, rez=1000.0, **extra))
    st0 = sb.seed_state(p, 5)
    out = {}
    for mask in (3, 2, 1, 0):
        box = sb.ShearBox(p, precision=prec)
        box.set_side_branch(mask)
        assert box.tuning()["side_branch"] == mask
        s = copy_state(st0)
        tr, _ = box.cross(s, 4)
        out[mask] = (s, tr, box.statistics())
    s3, tr3, st3 = out[3]
    for mask in (2, 1, 0):
        s, tr, stt = out[mask]
        for k in ("vor", "phi", "u00", "w00"):
            assert np.array_equal(s[k], s3[k]), (mask, k)
        assert np.array_equal(tr, tr3), mask
        for k, v in st3.items():
            assert np.array_equal(np.asarray(stt[k]), np.asarray(v)), (mask, k)
    box = sb.ShearBox(p, precision=prec)
    with pytest.raises(sb.ShearBoxError):
        box.set_side_branch(4)
    box.set_state(st0)
    assert box.autotune()["side_branch"] in (0, 1, 2, 3)
