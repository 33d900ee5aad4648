"""The hist accumulators (module statistics, mod.f90:94-115): per-plane stats
and stats2, the kx-kz spectra spl and spl2 and, with the temperature, tstats
and splt.  Oracle checks: the plane sums reproduce the UNER record, Parseval
ties the spectra to the plane sums, the Delta t weights and counts, odd and
even moments under u -> -u.  GPU: the accumulators against the oracle through
the C-ABI."""
import numpy as np
import pytest

import shear_nnf_gb300 as sb
from conftest import box_params, copy_state, rel_l2

LZ = 2 * np.pi


def _run(pp, nstep, seed=3, k0=4.0, deltat=0.0):
    import oracle
    st = sb.seed_state(sb.make_params(**pp), seed, k0=k0)
    o = oracle.Oracle(**pp)
    o.deltat = deltat
    tr, _ = o.cross(st, nstep)
    return o, tr, o.statistics()


def test_plane_sums_reproduce_the_record():
    pp = box_params(32, 32, 32, rez=1000.0, fixed_dt=0.01)
    o, tr, S = _run(pp, 1, deltat=0.02)
    my = pp["my"]
    st = S["stats"]
    r = tr[0]
    # uner(1:3) = sqrt(mean over planes), uner(4:6) means; stats 4..9
    np.testing.assert_allclose(np.sqrt(np.abs(st[:, 3:6].sum(0) / my)), r[2:5], rtol=1e-13)
    np.testing.assert_allclose(st[:, 6:9].sum(0) / my, r[5:8], rtol=1e-12)
    np.testing.assert_allclose(np.sqrt(np.abs(st[:, 12:15].sum(0) / my)), r[8:11], rtol=1e-13)
    assert st[:, 15].sum() / my == pytest.approx(r[11], rel=1e-13)  # eps
    assert st[:, 19].sum() / my == pytest.approx(r[20], rel=1e-12)  # Pk
    assert st[:, 20].sum() / my == pytest.approx(r[21], rel=1e-12, abs=1e-300)  # o1 o2
    # stats2 weights: the Delta t of the step before the record
    np.testing.assert_allclose(S["stats2"], st * 0.02, rtol=1e-15, atol=1e-300)
    assert S["nacum"] == 1 and S["total_dt"] == pytest.approx(0.01, rel=1e-15)


def test_spectra_parseval_and_means():
    pp = box_params(32, 32, 32, rez=1000.0, cfl=0.5)
    o, tr, S = _run(pp, 3, seed=5, deltat=0.0)
    st, sp = S["stats"], S["spec"]
    # summed over all modes the spectra equal the plane sums (same terms)
    pairs = {0: 3, 1: 4, 2: 5, 3: 6, 4: 12, 5: 13, 6: 14, 7: 20}
    for f, q in pairs.items():
        assert sp[:, :, f].sum() == pytest.approx(st[:, q].sum(), rel=1e-12, abs=1e-14), f
    assert S["nacum"] == 3
    assert S["total_dt"] == pytest.approx(tr[:, 1].sum(), rel=1e-14)
    # stats2 of the first record carry Delta t = 0 (the value before the run)
    assert np.all(np.isfinite(S["stats2"])) and np.all(np.isfinite(S["spec2"]))


def test_moments_under_velocity_reversal():
    pp = box_params(32, 32, 32, rez=1000.0, fixed_dt=0.01)
    import oracle
    st = sb.seed_state(sb.make_params(**pp), 7)
    neg = {k: (-v if isinstance(v, np.ndarray) else v) for k, v in st.items()}
    o1, o2 = oracle.Oracle(**pp), oracle.Oracle(**pp)
    o1.cross(copy_state(st), 1)
    o2.cross(neg, 1)
    a, b = o1.statistics()["stats"], o2.statistics()["stats"]
    # eps (15) and Pk (19) carry the laminar shear -s in omega_z: neither
    even = [3, 4, 5, 6, 7, 8, 12, 13, 14, 20]
    odd = [0, 2, 9, 10, 11, 16, 17, 18]
    np.testing.assert_allclose(b[:, even], a[:, even], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(b[:, odd], -a[:, odd], rtol=1e-12, atol=1e-14)
    assert np.abs(a[:, 16:19]).max() > 0


def test_temperature_statistics():
    pp = box_params(32, 32, 32, rez=1000.0, fixed_dt=0.01, temperature=1,
                    fkappa=LZ ** 2 / 1000.0 / 0.7, bym=1.0, gbeta=0.5)
    o, tr, S = _run(pp, 2, seed=9, deltat=0.01)
    my = pp["my"]
    ts, tsp = S["tstats"], S["tspec"]
    assert np.all(np.isfinite(ts)) and np.abs(tsp).max() > 0
    # tstats(1) is the Delta t-weighted mean profile tb00
    for f, q in {0: 1, 1: 2, 2: 3, 3: 4}.items():
        assert tsp[:, :, f].sum() == pytest.approx(ts[:, q].sum(), rel=1e-12, abs=1e-14)
    assert S["nacum"] == 2 and my == ts.shape[0]


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _compare(pp, nstep, seed=3, k0=4.0, tol=1e-11, precision=0):
    import oracle
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, seed, k0=k0)
    o = oracle.Oracle(**pp)
    o.cross(copy_state(st0), nstep)
    So = o.statistics()
    box = sb.ShearBox(p, precision=precision)
    box.cross(copy_state(st0), nstep)
    Sg = box.statistics()
    assert Sg["nacum"] == So["nacum"]
    assert Sg["total_dt"] == pytest.approx(So["total_dt"], rel=max(tol, 1e-12))
    for k in [k for k in Sg if isinstance(Sg[k], np.ndarray)]:
        err = rel_l2(Sg[k], So[k])
        assert err < tol, (k, err)
    return Sg, So


@pytest.mark.gpu
@pytest.mark.parametrize("grid,kw", [((64, 32, 32), {}),
                                     ((96, 48, 48), {"fixed_dt": 0.005}),
                                     ((64, 32, 32), {"les": 1, "les_visc": 1, "cs": 0.1}),
                                     ((64, 32, 32), {"temperature": 1, "fkappa": LZ ** 2 / 4000 / 0.7,
                                                     "bym": 1.0, "gbeta": 0.5})])
def test_gpu_statistics_match_oracle(grid, kw):
    pp = box_params(*grid, rez=4000.0, **kw)
    _compare(pp, 3, k0=6.0 if kw.get("les") else 4.0)


@pytest.mark.gpu
def test_gpu_statistics_every_second_step_and_reset():
    pp = box_params(64, 32, 32, rez=4000.0, nhist=2)
    Sg, So = _compare(pp, 5)
    assert Sg["nacum"] == 3  # steps 1, 3, 5


@pytest.mark.gpu
def test_gpu_statistics_mixed():
    pp = box_params(96, 48, 48, rez=4000.0)
    _compare(pp, 3, tol=1e-5, precision=sb.SB_MIXED)
