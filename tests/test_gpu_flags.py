"""Stop flags of the step on host-made states (cross.f90:1683-1690, 2102-2115):
a NaN in the statistics record, a laminarised box (v_rms / Lz < 1e-5) and a
CFL time step below 1e-10 ("Diverged").  Within one step call (one call of
cross) a flagged member is frozen from the step at which cross would leave its
loop -- the stop check runs from the third step on (cross.f90:221), so after
two steps -- while the other members of the batch go on exactly as if they ran
alone.  No GPU fault is involved: the failures are written into the state from
the host."""
import numpy as np
import pytest

from conftest import box_params

pytestmark = pytest.mark.gpu

SBF_DIVERGED, SBF_NAN, SBF_LAMINAR, SBF_ETIME = 1, 2, 4, 8
KEYS = ("vor", "phi", "u00", "w00")


def _params(**kw):
    import shear_nnf_gb300 as sb
    return sb.make_params(**box_params(64, 32, 32, rez=1000.0, cfl=0.5, **kw))


def _run(p, states, nstep):
    """A batch of the states stepped once by nstep steps: (states, statuses)."""
    import shear_nnf_gb300 as sb
    box = sb.ShearBox(p, batch=len(states))
    for m, st in enumerate(states):
        box.set_state(st, m)
    box.step(nstep)
    return ([box.get_state(m) for m in range(len(states))],
            [box.status(m) for m in range(len(states))])


def _bits(a):
    return np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) else np.float64).view(np.float64)


def _same(a, b):
    """Bitwise equality of two states, NaN equal to NaN."""
    for k in KEYS:
        x, y = _bits(a[k]), _bits(b[k])
        if not (np.array_equal(np.isnan(x), np.isnan(y)) and
                np.array_equal(x[~np.isnan(x)], y[~np.isnan(y)])):
            return False
    ta, tb = a["time"], b["time"]
    return ta == tb or (np.isnan(ta) and np.isnan(tb))


def test_nan_and_laminar_members_stop_others_go_on():
    import shear_nnf_gb300 as sb
    p = _params()
    good = sb.seed_state(p, 31)
    bad = sb.seed_state(p, 32)
    bad["vor"][1, 1, 5] = np.nan
    lam = sb.seed_state(p, 33, urms=1e-6)  # v_rms / Lz ~ 1e-7 < 1e-5
    out, stat = _run(p, [good, bad, lam], 6)
    s0, s1, s2 = stat
    assert s0.flags == 0 and s0.istop == 0 and s0.steps_done == 6
    assert s1.flags & SBF_NAN and s1.istop == 1 and s1.steps_done == 2
    assert s2.flags & SBF_LAMINAR and s2.istop == 1 and s2.steps_done == 2
    assert not s2.flags & SBF_NAN and not s1.flags & SBF_LAMINAR
    # member 0 is bit-identical to the same box run alone
    alone, st_alone = _run(p, [good], 6)
    assert _same(out[0], alone[0]) and st_alone[0].flags == 0
    # the flagged members were frozen after their second step
    two, _ = _run(p, [good, bad, lam], 2)
    assert _same(out[1], two[1]) and _same(out[2], two[2])
    assert not _same(out[0], two[0])


def test_laminar_member_goes_on_with_keep_laminar():
    """keep_laminar (the Newton searches' option) records the flag but does
    not stop the member."""
    import shear_nnf_gb300 as sb
    p = _params(keep_laminar=1)
    _, stat = _run(p, [sb.seed_state(p, 33, urms=1e-6)], 4)
    s = stat[0]
    assert s.flags & SBF_LAMINAR and s.istop == 0 and s.steps_done == 4


def test_cfl_step_underflow_flags_diverged():
    """A velocity of 1e12 makes the CFL time step ~1e-14 < 1e-10: the member is
    flagged as diverged and frozen after its second step; its neighbour in the
    batch is unaffected."""
    import shear_nnf_gb300 as sb
    p = _params()
    good = sb.seed_state(p, 41)
    fast = sb.seed_state(p, 42, urms=1e12)
    out, stat = _run(p, [good, fast], 5)
    s0, s1 = stat
    assert s1.flags & SBF_DIVERGED and s1.istop == 1 and s1.steps_done == 2
    assert 0.0 < s1.deltat < 1e-10
    assert s0.flags == 0 and s0.steps_done == 5
    alone, _ = _run(p, [good], 5)
    assert _same(out[0], alone[0])
    two, _ = _run(p, [good, fast], 2)
    assert _same(out[1], two[1])


def test_a_new_call_starts_afresh():
    """The flags belong to one call: the next call with a good state runs
    unflagged (the entry of cross resets istop)."""
    import shear_nnf_gb300 as sb
    p = _params()
    box = sb.ShearBox(p)
    bad = sb.seed_state(p, 32)
    bad["vor"][1, 1, 5] = np.nan
    box.set_state(bad)
    box.step(3)
    assert box.status().flags & SBF_NAN
    box.set_state(sb.seed_state(p, 31))
    box.step(3)
    s = box.status()
    assert s.flags == 0 and s.steps_done == 3
