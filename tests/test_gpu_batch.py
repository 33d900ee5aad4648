"""Batched boxes (ensembles): every member of a batch is bit-identical to the
same box run alone; per-member Reynolds numbers and seeds."""
import numpy as np
import pytest

from conftest import box_params, copy_state, rel_l2

pytestmark = pytest.mark.gpu


def test_batch_members_match_single_runs_fp64():
    import oracle
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005)
    p = sb.make_params(**pp)
    rez = [500.0, 1000.0, 2000.0, 750.0]
    states = [sb.seed_state(p, 20 + m) for m in range(len(rez))]
    box = sb.ShearBox(p, batch=len(rez))
    for m, (st, r) in enumerate(zip(states, rez)):
        box.set_state(st, m)
        box.set_re(m, r / (2 * np.pi) ** 2)
    box.step(3)
    for m, (st, r) in enumerate(zip(states, rez)):
        got = box.get_state(m)
        ref = copy_state(st)
        o = oracle.Oracle(**dict(pp, Re=r / (2 * np.pi) ** 2))
        o.cross(ref, 3)
        for k in ("vor", "phi", "u00", "w00"):
            assert rel_l2(got[k], ref[k]) < 1e-12, (m, k)
        assert box.status(m).steps_done == 3


def test_batch_stop_is_per_member():
    """A member that reaches its end time stops; the others go on."""
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, fixed_dt=0.005)
    p = sb.make_params(**pp)
    box = sb.ShearBox(p, batch=2)
    st = sb.seed_state(p, 1)
    box.set_state(st, 0)
    box.set_state(dict(st, time=1e10 - 0.007), 1)  # past etime = 1e10 after two steps
    box.step(5)
    assert box.status(0).steps_done == 5 and box.status(0).istop == 0
    s1 = box.status(1)
    assert s1.istop == 1 and s1.flags & 8 and s1.steps_done < 5
