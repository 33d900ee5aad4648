"""Golden fixtures (tests/golden/make_golden.py): the oracle reproduces them on
this machine; the GPU step reproduces them on a GB300."""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

CASES = ["step64_seed3", "les64_seed5", "filt64_seed4", "ydeal64_seed6", "temp64_seed7",
         "force64_seed8"]
INTS = ("mgalx", "my", "mgalz", "les", "les_visc", "ydeal", "temperature", "force", "damping")


def _case(name):
    g = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    params = {k[2:]: g[k].item() for k in g.files if k.startswith("p_")}
    for k in INTS:
        if k in params:
            params[k] = int(params[k])
    return g, params


def _keys(g):
    return ("vor", "phi", "u00", "w00") + (("tb", "tb00") if "tb" in g.files else ())


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    import oracle
    import shear_nnf_gb300 as sb
    g, params = _case(name)
    st = sb.seed_state(sb.make_params(**params), int(g["seed"]))
    tr, _ = oracle.Oracle(**params).cross(st, int(g["nstep"]))
    for k in _keys(g):
        assert rel_l2(st[k], g[k]) < 1e-13, k
    np.testing.assert_allclose(tr, g["trace"], rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_reproduces_golden(name):
    import shear_nnf_gb300 as sb
    g, params = _case(name)
    p = sb.make_params(**params)
    st = sb.seed_state(p, int(g["seed"]))
    box = sb.ShearBox(p)
    tr, status = box.cross(st, int(g["nstep"]))
    for k in _keys(g):
        assert rel_l2(st[k], g[k]) < 1e-12, k
    np.testing.assert_allclose(tr, g["trace"], rtol=1e-10, atol=1e-300)
    assert st["time"] == pytest.approx(float(g["time"]), abs=1e-15)
