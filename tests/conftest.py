"""Shared fixtures.  Tests marked ``gpu`` need a GB300 and the CUDA library;
everything else runs on the CPU (oracle, host logic, ABI surface)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def box_params(mgalx, my, mgalz, rez, fixed_dt=0.0, cfl=0.5, **kw):
    """Geometry of the benchmark configurations: Lx:Ly:Lz = 2:1:1 with Lz=2pi,
    S=1, Re = Re_z / Lz^2 (1/nu)."""
    lz = 2 * np.pi
    d = dict(mgalx=mgalx, my=my, mgalz=mgalz, Re=rez / lz ** 2, alp=0.5, Ly=lz, gam=1.0, s=1.0,
             chi=0.0, CFL=cfl, fixed_dt=fixed_dt)
    d.update(kw)
    return d


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def copy_state(st):
    return {k: (v.copy() if hasattr(v, "copy") else v) for k, v in st.items()}
