"""Generates the golden fixtures of the step tests from the C oracle.

The reference ships no test vectors (its verification was by hand: RDT runs,
log_changes rev.428-430), so these fixtures are produced by the oracle, whose
building blocks are pinned by tests/test_oracle.py.  Inputs are not stored:
they come from the seeded generator sb_seed_state (seed, grid below).

usage: python tests/golden/make_golden.py [case ...]   (all cases without names)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import shear_nnf_gb300 as sb  # noqa: E402

LZ = 2 * np.pi
CASES = {
    # 64x32x32, Re_z = 1000, fixed dt 0.005 (the CPU-runnable configuration), 2 steps
    "step64_seed3": dict(params=dict(mgalx=64, my=32, mgalz=32, Re=1000.0 / LZ ** 2, alp=0.5,
                                     Ly=LZ, gam=1.0, s=1.0, chi=0.0, CFL=0.5, fixed_dt=0.005),
                         seed=3, nstep=2),
    # the same box with the Smagorinsky model at Re_z = 20000 (Cs = 0.1), CFL steps
    "les64_seed5": dict(params=dict(mgalx=64, my=32, mgalz=32, Re=20000.0 / LZ ** 2, alp=0.5,
                                    Ly=LZ, gam=1.0, s=1.0, chi=0.0, CFL=0.5, les=1, les_visc=1,
                                    cs=0.1), seed=5, nstep=3),
    # the compact y-filter (iydealiasing = 3) and the y 2/3 rule (iydealiasing = 1)
    "filt64_seed4": dict(params=dict(mgalx=64, my=32, mgalz=32, Re=4000.0 / LZ ** 2, alp=0.5,
                                     Ly=LZ, gam=1.0, s=1.0, chi=0.0, CFL=0.5, ydeal=3),
                         seed=4, nstep=3),
    "ydeal64_seed6": dict(params=dict(mgalx=64, my=32, mgalz=32, Re=4000.0 / LZ ** 2, alp=0.5,
                                      Ly=LZ, gam=1.0, s=1.0, chi=0.0, CFL=0.5, ydeal=1),
                          seed=6, nstep=3),
    # crosst: the scalar at Pr = 0.7 with a mean gradient and buoyancy, CFL steps
    "temp64_seed7": dict(params=dict(mgalx=64, my=32, mgalz=32, Re=4000.0 / LZ ** 2, alp=0.5,
                                     Ly=LZ, gam=1.0, s=1.0, chi=0.0, CFL=0.5, temperature=1,
                                     fkappa=LZ ** 2 / 4000.0 / 0.7, bym=1.0, gbeta=0.5),
                         seed=7, nstep=3),
    # the two-pair roll force with the window damping of the mean (iadd_force = 2,
    # iadd_damping = 1), CFL steps
    "force64_seed8": dict(params=dict(mgalx=64, my=32, mgalz=32, Re=4000.0 / LZ ** 2, alp=0.5,
                                      Ly=LZ, gam=1.0, s=1.0, chi=0.0, CFL=0.5, force=2,
                                      force_roll=0.05, damping=1, damp_up=0.5, damp_aa=0.1),
                          seed=8, nstep=3),
}


def main(names):
    for name, c in CASES.items():
        if names and name not in names:
            continue
        st = sb.seed_state(sb.make_params(**c["params"]), c["seed"])
        o = oracle.Oracle(**c["params"])
        tr, istop = o.cross(st, c["nstep"])
        extra = {"tb": st["tb"], "tb00": st["tb00"]} if "tb" in st else {}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), vor=st["vor"], phi=st["phi"],
                            u00=st["u00"], w00=st["w00"], time=st["time"], xoffb=st["xoffb"],
                            xofft=st["xofft"], trace=tr, seed=c["seed"], nstep=c["nstep"],
                            **extra, **{"p_" + k: v for k, v in c["params"].items()})
        print(name, "written")


if __name__ == "__main__":
    main(sys.argv[1:])
