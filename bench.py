"""Benchmark of the shearing-box RK3 step on GB300 (one JSON line on rank 0).

Workload: one box of 192x96x96 (Lx:Ly:Lz = 2:1:1, Lz = 2pi, S = 1,
Re_z = 4000, CFL = 0.5), FP64, seeded synthetic divergence-free field with
E(k) ~ k^4 exp(-2 (k/k0)^2), k0 = 4, u_rms = 0.1 S Lz.  A "step" is one RK3
step (three substeps) of that box.

  value  steps/s of K consecutive steps with the state resident in HBM
         (one sb_step call, CUDA events on the library's stream).
  e2e    steps/s through the C-ABI drop-in sb_cross(nstep=1) with pinned host
         buffers: host->device state, one step, device->host state, per step.
  roofline  the dominant kernel (plane stage 2), timed alone with CUDA events:
         FP64 rate against the FP64 FMA peak measured in the same run (the
         binding roof on GB300) and bytes against the measured HBM copy peak.
  les     Smagorinsky LES on 384x192x192 (Re_z=20000), FP32-mixed vs FP64.
  temperature  the crosst variant (Boussinesq scalar, Pr=0.7) on the benchmark
         box, FP64 and FP32-mixed, against the plain step.
  newton  batched Newton Jv/s: 32 finite-difference products on 96x48x48
         (Re_z=1200, T=20/S) as one FP32-mixed batch (central differences)
         vs one FP64 product at a time; the search of that configuration to
         |F|/|x| <= 1e-10 (unbatched FP64 and batched FP32-mixed, wall time)
         and the 20 leading Floquet multipliers by block Arnoldi.
  cpu_baseline  the C oracle (restatement of the reference step) on the
         host cores, a bounded sample of steps of the same workload.

--impl reference times that CPU oracle alone (the reference Fortran cannot be
built on this machine: no Fortran compiler, MPI, FFTW or HDF5).
Multi-GPU: each rank advances its own box (replicas, no communication).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK3 steps/s at 192x96x96 FP64 vs FP32-mixed (err vs FP64); batched Newton Jv/s"
GRID = (192, 96, 96)
GRIDS = {64: (64, 32, 32), 96: (96, 48, 48), 192: (192, 96, 96), 384: (384, 192, 192)}
REZ = 4000.0
LZ = 2 * np.pi


def box_params():
    return dict(mgalx=GRID[0], my=GRID[1], mgalz=GRID[2], Re=REZ / LZ ** 2, alp=0.5, Ly=LZ,
                gam=1.0, s=1.0, chi=0.0, CFL=0.5)


def config(extra=None):
    c = {"workload": "shearing box 192x96x96 (Lx:Ly:Lz=2:1:1, Lz=2pi), Re_z=4000, CFL=0.5, "
                     "1 box per GPU, FP64 RK3 step",
         "grid": list(GRID), "boxes_per_gpu": 1, "seed": 3, "k0": 4.0,
         "l2": "per-step working set ~156 MB (8 fields, transform buffers, line factors) "
               "> 129 MB L2; no flush"}
    if extra:
        c.update(extra)
    return c


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        # one GPU per rank over NCCL; gloo where no GPU is visible (host tests)
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        return dist, rank, ws
    return None, rank, ws


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int):
        self.dev = dev
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "10"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
            return
        # the timed region starts once sampling runs
        t0 = time.time()
        while not self.rows and time.time() - t0 < 3.0 and self.proc.poll() is None:
            time.sleep(0.01)
        self.rows.clear()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for q, nm in enumerate(names):
                if r[5 + q].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def plane2_traffic():
    """dram bytes per launch of plane stage 2 from the committed ncu summary
    (profiles/k_p2_192x96x96.txt, line 'traffic_bytes_per_launch: N'), else None."""
    path = os.path.join(ROOT, "profiles", "k_p2_192x96x96.txt")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":")[1])
    except OSError:
        pass
    return None


def cpu_baseline(nsteps_sample: int, threads: int, warmup: int = 1):
    """The C oracle on the host cores, a bounded sample of steps after
    `warmup` untimed ones.  Loads only the oracle: the seeded field comes from
    the oracle's own generator, which the CPU tests hold bit-identical to the
    library's."""
    import oracle
    oracle.set_threads(threads)
    pp = box_params()
    st = oracle.seed_state(seed=3, **pp)
    o = oracle.Oracle(**pp)
    o.cross(st, warmup)
    t0 = time.perf_counter()
    o.cross(st, nsteps_sample)
    dt = time.perf_counter() - t0
    return {"value": nsteps_sample / dt, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{nsteps_sample} consecutive FP64 steps of the 192x96x96 box "
                      f"(C oracle, OpenMP, {threads} threads), after {warmup} warm-up "
                      f"step{'s' if warmup != 1 else ''}",
            "seconds": dt}


def run_reference(args):
    dist, rank, ws = dist_setup()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = max(1, min(args.steps, 20))
    res = cpu_baseline(n, threads, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": "steps/s",
            "n_gpus": args.gpus, "steps": n, "warmup": args.warmup,
            "ms_per_step": 1e3 / res["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config({"impl": "CPU oracle (C restatement of the reference step)"}),
            "cpu_baseline": {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": res["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def ensemble_leg(sb, torch, dist, ws, rank, args, nbox=64, n_oracle=4):
    """Batched ensemble: 64 boxes of 64x32x32 (geometry of the 64^3/2 case),
    Re_z log-uniform in [500, 2000] and one seed per box, FP32-mixed, all boxes
    advanced by one graph-captured step per launch sequence, args.ens_steps
    steps.  Reports box-steps/s, the HBM rate of the algorithmic bytes (72
    complex fields per box-step, FP32 storage), the largest relative field
    error of a member against the same ensemble in FP64 on the GPU, and for
    the first n_oracle members the error of both against the oracle (FP64 on
    the host cores, the members' own Re and seeds)."""
    pp = dict(mgalx=64, my=32, mgalz=32, Re=1000.0 / LZ ** 2, alp=0.5, Ly=LZ, gam=1.0, s=1.0,
              chi=0.0, CFL=0.5)
    p = sb.make_params(**pp)
    nsteps = args.ens_steps
    rng = np.random.default_rng(1234 + rank)
    rez = np.exp(rng.uniform(np.log(500.0), np.log(2000.0), nbox))
    states = [sb.seed_state(p, 1000 * rank + m) for m in range(nbox)]
    boxes = {}
    for prec in (sb.SB_MIXED, sb.SB_FP64):
        box = sb.ShearBox(p, batch=nbox, precision=prec)
        for m in range(nbox):
            box.set_state(states[m], m)
            box.set_re(m, rez[m] / LZ ** 2)
        boxes[prec] = box
    box = boxes[sb.SB_MIXED]
    tuning = box.autotune()
    box.step(3)
    box.sync()
    for m in range(nbox):
        box.set_state(states[m], m)
    stream = torch.cuda.ExternalStream(box.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(dist)
    torch.cuda.synchronize()
    e0.record(stream)
    box.step(nsteps)
    e1.record(stream)
    e1.synchronize()
    ms = allmax(dist, e0.elapsed_time(e1))
    boxes[sb.SB_FP64].step(nsteps)
    keys = ("vor", "phi", "u00", "w00")

    def err(a, b):
        return max(float(np.linalg.norm(a[k] - b[k]) / np.linalg.norm(b[k])) for k in keys)

    finals = {prec: [bx.get_state(m) for m in range(nbox)] for prec, bx in boxes.items()}
    err_mixed_fp64 = max(err(finals[sb.SB_MIXED][m], finals[sb.SB_FP64][m]) for m in range(nbox))
    steps_done = [boxes[sb.SB_MIXED].status(m).steps_done for m in range(nbox)]
    vs_oracle = None
    if rank == 0 and n_oracle > 0:
        import oracle
        oracle.set_threads(os.cpu_count() or 1)
        e_mixed, e_fp64 = [], []
        for m in range(n_oracle):
            o = oracle.Oracle(**dict(pp, Re=rez[m] / LZ ** 2))
            st = oracle.seed_state(seed=1000 * rank + m, **pp)
            o.cross(st, nsteps)
            e_mixed.append(err(finals[sb.SB_MIXED][m], st))
            e_fp64.append(err(finals[sb.SB_FP64][m], st))
        vs_oracle = {"members": n_oracle, "max_mixed": max(e_mixed), "max_fp64": max(e_fp64),
                     "mixed": e_mixed, "fp64": e_fp64}
    sz = sb.sizes(p)
    alg_bytes = 72.0 * sz["n"] * 8 * nbox  # per batch step, FP32 storage (8 B per complex)
    hbm_peak, hbm_src = measured_peaks()
    gbs = alg_bytes * nsteps / (ms * 1e-3) / 1e9
    return {"boxes_per_gpu": nbox, "grid": [64, 32, 32], "steps": nsteps,
            "steps_done_min": int(min(steps_done)),
            "value": ws * nbox * nsteps / (ms * 1e-3), "unit": "box-steps/s",
            "ms_per_step": ms / nsteps, "precision": "FP32-mixed",
            "max_member_rel_l2_err_vs_fp64": err_mixed_fp64,
            "max_member_rel_l2_err_vs_oracle": vs_oracle["max_mixed"] if vs_oracle else None,
            "vs_oracle": vs_oracle, "re_z_range": [500.0, 2000.0],
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": gbs / hbm_peak, "peak_source": f"MEASURED_PEAKS.json ({hbm_src})",
                         "algorithmic_bytes_per_step": alg_bytes,
                         "note": "72 complex fields per box-step (4S + 8S + 12S per substep)"},
            "tuning": tuning}


def les_leg(sb, torch, dist, ws, rank, args):
    """LES mode: Smagorinsky eddy viscosity (Cs = 0.1, filter width
    (dx dy dz)^(1/3)) on 384x192x192, Re_z = 20000, k0 = 6, CFL = 0.5, from the
    seeded field to t = args.les_tend (default 2 = Lx/(S Ly), one shear-periodic
    remesh period; the CFL step makes that about 800 steps, so the leg runs up
    to args.les_steps steps and stops at that time), FP32-mixed against the
    same run in FP64 on the GPU: steps/s of both (CUDA events, state in HBM;
    steps done over the timed call), the time reached and the relative
    deviation of the velocity variances (u', v', w' rms), the Reynolds shear
    stress <uv> and the mean eddy viscosity of the last statistics record."""
    pp = dict(mgalx=384, my=192, mgalz=192, Re=20000.0 / LZ ** 2, alp=0.5, Ly=LZ, gam=1.0,
              s=1.0, chi=0.0, CFL=0.5, les=1, les_visc=1, cs=0.1)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 6 + rank, k0=6.0)
    n = args.les_steps
    out = {"grid": [384, 192, 192], "re_z": 20000.0, "cs": 0.1, "k0": 6.0, "max_steps": n,
           "t_end": args.les_tend}
    recs = {}
    for key, prec in (("mixed", sb.SB_MIXED), ("fp64", sb.SB_FP64)):
        box = sb.ShearBox(p, precision=prec)
        box.set_state(st0)
        box.step(3)
        box.sync()
        box.set_state(st0)
        box.set_etime(0, args.les_tend)
        stream = torch.cuda.ExternalStream(box.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier(dist)
        torch.cuda.synchronize()
        e0.record(stream)
        box.step(n)
        e1.record(stream)
        e1.synchronize()
        ms = allmax(dist, e0.elapsed_time(e1))
        st = box.status()
        tr = box.trace(0)
        recs[key] = tr
        done = st.steps_done
        out[key] = {"value": ws * done / (ms * 1e-3), "unit": "steps/s",
                    "ms_per_step": ms / max(done, 1), "time_span": st.time,
                    "steps_done": done, "reached_t_end": bool(st.flags & 8)}
        del box
    a, b = recs["mixed"][-1], recs["fp64"][-1]
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["rel_dev_vs_fp64_last_record"] = {
        "u_rms": float(abs(a[2] - b[2]) / abs(b[2])), "v_rms": float(abs(a[3] - b[3]) / abs(b[3])),
        "w_rms": float(abs(a[4] - b[4]) / abs(b[4])), "uv": float(abs(a[5] - b[5]) / abs(b[5])),
        "nu_t_mean": float(abs(a[22] - b[22]) / abs(b[22]))}
    out["remesh_period_St"] = (2 * np.pi / 0.5) / LZ
    out["spans_remesh"] = bool(out["mixed"]["time_span"] >= out["remesh_period_St"] - 1e-12 and
                               out["fp64"]["time_span"] >= out["remesh_period_St"] - 1e-12)
    out["precision"] = "FP32-mixed (FP64 y-solves, Helmholtz, phases)"
    return out


def temperature_leg(sb, torch, dist, ws, rank, args, plain_steps_per_s):
    """crosst: the benchmark box with the scalar (Pr = 0.7, bym = 1,
    gbeta = 0.5), args.steps steps with the state in HBM, FP64 and FP32-mixed
    (CUDA events); the cost against the plain FP64 step and the mixed run's
    deviation of tb from FP64 after those steps."""
    pp = dict(box_params(), temperature=1, fkappa=LZ ** 2 / REZ / 0.7, bym=1.0, gbeta=0.5)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 7 + rank)
    n = args.steps
    out = {"pr": 0.7, "bym": 1.0, "gbeta": 0.5, "steps": n}
    finals = {}
    for key, prec in (("fp64", sb.SB_FP64), ("mixed", sb.SB_MIXED)):
        box = sb.ShearBox(p, precision=prec)
        box.set_state(st0)
        tuning = box.autotune()
        box.set_state(st0)
        box.step(3)
        box.sync()
        box.set_state(st0)
        stream = torch.cuda.ExternalStream(box.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier(dist)
        torch.cuda.synchronize()
        e0.record(stream)
        box.step(n)
        e1.record(stream)
        e1.synchronize()
        ms = allmax(dist, e0.elapsed_time(e1))
        finals[key] = box.get_state()
        out[key] = {"value": ws * n / (ms * 1e-3), "unit": "steps/s", "ms_per_step": ms / n,
                    "tuning": tuning}
        del box
    out["fp64"]["cost_vs_plain_fp64"] = plain_steps_per_s / out["fp64"]["value"]
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    a, b = finals["mixed"]["tb"], finals["fp64"]["tb"]
    out["mixed"]["tb_rel_l2_err_vs_fp64"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return out


def newton_search_leg(sb, torch, dist, ws, rank, args, T=20.0, s_star=0.37, pert=1e-3):
    """The periodic-orbit search of the 96x48x48 configuration (Re_z = 1200,
    T = 20/S, streamwise shift unknown) run to |F|/|x| <= 1e-10, every vector
    on the device.  No orbit of this flow ships with the reference, so the
    search targets a manufactured relative periodic orbit of the configuration's
    own period map: x* = Phi_20(seeded field) (a developed state), s* = 0.37,
    F(x, s) = shift_s(Phi_T(x)) - x - r with r = shift_s*(Phi_T(x*)) - x*, from
    the start x* + 1e-3 |x*| (random direction), s* - 0.005.
      unbatched_fp64  the reference's algorithm: GMRES one product at a time
                      (k_gmres 50, eps_gmresk 1e-3, gmres_shear.f90:24-25,2099),
                      FP64 forward differences at eps_jacobi 1e-7, the base
                      taken from the residual's integration
      batched_mixed   block GMRES, 16 forward differences (eps_jacobi 1e-3) and
                      their base as one 17-member FP32-mixed batch per block,
                      at most 3 blocks per Newton step, each solve after the
                      first starting from 15 Ritz directions of the previous
                      one (deflated restarting)
    Both take their residuals from the same FP64 map.  Then block Arnoldi
    (4 blocks of 32 FP32-mixed forward differences) at the converged point
    gives the 20 leading multipliers of the shifted map's Jacobian, their
    Ritz residual estimates and the exponents log(lambda)/T."""
    from shear_nnf_gb300 import krylov as kr
    from shear_nnf_gb300 import newton as nw
    pp = dict(mgalx=96, my=48, mgalz=48, Re=1200.0 / LZ ** 2, alp=0.5, Ly=LZ, gam=1.0, s=1.0,
              chi=0.0, CFL=0.5)
    p = sb.make_params(**pp)
    sca = nw.Packing.reference_scales(p)
    pk = nw.Packing(p, *sca)
    n = pk.n
    ks = kr.KSpace(n + 1, 1400)
    res64 = kr.DevPeriodMap(p, T, batch=1, sca=sca, autotune=True)
    xs, rhs, x = ks.alloc(1), ks.alloc(1), ks.alloc(1)
    ks.set(xs, pk.pack(sb.seed_state(p, 77 + rank)))
    res64(ks, [xs], [xs])
    res64(ks, [xs], [rhs], shift=(s_star, 0.0))
    ks.combine(rhs, [rhs, xs], [1.0, -1.0], n)
    xsv = ks.get(xs, 0, n)
    d = np.random.default_rng(15 + rank).standard_normal(n)
    x0v = np.concatenate([xsv + pert * np.linalg.norm(xsv) / np.linalg.norm(d) * d, [0.0]])
    pm32 = kr.DevPeriodMap(p, T, batch=17, precision=sb.SB_MIXED, sca=sca, autotune=True)
    cfgs = (("unbatched_fp64", dict(jac=res64, block=1, k=50, eps=1e-7, base=False, recycle=0)),
            ("batched_mixed", dict(jac=pm32, block=16, k=3, eps=1e-3, base=True, recycle=15)))
    out = {"grid": [96, 48, 48], "re_z": 1200.0, "period_T": T, "unknowns": n + 1,
           "target": "manufactured relative periodic orbit (x*, s*) of the configuration's map",
           "start_rel_perturbation": pert, "tol": 1e-10}
    for key, c in cfgs:
        ks.set(x, x0v)
        barrier(dist)
        t0 = time.perf_counter()
        s, hist, st = kr.newton_rpo(ks, p, x, s_star - 0.005, res64, c["jac"], rhs=rhs, k=c["k"],
                                    block=c["block"], itmax=12, tol=1e-10, gmres_tol=1e-3,
                                    eps_jacobi=c["eps"], order=1, base_in_batch=c["base"],
                                    recycle=c["recycle"])
        secs = allmax(dist, time.perf_counter() - t0)
        out[key] = {"seconds": secs, "converged": bool(hist[-1] <= 1e-10),
                    "final_rel_residual": hist[-1], "history": hist, "shift": s,
                    "newton_iterations": st["newton"], "gmres_iterations": st["gmres_iterations"],
                    "products": st["products"], "fp64_residual_integrations": st["residuals"],
                    "block": c["block"], "eps_jacobi": c["eps"],
                    "precision_products": "FP64" if c["jac"] is res64 else "FP32-mixed"}
    a, b = out["unbatched_fp64"], out["batched_mixed"]
    out["speedup_batched_vs_unbatched_wall"] = a["seconds"] / b["seconds"]
    # Floquet analysis at the point the batched search converged to
    pmf = kr.DevPeriodMap(p, T, batch=33, precision=sb.SB_MIXED, sca=sca, autotune=True)
    J = kr.DevJacobian(pmf, ks, x, shift=(b["shift"], 0.0), eps_jacobi=1e-3, order=1,
                       base_in_batch=True)
    t0 = time.perf_counter()
    lam, rres, _ = kr.arnoldi_dev(ks, J.matvec, 4, block=32, rows=n, seed=5)
    ta = time.perf_counter() - t0
    top = lam[:20]
    out["floquet"] = {"multipliers_abs": [float(abs(v)) for v in top],
                      "multipliers_arg": [float(np.angle(v)) for v in top],
                      "exponents_re": [float(np.log(abs(v)) / T) for v in top],
                      "ritz_residual": [float(r) for r in rres[:20]],
                      "products": J.products, "seconds": ta,
                      "method": "block Arnoldi, 4 x 32 FP32-mixed forward differences "
                                "(eps_jacobi 1e-3), base in every batch"}
    del pm32, pmf, res64, ks
    return out


def newton_leg(sb, torch, dist, ws, rank, args, nper=32, T=20.0):
    """Batched Newton Jv: the Jacobian-vector products of the periodic-orbit
    search on 96x48x48 (Re_z=1200, period T=20/S) through the Newton tools'
    public API (host vectors in, host vectors out).
      batched         32 products as one 64-member FP32-mixed batch of central
                      differences (eps_jacobi=3e-3: FP32 storage does not
                      resolve the 1e-7 step of the FP64 search)
      batched_forward 32 forward differences and the base as one 33-member
                      FP32-mixed batch (eps_jacobi=1e-3)
      unbatched_fp64  one forward-difference product in FP64 at eps_jacobi=1e-7,
                      the base integration done beforehand
    Errors are relative L2 against the FP64 product of the same direction."""
    from shear_nnf_gb300 import newton as nw
    pp = dict(mgalx=96, my=48, mgalz=48, Re=1200.0 / LZ ** 2, alp=0.5, Ly=LZ, gam=1.0, s=1.0,
              chi=0.0, CFL=0.5)
    p = sb.make_params(**pp)
    pk = nw.Packing(p, *nw.Packing.reference_scales(p))
    x0 = pk.pack(sb.seed_state(p, 77 + rank))
    D = np.random.default_rng(5 + rank).standard_normal((pk.n, nper))
    pm64 = nw.PeriodMap(p, T, batch=1, chunk=256, autotune=True)
    J64 = nw.Jacobian(pm64, pk, x0, eps_jacobi=1e-7)
    J64.gx0  # the base integration, untimed
    steps_T = pm64.last_steps[0]
    barrier(dist)
    t0 = time.perf_counter()
    jv64 = J64.matvec(D[:, :1])
    t64 = allmax(dist, time.perf_counter() - t0)
    del pm64, J64
    out = {"grid": [96, 48, 48], "re_z": 1200.0, "period_T": T,
           "rk3_steps_per_integration": steps_T, "unknowns": pk.n,
           "unbatched_fp64": {"value": ws / t64, "unit": "Jv/s", "eps_jacobi": 1e-7,
                              "seconds": t64}}
    for key, central, eps, members in (("batched", True, 3e-3, 2 * nper),
                                       ("batched_forward", False, 1e-3, nper + 1)):
        pm = nw.PeriodMap(p, T, batch=members, precision=sb.SB_MIXED, chunk=256, autotune=True)
        J = nw.Jacobian(pm, pk, x0, eps_jacobi=eps, central=central, base_in_batch=not central)
        barrier(dist)
        t0 = time.perf_counter()
        jv = J.matvec(D)
        t = allmax(dist, time.perf_counter() - t0)
        out[key] = {"value": ws * nper / t, "unit": "Jv/s", "products_per_batch": nper,
                    "members": members, "difference": "central" if central else "forward",
                    "precision": "FP32-mixed", "eps_jacobi": eps, "seconds": t,
                    "jv_rel_l2_err_vs_fp64": float(np.linalg.norm(jv[:, 0] - jv64[:, 0]) /
                                                   np.linalg.norm(jv64[:, 0])),
                    "speedup_vs_unbatched_fp64": (nper / t) * t64}
        del pm, J
    out["api"] = "shear_nnf_gb300.newton.Jacobian.matvec (host vectors)"
    return out


def run_ours(args):
    import torch

    import shear_nnf_gb300 as sb
    dist, rank, ws = dist_setup()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    torch.cuda.init()
    # clocks over the whole run (all legs), beside those of the timed region
    run_clocks = ClockSampler(dev)
    if not args.lite and rank == 0:
        run_clocks.start()
    pp = box_params()
    if args.variant == "les":
        pp.update(les=1, les_visc=1, cs=0.1)
    elif args.variant == "temperature":
        pp.update(temperature=1, fkappa=LZ ** 2 / REZ / 0.7, bym=1.0, gbeta=0.5)
    elif args.variant == "implicit":
        pp.update(implicit_visc=1)
    elif args.variant == "implicit-temperature":
        pp.update(implicit_visc=1, temperature=1, fkappa=LZ ** 2 / REZ / 0.7, bym=1.0, gbeta=0.5)
    p = sb.make_params(**pp)
    st0 = sb.seed_state(p, 3 + rank)
    nbox = args.boxes if args.lite else 1
    box = sb.ShearBox(p, batch=nbox, precision=sb.SB_MIXED if args.mixed else sb.SB_FP64)
    states = [st0] + [sb.seed_state(p, 1000 * rank + m) for m in range(1, nbox)]
    rez = np.exp(np.random.default_rng(1234 + rank).uniform(np.log(500.0), np.log(2000.0), nbox))

    def load():
        for m in range(nbox):
            box.set_state(states[m], m)
            if nbox > 1:
                box.set_re(m, rez[m] / LZ ** 2)

    load()
    tuning = box.autotune()  # plane-stage tiles for this grid (untimed set-up)
    if args.line_segments:
        box.set_line_segments(args.line_segments)
    if args.line_form != "auto":
        box.set_line_form(args.line_form)
    tuning = box.tuning()
    load()
    stream = torch.cuda.ExternalStream(box.stream)
    # warm-up
    box.step(max(args.warmup, 1))
    box.sync()
    clocks = ClockSampler(dev)
    clocks.start()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    box.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    status = box.status()
    ms_max = allmax(dist, ms)
    steps_per_s = ws * args.steps / (ms_max * 1e-3)
    # per step: 3 substeps x (3 plane stages, scalars, tables, 2 line kernels),
    # the spectra and plane sums of the statistics at substep 1, the
    # end-of-step kernel; LES adds 5 per substep; the fused y-line form runs
    # one line kernel per substep instead of two; + 4 entry launches
    # (the implicit variant: k_hfac + k_lineI per substep in place of the two
    # line kernels)
    per_step = (39 if args.variant == "les" else 24) - (3 if tuning.get("line_form") == "fused"
                                                         else 0)
    if args.variant == "implicit-temperature":
        per_step += 3  # the scalar's factor tables
    launches = per_step * args.steps + 4
    if args.lite:
        # profiling runs (ncu): the timed steps only, no side measurements
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": steps_per_s, "unit": "steps/s",
                              "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": ms_max / args.steps, "lite": True,
                              "config": config({"workload": (
                                  f"shearing box {GRID[0]}x{GRID[1]}x{GRID[2]}, {nbox} box(es), "
                                  f"{'FP32-mixed' if args.mixed else 'FP64'} RK3 step, "
                                  f"variant {args.variant} (profiling run)"),
                                                "grid": list(GRID), "tuning": tuning,
                                                "variant": args.variant, "boxes": nbox,
                                                "precision": "mixed" if args.mixed else "fp64"}),
                              "gpu_launches": launches}))
        return
    # dominant kernel alone: plane stage 2 (x transforms + u x omega)
    box.set_state(st0)
    box.step(1)
    box.sync()
    nrep = 20
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    box.launch_stage(2, 2, 2)
    k0.record(stream)
    box.launch_stage(2, 2, nrep)
    k1.record(stream)
    k1.synchronize()
    p2_ms = k0.elapsed_time(k1) / nrep
    # line kernel alone, for the record
    box.set_state(st0)
    box.step(1)
    box.sync()
    k0.record(stream)
    box.launch_stage(5, 2, 5)
    k1.record(stream)
    k1.synchronize()
    line_ms = k0.elapsed_time(k1) / 5
    box.set_state(st0)
    box.step(1)
    box.sync()
    k0.record(stream)
    box.launch_stage(6, 2, 5)
    k1.record(stream)
    k1.synchronize()
    line_ms = (line_ms, k0.elapsed_time(k1) / 5)
    # the fused y-line kernel (the step's default form where available)
    lineF_ms = None
    if box.tuning()["line_form"] == "fused":
        box.set_state(st0)
        box.step(1)
        box.sync()
        k0.record(stream)
        box.launch_stage(12, 2, 5)
        k1.record(stream)
        k1.synchronize()
        lineF_ms = k0.elapsed_time(k1) / 5
    fp64_peak = box.fp64_peak()
    mgalx, my, mgalz = GRID
    nkx = 2 * (mgalx // 3) // 2
    # algorithmic work of plane stage 2 per launch: 9 complex FFTs of length
    # mgalx per pair of z rows (5 N log2 N flops each), 12 flops per point of
    # the cross product, per plane; bytes: read 6 and write 3 fields of
    # (mgalz x nkx) complex per plane
    fft_fl = 9 * 5 * mgalx * np.log2(mgalx) * (mgalz // 2)
    prod_fl = 12 * mgalx * mgalz
    p2_flops = my * (fft_fl + prod_fl)
    p2_bytes = my * mgalz * nkx * 16 * (6 + 3)
    hbm_peak, hbm_src = measured_peaks()
    p2_tflops = p2_flops / (p2_ms * 1e-3) / 1e12
    p2_gbs = p2_bytes / (p2_ms * 1e-3) / 1e9
    traffic = plane2_traffic()
    # end to end through the drop-in with pinned host buffers
    nf = st0["vor"].size
    pin = {}
    for key in ("vor", "phi"):
        t = torch.empty(2 * nf, dtype=torch.float64, pin_memory=True)
        a = t.numpy().view(np.complex128).reshape(st0[key].shape)
        a[...] = st0[key]
        pin[key] = (t, a)
    host = {"vor": pin["vor"][1], "phi": pin["phi"][1]}
    for key in ("u00", "w00"):
        t = torch.empty(my, dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = st0[key]
        pin[key] = (t, t.numpy())
        host[key] = t.numpy()
    host.update(time=0.0, xoffb=0.0, xofft=0.0)
    ne2e = max(3, min(args.steps, 20))
    box.cross(host, 1)  # warm-up
    torch.cuda.synchronize()
    barrier(dist)
    calls = []
    t0 = time.perf_counter()
    for _ in range(ne2e):
        c0 = time.perf_counter()
        box.cross(host, 1)
        calls.append(time.perf_counter() - c0)
    t1 = time.perf_counter()
    barrier(dist)
    e2e_s = allmax(dist, t1 - t0)
    calls_ms = 1e3 * np.array(calls)
    bytes_io = 2 * nf * 16 + 2 * my * 8 + 3 * 8
    # FP32-mixed precision form: same workload, steps/s, and the field error
    # against the FP64 path at steps 1, 10, 100, 200 from the same initial field
    mixed = None
    if not args.no_mixed:
        mbox = sb.ShearBox(p, precision=sb.SB_MIXED)
        mbox.set_state(st0)
        mtuning = mbox.autotune()
        mbox.set_state(st0)
        mbox.step(max(args.warmup, 1))
        mbox.sync()
        mstream = torch.cuda.ExternalStream(mbox.stream)
        m0 = torch.cuda.Event(enable_timing=True)
        m1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        m0.record(mstream)
        mbox.step(args.steps)
        m1.record(mstream)
        m1.synchronize()
        mixed_ms = allmax(dist, m0.elapsed_time(m1))
        # the same marks for the FP64 GPU path against the oracle (the drop-in
        # bar: 1e-12 after one step, 1e-9 after 100); the oracle runs on the
        # host cores from the oracle's own seeded field
        errs, errs64 = {}, {}
        ref_box = box
        ref_box.set_state(st0)
        mbox.set_state(st0)
        orc = orc_st = None
        if rank == 0 and not args.no_oracle_table:
            import oracle
            oracle.set_threads(os.cpu_count() or 1)
            orc = oracle.Oracle(**pp)
            orc_st = oracle.seed_state(seed=3, **pp)
        done = 0
        for mark in (1, 10, 100, 200):
            ref_box.step(mark - done)
            mbox.step(mark - done)
            a = ref_box.get_state()
            b = mbox.get_state()
            errs[str(mark)] = max(float(np.linalg.norm(b[k] - a[k]) / np.linalg.norm(a[k]))
                                  for k in ("vor", "phi", "u00", "w00"))
            if orc is not None:
                orc.cross(orc_st, mark - done)
                errs64[str(mark)] = max(
                    float(np.linalg.norm(a[k] - orc_st[k]) / np.linalg.norm(orc_st[k]))
                    for k in ("vor", "phi", "u00", "w00"))
            done = mark
        del mbox
        mixed = {"value": ws * args.steps / (mixed_ms * 1e-3), "unit": "steps/s",
                 "ms_per_step": mixed_ms / args.steps,
                 "speedup_vs_fp64": (ws * args.steps / (mixed_ms * 1e-3)) / steps_per_s,
                 "rel_l2_err_vs_fp64_at_step": errs,
                 "fp64_rel_l2_err_vs_oracle_at_step": errs64 or None,
                 "precision": "FP32 storage, transforms, nonlinear product and RK3; FP64 "
                              "compact y-solves, Helmholtz solve, phase factors",
                 "tuning": mtuning}
    ensemble = None if args.no_ensemble else ensemble_leg(sb, torch, dist, ws, rank, args)
    newton = None if args.no_newton else newton_leg(sb, torch, dist, ws, rank, args)
    if newton is not None and not args.no_search:
        newton["search"] = newton_search_leg(sb, torch, dist, ws, rank, args)
    les = None if args.no_les else les_leg(sb, torch, dist, ws, rank, args)
    temp = (None if args.no_temp else
            temperature_leg(sb, torch, dist, ws, rank, args, steps_per_s))
    if rank != 0:
        return
    cpu = cpu_baseline(args.cpu_steps, os.cpu_count() or 1) if ws == 1 or rank == 0 else None
    line = {
        "metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded k^4 exp(-2(k/k0)^2) spectrum; no dataset in the reference)",
        "config": config({"parallelism": f"replicas x{ws}", "tuning": tuning, "mcell_steps_per_s":
                          steps_per_s * mgalx * my * mgalz / 1e6,
                          "status_after": {"istop": status.istop, "steps_done": status.steps_done,
                                           "time": status.time}}),
        "e2e": {"value": ws * ne2e / e2e_s, "unit": "steps/s",
                "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                "api": "sb_cross(nstep=1), pinned host buffers",
                "per_call_ms": {"median": float(np.median(calls_ms)), "min": float(calls_ms.min()),
                                "max": float(calls_ms.max())}},
        "gpu_launches": launches,
        "roofline": {
            "bound": "fp64", "kernel": "k_p2 (plane stage 2: x transforms, u x omega)",
            "achieved": p2_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": p2_tflops / fp64_peak,
            "peak_source": "FP64 FMA probe measured in this run (GB300 FP64 is the binding roof)",
            "algorithmic_flops_per_launch": p2_flops, "launch_ms": p2_ms,
            "hbm": {"achieved": p2_gbs, "peak": hbm_peak, "unit": "GB/s",
                    "frac": p2_gbs / hbm_peak, "peak_source": f"MEASURED_PEAKS.json ({hbm_src})",
                    "algorithmic_bytes_per_launch": p2_bytes},
            "traffic": traffic,
            "line_kernels_ms": {"k_lineA": line_ms[0], "k_lineB": line_ms[1], "k_lineF": lineF_ms},
        },
        "mixed_value": mixed["value"] if mixed else None,
        "mixed_speedup": mixed["speedup_vs_fp64"] if mixed else None,
        "mixed": mixed,
        "ensemble": ensemble,
        "newton": newton,
        "les": les,
        "temperature": temp,
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "clocks": clk,
        "clocks_all_legs": run_clocks.stop(),
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--grid", type=int, default=192, choices=sorted(GRIDS),
                    help="profiling only: run a different grid (the benchmark is 192)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the FP32-mixed leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble leg")
    ap.add_argument("--no-newton", action="store_true", help="skip the batched Newton Jv leg")
    ap.add_argument("--no-search", action="store_true",
                    help="skip the Newton search and Floquet analysis of the newton leg")
    ap.add_argument("--no-les", action="store_true", help="skip the LES leg")
    ap.add_argument("--les-steps", type=int, default=1000,
                    help="most steps of the LES leg (it stops at t = 2, one remesh period)")
    ap.add_argument("--les-tend", type=float, default=2.0,
                    help="end time of the LES leg (the remesh period Lx/(S Ly) = 2)")
    ap.add_argument("--ens-steps", type=int, default=1000, help="steps of the ensemble leg")
    ap.add_argument("--no-oracle-table", action="store_true",
                    help="skip the FP64-vs-oracle error table of the mixed leg")
    ap.add_argument("--no-temp", action="store_true", help="skip the temperature (crosst) leg")
    ap.add_argument("--lite", action="store_true",
                    help="profiling only: time the steps, skip e2e / CPU / per-kernel legs")
    ap.add_argument("--variant", default="plain",
                    choices=["plain", "les", "temperature", "implicit", "implicit-temperature"],
                    help="profiling only (with --lite): step the LES, temperature or semi-implicit box")
    ap.add_argument("--boxes", type=int, default=1,
                    help="profiling only (with --lite): boxes in the batch (Re_z log-uniform "
                         "in [500, 2000] beyond the first)")
    ap.add_argument("--mixed", action="store_true",
                    help="profiling only (with --lite): the FP32-mixed precision form")
    ap.add_argument("--line-form", default="auto", choices=["auto", "fused", "split"],
                    help="profiling only (with --lite): the y-line kernels after the autotuner")
    ap.add_argument("--line-segments", type=int, default=0,
                    help="profiling only (with --lite): warps per y-line solve after the autotuner")
    args = ap.parse_args()
    if (args.variant != "plain" or args.boxes != 1 or args.mixed or args.line_form != "auto"
            or args.line_segments) and not args.lite:
        ap.error("--variant, --boxes, --mixed, --line-form and --line-segments are for "
                 "profiling runs (--lite)")
    global GRID
    GRID = GRIDS[args.grid]
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
