"""GB300 shearing-box RK3 time stepper (Python host over the C-ABI).

The product is the CUDA library ``_build/libshearbox.so`` with the C interface
of ``include/shearbox.h``; this module is a thin ctypes host that mirrors the
reference's ``cross`` interface (cross.f90:3-4): state in the reference pencil
layout (complex (mz, nkx, my), y fastest), parameters of hre2.dat, and the
``.cfbin`` statistics record.  There is no CPU fallback: importing works
without a GPU, but creating a ``ShearBox`` fails loudly if the CUDA library or
a GPU is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .buildlib import LIB, build

TRACE_LEN = 24
TRACE_FIELDS = (
    ["time", "Deltat"] + [f"uner{q}" for q in range(1, 11)] + ["CFL", "CFLv", "umax1", "umax2",
    "umax3", "xoffb", "xofft", "umax0"] + [f"uner2_{q}" for q in range(1, 5)]
)
# crosst appends tbmax and tner(1:4) (crosst.f90:2456-2458)
TRACE_LEN_T = 29
TRACE_FIELDS_T = TRACE_FIELDS + ["tbmax"] + [f"tner{q}" for q in range(1, 5)]
SB_FP64 = 0
SB_MIXED = 1


class SbParams(ctypes.Structure):
    _fields_ = [
        ("mgalx", ctypes.c_int), ("my", ctypes.c_int), ("mgalz", ctypes.c_int),
        ("Re", ctypes.c_double), ("alp", ctypes.c_double), ("Ly", ctypes.c_double),
        ("gam", ctypes.c_double), ("s", ctypes.c_double), ("chi", ctypes.c_double),
        ("CFL", ctypes.c_double), ("vbulk", ctypes.c_double), ("fixed_dt", ctypes.c_double),
        ("readflag", ctypes.c_int), ("uprim", ctypes.c_double), ("nhist", ctypes.c_int),
        ("etime", ctypes.c_double), ("dumptime", ctypes.c_double), ("dtimag", ctypes.c_double),
        ("keep_laminar", ctypes.c_int), ("les", ctypes.c_int), ("les_visc", ctypes.c_int),
        ("cs", ctypes.c_double), ("ydeal", ctypes.c_int),
        ("temperature", ctypes.c_int), ("fkappa", ctypes.c_double), ("bym", ctypes.c_double),
        ("gbeta", ctypes.c_double),
        ("damping", ctypes.c_int), ("damp_up", ctypes.c_double), ("damp_aa", ctypes.c_double),
        ("force", ctypes.c_int), ("force_roll", ctypes.c_double), ("xforce", ctypes.c_double),
        ("implicit_visc", ctypes.c_int),
    ]


RESTART_MAXOPT = 32


class SbRestartInfo(ctypes.Structure):
    _fields_ = [
        ("mgalx", ctypes.c_int), ("my", ctypes.c_int), ("mgalz", ctypes.c_int),
        ("numerop", ctypes.c_int),
        ("time", ctypes.c_double), ("Re", ctypes.c_double), ("alp", ctypes.c_double),
        ("Ly", ctypes.c_double), ("gam", ctypes.c_double), ("s", ctypes.c_double),
        ("chi", ctypes.c_double),
        ("mx", ctypes.c_int), ("mye", ctypes.c_int), ("mz", ctypes.c_int),
        ("xoffb", ctypes.c_double), ("xofft", ctypes.c_double), ("zoffb", ctypes.c_double),
        ("zofft", ctypes.c_double),
        ("CFL", ctypes.c_double), ("uprim", ctypes.c_double), ("vbulk", ctypes.c_double),
        ("xforce", ctypes.c_double),
        ("has_footer", ctypes.c_int), ("irev", ctypes.c_int), ("nopt", ctypes.c_int),
        ("nparams", ctypes.c_int),
        ("options", ctypes.c_int * RESTART_MAXOPT), ("params", ctypes.c_double * RESTART_MAXOPT),
        ("run_xoffb", ctypes.c_double), ("run_xofft", ctypes.c_double),
        ("ymap", ctypes.c_int), ("ncopy", ctypes.c_int), ("xskip", ctypes.c_int),
    ]


RESTART_KEEP_VOR = 1


class SbStatus(ctypes.Structure):
    _fields_ = [
        ("istop", ctypes.c_int), ("steps_done", ctypes.c_int), ("ntrace", ctypes.c_int),
        ("flags", ctypes.c_int), ("time", ctypes.c_double), ("deltat", ctypes.c_double),
        ("xoffb", ctypes.c_double), ("xofft", ctypes.c_double), ("cfl", ctypes.c_double),
        ("cflv", ctypes.c_double),
    ]


ABI_FUNCTIONS = [
    "sb_create", "sb_destroy", "sb_set_member_re", "sb_set_state", "sb_get_state", "sb_step",
    "sb_get_status", "sb_get_trace", "sb_cross", "sb_get_stream", "sb_sync", "sb_sizes",
    "sb_seed_state", "sb_compact_coeffs", "sb_last_error", "sb_version", "sb_launch_stage",
    "sb_fp64_peak", "sb_op_derivyc", "sb_op_lapcdy", "sb_op_derivyc_noalloc",
    "sb_set_member_etime", "sb_op_filterc", "sb_op_cfty", "sb_op_rfty", "sb_write_restart",
    "sb_read_restart", "sb_autotune", "sb_physical_fields", "sb_set_temperature",
    "sb_get_temperature", "sb_crosst", "sb_stats", "sb_jv_batch", "sb_get_statistics",
    "sb_fft_twiddles", "sb_packed_length", "sb_set_state_packed", "sb_get_state_packed",
    "sb_packed_shift_tangent",
    "sb_kspace_create", "sb_kspace_destroy", "sb_kspace_col", "sb_kspace_stream",
    "sb_kspace_sync", "sb_kspace_gram", "sb_kspace_update", "sb_kspace_transform",
    "sb_kspace_combine", "sb_kspace_perturb", "sb_kspace_fd", "sb_kspace_set", "sb_kspace_get",
    "sb_read_restart_ex", "sb_get_tuning", "sb_set_line_segments", "sb_set_line_form",
    "sb_get_line_form", "sb_set_side_branch", "sb_get_side_branch",
]

_lib = None


def lib(auto_build: bool = False):
    """Load the CUDA library (building it first only if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    if auto_build:
        build()
    if not os.path.exists(LIB):
        raise RuntimeError(f"CUDA library {LIB} is missing: run __graft_entry__.build()")
    L = ctypes.CDLL(LIB)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    PP = ctypes.POINTER(SbParams)
    L.sb_create.argtypes = [PP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
    L.sb_destroy.argtypes = [vp]
    L.sb_set_member_re.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    L.sb_set_member_etime.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    L.sb_set_state.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double]
    L.sb_get_state.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp]
    L.sb_step.argtypes = [vp, ctypes.c_int]
    L.sb_get_status.argtypes = [vp, ctypes.c_int, ctypes.POINTER(SbStatus)]
    L.sb_get_trace.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, ip]
    L.sb_cross.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int, ctypes.POINTER(SbStatus)]
    L.sb_crosst.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int,
                            ctypes.POINTER(SbStatus)]
    L.sb_set_temperature.argtypes = [vp, ctypes.c_int, dp, dp]
    L.sb_stats.argtypes = [vp, ctypes.c_int, dp, dp]
    L.sb_get_statistics.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp, dp, dp, ip, dp]
    L.sb_jv_batch.argtypes = [vp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                              ctypes.c_double, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                              dp]
    L.sb_get_temperature.argtypes = [vp, ctypes.c_int, dp, dp]
    L.sb_get_stream.restype = vp
    L.sb_get_stream.argtypes = [vp]
    L.sb_sync.argtypes = [vp]
    L.sb_sizes.argtypes = [PP, ip]
    L.sb_fft_twiddles.argtypes = [ctypes.c_int, ctypes.c_int, dp]
    L.sb_seed_state.argtypes = [PP, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double, dp, dp,
                                dp, dp]
    L.sb_compact_coeffs.argtypes = [dp, dp, dp, dp]
    L.sb_last_error.restype = ctypes.c_char_p
    L.sb_last_error.argtypes = []
    L.sb_version.argtypes = []
    L.sb_launch_stage.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.sb_fp64_peak.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.sb_autotune.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.sb_get_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.sb_set_line_segments.argtypes = [vp, ctypes.c_int]
    L.sb_set_line_form.argtypes = [vp, ctypes.c_int]
    L.sb_get_line_form.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.sb_set_side_branch.argtypes = [vp, ctypes.c_int]
    L.sb_get_side_branch.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.sb_physical_fields.argtypes = [vp, ctypes.c_int, ctypes.c_uint, dp]
    L.sb_op_derivyc.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, vp,
                                ctypes.c_long, vp, ctypes.c_long, dp, dp, vp]
    L.sb_op_derivyc_noalloc.argtypes = list(L.sb_op_derivyc.argtypes)
    L.sb_op_lapcdy.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, vp, ctypes.c_long, vp,
                               ctypes.c_long, dp, dp, dp, vp]
    L.sb_op_filterc.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_long, vp, ctypes.c_long,
                                dp, vp]
    L.sb_op_cfty.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_long, ctypes.c_int, vp]
    L.sb_op_rfty.argtypes = list(L.sb_op_cfty.argtypes)
    L.sb_write_restart.argtypes = [ctypes.c_char_p, ctypes.POINTER(SbParams), dp, dp, dp, dp,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double]
    L.sb_read_restart.argtypes = [ctypes.c_char_p, ctypes.POINTER(SbParams), dp, dp, dp, dp,
                                  ctypes.POINTER(SbRestartInfo)]
    L.sb_read_restart_ex.argtypes = [ctypes.c_char_p, ctypes.POINTER(SbParams), ctypes.c_int, dp,
                                     dp, dp, dp, ctypes.POINTER(SbRestartInfo)]
    L.sb_packed_length.restype = ctypes.c_long
    L.sb_packed_length.argtypes = [vp]
    L.sb_set_state_packed.argtypes = [vp, ctypes.c_int, vp, dp, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double]
    L.sb_get_state_packed.argtypes = [vp, ctypes.c_int, vp, dp, ctypes.c_double, ctypes.c_double]
    L.sb_packed_shift_tangent.argtypes = [vp, vp, vp, ctypes.c_int]
    lg = ctypes.c_long
    L.sb_kspace_create.argtypes = [lg, ctypes.c_int, vp, ctypes.POINTER(vp)]
    L.sb_kspace_destroy.argtypes = [vp]
    L.sb_kspace_col.restype = vp
    L.sb_kspace_col.argtypes = [vp, ctypes.c_int]
    L.sb_kspace_stream.restype = vp
    L.sb_kspace_stream.argtypes = [vp]
    L.sb_kspace_sync.argtypes = [vp]
    L.sb_kspace_gram.argtypes = [vp, lg, lg, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, dp]
    L.sb_kspace_update.argtypes = [vp, lg, lg, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, dp, ctypes.c_double]
    L.sb_kspace_transform.argtypes = [vp, lg, lg, ctypes.c_int, ctypes.c_int, dp]
    L.sb_kspace_combine.argtypes = [vp, lg, lg, ctypes.c_int, ctypes.c_int, ip, dp]
    L.sb_kspace_perturb.argtypes = [vp, lg, lg, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double]
    L.sb_kspace_fd.argtypes = [vp, lg, lg, ctypes.c_int, ctypes.c_int, ip, ctypes.c_double]
    L.sb_kspace_set.argtypes = [vp, ctypes.c_int, lg, lg, dp]
    L.sb_kspace_get.argtypes = [vp, ctypes.c_int, lg, lg, dp]
    _lib = L
    return L


class ShearBoxError(RuntimeError):
    pass


def _check(rc: int):
    if rc != 0:
        raise ShearBoxError(f"shearbox error {rc}: {lib().sb_last_error().decode()}")


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(mgalx, my, mgalz, Re, alp, Ly, gam, s=1.0, chi=0.0, CFL=0.5, vbulk=0.0,
                fixed_dt=0.0, readflag=1, uprim=1.0, nhist=1, etime=1e10, dumptime=1e10,
                dtimag=1e10, keep_laminar=0, les=0, les_visc=1, cs=0.1, ydeal=0, temperature=0,
                fkappa=0.0, bym=0.0, gbeta=0.0, damping=0, damp_up=0.0, damp_aa=0.0, force=0,
                force_roll=0.0, xforce=0.0, implicit_visc=0) -> SbParams:
    return SbParams(mgalx, my, mgalz, Re, alp, Ly, gam, s, chi, CFL, vbulk, fixed_dt, readflag,
                    uprim, nhist, etime, dumptime, dtimag, keep_laminar, les, les_visc, cs, ydeal,
                    temperature, fkappa, bym, gbeta, damping, damp_up, damp_aa, force,
                    force_roll, xforce, implicit_visc)


def sizes(p: SbParams) -> dict:
    out = (ctypes.c_int * 8)()
    _check(lib().sb_sizes(ctypes.byref(p), out))
    keys = ["mx", "mz", "nkx", "my", "nz", "mgalx", "mgalz", "n"]
    return dict(zip(keys, list(out)))


def fft_twiddles(n: int, factored: bool = True) -> np.ndarray:
    """The device's twiddle table for transforms of length n (sb_fft_twiddles):
    factored: (n, 4) rows {mx, my, tau, swap bits}; else (n,) complex."""
    out = np.zeros(4 * n if factored else 2 * n)
    _check(lib().sb_fft_twiddles(int(n), 1 if factored else 0, _dp(out)))
    return out.reshape(n, 4) if factored else out.view(np.complex128)


def _seed_fields(p: SbParams, seed: int, k0: float, urms: float):
    sz = sizes(p)
    vor = np.zeros((sz["mz"], sz["nkx"], p.my), np.complex128)
    phi = np.zeros_like(vor)
    u00 = np.zeros(p.my)
    w00 = np.zeros(p.my)
    _check(lib().sb_seed_state(ctypes.byref(p), int(seed), float(k0), float(urms),
                               _dp(vor.view(np.float64)), _dp(phi.view(np.float64)), _dp(u00),
                               _dp(w00)))
    return vor, phi, u00, w00


def seed_state(p: SbParams, seed: int, k0: float = 4.0, urms: float = None) -> dict:
    """Seeded divergence-free initial field (pencil layout, complex128).  With
    the temperature also a seeded scalar: tb from the omega_y of a second seed
    scaled by 1/k0 (fluctuations of order urms) and tb00 from its u00."""
    if urms is None:
        urms = 0.1 * 1.0 * (2 * np.pi / p.gam)  # 0.1 * S * Lz
    vor, phi, u00, w00 = _seed_fields(p, seed, k0, urms)
    st = {"vor": vor, "phi": phi, "u00": u00, "w00": w00, "time": 0.0, "xoffb": 0.0,
          "xofft": 0.0}
    if p.temperature:
        tv, _, t00, _ = _seed_fields(p, (int(seed) * 7919 + 17) & 0xFFFFFFFF, k0, urms)
        st["tb"] = np.ascontiguousarray(tv / k0)
        st["tb00"] = t00
    return st


def compact_coeffs():
    a = [np.zeros(7) for _ in range(4)]
    _check(lib().sb_compact_coeffs(*[_dp(x) for x in a]))
    return tuple(a)


class ShearBox:
    """A batch of shearing boxes resident on the GPU."""

    def __init__(self, p: SbParams, batch: int = 1, precision: int = SB_FP64):
        self.p = p
        self.batch = batch
        self.sz = sizes(p)
        h = ctypes.c_void_p()
        _check(lib().sb_create(ctypes.byref(p), int(batch), int(precision), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().sb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(lib().sb_get_stream(self.h) or 0)

    def set_re(self, member: int, Re: float):
        _check(lib().sb_set_member_re(self.h, member, float(Re)))

    def set_etime(self, member: int, etime: float):
        _check(lib().sb_set_member_etime(self.h, member, float(etime)))

    def set_state(self, state: dict, member: int = 0):
        """Copies a state in; with the temperature the keys tb and tb00 are
        required."""
        if self.p.temperature:
            tb = np.ascontiguousarray(state["tb"], np.complex128)
            tb00 = np.ascontiguousarray(state["tb00"], np.float64)
            _check(lib().sb_set_temperature(self.h, member, _dp(tb.view(np.float64)), _dp(tb00)))
        vor = np.ascontiguousarray(state["vor"], np.complex128)
        phi = np.ascontiguousarray(state["phi"], np.complex128)
        u00 = np.ascontiguousarray(state["u00"], np.float64)
        w00 = np.ascontiguousarray(state["w00"], np.float64)
        _check(lib().sb_set_state(self.h, member, _dp(vor.view(np.float64)),
                                  _dp(phi.view(np.float64)), _dp(u00), _dp(w00),
                                  float(state["time"]), float(state["xoffb"]),
                                  float(state["xofft"])))

    def get_state(self, member: int = 0) -> dict:
        vor = np.zeros((self.sz["mz"], self.sz["nkx"], self.p.my), np.complex128)
        phi = np.zeros_like(vor)
        u00 = np.zeros(self.p.my)
        w00 = np.zeros(self.p.my)
        t = ctypes.c_double()
        xb = ctypes.c_double()
        xt = ctypes.c_double()
        _check(lib().sb_get_state(self.h, member, _dp(vor.view(np.float64)),
                                  _dp(phi.view(np.float64)), _dp(u00), _dp(w00), ctypes.byref(t),
                                  ctypes.byref(xb), ctypes.byref(xt)))
        st = {"vor": vor, "phi": phi, "u00": u00, "w00": w00, "time": t.value,
              "xoffb": xb.value, "xofft": xt.value}
        if self.p.temperature:
            tb = np.zeros_like(vor)
            tb00 = np.zeros(self.p.my)
            _check(lib().sb_get_temperature(self.h, member, _dp(tb.view(np.float64)), _dp(tb00)))
            st["tb"], st["tb00"] = tb, tb00
        return st

    def launch_stage(self, stage: int, rk: int = 1, count: int = 1):
        _check(lib().sb_launch_stage(self.h, int(stage), int(rk), int(count)))

    PHYSICAL = ("u", "v", "w", "ox", "oy", "oz", "Q", "R", "Qs", "Rs", "Qw")

    def physical(self, member: int = 0, fields=PHYSICAL) -> dict:
        """convh5 physical fields of a member's state: {name: (my, mgalz, mgalx)}."""
        mask = 0
        for f in fields:
            mask |= 1 << self.PHYSICAL.index(f)
        names = [f for f in self.PHYSICAL if mask >> self.PHYSICAL.index(f) & 1]
        out = np.zeros((len(names), self.p.my, self.p.mgalz, self.p.mgalx))
        _check(lib().sb_physical_fields(self.h, int(member), mask, _dp(out)))
        return dict(zip(names, out))

    def autotune(self) -> dict:
        """Picks the fastest plane-stage tiles, y-line tile (warps per line
        solve) and y-line form on the current state (keep the state set before
        calling); returns the choice."""
        _check(lib().sb_autotune(self.h, None))
        return self.tuning()

    def tuning(self) -> dict:
        """The current tiles (sb_get_tuning) and y-line form
        (sb_get_line_form: "fused" or "split")."""
        c = (ctypes.c_int * 4)()
        _check(lib().sb_get_tuning(self.h, c))
        f = ctypes.c_int(0)
        _check(lib().sb_get_line_form(self.h, ctypes.byref(f)))
        m = ctypes.c_int(0)
        _check(lib().sb_get_side_branch(self.h, ctypes.byref(m)))
        return {"p1_cols": c[0], "p3_cols": c[1], "p2_threads": c[2], "line_segments": c[3],
                "line_form": ("split", "fused", "implicit")[f.value], "side_branch": m.value}

    def set_line_segments(self, nseg: int):
        """Warps per y-line solve, 1..3 (sb_set_line_segments)."""
        _check(lib().sb_set_line_segments(self.h, int(nseg)))

    def set_line_form(self, form: str):
        """The y-line kernels of a substep: "fused" (one kernel; handles
        without temperature or y filter/dealiasing) or "split"
        (sb_set_line_form)."""
        if form not in ("fused", "split"):
            raise ValueError(f"line form {form!r}: 'fused' or 'split'")
        _check(lib().sb_set_line_form(self.h, 1 if form == "fused" else 0))

    def set_side_branch(self, mask: int):
        """Side work run as concurrent branches of the step graph: bit 0 the
        spectra, bit 1 the scalars and tables; 0 runs all of it in order
        (sb_set_side_branch)."""
        _check(lib().sb_set_side_branch(self.h, int(mask)))

    def statistics(self, member: int = 0) -> dict:
        """The hist accumulators of the last step call (sb_get_statistics):
        stats, stats2 (my, 23), spec, spec2 (mz, nkx, 8), with the temperature
        tstats (my, 5) and tspec (mz, nkx, 4), nacum, total_dt."""
        my, nkx, mz = self.p.my, self.sz["nkx"], self.sz["mz"]
        out = {"stats": np.zeros((my, 23)), "stats2": np.zeros((my, 23)),
               "spec": np.zeros((mz, nkx, 8)), "spec2": np.zeros((mz, nkx, 8))}
        if self.p.temperature:
            out["tstats"], out["tspec"] = np.zeros((my, 5)), np.zeros((mz, nkx, 4))
        n = ctypes.c_int(0)
        t = ctypes.c_double(0.0)
        ptr = [(_dp(out[k]) if k in out else None)
               for k in ("stats", "stats2", "spec", "spec2", "tstats", "tspec")]
        _check(lib().sb_get_statistics(self.h, int(member), *ptr, ctypes.byref(n), ctypes.byref(t)))
        out["nacum"], out["total_dt"] = n.value, t.value
        return out

    def stats(self, member: int = 0):
        """(uner[10], uner2[4]) of the member's last statistics record."""
        u, u2 = np.zeros(10), np.zeros(4)
        _check(lib().sb_stats(self.h, int(member), _dp(u), _dp(u2)))
        return u, u2

    def state_vector(self, st: dict) -> np.ndarray:
        """A state as the flat [vor | phi | u00 | w00] vector of sb_jv_batch."""
        return np.concatenate([np.ascontiguousarray(st["vor"], np.complex128).view(np.float64).ravel(),
                               np.ascontiguousarray(st["phi"], np.complex128).view(np.float64).ravel(),
                               np.asarray(st["u00"], np.float64), np.asarray(st["w00"], np.float64)])

    def jv_batch(self, x0: np.ndarray, dirs: np.ndarray, T: float, eps_jacobi: float = 1e-7,
                 central: bool = False, time0: float = 0.0, xoffb: float = 0.0,
                 xofft: float = 0.0) -> np.ndarray:
        """Batched finite-difference products of the period map on flat state
        vectors (sb_jv_batch): x0 (n,), dirs (ndir, n) -> (ndir, n)."""
        x0 = np.ascontiguousarray(x0, np.float64)
        d = np.ascontiguousarray(np.atleast_2d(dirs), np.float64)
        out = np.zeros_like(d)
        _check(lib().sb_jv_batch(self.h, _dp(x0), float(time0), float(xoffb), float(xofft),
                                 float(T), _dp(d), int(d.shape[0]), float(eps_jacobi),
                                 int(bool(central)), _dp(out)))
        return out

    @property
    def packed_length(self) -> int:
        """Length of the packed unknown vector (sb_packed_length)."""
        return int(lib().sb_packed_length(self.h))

    def set_state_packed(self, member: int, x_dev: int, sca, time=0.0, xoffb=0.0, xofft=0.0):
        """Sets a member from a packed vector at device address x_dev
        (sb_set_state_packed; queued on the handle's stream)."""
        sc = np.ascontiguousarray(sca, np.float64)
        _check(lib().sb_set_state_packed(self.h, int(member), ctypes.c_void_p(x_dev), _dp(sc),
                                         float(time), float(xoffb), float(xofft)))

    def get_state_packed(self, member: int, x_dev: int, sca, shiftx=0.0, shiftz=0.0):
        """Writes a member's state, phase-shifted, as a packed vector at device
        address x_dev (sb_get_state_packed; queued on the handle's stream)."""
        sc = np.ascontiguousarray(sca, np.float64)
        _check(lib().sb_get_state_packed(self.h, int(member), ctypes.c_void_p(x_dev), _dp(sc),
                                         float(shiftx), float(shiftz)))

    def shift_tangent_packed(self, x_dev: int, out_dev: int, which: str = "x"):
        """d/ds of the phase shift on a packed device vector (-i kx or -i kz
        times every mode; sb_packed_shift_tangent, handle's stream)."""
        _check(lib().sb_packed_shift_tangent(self.h, ctypes.c_void_p(x_dev),
                                             ctypes.c_void_p(out_dev), 0 if which == "x" else 1))

    def fp64_peak(self) -> float:
        v = ctypes.c_double()
        _check(lib().sb_fp64_peak(self.h, ctypes.byref(v)))
        return v.value

    def step(self, nsteps: int):
        _check(lib().sb_step(self.h, int(nsteps)))

    def sync(self):
        _check(lib().sb_sync(self.h))

    def status(self, member: int = 0) -> SbStatus:
        st = SbStatus()
        _check(lib().sb_get_status(self.h, member, ctypes.byref(st)))
        return st

    def trace(self, member: int = 0, max_records: int = 1 << 16) -> np.ndarray:
        n = ctypes.c_int()
        st = self.status(member)
        m = min(max_records, max(st.ntrace, 0))
        out = np.zeros((max(m, 1), TRACE_LEN_T if self.p.temperature else TRACE_LEN))
        _check(lib().sb_get_trace(self.h, member, _dp(out), m, ctypes.byref(n)))
        return out[: n.value]

    def cross(self, state: dict, nstep: int) -> tuple:
        """Drop-in for the reference ``cross`` (``crosst`` when the handle has
        the temperature, with state keys tb and tb00): advances box 0 by nstep
        steps in place on host arrays; returns (trace, status)."""
        keys = ("vor", "phi", "tb") if self.p.temperature else ("vor", "phi")
        for key in keys:
            assert state[key].dtype == np.complex128 and state[key].flags["C_CONTIGUOUS"]
        t = ctypes.c_double(state["time"])
        xb = ctypes.c_double(state["xoffb"])
        xt = ctypes.c_double(state["xofft"])
        st = SbStatus()
        if self.p.temperature:
            _check(lib().sb_crosst(self.h, _dp(state["vor"].view(np.float64)),
                                   _dp(state["phi"].view(np.float64)), _dp(state["u00"]),
                                   _dp(state["w00"]), _dp(state["tb"].view(np.float64)),
                                   _dp(state["tb00"]), ctypes.byref(t), ctypes.byref(xb),
                                   ctypes.byref(xt), int(nstep), ctypes.byref(st)))
        else:
            _check(lib().sb_cross(self.h, _dp(state["vor"].view(np.float64)),
                                  _dp(state["phi"].view(np.float64)), _dp(state["u00"]),
                                  _dp(state["w00"]), ctypes.byref(t), ctypes.byref(xb),
                                  ctypes.byref(xt), int(nstep), ctypes.byref(st)))
        state["time"], state["xoffb"], state["xofft"] = t.value, xb.value, xt.value
        # the records of this call (the status came with the state)
        m = max(st.ntrace, 0)
        out = np.zeros((max(m, 1), TRACE_LEN_T if self.p.temperature else TRACE_LEN))
        n = ctypes.c_int()
        _check(lib().sb_get_trace(self.h, 0, _dp(out), m, ctypes.byref(n)))
        return out[: n.value], st


def _lines(a, nlines: int, dtype, name: str) -> np.ndarray:
    """A per-line host array of at least nlines entries (the C side reads
    nlines of them)."""
    a = np.ascontiguousarray(a, dtype).ravel()
    if a.size < nlines:
        raise ValueError(f"{name} has {a.size} entries, fewer than nlines={nlines}")
    return a


def op_derivyc(my: int, Ly: float, iord: int, u_dev: int, out_dev: int, nlines: int,
               shp: np.ndarray, shm: np.ndarray, ldu: int = None, ldo: int = None,
               stream: int = 0):
    """d/dy (iord 1) or d2/dy2 (iord 2) of nlines device-resident complex lines
    ([j][line] layout, device pointers); shp/shm host complex arrays (nlines)."""
    sp = _lines(shp, nlines, np.complex128, "shp")
    sm = _lines(shm, nlines, np.complex128, "shm")
    _check(lib().sb_op_derivyc(int(my), float(Ly), int(iord), int(nlines), ctypes.c_void_p(u_dev),
                               int(ldu or nlines), ctypes.c_void_p(out_dev), int(ldo or nlines),
                               _dp(sp.view(np.float64)), _dp(sm.view(np.float64)),
                               ctypes.c_void_p(stream)))


def op_lapcdy(my: int, Ly: float, u_dev: int, out_dev: int, nlines: int, k2: np.ndarray,
              shp: np.ndarray, shm: np.ndarray, ldu: int = None, ldo: int = None,
              stream: int = 0):
    """Solves (d2/dy2 - k2) p = u on nlines device-resident complex lines."""
    kk = _lines(k2, nlines, np.float64, "k2")
    sp = _lines(shp, nlines, np.complex128, "shp")
    sm = _lines(shm, nlines, np.complex128, "shm")
    _check(lib().sb_op_lapcdy(int(my), float(Ly), int(nlines), ctypes.c_void_p(u_dev),
                              int(ldu or nlines), ctypes.c_void_p(out_dev), int(ldo or nlines),
                              _dp(kk), _dp(sp.view(np.float64)), _dp(sm.view(np.float64)),
                              ctypes.c_void_p(stream)))


def write_restart(path: str, p: SbParams, state: dict, deltat: float = 0.0):
    """Writes a state (pencil layout) as a restart file of the reference's
    binary layout (escru)."""
    vor = np.ascontiguousarray(state["vor"], np.complex128)
    phi = np.ascontiguousarray(state["phi"], np.complex128)
    u00 = np.ascontiguousarray(state["u00"], np.float64)
    w00 = np.ascontiguousarray(state["w00"], np.float64)
    _check(lib().sb_write_restart(str(path).encode(), ctypes.byref(p), _dp(vor.view(np.float64)),
                                  _dp(phi.view(np.float64)), _dp(u00), _dp(w00),
                                  float(state["time"]), float(state["xoffb"]),
                                  float(state["xofft"]), float(deltat)))


def read_restart(path: str, p: SbParams = None, keep_vor: bool = False):
    """Reads a restart file (getfil), mapping it on p's grid: kx/kz modes,
    the y planes (as read, every other one, stacked copies or a cubic spline
    in y) and the gam/Re rescaling (keep_vor: no vorticity rescaling for a
    changed Re, as the Newton drivers read).  Returns (state on p's grid with
    its offsets, info), or (None, info) without p."""
    info = SbRestartInfo()
    if p is None:
        _check(lib().sb_read_restart(str(path).encode(), None, None, None, None, None,
                                     ctypes.byref(info)))
        return None, info
    sz = sizes(p)
    vor = np.zeros((sz["mz"], sz["nkx"], p.my), np.complex128)
    phi = np.zeros_like(vor)
    u00 = np.zeros(p.my)
    w00 = np.zeros(p.my)
    _check(lib().sb_read_restart_ex(str(path).encode(), ctypes.byref(p),
                                    RESTART_KEEP_VOR if keep_vor else 0,
                                    _dp(vor.view(np.float64)), _dp(phi.view(np.float64)),
                                    _dp(u00), _dp(w00), ctypes.byref(info)))
    return {"vor": vor, "phi": phi, "u00": u00, "w00": w00, "time": info.time,
            "xoffb": info.run_xoffb, "xofft": info.run_xofft}, info


def params_from_restart(info: SbRestartInfo, **overrides) -> SbParams:
    """Step parameters recorded by a restart file: grid, Re, alp, Ly, gam, s, chi
    from the header and, with a footer, CFL, uprim, vbulk and the switches and
    parameters escru writes (ifix_dt with the Delta t as fixed_dt, iadd_force,
    force_roll, xforce, iadd_damping, damp_aa, damp_up, iuse_LES, iadd_visc, explicit,
    Cles; readwrite.f90:1336-1398).  Keyword arguments override any of them
    (the hre2.dat/hre3.dat settings of the run that reads the file)."""
    kw = dict(mgalx=info.mgalx, my=info.my, mgalz=info.mgalz, Re=info.Re, alp=info.alp,
              Ly=info.Ly, gam=info.gam, s=info.s, chi=info.chi)
    if info.has_footer:
        kw.update(CFL=info.CFL, uprim=info.uprim, vbulk=info.vbulk, xforce=info.xforce)
        opt = list(info.options)[:info.nopt]
        prm = list(info.params)[:info.nparams]
        if len(opt) >= 8 and len(prm) >= 7:
            if opt[1]:
                kw["fixed_dt"] = prm[0]
            kw.update(force=opt[2], force_roll=prm[1], xforce=prm[2], damping=opt[5],
                      damp_aa=prm[4], damp_up=prm[5], les=opt[6], les_visc=opt[7],
                      implicit_visc=0 if opt[0] else 1)
            if opt[6]:
                kw["cs"] = prm[6]
    kw.update(overrides)
    return make_params(**kw)


def op_filterc(my: int, u_dev: int, out_dev: int, nlines: int, shp: np.ndarray,
               ldu: int = None, ldo: int = None, stream: int = 0):
    """Compact y-filter of nlines device-resident complex lines (filterc)."""
    sp = _lines(shp, nlines, np.complex128, "shp")
    _check(lib().sb_op_filterc(int(my), int(nlines), ctypes.c_void_p(u_dev), int(ldu or nlines),
                               ctypes.c_void_p(out_dev), int(ldo or nlines),
                               _dp(sp.view(np.float64)), ctypes.c_void_p(stream)))


def op_cfty(my: int, c_dev: int, nlines: int, iopt: int, ldc: int = None, stream: int = 0):
    """In-place y transform of complex device lines (cfty conventions)."""
    _check(lib().sb_op_cfty(int(my), int(nlines), ctypes.c_void_p(c_dev), int(ldc or nlines),
                            int(iopt), ctypes.c_void_p(stream)))


def op_rfty(my: int, c_dev: int, nlines: int, iopt: int, ldc: int = None, stream: int = 0):
    """In-place y transform of real device lines of my+2 rows (rfty)."""
    _check(lib().sb_op_rfty(int(my), int(nlines), ctypes.c_void_p(c_dev), int(ldc or nlines),
                            int(iopt), ctypes.c_void_p(stream)))


def op_derivyc_noalloc(my: int, Ly: float, iord: int, u_dev: int, out_dev: int, nlines: int,
                       shp: np.ndarray, shm: np.ndarray, ldu: int = None, ldo: int = None,
                       stream: int = 0):
    """Same as op_derivyc without any device allocation: scratch in a fixed
    array of the library (limits and sharing rules in include/shearbox.h)."""
    sp = _lines(shp, nlines, np.complex128, "shp")
    sm = _lines(shm, nlines, np.complex128, "shm")
    _check(lib().sb_op_derivyc_noalloc(int(my), float(Ly), int(iord), int(nlines),
                                       ctypes.c_void_p(u_dev), int(ldu or nlines),
                                       ctypes.c_void_p(out_dev), int(ldo or nlines),
                                       _dp(sp.view(np.float64)), _dp(sm.view(np.float64)),
                                       ctypes.c_void_p(stream)))
