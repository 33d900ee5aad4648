"""CPU FP64 oracle for the shearing-box RK3 step -- TEST INFRASTRUCTURE ONLY.

This package is the checker.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it; the product package
(``shear_nnf_gb300``) never does.

The C restatement lives in ``shearbox_oracle.c`` (each routine cites the
reference file:line it follows).  Parity status: pinned against the reference's
own analytic checks (RDT solution ``rdtfunc``, operators.f90:1516-1562; design
conditions of the compact schemes, diffy_shear_hepta.f90:68-296) and against
numpy's DFT; not pinned to outputs of the reference binary, which cannot be
built here (no Fortran compiler, MPI, FFTW or HDF5).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
TRACE_LEN = 24
TRACE_LEN_T = 29  # crosst: the record plus tbmax, tner(1:4)


def build(force: bool = False) -> str:
    """Compile the C restatement with gcc (OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "shearbox_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", LIB, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB


class OrcParams(ctypes.Structure):
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


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_sizes.argtypes = [ctypes.c_void_p, ip]
        L.orc_coeffs.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_cross.restype = ctypes.c_int
        L.orc_cross.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int,
                                dp, ip, ip, dp]
        L.orc_statistics.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp, dp, ip, dp]
        L.orc_crosst.restype = ctypes.c_int
        L.orc_crosst.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp, dp, dp, dp, dp,
                                 ctypes.c_int, dp, ip, ip, dp]
        L.orc_derivyc.argtypes = [ctypes.c_void_p, dp, dp] + [ctypes.c_double] * 4 + [ctypes.c_int] * 2
        L.orc_lapcdy.argtypes = [ctypes.c_void_p, dp, ctypes.c_double, dp] + [ctypes.c_double] * 4 + [ctypes.c_int]
        L.orc_fourxz.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_int]
        L.orc_physical.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_uint, dp]
        L.orc_rfty.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
        L.orc_cfty.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
        L.orc_filterc.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int]
        L.orc_fft.argtypes = [ctypes.c_int, dp, ctypes.c_int]
        L.orc_seed_state.restype = ctypes.c_int
        L.orc_seed_state.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + \
            [ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def _seed_fields(mgalx, my, mgalz, alp, gam, Ly, seed, k0, urms):
    mz = 2 * (mgalz // 3) - 1
    nkx = (2 * (mgalx // 3)) // 2
    vor = np.zeros((mz, nkx, my), np.complex128)
    phi = np.zeros_like(vor)
    u00 = np.zeros(my)
    w00 = np.zeros(my)
    rc = lib().orc_seed_state(int(mgalx), int(my), int(mgalz), float(alp), float(gam), float(Ly),
                              ctypes.c_ulonglong(int(seed)), float(k0), float(urms),
                              _dp(vor.view(np.float64)), _dp(phi.view(np.float64)), _dp(u00),
                              _dp(w00))
    if rc != 0:
        raise MemoryError("orc_seed_state")
    return vor, phi, u00, w00


def seed_state(mgalx, my, mgalz, alp, Ly, gam, seed, k0=4.0, urms=None, temperature=0,
               **_ignored) -> dict:
    """The seeded initial field of the benchmark configurations, generated by the
    oracle (bit-identical to the library's sb_seed_state), as a state dict in
    the pencil layout; with temperature=1 also tb, tb00 from a second seed as
    the library draws them.  Extra keyword arguments (the other step
    parameters) are accepted and ignored, so a parameter dict can be passed."""
    if urms is None:
        urms = 0.1 * 1.0 * (2 * np.pi / gam)  # 0.1 * S * Lz
    vor, phi, u00, w00 = _seed_fields(mgalx, my, mgalz, alp, gam, Ly, seed, k0, urms)
    st = {"vor": vor, "phi": phi, "u00": u00, "w00": w00, "time": 0.0, "xoffb": 0.0,
          "xofft": 0.0}
    if temperature:
        tv, _, t00, _ = _seed_fields(mgalx, my, mgalz, alp, gam, Ly,
                                     (int(seed) * 7919 + 17) & 0xFFFFFFFF, k0, urms)
        st["tb"] = np.ascontiguousarray(tv / k0)
        st["tb00"] = t00
    return st


def fft(x: np.ndarray, sign: int) -> np.ndarray:
    """Unnormalised complex DFT (sign -1 forward, +1 backward)."""
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    lib().orc_fft(a.size, _dp(a.view(np.float64)), int(sign))
    return a


class Oracle:
    """One shearing box on the CPU, reference pencil layout."""

    def __init__(self, mgalx, my, mgalz, Re, alp, Ly, gam, s=1.0, chi=0.0, CFL=0.5,
                 vbulk=0.0, fixed_dt=0.0, readflag=1, uprim=1.0, nhist=1,
                 etime=1e10, dumptime=1e10, dtimag=1e10, keep_laminar=0, les=0, les_visc=1,
                 cs=0.1, ydeal=0, temperature=0, fkappa=0.0, bym=0.0, gbeta=0.0, damping=0,
                 damp_up=0.0, damp_aa=0.0, force=0, force_roll=0.0, xforce=0.0,
                 implicit_visc=0):
        if implicit_visc and (les or (temperature and not fkappa > 0)):
            # the reference stops on LES with explicit = 0 (initcr.f90:2179-2182);
            # crosst's semi-implicit branch divides by fkappa
            raise ValueError("implicit_visc needs les = 0 (and fkappa > 0 with the temperature)")
        self.p = OrcParams(mgalx, my, mgalz, Re, alp, Ly, gam, s, chi, CFL, vbulk, fixed_dt,
                           readflag, uprim, nhist, etime, dumptime, dtimag, keep_laminar, les,
                           les_visc, cs, ydeal, temperature, fkappa, bym, gbeta, damping,
                           damp_up, damp_aa, force, force_roll, xforce, implicit_visc)
        self.h = lib().orc_create(ctypes.byref(self.p))
        sz = (ctypes.c_int * 8)()
        lib().orc_sizes(self.h, sz)
        self.mx, self.mz, self.nkx, self.my, self.nz, _, _, self.buffsize = list(sz)
        self.deltat = 0.0

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.orc_destroy(h)
            self.h = None

    def coeffs(self):
        a = [np.zeros(7) for _ in range(4)]
        dy = ctypes.c_double()
        lib().orc_coeffs(self.h, *[_dp(x) for x in a], ctypes.byref(dy))
        return a[0], a[1], a[2], a[3], dy.value

    def derivyc(self, u: np.ndarray, shp=1.0 + 0j, shm=None, iord=1) -> np.ndarray:
        if shm is None:
            shm = np.conj(shp)
        if np.iscomplexobj(u):
            a = np.ascontiguousarray(u, dtype=np.complex128)
            out = np.zeros_like(a)
            lib().orc_derivyc(self.h, _dp(a.view(np.float64)), _dp(out.view(np.float64)),
                              shp.real, shp.imag, shm.real, shm.imag, iord, 2)
            return out
        a = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros_like(a)
        lib().orc_derivyc(self.h, _dp(a), _dp(out), 1.0, 0.0, 1.0, 0.0, iord, 1)
        return out

    def physical(self, state: dict, mask: int) -> np.ndarray:
        """convh5 fields (mask bits 0..10: u v w ox oy oz Q R Qs Rs Qw) of a
        state: array (nfields, my, mgalz, mgalx)."""
        nf = bin(mask & 0x7FF).count("1")
        out = np.zeros((nf, self.my, self.p.mgalz, self.p.mgalx))
        vor = np.ascontiguousarray(state["vor"], np.complex128)
        phi = np.ascontiguousarray(state["phi"], np.complex128)
        lib().orc_physical(self.h, _dp(vor.view(np.float64)), _dp(phi.view(np.float64)),
                           _dp(np.ascontiguousarray(state["u00"], np.float64)),
                           _dp(np.ascontiguousarray(state["w00"], np.float64)),
                           float(state["xoffb"]), float(state["xofft"]), int(mask), _dp(out))
        return out

    def statistics(self) -> dict:
        """The hist accumulators of the last cross call: stats, stats2 (my, 23),
        spec, spec2 (mz, nkx, 8), tstats (my, 5), tspec (mz, nkx, 4), nacum,
        total_dt (reference arrays with the first index fastest)."""
        my, nkx, mz = self.my, self.nkx, self.mz
        out = {"stats": np.zeros((my, 23)), "stats2": np.zeros((my, 23)),
               "spec": np.zeros((mz, nkx, 8)), "spec2": np.zeros((mz, nkx, 8)),
               "tstats": np.zeros((my, 5)), "tspec": np.zeros((mz, nkx, 4))}
        n = ctypes.c_int(0)
        t = ctypes.c_double(0.0)
        lib().orc_statistics(self.h, *[_dp(out[k]) for k in ("stats", "stats2", "spec", "spec2",
                                                            "tstats", "tspec")],
                             ctypes.byref(n), ctypes.byref(t))
        out["nacum"], out["total_dt"] = n.value, t.value
        return out

    def rfty(self, u: np.ndarray, iopt: int) -> np.ndarray:
        """rfty on one line: u of length my+2 (packed half spectrum)."""
        a = np.ascontiguousarray(u, dtype=np.float64).copy()
        lib().orc_rfty(self.h, _dp(a), int(iopt))
        return a

    def cfty(self, u: np.ndarray, iopt: int) -> np.ndarray:
        a = np.ascontiguousarray(u, dtype=np.complex128).copy()
        lib().orc_cfty(self.h, _dp(a.view(np.float64)), int(iopt))
        return a

    def filterc(self, u: np.ndarray, shp=1.0 + 0j) -> np.ndarray:
        """The compact y-filter of one line (complex: shear phase shp)."""
        if np.iscomplexobj(u):
            a = np.ascontiguousarray(u, dtype=np.complex128)
            out = np.zeros_like(a)
            lib().orc_filterc(self.h, _dp(a.view(np.float64)), _dp(out.view(np.float64)),
                              shp.real, shp.imag, 2)
            return out
        a = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros_like(a)
        lib().orc_filterc(self.h, _dp(a), _dp(out), 1.0, 0.0, 1)
        return out

    def lapcdy(self, u: np.ndarray, k2: float, shp=1.0 + 0j, shm=None) -> np.ndarray:
        if shm is None:
            shm = np.conj(shp)
        a = np.ascontiguousarray(u, dtype=np.complex128)
        out = np.zeros_like(a)
        lib().orc_lapcdy(self.h, _dp(a.view(np.float64)), float(k2), _dp(out.view(np.float64)),
                         shp.real, shp.imag, shm.real, shm.imag, 2)
        return out

    def fourxz_c2r(self, fou: np.ndarray) -> np.ndarray:
        """fou complex (mz, nkx) [kz, kx] -> physical (mgalz, mgalx+2)."""
        f = np.ascontiguousarray(fou, dtype=np.complex128).copy()
        phys = np.zeros((self.p.mgalz, self.p.mgalx + 2))
        lib().orc_fourxz(self.h, _dp(f.view(np.float64)), _dp(phys), 1)
        return phys

    def fourxz_r2c(self, phys: np.ndarray) -> np.ndarray:
        ph = np.ascontiguousarray(phys, dtype=np.float64).copy()
        f = np.zeros((self.mz, self.nkx), dtype=np.complex128)
        lib().orc_fourxz(self.h, _dp(f.view(np.float64)), _dp(ph), -1)
        return f

    def cross(self, state: dict, nstep: int):
        """Advance ``state`` in place by nstep steps.  state keys: vor, phi
        (complex (mz, nkx, my) pencil layout), u00, w00 (my,), time, xoffb,
        xofft; with temperature also tb (like vor) and tb00 (my,), stepped by
        crosst.  Returns (trace array (n, 24 or 29), istop)."""
        vor = state["vor"]
        phi = state["phi"]
        temp = bool(self.p.temperature)
        fields = (vor, phi, state["tb"]) if temp else (vor, phi)
        for a in fields:
            assert a.dtype == np.complex128 and a.flags["C_CONTIGUOUS"]
            assert a.shape == (self.mz, self.nkx, self.my)
        t = ctypes.c_double(state["time"])
        xb = ctypes.c_double(state["xoffb"])
        xt = ctypes.c_double(state["xofft"])
        tr = np.zeros((max(nstep, 1), TRACE_LEN_T if temp else TRACE_LEN))
        nt = ctypes.c_int(0)
        ist = ctypes.c_int(0)
        dt = ctypes.c_double(self.deltat)
        if temp:
            rc = lib().orc_crosst(self.h, _dp(vor.view(np.float64)), _dp(phi.view(np.float64)),
                                  _dp(state["u00"]), _dp(state["w00"]),
                                  _dp(state["tb"].view(np.float64)), _dp(state["tb00"]),
                                  ctypes.byref(t), ctypes.byref(xb), ctypes.byref(xt),
                                  int(nstep), _dp(tr), ctypes.byref(nt), ctypes.byref(ist),
                                  ctypes.byref(dt))
            assert rc >= 0, "orc_crosst needs temperature=1, tb and tb00"
        else:
            lib().orc_cross(self.h, _dp(vor.view(np.float64)), _dp(phi.view(np.float64)),
                            _dp(state["u00"]), _dp(state["w00"]), ctypes.byref(t),
                            ctypes.byref(xb), ctypes.byref(xt), int(nstep), _dp(tr),
                            ctypes.byref(nt), ctypes.byref(ist), ctypes.byref(dt))
        state["time"], state["xoffb"], state["xofft"] = t.value, xb.value, xt.value
        self.deltat = dt.value
        return tr[: nt.value], ist.value
