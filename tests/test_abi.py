"""The C-ABI library loads and exports every function declared in
include/shearbox.h; host-only entry points behave (no GPU compute here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, box_params


def _declared():
    txt = open(os.path.join(ROOT, "include", "shearbox.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sb_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from shear_nnf_gb300.buildlib import LIB, build
    build()
    return ctypes.CDLL(LIB)


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in shearbox.h but not exported"


def test_python_wrapper_lists_the_header():
    import shear_nnf_gb300 as sb
    assert sorted(sb.ABI_FUNCTIONS) == _declared()


def _prototypes():
    txt = open(os.path.join(ROOT, "include", "shearbox.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(sb_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S):
        args = " ".join(m.group(2).split())
        out[m.group(1)] = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
    return out


def test_python_argtypes_match_the_header():
    """Every entry point the Python host binds has one ctypes argument type per
    parameter of its prototype, pointers where the header has pointers."""
    import shear_nnf_gb300 as sb
    L = sb.lib()
    protos = _prototypes()
    assert sorted(protos) == sorted(sb.ABI_FUNCTIONS)
    for name, params in protos.items():
        at = getattr(L, name).argtypes
        assert at is not None and len(at) == len(params), (name, params, at)
        for decl, t in zip(params, at):
            is_ptr = "*" in decl or "[" in decl  # array parameters are pointers
            is_ctype_ptr = t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and \
                isinstance(getattr(t, "_type_"), type) and issubclass(t, ctypes._Pointer)
            assert is_ptr == bool(is_ctype_ptr), (name, decl, t)


def test_sizes_follow_initcr():
    import shear_nnf_gb300 as sb
    for (gx, gy, gz), (mx, mz) in {(192, 96, 96): (128, 63), (64, 32, 32): (42, 19),
                                    (96, 48, 48): (64, 31), (384, 192, 192): (256, 127)}.items():
        s = sb.sizes(sb.make_params(**box_params(gx, gy, gz, rez=1000.0)))
        assert (s["mx"], s["mz"], s["nkx"], s["nz"]) == (mx, mz, mx // 2, (mz - 1) // 2)


def test_compact_coefficients_match_oracle_bitwise():
    import oracle
    import shear_nnf_gb300 as sb
    pr1, rh1h, pr2, rh2h = sb.compact_coeffs()
    o = oracle.Oracle(64, 32, 32, Re=10.0, alp=0.5, Ly=2 * np.pi, gam=1.0)
    opr1, orh1, opr2, orh2, dy = o.coeffs()
    assert np.array_equal(pr1, opr1) and np.array_equal(pr2, opr2)
    np.testing.assert_allclose(rh1h / dy, orh1, rtol=1e-15)
    np.testing.assert_allclose(rh2h / dy ** 2, orh2, rtol=1e-15)


def test_seed_state_is_divergence_free_and_hermitian():
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(64, 32, 32, rez=1000.0))
    st = sb.seed_state(p, 5)
    s = sb.sizes(p)
    nz, mz = s["nz"], s["mz"]
    vor, phi = st["vor"], st["phi"]
    # kx = 0 column: conjugate symmetric in kz (the reality condition set_conj imposes)
    for k in range(nz + 1, mz):
        np.testing.assert_allclose(vor[k, 0], np.conj(vor[mz - k, 0]), atol=1e-12)
        np.testing.assert_allclose(phi[k, 0], np.conj(phi[mz - k, 0]), atol=1e-12)
    assert np.all(vor[0, 0] == 0) and np.all(phi[0, 0] == 0)
    # rms velocity of the seeded field is 0.1 S Lz (checked through the oracle's UNER)
    import oracle
    o = oracle.Oracle(**box_params(64, 32, 32, rez=1000.0, fixed_dt=1e-6))
    tr, _ = o.cross({k: (v.copy() if hasattr(v, "copy") else v) for k, v in st.items()}, 1)
    urms = np.sqrt((tr[0, 2] ** 2 + tr[0, 3] ** 2 + tr[0, 4] ** 2) / 3)
    assert abs(urms / (0.1 * 2 * np.pi) - 1) < 0.05


def test_seed_state_reproducible_and_seed_dependent():
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(64, 32, 32, rez=1000.0))
    a, b, c = sb.seed_state(p, 1), sb.seed_state(p, 1), sb.seed_state(p, 2)
    assert np.array_equal(a["vor"], b["vor"]) and np.array_equal(a["u00"], b["u00"])
    assert not np.allclose(a["vor"], c["vor"])


@pytest.mark.parametrize("grid,seed,k0", [((64, 32, 32), 3, 4.0), ((96, 48, 48), 77, 4.0),
                                          ((192, 96, 96), 3, 4.0), ((64, 32, 32), 11, 6.0)])
def test_oracle_seed_matches_library_bitwise(grid, seed, k0):
    """The oracle's restatement of the seeded field (used by the CPU baseline,
    which must not load the library under test) equals sb_seed_state bit for
    bit."""
    import oracle
    import shear_nnf_gb300 as sb
    pp = box_params(*grid, rez=1000.0)
    a = sb.seed_state(sb.make_params(**pp), seed, k0=k0)
    b = oracle.seed_state(seed=seed, k0=k0, **pp)
    for key in ("vor", "phi", "u00", "w00"):
        assert a[key].shape == b[key].shape
        assert np.array_equal(a[key].view(np.float64), b[key].view(np.float64)), key


def test_oracle_seed_matches_library_with_temperature():
    import oracle
    import shear_nnf_gb300 as sb
    pp = box_params(64, 32, 32, rez=1000.0, temperature=1, fkappa=0.01)
    a = sb.seed_state(sb.make_params(**pp), 7)
    b = oracle.seed_state(seed=7, **pp)
    for key in ("tb", "tb00", "vor"):
        assert np.array_equal(np.asarray(a[key]).view(np.float64),
                              np.asarray(b[key]).view(np.float64)), key


def test_operator_wrappers_reject_short_line_arrays():
    """The C side reads nlines entries of each per-line host array: shorter
    arrays are refused before any call."""
    import shear_nnf_gb300 as sb
    short = np.ones(3, np.complex128)
    full = np.ones(8, np.complex128)
    with pytest.raises(ValueError, match="shp"):
        sb.op_derivyc(32, 2 * np.pi, 1, 0, 0, 8, short, full)
    with pytest.raises(ValueError, match="shm"):
        sb.op_derivyc_noalloc(32, 2 * np.pi, 1, 0, 0, 8, full, short)
    with pytest.raises(ValueError, match="k2"):
        sb.op_lapcdy(32, 2 * np.pi, 0, 0, 8, np.ones(2), full, full)
    with pytest.raises(ValueError, match="shp"):
        sb.op_filterc(32, 0, 0, 8, short)


def test_invalid_grid_rejected_without_gpu():
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(100, 32, 32, rez=1000.0))
    with pytest.raises(sb.ShearBoxError, match="unsupported"):
        sb.sizes(p) and sb.seed_state(p, 1)


def test_no_cpu_fallback(monkeypatch):
    """Without a GPU the handle cannot be created: the library has no CPU path."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import shear_nnf_gb300 as sb
    with pytest.raises(sb.ShearBoxError, match="no CUDA device"):
        sb.ShearBox(sb.make_params(**box_params(64, 32, 32, rez=1000.0)))


def _f90():
    txt = open(os.path.join(ROOT, "include", "shearbox_c.f90")).read()
    return "\n".join(line.split("!")[0] for line in txt.splitlines())


def test_fortran_interface_binds_exported_symbols(lib):
    """Every bind(C, name=...) of include/shearbox_c.f90 is declared in the
    header and exported (the Fortran module is not compiled here)."""
    names = re.findall(r'bind\(C,\s*name="(sb_[a-z0-9_]+)"\)', _f90())
    assert len(names) >= 20
    declared = set(_declared())
    for n in names:
        assert n in declared and hasattr(lib, n), n


def test_fortran_interfaces_match_the_prototypes():
    """Each bind(C) interface has the header prototype's parameter count, and
    every entry point is bound except the test and benchmark helpers."""
    txt = re.sub(r"&\s*\n\s*&?", " ", _f90())
    funcs = re.findall(r'function\s+(sb_[a-z0-9_]+)\s*\(([^)]*)\)\s*bind\(C,\s*'
                       r'name="(sb_[a-z0-9_]+)"\)', txt, flags=re.I)
    protos = _prototypes()
    for fname, args, cname in funcs:
        assert fname == cname and cname in protos, cname
        assert len([a for a in args.split(",") if a.strip()]) == len(protos[cname]), cname
    helpers = {"sb_compact_coeffs", "sb_fft_twiddles", "sb_fp64_peak", "sb_launch_stage",
               "sb_seed_state"}
    assert set(protos) - {c for _, _, c in funcs} == helpers


def test_fortran_types_follow_the_c_structs():
    """The bind(C) derived types list the C struct members in order and type."""
    import shear_nnf_gb300 as sb
    txt = _f90()

    def fields(tname):
        body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type" % tname, txt, re.S).group(1)
        out = []
        for line in body.splitlines():
            m = re.match(r"\s*(integer\(c_int\)|real\(c_double\))\s*::\s*(.*)", line)
            if m:
                kind = ctypes.c_int if m.group(1).startswith("integer") else ctypes.c_double
                out += [(n.strip(), kind) for n in m.group(2).split(",")]
        return out

    for tname, cls in (("sb_params", sb.SbParams), ("sb_status", sb.SbStatus)):
        assert [(n.lower(), t) for n, t in fields(tname)] == \
            [(n.lower(), t) for n, t in cls._fields_], tname


def test_product_code_never_reaches_the_oracle():
    """The package and its CUDA sources name no oracle module, library or
    source: the oracle is test infrastructure only, and the product path has
    no CPU fallback to route through it."""
    pkg = os.path.join(ROOT, "shear_nnf_gb300")
    hits = []
    for d, _, files in os.walk(pkg):
        if "_build" in d or "__pycache__" in d:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                txt = open(os.path.join(d, f), errors="replace").read()
                if re.search(r"\boracle\b|liboracle|shearbox_oracle", txt, flags=re.I):
                    hits.append(f)
    assert hits == []
