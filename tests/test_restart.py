"""Restart files in the reference's binary layout (escru / getfil,
readwrite.f90:72-447,1336-1398): record structure, round trip, mapping onto a
different x/z grid, header-only reads and malformed files.  Host code only."""
import struct

import numpy as np
import pytest

from conftest import box_params

import shear_nnf_gb300 as sb


def _conj_state(st, p):
    sz = sb.sizes(p)
    out = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
    for key in ("vor", "phi"):
        for k in range(sz["nz"] + 1, sz["mz"]):
            out[key][k, 0, :] = np.conj(out[key][sz["mz"] - k, 0, :])
    return out


def _records(path):
    data = open(path, "rb").read()
    recs, pos = [], 0
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        recs.append(data[pos + 4:pos + 4 + n])
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        assert m == n
        pos += 8 + n
    return recs


def test_record_layout(tmp_path):
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    sz = sb.sizes(p)
    st = sb.seed_state(p, 7)
    st.update(time=1.25, xoffb=-0.5, xofft=0.5)
    f = tmp_path / "a.bin"
    sb.write_restart(f, p, st, deltat=0.003)
    recs = _records(f)
    my, nkx, mz = p.my, sz["nkx"], sz["mz"]
    assert len(recs) == 5 + my + 4
    assert [len(r) for r in recs[:5]] == [16, 68, 8 * my, 32, 16 * my]
    assert all(len(r) == 32 * nkx * mz for r in recs[5:5 + my])
    assert [len(r) for r in recs[5 + my:]] == [32, 12, 36, 104]
    assert struct.unpack("<4i", recs[0]) == (64, 32, 32, 1)
    t, Re, alp, lyp, gam, s, chi = struct.unpack_from("<7d", recs[1])
    assert (t, alp, gam, s) == (1.25, 0.5, 1.0, 1.0) and abs(lyp * np.pi - p.Ly) < 1e-14
    assert struct.unpack_from("<3i", recs[1], 56) == (2 * nkx, my, mz)
    y = np.frombuffer(recs[2], "<f8")
    assert abs(y[0] + p.Ly / 2) < 1e-15 and abs(y[1] - y[0] - p.Ly / my) < 1e-14
    assert struct.unpack("<4d", recs[3]) == (-0.5, 0.5, 0.0, 0.0)
    # plane j, mode (kz=k, kx=i): vor.re, phi.re, vor.im, phi.im
    j, k, i = 5, 2, 3
    e = struct.unpack_from("<4d", recs[5 + j], 32 * (k * nkx + i))
    assert e == (st["vor"][k, i, j].real, st["phi"][k, i, j].real, st["vor"][k, i, j].imag,
                 st["phi"][k, i, j].imag)
    assert struct.unpack("<3i", recs[5 + my + 1]) == (1742, 9, 13)
    assert struct.unpack_from("<d", recs[-1])[0] == 0.003


def test_round_trip(tmp_path):
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    st = sb.seed_state(p, 3)
    st.update(time=2.5, xoffb=-1.0, xofft=1.0)
    f = tmp_path / "r.bin"
    sb.write_restart(f, p, st)
    back, info = sb.read_restart(f, p)
    ref = _conj_state(st, p)
    for key in ("vor", "phi", "u00", "w00"):
        assert np.array_equal(back[key], ref[key]), key
    assert (back["time"], back["xoffb"], back["xofft"]) == (2.5, -1.0, 1.0)
    assert info.has_footer and info.irev == 1742 and info.CFL == p.CFL
    _, hdr = sb.read_restart(f)
    assert (hdr.mgalx, hdr.my, hdr.mgalz, hdr.mx, hdr.mz) == (64, 32, 32, 42, 19)


def test_footer_carries_forces_and_damping(tmp_path):
    """The option switches and parameters of the footer record the body force
    and the window damping of the run (iadd_force, iadd_damping; force_roll,
    xforce, damp_aa, damp_up), as escru writes them."""
    p = sb.make_params(**box_params(64, 32, 32, 1000.0, force=1, force_roll=0.25, xforce=0.0,
                                    damping=1, damp_up=0.4, damp_aa=0.125))
    st = sb.seed_state(p, 2)
    f = tmp_path / "f.bin"
    sb.write_restart(f, p, st, deltat=0.002)
    recs = _records(f)
    opts = struct.unpack("<9i", recs[-2])
    assert opts[2] == 1 and opts[5] == 1 and opts[3] == 5
    prm = struct.unpack("<13d", recs[-1])
    assert prm[:6] == (0.002, 0.25, 0.0, 0.0, 0.125, 0.4)
    q = sb.make_params(**box_params(64, 32, 32, 1000.0, force=-1, xforce=0.05))
    sb.write_restart(f, q, st)
    recs = _records(f)
    assert struct.unpack("<4d", recs[-4])[3] == 0.05
    assert struct.unpack("<9i", recs[-2])[2] == -1


def test_params_from_restart(tmp_path):
    """The parameters a restart records come back as step parameters."""
    kw = box_params(64, 32, 32, 1000.0, fixed_dt=0.004, force=2, force_roll=0.3, damping=1,
                    damp_up=0.2, damp_aa=0.15, les=1, les_visc=0, cs=0.12, CFL=0.4)
    kw.pop("cfl", None)
    p = sb.make_params(**kw)
    st = sb.seed_state(p, 4)
    f = tmp_path / "p.bin"
    sb.write_restart(f, p, st, deltat=0.004)
    _, info = sb.read_restart(f)
    q = sb.params_from_restart(info)
    for name, _ in sb.SbParams._fields_:
        if name in ("mgalx", "my", "mgalz", "Re", "alp", "Ly", "gam", "s", "chi", "CFL",
                    "uprim", "vbulk", "fixed_dt", "force", "force_roll", "xforce", "damping",
                    "damp_up", "damp_aa", "les", "les_visc", "cs"):
            assert getattr(q, name) == pytest.approx(getattr(p, name), rel=1e-14, abs=1e-300), name
    r = sb.params_from_restart(info, Re=2.0, damping=0)
    assert r.Re == 2.0 and r.damping == 0 and r.force == 2


@pytest.mark.parametrize("target", [(96, 32, 48), (48, 32, 32)])
def test_grid_change(tmp_path, target):
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    q = sb.make_params(**box_params(*target, 1000.0))
    st = sb.seed_state(p, 4)
    f = tmp_path / "g.bin"
    sb.write_restart(f, p, st)
    got, _ = sb.read_restart(f, q)
    sp, sq = sb.sizes(p), sb.sizes(q)
    nk = min(sp["nkx"], sq["nkx"])
    klen = (min(sp["mz"], sq["mz"]) + 1) // 2
    ref = _conj_state(st, p)
    for key in ("vor", "phi"):
        a, b = got[key], ref[key]
        np.testing.assert_array_equal(a[:klen, :nk], b[:klen, :nk])
        if klen > 1:
            np.testing.assert_array_equal(a[sq["mz"] - klen + 1:, :nk], b[sp["mz"] - klen + 1:, :nk])
        assert np.all(a[:, nk:] == 0) and np.all(a[klen:sq["mz"] - klen + 1] == 0)


def test_malformed_and_unsupported(tmp_path):
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    f = tmp_path / "m.bin"
    sb.write_restart(f, p, sb.seed_state(p, 1))
    data = open(f, "rb").read()
    bad = tmp_path / "bad.bin"
    open(bad, "wb").write(data[:300])
    with pytest.raises(sb.ShearBoxError):
        sb.read_restart(bad, p)
    q = sb.make_params(**box_params(64, 48, 32, 1000.0))
    with pytest.raises(sb.ShearBoxError, match="my="):
        sb.read_restart(f, q)
    with pytest.raises(sb.ShearBoxError):
        sb.read_restart(tmp_path / "missing.bin", p)
