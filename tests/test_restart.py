"""Restart files in the reference's binary layout (escru / getfil,
readwrite.f90:72-447,1336-1398): record structure, round trip, mapping onto a
different x/z grid, the y mappings of getfil (every other plane, stacked
copies, cubic spline), the gam/Re rescaling, header-only reads and malformed
files.  Host code only."""
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
    assert q.implicit_visc == 0


def test_footer_records_the_integrator(tmp_path):
    """The first footer switch is the reference's explicit flag: 1 for the
    explicit branch, 0 for the semi-implicit one (implicit_visc)."""
    st = sb.seed_state(sb.make_params(**box_params(64, 32, 32, 1000.0)), 2)
    f = tmp_path / "i.bin"
    for imp in (0, 1):
        p = sb.make_params(**box_params(64, 32, 32, 1000.0), implicit_visc=imp)
        sb.write_restart(f, p, st)
        assert struct.unpack("<9i", _records(f)[-2])[0] == 1 - imp
        _, info = sb.read_restart(f)
        assert sb.params_from_restart(info).implicit_visc == imp


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
    # x and y together (readwrite.f90:116-120), alp and my together (:172-175),
    # a spline in y with another Ly (:404-413)
    for q in (sb.make_params(**box_params(96, 48, 32, 1000.0)),
              sb.make_params(**dict(box_params(64, 48, 32, 1000.0), alp=0.7)),
              sb.make_params(**dict(box_params(64, 48, 32, 1000.0), Ly=5.0))):
        with pytest.raises(sb.ShearBoxError, match="error 9"):
            sb.read_restart(f, q)
    with pytest.raises(sb.ShearBoxError):
        sb.read_restart(tmp_path / "missing.bin", p)


def _spline_ref(x, y, c):
    """A numpy restatement of the natural cubic spline of getfil's interp_y
    (cubic_spline + interpolate, readwrite.f90:774-812,1131-1155)."""
    N = len(x)
    d2, u = np.zeros(N), np.zeros(N)
    for i in range(1, N - 1):
        sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1])
        pp = sig * d2[i - 1] + 2.0
        d2[i] = (sig - 1.0) / pp
        u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]))
                / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / pp
    for k in range(N - 2, 0, -1):
        d2[k] = d2[k] * d2[k + 1] + u[k]
    out = []
    for cc in c:
        klo, khi = 0, N - 1
        while khi - klo > 1:
            k = (khi + klo) // 2
            if x[k] > cc:
                khi = k
            else:
                klo = k
        h = x[khi] - x[klo]
        a, b = (x[khi] - cc) / h, (cc - x[klo]) / h
        out.append(a * y[klo] + b * y[khi] + ((a * a * a - a) * d2[klo] + (b * b * b - b) * d2[khi])
                   * (h * h) / 6.0)
    return np.array(out)


def test_y_spline_interpolation(tmp_path):
    """my 32 -> 48 (not a 3x or 5x stack): per mode line a natural cubic spline
    through the file's planes and the wrapped first plane at Ly/2 (shifted by
    exp(-i kx xofft)), on the run's y grid; the same for u00, w00."""
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    q = sb.make_params(**box_params(64, 48, 32, 1000.0))
    st = _conj_state(sb.seed_state(p, 9), p)
    st.update(xoffb=-0.3, xofft=0.3)
    f = tmp_path / "s.bin"
    sb.write_restart(f, p, st)
    got, info = sb.read_restart(f, q)
    assert info.ymap == 3 and (got["xoffb"], got["xofft"]) == (-0.3, 0.3)
    ye = np.append(np.arange(32) * (p.Ly / 32) - p.Ly / 2, p.Ly / 2)
    y = np.arange(48) * (q.Ly / 48) - q.Ly / 2
    for (k, i) in [(0, 1), (2, 3), (5, 0), (17, 7)]:
        shp = np.exp(-1j * (q.alp * i) * 0.3)
        for key in ("vor", "phi"):
            line = st[key][k, i]
            ext = np.append(line, line[0] * shp)
            want = _spline_ref(ye, ext.real, y) + 1j * _spline_ref(ye, ext.imag, y)
            np.testing.assert_allclose(got[key][k, i], want, rtol=0, atol=1e-14 * np.abs(line).max())
    np.testing.assert_allclose(got["u00"], _spline_ref(ye, np.append(st["u00"], st["u00"][0]), y),
                               rtol=0, atol=1e-14 * np.abs(st["u00"]).max())
    # a line smooth in y is reproduced to the spline's accuracy (largest next
    # to the ends, where the natural spline's zero curvature is imposed)
    p2 = sb.make_params(**box_params(64, 32, 32, 1000.0))
    st2 = {key: np.zeros_like(st[key]) for key in ("vor", "phi")}
    y32 = np.arange(32) * (p2.Ly / 32) - p2.Ly / 2
    st2["vor"][1, 0] = np.exp(1j * 2 * np.pi / p2.Ly * y32)  # one y wave, kx = 0
    st2["vor"][sb.sizes(p2)["mz"] - 1, 0] = np.conj(st2["vor"][1, 0])
    st2.update(phi=st2["phi"], u00=np.cos(2 * np.pi / p2.Ly * y32), w00=np.zeros(32), time=0.0,
               xoffb=0.0, xofft=0.0)
    f2 = tmp_path / "s2.bin"
    sb.write_restart(f2, p2, st2)
    got2, _ = sb.read_restart(f2, q)
    err = np.abs(got2["vor"][1, 0] - np.exp(1j * 2 * np.pi / q.Ly * y))
    assert err.max() < 2e-3 and err[8:40].max() < 1e-4
    assert np.abs(got2["u00"] - np.cos(2 * np.pi / q.Ly * y)).max() < 2e-3


@pytest.mark.parametrize("ncopy", [3, 5])
def test_y_stack_copies(tmp_path, ncopy):
    """my = 3 or 5 x the file's (ncopy_y, readwrite.f90:449-489): the box
    stacked in y, copy n times exp(-i kx xofft n), offsets times ncopy."""
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    q = sb.make_params(**dict(box_params(64, 32 * ncopy, 32, 1000.0), Ly=p.Ly * ncopy))
    st = _conj_state(sb.seed_state(p, 5), p)
    st.update(xoffb=-0.2, xofft=0.2)
    f = tmp_path / "c.bin"
    sb.write_restart(f, p, st)
    got, info = sb.read_restart(f, q)
    assert info.ymap == 2 and info.ncopy == ncopy
    assert np.isclose(got["xofft"], 0.2 * ncopy) and np.isclose(got["xoffb"], -0.2 * ncopy)
    kx = q.alp * np.arange(sb.sizes(q)["nkx"])
    for n in range(ncopy):
        ph = np.exp(-1j * kx * 0.2 * n)[None, :, None]
        for key in ("vor", "phi"):
            np.testing.assert_allclose(got[key][:, :, 32 * n:32 * (n + 1)], st[key] * ph,
                                       rtol=0, atol=1e-15 * np.abs(st[key]).max())
        np.testing.assert_array_equal(got["u00"][32 * n:32 * (n + 1)], st["u00"])


def test_y_half_and_x_half(tmp_path):
    """my = file my / 2 keeps every other plane (ihalfy); a doubled alp with
    half the x points keeps the even kx modes and the offsets (ihalf,
    readwrite.f90:152-171,229-239)."""
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    st = _conj_state(sb.seed_state(p, 6), p)
    st.update(xoffb=-0.4, xofft=0.4)
    f = tmp_path / "h.bin"
    sb.write_restart(f, p, st)
    qy = sb.make_params(**box_params(64, 16, 32, 1000.0))
    got, info = sb.read_restart(f, qy)
    assert info.ymap == 1
    np.testing.assert_array_equal(got["vor"], st["vor"][:, :, ::2])
    np.testing.assert_array_equal(got["w00"], st["w00"][::2])
    qx = sb.make_params(**dict(box_params(32, 32, 32, 1000.0), alp=2 * p.alp))
    got, info = sb.read_restart(f, qx)
    nk = sb.sizes(qx)["nkx"]
    assert info.xskip == 2 and (got["xoffb"], got["xofft"]) == (-0.4, 0.4)
    klen = (sb.sizes(qx)["mz"] + 1) // 2
    np.testing.assert_array_equal(got["phi"][:klen, :nk], st["phi"][:klen, 0:2 * nk:2])


def test_rescaling_of_gam_and_re(tmp_path):
    """getfil's rescaling (readwrite.f90:427-442): a changed gam scales u00,
    w00 by gam_file/gam, phi by gam/gam_file and vor by (gam_file/gam)
    sqrt(Re/Re_file); a changed Re alone scales vor by sqrt(Re/Re_file)
    unless the vorticity is kept (the Newton drivers), and never with LES."""
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    st = _conj_state(sb.seed_state(p, 8), p)
    f = tmp_path / "r.bin"
    sb.write_restart(f, p, st)
    q = sb.make_params(**dict(box_params(64, 32, 32, 2000.0)))
    got, _ = sb.read_restart(f, q)
    np.testing.assert_allclose(got["vor"], st["vor"] * np.sqrt(q.Re / p.Re), rtol=1e-15)
    np.testing.assert_array_equal(got["phi"], st["phi"])
    got, _ = sb.read_restart(f, q, keep_vor=True)
    np.testing.assert_array_equal(got["vor"], st["vor"])
    got, _ = sb.read_restart(f, sb.make_params(**dict(box_params(64, 32, 32, 2000.0), les=1)))
    np.testing.assert_array_equal(got["vor"], st["vor"])
    qg = sb.make_params(**dict(box_params(64, 32, 32, 1000.0), gam=2.0))
    got, _ = sb.read_restart(f, qg)
    np.testing.assert_allclose(got["u00"], st["u00"] * 0.5, rtol=1e-15)
    np.testing.assert_allclose(got["phi"], st["phi"] * 2.0, rtol=1e-15)
    np.testing.assert_allclose(got["vor"], st["vor"] * 0.5, rtol=1e-15)
