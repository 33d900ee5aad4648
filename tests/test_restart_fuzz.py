"""The restart reader (getfil, readwrite.f90:72-447) on damaged files: cut at
and around every record boundary, wrong record markers, absurd grid sizes
and counts in the header and footer, non-finite parameters and random byte
changes.  Every read either succeeds or returns error 8 (malformed) or 9
(unsupported grid change) with a message: no crash, no read past a record.
The reads run in a child process so that a crash fails the test instead of
ending the session."""
import os
import shutil
import struct
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, box_params

CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import shear_nnf_gb300 as sb
p = sb.make_params(mgalx=64, my=32, mgalz=32, Re=25.0, alp=0.5, Ly=6.283185307179586,
                   gam=1.0, s=1.0, chi=0.0, CFL=0.5)
for path in sys.argv[2:]:
    for q in (p, None):
        try:
            sb.read_restart(path, q)
            print("ok")
        except sb.ShearBoxError as e:
            print(str(e).split(":")[0])
"""


def _cases(data, bounds, rng):
    """The damaged files; the first ones are cut inside a record of the state
    (the footer's four records are optional, as in old files, and are read
    leniently: a file cut in its footer reads as one without it)."""
    out = []
    for b, n in bounds[:-4]:
        for cut in (b + 2, b + 4, b + 4 + n // 2, b + 4 + n, b + 4 + n + 2):
            out.append(bytes(data[:cut]))
    ncut = len(out)
    for b, n in bounds[-4:]:
        for cut in (b + 2, b + 4 + n // 2, b + 4 + n):
            if cut < len(data):
                out.append(bytes(data[:cut]))
    for b, n in bounds:
        if b > 0:
            out.append(bytes(data[:b]))  # cut at a record boundary
        for val in (-1, 0, n - 8, n + 8, 2 ** 31 - 1, -2 ** 31):
            for at in (b, b + 4 + n):
                buf = bytearray(data)
                struct.pack_into("<i", buf, at, val)
                out.append(bytes(buf))
    # grid sizes of record 1 and mx, my, mz of record 2
    for off in [4, 8, 12, 16] + [bounds[1][0] + 4 + k for k in (56, 60, 64)]:
        for val in (-5, 0, 1, 3, 100000, 2 ** 31 - 1):
            buf = bytearray(data)
            struct.pack_into("<i", buf, off, val)
            out.append(bytes(buf))
    # time, Re, alp, Ly/pi, gam, s, chi
    for k in range(7):
        for val in (0.0, -1.0, float("nan"), float("inf")):
            buf = bytearray(data)
            struct.pack_into("<d", buf, bounds[1][0] + 4 + 8 * k, val)
            out.append(bytes(buf))
    # the footer's counts and switches
    for b, n in bounds[-4:]:
        for k in range(0, n, 4):
            for val in (-1, 33, 2 ** 31 - 1):
                buf = bytearray(data)
                struct.pack_into("<i", buf, b + 4 + k, val)
                out.append(bytes(buf))
    for _ in range(150):
        buf = bytearray(data)
        for _ in range(int(rng.integers(1, 6))):
            lim = 2000 if rng.random() < 0.5 else len(buf)
            buf[int(rng.integers(0, lim))] = int(rng.integers(0, 256))
        out.append(bytes(buf))
    return out, ncut


# the reader alone (sb_io.cpp) under AddressSanitizer and UBSan: every case
# read onto a 64x32x32 grid and header-only
HARNESS = r"""
#include <cstdio>
#include <string>
#include <vector>
#include "shearbox.h"
namespace sb {
std::string g_msg;
void set_error(const std::string &m) { g_msg = m; }
}  // namespace sb
int main(int argc, char **argv) {
  sb_params p{};
  p.mgalx = 64; p.my = 32; p.mgalz = 32; p.Re = 25.0; p.alp = 0.5;
  p.Ly = 6.283185307179586; p.gam = 1.0; p.s = 1.0; p.CFL = 0.5; p.nhist = 1;
  std::vector<double> vor(2 * 21 * 19 * 32), phi(vor.size()), u00(32), w00(32);
  int bad = 0;
  for (int i = 1; i < argc; i++) {
    sb_restart_info info;
    bad += sb_read_restart(argv[i], nullptr, nullptr, nullptr, nullptr, nullptr, &info) != 0;
    bad += sb_read_restart_ex(argv[i], &p, 0, vor.data(), phi.data(), u00.data(), w00.data(),
                              &info) != 0;
  }
  std::printf("failed reads %d\n", bad);
  return 0;
}
"""


def _write_cases(tmp_path):
    import shear_nnf_gb300 as sb
    p = sb.make_params(**box_params(64, 32, 32, 1000.0))
    good = tmp_path / "good.bin"
    sb.write_restart(good, p, sb.seed_state(p, 1))
    data = bytearray(open(good, "rb").read())
    bounds, pos = [], 0
    while pos < len(data):
        n = struct.unpack_from("<i", data, pos)[0]
        bounds.append((pos, n))
        pos += 8 + n
    # 4 header records, the mean profiles, one record per plane, the footer
    assert pos == len(data) and len(bounds) == 5 + p.my + 4
    cases, ncut = _cases(data, bounds, np.random.default_rng(0))
    paths = []
    for i, c in enumerate(cases):
        f = tmp_path / f"c{i:04d}.bin"
        f.write_bytes(c)
        paths.append(str(f))
    return paths, ncut


def test_damaged_restart_files_fail_cleanly(tmp_path):
    paths, ncut = _write_cases(tmp_path)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, *paths], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    outcomes = r.stdout.splitlines()
    assert len(outcomes) == 2 * len(paths)
    kinds = set(outcomes)
    assert kinds <= {"ok", "shearbox error 8", "shearbox error 9"}, kinds
    # a file cut inside a record of the state is malformed for the full read
    # (outcomes come in pairs: the read onto the grid, then the header-only
    # read)
    assert all(o == "shearbox error 8" for o in outcomes[0:2 * ncut:2])
    assert outcomes.count("shearbox error 8") > len(paths) // 2


def test_damaged_restart_files_under_address_sanitizer(tmp_path):
    """The same cases through the reader built with -fsanitize=address,undefined:
    no invalid access, leak or undefined behaviour is reported."""
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "harness.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "harness"
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-I", os.path.join(ROOT, "include"),
           "-x", "c++", os.path.join(ROOT, "shear_nnf_gb300", "csrc", "sb_io.cpp"),
           str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]
    paths, _ = _write_cases(tmp_path)
    r = subprocess.run([str(exe), *paths], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "Sanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]
    assert r.stdout.startswith("failed reads ")
