"""include/shearbox.h from a C caller: a C99 program compiled with gcc
(-Wall -Wextra -Werror -pedantic) against the header and linked to the
library calls the host-only entry points -- sizes, the escru writer, the getfil
reader with and without a grid, an I/O error -- and its results equal the
Python binding's.  No GPU: these entry points make no CUDA call."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, box_params

C_SOURCE = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "shearbox.h"

static int fail(const char *what) {
  fprintf(stderr, "%s: %s\n", what, sb_last_error());
  return 1;
}

static int read_all(FILE *f, double *dst, long n) {
  return fread(dst, sizeof(double), (size_t)n, f) == (size_t)n ? 0 : 1;
}

int main(int argc, char **argv) {
  sb_params p;
  sb_restart_info info;
  int sz[8], rc;
  long n, my;
  double *vor, *phi, *u00, *w00, sc[3];
  FILE *f;
  if (argc != 4) return 2;
  memset(&p, 0, sizeof p);
  p.mgalx = 64;
  p.my = 32;
  p.mgalz = 32;
  p.Re = 25.0;
  p.alp = 0.5;
  p.Ly = 6.283185307179586;
  p.gam = 1.0;
  p.s = 1.0;
  p.CFL = 0.5;
  p.nhist = 1;
  if (sb_sizes(&p, sz)) return fail("sb_sizes");
  n = sz[7];
  my = sz[3];
  printf("sizes %d %d %d %d %d %d %d %d\n", sz[0], sz[1], sz[2], sz[3], sz[4], sz[5], sz[6],
         sz[7]);
  vor = malloc(sizeof(double) * 2 * n);
  phi = malloc(sizeof(double) * 2 * n);
  u00 = malloc(sizeof(double) * my);
  w00 = malloc(sizeof(double) * my);
  if (!vor || !phi || !u00 || !w00) return 3;
  /* the state: vor, phi, u00, w00, time, xoffb, xofft as raw doubles */
  f = fopen(argv[1], "rb");
  if (!f || read_all(f, vor, 2 * n) || read_all(f, phi, 2 * n) || read_all(f, u00, my) ||
      read_all(f, w00, my) || read_all(f, sc, 3))
    return 4;
  fclose(f);
  if (sb_write_restart(argv[2], &p, vor, phi, u00, w00, sc[0], sc[1], sc[2], 0.01))
    return fail("sb_write_restart");
  /* header only */
  memset(&info, 0, sizeof info);
  if (sb_read_restart(argv[2], NULL, NULL, NULL, NULL, NULL, &info))
    return fail("sb_read_restart (info)");
  printf("info %d %d %d %.17g %.17g %.17g\n", info.mgalx, info.my, info.mgalz, info.time,
         info.Re, info.xoffb);
  /* the state mapped on the run's grid */
  memset(vor, 0, sizeof(double) * 2 * n);
  memset(phi, 0, sizeof(double) * 2 * n);
  if (sb_read_restart(argv[2], &p, vor, phi, u00, w00, &info)) return fail("sb_read_restart");
  f = fopen(argv[3], "wb");
  if (!f) return 5;
  fwrite(vor, sizeof(double), (size_t)(2 * n), f);
  fwrite(phi, sizeof(double), (size_t)(2 * n), f);
  fwrite(u00, sizeof(double), (size_t)my, f);
  fwrite(w00, sizeof(double), (size_t)my, f);
  sc[0] = info.time;
  sc[1] = info.run_xoffb;
  sc[2] = info.run_xofft;
  fwrite(sc, sizeof(double), 3, f);
  fclose(f);
  /* a missing file is error 7 with a message */
  rc = sb_read_restart("no/such/file", NULL, NULL, NULL, NULL, NULL, &info);
  printf("missing %d %d\n", rc, (int)(strlen(sb_last_error()) > 0));
  free(vor);
  free(phi);
  free(u00);
  free(w00);
  printf("version %d\n", sb_version());
  return 0;
}
"""


@pytest.fixture(scope="module")
def c_program(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    from shear_nnf_gb300.buildlib import LIB, build
    build()
    d = tmp_path_factory.mktemp("c_caller")
    src = d / "caller.c"
    src.write_text(C_SOURCE)
    exe = d / "caller"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
           "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", os.path.dirname(LIB), "-lshearbox", "-Wl,-rpath," + os.path.dirname(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, d


def test_header_compiles_as_c99_and_the_host_entry_points_agree(c_program):
    import shear_nnf_gb300 as sb
    exe, d = c_program
    p = sb.make_params(**box_params(64, 32, 32, rez=25.0 * (2 * np.pi) ** 2))
    st = sb.seed_state(p, 21)
    st.update(time=1.25, xoffb=0.375, xofft=-0.125)
    raw_in, restart, raw_out = d / "in.bin", d / "state.rst", d / "out.bin"
    np.concatenate([st["vor"].ravel().view(np.float64), st["phi"].ravel().view(np.float64),
                    st["u00"], st["w00"], [st["time"], st["xoffb"], st["xofft"]]]).tofile(raw_in)
    r = subprocess.run([str(exe), str(raw_in), str(restart), str(raw_out)], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    s = sb.sizes(p)
    assert [int(v) for v in out["sizes"].split()] == [
        s["mx"], s["mz"], s["nkx"], p.my, s["nz"], p.mgalx, p.mgalz, s["nkx"] * s["mz"] * p.my]
    gx, gy, gz, t, re, xb = out["info"].split()
    assert (int(gx), int(gy), int(gz)) == (64, 32, 32)
    assert float(t) == 1.25 and float(re) == 25.0 and float(xb) == 0.375
    assert out["missing"] == "7 1"
    assert int(out["version"]) >= 1
    # the C reader's state equals the Python reader's bit for bit, and the
    # seeded state survives the round trip
    n = s["nkx"] * s["mz"] * p.my
    v = np.fromfile(raw_out)
    ref, info = sb.read_restart(str(restart), p)
    assert np.array_equal(v[: 2 * n], ref["vor"].ravel().view(np.float64))
    assert np.array_equal(v[2 * n: 4 * n], ref["phi"].ravel().view(np.float64))
    assert np.array_equal(v[4 * n: 4 * n + p.my], ref["u00"])
    assert np.array_equal(v[4 * n + p.my: 4 * n + 2 * p.my], ref["w00"])
    assert list(v[-3:]) == [ref["time"], ref["xoffb"], ref["xofft"]]
    for k in ("vor", "phi"):
        np.testing.assert_allclose(ref[k], st[k], rtol=0, atol=1e-15 * np.abs(st[k]).max())
    assert np.array_equal(ref["u00"], st["u00"]) and np.array_equal(ref["w00"], st["w00"])
