"""The C oracle (the parity reference of every GPU test) built with
AddressSanitizer and UBSan and run through each variant of the step it
restates -- plain, LES, y dealiasing 1/2, the y filter, the temperature,
the semi-implicit branch with and without the temperature, damping and
forcing -- plus its operators: no invalid access, leak or undefined
behaviour, and every run ends with finite fields."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "shearbox_oracle.h"

static int finite_all(const double *v, long n) {
  for (long i = 0; i < n; i++)
    if (!isfinite(v[i])) return 0;
  return 1;
}

static int run(const char *name, orc_params p, int nstep) {
  void *h = orc_create(&p);
  if (!h) return 1;
  int sz[8];
  orc_sizes(h, sz);
  const long nb = sz[7], my = sz[3];
  double *vor = calloc(nb, 8), *phi = calloc(nb, 8), *tb = calloc(nb, 8);
  double *u00 = calloc(my, 8), *w00 = calloc(my, 8), *tb00 = calloc(my, 8);
  double *trace = calloc((size_t)(nstep + 1) * ORC_TRACE_LEN_T, 8);
  if (!vor || !phi || !tb || !u00 || !w00 || !tb00 || !trace) return 2;
  orc_seed_state(p.mgalx, p.my, p.mgalz, p.alp, p.gam, p.Ly, 5, 4.0, 0.1 * p.Ly, vor, phi, u00,
                 w00);
  for (long i = 0; i < nb; i++) tb[i] = 0.01 * vor[i];
  double time = 0, xb = 0.1, xt = -0.1, dt = 0;
  int ntr = 0, istop = 0, rc;
  if (p.temperature)
    rc = orc_crosst(h, vor, phi, u00, w00, tb, tb00, &time, &xb, &xt, nstep, trace, &ntr,
                    &istop, &dt);
  else
    rc = orc_cross(h, vor, phi, u00, w00, &time, &xb, &xt, nstep, trace, &ntr, &istop, &dt);
  /* the steps done (cross.f90's loop ran to nstep) */
  int ok = rc == nstep && finite_all(vor, nb) && finite_all(phi, nb) && finite_all(u00, my) &&
           (!p.temperature || finite_all(tb, nb));
  /* statistics and physical fields of the final state */
  double *stats = calloc(64 * my, 8), *stats2 = calloc(64 * my, 8);
  double *spec = calloc(8 * nb, 8), *spec2 = calloc(8 * nb, 8);
  double *tst = calloc(8 * my, 8), *tsp = calloc(4 * nb, 8), tot = 0;
  int nac = 0;
  orc_statistics(h, stats, stats2, spec, spec2, tst, tsp, &nac, &tot);
  double *phys = calloc((size_t)11 * my * p.mgalz * p.mgalx, 8);
  if (orc_physical(h, vor, phi, u00, w00, xb, xt, 0x7ff, phys) != 11) ok = 0;  /* fields */
  if (!finite_all(phys, (long)11 * my * p.mgalz * p.mgalx)) ok = 0;
  printf("%s rc %d steps %d ok %d\n", name, rc, ntr, ok);
  free(vor); free(phi); free(tb); free(u00); free(w00); free(tb00); free(trace);
  free(stats); free(stats2); free(spec); free(spec2); free(tst); free(tsp); free(phys);
  orc_destroy(h);
  return ok ? 0 : 3;
}

int main(void) {
  orc_set_threads(1);
  orc_params b;
  memset(&b, 0, sizeof b);
  b.mgalx = 64; b.my = 32; b.mgalz = 32;
  b.Re = 1000.0 / (4.0 * M_PI * M_PI); b.alp = 0.5; b.Ly = 2.0 * M_PI; b.gam = 1.0;
  b.s = 1.0; b.CFL = 0.5; b.fixed_dt = 0.005; b.nhist = 1; b.keep_laminar = 1;
  int bad = 0;
  orc_params p = b;
  bad += run("plain", p, 3);
  p = b; p.les = 1; p.les_visc = 1; p.cs = 0.1;
  bad += run("les", p, 3);
  p = b; p.ydeal = 1;
  bad += run("ydeal1", p, 2);
  p = b; p.ydeal = 2;
  bad += run("ydeal2", p, 2);
  p = b; p.ydeal = 3;
  bad += run("yfilter", p, 2);
  p = b; p.temperature = 1; p.fkappa = 0.01; p.bym = 1.0; p.gbeta = 0.5;
  bad += run("temperature", p, 3);
  p = b; p.implicit_visc = 1;
  bad += run("implicit", p, 3);
  p = b; p.implicit_visc = 1; p.temperature = 1; p.fkappa = 0.01; p.bym = 1.0; p.gbeta = 0.5;
  bad += run("implicit-temperature", p, 3);
  p = b; p.damping = 1; p.damp_up = 0.5; p.damp_aa = 0.2; p.force = 1; p.force_roll = 0.01;
  bad += run("damping-force", p, 2);
  p = b; p.mgalx = 96; p.my = 48; p.mgalz = 48; p.fixed_dt = 0;
  bad += run("cfl-96", p, 2);
  /* the operators on one line */
  void *h = orc_create(&b);
  double u[64], du[64], pp[64], phys[66 * 32];
  for (int j = 0; j < 64; j++) u[j] = sin(0.3 * j);
  orc_derivyc(h, u, du, 0.8, 0.6, 0.8, -0.6, 1, 2);
  orc_derivyc(h, u, du, 0.8, 0.6, 0.8, -0.6, 2, 2);
  orc_lapcdy(h, u, 4.0, pp, 0.8, 0.6, 0.8, -0.6, 2);
  orc_filterc(h, u, du, 0.8, 0.6, 2);
  orc_cfty(h, u, -1);
  orc_cfty(h, u, 1);
  double fou[2 * 21 * 19];
  for (int i = 0; i < 2 * 21 * 19; i++) fou[i] = cos(0.1 * i);
  orc_fourxz(h, fou, phys, 1);
  orc_fourxz(h, fou, phys, -1);
  orc_destroy(h);
  printf("bad %d\n", bad);
  return bad;
}
"""


def test_oracle_under_address_sanitizer(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "harness.c"
    src.write_text(HARNESS)
    exe = tmp_path / "harness"
    odir = os.path.join(ROOT, "oracle")
    cmd = ["gcc", "-std=gnu11", "-O1", "-g", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-Wno-unknown-pragmas", "-I", odir,
           os.path.join(odir, "shearbox_oracle.c"), str(src), "-o", str(exe), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    assert "Sanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]
    assert r.returncode == 0, r.stdout + r.stderr[-2000:]
    assert r.stdout.strip().endswith("bad 0")
