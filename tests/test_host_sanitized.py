"""The host set-up code that sb_create runs (sb_host.cpp: compact-scheme and
filter coefficients, the real base factorisations and segment tables of the
cyclic LDL^H solves, FFT twiddles, the seeded field) built with
AddressSanitizer and UBSan and run over every line length and segment count
the library accepts: no invalid access, leak or undefined behaviour, and the
factorisations reproduce their band matrices."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <vector>
#include "sb_host.h"

// the cyclic band matrix a(-3..3) of size n times the LDL^T factors of the
// banded part, compared where both are defined (rows 1..n-3 of the band)
static double band_residual(const double a[7], int n, const sbh::BaseFac &f) {
  double worst = 0.0;
  const int nb = n - 3;  // banded rows
  for (int i = 0; i < nb; i++) {
    for (int d = 0; d <= 3; d++) {
      const int j = i - d;
      if (j < 0) continue;
      // (L D L^T)_{i,j} = sum_k L_{i,k} D_k L_{j,k}, L unit lower with
      // sub-diagonals La (1), Lb (2), Lc (3)
      auto L = [&](int r, int c) -> double {
        if (r == c) return 1.0;
        const int s = r - c;
        if (s == 1) return f.La[r];
        if (s == 2) return f.Lb[r];
        if (s == 3) return f.Lc[r];
        return 0.0;
      };
      double v = 0.0;
      for (int k = (i - 3 > 0 ? i - 3 : 0); k <= j; k++) v += L(i, k) * f.Dd[k] * L(j, k);
      worst = std::fmax(worst, std::fabs(v - a[3 - d]));
    }
  }
  return worst;
}

int main() {
  sbh::Coeffs c;
  sbh::compact_coeffs(&c);
  double flhs[7], frhs[9];
  sbh::filter_coeffs(flhs, frhs);
  double worst = 0.0;
  int nfac = 0;
  for (int n = 16; n <= 512; n += (n < 64 ? 1 : 16)) {
    const double h = 2.0 * M_PI / n;
    for (int m = 0; m < 4; m++) {
      double a[7];
      for (int d = 0; d < 7; d++) {
        if (m == 0) a[d] = c.pr1[d];
        else if (m == 1) a[d] = c.pr2[d];
        else if (m == 2) a[d] = flhs[d];
        else a[d] = c.rh2h[d] / (h * h) - 9.0 * c.pr2[d];  // a Helmholtz band, k^2 = 9
      }
      sbh::BaseFac f;
      sbh::base_factor(a, n, &f);
      nfac++;
      if (m < 3) worst = std::fmax(worst, band_residual(a, n, f) / (std::fabs(a[3]) + 1e-300));
      for (int nseg = 1; nseg <= 3; nseg++) {
        if ((n - 3) / nseg < 6) continue;
        sbh::SegPlan plan;
        sbh::seg_plan(n, nseg, &plan);
        sbh::SegFac sf;
        sbh::seg_factor(f, n, plan, &sf);
      }
    }
  }
  const int lens[] = {32, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384};
  for (int n : lens) {
    std::vector<double> t = sbh::fft_twiddles(n), tf = sbh::fft_twiddles_factored(n);
    if (t.size() != 2 * (size_t)n || tf.empty()) return 3;
  }
  const int grids[][3] = {{64, 32, 32}, {96, 48, 48}, {192, 96, 96}, {80, 16, 160}};
  for (const auto &g : grids) {
    const int mx = 2 * (g[0] / 3), mz = 2 * (g[2] / 3) - 1;
    std::vector<double> vor(2 * (size_t)(mx / 2) * mz * g[1]), phi(vor.size()), u00(g[1]),
        w00(g[1]);
    if (sbh::seed_state(g[0], g[1], g[2], 0.5, 1.0, 2.0 * M_PI, 7, 4.0, 0.1, vor.data(),
                        phi.data(), u00.data(), w00.data()))
      return 4;
  }
  std::printf("factorisations %d worst band residual %.3e\n", nfac, worst);
  return worst < 1e-12 ? 0 : 5;
}
"""


def test_host_setup_under_address_sanitizer(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "harness.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "harness"
    csrc = os.path.join(ROOT, "shear_nnf_gb300", "csrc")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-ffp-contract=off", "-I", csrc,
           os.path.join(csrc, "sb_host.cpp"), str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert "Sanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]
    assert r.returncode == 0, r.stdout + r.stderr[-2000:]
    assert r.stdout.startswith("factorisations ")
