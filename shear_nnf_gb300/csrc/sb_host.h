// sb_host.h -- host-side set-up of the shearing-box step (no CUDA calls).
#pragma once
#include <stdint.h>
#include <vector>

namespace sbh {

// Compact-scheme coefficients of the spectral-like heptadiagonal schemes
// (diffy_shear_hepta.f90:68-296): B u' = A u with B = pr1, A = rh1h/h, and
// B u'' = A u with B = pr2, A = rh2h/h^2.  Arrays are a(-3..3) stored [d+3].
struct Coeffs {
  double pr1[7], rh1h[7], pr2[7], rh2h[7];
};
void compact_coeffs(Coeffs *c);

// Real base of the cyclic LDL^H factorisation of the band matrix a(-3..3) of
// size n with the shear phase factored out: for shp = 1 the factorisation of
// modChol7cyclic_cmplx (diffy_shear_hepta.f90:578-755) is real; for a general
// shp the first n-6 / n-5 / n-4 entries of the three border rows are this base
// times shp, and only a few tail entries depend on shp non-linearly.
// Outputs 0-based rows q = i-1; entries outside their definition range are 0.
struct BaseFac {
  std::vector<double> La, Lb, Lc, Dd, Ddm1, e, f, g;
  double sums[6];  // See Sfe Sff Sge Sgf Sgg
};
void base_factor(const double a[7], int n, BaseFac *out);

// Seeded divergence-free initial field (synthetic stand-in for the reference's
// getini spectrum, initcr.f90:664-822): random-phase Fourier modes with energy
// spectrum E(k) ~ k^4 exp(-2 (k/k0)^2), rms velocity urms.  Outputs the
// reference pencil layout: vor/phi complex (0:my1, 0:mx1, 0:mz1) as
// interleaved doubles, u00/w00 real (my).
int seed_state(int mgalx, int my, int mgalz, double alp, double gam, double Ly,
               uint64_t seed, double k0, double urms, double *vor, double *phi,
               double *u00, double *w00);

}  // namespace sbh
