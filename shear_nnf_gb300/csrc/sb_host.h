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

// Fixed coefficients of the compact y-filter (prefilter,
// filter_shear_hepta.f90:55-73): left-hand side lhs(-3..3) stored [d+3],
// right-hand side rhs(-4..4) stored [d+4]; unscaled.
void filter_coeffs(double lhs[7], double rhs[9]);

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

// Segmented solves: the banded rows 1..n-3 split into nseg consecutive
// segments solved in parallel.  For segment s (rows lo..hi, 1-based) and
// t = 1..3: hf[t-1][i-1] is the solution of the homogeneous forward recurrence
// h_i = -Lc_i h_{i-3} - Lb_i h_{i-2} - La_i h_{i-1} on lo..hi started from a unit
// value at row lo-t; hb[t-1][i-1] that of the backward recurrence
// g_i = -La_{i+1} g_{i+1} - Lb_{i+2} g_{i+2} - Lc_{i+3} g_{i+3} on hi..lo started from
// a unit value at row hi+t (segments below the top one only); ef[(s*3+q)*3+t-1]
// = sum over the segment of border-row base q (e, f, g) times hf.
struct SegPlan {
  int nseg, lo[4], hi[4];
};
void seg_plan(int n, int nseg, SegPlan *p);
struct SegFac {
  std::vector<double> hf[3], hb[3], ef;
};
void seg_factor(const BaseFac &b, int n, const SegPlan &p, SegFac *out);

// FFT twiddles of length n: the complex table e^{-2 pi i t/n} (t = 0..n-1,
// re/im interleaved) and its factored FP64 form for sb_fft.cuh: entry t =
// {mx, my, tau, swap} with e^{-2 pi i t/n} = (-i)^q c (1 + i tau), q the
// nearest quarter turn (so c >= cos(pi/4), |tau| <= 1), mx the signed c of the
// real output component, my = (odd q ? -mx : mx), swap = q & 1 stored as the
// bits of an integer.
std::vector<double> fft_twiddles(int n);
std::vector<double> fft_twiddles_factored(int n);

// Seeded divergence-free initial field (synthetic stand-in for the reference's
// getini spectrum, initcr.f90:664-822): random-phase Fourier modes with energy
// spectrum E(k) ~ k^4 exp(-2 (k/k0)^2), rms velocity urms.  Outputs the
// reference pencil layout: vor/phi complex (0:my1, 0:mx1, 0:mz1) as
// interleaved doubles, u00/w00 real (my).
int seed_state(int mgalx, int my, int mgalz, double alp, double gam, double Ly,
               uint64_t seed, double k0, double urms, double *vor, double *phi,
               double *u00, double *w00);

}  // namespace sbh
