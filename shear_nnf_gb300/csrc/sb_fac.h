// sb_fac.h -- host staging of the factor tables of one y operator (internal).
//
// The operator entry points (sb_op_derivyc, sb_op_lapcdy, sb_op_filterc and
// the allocation-free derivyc) all hand the device the same packed block: the
// real base factorisation of the band (La Lb Lc Ddm1 Dd e f g, n rows each,
// per line when the band differs per line) followed by the six border sums and
// the band's diagonal a(0..3).  This header is the one place that layout is
// written down on the host.
#pragma once
#include <vector>

#include "sb_common.cuh"
#include "sb_host.h"

namespace sb {

// Factor tables of one operator staged on the host, packed into one buffer so
// that a single copy places them on the device.
struct HostFac {
  std::vector<double> buf;  // La Lb Lc Ddm1 Dd e f g (each n*lines) then sums (10*lines)
  long lines = 1, n = 0;
};

inline void host_fac_init(HostFac *h, long n, long lines) {
  h->n = n;
  h->lines = lines;
  h->buf.assign((size_t)(8 * n + 10) * lines, 0.0);
}

inline void host_fac_add(HostFac *h, long line, const sbh::BaseFac &b, const double a[7]) {
  const long n = h->n, L = h->lines;
  const std::vector<double> *arr[8] = {&b.La, &b.Lb, &b.Lc, &b.Ddm1, &b.Dd, &b.e, &b.f, &b.g};
  for (int q = 0; q < 8; q++)
    for (long j = 0; j < n; j++) h->buf[((long)q * n + j) * L + line] = (*arr[q])[j];
  for (int q = 0; q < 6; q++) h->buf[(8 * n + q) * L + line] = b.sums[q];
  for (int q = 0; q < 4; q++) h->buf[(8 * n + 6 + q) * L + line] = a[3 + q];
}

// Device view of a HostFac block copied to d.
inline Fac fac_bind(const HostFac &h, const double *d) {
  Fac F;
  const long n = h.n, L = h.lines;
  const double **dst[8] = {&F.La, &F.Lb, &F.Lc, &F.Ddm1, &F.Dd, &F.e, &F.f, &F.g};
  for (int q = 0; q < 8; q++) *dst[q] = d + (long)q * n * L;
  F.sums = d + 8 * n * L;
  F.stride = (L > 1) ? L : 0;
  return F;
}

// derivative operator d/dy (iord 1) or d2/dy2 (iord 2): band of the left-hand
// side and right-hand-side stencil (r0; r1..r3), antisymmetric for iord 1
inline void deriv_operator(int iord, double dy, const sbh::Coeffs &co, const double **a,
                           double r[4], int *anti) {
  if (iord == 1) {
    *a = co.pr1;
    r[0] = 0.0;
    for (int d = 1; d <= 3; d++) r[d] = co.rh1h[3 + d] / dy;
    *anti = 1;
  } else {
    *a = co.pr2;
    for (int d = 0; d <= 3; d++) r[d] = co.rh2h[3 + d] / (dy * dy);
    *anti = 0;
  }
}

// The packed derivyc block: the operator's HostFac, then shp and shm (2*nlines
// doubles each).  Returns the HostFac layout in *hf.
inline std::vector<double> derivyc_block(int my, double Ly, int iord, int nlines,
                                         const double *shp, const double *shm, HostFac *hf,
                                         double r[4], int *anti) {
  sbh::Coeffs co;
  sbh::compact_coeffs(&co);
  const double dy = Ly / (double)my;
  const double *a;
  deriv_operator(iord, dy, co, &a, r, anti);
  host_fac_init(hf, my, 1);
  sbh::BaseFac b;
  sbh::base_factor(a, my, &b);
  host_fac_add(hf, 0, b, a);
  const size_t nfac = hf->buf.size();
  std::vector<double> host(nfac + 4 * (size_t)nlines);
  std::copy(hf->buf.begin(), hf->buf.end(), host.begin());
  std::copy(shp, shp + 2 * (size_t)nlines, host.begin() + nfac);
  std::copy(shm, shm + 2 * (size_t)nlines, host.begin() + nfac + 2 * (size_t)nlines);
  return host;
}

}  // namespace sb
