// sb_noalloc.cu -- allocation-free variant of the derivyc operator.
//
// Some callers cannot allocate device memory at the point where they need the
// y-derivative: an application that has handed all device memory to its own
// pool, or a loop that must not pay the synchronisation an allocation may
// cause.  sb_op_derivyc_noalloc serves them: its scratch (factor tables, shear
// phases, forward-substitution buffer) lives in a fixed array of this file
// that every GPU which loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/shearbox.h"
#include "sb_common.cuh"
#include "sb_host.h"
#include "sb_kernels.h"

namespace {

// Limits of the scratch array (see shearbox.h): my <= SB_MAX_NY points per line,
// my * pad32(2*nlines) <= SB_NOALLOC_YBUF doubles, nlines <= SB_NOALLOC_LINES.
constexpr long kYbuf = SB_NOALLOC_YBUF;
constexpr long kLines = SB_NOALLOC_LINES;
constexpr long kFac = 8L * SB_MAX_NY + 16;
constexpr long kTotal = kFac + 4 * kLines + kYbuf;

// The device-side scratch.  In host code this name is only a stand-in for the
// symbol: kernels are given the address from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_scratch[kTotal];

std::mutex g_mu;
std::vector<double *> g_addr;  // per device ordinal, nullptr until set up

// Address of the scratch array on the current device (set-up once per device,
// with that device current).
int scratch_address(double **out, std::string *err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return 3;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if ((int)g_addr.size() <= dev) g_addr.resize(dev + 1, nullptr);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return 3;
    }
    g_addr[dev] = (double *)p;
  }
  *out = g_addr[dev];
  return 0;
}

}  // namespace

namespace sb {
int noalloc_derivyc(int my, double Ly, int iord, int nlines, const double *u, long ldu,
                    double *out, long ldo, const double *shp, const double *shm, void *stream,
                    std::string *err) {
  if (my < 16 || my > SB_MAX_NY) {
    *err = "my outside 16..512";
    return 1;
  }
  if (iord != 1 && iord != 2) {
    *err = "iord must be 1 or 2";
    return 1;
  }
  if (!(Ly > 0) || nlines < 1 || !u || !out || !shp || !shm || ldu < nlines || ldo < nlines) {
    *err = "invalid argument";
    return 1;
  }
  const long nthr = op_threads(nlines);
  if (nlines > kLines || (long)my * nthr > kYbuf) {
    char b[256];
    snprintf(b, sizeof(b),
             "sb_op_derivyc_noalloc: %d lines of %d points exceed the fixed scratch "
             "(nlines <= %ld and my*pad32(2*nlines) <= %ld)",
             nlines, my, kLines, kYbuf);
    *err = b;
    return 6;
  }
  double *base = nullptr;
  int rc = scratch_address(&base, err);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // host-side tables: factor arrays of the operator, then the shear phases
  sbh::Coeffs co;
  sbh::compact_coeffs(&co);
  const double dy = Ly / (double)my;
  const double *a = (iord == 1) ? co.pr1 : co.pr2;
  double r[4];
  int anti;
  if (iord == 1) {
    r[0] = 0.0;
    for (int d = 1; d <= 3; d++) r[d] = co.rh1h[3 + d] / dy;
    anti = 1;
  } else {
    for (int d = 0; d <= 3; d++) r[d] = co.rh2h[3 + d] / (dy * dy);
    anti = 0;
  }
  sbh::BaseFac b;
  sbh::base_factor(a, my, &b);
  const long n = my;
  std::vector<double> host(8 * n + 10 + 4 * (size_t)nlines, 0.0);
  const std::vector<double> *arr[8] = {&b.La, &b.Lb, &b.Lc, &b.Ddm1, &b.Dd, &b.e, &b.f, &b.g};
  for (int q = 0; q < 8; q++)
    for (long j = 0; j < n; j++) host[q * n + j] = (*arr[q])[j];
  for (int q = 0; q < 6; q++) host[8 * n + q] = b.sums[q];
  for (int q = 0; q < 4; q++) host[8 * n + 6 + q] = a[3 + q];
  double *dfac = base;
  double *dsh = base + kFac;
  double *ybuf = base + kFac + 4 * kLines;
  for (long q = 0; q < 2L * nlines; q++) {
    host[8 * n + 10 + q] = shp[q];
    host[8 * n + 10 + 2L * nlines + q] = shm[q];
  }
  cudaError_t e = cudaMemcpyAsync(dfac, host.data(), sizeof(double) * (8 * n + 10),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dsh, host.data() + 8 * n + 10, sizeof(double) * 4 * (size_t)nlines,
                        cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    *err = std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e);
    return 3;
  }
  Fac F;
  F.La = dfac;
  F.Lb = dfac + n;
  F.Lc = dfac + 2 * n;
  F.Ddm1 = dfac + 3 * n;
  F.Dd = dfac + 4 * n;
  F.e = dfac + 5 * n;
  F.f = dfac + 6 * n;
  F.g = dfac + 7 * n;
  F.sums = dfac + 8 * n;
  F.stride = 0;
  e = launch_op_line(nlines, my, u, ldu, out, ldo, ybuf, F, dsh, dsh + 2 * nlines, r, anti, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    *err = std::string("derivyc launch: ") + cudaGetErrorString(e);
    return 3;
  }
  return 0;
}
}  // namespace sb
