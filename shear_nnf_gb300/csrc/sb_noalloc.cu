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
#include <string>
#include <vector>

#include "../../include/shearbox.h"
#include "sb_common.cuh"
#include "sb_fac.h"
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

// Address of the scratch array in the current device's context.  Looked up on
// every call (no synchronisation, no allocation): a cached address would go
// stale if the context were torn down and the module loaded again elsewhere.
int scratch_address(double **out, std::string *err) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return 3;
  }
  *out = (double *)p;
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
  // the operator's factor block and the shear phases, one copy into the scratch
  HostFac hf;
  double r[4];
  int anti;
  const std::vector<double> host = derivyc_block(my, Ly, iord, nlines, shp, shm, &hf, r, &anti);
  const size_t nfac = hf.buf.size();  // 8*my + 10 <= kFac
  double *dfac = base;
  double *dsh = base + kFac;
  double *ybuf = base + kFac + 4 * kLines;
  cudaError_t e = cudaMemcpyAsync(dfac, host.data(), sizeof(double) * nfac,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dsh, host.data() + nfac, sizeof(double) * 4 * (size_t)nlines,
                        cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    *err = std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e);
    return 3;
  }
  const Fac F = fac_bind(hf, dfac);
  e = launch_op_line(nlines, my, u, ldu, out, ldo, ybuf, F, dsh, dsh + 2 * nlines, r, anti, st);
  // the copies read the pageable host block: wait before it goes out of scope
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    *err = std::string("derivyc launch: ") + cudaGetErrorString(e);
    return 3;
  }
  return 0;
}
}  // namespace sb
