// sb_ops.cu -- standalone y-line operators: derivyc and lapcdy on batches of
// device-resident complex lines (diffy_shear_hepta.f90:333-525).  Line data is
// [j][line] complex: element (line, j) at base + 2*(j*ld + line).
#include <cuda_runtime.h>

#include "sb_common.cuh"
#include "sb_kernels.h"
#include "sb_line.cuh"

namespace sb {

// one lane per (line, component); lane t keeps its forward substitution in
// column t of ybuf ([N][nthr] doubles)
__global__ void __launch_bounds__(128) k_op_line(int nlines, int N, const double *u, long ldu,
                                                 double *out, long ldo, double *ybuf, long nthr,
                                                 Fac F, const double *shp, const double *shm,
                                                 double r0, double r1, double r2, double r3,
                                                 int anti) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nthr) return;  // nthr is a multiple of 32: whole warps leave together
  const int c = (int)(t & 1);
  long line = t >> 1;
  const bool active = line < nlines;
  if (!active) line = nlines - 1;
  const cd sp = mk(shp[2 * line], shp[2 * line + 1]);
  const cd sm = mk(shm[2 * line], shm[2 * line + 1]);
  const FacView V(F, line);
  const Tail T = make_tail(V, sp, N);
  solve_line(u + 2 * line + c, 2 * ldu, ybuf + t, nthr, N, V, T, sp, sm, c, r0, r1, r2, r3,
             anti != 0, [&](int j, double x) {
               if (active) out[2 * ((long)j * ldo + line) + c] = x;
             });
}

long op_threads(int nlines) { return ((2L * nlines + 31) / 32) * 32; }

// right-hand side of the compact y-filter (matvecNcyclic with na = 4,
// diffy_shear_hepta.f90:960-996): one thread per (line, row, component);
// rows wrapped around the line take u(y-Ly) = conj(shp) u and u(y+Ly) = shp u
__global__ void k_filter_rhs(int nlines, int N, const double *u, long ldu, double *out, long ldo,
                             const double *shp, double r0, double r1, double r2, double r3,
                             double r4) {
  const long n = 2L * N * nlines;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t & 1);
    const long q = t >> 1;
    const int line = (int)(q % nlines), j = (int)(q / nlines);
    const cd sp = mk(shp[2 * line], shp[2 * line + 1]);
    const double rr[5] = {r0, r1, r2, r3, r4};
    double s = 0.0;
    for (int d = -4; d <= 4; d++) {
      int jj = j + d;
      cd ph = mk(1.0, 0.0);
      if (jj < 0) {
        jj += N;
        ph = cj(sp);
      } else if (jj >= N) {
        jj -= N;
        ph = sp;
      }
      const cd v = mk(u[2 * ((long)jj * ldu + line)], u[2 * ((long)jj * ldu + line) + 1]);
      const cd w = ph * v;
      s += rr[d < 0 ? -d : d] * (c ? w.y : w.x);
    }
    out[2 * ((long)j * ldo + line) + c] = s;
  }
}

cudaError_t launch_filter_rhs(int nlines, int N, const double *u, long ldu, double *out, long ldo,
                              const double *shp, const double r[5], cudaStream_t st) {
  k_filter_rhs<<<256, 256, 0, st>>>(nlines, N, u, ldu, out, ldo, shp, r[0], r[1], r[2], r[3], r[4]);
  return cudaGetLastError();
}

cudaError_t launch_op_line(int nlines, int N, const double *u, long ldu, double *out, long ldo,
                           double *ybuf, const Fac &F, const double *shp, const double *shm,
                           const double r[4], int anti, cudaStream_t st) {
  const long nthr = op_threads(nlines);
  const int T = 128;
  k_op_line<<<(unsigned)((nthr + T - 1) / T), T, 0, st>>>(nlines, N, u, ldu, out, ldo, ybuf, nthr,
                                                         F, shp, shm, r[0], r[1], r[2], r[3], anti);
  return cudaGetLastError();
}

}  // namespace sb
