// sb_krylov.cu -- device-resident Krylov spaces for the Newton-Krylov and
// Arnoldi searches, and the state <-> unknown-vector maps of a handle.
//
// The reference keeps its Krylov vectors on MPI rank 0 and forms every inner
// product, vector update and norm there (dotp, vecadd, norm, gmres_shear.f90:
// 3680-3919; the MGS loops of gmres_k_shear 1905-2207 and arnoldi_shear.f90:
// 222-330).  Here the vectors live in one device buffer of FP64 columns, the
// products of a block of columns are formed with fixed-order (deterministic)
// reductions, and only the small matrices of coefficients cross to the host,
// where the Hessenberg least-squares problems are solved.  The unknown vector
// is `throwing`'s (gmres_shear.f90:2229-2426, iuse_fou_mode 2): u00, w00 and,
// per y plane, the selected (kz, kx) entries of omega_y and phi; the period
// map reads and writes it on the device (sb_set_state_packed,
// sb_get_state_packed), so no state crosses the host during a search.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/shearbox.h"
#include "sb_common.cuh"
#include "sb_kernels.h"

namespace sb {
void set_error(const std::string &msg);
}

using sb::Grid;

namespace {

int kfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  sb::set_error(buf);
  return code;
}
#define KCK(x)                                                                    \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess)                                                        \
      return kfail(3, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

constexpr int kThreads = 256;
constexpr int kTA = 4;  // columns of the left block per gram tile
constexpr int kTB = 8;  // columns of the right block per gram tile
constexpr int kMaxSrc = 8;

// ---------------------------------------------------------------------------
// C[a][b] = sum_r A[r, a0 + a] B[r, b0 + b] over rows [r0, r1): partial sums
// per row chunk, then a fixed-order sum over the chunks.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_gram(const double *__restrict__ V, long ld, long r0, long r1, long chunk, int a0, int m, int b0,
       int p, double *__restrict__ part) {
  const int ta = blockIdx.y * kTA, tb = blockIdx.z * kTB;
  const long lo = r0 + (long)blockIdx.x * chunk;
  const long hi = min(r1, lo + chunk);
  double acc[kTA][kTB];
#pragma unroll
  for (int a = 0; a < kTA; a++)
#pragma unroll
    for (int b = 0; b < kTB; b++) acc[a][b] = 0.0;
  const double *A[kTA];
  const double *B[kTB];
#pragma unroll
  for (int a = 0; a < kTA; a++) A[a] = V + (long)(a0 + min(ta + a, m - 1)) * ld;
#pragma unroll
  for (int b = 0; b < kTB; b++) B[b] = V + (long)(b0 + min(tb + b, p - 1)) * ld;
  for (long r = lo + threadIdx.x; r < hi; r += kThreads) {
    double va[kTA], vb[kTB];
#pragma unroll
    for (int a = 0; a < kTA; a++) va[a] = A[a][r];
#pragma unroll
    for (int b = 0; b < kTB; b++) vb[b] = B[b][r];
#pragma unroll
    for (int a = 0; a < kTA; a++)
#pragma unroll
      for (int b = 0; b < kTB; b++) acc[a][b] = fma(va[a], vb[b], acc[a][b]);
  }
  // block reduction in a fixed order: warp trees, then the warps in order
  __shared__ double s[kThreads / 32][kTA * kTB];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < kTA; a++)
#pragma unroll
    for (int b = 0; b < kTB; b++) {
      double v = acc[a][b];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) s[w][a * kTB + b] = v;
    }
  __syncthreads();
  if (threadIdx.x < kTA * kTB) {
    const int a = threadIdx.x / kTB, b = threadIdx.x % kTB;
    double v = 0.0;
    for (int q = 0; q < kThreads / 32; q++) v += s[q][threadIdx.x];
    if (ta + a < m && tb + b < p) part[((long)blockIdx.x * m + ta + a) * p + tb + b] = v;
  }
}

__global__ void k_gram_sum(const double *__restrict__ part, int nchunk, int m, int p,
                           double *__restrict__ C) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m * p) return;
  double v = 0.0;
  for (int c = 0; c < nchunk; c++) v += part[(long)c * m * p + q];
  C[q] = v;
}

// W[r, b0 + b] += alpha * sum_a V[r, a0 + a] C[a][b] over rows [r0, r1)
__global__ void __launch_bounds__(kThreads)
k_update(double *__restrict__ V, long ld, long r0, long r1, int a0, int m, int b0, int p,
         const double *__restrict__ C, double alpha) {
  const long r = r0 + (long)blockIdx.x * kThreads + threadIdx.x;
  if (r >= r1) return;
  for (int g = 0; g < p; g += 8) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int nb = min(8, p - g);
    for (int a = 0; a < m; a++) {
      const double v = V[(long)(a0 + a) * ld + r];
      const double *c = C + (long)a * p + g;
#pragma unroll
      for (int b = 0; b < 8; b++)
        if (b < nb) acc[b] = fma(v, c[b], acc[b]);
    }
#pragma unroll
    for (int b = 0; b < 8; b++)
      if (b < nb) {
        double *w = V + (long)(b0 + g + b) * ld + r;
        *w = fma(alpha, acc[b], *w);
      }
  }
}

// W[r, b0 + b] = sum_a W[r, b0 + a] M[a][b] (in place, p <= 64 columns)
__global__ void __launch_bounds__(kThreads)
k_transform(double *__restrict__ V, long ld, long r0, long r1, int b0, int p,
            const double *__restrict__ M) {
  const long r = r0 + (long)blockIdx.x * kThreads + threadIdx.x;
  if (r >= r1) return;
  double x[64];
  for (int a = 0; a < p; a++) x[a] = V[(long)(b0 + a) * ld + r];
  for (int b = 0; b < p; b++) {
    double acc = 0.0;
    for (int a = 0; a < p; a++) acc = fma(x[a], M[(long)a * p + b], acc);
    V[(long)(b0 + b) * ld + r] = acc;
  }
}

struct Srcs {
  int n;
  int col[kMaxSrc];
  double coef[kMaxSrc];
};

// V[r, dst] = sum_k coef_k V[r, src_k]
__global__ void k_combine(double *__restrict__ V, long ld, long r0, long r1, int dst, Srcs s) {
  const long r = r0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= r1) return;
  double v = 0.0;
  for (int k = 0; k < s.n; k++) v = fma(s.coef[k], V[(long)s.col[k] * ld + r], v);
  V[(long)dst * ld + r] = v;
}

// the representable finite-difference step of matvec_dns_disk3d (iuse_hej):
// V[dst] = x0 + ((x0 + e d) - x0), each operation rounded on its own
__global__ void k_perturb(double *__restrict__ V, long ld, long r0, long r1, int dst, int x0c,
                          int dc, double e) {
  const long r = r0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= r1) return;
  const double x0 = V[(long)x0c * ld + r], d = V[(long)dc * ld + r];
  const double h = __dsub_rn(__dadd_rn(x0, __dmul_rn(e, d)), x0);
  V[(long)dst * ld + r] = __dadd_rn(x0, h);
}

// finite-difference products: order 1 (g0 - g1) / eps, order 2
// (g0 - g1) / (2 eps), order 4 (8 (g0 - g1) - (g2 - g3)) / (12 eps)
__global__ void k_fd(double *__restrict__ V, long ld, long r0, long r1, int dst, int order,
                     Srcs s, double eps) {
  const long r = r0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= r1) return;
  const double a = V[(long)s.col[0] * ld + r], b = V[(long)s.col[1] * ld + r];
  double v;
  if (order == 1) {
    v = __ddiv_rn(__dsub_rn(a, b), eps);
  } else if (order == 2) {
    v = __ddiv_rn(__dsub_rn(a, b), __dmul_rn(2.0, eps));
  } else {
    const double c = V[(long)s.col[2] * ld + r], d = V[(long)s.col[3] * ld + r];
    v = __ddiv_rn(__dsub_rn(__dmul_rn(8.0, __dsub_rn(a, b)), __dsub_rn(c, d)),
                  __dmul_rn(12.0, eps));
  }
  V[(long)dst * ld + r] = v;
}

// ---------------------------------------------------------------------------
// state <-> unknown vector.  Complex entry sc of a y plane <-> (kz index k,
// kx index i): row k = 0 without i = 0, rows 1..nz all i, rows nz+1..mz-1
// without i = 0 (the conjugates of rows mz-k); x = [u00/su | w00/su | per
// plane j and entry sc: vor.re/sg, phi.re/sp, vor.im/sg, phi.im/sp].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void entry_of(const Grid &g, int sc, int *k, int *i) {
  const int n0 = g.nkx - 1, n1 = g.nz * g.nkx;
  if (sc < n0) {
    *k = 0;
    *i = sc + 1;
  } else if (sc < n0 + n1) {
    const int s = sc - n0;
    *k = 1 + s / g.nkx;
    *i = s % g.nkx;
  } else {
    const int s = sc - n0 - n1;
    *k = g.nz + 1 + s / (g.nkx - 1);
    *i = 1 + s % (g.nkx - 1);
  }
}
__device__ __forceinline__ int index_of(const Grid &g, int k, int i) {
  if (k == 0) return i - 1;
  if (k <= g.nz) return (g.nkx - 1) + (k - 1) * g.nkx + i;
  return (g.nkx - 1) + g.nz * g.nkx + (k - g.nz - 1) * (g.nkx - 1) + (i - 1);
}

template <typename R>
__global__ void k_pack(Grid g, const R *__restrict__ vor, const R *__restrict__ phi,
                       const R *__restrict__ mu, double *__restrict__ x, double su, double sg,
                       double sp, double sx, double sz) {
  const int nselc = g.mz * g.nkx - 1 - g.nz;  // complex entries per plane
  const long nb = (long)g.my * nselc;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.my) {
    x[t] = (double)mu[2 * t] / su;
    x[g.my + t] = (double)mu[2 * t + 1] / su;
  }
  if (t >= nb) return;
  const int j = (int)(t / nselc), sc = (int)(t - (long)j * nselc);
  int k, i;
  entry_of(g, sc, &k, &i);
  const long o = 2 * (((long)j * g.mz + k) * g.nkx + i);
  double vr = (double)vor[o], vi = (double)vor[o + 1];
  double pr = (double)phi[o], pi = (double)phi[o + 1];
  if (sx != 0.0 || sz != 0.0) {
    // phase_shift_fou: the mode times exp(-i kx sx) exp(-i kz sz)
    const double kz = g.gam * (double)(k <= g.nz ? k : k - g.mz);
    double s1, c1, s2, c2;
    sincos(g.alp * (double)i * sx, &s1, &c1);
    sincos(kz * sz, &s2, &c2);
    const double fr = c1 * c2 - s1 * s2, fi = -(s1 * c2 + c1 * s2);
    const double a = vr * fr - vi * fi, b = vr * fi + vi * fr;
    const double c = pr * fr - pi * fi, d = pr * fi + pi * fr;
    vr = a;
    vi = b;
    pr = c;
    pi = d;
  }
  double *o4 = x + 2 * (long)g.my + 4 * t;
  o4[0] = vr / sg;
  o4[1] = pr / sp;
  o4[2] = vi / sg;
  o4[3] = pi / sp;
}

template <typename R>
__global__ void k_unpack(Grid g, const double *__restrict__ x, R *__restrict__ vor,
                         R *__restrict__ phi, R *__restrict__ mu, double su, double sg,
                         double sp) {
  const int nselc = g.mz * g.nkx - 1 - g.nz;
  const long n = (long)g.my * g.mz * g.nkx;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.my) {
    mu[2 * t] = (R)(x[t] * su);
    mu[2 * t + 1] = (R)(x[g.my + t] * su);
  }
  if (t >= n) return;
  const int i = (int)(t % g.nkx);
  const int k = (int)((t / g.nkx) % g.mz);
  const int j = (int)(t / ((long)g.nkx * g.mz));
  double vr = 0.0, vi = 0.0, pr = 0.0, pi = 0.0;
  if (i != 0 || k != 0) {
    const bool cj = (i == 0 && k > g.nz);  // set_conj: the conjugate of row mz-k
    const int sc = index_of(g, cj ? g.mz - k : k, i);
    const double *s4 = x + 2 * (long)g.my + 4 * ((long)j * nselc + sc);
    vr = s4[0] * sg;
    pr = s4[1] * sp;
    vi = s4[2] * sg;
    pi = s4[3] * sp;
    if (cj) {
      vi = -vi;
      pi = -pi;
    }
  }
  vor[2 * t] = (R)vr;
  vor[2 * t + 1] = (R)vi;
  phi[2 * t] = (R)pr;
  phi[2 * t + 1] = (R)pi;
}

// d/ds of the phase shift at s = 0 on a packed vector: every mode times
// -i kx (dir 0) or -i kz (dir 1); the mean profiles have no derivative
__global__ void k_tangent(Grid g, const double *__restrict__ x, double *__restrict__ out,
                          int dir) {
  const int nselc = g.mz * g.nkx - 1 - g.nz;
  const long nb = (long)g.my * nselc;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 2L * g.my) out[t] = 0.0;
  if (t >= nb) return;
  const int sc = (int)(t % nselc);
  int k, i;
  entry_of(g, sc, &k, &i);
  const double kk = dir == 0 ? g.alp * (double)i : g.gam * (double)(k <= g.nz ? k : k - g.mz);
  const double *s4 = x + 2 * (long)g.my + 4 * t;
  double *o4 = out + 2 * (long)g.my + 4 * t;
  const double vr = s4[0], pr = s4[1], vi = s4[2], pi = s4[3];
  o4[0] = kk * vi;
  o4[1] = kk * pi;
  o4[2] = -kk * vr;
  o4[3] = -kk * pr;
}

long chunk_rows(long rows, long *nchunk) {
  long nc = (rows + 2047) / 2048;
  if (nc > 608) nc = 608;
  if (nc < 1) nc = 1;
  const long ch = (rows + nc - 1) / nc;
  *nchunk = (rows + ch - 1) / ch;
  return ch;
}

}  // namespace

namespace sb {

long packed_length(const Grid &g) {
  const long nselc = (long)g.mz * g.nkx - 1 - g.nz;
  return 2L * g.my + 4L * g.my * nselc;
}

cudaError_t launch_pack(const Grid &g, const double *vor, const double *phi, const double *mu,
                        double *x, const double sca[3], double sx, double sz, cudaStream_t st) {
  const long nselc = (long)g.mz * g.nkx - 1 - g.nz;
  const long n = std::max((long)g.my * nselc, (long)g.my);
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (g.prec)
    k_pack<float><<<nb, 256, 0, st>>>(g, (const float *)vor, (const float *)phi,
                                      (const float *)mu, x, sca[0], sca[1], sca[2], sx, sz);
  else
    k_pack<double><<<nb, 256, 0, st>>>(g, vor, phi, mu, x, sca[0], sca[1], sca[2], sx, sz);
  return cudaGetLastError();
}

cudaError_t launch_tangent(const Grid &g, const double *x, double *out, int dir,
                           cudaStream_t st) {
  const long nselc = (long)g.mz * g.nkx - 1 - g.nz;
  const long n = std::max((long)g.my * nselc, 2L * g.my);
  k_tangent<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, x, out, dir);
  return cudaGetLastError();
}

cudaError_t launch_unpack(const Grid &g, const double *x, double *vor, double *phi, double *mu,
                          const double sca[3], cudaStream_t st) {
  const long n = std::max((long)g.my * g.mz * g.nkx, (long)g.my);
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (g.prec)
    k_unpack<float><<<nb, 256, 0, st>>>(g, x, (float *)vor, (float *)phi, (float *)mu, sca[0],
                                        sca[1], sca[2]);
  else
    k_unpack<double><<<nb, 256, 0, st>>>(g, x, vor, phi, mu, sca[0], sca[1], sca[2]);
  return cudaGetLastError();
}

}  // namespace sb

// ---------------------------------------------------------------------------
// the Krylov space object of the C-ABI
// ---------------------------------------------------------------------------
struct sb_kspace {
  long n = 0, ld = 0;
  int cols = 0;
  double *V = nullptr;     // cols columns of ld doubles (n used)
  double *part = nullptr;  // gram partial sums
  long part_cap = 0;
  double *small = nullptr;  // device copy of a coefficient matrix
  long small_cap = 0;
  double *hsmall = nullptr;  // pinned host staging of the same
  cudaStream_t st = nullptr;
  bool own_stream = false;
  int dev = 0;
};

namespace {

int check_rows(const sb_kspace *ks, long r0, long r1) {
  if (r0 < 0 || r1 > ks->n || r0 > r1) return kfail(1, "row range [%ld, %ld) outside [0, %ld)", r0, r1, ks->n);
  return 0;
}
int check_cols(const sb_kspace *ks, int c0, int m) {
  if (c0 < 0 || m < 0 || c0 + m > ks->cols)
    return kfail(1, "columns [%d, %d) outside [0, %d)", c0, c0 + m, ks->cols);
  return 0;
}
int ensure_small(sb_kspace *ks, long count) {
  if (count <= ks->small_cap) return 0;
  if (ks->small) cudaFree(ks->small);
  if (ks->hsmall) cudaFreeHost(ks->hsmall);
  ks->small = nullptr;
  ks->hsmall = nullptr;
  ks->small_cap = 0;
  KCK(cudaMalloc((void **)&ks->small, sizeof(double) * count));
  KCK(cudaMallocHost((void **)&ks->hsmall, sizeof(double) * count));
  ks->small_cap = count;
  return 0;
}

}  // namespace

extern "C" {

int sb_kspace_create(long n, int cols, void *stream, sb_kspace **out) {
  if (!out || n < 1 || cols < 1) return kfail(1, "sb_kspace_create: bad argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return kfail(2, "no CUDA device");
  sb_kspace *ks = new sb_kspace;
  ks->n = n;
  ks->ld = (n + 31) / 32 * 32;  // 256-byte aligned columns
  ks->cols = cols;
  cudaGetDevice(&ks->dev);
  cudaError_t e = cudaMalloc((void **)&ks->V, sizeof(double) * (size_t)ks->ld * cols);
  if (e == cudaSuccess) e = cudaMemset(ks->V, 0, sizeof(double) * (size_t)ks->ld * cols);
  if (e == cudaSuccess && !stream) {
    e = cudaStreamCreateWithFlags(&ks->st, cudaStreamNonBlocking);
    ks->own_stream = true;
  } else {
    ks->st = (cudaStream_t)stream;
  }
  if (e != cudaSuccess) {
    sb_kspace_destroy(ks);
    return kfail(3, "sb_kspace_create: %s", cudaGetErrorString(e));
  }
  *out = ks;
  return 0;
}

int sb_kspace_destroy(sb_kspace *ks) {
  if (!ks) return 0;
  if (ks->st) cudaStreamSynchronize(ks->st);
  if (ks->V) cudaFree(ks->V);
  if (ks->part) cudaFree(ks->part);
  if (ks->small) cudaFree(ks->small);
  if (ks->hsmall) cudaFreeHost(ks->hsmall);
  if (ks->own_stream && ks->st) cudaStreamDestroy(ks->st);
  delete ks;
  return 0;
}

double *sb_kspace_col(sb_kspace *ks, int col) {
  if (!ks || col < 0 || col >= ks->cols) return nullptr;
  return ks->V + (size_t)col * ks->ld;
}

void *sb_kspace_stream(sb_kspace *ks) { return ks ? (void *)ks->st : nullptr; }

int sb_kspace_gram(sb_kspace *ks, long r0, long r1, int a0, int m, int b0, int p, double *C) {
  if (!ks || !C) return kfail(1, "null argument");
  int rc;
  if ((rc = check_rows(ks, r0, r1)) || (rc = check_cols(ks, a0, m)) || (rc = check_cols(ks, b0, p)))
    return rc;
  if (m == 0 || p == 0) return 0;
  long nchunk;
  const long rows = r1 - r0;
  const long ch = chunk_rows(rows > 0 ? rows : 1, &nchunk);
  const long need = nchunk * (long)m * p;
  if (need > ks->part_cap) {
    if (ks->part) cudaFree(ks->part);
    ks->part = nullptr;
    ks->part_cap = 0;
    KCK(cudaMalloc((void **)&ks->part, sizeof(double) * need));
    ks->part_cap = need;
  }
  if ((rc = ensure_small(ks, (long)m * p))) return rc;
  const dim3 grid((unsigned)nchunk, (unsigned)((m + kTA - 1) / kTA), (unsigned)((p + kTB - 1) / kTB));
  if (grid.y > 65535 || grid.z > 65535) return kfail(1, "sb_kspace_gram: block too large");
  k_gram<<<grid, kThreads, 0, ks->st>>>(ks->V, ks->ld, r0, r1, ch, a0, m, b0, p, ks->part);
  KCK(cudaGetLastError());
  k_gram_sum<<<(unsigned)((m * p + 255) / 256), 256, 0, ks->st>>>(ks->part, (int)nchunk, m, p,
                                                                   ks->small);
  KCK(cudaGetLastError());
  KCK(cudaMemcpyAsync(ks->hsmall, ks->small, sizeof(double) * m * p, cudaMemcpyDeviceToHost,
                      ks->st));
  KCK(cudaStreamSynchronize(ks->st));
  for (long q = 0; q < (long)m * p; q++) C[q] = ks->hsmall[q];
  return 0;
}

int sb_kspace_update(sb_kspace *ks, long r0, long r1, int a0, int m, int b0, int p,
                     const double *C, double alpha) {
  if (!ks || !C) return kfail(1, "null argument");
  int rc;
  if ((rc = check_rows(ks, r0, r1)) || (rc = check_cols(ks, a0, m)) || (rc = check_cols(ks, b0, p)))
    return rc;
  if (a0 < b0 + p && b0 < a0 + m) return kfail(1, "sb_kspace_update: overlapping column ranges");
  if (m == 0 || p == 0 || r1 == r0) return 0;
  if ((rc = ensure_small(ks, (long)m * p))) return rc;
  // the staging buffer may still feed an earlier update: wait for the stream
  KCK(cudaStreamSynchronize(ks->st));
  for (long q = 0; q < (long)m * p; q++) ks->hsmall[q] = C[q];
  KCK(cudaMemcpyAsync(ks->small, ks->hsmall, sizeof(double) * m * p, cudaMemcpyHostToDevice,
                      ks->st));
  k_update<<<(unsigned)((r1 - r0 + kThreads - 1) / kThreads), kThreads, 0, ks->st>>>(
      ks->V, ks->ld, r0, r1, a0, m, b0, p, ks->small, alpha);
  KCK(cudaGetLastError());
  return 0;
}

int sb_kspace_transform(sb_kspace *ks, long r0, long r1, int b0, int p, const double *M) {
  if (!ks || !M) return kfail(1, "null argument");
  int rc;
  if ((rc = check_rows(ks, r0, r1)) || (rc = check_cols(ks, b0, p))) return rc;
  if (p > 64) return kfail(1, "sb_kspace_transform: at most 64 columns");
  if (p == 0 || r1 == r0) return 0;
  if ((rc = ensure_small(ks, (long)p * p))) return rc;
  KCK(cudaStreamSynchronize(ks->st));
  for (long q = 0; q < (long)p * p; q++) ks->hsmall[q] = M[q];
  KCK(cudaMemcpyAsync(ks->small, ks->hsmall, sizeof(double) * p * p, cudaMemcpyHostToDevice,
                      ks->st));
  k_transform<<<(unsigned)((r1 - r0 + kThreads - 1) / kThreads), kThreads, 0, ks->st>>>(
      ks->V, ks->ld, r0, r1, b0, p, ks->small);
  KCK(cudaGetLastError());
  return 0;
}

int sb_kspace_combine(sb_kspace *ks, long r0, long r1, int dst, int nsrc, const int *src,
                      const double *coef) {
  if (!ks || (nsrc > 0 && (!src || !coef))) return kfail(1, "null argument");
  if (nsrc < 0 || nsrc > kMaxSrc) return kfail(1, "sb_kspace_combine: 0..%d sources", kMaxSrc);
  int rc;
  if ((rc = check_rows(ks, r0, r1)) || (rc = check_cols(ks, dst, 1))) return rc;
  Srcs s{};
  s.n = nsrc;
  for (int k = 0; k < nsrc; k++) {
    if ((rc = check_cols(ks, src[k], 1))) return rc;
    s.col[k] = src[k];
    s.coef[k] = coef[k];
  }
  if (r1 == r0) return 0;
  k_combine<<<(unsigned)((r1 - r0 + 255) / 256), 256, 0, ks->st>>>(ks->V, ks->ld, r0, r1, dst, s);
  KCK(cudaGetLastError());
  return 0;
}

int sb_kspace_perturb(sb_kspace *ks, long r0, long r1, int dst, int x0, int d, double e) {
  if (!ks) return kfail(1, "null argument");
  int rc;
  if ((rc = check_rows(ks, r0, r1)) || (rc = check_cols(ks, dst, 1)) || (rc = check_cols(ks, x0, 1)) ||
      (rc = check_cols(ks, d, 1)))
    return rc;
  if (r1 == r0) return 0;
  k_perturb<<<(unsigned)((r1 - r0 + 255) / 256), 256, 0, ks->st>>>(ks->V, ks->ld, r0, r1, dst, x0,
                                                                    d, e);
  KCK(cudaGetLastError());
  return 0;
}

int sb_kspace_fd(sb_kspace *ks, long r0, long r1, int dst, int order, const int *g, double eps) {
  if (!ks || !g) return kfail(1, "null argument");
  if (order != 1 && order != 2 && order != 4) return kfail(1, "order must be 1, 2 or 4");
  int rc;
  if ((rc = check_rows(ks, r0, r1)) || (rc = check_cols(ks, dst, 1))) return rc;
  Srcs s{};
  s.n = order == 4 ? 4 : 2;
  for (int k = 0; k < s.n; k++) {
    if ((rc = check_cols(ks, g[k], 1))) return rc;
    s.col[k] = g[k];
  }
  if (r1 == r0) return 0;
  k_fd<<<(unsigned)((r1 - r0 + 255) / 256), 256, 0, ks->st>>>(ks->V, ks->ld, r0, r1, dst, order,
                                                               s, eps);
  KCK(cudaGetLastError());
  return 0;
}

int sb_kspace_set(sb_kspace *ks, int col, long off, long len, const double *host) {
  if (!ks || (!host && len > 0)) return kfail(1, "null argument");
  int rc;
  if ((rc = check_cols(ks, col, 1)) || (rc = check_rows(ks, off, off + len))) return rc;
  if (len == 0) return 0;
  KCK(cudaMemcpyAsync(ks->V + (size_t)col * ks->ld + off, host, sizeof(double) * len,
                      cudaMemcpyHostToDevice, ks->st));
  KCK(cudaStreamSynchronize(ks->st));
  return 0;
}

int sb_kspace_get(sb_kspace *ks, int col, long off, long len, double *host) {
  if (!ks || (!host && len > 0)) return kfail(1, "null argument");
  int rc;
  if ((rc = check_cols(ks, col, 1)) || (rc = check_rows(ks, off, off + len))) return rc;
  if (len == 0) return 0;
  KCK(cudaMemcpyAsync(host, ks->V + (size_t)col * ks->ld + off, sizeof(double) * len,
                      cudaMemcpyDeviceToHost, ks->st));
  KCK(cudaStreamSynchronize(ks->st));
  return 0;
}

int sb_kspace_sync(sb_kspace *ks) {
  if (!ks) return kfail(1, "null argument");
  KCK(cudaStreamSynchronize(ks->st));
  return 0;
}

}  // extern "C"
