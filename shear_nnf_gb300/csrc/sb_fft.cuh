// sb_fft.cuh -- batched shared-memory Stockham FFTs for the x/z transforms.
//
// Replaces FFTW's 2-D r2c/c2r plans of fou3D_thread.f:1-20.  A thread block
// transforms M sequences of length N held contiguously in shared memory
// (sequence m at [m*N]); the result lands in one of the two ping-pong buffers.
// Conventions match FFTW: SIGN=-1 is the forward e^{-i} transform, SIGN=+1 the
// backward e^{+i} transform, both unnormalised.  Autosort stages (no bit
// reversal).
//
// Two forms share the stage layout:
//  * fft_batch_std: radix 4/2/3/5 stages, twiddles from a per-length table of
//    e^{-2 pi i t/N} (FP32 storage and the standalone y operators);
//  * the FP64 form (fft_batch on double2): GB300 issues one FP64 instruction per
//    two lanes and cycle on each SM sub-partition, so FP64 instruction count is
//    the cost of a transform.  A twiddle w = e^{-2 pi i t/N} is stored as
//    w = (-i)^q c (1 + i tau), with q the nearest quarter turn, so c >= cos(pi/4)
//    and |tau| <= 1; then a +- w b is two FMAs for z = b (1 + i tau) and two per
//    output (a + c z, a - c z) with the quarter turn a swap of the components of
//    z (6 FP64 instructions instead of 8 for the complex product and the two
//    sums).  The radix-4 butterfly uses w3 = w1 w2 to apply only w2 and w1 in
//    this form (24 instead of 28 per four points), and the radix-3 stage comes
//    first, where it has no twiddles.  Instructions per point at N = 192:
//    22 instead of 25.3.  Table entry t: {(mx, my), (tau, swap)} with
//    (mx, my) = the signed c of the real and imaginary output components and
//    swap (integer bits) set for odd q.
#pragma once
#include <type_traits>

// Build-time choice of the FP64 stage order where a length has a radix-2
// factor: 0 (default) radix 3, 4, ..., 2 last; 1 the radix-2 stage second
// (for 192 = 3*4*4*4 plan 1 splits one radix-4 stage into two radix-2
// stages).  The FP64 instruction count per point is the same for both (a
// radix-2 layer costs 3 per point in the factored form, a radix-4 stage 6);
// the stages differ in shared-memory strides and barrier count.
#ifndef SB_FFT_PLAN
#define SB_FFT_PLAN 0
#endif

#include "sb_common.cuh"

namespace sb {

template <typename R2>
__device__ __forceinline__ R2 c2mul(R2 a, R2 b) {
  R2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

template <int R, int SIGN, typename R2>
__device__ __forceinline__ void butterfly(R2 *v) {
  if constexpr (R == 2) {
    R2 a = v[0], b = v[1];
    v[0].x = a.x + b.x; v[0].y = a.y + b.y;
    v[1].x = a.x - b.x; v[1].y = a.y - b.y;
  } else if constexpr (R == 4) {
    R2 a0, a1, b0, b1, jb;
    a0.x = v[0].x + v[2].x; a0.y = v[0].y + v[2].y;
    a1.x = v[0].x - v[2].x; a1.y = v[0].y - v[2].y;
    b0.x = v[1].x + v[3].x; b0.y = v[1].y + v[3].y;
    b1.x = v[1].x - v[3].x; b1.y = v[1].y - v[3].y;
    if (SIGN < 0) { jb.x = b1.y; jb.y = -b1.x; }   // -i * b1
    else          { jb.x = -b1.y; jb.y = b1.x; }   // +i * b1
    v[0].x = a0.x + b0.x; v[0].y = a0.y + b0.y;
    v[2].x = a0.x - b0.x; v[2].y = a0.y - b0.y;
    v[1].x = a1.x + jb.x; v[1].y = a1.y + jb.y;
    v[3].x = a1.x - jb.x; v[3].y = a1.y - jb.y;
  } else if constexpr (R == 5) {
    // X_k = sum_n v_n w^(nk), w = exp(SIGN 2 pi i/5), from the sums and
    // differences of the symmetric pairs (v1, v4), (v2, v3)
    typedef decltype(v[0].x) T;
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;  // cos(2pi/5), cos(4pi/5)
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;   // sin(2pi/5), sin(4pi/5)
    R2 t1, t2, t3, t4, a1, a2, b1, b2;
    t1.x = v[1].x + v[4].x; t1.y = v[1].y + v[4].y;
    t2.x = v[2].x + v[3].x; t2.y = v[2].y + v[3].y;
    t3.x = v[1].x - v[4].x; t3.y = v[1].y - v[4].y;
    t4.x = v[2].x - v[3].x; t4.y = v[2].y - v[3].y;
    a1.x = v[0].x + c1 * t1.x + c2 * t2.x; a1.y = v[0].y + c1 * t1.y + c2 * t2.y;
    a2.x = v[0].x + c2 * t1.x + c1 * t2.x; a2.y = v[0].y + c2 * t1.y + c1 * t2.y;
    b1.x = s1 * t3.x + s2 * t4.x; b1.y = s1 * t3.y + s2 * t4.y;
    b2.x = s2 * t3.x - s1 * t4.x; b2.y = s2 * t3.y - s1 * t4.y;
    // i SIGN b = SIGN (-b.y, b.x)
    const T sg = (SIGN < 0) ? (T)-1 : (T)1;
    v[0].x = v[0].x + t1.x + t2.x; v[0].y = v[0].y + t1.y + t2.y;
    v[1].x = a1.x - sg * b1.y; v[1].y = a1.y + sg * b1.x;
    v[4].x = a1.x + sg * b1.y; v[4].y = a1.y - sg * b1.x;
    v[2].x = a2.x - sg * b2.y; v[2].y = a2.y + sg * b2.x;
    v[3].x = a2.x + sg * b2.y; v[3].y = a2.y - sg * b2.x;
  } else if constexpr (R == 3) {
    typedef decltype(v[0].x) T;
    const T s3 = (T)0.86602540378443864676;  // sin(pi/3)
    R2 t1, t2, t3, jt;
    t1.x = v[1].x + v[2].x; t1.y = v[1].y + v[2].y;
    t2.x = v[0].x - (T)0.5 * t1.x; t2.y = v[0].y - (T)0.5 * t1.y;
    t3.x = s3 * (v[1].x - v[2].x); t3.y = s3 * (v[1].y - v[2].y);
    if (SIGN < 0) { jt.x = t3.y; jt.y = -t3.x; }
    else          { jt.x = -t3.y; jt.y = t3.x; }
    v[0].x = v[0].x + t1.x; v[0].y = v[0].y + t1.y;
    v[1].x = t2.x + jt.x; v[1].y = t2.y + jt.y;
    v[2].x = t2.x - jt.x; v[2].y = t2.y - jt.y;
  }
}

// one Stockham stage: radix R, sub-transform size Ns before the stage
template <int N, int Ns, int R, int SIGN, int M, int T, typename R2>
__device__ __forceinline__ void fft_stage(const R2 *__restrict__ in, R2 *__restrict__ out,
                                          const R2 *__restrict__ tw) {
  constexpr int NR = N / R;
  constexpr int STEP = N / (Ns * R);
  for (int bt = threadIdx.x; bt < M * NR; bt += T) {
    const int m = bt / NR;
    const int j = bt - m * NR;
    const R2 *src = in + m * N;
    R2 *dst = out + m * N;
    R2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * NR];
    const int jm = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        R2 w = tw[r * jm * STEP];
        if (SIGN > 0) w.y = -w.y;
        v[r] = c2mul(v[r], w);
      }
    }
    butterfly<R, SIGN>(v);
    const int idxD = (j / Ns) * Ns * R + jm;
#pragma unroll
    for (int r = 0; r < R; r++) dst[idxD + r * Ns] = v[r];
  }
}

// Full transform of M length-N sequences in A (scratch B), standard twiddle
// table; returns the buffer that holds the result.  Ends with a __syncthreads().
template <int N, int SIGN, int M, int T, typename R2>
__device__ __forceinline__ R2 *fft_batch_std(R2 *A, R2 *B, const R2 *__restrict__ tw) {
  __syncthreads();
  if constexpr (N == 32) {
    fft_stage<32, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<32, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<32, 16, 2, SIGN, M, T>(A, B, tw); __syncthreads();
    return B;
  } else if constexpr (N == 48) {
    fft_stage<48, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<48, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<48, 16, 3, SIGN, M, T>(A, B, tw); __syncthreads();
    return B;
  } else if constexpr (N == 64) {
    fft_stage<64, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<64, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<64, 16, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    return B;
  } else if constexpr (N == 80) {
    fft_stage<80, 1, 5, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<80, 5, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<80, 20, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    return B;
  } else if constexpr (N == 128) {
    fft_stage<128, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<128, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<128, 16, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<128, 64, 2, SIGN, M, T>(B, A, tw); __syncthreads();
    return A;
  } else if constexpr (N == 160) {
    fft_stage<160, 1, 5, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<160, 5, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<160, 20, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<160, 80, 2, SIGN, M, T>(B, A, tw); __syncthreads();
    return A;
  } else if constexpr (N == 256) {
    fft_stage<256, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<256, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<256, 16, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<256, 64, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    return A;
  } else if constexpr (N == 320) {
    fft_stage<320, 1, 5, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<320, 5, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<320, 20, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<320, 80, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    return A;
  } else if constexpr (N == 96) {
    fft_stage<96, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<96, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<96, 16, 2, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<96, 32, 3, SIGN, M, T>(B, A, tw); __syncthreads();
    return A;
  } else if constexpr (N == 192) {
    fft_stage<192, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<192, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<192, 16, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<192, 64, 3, SIGN, M, T>(B, A, tw); __syncthreads();
    return A;
  } else if constexpr (N == 384) {
    fft_stage<384, 1, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<384, 4, 4, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<384, 16, 4, SIGN, M, T>(A, B, tw); __syncthreads();
    fft_stage<384, 64, 2, SIGN, M, T>(B, A, tw); __syncthreads();
    fft_stage<384, 128, 3, SIGN, M, T>(A, B, tw); __syncthreads();
    return B;
  } else {
    static_assert(N == 32, "unsupported transform length");
    return A;
  }
}

// ---------------------------------------------------------------------------
// FP64 form with factored twiddles
// ---------------------------------------------------------------------------

// Twiddle t of the factored table, for the direction SIGN (the backward
// transform takes the conjugate: tau -> -tau, (mx, my) -> (my, mx)).
struct GTw {
  double mx, my, tau;
  bool sw;
};
template <int SIGN>
__device__ __forceinline__ GTw gtw_load(const double2 *__restrict__ G, int t) {
  const double2 a = G[2 * t], b = G[2 * t + 1];
  GTw w;
  w.mx = (SIGN < 0) ? a.x : a.y;
  w.my = (SIGN < 0) ? a.y : a.x;
  w.tau = b.x;
  w.sw = __double_as_longlong(b.y) != 0;
  return w;
}
// z = v (1 + i tau) (forward) or v (1 - i tau) (backward), components swapped
// for odd quarter turns: w v = (mx s.x, my s.y)
template <int SIGN>
__device__ __forceinline__ double2 gtw_apply(const GTw &w, double2 v) {
  double za, zb;
  if (SIGN < 0) {
    za = fma(-w.tau, v.y, v.x);
    zb = fma(w.tau, v.x, v.y);
  } else {
    za = fma(w.tau, v.y, v.x);
    zb = fma(-w.tau, v.x, v.y);
  }
  double2 s;
  s.x = w.sw ? zb : za;
  s.y = w.sw ? za : zb;
  return s;
}

// radix-3 stage without twiddles (first stage, Ns = 1): 12 FP64 instructions.
// GAP: the middle third of every input sequence is zero (a spectrum under the
// 2/3 rule with N = 3 * (modes kept per sign)), v1 = 0: 8 instructions.
template <int N, int SIGN, int M, int T, bool GAP>
__device__ __forceinline__ void gstage3(const double2 *__restrict__ in, double2 *__restrict__ out) {
  constexpr int NR = N / 3;
  const double s3 = (SIGN < 0) ? 0.86602540378443864676 : -0.86602540378443864676;
  for (int bt = threadIdx.x; bt < M * NR; bt += T) {
    const int m = bt / NR;
    const int j = bt - m * NR;
    const double2 *src = in + m * N;
    double2 *dst = out + m * N + 3 * j;
    const double2 v0 = src[j], v2 = src[j + 2 * NR];
    if constexpr (GAP) {
      // X0 = v0 + v2, X1,2 = v0 - v2/2 -+ J s3 v2
      const double hx = fma(-0.5, v2.x, v0.x), hy = fma(-0.5, v2.y, v0.y);
      dst[0] = make_double2(v0.x + v2.x, v0.y + v2.y);
      dst[1] = make_double2(fma(-s3, v2.y, hx), fma(s3, v2.x, hy));
      dst[2] = make_double2(fma(s3, v2.y, hx), fma(-s3, v2.x, hy));
    } else {
      const double2 v1 = src[j + NR];
      const double tx = v1.x + v2.x, ty = v1.y + v2.y;
      const double dx = v1.x - v2.x, dy = v1.y - v2.y;
      const double hx = fma(-0.5, tx, v0.x), hy = fma(-0.5, ty, v0.y);
      dst[0] = make_double2(v0.x + tx, v0.y + ty);
      dst[1] = make_double2(fma(s3, dy, hx), fma(-s3, dx, hy));
      dst[2] = make_double2(fma(-s3, dy, hx), fma(s3, dx, hy));
    }
  }
}

// radix-5 stage without twiddles (first stage, Ns = 1): the 5-point DFT of
// butterfly<5>, 36 FP64 instructions
template <int N, int SIGN, int M, int T>
__device__ __forceinline__ void gstage5_first(const double2 *__restrict__ in,
                                              double2 *__restrict__ out) {
  constexpr int NR = N / 5;
  for (int bt = threadIdx.x; bt < M * NR; bt += T) {
    const int m = bt / NR;
    const int j = bt - m * NR;
    const double2 *src = in + m * N;
    double2 *dst = out + m * N + 5 * j;
    double2 v[5];
#pragma unroll
    for (int r = 0; r < 5; r++) v[r] = src[j + r * NR];
    butterfly<5, SIGN>(v);
#pragma unroll
    for (int r = 0; r < 5; r++) dst[r] = v[r];
  }
}

// radix-4 stage without twiddles (first stage, Ns = 1): 16 FP64 instructions
template <int N, int SIGN, int M, int T>
__device__ __forceinline__ void gstage4_first(const double2 *__restrict__ in,
                                              double2 *__restrict__ out) {
  constexpr int NR = N / 4;
  for (int bt = threadIdx.x; bt < M * NR; bt += T) {
    const int m = bt / NR;
    const int j = bt - m * NR;
    const double2 *src = in + m * N;
    double2 *dst = out + m * N + 4 * j;
    double2 v[4];
#pragma unroll
    for (int r = 0; r < 4; r++) v[r] = src[j + r * NR];
    butterfly<4, SIGN>(v);
#pragma unroll
    for (int r = 0; r < 4; r++) dst[r] = v[r];
  }
}

// twiddled radix-4 stage, sub-transform size Ns: with w1 = w(jm STEP) and
// w2 = w1^2, a = v0 +- w2 v2, e = v1 +- w2 v3, X0,2 = a0 +- w1 e0,
// X1,3 = a1 +- J w1 e1 (J = -i forward, +i backward): 24 FP64 instructions
template <int N, int Ns, int SIGN, int M, int T>
__device__ __forceinline__ void gstage4(const double2 *__restrict__ in, double2 *__restrict__ out,
                                        const double2 *__restrict__ G) {
  constexpr int NR = N / 4;
  constexpr int STEP = N / (Ns * 4);
  for (int bt = threadIdx.x; bt < M * NR; bt += T) {
    const int m = bt / NR;
    const int j = bt - m * NR;
    const double2 *src = in + m * N;
    const int jm = j % Ns;
    double2 *dst = out + m * N + (j / Ns) * Ns * 4 + jm;
    const double2 v0 = src[j], v1 = src[j + NR], v2 = src[j + 2 * NR], v3 = src[j + 3 * NR];
    const GTw w2 = gtw_load<SIGN>(G, 2 * jm * STEP);
    const GTw w1 = gtw_load<SIGN>(G, jm * STEP);
    const double2 s2 = gtw_apply<SIGN>(w2, v2);
    const double a0x = fma(w2.mx, s2.x, v0.x), a0y = fma(w2.my, s2.y, v0.y);
    const double a1x = fma(-w2.mx, s2.x, v0.x), a1y = fma(-w2.my, s2.y, v0.y);
    const double2 s3 = gtw_apply<SIGN>(w2, v3);
    const double2 e0 = make_double2(fma(w2.mx, s3.x, v1.x), fma(w2.my, s3.y, v1.y));
    const double2 e1 = make_double2(fma(-w2.mx, s3.x, v1.x), fma(-w2.my, s3.y, v1.y));
    const double2 p = gtw_apply<SIGN>(w1, e0);
    dst[0] = make_double2(fma(w1.mx, p.x, a0x), fma(w1.my, p.y, a0y));
    dst[2 * Ns] = make_double2(fma(-w1.mx, p.x, a0x), fma(-w1.my, p.y, a0y));
    const double2 q = gtw_apply<SIGN>(w1, e1);
    // J (w1 e1) = (my q.y, -mx q.x) forward, (-my q.y, mx q.x) backward
    if (SIGN < 0) {
      dst[Ns] = make_double2(fma(w1.my, q.y, a1x), fma(-w1.mx, q.x, a1y));
      dst[3 * Ns] = make_double2(fma(-w1.my, q.y, a1x), fma(w1.mx, q.x, a1y));
    } else {
      dst[Ns] = make_double2(fma(-w1.my, q.y, a1x), fma(w1.mx, q.x, a1y));
      dst[3 * Ns] = make_double2(fma(w1.my, q.y, a1x), fma(-w1.mx, q.x, a1y));
    }
  }
}

// twiddled radix-2 stage: X0,1 = v0 +- w1 v1, 6 FP64 instructions
template <int N, int Ns, int SIGN, int M, int T>
__device__ __forceinline__ void gstage2(const double2 *__restrict__ in, double2 *__restrict__ out,
                                        const double2 *__restrict__ G) {
  constexpr int NR = N / 2;
  constexpr int STEP = N / (Ns * 2);
  for (int bt = threadIdx.x; bt < M * NR; bt += T) {
    const int m = bt / NR;
    const int j = bt - m * NR;
    const double2 *src = in + m * N;
    const int jm = j % Ns;
    double2 *dst = out + m * N + (j / Ns) * Ns * 2 + jm;
    const double2 v0 = src[j], v1 = src[j + NR];
    const GTw w = gtw_load<SIGN>(G, jm * STEP);
    const double2 s = gtw_apply<SIGN>(w, v1);
    dst[0] = make_double2(fma(w.mx, s.x, v0.x), fma(w.my, s.y, v0.y));
    dst[Ns] = make_double2(fma(-w.mx, s.x, v0.x), fma(-w.my, s.y, v0.y));
  }
}

// Full FP64 transform with the factored table G (2 N double2 entries); GAP as
// for gstage3 (used where N is a multiple of 3).
template <int N, int SIGN, int M, int T, bool GAP = false>
__device__ __forceinline__ double2 *fft_batch_g(double2 *A, double2 *B,
                                                const double2 *__restrict__ G) {
  __syncthreads();
  if constexpr (N == 32) {
    gstage4_first<32, SIGN, M, T>(A, B); __syncthreads();
    gstage4<32, 4, SIGN, M, T>(B, A, G); __syncthreads();
    gstage2<32, 16, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else if constexpr (N == 48) {
    gstage3<48, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage4<48, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<48, 12, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else if constexpr (N == 64) {
    gstage4_first<64, SIGN, M, T>(A, B); __syncthreads();
    gstage4<64, 4, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<64, 16, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else if constexpr (N == 80) {
    gstage5_first<80, SIGN, M, T>(A, B); __syncthreads();
    gstage4<80, 5, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<80, 20, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else if constexpr (N == 128) {
    gstage4_first<128, SIGN, M, T>(A, B); __syncthreads();
    gstage4<128, 4, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<128, 16, SIGN, M, T>(A, B, G); __syncthreads();
    gstage2<128, 64, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 160) {
    gstage5_first<160, SIGN, M, T>(A, B); __syncthreads();
    gstage4<160, 5, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<160, 20, SIGN, M, T>(A, B, G); __syncthreads();
    gstage2<160, 80, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 256) {
    gstage4_first<256, SIGN, M, T>(A, B); __syncthreads();
    gstage4<256, 4, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<256, 16, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<256, 64, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 320) {
    gstage5_first<320, SIGN, M, T>(A, B); __syncthreads();
    gstage4<320, 5, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<320, 20, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<320, 80, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 96 && SB_FFT_PLAN == 1) {
    gstage3<96, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage2<96, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<96, 6, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<96, 24, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 96) {
    gstage3<96, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage4<96, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<96, 12, SIGN, M, T>(A, B, G); __syncthreads();
    gstage2<96, 48, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 192 && SB_FFT_PLAN == 1) {
    gstage3<192, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage2<192, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<192, 6, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<192, 24, SIGN, M, T>(B, A, G); __syncthreads();
    gstage2<192, 96, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else if constexpr (N == 192) {
    gstage3<192, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage4<192, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<192, 12, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<192, 48, SIGN, M, T>(B, A, G); __syncthreads();
    return A;
  } else if constexpr (N == 384 && SB_FFT_PLAN == 1) {
    gstage3<384, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage2<384, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<384, 6, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<384, 24, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<384, 96, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else if constexpr (N == 384) {
    gstage3<384, SIGN, M, T, GAP>(A, B); __syncthreads();
    gstage4<384, 3, SIGN, M, T>(B, A, G); __syncthreads();
    gstage4<384, 12, SIGN, M, T>(A, B, G); __syncthreads();
    gstage4<384, 48, SIGN, M, T>(B, A, G); __syncthreads();
    gstage2<384, 192, SIGN, M, T>(A, B, G); __syncthreads();
    return B;
  } else {
    static_assert(N == 32, "unsupported transform length");
    return A;
  }
}

// Transform with the device table of the storage type: the factored FP64
// table for double2, the standard table for float2.  GAP: the caller's input
// has the zero middle third of the 2/3 rule (backward transforms of a
// truncated spectrum); only the FP64 form uses it.
template <int N, int SIGN, int M, int T, bool GAP = false, typename R2>
__device__ __forceinline__ R2 *fft_batch(R2 *A, R2 *B, const R2 *__restrict__ tw) {
  if constexpr (std::is_same<R2, double2>::value)
    return fft_batch_g<N, SIGN, M, T, GAP>(A, B, tw);
  else
    return fft_batch_std<N, SIGN, M, T>(A, B, tw);
}

}  // namespace sb
