// sb_fft.cuh -- batched shared-memory Stockham FFTs for the x/z transforms.
//
// Replaces FFTW's 2-D r2c/c2r plans of fou3D_thread.f:1-20.  A thread block
// transforms M sequences of length N held contiguously in shared memory
// (sequence m at [m*N]); the result lands in one of the two ping-pong buffers.
// Conventions match FFTW: SIGN=-1 is the forward e^{-i} transform, SIGN=+1 the
// backward e^{+i} transform, both unnormalised.  Radix 4/2/3 stages, autosort
// (no bit reversal), twiddles from a per-length global table e^{-2 pi i t/N}.
#pragma once
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

// Full transform of M length-N sequences in A (scratch B); returns the buffer
// that holds the result.  Ends with a __syncthreads().
template <int N, int SIGN, int M, int T, typename R2>
__device__ __forceinline__ R2 *fft_batch(R2 *A, R2 *B, const R2 *__restrict__ tw) {
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

}  // namespace sb
