// sb_line.cuh -- cyclic heptadiagonal y-line solver shared by the step kernels
// and the standalone operators.  One lane per (line, component); lane pairs
// (2l, 2l+1) hold the real and imaginary parts of one complex line.
#pragma once
#include "sb_common.cuh"

namespace sb {

// ---------------------------------------------------------------------------
// y-line solver
// ---------------------------------------------------------------------------
struct Tail {
  cd Le5, Le4, Le3, Lf4, Lf3, Lf2, Lg3, Lg2, Lg1;
  double Dm2, Dm1, Dm0;  // 1/D at rows N-2, N-1, N
};

struct FacView {
  const Fac &F;
  long line;
  __device__ FacView(const Fac &f, long l) : F(f), line(l) {}
  // 1-based row accessors
  __device__ __forceinline__ double ld(const double *p, int i) const {
    return __ldg(p + (F.stride ? (long)(i - 1) * F.stride + line : (long)(i - 1)));
  }
  __device__ __forceinline__ double La(int i) const { return ld(F.La, i); }
  __device__ __forceinline__ double Lb(int i) const { return ld(F.Lb, i); }
  __device__ __forceinline__ double Lc(int i) const { return ld(F.Lc, i); }
  __device__ __forceinline__ double Dm(int i) const { return ld(F.Ddm1, i); }
  __device__ __forceinline__ double Dd(int i) const { return ld(F.Dd, i); }
  __device__ __forceinline__ double e(int i) const { return ld(F.e, i); }
  __device__ __forceinline__ double f(int i) const { return ld(F.f, i); }
  __device__ __forceinline__ double g(int i) const { return ld(F.g, i); }
  __device__ __forceinline__ double sum(int q) const {
    return __ldg(F.sums + (F.stride ? (long)q * F.stride + line : (long)q));
  }
};

// Shear-dependent tail of the cyclic LDL^H factorisation: the entries that
// modChol_addshear (diffy_shear_hepta.f90:760-870) recomputes, evaluated from
// the shear-free base with the phase factored out of the border rows.
__device__ __forceinline__ Tail make_tail(const FacView &V, cd shp, int N) {
  Tail T;
  const double a0 = V.sum(6), a1 = V.sum(7), a2 = V.sum(8), a3 = V.sum(9);
  const double shp2 = abs2(shp);
  cd E8 = V.e(N - 8) * shp, E7 = V.e(N - 7) * shp, E6 = V.e(N - 6) * shp;
  T.Le5 = V.Dm(N - 5) * (mk(a3, 0.0) - (V.Dd(N - 8) * V.Lc(N - 5)) * E8 -
                         (V.Dd(N - 7) * V.Lb(N - 5)) * E7 - (V.Dd(N - 6) * V.La(N - 5)) * E6);
  T.Le4 = V.Dm(N - 4) * (mk(a2, 0.0) - (V.Dd(N - 7) * V.Lc(N - 4)) * E7 -
                         (V.Dd(N - 6) * V.Lb(N - 4)) * E6 - (V.Dd(N - 5) * V.La(N - 4)) * T.Le5);
  T.Le3 = V.Dm(N - 3) * (mk(a1, 0.0) - (V.Dd(N - 6) * V.Lc(N - 3)) * E6 -
                         (V.Dd(N - 5) * V.Lb(N - 3)) * T.Le5 - (V.Dd(N - 4) * V.La(N - 3)) * T.Le4);
  const double DdN2 = a0 - (shp2 * V.sum(0) + abs2(T.Le5) * V.Dd(N - 5) +
                            abs2(T.Le4) * V.Dd(N - 4) + abs2(T.Le3) * V.Dd(N - 3));
  T.Dm2 = 1.0 / DdN2;
  cd F7 = V.f(N - 7) * shp, F6 = V.f(N - 6) * shp, F5 = V.f(N - 5) * shp;
  T.Lf4 = V.Dm(N - 4) * (mk(a3, 0.0) - (V.Dd(N - 7) * V.Lc(N - 4)) * F7 -
                         (V.Dd(N - 6) * V.Lb(N - 4)) * F6 - (V.Dd(N - 5) * V.La(N - 4)) * F5);
  T.Lf3 = V.Dm(N - 3) * (mk(a2, 0.0) - (V.Dd(N - 6) * V.Lc(N - 3)) * F6 -
                         (V.Dd(N - 5) * V.Lb(N - 3)) * F5 - (V.Dd(N - 4) * V.La(N - 3)) * T.Lf4);
  cd tmp = mk(shp2 * V.sum(1), 0.0) + V.Dd(N - 5) * (F5 * cj(T.Le5)) +
           V.Dd(N - 4) * (T.Lf4 * cj(T.Le4)) + V.Dd(N - 3) * (T.Lf3 * cj(T.Le3));
  T.Lf2 = T.Dm2 * (mk(a1, 0.0) - tmp);
  const double DdN1 = a0 - (shp2 * V.sum(2) + abs2(T.Lf4) * V.Dd(N - 4) +
                            abs2(T.Lf3) * V.Dd(N - 3) + abs2(T.Lf2) * DdN2);
  T.Dm1 = 1.0 / DdN1;
  cd G6 = V.g(N - 6) * shp, G5 = V.g(N - 5) * shp, G4 = V.g(N - 4) * shp;
  T.Lg3 = V.Dm(N - 3) * (mk(a3, 0.0) - (V.Dd(N - 6) * V.Lc(N - 3)) * G6 -
                         (V.Dd(N - 5) * V.Lb(N - 3)) * G5 - (V.Dd(N - 4) * V.La(N - 3)) * G4);
  tmp = mk(shp2 * V.sum(3), 0.0) + V.Dd(N - 5) * (G5 * cj(T.Le5)) +
        V.Dd(N - 4) * (G4 * cj(T.Le4)) + V.Dd(N - 3) * (T.Lg3 * cj(T.Le3));
  T.Lg2 = T.Dm2 * (mk(a2, 0.0) - tmp);
  tmp = mk(shp2 * V.sum(4), 0.0) + V.Dd(N - 4) * (G4 * cj(T.Lf4)) +
        V.Dd(N - 3) * (T.Lg3 * cj(T.Lf3)) + DdN2 * (T.Lg2 * cj(T.Lf2));
  T.Lg1 = T.Dm1 * (mk(a1, 0.0) - tmp);
  const double DdN0 = a0 - (shp2 * V.sum(5) + abs2(T.Lg3) * V.Dd(N - 3) +
                            abs2(T.Lg2) * DdN2 + abs2(T.Lg1) * DdN1);
  T.Dm0 = 1.0 / DdN0;
  return T;
}

// shear tails kept in tables (SB_TAIL doubles each)
__device__ __forceinline__ void store_tail(double *p, const Tail &T) {
  const cd v[9] = {T.Le5, T.Le4, T.Le3, T.Lf4, T.Lf3, T.Lf2, T.Lg3, T.Lg2, T.Lg1};
#pragma unroll
  for (int q = 0; q < 9; q++) {
    p[2 * q] = v[q].x;
    p[2 * q + 1] = v[q].y;
  }
  p[18] = T.Dm2;
  p[19] = T.Dm1;
  p[20] = T.Dm0;
}
__device__ __forceinline__ Tail load_tail(const double *p) {
  Tail T;
  cd *v[9] = {&T.Le5, &T.Le4, &T.Le3, &T.Lf4, &T.Lf3, &T.Lf2, &T.Lg3, &T.Lg2, &T.Lg1};
#pragma unroll
  for (int q = 0; q < 9; q++) *v[q] = mk(__ldg(p + 2 * q), __ldg(p + 2 * q + 1));
  T.Dm2 = __ldg(p + 18);
  T.Dm1 = __ldg(p + 19);
  T.Dm0 = __ldg(p + 20);
  return T;
}

// component c of a complex value held by the lane pair (c=0: re, c=1: im)
__device__ __forceinline__ cd pair_full(double own, int c) {
  double oth = __shfl_xor_sync(0xffffffffu, own, 1);
  return c ? mk(oth, own) : mk(own, oth);
}
__device__ __forceinline__ double comp(cd z, int c) { return c ? z.y : z.x; }
// component c of (own, other) * s
__device__ __forceinline__ double cmul_c(double own, double oth, cd s, int c) {
  return c ? fma(own, s.x, oth * s.y) : fma(own, s.x, -(oth * s.y));
}

// Solves B x = A u_ext on one complex y-line (this lane: component c) with the
// shear-periodic extension u(j+my) = u(j)*shp, u(j-my) = u(j)*shm
// (derivyc / lapcdy, diffy_shear_hepta.f90:333-525; solve7cyclic 900-954).
// A is the 7-point stencil (r0; r1..r3) -- antisymmetric if anti -- and B the
// factorised heptadiagonal.  u is read with stride ps; y (the forward
// substitution) is kept in ybuf (stride ys).  epi(j, x_j) receives the
// solution in descending j.  All 32 lanes of the warp must call this together.
template <typename TU, class EPI>
__device__ __forceinline__ void solve_line(const TU *u, long ps, double *ybuf, long ys, int N,
                                           const FacView &V, const Tail &T, cd shp, cd shm, int c,
                                           double r0, double r1, double r2, double r3, bool anti,
                                           EPI epi) {
  // wrapped values u(-3..-1) = u(N-3..N-1)*shm and u(N..N+2) = u(0..2)*shp
  double uN3 = (double)u[(long)(N - 3) * ps], uN2 = (double)u[(long)(N - 2) * ps],
         uN1 = (double)u[(long)(N - 1) * ps];
  double u0 = (double)u[0], u1 = (double)u[ps], u2 = (double)u[2 * ps];
  double pN3 = __shfl_xor_sync(0xffffffffu, uN3, 1), pN2 = __shfl_xor_sync(0xffffffffu, uN2, 1),
         pN1 = __shfl_xor_sync(0xffffffffu, uN1, 1);
  double p0 = __shfl_xor_sync(0xffffffffu, u0, 1), p1 = __shfl_xor_sync(0xffffffffu, u1, 1),
         p2 = __shfl_xor_sync(0xffffffffu, u2, 1);
  const double lo3 = cmul_c(uN3, pN3, shm, c), lo2 = cmul_c(uN2, pN2, shm, c),
               lo1 = cmul_c(uN1, pN1, shm, c);
  const double hi0 = cmul_c(u0, p0, shp, c), hi1 = cmul_c(u1, p1, shp, c),
               hi2 = cmul_c(u2, p2, shp, c);
  double w0 = lo3, w1 = lo2, w2 = lo1, w3 = u0, w4 = u1, w5 = u2, w6 = (double)u[3 * ps];
  double y1 = 0.0, y2 = 0.0, y3 = 0.0;
  double Se = 0.0, Sf = 0.0, Sg = 0.0;
  double bN2 = 0.0, bN1 = 0.0, bN0 = 0.0;
#pragma unroll 4
  for (int j = 0; j < N; j++) {
    double rhs;
    if (anti)
      rhs = r1 * (w4 - w2) + r2 * (w5 - w1) + r3 * (w6 - w0);
    else
      rhs = r0 * w3 + r1 * (w4 + w2) + r2 * (w5 + w1) + r3 * (w6 + w0);
    if (j < N - 3) {
      const int i = j + 1;  // 1-based row
      double y = rhs - V.Lc(i) * y3 - V.Lb(i) * y2 - V.La(i) * y1;
      ybuf[(long)j * ys] = y;
      Se = fma(V.e(i), y, Se);
      Sf = fma(V.f(i), y, Sf);
      Sg = fma(V.g(i), y, Sg);
      y3 = y2;
      y2 = y1;
      y1 = y;
    } else if (j == N - 3) {
      bN2 = rhs;
    } else if (j == N - 2) {
      bN1 = rhs;
    } else {
      bN0 = rhs;
    }
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6;
    const int jn = j + 4;
    w6 = (jn < N) ? (double)u[(long)jn * ps] : (jn == N ? hi0 : (jn == N + 1 ? hi1 : hi2));
  }
  // bordered rows N-2..N and the first rows of the back substitution (complex)
  const cd Y3 = pair_full(y1, c), Y4 = pair_full(y2, c), Y5 = pair_full(y3, c);
  const cd cSe = pair_full(Se, c), cSf = pair_full(Sf, c), cSg = pair_full(Sg, c);
  const cd b2 = pair_full(bN2, c), b1 = pair_full(bN1, c), b0 = pair_full(bN0, c);
  const cd yN2 = b2 - (shp * cSe + T.Le5 * Y5 + T.Le4 * Y4 + T.Le3 * Y3);
  const cd yN1 = b1 - (shp * cSf + T.Lf4 * Y4 + T.Lf3 * Y3 + T.Lf2 * yN2);
  const cd yN0 = b0 - (shp * cSg + T.Lg3 * Y3 + T.Lg2 * yN2 + T.Lg1 * yN1);
  const cd xN0 = T.Dm0 * yN0;
  const cd xN1 = T.Dm1 * yN1 - cj(T.Lg1) * xN0;
  const cd xN2 = T.Dm2 * yN2 - cj(T.Lf2) * xN1 - cj(T.Lg2) * xN0;
  const cd csh = cj(shp);
  const cd Pe = csh * xN2, Pf = csh * xN1, Pg = csh * xN0;
  const cd x3 = V.Dm(N - 3) * Y3 - cj(T.Le3) * xN2 - cj(T.Lf3) * xN1 - cj(T.Lg3) * xN0;
  const cd x4 = V.Dm(N - 4) * Y4 - V.La(N - 3) * x3 - cj(T.Le4) * xN2 - cj(T.Lf4) * xN1 -
                V.g(N - 4) * Pg;
  const cd x5 = V.Dm(N - 5) * Y5 - V.La(N - 4) * x4 - V.Lb(N - 3) * x3 - cj(T.Le5) * xN2 -
                V.f(N - 5) * Pf - V.g(N - 5) * Pg;
  epi(N - 1, comp(xN0, c));
  epi(N - 2, comp(xN1, c));
  epi(N - 3, comp(xN2, c));
  epi(N - 4, comp(x3, c));
  epi(N - 5, comp(x4, c));
  epi(N - 6, comp(x5, c));
  const double pe = comp(Pe, c), pf = comp(Pf, c), pg = comp(Pg, c);
  double xa = comp(x5, c), xb = comp(x4, c), xc = comp(x3, c);
#pragma unroll 4
  for (int j = N - 7; j >= 0; j--) {
    const int i = j + 1;
    double x = V.Dm(i) * ybuf[(long)j * ys] - V.e(i) * pe - V.f(i) * pf - V.g(i) * pg -
               V.Lc(i + 3) * xc - V.Lb(i + 2) * xb - V.La(i + 1) * xa;
    epi(j, x);
    xc = xb;
    xb = xa;
    xa = x;
  }
}

}  // namespace sb
