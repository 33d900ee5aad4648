// sb_seg.cuh -- segmented cyclic heptadiagonal y-line solve.
//
// The banded part of the LDL^H substitutions (rows 1..my-3) is split into S
// consecutive segments solved at the same time by S warps of one block; warp
// s owns segment s of 16 lines (lane = 2*line + component).  Each segment
// runs its recurrences from a zero incoming state; the true solution adds a
// combination of three precomputed homogeneous solutions whose weights -- the
// three values entering the segment -- follow from a short prefix over the
// segments, exchanged through shared memory.  The arithmetic otherwise
// follows solve_line (sb_line.cuh): forward substitution with the border-row
// sums, the complex bordered rows N-2..N, back substitution.
#pragma once
#include "sb_line.cuh"

namespace sb {

// exchange slots per (segment, line, component)
#define SB_XS 12

struct SegView {
  const Fac &F;
  long line;
  __device__ SegView(const Fac &f, long l) : F(f), line(l) {}
  __device__ __forceinline__ double at(const double *p, long q) const {
    return __ldg(p + (F.stride ? q * F.stride + line : q));
  }
  // homogeneous solutions, 1-based row i, t = 1..3
  __device__ __forceinline__ double hf(int t, int i) const { return at(F.hf[t - 1], i - 1); }
  __device__ __forceinline__ double hb(int t, int i) const { return at(F.hb[t - 1], i - 1); }
  // border-row sums of segment s, q = 0 (e), 1 (f), 2 (g)
  __device__ __forceinline__ double ef(int s, int q, int t) const { return at(F.ef, (s * 3 + q) * 3 + t - 1); }
};

// Per-row record of the interleaved factor table (Fac::rows), 16 doubles:
// La Lb Lc e f g Dm 0 | hf1 hf2 hf3 0 | hb1 hb2 hb3 0.  The row loops read it
// with 16-byte loads from one pointer per line (a few load instructions per
// row instead of one indexed load per coefficient).
struct RowPtr {
  const double *p;
  long rs;  // doubles per row
  __device__ RowPtr(const Fac &F, long line)
      : p(F.rows + (F.stride ? line * 16 : 0)), rs(F.stride ? 16 * F.stride : 16) {}
  __device__ __forceinline__ const double2 *row(int i) const {
    return reinterpret_cast<const double2 *>(p + (long)(i - 1) * rs);
  }
};

// Solves the line of lane (l, c) in segment s; on return ys[k*ystr] holds the
// solution at row r0+k (1-based) for the rows this segment owns: lo..hi, and
// for the top segment also lo..N.  All threads of the block must call this
// together (it synchronises the block twice).  The shared column holds
// rend - lo + 5 rows (the segment's rows and four rows of the extension).
// Sources of the shear tail (Tail) of the factorisation, evaluated only where
// the bordered rows need it, so that its 21 values are not live through the
// row loops: from the per-kx table of k_tables, or computed for a per-line
// factorisation.
struct TailLoad {
  const double *p;
  __device__ __forceinline__ Tail operator()() const { return load_tail(p); }
};
struct TailMake {
  const FacView &V;
  cd shp;
  int N;
  __device__ __forceinline__ Tail operator()() const { return make_tail(V, shp, N); }
};

template <int S, typename TU, class TF>
__device__ __forceinline__ void solve_seg(const TU *u, long ps, double *ys, int ystr, int N,
                                          const FacView &V, const SegView &W, const TF &tailf, cd shp,
                                          cd shm, int c, int s, int l, const int *slo,
                                          const int *shi, double r0, double r1, double r2,
                                          double r3, bool anti, double *xch) {
  const int lo = slo[s], hi = shi[s];
  const bool top = (s == S - 1);
  double *mine = xch + ((s * 16 + l) * 2 + c) * SB_XS;
  const RowPtr RP(V.F, V.line);
  // wrapped values u(-2..0) = u(N-2..N)*shm, u(N+1..N+3) = u(1..3)*shp (1-based)
  const double uN3 = (double)u[(long)(N - 3) * ps], uN2 = (double)u[(long)(N - 2) * ps],
               uN1 = (double)u[(long)(N - 1) * ps];
  const double u0 = (double)u[0], u1 = (double)u[ps], u2 = (double)u[2 * ps];
  const double lo3 = cmul_c(uN3, __shfl_xor_sync(0xffffffffu, uN3, 1), shm, c),
               lo2 = cmul_c(uN2, __shfl_xor_sync(0xffffffffu, uN2, 1), shm, c),
               lo1 = cmul_c(uN1, __shfl_xor_sync(0xffffffffu, uN1, 1), shm, c);
  const double hi0 = cmul_c(u0, __shfl_xor_sync(0xffffffffu, u0, 1), shp, c),
               hi1 = cmul_c(u1, __shfl_xor_sync(0xffffffffu, u1, 1), shp, c),
               hi2 = cmul_c(u2, __shfl_xor_sync(0xffffffffu, u2, 1), shp, c);
  const int rend = top ? N : hi;
  auto ext = [&](int i) -> double {  // extended line, 1-based row, from the field
    if (i < 1) return i == -2 ? lo3 : (i == -1 ? lo2 : lo1);
    if (i > N) return i == N + 1 ? hi0 : (i == N + 2 ? hi1 : hi2);
    return (double)u[(long)(i - 1) * ps];
  };
  // stage the segment's rows of u and the next four rows of the extended line
  // in the solution column: all loads issued up front, and the forward sweep
  // reads row i+4 from the column (before the row is overwritten)
#pragma unroll 8
  for (int i = lo; i <= rend; i++) ys[(i - lo) * ystr] = (double)u[(long)(i - 1) * ps];
#pragma unroll
  for (int t = 1; t <= 4; t++) ys[(rend - lo + t) * ystr] = ext(rend + t);
  // ---- forward substitution of the segment from a zero incoming state
  double w0 = ext(lo - 3), w1 = ext(lo - 2), w2 = ext(lo - 1), w3 = ys[0], w4 = ys[ystr],
         w5 = ys[2 * ystr], w6 = ys[3 * ystr];
  double y1 = 0.0, y2 = 0.0, y3 = 0.0, Se = 0.0, Sf = 0.0, Sg = 0.0;
  auto stencil = [&]() -> double {
    return anti ? r1 * (w4 - w2) + r2 * (w5 - w1) + r3 * (w6 - w0)
                : r0 * w3 + r1 * (w4 + w2) + r2 * (w5 + w1) + r3 * (w6 + w0);
  };
#pragma unroll 4
  for (int i = lo; i <= hi; i++) {
    const double2 *rw = RP.row(i);
    const double2 ab = __ldg(rw), ce = __ldg(rw + 1), fg = __ldg(rw + 2);
    const double rhs = stencil();
    const double y = rhs - ce.x * y3 - ab.y * y2 - ab.x * y1;
    ys[(i - lo) * ystr] = y;
    Se = fma(ce.y, y, Se);
    Sf = fma(fg.x, y, Sf);
    Sg = fma(fg.y, y, Sg);
    y3 = y2;
    y2 = y1;
    y1 = y;
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6;
    w6 = ys[(i + 4 - lo) * ystr];
  }
  // the right-hand sides of the bordered rows N-2..N (top segment)
  double bN2 = 0.0, bN1 = 0.0, bN0 = 0.0;
  if (top) {
    bN2 = stencil();
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6;
    w6 = ys[(N + 2 - lo) * ystr];
    bN1 = stencil();
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6;
    w6 = ys[(N + 3 - lo) * ystr];
    bN0 = stencil();
  }
  mine[0] = y1;  // rows hi, hi-1, hi-2
  mine[1] = y2;
  mine[2] = y3;
  mine[3] = Se;
  mine[4] = Sf;
  mine[5] = Sg;
  mine[6] = bN2;
  mine[7] = bN1;
  mine[8] = bN0;
  __syncthreads();
  // ---- prefix over the segments: values entering each segment, border sums,
  // and the true last rows N-3..N-5 (both components, to form the complex rows)
  double Yown[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  double tot[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  double ylast[2][3];
  for (int cc = 0; cc < 2; cc++) {
    double Y[3] = {0.0, 0.0, 0.0};
    for (int sp = 0; sp < S; sp++) {
      const double *x = xch + ((sp * 16 + l) * 2 + cc) * SB_XS;
      if (sp == s) {
        Yown[cc][0] = Y[0];
        Yown[cc][1] = Y[1];
        Yown[cc][2] = Y[2];
      }
      for (int q = 0; q < 3; q++)
        tot[cc][q] += x[3 + q] + W.ef(sp, q, 1) * Y[0] + W.ef(sp, q, 2) * Y[1] + W.ef(sp, q, 3) * Y[2];
      // values leaving segment sp: rows hi, hi-1, hi-2
      double Yn[3];
      for (int r = 0; r < 3; r++) {
        const int row = shi[sp] - r;
        Yn[r] = x[r] + W.hf(1, row) * Y[0] + W.hf(2, row) * Y[1] + W.hf(3, row) * Y[2];
      }
      Y[0] = Yn[0];
      Y[1] = Yn[1];
      Y[2] = Yn[2];
    }
    ylast[cc][0] = Y[0];  // y(N-3)
    ylast[cc][1] = Y[1];  // y(N-4)
    ylast[cc][2] = Y[2];  // y(N-5)
  }
  const double *xt0 = xch + (((S - 1) * 16 + l) * 2 + 0) * SB_XS;
  const double *xt1 = xch + (((S - 1) * 16 + l) * 2 + 1) * SB_XS;
  // ---- bordered rows N-2..N and the first back-substitution rows (complex)
  const Tail T = tailf();
  const cd Y3 = mk(ylast[0][0], ylast[1][0]), Y4 = mk(ylast[0][1], ylast[1][1]),
           Y5 = mk(ylast[0][2], ylast[1][2]);
  const cd cSe = mk(tot[0][0], tot[1][0]), cSf = mk(tot[0][1], tot[1][1]),
           cSg = mk(tot[0][2], tot[1][2]);
  const cd b2 = mk(xt0[6], xt1[6]), b1 = mk(xt0[7], xt1[7]), b0 = mk(xt0[8], xt1[8]);
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
  const double pe = comp(Pe, c), pf = comp(Pf, c), pg = comp(Pg, c);
  const double Ya = Yown[c][0], Yb = Yown[c][1], Yc = Yown[c][2];
  // ---- back substitution of the segment (the top one from the true values)
  double xa = 0.0, xb = 0.0, xc = 0.0;
  int ibeg = hi;
  if (top) {
    ys[(N - 1 - (lo - 1)) * ystr] = comp(xN0, c);
    ys[(N - 2 - (lo - 1)) * ystr] = comp(xN1, c);
    ys[(N - 3 - (lo - 1)) * ystr] = comp(xN2, c);
    ys[(N - 4 - (lo - 1)) * ystr] = comp(x3, c);
    ys[(N - 5 - (lo - 1)) * ystr] = comp(x4, c);
    ys[(N - 6 - (lo - 1)) * ystr] = comp(x5, c);
    xa = comp(x5, c);
    xb = comp(x4, c);
    xc = comp(x3, c);
    ibeg = N - 6;
  }
  // La(i+1), Lb(i+1..i+2), Lc(i+1..i+3) of the rows above, carried down
  double La1 = V.La(ibeg + 1), Lb1 = V.Lb(ibeg + 1), Lb2 = V.Lb(ibeg + 2), Lc1 = V.Lc(ibeg + 1),
         Lc2 = V.Lc(ibeg + 2), Lc3 = V.Lc(ibeg + 3);
  // the first segment starts from the true zero state: no homogeneous part
  const bool hom = (s > 0);
#pragma unroll 4
  for (int i = ibeg; i >= lo; i--) {
    const double2 *rw = RP.row(i);
    const double2 ab = __ldg(rw), ce = __ldg(rw + 1), fg = __ldg(rw + 2), dm = __ldg(rw + 3);
    double y = ys[(i - lo) * ystr];
    if (hom) {
      const double2 h12 = __ldg(rw + 4), h3 = __ldg(rw + 5);
      y = y + h12.x * Ya + h12.y * Yb + h3.x * Yc;
    }
    // the previous row enters last: one dependent multiply-add per row on the
    // loop-carried path (the reference's order puts it first)
    const double x = dm.x * y - ce.y * pe - fg.x * pf - fg.y * pg - Lc3 * xc - Lb2 * xb - La1 * xa;
    ys[(i - lo) * ystr] = x;
    xc = xb;
    xb = xa;
    xa = x;
    Lc3 = Lc2; Lc2 = Lc1; Lc1 = ce.x;
    Lb2 = Lb1; Lb1 = ab.y;
    La1 = ab.x;
  }
  mine[9] = ys[0];  // rows lo, lo+1, lo+2
  mine[10] = ys[ystr];
  mine[11] = ys[2 * ystr];
  __syncthreads();
  if (top) return;
  // ---- values entering this segment from above: x(hi+1..hi+3)
  double X[3];
  {
    const double *x = xch + (((S - 1) * 16 + l) * 2 + c) * SB_XS;
    X[0] = x[9];
    X[1] = x[10];
    X[2] = x[11];
  }
  for (int sp = S - 2; sp > s; sp--) {
    const double *x = xch + ((sp * 16 + l) * 2 + c) * SB_XS;
    double Xn[3];
    for (int r = 0; r < 3; r++) {
      const int row = slo[sp] + r;
      Xn[r] = x[9 + r] + W.hb(1, row) * X[0] + W.hb(2, row) * X[1] + W.hb(3, row) * X[2];
    }
    X[0] = Xn[0];
    X[1] = Xn[1];
    X[2] = Xn[2];
  }
#pragma unroll 4
  for (int i = lo; i <= hi; i++) {
    const double2 *rw = RP.row(i);
    const double2 h12 = __ldg(rw + 6), h3 = __ldg(rw + 7);
    ys[(i - lo) * ystr] += h12.x * X[0] + h12.y * X[1] + h3.x * X[2];
  }
}

}  // namespace sb
