// sb_implicit.cu -- factor tables of the semi-implicit viscous branch of cross
// and crosst (explicit = 0, cross.f90:797-989, crosst.f90:916-1195).
//
// That branch solves, per substep k and (kx, kz) line,
//   (d2/dy2 - k^2 - dtr1) f_new = rhs,   dtr1 = Re ibeta_k / Delta t,
// and for the mean profiles (d2/dy2 - dtr1) u00 = rhs (lapcdy(., rk2, .),
// cross.f90:898-925,965-967); crosst's scalar the same with dtr1k = ibeta_k /
// (fkappa Delta t).  Delta t follows the CFL rule per step and per box, so the
// Helmholtz factorisations are rebuilt on the device every substep, after
// k_tables, for the lines (kx, kz >= 0) of every box (a line (kx, -kz) has the
// same k^2) and the mean line.  The tables have the layout of the per-line
// Helmholtz tables of the explicit step (Fac with stride = boxes x (lines +
// 1)): the LDL^H base
// with the shear phase factored out of the border rows (the steps of
// base_factor in sb_host.cpp, after modChol7cyclic_cmplx,
// diffy_shear_hepta.f90:578-755), the homogeneous solutions and border sums
// of the segment plan (seg_factor) and the interleaved row records the
// segmented solve reads.
#include <cuda_runtime.h>

#include "sb_common.cuh"
#include "sb_kernels.h"

namespace sb {

__device__ __constant__ static const double kIbeta[3] = {160.0 / 37.0, 24.0 / 5.0, 6.0};

// Lanes: (part, line) = (lane / kHfLines, lane % kHfLines), 10 lines per warp
// and three parts per line (lanes 30, 31 idle).  GB300 issues an FP64 warp
// instruction in the same time however many lanes it carries, so the parts of
// a line repeat the serial banded factorisation (at no extra cost) and then
// take one border row each (e, f, g) and one homogeneous solution index
// t = part + 1 each; a warp's instruction stream is then one line's chain
// with the three-way work in parallel.  The banded recurrence of a
// Toeplitz band reaches an exact fixed point after a few dozen rows for the
// strongly diagonal operators of this branch (dtr1 dominates); from the row
// where the carried state repeats bit for bit, every further row is the
// same, so those rows are copied instead of recomputed.
constexpr int kHfLines = 10;

// which = 0: the flow's operators (dtr1 = Re ibeta_k / Dt, tables bf.hi);
// 1: the scalar's of crosst (dtr1k = ibeta_k / (fkappa Dt), crosst.f90:1976-1977,
// tables bf.hit)
__global__ void __launch_bounds__(128) k_hfac(Grid g, Bufs bf, int rk, int which) {
  // lines (kx, kz >= 0): (kx, -kz) has the same k^2; slot nl is the mean line
  const int n = g.my, nl = g.nkx * (g.nz + 1), per = nl + 1;
  const long nslots = (long)g.B * per;
  const int lane = threadIdx.x & 31, part = lane / kHfLines, l = lane - part * kHfLines;
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  long line = warp * kHfLines + l;
  const bool on = part < 3 && line < nslots;
  if (line >= nslots) line = nslots - 1;
  const int b = (int)(line / per), lc = (int)(line - (long)b * per);
  const Member &M = bf.mem[b];
  const bool wr = on && !M.halted;  // this lane writes
  const long stride = nslots;
  Fac &F = which ? bf.hit : bf.hi;
  double *La = const_cast<double *>(F.La), *Lb = const_cast<double *>(F.Lb),
         *Lc = const_cast<double *>(F.Lc), *Dd = const_cast<double *>(F.Dd),
         *Dm = const_cast<double *>(F.Ddm1), *E = const_cast<double *>(F.e),
         *Fb = const_cast<double *>(F.f), *Gb = const_cast<double *>(F.g),
         *sums = const_cast<double *>(F.sums), *ef = const_cast<double *>(F.ef),
         *rows = const_cast<double *>(F.rows);
  // the operator rh2 - k2 pr2 with k2 = kx^2 + kz^2 + dtr1 (dtr1 alone on the
  // mean line; the (0,0) line is never solved and gets the mean line's k2)
  const double dtr1 = which ? ((1.0 / g.kappa) / M.Deltat) * kIbeta[rk]
                            : (M.Re / M.Deltat) * kIbeta[rk];
  double k2 = dtr1;
  if (lc < nl) {
    const int i = lc % g.nkx, k = lc / g.nkx;
    const double gz = g.gam * k, ax = g.alp * i;
    if (i != 0 || k != 0) k2 = dtr1 + (gz * gz + ax * ax);
  }
  double a[7];
#pragma unroll
  for (int d = 0; d < 7; d++) a[d] = g.rh2[d] - k2 * g.pr2[d];
  const double a0 = a[3], a1 = a[4], a2 = a[5], a3 = a[6];
  auto at = [&](long q) { return q * stride + line; };  // 0-based row q
  // ---- banded rows 1..n-3 (base_factor): carried state La[j], Lb[j], Lb[j+1],
  // Lc[j], Lc[j+1], Lc[j+2], Dd[j-1], Dd[j-2], Dd[j-3] entering row j.  Rows 1-3
  // have their own forms and the last three rows drop the entries beyond row
  // n-3; the loop between them has neither (my >= 16 keeps them apart).
  const bool w0 = wr && part == 0;
  double la0 = 0.0, lb0 = 0.0, lb1 = 0.0, lc0 = 0.0, lc1 = 0.0, lc2 = 0.0;
  double d1 = 0.0, d2 = 0.0, d3 = 0.0, dd = 0.0, dm = 0.0;
  auto put = [&](int j) {
    if (w0) {
      const long o = at(j - 1);
      La[o] = la0; Lb[o] = lb0; Lc[o] = lc0; Dd[o] = dd; Dm[o] = dm;
      double *r = rows + o * 16;
      r[0] = la0; r[1] = lb0; r[2] = lc0; r[6] = dm;
    }
  };
  // one row: s and t are the sums of row j; la1, lb2, lc3 the entries it
  // passes on (zero beyond row n-3)
  auto row = [&](int j, double s, double t, bool k1, bool k2, bool k3, bool first) -> bool {
    dd = first ? a0 : a0 - s;
    dm = __drcp_rn(dd);  // 1/dd, correctly rounded as the division
    const double la1 = k1 ? (first ? dm * a1 : dm * (a1 - t)) : 0.0;
    const double lb2 = k2 ? (first ? dm * a2 : dm * (a2 - lc2 * d1 * la0)) : 0.0;
    const double lc3 = k3 ? dm * a3 : 0.0;
    put(j);
    // a repeat of the state entering row j is a fixed point
    bool fixed = false;
    if (k3 && j >= 4 && dd == d1)
      fixed = la1 == la0 && lb1 == lb0 && lb2 == lb1 && lc1 == lc0 && lc2 == lc1 && lc3 == lc2 &&
              d1 == d2 && d2 == d3;
    d3 = d2; d2 = d1; d1 = dd;
    la0 = la1; lb0 = lb1; lb1 = lb2; lc0 = lc1; lc1 = lc2; lc2 = lc3;
    return fixed;
  };
  row(1, 0.0, 0.0, true, true, true, true);
  row(2, la0 * d1 * la0, lb1 * d1 * la0, true, true, true, false);
  row(3, lb0 * d2 * lb0 + la0 * d1 * la0, lc1 * d2 * lb0 + lb1 * d1 * la0, true, true, true,
      false);
  int j = 4;
  bool fixed = false;
  for (; j <= n - 6 && !fixed; j++)
    fixed = row(j, lc0 * d3 * lc0 + lb0 * d2 * lb0 + la0 * d1 * la0,
                lc1 * d2 * lb0 + lb1 * d1 * la0, true, true, true, false);
  if (fixed) {
    // rows j .. n-3 repeat the last row
    for (; j <= n - 3; j++) put(j);
  } else {
    for (; j <= n - 3; j++)
      row(j, lc0 * d3 * lc0 + lb0 * d2 * lb0 + la0 * d1 * la0, lc1 * d2 * lb0 + lb1 * d1 * la0,
          j + 1 <= n - 3, j + 2 <= n - 3, false, false);
  }
  __syncwarp();
  // ---- border rows with the shear phase factored out: part 0 e (rows
  // 1..n-6), part 1 f (1..n-5), part 2 g (1..n-4), and the six border sums
  {
    const int last = n - 6 + part;
    double l1 = 0.0, l2 = 0.0, l3 = 0.0, dd1 = 0.0, dd2 = 0.0, dd3 = 0.0;
    // the same three products on every part (no divergent branches): part 0
    // keeps See in s0, part 1 Sfe, Sff in s0, s1, part 2 Sge, Sgf, Sgg
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    const int src0 = l, src1 = kHfLines + l;
    // the right-hand sides of rows 1-3: part 0 (a3), part 1 (a2, a3), part 2
    // (a1, a2, a3)
    const double b1 = part == 0 ? a3 : (part == 1 ? a2 : a1);
    const double b2 = part == 0 ? 0.0 : (part == 1 ? a3 : a2);
    const double b3 = part == 2 ? a3 : 0.0;
    auto brow = [&](int i, double t, bool live) {
      const long o = at(i - 1);
      const double dd = Dd[o];
      const double L = live ? Dm[o] * t : 0.0;
      const double ei = __shfl_sync(0xffffffffu, L, src0);
      const double fi = __shfl_sync(0xffffffffu, L, src1);
      s0 += L * ei * dd;
      s1 += L * fi * dd;
      s2 += L * L * dd;
      if (wr && live) {
        (part == 0 ? E : (part == 1 ? Fb : Gb))[o] = L;
        rows[o * 16 + 3 + part] = L;
      }
      l3 = l2; l2 = l1; l1 = L;
      dd3 = dd2; dd2 = dd1; dd1 = dd;
    };
    brow(1, b1, true);
    brow(2, b2 - l1 * dd1 * La[at(1)], true);
    brow(3, b3 - l2 * dd2 * Lb[at(2)] - l1 * dd1 * La[at(2)], true);
    // The border rows decay geometrically along the band (a linear recurrence
    // of the diagonally dominant factors): once the last three entries of
    // every line of the warp are below 2^-64 of their largest (checked every
    // fourth row), all further entries and their share of the sums lie below
    // FP64 rounding and are written as zeros.
    double lmax = fmax(fabs(l1), fmax(fabs(l2), fabs(l3)));
    int i = 4;
    bool cut = false;
    for (; i <= n - 6; i++) {
      const long o = at(i - 1);
      brow(i, -(l3 * dd3 * Lc[o]) - l2 * dd2 * Lb[o] - l1 * dd1 * La[o], true);
      if ((i & 3) == 3) {
        lmax = fmax(lmax, fmax(fabs(l1), fmax(fabs(l2), fabs(l3))));
        const double thr = lmax * 0x1p-64;
        const bool small = !on || (fabs(l1) <= thr && fabs(l2) <= thr && fabs(l3) <= thr);
        if (__all_sync(0xffffffffu, small)) {
          cut = true;
          i++;
          break;
        }
      }
    }
    if (cut) {
      if (wr) {
        double *Lp = part == 0 ? E : (part == 1 ? Fb : Gb);
        for (int r = i; r <= last; r++) {
          Lp[at(r - 1)] = 0.0;
          rows[at(r - 1) * 16 + 3 + part] = 0.0;
        }
      }
    } else {
      for (i = n - 5; i <= n - 4; i++) {
        const long o = at(i - 1);
        brow(i, -(l3 * dd3 * Lc[o]) - l2 * dd2 * Lb[o] - l1 * dd1 * La[o], i <= last);
      }
    }
    if (wr) {
      if (part == 0) {
        sums[at(0)] = s0;
        for (int q = 0; q < 4; q++) sums[at(6 + q)] = a[3 + q];
      } else if (part == 1) {
        sums[at(1)] = s0;
        sums[at(2)] = s1;
      } else if (part == 2) {
        sums[at(3)] = s0;
        sums[at(4)] = s1;
        sums[at(5)] = s2;
      }
    }
  }
  __syncwarp();
  // ---- homogeneous solutions of the segment plan (seg_factor), t = part + 1
  if (part < 3) {
    const int t = part + 1;
    double *hf = const_cast<double *>(F.hf[part]), *hb = const_cast<double *>(F.hb[part]);
    for (int sg = 0; sg < g.nseg; sg++) {
      const int lo = g.slo[sg], hi = g.shi[sg];
      // the homogeneous solutions decay away from their unit start like the
      // border rows: below 2^-64 over three rows, the rest is written as zeros
      double h1 = (t == 1), h2 = (t == 2), h3 = (t == 3), se = 0.0, sf = 0.0, sgs = 0.0;
      int i = lo;
      for (; i <= hi; i++) {
        const long o = at(i - 1);
        const double h = -Lc[o] * h3 - Lb[o] * h2 - La[o] * h1;
        se += E[o] * h;
        sf += Fb[o] * h;
        sgs += Gb[o] * h;
        if (wr) {
          hf[o] = h;
          rows[o * 16 + 8 + part] = h;
        }
        h3 = h2; h2 = h1; h1 = h;
        if (((i - lo) & 3) == 3 && fabs(h1) <= 0x1p-64 && fabs(h2) <= 0x1p-64 &&
            fabs(h3) <= 0x1p-64) {
          i++;
          break;
        }
      }
      if (wr)
        for (; i <= hi; i++) {
          hf[at(i - 1)] = 0.0;
          rows[at(i - 1) * 16 + 8 + part] = 0.0;
        }
      if (wr) {
        ef[at((sg * 3 + 0) * 3 + t - 1)] = se;
        ef[at((sg * 3 + 1) * 3 + t - 1)] = sf;
        ef[at((sg * 3 + 2) * 3 + t - 1)] = sgs;
      }
      if (sg < g.nseg - 1) {
        double g1 = (t == 1), g2 = (t == 2), g3 = (t == 3);
        int ib = hi;
        for (; ib >= lo; ib--) {
          // rows above n-3 hold zeros (at() of seg_factor)
          const double v = -La[at(ib)] * g1 - Lb[at(ib + 1)] * g2 - Lc[at(ib + 2)] * g3;
          if (wr) {
            hb[at(ib - 1)] = v;
            rows[at(ib - 1) * 16 + 12 + part] = v;
          }
          g3 = g2; g2 = g1; g1 = v;
          if (((hi - ib) & 3) == 3 && fabs(g1) <= 0x1p-64 && fabs(g2) <= 0x1p-64 &&
              fabs(g3) <= 0x1p-64) {
            ib--;
            break;
          }
        }
        if (wr)
          for (; ib >= lo; ib--) {
            hb[at(ib - 1)] = 0.0;
            rows[at(ib - 1) * 16 + 12 + part] = 0.0;
          }
      }
    }
  }
}

cudaError_t launch_hfac(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  const long warps = ((long)g.B * (g.nkx * (g.nz + 1) + 1) + kHfLines - 1) / kHfLines;
  const unsigned nb = (unsigned)((warps + 3) / 4);
  k_hfac<<<nb, 128, 0, st>>>(g, bf, rk - 1, 0);
  if (g.temp) k_hfac<<<nb, 128, 0, st>>>(g, bf, rk - 1, 1);
  return cudaGetLastError();
}

}  // namespace sb
