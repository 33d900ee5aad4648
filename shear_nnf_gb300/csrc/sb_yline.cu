// sb_yline.cu -- y-line stage, per-box scalars and phase tables of the RK3 step.
//
// The y-operators of one substep (cross.f90:565-795 and the first derivatives of
// the next substep, cross.f90:434-445) run as two kernels so that independent
// solves occupy separate warps (GB300's FP64 pipe needs about one busy warp per
// SM sub-partition, and one warp per line component is too few):
//   k_lineA  role 0: d/dy of dH1/dx + dH3/dz                 (derivyc, -> T)
//            role 1: nu*lap(omega_y) (d2/dy2 from Lv, taken by k_lineB of the
//                    previous substep), RK3 update of omega_y, zeta store and
//                    moving_frame remaps                       (visc3d + update)
//            role 2: d2(phi)/dy2                               (derivyc, -> S)
//            mean warp: nu*u00'', RK3 update of u00, w00
//   k_lineB  role 0: d(omega_y)/dy and d2(omega_y)/dy2 for the next
//                    substep                                   (-> D, Lv)
//            role 1: RK3 update of phi, v = lapcdy(phi), dv/dy  (-> phi, G, V)
//            mean warp: du00/dy, dw00/dy for the next substep
// With the temperature (crosst) the same kernels carry the scalar: k_lineA
// role 0 also adds d(-vT)/dy to ht, role 1 also takes lap(tb), the mean block
// updates tb00; k_lineB role 1 adds the buoyancy gbeta lap(tb) to the phi
// right-hand side and a third role updates tb.
// The same k_lineB (mode 0) is the prologue of a cross call: v from phi on the
// first step (cross.f90:408-426) and the first derivatives.  For the plain
// step (no temperature, no y filter or y dealiasing) k_lineF does both
// kernels' work in one launch, each block taking its 16 lines through all
// the solves with two pipelines of warps; the handle chooses the form.  Forward
// substitutions are kept in shared memory, one column per thread.  The
// per-box kernels of the step (k_scalar, k_tables, k_finish) are in
// sb_box.cu.
#include <cuda_runtime.h>

#include "sb_common.cuh"
#include "sb_kernels.h"
#include "sb_line.cuh"
#include "sb_seg.cuh"

// This file is compiled once per (segment count, storage precision):
// SB_KSEG = 1, 2 or 3 warps per line solve, SB_FLOAT_TU = 0 (FP64) or 1
// (FP32-mixed).  Each compilation puts its kernels and launchers in the
// namespace sb::seg<SB_KSEG> and exports them with a _f64 or _f32 suffix; the
// handle picks a segment count at run time (sb_box.cu dispatches on
// Grid::nseg), so the autotuner can choose the line tile per grid.
#ifndef SB_FLOAT_TU
#define SB_FLOAT_TU 0
#endif
#ifndef SB_KSEG
#define SB_KSEG 2
#endif
#define SB_CAT2(a, b) a##b
#define SB_CAT(a, b) SB_CAT2(a, b)
#define SB_SEGNS SB_CAT(seg, SB_KSEG)
#if SB_FLOAT_TU
#define SB_PSUF(name) SB_CAT(name, _f32)
typedef float SbR;
#else
#define SB_PSUF(name) SB_CAT(name, _f64)
typedef double SbR;
#endif

namespace sb {
namespace SB_SEGNS {

__device__ __forceinline__ cd ldc2(const double *p) { return mk(p[0], p[1]); }

// Block -> (member, role, group of 16 lines); warp -> segment of the banded
// rows; lane -> (line of the group, component).  The last block of every
// member is the mean line u00 + i w00 (line slot 0).
// the blocks per SM the line kernels are register-budgeted for (build-time
// tuning knobs)
#ifndef SB_LINE_MINB
#define SB_LINE_MINB 1
#endif
// k_lineA: six blocks per SM (170 registers) keep its three roles resident
#ifndef SB_LINEA_MINB
#define SB_LINEA_MINB 6
#endif
constexpr int kSeg = SB_KSEG;
struct LineThread {
  int b, role, c, s, l, i, k, r0, r1;
  long lc;
  bool active, mean;
};
__device__ __forceinline__ bool line_thread(const Grid &g, int roles, LineThread *L) {
  const int per = roles * g.ngrp + 1;
  L->b = blockIdx.x / per;
  if (L->b >= g.B) return false;
  const int r = blockIdx.x - L->b * per;
  L->role = r / g.ngrp;
  L->mean = L->role >= roles;
  const int lane = threadIdx.x & 31;
  L->s = threadIdx.x >> 5;
  L->l = lane >> 1;
  L->c = lane & 1;
  const int nl = g.nkx * g.mz;
  if (L->mean) {
    L->lc = 0;
    L->active = (L->l == 0);
  } else {
    L->lc = (long)(r - L->role * g.ngrp) * 16 + L->l;
    L->active = L->lc < nl;
    if (!L->active) L->lc = nl - 1;
  }
  L->i = (int)(L->lc % g.nkx);
  L->k = (int)(L->lc / g.nkx);
  L->r0 = g.slo[L->s];
  L->r1 = (L->s == kSeg - 1) ? g.my : g.shi[L->s];
  return true;
}

// the entry of line lc in the per-line Helmholtz table: the table holds the
// kz >= 0 lines, (kx, -kz) has the k^2 of (kx, kz)
__device__ __forceinline__ long hz_line(const Grid &g, long lc) {
  const int i = (int)(lc % g.nkx), k = (int)(lc / g.nkx);
  return (long)((k <= g.nz) ? k : g.mz - k) * g.nkx + i;
}

// one thread's column of the shared-memory buffer (its segment's rows)
__device__ __forceinline__ double *ycol() {
  extern __shared__ double sm_y[];
  return sm_y + threadIdx.x;
}

// copy this segment's rows of a solution kept in shared memory to a field line
template <typename R>
__device__ __forceinline__ void store_col(const double *ys, int ystr, R *__restrict__ dst, long ps,
                                          const LineThread &L) {
  if (!L.active) return;
#pragma unroll 4
  for (int i = L.r0; i <= L.r1; i++) dst[(long)(i - 1) * ps] = (R)ys[(i - L.r0) * ystr];
}

// RK3 accumulate/update of this segment's rows of one field line with the
// zeta store and both moving_frame remaps (cross.f90:694-781), fused per
// point.  x = d2f/dy2 in the shared buffer (FP64); rhs = the nonlinear
// right-hand side (minus `sub` if given); f, fwk the field and its RK work
// array.  The RK arithmetic runs in the storage precision R; the viscous term
// and the remaps (phase factors) in FP64.  With `lap` the viscous term is
// nuv * lap (a Laplacian computed before) instead of nuv (x - k2 f); `buo`
// adds gb * buo (the buoyancy of the phi equation, crosst.f90:737).
template <typename R>
__device__ __forceinline__ void rk_update(const double *ys, int ystr, const R *__restrict__ rhs,
                                          const R *__restrict__ sub, R *__restrict__ f,
                                          R *__restrict__ fwk, long ps, const LineThread &L,
                                          int rk, double nuv, double k2, double Dt,
                                          const double *__restrict__ mf1,
                                          const double *__restrict__ mf2, long mfs,
                                          const R *__restrict__ lap = nullptr,
                                          const R *__restrict__ buo = nullptr, double gb = 0.0) {
  const R gk = (R)kGama[rk], zk = (R)kZeta[rk], dtr = (R)Dt;
  const int c = L.c;
#pragma unroll 2
  for (int i = L.r0; i <= L.r1; i++) {
    const int j = i - 1;
    const long q = (long)j * ps;
    const R fo = f[q];
    R h = rhs[q];
    if (sub) h = h - sub[q];
    const double vis = lap ? (double)lap[q] : (-(k2 * (double)fo) + ys[(i - L.r0) * ystr]);
    h = h + (R)(nuv * vis);
    if (buo) h = h + (R)(gb * (double)buo[q]);
    R wk = (rk == 0) ? gk * h : fwk[q] + gk * h;
    const double fn = (double)(fo + dtr * wk);
    const cd m2 = ldc2(mf2 + (long)j * mfs);
    const double fnm = cmul_c(fn, __shfl_xor_sync(0xffffffffu, fn, 1), m2, c);
    if (rk < 2) {
      const cd m1 = ldc2(mf1 + (long)j * mfs);
      const double wz = (double)(h * zk);
      wk = (R)cmul_c(wz, __shfl_xor_sync(0xffffffffu, wz, 1), m1, c);
    }
    if (L.active) {
      f[q] = (R)fnm;
      fwk[q] = wk;
    }
  }
}

#define SEG_SOLVE(U, PS, VIEW, SVIEW, TAIL, SHP, SHM, R0, R1, R2, R3, ANTI)                     \
  solve_seg<kSeg>(U, PS, ys, ystr, N, VIEW, SVIEW, TAIL, SHP, SHM, L.c, L.s, L.l, g.slo, g.shi, \
                  R0, R1, R2, R3, ANTI, &xch[0][0][0][0])

// TEMP: the temperature roles are compiled in (a separate instantiation, so
// that the plain step keeps its register budget)
template <typename R, bool TEMP>
__global__ void __launch_bounds__(32 * kSeg, TEMP ? 5 : SB_LINEA_MINB) k_lineA(Grid g, Bufs bf, int rk1) {
  __shared__ double xch[kSeg][16][2][SB_XS];
  LineThread L;
  if (!line_thread(g, 3, &L)) return;  // whole blocks
  Member &M = bf.mem[L.b];
  if (M.halted) return;  // uniform per block
  const int N = g.my, ystr = blockDim.x;
  const int rk = rk1 - 1;
  double *ys = ycol();
  const FacView V1(bf.d1, 0), V2(bf.d2, 0);
  const SegView W1(bf.d1, 0), W2(bf.d2, 0);
  const double Dt = M.Deltat, nu = M.nu;
  if (L.mean) {
    // visc3d(u00, rf0u, m=1, rk=0) and the RK3 update of the mean profiles
    // (cross.f90:666-672,703-723,753-756); no shear phase, no remap
    R *mu = (R *)bf.mu + (long)L.b * 2 * N + L.c;
    R *mwk = (R *)bf.mwk + (long)L.b * 2 * N + L.c;
    const R *mrf = (const R *)bf.mrf + (long)L.b * 2 * N + L.c;
    const cd one = mk(1.0, 0.0);
    // with the temperature, line slot 1 carries tb00: rf0tb = d(-vT_00)/dy
    // (crosst.f90:642-645) from the (0,0) line of -vT, kept in mtr; slot 0
    // computes a d/dy of the mean that is not used
    const bool ts = TEMP && L.l == 1;
    if (TEMP) {
      const TailLoad T1{bf.tl1o + (long)L.b * g.nkx * SB_TAIL};
      const R *src = ts ? (const R *)bf.R2 + (long)L.b * g.field + L.c : (const R *)mu;
      SEG_SOLVE(src, ts ? g.plane : 2L, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6],
                true);
      if (ts && L.c == 0) {
        R *mtr = (R *)bf.mtr + (long)L.b * 2 * N;
        for (int i = L.r0; i <= L.r1; i++) mtr[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
      }
    }
    const TailLoad T2{bf.tl2o + (long)L.b * g.nkx * SB_TAIL};
    R *mline = ts ? (R *)bf.mt + (long)L.b * 2 * N + L.c : mu;
    SEG_SOLVE(mline, 2, V2, W2, T2, one, one, g.rh2[3], g.rh2[4], g.rh2[5], g.rh2[6], false);
    const R gk = (R)kGama[rk], zk = (R)kZeta[rk];
    if (ts) {
      // visc3d(tb00, rf0tb, rk=0, fkappa) and the RK3 update of tb00
      // (crosst.f90:751-754,797-826,877-880)
      if (L.c == 0) {
        R *mt = mline, *mtwk = (R *)bf.mtwk + (long)L.b * 2 * N;
        const R *mtr = (const R *)bf.mtr + (long)L.b * 2 * N;
        for (int i = L.r0; i <= L.r1; i++) {
          const int j = i - 1;
          const R rf = mtr[2 * j] +
                       (R)(g.kappa * (-(0.0 * (double)mt[2 * j]) + ys[(i - L.r0) * ystr]));
          R wk = (rk == 0) ? gk * rf : mtwk[2 * j] + gk * rf;
          const R tn = mt[2 * j] + (R)Dt * wk;
          if (rk < 2) wk = rf * zk;
          mt[2 * j] = tn;
          mtwk[2 * j] = wk;
        }
      }
      return;
    }
    // inertial force and window damping of rf0u (cross.f90:622-626;
    // add_damping, operators.f90:60-78)
    const bool damp = g.damp && L.c == 0;
    const bool xf = g.force == -1 && L.c == 0;
    for (int i = L.r0; i <= L.r1; i++) {
      const int j = i - 1;
      R rf0 = mrf[2 * j];
      if (xf) rf0 = (R)((double)rf0 + g.xforce);
      if (damp) {
        const double y = (double)j * g.dy - 0.5 * g.Ly;
        const double hw = 1.0 - (0.25 * (1.0 + tanh(6.0 * (g.damp_a - y) / g.lz + 3.0))) *
                                    (1.0 + tanh(6.0 * (g.damp_a + y) / g.lz + 3.0));
        rf0 = (R)((double)rf0 - g.damp_up * hw * (double)mu[2 * j]);
      }
      const R rf = rf0 + (R)(nu * (-(0.0 * (double)mu[2 * j]) + ys[(i - L.r0) * ystr]));
      R wk = (rk == 0) ? gk * rf : mwk[2 * j] + gk * rf;
      const R un = mu[2 * j] + (R)Dt * wk;
      if (rk < 2) wk = rf * zk;
      if (L.active) {
        mu[2 * j] = un;
        mwk[2 * j] = wk;
      }
    }
    return;
  }
  const long off = (long)L.b * g.field + 2 * L.lc + L.c;
  const long ps = g.plane;
  const int i = L.i, k = L.k;
  const cd shp = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * i);
  const cd shm = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
  const double a = g.alp * i;
  const double gz = g.gam * ((k <= g.nz) ? k : k - g.mz);
  if (L.role == 0) {
    const TailLoad T1{bf.tl1o + ((long)L.b * g.nkx + i) * SB_TAIL};
    // d/dy (dH1/dx + dH3/dz) (cross.f90:565-575)
    SEG_SOLVE((const R *)bf.D + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
              g.rh1[6], true);
    store_col(ys, ystr, (R *)bf.T + off, ps, L);
    if (TEMP) {
      // temperature: ht += d(-vT)/dy (crosst.f90:633-636,677)
      SEG_SOLVE((const R *)bf.R2 + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                g.rh1[6], true);
      if (L.active) {
        R *ht = (R *)bf.Ht + off;
        for (int r = L.r0; r <= L.r1; r++) {
          const long q = (long)(r - 1) * ps;
          ht[q] = ht[q] + (R)ys[(r - L.r0) * ystr];
        }
      }
    }
    return;
  }
  const TailLoad T2{bf.tl2o + ((long)L.b * g.nkx + i) * SB_TAIL};
  if (L.role == 2) {
    // d2(phi)/dy2 for the viscous term of the phi equation (cross.f90:660)
    SEG_SOLVE((const R *)bf.phi + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5],
              g.rh2[6], false);
    store_col(ys, ystr, (R *)bf.S + off, ps, L);
    return;
  }
  if (TEMP) {
    // temperature, beside the omega_y update of this role: lap(tb) =
    // d2(tb)/dy2 - k^2 tb, shared by the thermal diffusion and the buoyancy
    // term (visc3d, crosst.f90:734-738)
    SEG_SOLVE((const R *)bf.tb + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5],
              g.rh2[6], false);
    if (L.active) {
      const R *tb = (const R *)bf.tb + off;
      R *lt = (R *)bf.Lt + off;
      const double k2 = a * a + gz * gz;
      for (int r = L.r0; r <= L.r1; r++) {
        const long q = (long)(r - 1) * ps;
        lt[q] = (R)(-(k2 * (double)tb[q]) + ys[(r - L.r0) * ystr]);
      }
    }
  }
  // role 1: hg += nu*lap(omega_y) (visc3d, cross.f90:659), RK3 update, remaps.
  // d2(omega_y)/dy2 of the substep's starting state was taken by k_lineB of the
  // previous substep, unless a y filter changed the state since
  if (g.ydeal) {
    SEG_SOLVE((const R *)bf.vor + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5],
              g.rh2[6], false);
  } else {
    const R *lv = (const R *)bf.Lv + off;
    for (int r = L.r0; r <= L.r1; r++) ys[(r - L.r0) * ystr] = (double)lv[(long)(r - 1) * ps];
  }
  const bool is00 = (i == 0 && k == 0);
  const double *mf1 = bf.mf1 + (long)L.b * 2 * N * g.nkx + 2 * i;
  const double *mf2 = bf.mf2 + (long)L.b * 2 * N * g.nkx + 2 * i;
  rk_update<R>(ys, ystr, (const R *)bf.G + off, nullptr, (R *)bf.vor + off, (R *)bf.vorwk + off,
               ps, L, rk, is00 ? 0.0 : nu, a * a + gz * gz, Dt, mf1, mf2, 2 * g.nkx);
}

template <typename R, bool TEMP>
__global__ void __launch_bounds__(32 * kSeg, SB_LINE_MINB) k_lineB(Grid g, Bufs bf, int mode) {
  __shared__ double xch[kSeg][16][2][SB_XS];
  LineThread L;
  if (!line_thread(g, TEMP ? 3 : 2, &L)) return;
  Member &M = bf.mem[L.b];
  if (M.halted) return;
  const int N = g.my, ystr = blockDim.x;
  double *ys = ycol();
  const FacView V1(bf.d1, 0);
  const SegView W1(bf.d1, 0);
  if (L.mean) {
    // derivyc(u00, rf0u, 1, 1, 0) and of w00, used by hvhg (cross.f90:1186-1192)
    const R *mu = (const R *)bf.mu + (long)L.b * 2 * N + L.c;
    R *mdu = (R *)bf.mdu + (long)L.b * 2 * N + L.c;
    const cd one = mk(1.0, 0.0);
    const TailLoad T1{bf.tl1o + (long)L.b * g.nkx * SB_TAIL};
    SEG_SOLVE(mu, 2, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
    if (L.active)
      for (int i = L.r0; i <= L.r1; i++) mdu[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
    return;
  }
  const long off = (long)L.b * g.field + 2 * L.lc + L.c;
  const long ps = g.plane;
  const int i = L.i, k = L.k;
  // the phase at t + c_k dt (substeps) or at t (prologue)
  const double *sh = (mode == 0) ? bf.sh_old : bf.sh_new;
  const double *tl1 = (mode == 0) ? bf.tl1o : bf.tl1n;
  const double *tl2 = (mode == 0) ? bf.tl2o : bf.tl2n;
  const cd shp = ldc2(sh + (long)L.b * 4 * g.nkx + 2 * i);
  const cd shm = ldc2(sh + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
  const TailLoad T1{tl1 + ((long)L.b * g.nkx + i) * SB_TAIL};
  if (L.role == 0) {
    // d(omega_y)/dy (cross.f90:440)
    SEG_SOLVE((const R *)bf.vor + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
              g.rh1[6], true);
    store_col(ys, ystr, (R *)bf.D + off, ps, L);
    if (!g.ydeal) {
      // d2(omega_y)/dy2 of the next substep's starting state (its visc3d,
      // cross.f90:659), same phase
      const FacView V2(bf.d2, 0);
      const SegView W2(bf.d2, 0);
      const TailLoad T2{tl2 + ((long)L.b * g.nkx + i) * SB_TAIL};
      SEG_SOLVE((const R *)bf.vor + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5],
                g.rh2[6], false);
      store_col(ys, ystr, (R *)bf.Lv + off, ps, L);
    }
    return;
  }
  const bool is00 = (i == 0 && k == 0);
  if (TEMP && L.role == 2) {
    // temperature: ht + fkappa lap(tb), RK3 update of tb, zeta store and
    // moving_frame_t remaps (crosst.f90:734-735,782-872); nothing in the
    // prologue
    if (mode >= 1) {
      const double *mf1 = bf.mf1 + (long)L.b * 2 * N * g.nkx + 2 * i;
      const double *mf2 = bf.mf2 + (long)L.b * 2 * N * g.nkx + 2 * i;
      rk_update<R>(ys, ystr, (const R *)bf.Ht + off, nullptr, (R *)bf.tb + off,
                   (R *)bf.tbwk + off, ps, L, mode - 1, is00 ? 0.0 : g.kappa, 0.0, M.Deltat, mf1,
                   mf2, 2 * g.nkx, (const R *)bf.Lt + off);
    }
    return;
  }
  if (mode >= 1) {
    // hv = hv - d/dy(dH1/dx + dH3/dz) + nu*lap(phi), RK3 update, remaps
    // (cross.f90:607,660,694-781); with the temperature + gbeta lap(tb)
    // (crosst.f90:737)
    const int rk = mode - 1;
    const double a = g.alp * i;
    const double gz = g.gam * ((k <= g.nz) ? k : k - g.mz);
    const double *mf1 = bf.mf1 + (long)L.b * 2 * N * g.nkx + 2 * i;
    const double *mf2 = bf.mf2 + (long)L.b * 2 * N * g.nkx + 2 * i;
    // the d2(phi)/dy2 of k_lineA goes through the shared buffer
    const R *S = (const R *)bf.S + off;
    for (int r = L.r0; r <= L.r1; r++) ys[(r - L.r0) * ystr] = (double)S[(long)(r - 1) * ps];
    rk_update<R>(ys, ystr, (const R *)bf.V + off, (const R *)bf.T + off, (R *)bf.phi + off,
                 (R *)bf.phiwk + off, ps, L, rk, is00 ? 0.0 : M.nu, a * a + gz * gz, M.Deltat,
                 mf1, mf2, 2 * g.nkx, nullptr,
                 (TEMP && !is00) ? (const R *)bf.Lt + off : nullptr, g.gbeta);
    __syncthreads();  // the whole updated line is read below
  }
  // v = lapcdy(phi) (cross.f90:784-795, first step: 408-426); hg(0,0) keeps
  // the value the nonlinear stage left (zero), or zero in the prologue
  {
    const FacView VH(bf.hz, hz_line(g, L.lc));
    const SegView WH(bf.hz, hz_line(g, L.lc));
    const TailMake TH{VH, shp, N};
    SEG_SOLVE((const R *)bf.phi + off, ps, VH, WH, TH, shp, shm, g.pr2[3], g.pr2[4], g.pr2[5],
              g.pr2[6], false);
    if (is00) {
      if (mode == 0 && L.active)
        for (int r = L.r0; r <= L.r1; r++) ((R *)bf.G)[off + (long)(r - 1) * ps] = (R)0;
    } else {
      store_col(ys, ystr, (R *)bf.G + off, ps, L);
    }
  }
  __syncthreads();  // v of all segments is read below
  // dv/dy (cross.f90:442)
  SEG_SOLVE((const R *)bf.G + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5], g.rh1[6],
            true);
  store_col(ys, ystr, (R *)bf.V + off, ps, L);
}

// ---------------------------------------------------------------------------
// k_lineF: the y-line work of one substep in one kernel, for the plain step
// (no temperature, no y filter or y dealiasing; an LES step qualifies, its
// k_lineL runs before).  Per line, k_lineA's and k_lineB's work is a chain of
// solves that never leaves the line, so one block can take 16 lines through
// all of it with two pipelines of kSeg warps (pipeline 0: omega_y, pipeline
// 1: phi), each doing one solve or one pointwise update per phase:
//   phase  pipeline 0                             pipeline 1
//   1      T = d/dy(dH1/dx + dH3/dz)              S = d2(phi)/dy2
//   2      omega_y: hg + nu lap, RK3 update,      phi: hv - T + nu lap, RK3
//          zeta store, remaps (d2 from Lv)        update, zeta store, remaps
//   3      d(omega_y)/dy -> D                     v = lapcdy(phi) -> G
//   4      d2(omega_y)/dy2 -> Lv                  dv/dy -> V
// All warps of a block then carry the same work (the split kernels pair a
// heavy role with a light one on the SM sub-partitions), and T and S stay in
// shared memory, rounded to the storage type as k_lineA stores them, so the
// step is the split kernels' step.  The mean block runs the mean lines on
// pipeline 0 (nu u00'' and the mean update, then du00/dy for the next
// substep).  Every phase passes the same block barriers on both pipelines
// (two per solve, `seg_idle` where a pipeline has no solve, one after each
// of phases 1-3); the pipeline branches are uniform per warp.
__device__ __forceinline__ void seg_idle() {
  __syncthreads();
  __syncthreads();
}

// rk_update with the subtracted right-hand-side term and d2f/dy2 given per
// row by functors (sub(h, i) returns h minus the term; d2(i) the derivative),
// the same arithmetic
template <typename R, class SubF, class D2F>
__device__ __forceinline__ void rk_update_fn(const SubF &sub, const D2F &d2,
                                             const R *__restrict__ rhs, R *__restrict__ f,
                                             R *__restrict__ fwk, long ps, const LineThread &L,
                                             int rk, double nuv, double k2, double Dt,
                                             const double *__restrict__ mf1,
                                             const double *__restrict__ mf2, long mfs) {
  const R gk = (R)kGama[rk], zk = (R)kZeta[rk], dtr = (R)Dt;
  const int c = L.c;
#pragma unroll 2
  for (int i = L.r0; i <= L.r1; i++) {
    const int j = i - 1;
    const long q = (long)j * ps;
    const R fo = f[q];
    R h = sub(rhs[q], i);
    const double vis = -(k2 * (double)fo) + d2(i, q);
    h = h + (R)(nuv * vis);
    R wk = (rk == 0) ? gk * h : fwk[q] + gk * h;
    const double fn = (double)(fo + dtr * wk);
    const cd m2 = ldc2(mf2 + (long)j * mfs);
    const double fnm = cmul_c(fn, __shfl_xor_sync(0xffffffffu, fn, 1), m2, c);
    if (rk < 2) {
      const cd m1 = ldc2(mf1 + (long)j * mfs);
      const double wz = (double)(h * zk);
      wk = (R)cmul_c(wz, __shfl_xor_sync(0xffffffffu, wz, 1), m1, c);
    }
    if (L.active) {
      f[q] = (R)fnm;
      fwk[q] = wk;
    }
  }
}

// block -> (member, group of 16 lines), the member's mean block last; warp ->
// (pipeline, segment); lane -> (line of the group, component)
__device__ __forceinline__ bool line_thread_f(const Grid &g, LineThread *L, int *pipe) {
  const int per = g.ngrp + 1;
  L->b = blockIdx.x / per;
  if (L->b >= g.B) return false;
  const int r = blockIdx.x - L->b * per;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  *pipe = w / kSeg;
  L->role = *pipe;
  L->mean = r >= g.ngrp;
  L->s = w - *pipe * kSeg;
  L->l = lane >> 1;
  L->c = lane & 1;
  const int nl = g.nkx * g.mz;
  if (L->mean) {
    L->lc = 0;
    L->active = (L->l == 0);
  } else {
    L->lc = (long)r * 16 + L->l;
    L->active = L->lc < nl;
    if (!L->active) L->lc = nl - 1;
  }
  L->i = (int)(L->lc % g.nkx);
  L->k = (int)(L->lc / g.nkx);
  L->r0 = g.slo[L->s];
  L->r1 = (L->s == kSeg - 1) ? g.my : g.shi[L->s];
  return true;
}

#define SEG_SOLVE_P(U, PS, VIEW, SVIEW, TAIL, SHP, SHM, R0, R1, R2, R3, ANTI)                   \
  solve_seg<kSeg>(U, PS, ys, ystr, N, VIEW, SVIEW, TAIL, SHP, SHM, L.c, L.s, L.l, g.slo, g.shi, \
                  R0, R1, R2, R3, ANTI, &xch[pipe][0][0][0][0])

// k_lineF: resident warps per SM the kernel is register-budgeted for (a
// build-time knob; 0 leaves the registers to the compiler).  12 warps cap it
// at 168 registers without spills (from 202-214): the 64-box 64x32x32 mixed
// ensemble steps 2.3% faster (more lines in flight per SM), the one-box
// 192x96x96 step is unchanged (its 253 blocks fit one wave either way), and
// 16 warps (128 registers) spill and lose 4%.
#ifndef SB_LINEF_WARPS
#define SB_LINEF_WARPS 12
#endif
template <typename R>
__global__ void __launch_bounds__(64 * kSeg, SB_LINEF_WARPS / (2 * kSeg) > 0 ? SB_LINEF_WARPS / (2 * kSeg) : 1)
    k_lineF(Grid g, Bufs bf, int rk1) {
  __shared__ double xch[2][kSeg][16][2][SB_XS];
  LineThread L;
  int pipe = 0;
  if (!line_thread_f(g, &L, &pipe)) return;  // whole blocks
  Member &M = bf.mem[L.b];
  if (M.halted) return;  // uniform per block
  const int N = g.my, ystr = blockDim.x;
  const int rk = rk1 - 1;
  double *ys = ycol();
  const FacView V1(bf.d1, 0), V2(bf.d2, 0);
  const SegView W1(bf.d1, 0), W2(bf.d2, 0);
  const double Dt = M.Deltat, nu = M.nu;
  if (L.mean) {
    R *mu = (R *)bf.mu + (long)L.b * 2 * N + L.c;
    const cd one = mk(1.0, 0.0);
    // phase 1: nu u00'' (visc3d(u00, rf0u, m=1, rk=0), cross.f90:666-672)
    if (pipe == 0) {
      const TailLoad T2{bf.tl2o + (long)L.b * g.nkx * SB_TAIL};
      SEG_SOLVE_P(mu, 2, V2, W2, T2, one, one, g.rh2[3], g.rh2[4], g.rh2[5], g.rh2[6], false);
    } else {
      seg_idle();
    }
    __syncthreads();
    // phase 2: forcing, damping and the RK3 update of the mean profiles
    // (cross.f90:622-626,703-723,753-756), k_lineA's mean block
    if (pipe == 0) {
      R *mwk = (R *)bf.mwk + (long)L.b * 2 * N + L.c;
      const R *mrf = (const R *)bf.mrf + (long)L.b * 2 * N + L.c;
      const R gk = (R)kGama[rk], zk = (R)kZeta[rk];
      const bool damp = g.damp && L.c == 0;
      const bool xf = g.force == -1 && L.c == 0;
      for (int i = L.r0; i <= L.r1; i++) {
        const int j = i - 1;
        R rf0 = mrf[2 * j];
        if (xf) rf0 = (R)((double)rf0 + g.xforce);
        if (damp) {
          const double y = (double)j * g.dy - 0.5 * g.Ly;
          const double hw = 1.0 - (0.25 * (1.0 + tanh(6.0 * (g.damp_a - y) / g.lz + 3.0))) *
                                      (1.0 + tanh(6.0 * (g.damp_a + y) / g.lz + 3.0));
          rf0 = (R)((double)rf0 - g.damp_up * hw * (double)mu[2 * j]);
        }
        const R rf = rf0 + (R)(nu * (-(0.0 * (double)mu[2 * j]) + ys[(i - L.r0) * ystr]));
        R wk = (rk == 0) ? gk * rf : mwk[2 * j] + gk * rf;
        const R un = mu[2 * j] + (R)Dt * wk;
        if (rk < 2) wk = rf * zk;
        if (L.active) {
          mu[2 * j] = un;
          mwk[2 * j] = wk;
        }
      }
    }
    __syncthreads();
    // phase 3: du00/dy, dw00/dy of the updated profiles (cross.f90:1186-1192)
    if (pipe == 0) {
      R *mdu = (R *)bf.mdu + (long)L.b * 2 * N + L.c;
      const TailLoad T1{bf.tl1o + (long)L.b * g.nkx * SB_TAIL};
      SEG_SOLVE_P(mu, 2, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
      if (L.active)
        for (int i = L.r0; i <= L.r1; i++) mdu[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
    } else {
      seg_idle();
    }
    __syncthreads();
    seg_idle();  // phase 4
    return;
  }
  const long off = (long)L.b * g.field + 2 * L.lc + L.c;
  const long ps = g.plane;
  const int i = L.i, k = L.k;
  const bool is00 = (i == 0 && k == 0);
  const double a = g.alp * i;
  const double gz = g.gam * ((k <= g.nz) ? k : k - g.mz);
  const double k2 = a * a + gz * gz;
  const double *mf1 = bf.mf1 + (long)L.b * 2 * N * g.nkx + 2 * i;
  const double *mf2 = bf.mf2 + (long)L.b * 2 * N * g.nkx + 2 * i;
  {
    // phases 1-2 at the phase of time t
    const cd shp = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * i);
    const cd shm = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
    if (pipe == 0) {
      // T = d/dy (dH1/dx + dH3/dz) (cross.f90:565-575)
      const TailLoad T1{bf.tl1o + ((long)L.b * g.nkx + i) * SB_TAIL};
      SEG_SOLVE_P((const R *)bf.D + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                  g.rh1[6], true);
      // the value k_lineA would store
      for (int r = L.r0; r <= L.r1; r++)
        ys[(r - L.r0) * ystr] = (double)(R)ys[(r - L.r0) * ystr];
    } else {
      // S = d2(phi)/dy2 for the viscous term of the phi equation (cross.f90:660)
      const TailLoad T2{bf.tl2o + ((long)L.b * g.nkx + i) * SB_TAIL};
      SEG_SOLVE_P((const R *)bf.phi + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4],
                  g.rh2[5], g.rh2[6], false);
      for (int r = L.r0; r <= L.r1; r++)
        ys[(r - L.r0) * ystr] = (double)(R)ys[(r - L.r0) * ystr];
    }
  }
  __syncthreads();
  if (pipe == 0) {
    // hg += nu lap(omega_y) (visc3d, cross.f90:659) with d2(omega_y)/dy2 of
    // the substep's starting state, taken in phase 4 of the previous substep
    // (or the prologue); RK3 update, zeta store, remaps (cross.f90:694-781)
    const R *lv = (const R *)bf.Lv + off;
    rk_update_fn<R>([](R h, int) { return h; },
                    [lv](int, long q) { return (double)lv[q]; }, (const R *)bf.G + off,
                    (R *)bf.vor + off, (R *)bf.vorwk + off, ps, L, rk, is00 ? 0.0 : nu, k2, Dt,
                    mf1, mf2, 2 * g.nkx);
  } else {
    // hv - d/dy(dH1/dx + dH3/dz) + nu lap(phi), RK3 update, zeta store, remaps
    // (cross.f90:607,660,694-781); T from pipeline 0's column of the same
    // (segment, line, component)
    const double *ys0 = ys - 32 * kSeg;
    const int r0 = L.r0;
    const double *yb = ys;
    rk_update_fn<R>([ys0, r0, ystr](R h, int r) { return h - (R)ys0[(r - r0) * ystr]; },
                    [yb, r0, ystr](int r, long) { return yb[(r - r0) * ystr]; },
                    (const R *)bf.V + off, (R *)bf.phi + off, (R *)bf.phiwk + off, ps, L, rk,
                    is00 ? 0.0 : M.nu, k2, Dt, mf1, mf2, 2 * g.nkx);
  }
  __syncthreads();  // whole updated lines are read below
  // phases 3-4 at the phase of time t + c_k dt
  const cd shp = ldc2(bf.sh_new + (long)L.b * 4 * g.nkx + 2 * i);
  const cd shm = ldc2(bf.sh_new + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
  const TailLoad T1{bf.tl1n + ((long)L.b * g.nkx + i) * SB_TAIL};
  if (pipe == 0) {
    // d(omega_y)/dy (cross.f90:440)
    SEG_SOLVE_P((const R *)bf.vor + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                g.rh1[6], true);
    store_col(ys, ystr, (R *)bf.D + off, ps, L);
  } else {
    // v = lapcdy(phi) (cross.f90:784-795); hg(0,0) keeps the value the
    // nonlinear stage left (zero)
    const FacView VH(bf.hz, hz_line(g, L.lc));
    const SegView WH(bf.hz, hz_line(g, L.lc));
    const TailMake TH{VH, shp, N};
    SEG_SOLVE_P((const R *)bf.phi + off, ps, VH, WH, TH, shp, shm, g.pr2[3], g.pr2[4], g.pr2[5],
                g.pr2[6], false);
    if (!is00) store_col(ys, ystr, (R *)bf.G + off, ps, L);
  }
  __syncthreads();  // v of all segments is read below
  if (pipe == 0) {
    // d2(omega_y)/dy2 of the next substep's starting state (its visc3d,
    // cross.f90:659)
    const TailLoad T2{bf.tl2n + ((long)L.b * g.nkx + i) * SB_TAIL};
    SEG_SOLVE_P((const R *)bf.vor + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5],
                g.rh2[6], false);
    store_col(ys, ystr, (R *)bf.Lv + off, ps, L);
  } else {
    // dv/dy (cross.f90:442)
    SEG_SOLVE_P((const R *)bf.G + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                g.rh1[6], true);
    store_col(ys, ystr, (R *)bf.V + off, ps, L);
  }
}

// ---------------------------------------------------------------------------
// k_lineI: the y-line work of one substep of the semi-implicit viscous branch
// (explicit = 0, cross.f90:797-989; crosst.f90:916-1195 with TEMP), without
// LES, y filter or y dealiasing.  k_lineF's block (pipelines of kSeg warps on
// 16 lines), with a third pipeline for the scalar tb under TEMP:
//   phase  pipeline 0 (omega_y)         pipeline 1 (phi)          pipeline 2 (tb)
//   1      T = d/dy(dH1/dx + dH3/dz)    S = d2(phi)/dy2           Lt = lap(tb)
//   2      -                            -                         ht += d(-vT)/dy
//   3      right-hand side -> T buf,    the same for phi with     the same for tb
//          zeta store -> vorwk          hv - T + gbeta Lt         -> R2 buf
//   4      omega_y = lapcdy(rhs,        phi = lapcdy(rhs,         tb = lapcdy(rhs,
//          k^2 + dtr1)                  k^2 + dtr1)               k^2 + dtr1k)
//   5      d(omega_y)/dy -> D           v = lapcdy(phi, k^2) -> G -
//   6      d2(omega_y)/dy2 -> Lv        dv/dy -> V                -
// (phase 2 and pipeline 2 only with TEMP), with, per point (cross.f90:800-867,
// crosst.f90:934-1028, in this order),
//   wk = [wk +] gama_k h;  wk += alpha_k nu (f'' - k^2 f);  wk += f/Dt;
//   rhs = -Re ibeta_k wk (tb: -ibeta_k/fkappa, diffusivity fkappa), moved to
//   the frame of t + c_k Dt (moving_frame, moving_frame_t);
// dtr1 = Re ibeta_k / Dt, dtr1k = ibeta_k / (fkappa Dt); the Helmholtz factors
// of the substep come from k_hfac.  The mean block: u00, w00 on pipeline 0
// (u00'' in phase 1, the right-hand side in phase 3 through mdu, the real
// Helmholtz solve of dtr1 in phase 4, du00/dy in phase 5), tb00 on pipeline 2
// (d(-vT00)/dy -> mtr in phase 1, tb00'' in phase 2, the right-hand side
// through mtr in phase 3, the solve of dtr1k in phase 4).  The (0,0) line
// keeps its state (cross.f90 and crosst.f90 skip it).
__device__ __constant__ static const double kAlpha[3] = {29.0 / 96.0, -3.0 / 40.0, 1.0 / 6.0};
__device__ __constant__ static const double kIbetaL[3] = {160.0 / 37.0, 24.0 / 5.0, 6.0};

template <typename R, bool TEMP>
__global__ void __launch_bounds__((TEMP ? 96 : 64) * kSeg, 1) k_lineI(Grid g, Bufs bf, int rk1) {
  constexpr int NP = TEMP ? 3 : 2;
  __shared__ double xch[NP][kSeg][16][2][SB_XS];
  LineThread L;
  int pipe = 0;
  if (!line_thread_f(g, &L, &pipe)) return;  // whole blocks
  Member &M = bf.mem[L.b];
  if (M.halted) return;  // uniform per block
  const int N = g.my, ystr = blockDim.x;
  const int rk = rk1 - 1;
  double *ys = ycol();
  const FacView V1(bf.d1, 0), V2(bf.d2, 0);
  const SegView W1(bf.d1, 0), W2(bf.d2, 0);
  const double Dt = M.Deltat, nu = M.nu;
  const double fa = kAlpha[rk] * nu, fb = -M.Re * kIbetaL[rk], rdt = 1.0 / Dt;
  const double fat = TEMP ? kAlpha[rk] * g.kappa : 0.0;
  const double fbt = TEMP ? -(1.0 / g.kappa) * kIbetaL[rk] : 0.0;
  const R gk = (R)kGama[rk], zk = (R)kZeta[rk];
  // this box's entries of the implicit factors: lines (kx, kz >= 0), then the mean line
  const int nl = g.nkx * (g.nz + 1);
  const long hline0 = (long)L.b * (nl + 1);
  if (L.mean) {
    R *mu = (R *)bf.mu + (long)L.b * 2 * N + L.c;
    R *mdu = (R *)bf.mdu + (long)L.b * 2 * N + L.c;
    R *mt = TEMP ? (R *)bf.mt + (long)L.b * 2 * N + L.c : nullptr;
    R *mtr = TEMP ? (R *)bf.mtr + (long)L.b * 2 * N + L.c : nullptr;
    const cd one = mk(1.0, 0.0);
    const TailLoad T1{bf.tl1o + (long)L.b * g.nkx * SB_TAIL};
    const TailLoad T2{bf.tl2o + (long)L.b * g.nkx * SB_TAIL};
    // phase 1: u00'' (visc3d(u00, u00wk, m=1, rk=0), cross.f90:842-845);
    // rf0tb = d(-vT_00)/dy from the (0,0) line of -vT (crosst.f90:642-645)
    if (pipe == 0) {
      SEG_SOLVE_P(mu, 2, V2, W2, T2, one, one, g.rh2[3], g.rh2[4], g.rh2[5], g.rh2[6], false);
    } else if (TEMP && pipe == 2) {
      const R *src = (const R *)bf.R2 + (long)L.b * g.field + L.c;
      SEG_SOLVE_P(src, g.plane, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
      if (L.active && L.c == 0)
        for (int i = L.r0; i <= L.r1; i++) mtr[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
    } else {
      seg_idle();
    }
    __syncthreads();
    if constexpr (TEMP) {
      // phase 2: tb00'' (visc3d(tb00, tb00wk, rk=0), crosst.f90:994-997)
      if (pipe == 2)
        SEG_SOLVE_P(mt, 2, V2, W2, T2, one, one, g.rh2[3], g.rh2[4], g.rh2[5], g.rh2[6], false);
      else
        seg_idle();
      __syncthreads();
    }
    // phase 3: forcing, damping, the mean right-hand sides and the zeta stores
    // (cross.f90:622-626,830-867,972-975; crosst.f90:975-1028,1163-1168)
    if (pipe == 0) {
      R *mwk = (R *)bf.mwk + (long)L.b * 2 * N + L.c;
      const R *mrf = (const R *)bf.mrf + (long)L.b * 2 * N + L.c;
      const bool damp = g.damp && L.c == 0;
      const bool xf = g.force == -1 && L.c == 0;
      for (int i = L.r0; i <= L.r1; i++) {
        const int j = i - 1;
        R rf0 = mrf[2 * j];
        if (xf) rf0 = (R)((double)rf0 + g.xforce);
        if (damp) {
          const double y = (double)j * g.dy - 0.5 * g.Ly;
          const double hw = 1.0 - (0.25 * (1.0 + tanh(6.0 * (g.damp_a - y) / g.lz + 3.0))) *
                                      (1.0 + tanh(6.0 * (g.damp_a + y) / g.lz + 3.0));
          rf0 = (R)((double)rf0 - g.damp_up * hw * (double)mu[2 * j]);
        }
        const R wk = (rk == 0) ? gk * rf0 : mwk[2 * j] + gk * rf0;
        double w = (double)wk;
        w = w + fa * (-(0.0 * (double)mu[2 * j]) + ys[(i - L.r0) * ystr]);
        const double rhs = fb * (w + rdt * (double)mu[2 * j]);
        if (L.active) {
          mdu[2 * j] = (R)rhs;
          if (rk < 2) mwk[2 * j] = zk * rf0;
        }
      }
    } else if (TEMP && pipe == 2 && L.c == 0) {
      R *mtwk = (R *)bf.mtwk + (long)L.b * 2 * N;
      for (int i = L.r0; i <= L.r1; i++) {
        const int j = i - 1;
        const R rf0 = mtr[2 * j];
        const R wk = (rk == 0) ? gk * rf0 : mtwk[2 * j] + gk * rf0;
        double w = (double)wk;
        w = w + fat * (-(0.0 * (double)mt[2 * j]) + ys[(i - L.r0) * ystr]);
        const double rhs = fbt * (w + rdt * (double)mt[2 * j]);
        if (L.active) {
          mtr[2 * j] = (R)rhs;
          if (rk < 2) mtwk[2 * j] = zk * rf0;
        }
      }
    }
    __syncthreads();
    // phase 4: u00 = lapcdy(rhs, dtr1) (cross.f90:965-967), tb00 =
    // lapcdy(rhs, dtr1k) (crosst.f90:1158-1161), real lines
    if (pipe == 0) {
      const FacView VI(bf.hi, hline0 + nl);
      const SegView WI(bf.hi, hline0 + nl);
      const TailMake TI{VI, one, N};
      SEG_SOLVE_P((const R *)mdu, 2, VI, WI, TI, one, one, g.pr2[3], g.pr2[4], g.pr2[5], g.pr2[6],
                  false);
      store_col(ys, ystr, mu, 2, L);
    } else if (TEMP && pipe == 2) {
      const FacView VK(bf.hit, hline0 + nl);
      const SegView WK(bf.hit, hline0 + nl);
      const TailMake TK{VK, one, N};
      SEG_SOLVE_P((const R *)mtr, 2, VK, WK, TK, one, one, g.pr2[3], g.pr2[4], g.pr2[5],
                  g.pr2[6], false);
      if (L.active && L.c == 0)
        for (int i = L.r0; i <= L.r1; i++) mt[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
    } else {
      seg_idle();
    }
    __syncthreads();
    // phase 5: du00/dy, dw00/dy of the new profiles (cross.f90:1186-1192)
    if (pipe == 0) {
      SEG_SOLVE_P(mu, 2, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
      store_col(ys, ystr, mdu, 2, L);
    } else {
      seg_idle();
    }
    __syncthreads();
    seg_idle();  // phase 6
    return;
  }
  const long off = (long)L.b * g.field + 2 * L.lc + L.c;
  const long ps = g.plane;
  const int i = L.i, k = L.k;
  const bool is00 = (i == 0 && k == 0);
  const double a = g.alp * i;
  const double gz = g.gam * ((k <= g.nz) ? k : k - g.mz);
  const double k2 = gz * gz + a * a;
  const double *mf1 = bf.mf1 + (long)L.b * 2 * N * g.nkx + 2 * i;
  const double *mf2 = bf.mf2 + (long)L.b * 2 * N * g.nkx + 2 * i;
  {
    // phases 1-2 at the phase of time t
    const cd shp = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * i);
    const cd shm = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
    const TailLoad T1{bf.tl1o + ((long)L.b * g.nkx + i) * SB_TAIL};
    const TailLoad T2{bf.tl2o + ((long)L.b * g.nkx + i) * SB_TAIL};
    if (pipe == 0) {
      // T = d/dy (dH1/dx + dH3/dz) (cross.f90:565-575), as k_lineA stores it
      SEG_SOLVE_P((const R *)bf.D + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                  g.rh1[6], true);
      for (int r = L.r0; r <= L.r1; r++)
        ys[(r - L.r0) * ystr] = (double)(R)ys[(r - L.r0) * ystr];
    } else if (pipe == 1) {
      // S = d2(phi)/dy2 (visc3d, cross.f90:824)
      SEG_SOLVE_P((const R *)bf.phi + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4],
                  g.rh2[5], g.rh2[6], false);
    } else if (TEMP) {
      // lap(tb) = d2(tb)/dy2 - k^2 tb, for the buoyancy of the phi equation and
      // the diffusion of tb (crosst.f90:919-932,954-970)
      SEG_SOLVE_P((const R *)bf.tb + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4],
                  g.rh2[5], g.rh2[6], false);
      if (L.active) {
        const R *tb = (const R *)bf.tb + off;
        R *lt = (R *)bf.Lt + off;
        for (int r = L.r0; r <= L.r1; r++) {
          const long q = (long)(r - 1) * ps;
          lt[q] = (R)(-(k2 * (double)tb[q]) + ys[(r - L.r0) * ystr]);
        }
      }
    }
    __syncthreads();
    if constexpr (TEMP) {
      // phase 2: ht += d(-vT)/dy (crosst.f90:633-636,677)
      if (pipe == 2) {
        SEG_SOLVE_P((const R *)bf.R2 + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                    g.rh1[6], true);
        if (L.active) {
          R *ht = (R *)bf.Ht + off;
          for (int r = L.r0; r <= L.r1; r++) {
            const long q = (long)(r - 1) * ps;
            ht[q] = ht[q] + (R)ys[(r - L.r0) * ystr];
          }
        }
      } else {
        seg_idle();
      }
      __syncthreads();
    }
  }
  {
    // phase 3: right-hand sides of the Helmholtz equations and the zeta
    // stores (cross.f90:800-867,886-941; crosst.f90:934-1028,1106-1125);
    // omega_y'' from Lv, taken at the end of the previous substep (or by the
    // prologue)
    const R *h0 = pipe == 0 ? (const R *)bf.G + off
                            : (pipe == 1 ? (const R *)bf.V + off : (const R *)bf.Ht + off);
    R *f = pipe == 0 ? (R *)bf.vor + off : (pipe == 1 ? (R *)bf.phi + off : (R *)bf.tb + off);
    R *fwk = pipe == 0 ? (R *)bf.vorwk + off
                       : (pipe == 1 ? (R *)bf.phiwk + off : (R *)bf.tbwk + off);
    R *rhs_out = pipe == 0 ? (R *)bf.T + off : (pipe == 1 ? (R *)bf.S + off : (R *)bf.R2 + off);
    const R *lv = (const R *)bf.Lv + off;
    const R *lt = TEMP ? (const R *)bf.Lt + off : nullptr;
    const double *ys0 = ys - 32 * kSeg * pipe;  // pipeline 0's column (T)
    const double fvis = pipe == 2 ? fat : fa, fscale = pipe == 2 ? fbt : fb;
    const int c = L.c;
#pragma unroll 2
    for (int r = L.r0; r <= L.r1; r++) {
      const int j = r - 1;
      const long q = (long)j * ps;
      R h = h0[q];
      if (pipe == 1) {
        h = h - (R)ys0[(r - L.r0) * ystr];  // hv = hv - d/dy(...)
        if (TEMP && !is00) h = h + (R)(g.gbeta * (double)lt[q]);  // buoyancy
      }
      const R fo = f[q];
      const R wk = (rk == 0) ? gk * h : fwk[q] + gk * h;
      double w = (double)wk;
      if (!is00) {
        const double lap = pipe == 0 ? -(k2 * (double)fo) + (double)lv[q]
                                     : (pipe == 1 ? -(k2 * (double)fo) + ys[(r - L.r0) * ystr]
                                                  : (double)lt[q]);
        w = w + fvis * lap;
      }
      w = fscale * (w + rdt * (double)fo);
      const cd m2 = ldc2(mf2 + (long)j * 2 * g.nkx);
      const double rm = cmul_c(w, __shfl_xor_sync(0xffffffffu, w, 1), m2, c);
      double zs = 0.0;
      if (rk < 2) {
        const cd m1 = ldc2(mf1 + (long)j * 2 * g.nkx);
        const double wz = (double)(zk * h);
        zs = cmul_c(wz, __shfl_xor_sync(0xffffffffu, wz, 1), m1, c);
      }
      if (L.active) {
        rhs_out[q] = (R)rm;
        if (rk < 2) fwk[q] = (R)zs;
      }
    }
  }
  __syncthreads();
  // phases 4-6 at the phase of time t + c_k dt
  const cd shp = ldc2(bf.sh_new + (long)L.b * 4 * g.nkx + 2 * i);
  const cd shm = ldc2(bf.sh_new + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
  {
    // phase 4: the Helmholtz solves (cross.f90:894-925; crosst.f90:1094-1104)
    const Fac &FI = pipe == 2 ? bf.hit : bf.hi;
    const FacView VI(FI, hline0 + hz_line(g, L.lc));
    const SegView WI(FI, hline0 + hz_line(g, L.lc));
    const TailMake TI{VI, shp, N};
    const R *src = pipe == 0 ? (const R *)bf.T + off
                             : (pipe == 1 ? (const R *)bf.S + off : (const R *)bf.R2 + off);
    SEG_SOLVE_P(src, ps, VI, WI, TI, shp, shm, g.pr2[3], g.pr2[4], g.pr2[5], g.pr2[6], false);
    if (!is00)
      store_col(ys, ystr,
                pipe == 0 ? (R *)bf.vor + off : (pipe == 1 ? (R *)bf.phi + off : (R *)bf.tb + off),
                ps, L);
  }
  __syncthreads();  // whole updated lines are read below
  const TailLoad T1{bf.tl1n + ((long)L.b * g.nkx + i) * SB_TAIL};
  if (pipe == 0) {
    // d(omega_y)/dy (cross.f90:440)
    SEG_SOLVE_P((const R *)bf.vor + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                g.rh1[6], true);
    store_col(ys, ystr, (R *)bf.D + off, ps, L);
  } else if (pipe == 1) {
    // v = lapcdy(phi, k^2) (cross.f90:942-956); hg(0,0) keeps the value the
    // nonlinear stage left (zero)
    const FacView VH(bf.hz, hz_line(g, L.lc));
    const SegView WH(bf.hz, hz_line(g, L.lc));
    const TailMake TH{VH, shp, N};
    SEG_SOLVE_P((const R *)bf.phi + off, ps, VH, WH, TH, shp, shm, g.pr2[3], g.pr2[4], g.pr2[5],
                g.pr2[6], false);
    if (!is00) store_col(ys, ystr, (R *)bf.G + off, ps, L);
  } else {
    seg_idle();
  }
  __syncthreads();  // v of all segments is read below
  if (pipe == 0) {
    // d2(omega_y)/dy2 of the next substep's starting state
    const TailLoad T2{bf.tl2n + ((long)L.b * g.nkx + i) * SB_TAIL};
    SEG_SOLVE_P((const R *)bf.vor + off, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5],
                g.rh2[6], false);
    store_col(ys, ystr, (R *)bf.Lv + off, ps, L);
  } else if (pipe == 1) {
    // dv/dy (cross.f90:442)
    SEG_SOLVE_P((const R *)bf.G + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5],
                g.rh1[6], true);
    store_col(ys, ystr, (R *)bf.V + off, ps, L);
  } else {
    seg_idle();
  }
}

// LES y-operators (iuse_LES, cross.f90:565-608,639-647), between k_tables and
// k_lineA:
//   role 0: hg += d(rhgc2)/dy                       (derivyc, -> G)
//   role 1: hv += (kx^2 + kz^2 - d2/dy2)(-rhvc2), i.e. visc3d(rhvc2, hv,
//           rk = -(kx^2 + kz^2), fac = -1)          (-> V)
//   mean:   rf0u += d(T12_00)/dy, rf0w += d(T23_00)/dy
template <typename R>
__global__ void __launch_bounds__(32 * kSeg, SB_LINE_MINB) k_lineL(Grid g, Bufs bf) {
  __shared__ double xch[kSeg][16][2][SB_XS];
  LineThread L;
  if (!line_thread(g, 2, &L)) return;
  const Member &M = bf.mem[L.b];
  if (M.halted) return;
  const int N = g.my, ystr = blockDim.x;
  double *ys = ycol();
  const FacView V1(bf.d1, 0), V2(bf.d2, 0);
  const SegView W1(bf.d1, 0), W2(bf.d2, 0);
  if (L.mean) {
    const R *tx = (const R *)bf.txy + (long)L.b * 2 * N + L.c;
    R *mrf = (R *)bf.mrf + (long)L.b * 2 * N + L.c;
    const cd one = mk(1.0, 0.0);
    const TailLoad T1{bf.tl1o + (long)L.b * g.nkx * SB_TAIL};
    SEG_SOLVE(tx, 2, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
    if (L.active)
      for (int i = L.r0; i <= L.r1; i++)
        mrf[2 * (i - 1)] = mrf[2 * (i - 1)] + (R)ys[(i - L.r0) * ystr];
    return;
  }
  const long off = (long)L.b * g.field + 2 * L.lc + L.c;
  const long ps = g.plane;
  const int i = L.i, k = L.k;
  const cd shp = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * i);
  const cd shm = ldc2(bf.sh_old + (long)L.b * 4 * g.nkx + 2 * (g.nkx + i));
  if (L.role == 0) {
    const TailLoad T1{bf.tl1o + ((long)L.b * g.nkx + i) * SB_TAIL};
    SEG_SOLVE((const R *)bf.L2 + off, ps, V1, W1, T1, shp, shm, 0.0, g.rh1[4], g.rh1[5], g.rh1[6],
              true);
    R *G = (R *)bf.G + off;
    if (L.active)
      for (int r = L.r0; r <= L.r1; r++) {
        const long q = (long)(r - 1) * ps;
        G[q] = G[q] + (R)ys[(r - L.r0) * ystr];
      }
    return;
  }
  const TailLoad T2{bf.tl2o + ((long)L.b * g.nkx + i) * SB_TAIL};
  const R *u = (const R *)bf.L1 + off;
  SEG_SOLVE(u, ps, V2, W2, T2, shp, shm, g.rh2[3], g.rh2[4], g.rh2[5], g.rh2[6], false);
  if ((i == 0 && k == 0) || !L.active) return;
  const double a = g.alp * i;
  const double gz = g.gam * ((k <= g.nz) ? k : k - g.mz);
  const double rk = -(gz * gz + a * a);
  R *Vv = (R *)bf.V + off;
  for (int r = L.r0; r <= L.r1; r++) {
    const long q = (long)(r - 1) * ps;
    const double t = -(rk * (double)u[q]) + ys[(r - L.r0) * ystr];
    Vv[q] = Vv[q] + (R)(-1.0 * t);
  }
}

// Compact y-filter of the state (iydealiasing = 3: filterc,
// filter_shear_hepta.f90:104-148, called at cross.f90:214-227 and 476-490) at
// the start of substep rk (rk = 0: entry of a cross call), with the shear
// phase of the substep's starting offsets:
//   role 0: omega_y, role 1: phi (9-point right-hand side through the free
//           scratch fields S and T, then the heptadiagonal solve, in place)
//   mean:   u00, w00 (no phase), then their d/dy, which the nonlinear stage
//           takes from the filtered profiles (cross.f90:1186-1192)
template <typename R>
__global__ void __launch_bounds__(32 * kSeg) k_filter(Grid g, Bufs bf, int rk) {
  __shared__ double xch[kSeg][16][2][SB_XS];
  LineThread L;
  if (!line_thread(g, 2, &L)) return;
  const Member &M = bf.mem[L.b];
  if (M.halted) return;
  const int N = g.my, ystr = blockDim.x;
  double *ys = ycol();
  const FacView VF(bf.flt, 0);
  const SegView WF(bf.flt, 0);
  const long ps = L.mean ? 2 : g.plane;
  R *f, *scr;
  cd shp = mk(1.0, 0.0);
  if (L.mean) {
    f = (R *)bf.mu + (long)L.b * 2 * N + L.c;
    scr = (R *)bf.mdu + (long)L.b * 2 * N + L.c;
  } else {
    const long off = (long)L.b * g.field + 2 * L.lc + L.c;
    f = (R *)(L.role == 0 ? bf.vor : bf.phi) + off;
    scr = (R *)(L.role == 0 ? bf.S : bf.T) + off;
    if (fabs(g.s) > 0.01) {
      const double a = g.alp * L.i;
      const double xt = M.xwt[rk == 0 ? 0 : rk - 1];
      sincos((-a) * xt, &shp.y, &shp.x);
    }
  }
  const cd shm = cj(shp);  // matvecNcyclic takes shm = conj(shp)
  {
    // u(N-3..N) shm and u(1..4) shp, this lane's component
    double lo[4], hi[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const double a = (double)f[(long)(N - 4 + q) * ps];
      const double b = (double)f[(long)q * ps];
      lo[q] = cmul_c(a, __shfl_xor_sync(0xffffffffu, a, 1), shm, L.c);
      hi[q] = cmul_c(b, __shfl_xor_sync(0xffffffffu, b, 1), shp, L.c);
    }
    if (L.mean) {  // two real lines, no phase
#pragma unroll
      for (int q = 0; q < 4; q++) {
        lo[q] = (double)f[(long)(N - 4 + q) * ps];
        hi[q] = (double)f[(long)q * ps];
      }
    }
    for (int i = L.r0; i <= L.r1; i++) {
      double s = 0.0;
#pragma unroll
      for (int d = -4; d <= 4; d++) {
        const int r = i + d;
        const double x = (r < 1) ? lo[r + 3] : (r > N ? hi[r - N - 1] : (double)f[(long)(r - 1) * ps]);
        s += g.frh[d < 0 ? -d : d] * x;
      }
      if (L.active) scr[(long)(i - 1) * ps] = (R)s;
    }
  }
  __syncthreads();  // the right-hand side of all segments is read below
  const TailMake TF{VF, shp, N};
  SEG_SOLVE(scr, ps, VF, WF, TF, shp, shm, 1.0, 0.0, 0.0, 0.0, false);
  store_col(ys, ystr, f, ps, L);
  if (!L.mean) return;
  __syncthreads();  // the filtered profiles of all segments are read below
  const FacView V1(bf.d1, 0);
  const SegView W1(bf.d1, 0);
  const cd one = mk(1.0, 0.0);
  const TailLoad T1{bf.tl1o + (long)L.b * g.nkx * SB_TAIL};
  SEG_SOLVE(f, 2, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
  if (L.active)
    for (int i = L.r0; i <= L.r1; i++) scr[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
}

// d/dy of the mean profiles u00, w00 (derivyc with m = 1, as hvhg computes
// them, cross.f90:1186-1192) after the y dealiasing changed them: one block
// per box (the mean-line slot of line_thread with a single role-less group)
template <typename R>
__global__ void __launch_bounds__(32 * kSeg) k_meand1(Grid g, Bufs bf) {
  __shared__ double xch[kSeg][16][2][SB_XS];
  const int b = blockIdx.x;
  if (bf.mem[b].halted) return;
  LineThread L;
  const int lane = threadIdx.x & 31;
  L.b = b;
  L.role = 0;
  L.mean = true;
  L.s = threadIdx.x >> 5;
  L.l = lane >> 1;
  L.c = lane & 1;
  L.lc = 0;
  L.active = (L.l == 0);
  L.i = 0;
  L.k = 0;
  L.r0 = g.slo[L.s];
  L.r1 = (L.s == kSeg - 1) ? g.my : g.shi[L.s];
  const int N = g.my, ystr = blockDim.x;
  double *ys = ycol();
  const FacView V1(bf.d1, 0);
  const SegView W1(bf.d1, 0);
  const R *mu = (const R *)bf.mu + (long)b * 2 * N + L.c;
  R *mdu = (R *)bf.mdu + (long)b * 2 * N + L.c;
  const cd one = mk(1.0, 0.0);
  const TailLoad T1{bf.tl1o + (long)b * g.nkx * SB_TAIL};
  SEG_SOLVE(mu, 2, V1, W1, T1, one, one, 0.0, g.rh1[4], g.rh1[5], g.rh1[6], true);
  if (L.active)
    for (int i = L.r0; i <= L.r1; i++) mdu[2 * (i - 1)] = (R)ys[(i - L.r0) * ystr];
}



// ---------------------------------------------------------------------------
static const int kLineT = 32 * kSeg;

// shared-memory bytes of the line kernels: one column per thread of the
// longest segment and four rows of the extended line beyond it
static size_t smem_of(const Grid &g) {
  int rows = 0;
  for (int s = 0; s < g.nseg; s++) {
    const int r1 = (s == g.nseg - 1) ? g.my : g.shi[s];
    rows = rows > r1 - g.slo[s] + 1 ? rows : r1 - g.slo[s] + 1;
  }
  return sizeof(double) * kLineT * (rows + 4);
}

// the exported launchers of this compilation (sb::seg<K>::name_f64/_f32)
size_t SB_PSUF(line_smem)(const Grid &g) { return smem_of(g); }

// a block of np pipelines (k_lineF, k_lineI: np times the threads and
// columns of the split kernels, np exchange areas) fits the device's shared
// memory per block
bool SB_PSUF(lineI_fits)(const Grid &g, int np) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;
  const size_t xs = sizeof(double) * np * kSeg * 16 * 2 * SB_XS;
  return np * smem_of(g) + xs <= (size_t)optin;
}
bool SB_PSUF(lineF_fits)(const Grid &g) { return SB_PSUF(lineI_fits)(g, 2); }

cudaError_t SB_PSUF(prepare_line)(const Grid &g) {
  typedef SbR R;
  const int sm = (int)smem_of(g);
  cudaFuncSetAttribute(k_lineA<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  cudaFuncSetAttribute(k_lineB<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  cudaFuncSetAttribute(k_lineA<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  cudaFuncSetAttribute(k_lineB<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  cudaFuncSetAttribute(k_lineL<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  cudaFuncSetAttribute(k_filter<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  cudaFuncSetAttribute(k_meand1<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (SB_PSUF(lineF_fits)(g)) {
    cudaFuncSetAttribute(k_lineF<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * sm);
    cudaFuncSetAttribute(k_lineI<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * sm);
  }
  if (SB_PSUF(lineI_fits)(g, 3))
    cudaFuncSetAttribute(k_lineI<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * sm);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(lineA)(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  typedef SbR R;
  const unsigned nb = (unsigned)(g.B * (3 * g.ngrp + 1));
  if (g.temp)
    k_lineA<R, true><<<nb, kLineT, smem_of(g), st>>>(g, bf, rk);
  else
    k_lineA<R, false><<<nb, kLineT, smem_of(g), st>>>(g, bf, rk);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(lineB)(const Grid &g, const Bufs &bf, int mode, cudaStream_t st) {
  typedef SbR R;
  const unsigned nb = (unsigned)(g.B * ((g.temp ? 3 : 2) * g.ngrp + 1));
  if (g.temp)
    k_lineB<R, true><<<nb, kLineT, smem_of(g), st>>>(g, bf, mode);
  else
    k_lineB<R, false><<<nb, kLineT, smem_of(g), st>>>(g, bf, mode);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(lineF)(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  typedef SbR R;
  const unsigned nb = (unsigned)(g.B * (g.ngrp + 1));
  k_lineF<R><<<nb, 2 * kLineT, 2 * smem_of(g), st>>>(g, bf, rk);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(lineI)(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  typedef SbR R;
  const unsigned nb = (unsigned)(g.B * (g.ngrp + 1));
  if (g.temp)
    k_lineI<R, true><<<nb, 3 * kLineT, 3 * smem_of(g), st>>>(g, bf, rk);
  else
    k_lineI<R, false><<<nb, 2 * kLineT, 2 * smem_of(g), st>>>(g, bf, rk);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(lineL)(const Grid &g, const Bufs &bf, cudaStream_t st) {
  k_lineL<SbR><<<(unsigned)(g.B * (2 * g.ngrp + 1)), kLineT, smem_of(g), st>>>(g, bf);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(meand1)(const Grid &g, const Bufs &bf, cudaStream_t st) {
  k_meand1<SbR><<<g.B, kLineT, smem_of(g), st>>>(g, bf);
  return cudaGetLastError();
}

cudaError_t SB_PSUF(filter)(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  k_filter<SbR><<<(unsigned)(g.B * (2 * g.ngrp + 1)), kLineT, smem_of(g), st>>>(g, bf, rk);
  return cudaGetLastError();
}

}  // namespace SB_SEGNS
}  // namespace sb
