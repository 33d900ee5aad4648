// sb_box.cu -- per-box kernels of the RK3 step and the dispatch of the
// y-line kernels.
//
//   k_setconj set_conj on the state at the entry of a cross call
//             (operators.f90:1382-1429)
//   k_hsum    plane sums of the hist partials of a statistics step
//   k_scalar  per box: Delta t from the CFL (cross.f90:1598-1711), the UNER
//             record (cross.f90:2064-2118), image offsets (cross.f90:726-746)
//   k_tables  shear phases exp(-i kx xoff), the shear tails of the d/dy and
//             d2/dy2 factorisations per kx (modChol_addshear,
//             diffy_shear_hepta.f90:760-870) and the moving_frame phases
//             (operators.f90:86-145)
//   k_finish  end of a step (cross.f90:1002-1013) and the stop check
//             (cross.f90:356)
// The y-line kernels (sb_yline.cu) exist for 1, 2 and 3 warps per line
// solve; the launchers here pick the compilation that matches the handle's
// segment plan (Grid::nseg).
#include <cuda_runtime.h>

#include "sb_common.cuh"
#include "sb_kernels.h"
#include "sb_line.cuh"

namespace sb {

__device__ __forceinline__ cd ldc2(const double *p) { return mk(p[0], p[1]); }

// set_conj on the state (operators.f90:1382-1429) at entry of a cross call
template <typename R>
__global__ void k_setconj(Grid g, Bufs bf) {
  const int nneg = g.mz - 1 - g.nz;
  const long n = (long)g.B * g.my * nneg * 2;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t & 1);
    const long r = t >> 1;
    const int kk = (int)(r % nneg);
    const int j = (int)((r / nneg) % g.my);
    const int b = (int)(r / ((long)nneg * g.my));
    const int k = g.nz + 1 + kk;
    const long base = (long)b * g.field + (long)j * g.plane;
    const long dst = base + 2L * k * g.nkx + c, src = base + 2L * (g.mz - k) * g.nkx + c;
    R *vor = (R *)bf.vor, *phi = (R *)bf.phi;
    const R v = vor[src], p = phi[src];
    vor[dst] = c ? -v : v;
    phi[dst] = c ? -p : p;
    if (g.temp) {  // set_conj_t (crosst.f90:333-337)
      R *tb = (R *)bf.tb;
      const R t = tb[src];
      tb[dst] = c ? -t : t;
    }
  }
}

// ---------------------------------------------------------------------------
// plane sums of the hist partials of plane stages 1 and 2 and of the LES
// stage at the first substep of a statistics step: one warp per (box, plane),
// lanes over the partials, a fixed reduction tree
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) k_hsum(Grid g, Bufs bf) {
  const int j = blockIdx.x, b = blockIdx.y;
  const Member &M = bf.mem[b];
  if (M.halted || !M.ihist) return;
  // one partial per block of k_spectra (16 modes each)
  const int nparts = (g.nkx * g.mz + 15) / 16;
  const int nzp = g.mgalz / 2;
  const int lane = threadIdx.x;
  constexpr int NS = SB_NHIST_Q + 5;
  double v[NS];
#pragma unroll
  for (int q = 0; q < NS; q++) v[q] = 0.0;
  const double *hp = bf.hpart + ((long)b * g.my + j) * nparts * SB_NHIST_Q;
  for (int pp = lane; pp < nparts; pp += 32)
#pragma unroll
    for (int q = 0; q < SB_NHIST_Q; q++) v[q] += hp[pp * SB_NHIST_Q + q];
  // plane stage 2 leaves one triple per (row pair, warp of its block)
  const int np2 = nzp * (g.t2 / 32);
  const double *ph = bf.ppart + ((long)b * g.my + j) * np2 * 3;
  for (int z = lane; z < np2; z += 32)
#pragma unroll
    for (int q = 0; q < 3; q++) v[SB_NHIST_Q + q] += ph[3 * z + q];
  if (g.les) {
    const double *lp = bf.lpart + ((long)b * g.my + j) * nzp * 2;
    for (int z = lane; z < nzp; z += 32) {
      v[SB_NHIST_Q + 3] += lp[2 * z];
      v[SB_NHIST_Q + 4] += lp[2 * z + 1];
    }
  }
  double mine = 0.0;
#pragma unroll
  for (int q = 0; q < NS; q++) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == q) mine = x;
  }
  if (lane < NS) bf.hsum[((long)b * g.my + j) * NS + lane] = mine;
}

// ---------------------------------------------------------------------------
// per-box scalars: entry flags, hist reduction and UNER record, Delta t,
// image offsets.  One block per box.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_scalar(Grid g, Bufs bf, int rk) {
  const int b = blockIdx.x;
  Member &M = bf.mem[b];
  // per-plane sums: SB_NHIST_Q hist partials, Pk, and with LES nu_t and nu_t |S|^2
  constexpr int NQ = SB_NHIST_Q + 3;
  __shared__ double s_q[NQ];
  __shared__ double s_part[NQ][256 / 32];
  __shared__ int s_halt;
  if (threadIdx.x == 0) {
    if (rk == 0) {  // entry of a cross() call (cross.f90:76-113)
      M.istop = 0;
      M.idump = 0;
      M.halted = 0;
      M.istep = 1;
      M.ihist = 1;
      M.ntrace = 0;
      M.flags = 0;
      for (int q = 0; q < 4; q++) M.umax_bits[q] = 0ull;
      M.nut_bits = 0ull;
      M.tbmax_bits = 0ull;
      M.nacum = 0;
      M.total_dt = 0.0;
      M.xwb[0] = M.xoffb;
      M.xwt[0] = M.xofft;
    }
    s_halt = M.halted;
  }
  if (rk == 0) {
    // the statistics of a call start from zero (cross.f90:139-155)
    const long nst = (long)g.my * 23, nsp = (long)g.nkx * g.mz * 8;
    for (long q = threadIdx.x; q < nst; q += blockDim.x) {
      bf.stats[b * nst + q] = 0.0;
      bf.stats2[b * nst + q] = 0.0;
    }
    for (long q = threadIdx.x; q < nsp; q += blockDim.x) {
      bf.spec[b * nsp + q] = 0.0;
      bf.spec2[b * nsp + q] = 0.0;
    }
    if (g.temp) {
      for (long q = threadIdx.x; q < (long)g.my * 5; q += blockDim.x) bf.tstats[b * g.my * 5L + q] = 0.0;
      for (long q = threadIdx.x; q < nsp / 2; q += blockDim.x) bf.tspec[b * (nsp / 2) + q] = 0.0;
    }
  }
  __syncthreads();
  if (s_halt || rk == 0) return;
  const bool shear = fabs(g.s) > 0.01;
  const bool hist = (rk == 1) && M.ihist;
  if (hist) {
    // hist 'w': sum over planes of the per-block partials (cross.f90:2070-2080)
    // and the production Pk, whose mean omega_z includes -s (cross.f90:1901-1912)
    const int nq = NQ;
    double acc[NQ];
    for (int q = 0; q < nq; q++) acc[q] = 0.0;
    const double nufac = g.les_visc ? (1.0 / M.Re) : 0.0;
    const double nxz = (double)(g.mgalx * g.mgalz);
    for (int j = threadIdx.x; j < g.my; j += blockDim.x) {
      const double *hs = bf.hsum + ((long)b * g.my + j) * (SB_NHIST_Q + 5);
      double pl[SB_NHIST_Q];
      for (int q = 0; q < SB_NHIST_Q; q++) pl[q] = hs[q];
      for (int q = 0; q < SB_NHIST_Q; q++) acc[q] += pl[q];
      const long mj = 2 * ((long)b * g.my + j);
      auto rdm = [&](const double *p, int c) -> double {
        return g.prec ? (double)((const float *)p)[mj + c] : p[mj + c];
      };
      const double du = rdm(bf.mdu, 0);
      const double o3 = -du - g.s;
      double Pk, nuty = 0.0, disp = 0.0;
      if (g.les) {
        // Pk with the resolved mean stress (cross.f90:1886-1899), nu_t and the
        // energy transfer to the subgrid scales (cross.f90:1892,1950-1952)
        const double txy = rdm(bf.txy, 0);
        Pk = -(o3 * (-pl[3] + txy)) + nufac * (o3 * o3);
        nuty = hs[SB_NHIST_Q + 3] / nxz;
        disp = hs[SB_NHIST_Q + 4] / nxz;
        acc[SB_NHIST_Q + 1] += nuty;
        acc[SB_NHIST_Q + 2] += disp;
      } else {
        Pk = -o3 * (-pl[3]) + (o3 * o3) * (1.0 / M.Re);
      }
      acc[SB_NHIST_Q] += Pk;
      // the plane's statistics (hist 'f', 'p': cross.f90:1830-1955, 2038-2048)
      // with the Delta t of the previous step
      double v[23];
      v[0] = rdm(bf.mu, 0);
      v[1] = M.vbulk;
      v[2] = rdm(bf.mu, 1);
      for (int q = 0; q < 6; q++) v[3 + q] = pl[q];
      v[9] = rdm(bf.mdu, 1);
      v[10] = g.prec ? (double)((const float *)bf.vor)[b * g.field + j * g.plane]
                     : bf.vor[b * g.field + j * g.plane];
      v[11] = -du;
      for (int q = 0; q < 3; q++) v[12 + q] = pl[6 + q];
      v[15] = pl[10];
      v[16] = hs[SB_NHIST_Q];
      v[17] = hs[SB_NHIST_Q + 1];
      v[18] = hs[SB_NHIST_Q + 2];
      v[19] = Pk;
      v[20] = pl[9];
      v[21] = nuty;
      v[22] = disp;
      const double dto = M.Deltat;
      double *st = bf.stats + ((long)b * g.my + j) * 23, *st2 = bf.stats2 + ((long)b * g.my + j) * 23;
      for (int q = 0; q < 23; q++) {
        st[q] += v[q];
        st2[q] += v[q] * dto;
      }
      if (g.temp) {
        // tstats (crosst.f90:2201-2205)
        double *ts = bf.tstats + ((long)b * g.my + j) * 5;
        ts[0] += rdm(bf.mt, 0) * dto;
        for (int q = 0; q < 4; q++) ts[1 + q] += pl[11 + q] * dto;
      }
    }
    for (int q = 0; q < nq; q++) {
      double v = acc[q];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if ((threadIdx.x & 31) == 0) s_part[q][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < nq) {
      double v = 0.0;
      for (int w = 0; w < (int)(blockDim.x / 32); w++) v += s_part[threadIdx.x][w];
      s_q[threadIdx.x] = v;
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  if (rk == 1) {
    // umax (cross.f90:1205-1216,1436-1442) and Delta t (cross.f90:1598-1711)
    double uinit = 0.0;
    if (M.istep == 1 && M.readflag == 0) uinit = (fabs(g.s) > 0.5) ? 1.0 : M.uprim;
    for (int q = 0; q < 4; q++) {
      const double v = __longlong_as_double((long long)M.umax_bits[q]);
      M.umax[q] = v > uinit ? v : uinit;
    }
    // max |tb| of the step (crosst.f90:1443-1445,1674-1676,1864-1867)
    if (g.temp) M.tbmax = __longlong_as_double((long long)M.tbmax_bits);
    if (g.les) {
      // running maximum of |nu_t| (cross.f90:1430-1436, 1604)
      const double v = __longlong_as_double((long long)M.nut_bits);
      if (v > M.max_nut) M.max_nut = v;
    }
    const double nutmax = M.max_nut;
    const double vv = fmax(fmax(g.pi * g.pi / g.dx / g.dx, 6.25 / g.dy / g.dy), g.pi * g.pi / g.dz / g.dz);
    double dt;
    if (M.fixed_dt > 0.0) {
      dt = M.fixed_dt;
      const double m = fmax(fmax(M.umax[0] * g.pi / g.dx, M.umax[2] * 2.5 / g.dy), M.umax[3] * g.pi / g.dz);
      M.CFLcur = dt * m;
      if (g.les) {
        // cross.f90:1620-1635
        const double vn = 2.0 * nutmax * dt * vv;
        M.CFLv = g.les_visc ? fmax(fabs(1.0 / M.Re) * dt * vv, vn) : vn;
      } else {
        M.CFLv = (1.0 / M.Re) * dt * vv;
      }
    } else {
      const double m = fmax(fmax(M.umax[0] * M.cflx, M.umax[2] * M.cfly), M.umax[3] * M.cflz);
      dt = 1.0 / m;
      if (g.les) {
        // cross.f90:1652-1666
        const double vn = nutmax / M.CFL * vv;
        M.cflvv = g.les_visc ? fmax(fabs(1.0 / M.Re) / M.CFL * vv, vn) : vn;
      }
      M.CFLcur = M.CFL;
      M.CFLv = M.CFL * M.cflvv * dt;
      if (g.temp) {
        // the thermal-diffusion limit enters only where the viscous one
        // does (crosst.f90:1929-1968): explicit, within both limits;
        // semi-implicit, at most 6/CFL times them once CFLv exceeds 2
        const double CFLk = M.CFL * M.cflkk * dt;
        if (!g.impl) {
          if (M.CFLv > M.CFL) dt = (CFLk > M.CFLv) ? 1.0 / M.cflkk : 1.0 / M.cflvv;
        } else if (M.CFLv > 2.0) {
          dt = (CFLk > M.CFLv) ? 1.0 / M.cflkk / M.CFL * 6.0 : 1.0 / M.cflvv / M.CFL * 6.0;
        }
      } else if (M.CFLv > M.CFL && !g.impl) {
        // the viscous limit of the explicit branch only (cross.f90:1669)
        dt = 1.0 / M.cflvv;
      }
    }
    double Deltat = dt;
    if (Deltat < 1e-10) {
      M.istop = 1;
      M.flags |= SBF_DIVERGED;
    }
    if ((M.time + Deltat) > M.dumptime) {
      Deltat = fabs(M.dumptime - M.time);
      if (M.dumptime > (M.etime - 1e-13)) {
        M.istop = 1;
        M.flags |= SBF_ETIME;
      }
      M.dumptime = M.dumptime + M.dtimag;
      M.idump = 1;
    } else if ((M.time + Deltat) > M.etime) {
      Deltat = fabs(M.etime - M.time);
      M.istop = 1;
      M.flags |= SBF_ETIME;
    }
    M.Deltat = Deltat;
    if (hist) {
      double uner[10], uner2[4];
      const double my = (double)g.my;
      for (int q = 0; q < 3; q++) uner[q] = sqrt(fabs(s_q[q] / my));
      for (int q = 3; q < 6; q++) uner[q] = s_q[q] / my;
      for (int q = 6; q < 9; q++) uner[q] = sqrt(fabs(s_q[q] / my));
      uner[9] = s_q[10] / my;
      uner2[0] = s_q[SB_NHIST_Q] / my;
      uner2[1] = s_q[9] / my;
      uner2[2] = g.les ? s_q[SB_NHIST_Q + 1] / my : 0.0;
      uner2[3] = g.les ? s_q[SB_NHIST_Q + 2] / my : 0.0;
      if (M.ntrace < M.trace_cap) {
        double *rec = bf.trace + ((long)b * M.trace_cap + M.ntrace) * g.tlen;
        rec[0] = M.time;
        rec[1] = M.Deltat;
        for (int q = 0; q < 10; q++) rec[2 + q] = uner[q];
        rec[12] = M.CFLcur;
        rec[13] = M.CFLv;
        rec[14] = M.umax[1];
        rec[15] = M.umax[2];
        rec[16] = M.umax[3];
        rec[17] = M.xoffb;
        rec[18] = M.xofft;
        rec[19] = M.umax[0];
        for (int q = 0; q < 4; q++) rec[20 + q] = uner2[q];
        if (g.temp) {
          // tbmax, tner(1:4) of histt 'w' (crosst.f90:2446-2458)
          rec[24] = M.tbmax;
          rec[25] = sqrt(fabs(s_q[11] / my));
          for (int q = 1; q < 4; q++) rec[25 + q] = s_q[11 + q] / my;
        }
      }
      M.ntrace++;
      // counts of the accumulated statistics (cross.f90:2070-2072)
      M.nacum++;
      M.total_dt += M.Deltat;
      if (isnan(uner[0])) {
        M.istop = 1;
        M.flags |= SBF_NAN;
      }
      if (uner[1] / (2.0 * g.pi / g.gam) < 1e-5) {
        if (!M.keep_laminar) M.istop = 1;
        M.flags |= SBF_LAMINAR;
      }
      M.ihist = 0;
    }
  }
  // image offsets after this substep (cross.f90:728-731)
  const double r1 = kCa[rk - 1] * M.Deltat;
  if (shear) {
    M.xwb[rk] = M.xoffb + r1 * (g.s * (-g.Ly));
    M.xwt[rk] = M.xofft + r1 * (g.s * g.Ly);
    if (g.ydeal == 2) {  // cross.f90:733-736
      M.xwb[rk] = (M.xwb[rk] / g.Lx - trunc(M.xwb[rk] / g.Lx)) * g.Lx;
      M.xwt[rk] = -M.xwb[rk];
    }
  } else {
    M.xwb[rk] = M.xwb[rk - 1];
    M.xwt[rk] = M.xwt[rk - 1];
  }
}

// ---------------------------------------------------------------------------
// per-box tables of substep rk (0: prologue): shear phases at the offsets
// before (old) and after (new) the substep, shear tails of the uniform
// operators, moving_frame phases.  Grid (blocks, B).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_tables(Grid g, Bufs bf, int rk) {
  const int b = blockIdx.y;
  const Member &M = bf.mem[b];
  if (M.halted) return;
  const int nkx = g.nkx, my = g.my;
  const bool shear = fabs(g.s) > 0.01;
  const int ro = (rk == 0) ? 0 : rk - 1;
  const double xob = M.xwb[ro], xot = M.xwt[ro];
  const double xnb = M.xwb[rk], xnt = M.xwt[rk];
  const double Dt = M.Deltat;
  const long ntail = (rk == 0) ? 2L * nkx : 4L * nkx;
  const long nmf = (rk == 0) ? 0 : (long)my * nkx;
  const long n = ntail + nmf;
  const FacView V1(bf.d1, 0), V2(bf.d2, 0);
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    if (q < ntail) {
      // which: 0 d/dy old phase, 1 d2/dy2 old, 2 d/dy new, 3 d2/dy2 new
      const int which = (int)(q / nkx), i = (int)(q - (long)which * nkx);
      const double a = g.alp * i;
      const bool nw = (which >= 2);
      const double xt = nw ? xnt : xot, xb = nw ? xnb : xob;
      cd shp = mk(1.0, 0.0), shm = mk(1.0, 0.0);
      if (shear) {
        sincos((-a) * xt, &shp.y, &shp.x);
        sincos((-a) * xb, &shm.y, &shm.x);
      }
      // the phase tables themselves (written once per kx)
      double *sh = (nw ? bf.sh_new : bf.sh_old) + (long)b * 4 * nkx;
      if (which == 0 || which == 2) {
        sh[2 * i] = shp.x;
        sh[2 * i + 1] = shp.y;
        sh[2 * (nkx + i)] = shm.x;
        sh[2 * (nkx + i) + 1] = shm.y;
      }
      const Tail T = make_tail((which & 1) ? V2 : V1, shp, my);
      double *const tl[4] = {bf.tl1o, bf.tl2o, bf.tl1n, bf.tl2n};
      double *dst = tl[which] + ((long)b * nkx + i) * SB_TAIL;
      store_tail(dst, T);
    } else {
      // moving_frame phases exp(i kx y_j tau) (operators.f90:119-123)
      const long p = q - ntail;
      const int jj = (int)(p / nkx), i = (int)(p - (long)jj * nkx);
      const double f1 = (rk == 1) ? -(kGama[0] * Dt * g.s) : -((kGama[1] + kZeta[0]) * Dt * g.s);
      const double f2 = (rk == 1) ? -(g.s * (kCa[0] * Dt)) : -(g.s * (kCa[rk - 1] - kCa[rk - 2]) * Dt);
      const double ay = (g.alp * i) * ((double)jj * g.dy - 0.5 * g.Ly);
      double sn, cs;
      double *m1 = bf.mf1 + (long)b * 2 * my * nkx;
      double *m2 = bf.mf2 + (long)b * 2 * my * nkx;
      if (rk < 3) {
        sincos(ay * f1, &sn, &cs);
        m1[2 * p] = cs;
        m1[2 * p + 1] = sn;
      }
      sincos(ay * f2, &sn, &cs);
      m2[2 * p] = cs;
      m2[2 * p + 1] = sn;
    }
  }
}

// end of a step: offsets, time, next-step flags (cross.f90:1002-1013, 336-376)
__global__ void k_finish(Grid g, Bufs bf) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.B) return;
  Member &M = bf.mem[b];
  if (M.halted) return;
  M.xoffb = M.xwb[3];
  M.xofft = M.xwt[3];
  M.xwb[0] = M.xoffb;
  M.xwt[0] = M.xofft;
  M.time = M.time + M.Deltat;
  M.istep += 1;
  // cross checks the stop flag from its third step on (cross.f90:221),
  // crosst from its second (crosst.f90:259)
  if ((g.temp || (M.istep - 1) != 1) && M.istop) M.halted = 1;
  if ((M.istep - 1) % M.nhist == 0) M.ihist = 1;
  for (int q = 0; q < 4; q++) M.umax_bits[q] = 0ull;
  M.nut_bits = 0ull;
  M.tbmax_bits = 0ull;
}


template <typename R>
static cudaError_t setconj_t(const Grid &g, const Bufs &bf, cudaStream_t st) {
  k_setconj<R><<<64, 256, 0, st>>>(g, bf);
  return cudaGetLastError();
}

cudaError_t launch_setconj(const Grid &g, const Bufs &bf, cudaStream_t st) {
  return g.prec ? setconj_t<float>(g, bf, st) : setconj_t<double>(g, bf, st);
}

cudaError_t launch_scalar(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  if (rk == 1) {
    // the plane sums of a statistics step (the kernel returns at once otherwise)
    k_hsum<<<dim3((unsigned)g.my, (unsigned)g.B), 32, 0, st>>>(g, bf);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_scalar<<<g.B, 256, 0, st>>>(g, bf, rk);
  return cudaGetLastError();
}

cudaError_t launch_tables(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  const long n = 4L * g.nkx + (long)g.my * g.nkx;
  const int T = 128;
  dim3 grid((unsigned)((n + T - 1) / T), g.B);
  k_tables<<<grid, T, 0, st>>>(g, bf, rk);
  return cudaGetLastError();
}

cudaError_t launch_finish(const Grid &g, const Bufs &bf, cudaStream_t st) {
  k_finish<<<(g.B + 127) / 128, 128, 0, st>>>(g, bf);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// y-line kernels: one compilation of sb_yline.cu per segment count
// ---------------------------------------------------------------------------
#define SB_DECLARE_SEG(K)                                                                  \
  namespace seg##K {                                                                       \
  size_t line_smem_f64(const Grid &g);                                                     \
  cudaError_t prepare_line_f64(const Grid &g);                                             \
  cudaError_t prepare_line_f32(const Grid &g);                                             \
  cudaError_t lineA_f64(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);           \
  cudaError_t lineA_f32(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);           \
  cudaError_t lineB_f64(const Grid &g, const Bufs &bf, int mode, cudaStream_t st);         \
  cudaError_t lineB_f32(const Grid &g, const Bufs &bf, int mode, cudaStream_t st);         \
  cudaError_t lineF_f64(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);           \
  cudaError_t lineF_f32(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);           \
  bool lineF_fits_f64(const Grid &g);                                                      \
  bool lineI_fits_f64(const Grid &g, int np);                                              \
  bool lineI_fits_f32(const Grid &g, int np);                                              \
  cudaError_t lineI_f64(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);           \
  cudaError_t lineI_f32(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);           \
  bool lineF_fits_f32(const Grid &g);                                                      \
  cudaError_t lineL_f64(const Grid &g, const Bufs &bf, cudaStream_t st);                   \
  cudaError_t lineL_f32(const Grid &g, const Bufs &bf, cudaStream_t st);                   \
  cudaError_t meand1_f64(const Grid &g, const Bufs &bf, cudaStream_t st);                  \
  cudaError_t meand1_f32(const Grid &g, const Bufs &bf, cudaStream_t st);                  \
  cudaError_t filter_f64(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);          \
  cudaError_t filter_f32(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);          \
  }
SB_DECLARE_SEG(1)
SB_DECLARE_SEG(2)
SB_DECLARE_SEG(3)

#define SB_SEG_CALL(name, ...)                                                             \
  switch (g.nseg) {                                                                        \
    case 1: return g.prec ? seg1::name##_f32(__VA_ARGS__) : seg1::name##_f64(__VA_ARGS__); \
    case 3: return g.prec ? seg3::name##_f32(__VA_ARGS__) : seg3::name##_f64(__VA_ARGS__); \
    default: return g.prec ? seg2::name##_f32(__VA_ARGS__) : seg2::name##_f64(__VA_ARGS__); \
  }

int line_segments() { return 2; }
bool line_segments_supported(int nseg) { return nseg >= 1 && nseg <= 3; }

size_t line_smem(const Grid &g) {
  switch (g.nseg) {
    case 1: return seg1::line_smem_f64(g);
    case 3: return seg3::line_smem_f64(g);
    default: return seg2::line_smem_f64(g);
  }
}

cudaError_t prepare_line(const Grid &g) {
  cudaError_t e;
  switch (g.nseg) {
    case 1: e = seg1::prepare_line_f64(g); return e != cudaSuccess ? e : seg1::prepare_line_f32(g);
    case 3: e = seg3::prepare_line_f64(g); return e != cudaSuccess ? e : seg3::prepare_line_f32(g);
    default: e = seg2::prepare_line_f64(g); return e != cudaSuccess ? e : seg2::prepare_line_f32(g);
  }
}

cudaError_t launch_lineA(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  SB_SEG_CALL(lineA, g, bf, rk, st)
}
cudaError_t launch_lineB(const Grid &g, const Bufs &bf, int mode, cudaStream_t st) {
  SB_SEG_CALL(lineB, g, bf, mode, st)
}
cudaError_t launch_lineF(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  SB_SEG_CALL(lineF, g, bf, rk, st)
}
// the fused y-line kernel covers the plain step: no temperature, no y filter
// or y dealiasing, and its block's shared memory fits
bool line_fused_ok(const Grid &g) {
  if (g.temp || g.ydeal || g.impl) return false;
  SB_SEG_CALL(lineF_fits, g)
}
cudaError_t launch_lineI(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  SB_SEG_CALL(lineI, g, bf, rk, st)
}
// k_lineI has k_lineF's block (two pipelines, three with the temperature)
bool line_implicit_ok(const Grid &g) { SB_SEG_CALL(lineI_fits, g, g.temp ? 3 : 2) }
cudaError_t launch_lineL(const Grid &g, const Bufs &bf, cudaStream_t st) {
  SB_SEG_CALL(lineL, g, bf, st)
}
cudaError_t launch_meand1(const Grid &g, const Bufs &bf, cudaStream_t st) {
  SB_SEG_CALL(meand1, g, bf, st)
}
cudaError_t launch_filter(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  SB_SEG_CALL(filter, g, bf, rk, st)
}

}  // namespace sb
