// sb_kernels.cu -- FP64 kernels of the shearing-box RK3 substep on sm_103a.
//
// One RK3 substep of the reference (cross.f90:428-1000, explicit branch,
// iadd_mode=5) is five launches:
//   k_spectra  (first substep of a statistics step, beside stages 1-2) hist
//           plane sums and kx-kz spectra (cross.f90:1796-2014)
//   k_p1    per (plane, kx block): u, w, omega_x, omega_z from v, omega_y
//           (cross.f90:1226-1276) and the six backward z-transforms with zero
//           padding (fill00, fou3D_thread.f:73-126)
//   k_p2    per (plane, z row pair): backward x-transforms, |u| maxima for the CFL
//           (cross.f90:1438-1441), u x (omega + 2 chi z) (cross.f90:1453-1462) and
//           the three forward x-transforms
//   k_p3    per (plane, kx block): forward z-transforms, 1/(mgalx*mgalz) scaling and
//           truncation (pack00), right-hand sides of iadd_mode 5
//           (cross.f90:1536-1546) and the mean-mode forcing (cross.f90:1489-1490)
//   k_phase per box: Delta t from the CFL (cross.f90:1598-1711), the UNER record
//           (cross.f90:2064-2118), shear offsets and phase tables
//   k_line  per (kx, kz) y-line: every y-operator of the substep in one pass --
//           derivyc of d(omega_y)/dy, the viscous terms (visc3d), the RK3 update
//           (cross.f90:694-723), the zeta store and moving_frame remaps
//           (cross.f90:752-781), the Helmholtz solve for v (lapcdy, cross.f90:784-795)
//           and the derivatives the next substep starts from (cross.f90:434-445).
// The per-plane/per-line split replaces the reference's plane<->pencil MPI
// transposes (change.allfac_ieor.f): every kernel reads the same plane-major
// layout, so no data is reordered.
#include <cuda_runtime.h>

#include "sb_common.cuh"
#include "sb_fft.cuh"
#include "sb_kernels.h"
#include "sb_line.cuh"

// This file is compiled twice: SB_FLOAT_TU=0 gives the FP64 instantiations
// and the shared entry points, SB_FLOAT_TU=1 only the FP32-mixed
// instantiations, so that the two halves compile in parallel.
#ifndef SB_FLOAT_TU
#define SB_FLOAT_TU 0
#endif

namespace sb {

__device__ __forceinline__ cd ldc(const double *p) { return mk(p[0], p[1]); }

// ---------------------------------------------------------------------------
// storage/arithmetic types: R = double (FP64 path) or float (FP32-mixed path)
// ---------------------------------------------------------------------------
template <typename R> struct Vec2;
template <> struct Vec2<double> { typedef double2 t; };
template <> struct Vec2<float> { typedef float2 t; };
template <typename R>
__device__ __forceinline__ typename Vec2<R>::t mk2(R a, R b) {
  typename Vec2<R>::t v;
  v.x = a;
  v.y = b;
  return v;
}
template <typename R> __device__ __forceinline__ const R *tw_of(const Bufs &bf, bool z);
template <> __device__ __forceinline__ const double *tw_of<double>(const Bufs &bf, bool z) {
  return z ? bf.twz : bf.twx;
}
template <> __device__ __forceinline__ const float *tw_of<float>(const Bufs &bf, bool z) {
  return z ? bf.twzf : bf.twxf;
}
template <typename R> __device__ __forceinline__ R kinv_of(const Bufs &bf, long q);
template <> __device__ __forceinline__ double kinv_of<double>(const Bufs &bf, long q) { return bf.kinv[q]; }
template <> __device__ __forceinline__ float kinv_of<float>(const Bufs &bf, long q) { return bf.kinvf[q]; }

// ---------------------------------------------------------------------------
// plane stage 1: reconstruction + backward z-transforms
// ---------------------------------------------------------------------------
// k index -> position on the padded z grid (fill00)
__device__ __forceinline__ int kgrid(int k, int nz, int NZ, int mz) { return k <= nz ? k : k + (NZ - mz); }

// TEMP: with the temperature round and statistics (a separate instantiation,
// so that the plain step keeps its register budget)
template <typename R, int NZ, int CB, int T, bool TEMP>
__global__ void __launch_bounds__(T) k_p1(Grid g, Bufs bf, int rk) {
  typedef typename Vec2<R>::t V;
  // one block per (kx block, pair of fields): the three (five with LES) pairs
  // of a column block run as separate blocks, which evens out the last wave
  const int round = blockIdx.x / g.ncb, cb = blockIdx.x - round * g.ncb;
  const int j = blockIdx.y, b = blockIdx.z;
  Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + 2 * CB * NZ;
  const int nkx = g.nkx, mz = g.mz, nz = g.nz;
  const int i0 = cb * CB;
  const long pbase = (long)b * g.field + (long)j * g.plane;
  const V *vor = (const V *)((const R *)bf.vor + pbase);
  const V *phi = (const V *)((const R *)bf.phi + pbase);
  const V *Dv = (const V *)((const R *)bf.D + pbase);
  const V *Vv = (const V *)((const R *)bf.V + pbase);
  const V *Gv = (const V *)((const R *)bf.G + pbase);
  const V mu = ((const V *)bf.mu)[(long)b * g.my + j];
  const V mdu = ((const V *)bf.mdu)[(long)b * g.my + j];
  // temperature: tb as stored (its copy gets no set_conj, crosst.f90:556-559)
  // with the (0,0) mode replaced by tb00 (crosst.f90:1459-1462)
  const V *tbv = TEMP ? (const V *)((const R *)bf.tb + pbase) : nullptr;
  const R tb00 = TEMP ? ((const V *)bf.mt)[(long)b * g.my + j].x : (R)0;
  // omega_y and phi with the kx=0 conjugate symmetry imposed (set_conj on the
  // copies buff1/buff2, cross.f90:493-502)
  auto ld_sym = [&](const V *p, int i, int k) -> V {
    if (i == 0 && k > nz) {
      V v = p[(mz - k) * nkx];
      v.y = -v.y;
      return v;
    }
    return p[k * nkx + i];
  };
  V *zb = (V *)bf.zbuf + ((long)b * g.my + j) * (long)NZ * g.nzf * nkx;
  const V zero = mk2<R>((R)0, (R)0);
  if (TEMP && round == g.tround) {
    // the temperature alone: CB sequences
    for (int idx = threadIdx.x; idx < CB * NZ; idx += T) A[idx] = zero;
    __syncthreads();
    for (int idx = threadIdx.x; idx < CB * mz; idx += T) {
      const int ci = idx % CB, k = idx / CB, i = i0 + ci;
      if (i >= nkx) continue;
      A[ci * NZ + kgrid(k, nz, NZ, mz)] = (i == 0 && k == 0) ? mk2<R>(tb00, (R)0) : tbv[k * nkx + i];
    }
    V *res = fft_batch<NZ, +1, CB, T, true>(A, Bs, (const V *)tw_of<R>(bf, true));
    for (int idx = threadIdx.x; idx < CB * NZ; idx += T) {
      const int ci = idx % CB, z = idx / CB, i = i0 + ci;
      if (i < nkx) zb[((long)z * g.nzf + g.tzf) * nkx + i] = res[ci * NZ + z];
    }
    return;
  }
  {
    // fill two fields (zero the 2/3-rule gap) on the padded z grid
    for (int idx = threadIdx.x; idx < 2 * CB * NZ; idx += T) A[idx] = zero;
    __syncthreads();
    for (int idx = threadIdx.x; idx < CB * mz; idx += T) {
      const int ci = idx % CB, k = idx / CB, i = i0 + ci;
      if (i >= nkx) continue;
      const int kg = kgrid(k, nz, NZ, mz);
      const R a = (R)(g.alp * i);
      const int kzs = (k <= nz) ? k : k - mz;
      const R gz = (R)(g.gam * kzs);
      const R iK = kinv_of<R>(bf, (long)k * nkx + i);
      V fa, fb;
      const bool z00 = (i == 0 && k == 0);
      if (round == 0) {  // u (f=0) and w (f=1) from dv/dy and omega_y
        if (z00) {
          fa = mk2<R>(mu.x, (R)0);
          fb = mk2<R>(mu.y, (R)0);
        } else {
          const V dv = Vv[k * nkx + i], vr = ld_sym(vor, i, k);
          R tx = a * dv.x - gz * vr.x, ty = a * dv.y - gz * vr.y;
          fa = mk2<R>(-ty * iK, tx * iK);
          tx = gz * dv.x + a * vr.x; ty = gz * dv.y + a * vr.y;
          fb = mk2<R>(-ty * iK, tx * iK);
        }
      } else if (round == 1) {  // omega_x (f=2) and omega_z (f=3) from d(omega_y)/dy and phi
        if (z00) {
          fa = mk2<R>(mdu.y, (R)0);
          fb = mk2<R>(-mdu.x, (R)0);
        } else {
          const V w1 = Dv[k * nkx + i], ph = ld_sym(phi, i, k);
          R tx = a * w1.x + gz * ph.x, ty = a * w1.y + gz * ph.y;
          fa = mk2<R>(-ty * iK, tx * iK);
          tx = gz * w1.x - a * ph.x; ty = gz * w1.y - a * ph.y;
          fb = mk2<R>(-ty * iK, tx * iK);
        }
      } else if (round == 2) {  // v (f=4) and omega_y (f=5)
        fa = z00 ? mk2<R>((R)M.vbulk, (R)0) : Gv[k * nkx + i];
        fb = ld_sym(vor, i, k);
      } else if (round == 3) {
        // LES (cross.f90:1293-1325): dv/dy (f=6) and i kz w (f=7)
        if (z00) {
          fa = zero;
          fb = zero;
        } else {
          const V dv = Vv[k * nkx + i], vr = ld_sym(vor, i, k);
          fa = dv;
          const R tx = gz * dv.x + a * vr.x, ty = gz * dv.y + a * vr.y;
          const V u3 = mk2<R>(-ty * iK, tx * iK);
          fb = mk2<R>(-gz * u3.y, gz * u3.x);
        }
      } else {
        // LES: 2 i kz v + omega_x (f=8, dv/dz + dw/dy) and i kz u (f=9)
        if (z00) {
          fa = mk2<R>(mdu.y, (R)0);
          fb = zero;
        } else {
          const V w1 = Dv[k * nkx + i], ph = ld_sym(phi, i, k);
          R tx = a * w1.x + gz * ph.x, ty = a * w1.y + gz * ph.y;
          const V o1 = mk2<R>(-ty * iK, tx * iK);
          const V u2 = Gv[k * nkx + i];
          fa = mk2<R>((R)2 * (-gz * u2.y) + o1.x, (R)2 * (gz * u2.x) + o1.y);
          const V dv = Vv[k * nkx + i], vr = ld_sym(vor, i, k);
          tx = a * dv.x - gz * vr.x; ty = a * dv.y - gz * vr.y;
          const V u1 = mk2<R>(-ty * iK, tx * iK);
          fb = mk2<R>(-gz * u1.y, gz * u1.x);
        }
      }
      A[ci * NZ + kg] = fa;
      A[(CB + ci) * NZ + kg] = fb;
    }
    V *res = fft_batch<NZ, +1, 2 * CB, T, true>(A, Bs, (const V *)tw_of<R>(bf, true));
    // store Zbuf[z][f][i]
    for (int idx = threadIdx.x; idx < 2 * CB * NZ; idx += T) {
      const int ci = idx % CB, rem = idx / CB;
      const int z = rem % NZ, f = rem / NZ;
      const int i = i0 + ci;
      if (i < nkx) zb[((long)z * g.nzf + 2 * round + f) * nkx + i] = res[(f * CB + ci) * NZ + z];
    }
  }
}

// ---------------------------------------------------------------------------
// hist at the first substep of a statistics step (cross.f90:1796-2014;
// crosst.f90:2151-2160,2364-2374), from the substep's starting state (the
// inputs of plane stage 1, u, v, w and the vorticity reconstructed as
// there, cross.f90:1226-1276): per mode the spectra for HSF (nspec = 8: uu
// vv ww uv o1o1 o2o2 o3o3 o1o2) summed over the planes and, with the
// temperature, splt (tt ut vt wt); per plane the partial sums over the
// block's modes of the 11 hist quantities (up vp wp uvr uwr vwr o1p o2p o3p
// o12p eps) and of tbp utbp vtbp wtbp, reduced per plane by k_hsum.  A block
// takes 16 modes of a box; its 8 thread slices take every 8th plane; the
// per-mode slices are added in a fixed order, the per-plane modes in mode
// order through shared memory.  FP64 arithmetic whatever the storage precision.  Runs
// before the per-box scalars update Delta t: spl2 and splt carry the Delta t
// of the previous step, as in hist 'f'.
// ---------------------------------------------------------------------------
constexpr int kSpecModes = 16, kSpecSlices = 8;
template <typename R, bool TEMP>
__global__ void __launch_bounds__(kSpecModes * kSpecSlices) k_spectra(Grid g, Bufs bf) {
  typedef typename Vec2<R>::t V;
  const int b = blockIdx.y;
  const Member &M = bf.mem[b];
  if (M.halted || !M.ihist) return;  // uniform per block
  const int nkx = g.nkx, mz = g.mz, nz = g.nz, nl = nkx * mz;
  const int mi = threadIdx.x % kSpecModes, sl = threadIdx.x / kSpecModes;
  const int q0 = blockIdx.x * kSpecModes + mi;
  const bool valid = q0 < nl;
  const int q = valid ? q0 : nl - 1;
  const int i = q % nkx, k = q / nkx;
  const double a = g.alp * i;
  const double gz = g.gam * ((k <= nz) ? k : k - mz);
  const double Kk = a * a + gz * gz;
  const double iK = bf.kinv[q];
  // invalid threads (past the last mode) carry weight 0
  const double wm = valid ? ((i == 0) ? 1.0 : 2.0) : 0.0;
  const bool z00 = (i == 0 && k == 0);
  // set_conj of the omega_y and phi copies (cross.f90:502)
  const int qs = (i == 0 && k > nz) ? (mz - k) * nkx : q;
  const double cs = (i == 0 && k > nz) ? -1.0 : 1.0;
  const int nblk = gridDim.x;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, tacc[4] = {0, 0, 0, 0};
  // per-plane products of the 16 modes, double-buffered across iterations
  constexpr int NQ = TEMP ? SB_NHIST_Q : 11;
  __shared__ double tpart[2][kSpecSlices][NQ][kSpecModes + 1];
  // the same number of iterations on every slice (the block barrier in the
  // loop needs every thread): planes past the last carry weight 0
  const int niter = (g.my + kSpecSlices - 1) / kSpecSlices;
  for (int it = 0; it < niter; it++) {
    const int jr = sl + kSpecSlices * it;
    const bool jok = jr < g.my;
    const int j = jok ? jr : g.my - 1;
    const double w = jok ? wm : 0.0;
    const long pb = (long)b * g.field + (long)j * g.plane;
    const V *vor = (const V *)((const R *)bf.vor + pb), *phi = (const V *)((const R *)bf.phi + pb);
    const V *Dv = (const V *)((const R *)bf.D + pb), *Vv = (const V *)((const R *)bf.V + pb);
    const V *Gv = (const V *)((const R *)bf.G + pb);
    const V vr0 = vor[qs], ph0 = phi[qs];
    const V dvr = Vv[q];
    const double vrx = vr0.x, vry = cs * (double)vr0.y, phx = ph0.x, phy = cs * (double)ph0.y;
    const double dvx = dvr.x, dvy = dvr.y;
    double u1x, u1y, u2x, u2y, u3x, u3y, o1x, o1y, o3x, o3y;
    if (z00) {
      const V mu = ((const V *)bf.mu)[(long)b * g.my + j];
      const V mdu = ((const V *)bf.mdu)[(long)b * g.my + j];
      u1x = mu.x; u1y = 0.0;
      u3x = mu.y; u3y = 0.0;
      o3x = -(double)mdu.x; o3y = 0.0;
      o1x = mdu.y; o1y = 0.0;
      u2x = M.vbulk; u2y = 0.0;
    } else {
      const V w1 = Dv[q], gv = Gv[q];
      double tx, ty;
      tx = gz * w1.x - a * phx; ty = gz * w1.y - a * phy;
      o3x = -ty * iK; o3y = tx * iK;
      tx = a * w1.x + gz * phx; ty = a * w1.y + gz * phy;
      o1x = -ty * iK; o1y = tx * iK;
      tx = gz * dvx + a * vrx; ty = gz * dvy + a * vry;
      u3x = -ty * iK; u3y = tx * iK;
      tx = a * dvx - gz * vrx; ty = a * dvy - gz * vry;
      u1x = -ty * iK; u1y = tx * iK;
      u2x = gv.x; u2y = gv.y;
    }
    const double uu = u1x * u1x + u1y * u1y, vv = u2x * u2x + u2y * u2y,
                 ww = u3x * u3x + u3y * u3y;
    double pq[SB_NHIST_Q];
    pq[0] = w * uu;
    pq[1] = w * vv;
    pq[2] = w * ww;
    pq[3] = w * (u1x * u2x + u1y * u2y);
    pq[4] = w * (u1x * u3x + u1y * u3y);
    pq[5] = w * (u2x * u3x + u2y * u3y);
    pq[6] = w * (o1x * o1x + o1y * o1y);
    pq[7] = w * (vrx * vrx + vry * vry);
    pq[8] = w * (o3x * o3x + o3y * o3y);
    pq[9] = w * (o1x * vrx + o1y * vry);
    {
      // dissipation (cross.f90:1926-1944); omega_z of the mean includes -s
      const double o3sx = z00 ? o3x - g.s : o3x;
      const double c1x = o1x - gz * u2y, c1y = o1y + gz * u2x;   // o1 + i gz u2
      const double c3x = o3sx + a * u2y, c3y = o3y - a * u2x;    // o3 - i a u2
      pq[10] = w * (Kk * (uu + vv + ww) + (dvx * dvx + dvy * dvy) + (c1x * c1x + c1y * c1y) +
                    (c3x * c3x + c3y * c3y));
    }
    // spectra: omega_z of the mean without -s (cross.f90:1968)
    acc[0] += pq[0];
    acc[1] += pq[1];
    acc[2] += pq[2];
    acc[3] += pq[3];
    acc[4] += pq[6];
    acc[5] += pq[7];
    acc[6] += pq[8];
    acc[7] += pq[9];
    if (TEMP) {
      double tx, ty = 0.0;
      if (z00) {
        tx = ((const V *)bf.mt)[(long)b * g.my + j].x;
      } else {
        const V t = ((const V *)((const R *)bf.tb + pb))[q];
        tx = t.x;
        ty = t.y;
      }
      pq[11] = w * (tx * tx + ty * ty);
      pq[12] = w * (u1x * tx + u1y * ty);
      pq[13] = w * (u2x * tx + u2y * ty);
      pq[14] = w * (u3x * tx + u3y * ty);
#pragma unroll
      for (int f = 0; f < 4; f++) tacc[f] += pq[11 + f];
    }
    // the plane's partial over the block's 16 modes: the products go through
    // shared memory and one thread per (slice, quantity) adds its 16 modes in
    // order (15 FP64 adds per quantity, where a shuffle tree spends 4 adds on
    // every lane)
    double(*tp)[NQ][kSpecModes + 1] = tpart[it & 1];
#pragma unroll
    for (int f = 0; f < NQ; f++) tp[sl][f][mi] = pq[f];
    __syncthreads();
    if (threadIdx.x < kSpecSlices * NQ) {
      const int s2 = threadIdx.x / NQ, f = threadIdx.x - s2 * NQ;
      const int j2 = s2 + kSpecSlices * it;
      if (j2 < g.my) {
        double x = tp[s2][f][0];
#pragma unroll
        for (int m = 1; m < kSpecModes; m++) x += tp[s2][f][m];
        double *hp = bf.hpart + (((long)b * g.my + j2) * nblk + blockIdx.x) * SB_NHIST_Q;
        hp[f] = x;
        if (!TEMP && f == 0)
          for (int f2 = NQ; f2 < SB_NHIST_Q; f2++) hp[f2] = 0.0;
      }
    }
    // the next iteration writes the other buffer; the one after waits for this
    // iteration's readers at the next barrier
  }
  __shared__ double red[kSpecSlices][12][kSpecModes];
#pragma unroll
  for (int f = 0; f < 8; f++) red[sl][f][mi] = acc[f];
#pragma unroll
  for (int f = 0; f < 4; f++) red[sl][8 + f][mi] = tacc[f];
  __syncthreads();
  if (sl != 0 || !valid) return;
  const double dt = M.Deltat;
  double *sp = bf.spec + ((long)b * nl + q) * 8, *sp2 = bf.spec2 + ((long)b * nl + q) * 8;
  for (int f = 0; f < (TEMP ? 12 : 8); f++) {
    double x = 0.0;
    for (int s2 = 0; s2 < kSpecSlices; s2++) x += red[s2][f][mi];
    if (f < 8) {
      sp[f] += x;
      sp2[f] += x * dt;
    } else {
      bf.tspec[((long)b * nl + q) * 4 + (f - 8)] += x * dt;
    }
  }
}

// ---------------------------------------------------------------------------
// plane stage 2: x-transforms and u x omega on pairs of z rows
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dbits(double v) {
  return (unsigned long long)__double_as_longlong(fabs(v));
}

// NF = 6 fields to physical x, or 7 with the temperature (then 6 products:
// u x omega and the fluxes uT, wT, vT of crosst.f90:1680-1693)
template <typename R, int NX, int T, int NF>
__global__ void __launch_bounds__(T) k_p2(Grid g, Bufs bf, int rk) {
  typedef typename Vec2<R>::t V;
  constexpr int NO = (NF == 7) ? 6 : 3;
  const int zp = blockIdx.x, j = blockIdx.y, b = blockIdx.z;
  Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + NF * NX;
  const int nkx = g.nkx, NZ = g.mgalz;
  const int z = 2 * zp;
  const V *zb = (const V *)bf.zbuf + ((long)b * g.my + j) * (long)NZ * g.nzf * nkx;
  // Hermitian extension of two rows into one complex sequence (c2r of both rows
  // at once); FFTW's c2r ignores the imaginary part of the kx = 0 entry
  const V zero = mk2<R>((R)0, (R)0);
  for (int idx = threadIdx.x; idx < NF * NX; idx += T) A[idx] = zero;
  __syncthreads();
  for (int idx = threadIdx.x; idx < NF * nkx; idx += T) {
    const int f = idx / nkx, i = idx - f * nkx;
    const int zf = (f < 6) ? f : g.tzf;
    V X1 = zb[((long)z * g.nzf + zf) * nkx + i];
    V X2 = zb[((long)(z + 1) * g.nzf + zf) * nkx + i];
    if (i == 0) {
      X1.y = (R)0;
      X2.y = (R)0;
    }
    A[f * NX + i] = mk2<R>(X1.x - X2.y, X1.y + X2.x);
    if (i > 0) A[f * NX + NX - i] = mk2<R>(X1.x + X2.y, -X1.y + X2.x);
  }
  V *P = fft_batch<NX, +1, NF, T, true>(A, Bs, (const V *)tw_of<R>(bf, false));
  V *Q = (P == A) ? Bs : A;
  // fields: 0 u, 1 w, 2 omega_x, 3 omega_z, 4 v, 5 omega_y (, 6 tb)
  const R chi2 = (R)(2.0 * g.chi);
  const R sy = (R)(g.s * ((double)j * g.dy - 0.5 * g.Ly));
  R m0 = 0, m1 = 0, m2 = 0, m3 = 0, mt = 0;
  // hist 'p' (cross.f90:2038-2042): v u^2, v w^2, v^3 over the two rows; the
  // products in the storage precision, the sums in FP64
  const bool hist = (rk == 1) && M.ihist;
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  for (int x = threadIdx.x; x < NX; x += T) {
    const V u1 = P[0 * NX + x], u3 = P[1 * NX + x], o1 = P[2 * NX + x], o3 = P[3 * NX + x],
            u2 = P[4 * NX + x], o2 = P[5 * NX + x];
    if (hist) {
      s1 += (double)(u2.x * (u1.x * u1.x) + u2.y * (u1.y * u1.y));
      s2 += (double)(u2.x * (u3.x * u3.x) + u2.y * (u3.y * u3.y));
      s3 += (double)(u2.x * u2.x * u2.x + u2.y * u2.y * u2.y);
    }
    if (rk == 1) {
      m0 = fmax(m0, fmax(fabs(u1.x), fabs(u1.y)));
      m1 = fmax(m1, fmax(fabs(u1.x + sy), fabs(u1.y + sy)));
      m2 = fmax(m2, fmax(fabs(u2.x), fabs(u2.y)));
      m3 = fmax(m3, fmax(fabs(u3.x), fabs(u3.y)));
    }
    V h1, h2, h3;
    h1.x = u2.x * (o3.x + chi2) - u3.x * o2.x;
    h1.y = u2.y * (o3.y + chi2) - u3.y * o2.y;
    h2.x = u3.x * o1.x - u1.x * (o3.x + chi2);
    h2.y = u3.y * o1.y - u1.y * (o3.y + chi2);
    h3.x = u1.x * o2.x - u2.x * o1.x;
    h3.y = u1.y * o2.y - u2.y * o1.y;
    Q[0 * NX + x] = h1;
    Q[1 * NX + x] = h2;
    Q[2 * NX + x] = h3;
    if (NF == 7) {
      const V tb = P[6 * NX + x];
      if (rk == 1) mt = fmax(mt, fmax(fabs(tb.x), fabs(tb.y)));
      Q[3 * NX + x] = mk2<R>(u1.x * tb.x, u1.y * tb.y);
      Q[4 * NX + x] = mk2<R>(u3.x * tb.x, u3.y * tb.y);
      Q[5 * NX + x] = mk2<R>(u2.x * tb.x, u2.y * tb.y);
    }
  }
  if (rk == 1) {
    unsigned long long b0 = dbits(m0), b1 = dbits(m1), b2 = dbits(m2), b3 = dbits(m3);
    for (int o = 16; o > 0; o >>= 1) {
      b0 = max(b0, __shfl_xor_sync(0xffffffffu, b0, o));
      b1 = max(b1, __shfl_xor_sync(0xffffffffu, b1, o));
      b2 = max(b2, __shfl_xor_sync(0xffffffffu, b2, o));
      b3 = max(b3, __shfl_xor_sync(0xffffffffu, b3, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&M.umax_bits[0], b0);
      atomicMax(&M.umax_bits[1], b1);
      atomicMax(&M.umax_bits[2], b2);
      atomicMax(&M.umax_bits[3], b3);
    }
    if (NF == 7) {
      unsigned long long bt = dbits(mt);
      for (int o = 16; o > 0; o >>= 1) bt = max(bt, __shfl_xor_sync(0xffffffffu, bt, o));
      if ((threadIdx.x & 31) == 0) atomicMax(&M.tbmax_bits, bt);
    }
  }
  if (hist) {
    // warp sums in a fixed tree, one triple per (plane, row pair, warp); the
    // plane sums follow in k_hsum
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_down_sync(0xffffffffu, s1, o);
      s2 += __shfl_down_sync(0xffffffffu, s2, o);
      s3 += __shfl_down_sync(0xffffffffu, s3, o);
    }
    if ((threadIdx.x & 31) == 0) {
      double *pp = bf.ppart + ((((long)b * g.my + j) * (g.mgalz / 2) + zp) * (T / 32) +
                               (threadIdx.x >> 5)) * 3;
      pp[0] = s1;
      pp[1] = s2;
      pp[2] = s3;
    }
  }
  V *Rr = fft_batch<NX, -1, NO, T>(Q, P, (const V *)tw_of<R>(bf, false));
  V *xb = (V *)bf.xbuf + ((long)b * g.my + j) * (long)NZ * NO * nkx;
  // the two rows' spectra, each times 2: (Z_k + conj Z_-k) and
  // -i (Z_k - conj Z_-k); k_p3 takes the factor 1/2 with the normalisation
  // (a power of two: the same rounding)
  for (int idx = threadIdx.x; idx < NO * nkx; idx += T) {
    const int f = idx / nkx, i = idx - f * nkx;
    const V zk = Rr[f * NX + i];
    const V zm = Rr[f * NX + ((NX - i) % NX)];
    xb[((long)z * NO + f) * nkx + i] = mk2<R>(zk.x + zm.x, zk.y - zm.y);
    xb[((long)(z + 1) * NO + f) * nkx + i] = mk2<R>(zk.y + zm.y, zm.x - zk.x);
  }
}

// ---------------------------------------------------------------------------
// plane stage 3: forward z-transforms, truncation and right-hand sides
// ---------------------------------------------------------------------------
// NF = 3 nonlinear terms, or 6 with the temperature fluxes
template <typename R, int NZ, int CB, int T, int NF>
__global__ void __launch_bounds__(T) k_p3(Grid g, Bufs bf) {
  typedef typename Vec2<R>::t V;
  const int cb = blockIdx.x, j = blockIdx.y, b = blockIdx.z;
  Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + NF * CB * NZ;
  const int nkx = g.nkx, mz = g.mz, nz = g.nz;
  const int i0 = cb * CB;
  const V *xb = (const V *)bf.xbuf + ((long)b * g.my + j) * (long)NZ * NF * nkx;
  // the block's columns of the x-transformed rows, copied to shared memory
  // asynchronously (all of a thread's copies in flight at once); columns
  // beyond nkx are zero
  for (int idx = threadIdx.x; idx < NF * CB * NZ; idx += T) {
    const int ci = idx % CB, rem = idx / CB;
    const int f = rem % NF, z = rem / NF;
    const int i = i0 + ci;
    cp_async<sizeof(V)>(&A[(f * CB + ci) * NZ + z], xb + ((long)z * NF + f) * nkx + (i < nkx ? i : 0),
                        i < nkx);
  }
  cp_async_wait_all();
  V *P = fft_batch<NZ, -1, NF * CB, T>(A, Bs, (const V *)tw_of<R>(bf, true));
  const long pbase = (long)b * g.field + (long)j * g.plane;
  V *Dv = (V *)((R *)bf.D + pbase);
  V *Gv = (V *)((R *)bf.G + pbase);
  V *Vv = (V *)((R *)bf.V + pbase);
  // 1/(mgalx mgalz) of the forward transform and the 1/2 of k_p2's row split
  const R norm = (R)(0.5 / (double)(g.mgalx * g.mgalz));
  const R s = (R)g.s;
  // streamwise-roll force of this plane on hv(kx=0, kz=1) (add_force,
  // operators.f90:14-37)
  const bool force = g.force > 0;
  double fj = 0.0;
  if (force) {
    const double y = (double)j * g.dy - 0.5 * g.Ly, w = 1.0 - y * y, gm = g.gam;
    fj = (g.force == 1) ? -0.5 * g.force_roll * (-4.0 * (1.0 - 3.0 * y * y) - gm * gm * w * w)
                        : 0.5 * g.force_roll * (4.0 * y * (-3.0 + 5.0 * y * y) - y * w * w * gm * gm);
  }
  for (int idx = threadIdx.x; idx < CB * mz; idx += T) {
    const int ci = idx % CB, k = idx / CB, i = i0 + ci;
    if (i >= nkx) continue;
    const int kg = kgrid(k, nz, NZ, mz);
    V H1 = P[(0 * CB + ci) * NZ + kg], H2 = P[(1 * CB + ci) * NZ + kg],
      H3 = P[(2 * CB + ci) * NZ + kg];
    H1.x *= norm; H1.y *= norm;
    H2.x *= norm; H2.y *= norm;
    H3.x *= norm; H3.y *= norm;
    const R a = (R)(g.alp * i);
    const int kzs = (k <= nz) ? k : k - mz;
    const R gz = (R)(g.gam * kzs);
    const R Kk = a * a + gz * gz;
    const long q = (long)k * nkx + i;
    const V v = Gv[q];
    if (NF == 6) {
      // ht = -i a uT - i gz wT - bym v with the input v, and -vT
      // (crosst.f90:1148-1152,1691-1692)
      V uT = P[(3 * CB + ci) * NZ + kg], wT = P[(4 * CB + ci) * NZ + kg],
        vT = P[(5 * CB + ci) * NZ + kg];
      uT.x *= norm; uT.y *= norm;
      wT.x *= norm; wT.y *= norm;
      vT.x *= norm; vT.y *= norm;
      const R bym = (R)g.bym;
      const R tx = a * uT.y + gz * wT.y, ty = -(a * uT.x) - gz * wT.x;
      ((V *)((R *)bf.Ht + pbase))[q] = mk2<R>(tx - bym * v.x, ty - bym * v.y);
      ((V *)((R *)bf.R2 + pbase))[q] = mk2<R>(-vT.x, -vT.y);
    }
    // dvordy = i a H1 + i gz H3
    R tx = a * H1.x + gz * H3.x, ty = a * H1.y + gz * H3.y;
    Dv[q] = mk2<R>(-ty, tx);
    // hg = -i a H3 + i gz (H1 - s v)
    tx = gz * (H1.x - s * v.x) - a * H3.x;
    ty = gz * (H1.y - s * v.y) - a * H3.y;
    Gv[q] = mk2<R>(-ty, tx);
    // hv = -(kx^2 + kz^2) H2
    V hv = mk2<R>(-(Kk * H2.x), -(Kk * H2.y));
    if (force && i == 0 && k == 1) hv.x = (R)((double)hv.x + fj);
    Vv[q] = hv;
    if (i == 0 && k == 0) ((V *)bf.mrf)[(long)b * g.my + j] = mk2<R>(H1.x, H3.x);
  }
}

// ---------------------------------------------------------------------------
// Smagorinsky LES stage (iuse_LES, cross.f90:1291-1406).  Per substep, after
// k_p2 (the zbuf z-transforms also hold dv/dy, i kz w, 2 i kz v + omega_x and
// i kz u, written by k_p1):
//   k_les2  per (plane, z row pair): the six strain-rate combinations
//           du/dx, dv/dy, dw/dz, dv/dz+dw/dy, du/dy+dv/dx, du/dz+dw/dx to
//           physical x (kept in gbuf), |S|^2 with the mean shear, its
//           forward x-transform
//   k_les3  per (plane, kx block): forward z-transform, 2/3 truncation and
//           backward z-transform of |S|^2 (the r2c/c2r pair of rev.1317)
//   k_les4  per (plane, z row pair): dealiased |S|^2 to physical x,
//           nu_t = (Cles Deltag)^2 |S|, the stresses T11..T33, nu_t maxima and
//           statistics, forward x-transforms of the stresses
//   k_les5  per (plane, kx block, after k_p3): forward z-transforms of the
//           stresses, the right-hand-side pieces rhvc1 (subtracted from
//           dH1/dx + dH3/dz), rhgc1 (added to the omega_y right-hand side),
//           rhvc2 and rhgc2 (y-operators applied by k_lineL), T12 and T23 of
//           the (0,0) mode
// ---------------------------------------------------------------------------
template <typename R, int NX, int T>
__global__ void __launch_bounds__(T) k_les2(Grid g, Bufs bf) {
  typedef typename Vec2<R>::t V;
  const int zp = blockIdx.x, j = blockIdx.y, b = blockIdx.z;
  const Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + 6 * NX;
  const int nkx = g.nkx, NZ = g.mgalz, nzf = g.nzf;
  const int z = 2 * zp;
  const V *zb = (const V *)bf.zbuf + ((long)b * g.my + j) * (long)NZ * nzf * nkx;
  const V zero = mk2<R>((R)0, (R)0);
  for (int idx = threadIdx.x; idx < 6 * NX; idx += T) A[idx] = zero;
  __syncthreads();
  // zbuf fields: 0 u, 1 w, 2 omega_x, 3 omega_z, 4 v, 5 omega_y, 6 dv/dy,
  // 7 i kz w, 8 2 i kz v + omega_x, 9 i kz u
  for (int idx = threadIdx.x; idx < 6 * nkx; idx += T) {
    const int f = idx / nkx, i = idx - f * nkx;
    const R a = (R)(g.alp * i);
    V X[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const V *row = zb + (long)(z + r) * nzf * nkx;
      V x;
      if (f == 0) {  // du/dx
        const V u = row[i];
        x = mk2<R>(-a * u.y, a * u.x);
      } else if (f == 1) {  // dv/dy
        x = row[6 * nkx + i];
      } else if (f == 2) {  // dw/dz
        x = row[7 * nkx + i];
      } else if (f == 3) {  // dv/dz + dw/dy
        x = row[8 * nkx + i];
      } else if (f == 4) {  // du/dy + dv/dx = 2 dv/dx - omega_z
        const V v = row[4 * nkx + i], o3 = row[3 * nkx + i];
        x = mk2<R>((R)2 * (-a * v.y) - o3.x, (R)2 * (a * v.x) - o3.y);
      } else {  // du/dz + dw/dx
        const V w = row[nkx + i], izu = row[9 * nkx + i];
        x = mk2<R>(izu.x + (-a * w.y), izu.y + a * w.x);
      }
      X[r] = x;
    }
    if (i == 0) {
      X[0].y = (R)0;
      X[1].y = (R)0;
    }
    A[f * NX + i] = mk2<R>(X[0].x - X[1].y, X[0].y + X[1].x);
    if (i > 0) A[f * NX + NX - i] = mk2<R>(X[0].x + X[1].y, -X[0].y + X[1].x);
  }
  V *P = fft_batch<NX, +1, 6, T, true>(A, Bs, (const V *)tw_of<R>(bf, false));
  V *Q = (P == A) ? Bs : A;
  R *gb = (R *)bf.gbuf + (((long)b * g.my + j) * (NZ / 2) + zp) * 12L * NX;
  const R s = (R)g.s;
  for (int x = threadIdx.x; x < NX; x += T) {
    const V ux = P[x], vy = P[NX + x], wz = P[2 * NX + x], vz = P[3 * NX + x],
            uy = P[4 * NX + x], uz = P[5 * NX + x];
#pragma unroll
    for (int f = 0; f < 6; f++) {
      gb[(2 * f) * NX + x] = P[f * NX + x].x;
      gb[(2 * f + 1) * NX + x] = P[f * NX + x].y;
    }
    // Sij2 (cross.f90:1330-1337)
    const R s0 = (R)2 * ux.x * ux.x + (uy.x + s) * (uy.x + s) + (R)2 * vy.x * vy.x +
                 uz.x * uz.x + (R)2 * wz.x * wz.x + vz.x * vz.x;
    const R s1 = (R)2 * ux.y * ux.y + (uy.y + s) * (uy.y + s) + (R)2 * vy.y * vy.y +
                 uz.y * uz.y + (R)2 * wz.y * wz.y + vz.y * vz.y;
    Q[x] = mk2<R>(s0, s1);
  }
  V *Rr = fft_batch<NX, -1, 1, T>(Q, P, (const V *)tw_of<R>(bf, false));
  V *sbp = (V *)bf.sbuf + ((long)b * g.my + j) * (long)NZ * nkx;
  // the two rows' spectra times 2 (k_les3 takes the 1/2 with the normalisation)
  for (int i = threadIdx.x; i < nkx; i += T) {
    const V zk = Rr[i];
    const V zm = Rr[(NX - i) % NX];
    sbp[(long)z * nkx + i] = mk2<R>(zk.x + zm.x, zk.y - zm.y);
    sbp[(long)(z + 1) * nkx + i] = mk2<R>(zk.y + zm.y, zm.x - zk.x);
  }
}

template <typename R, int NZ, int CB, int T>
__global__ void __launch_bounds__(T) k_les3(Grid g, Bufs bf) {
  typedef typename Vec2<R>::t V;
  const int cb = blockIdx.x, j = blockIdx.y, b = blockIdx.z;
  const Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + CB * NZ;
  const int nkx = g.nkx, nz = g.nz, i0 = cb * CB;
  V *sbp = (V *)bf.sbuf + ((long)b * g.my + j) * (long)NZ * nkx;
  const V zero = mk2<R>((R)0, (R)0);
  for (int idx = threadIdx.x; idx < CB * NZ; idx += T) {
    const int ci = idx % CB, z = idx / CB, i = i0 + ci;
    A[ci * NZ + z] = (i < nkx) ? sbp[(long)z * nkx + i] : zero;
  }
  V *P = fft_batch<NZ, -1, CB, T>(A, Bs, (const V *)tw_of<R>(bf, true));
  // 1/(mgalx mgalz) and the 1/2 of k_les2's row split (a power of two)
  const R norm = (R)(0.5 / (double)(g.mgalx * g.mgalz));
  for (int idx = threadIdx.x; idx < CB * NZ; idx += T) {
    const int z = idx % NZ;
    const bool keep = (z <= nz) || (z >= NZ - nz);
    V v = P[idx];
    P[idx] = keep ? mk2<R>(norm * v.x, norm * v.y) : zero;
  }
  // the truncated spectrum has the zero middle third of the 2/3 rule
  V *Q = fft_batch<NZ, +1, CB, T, true>(P, (P == A) ? Bs : A, (const V *)tw_of<R>(bf, true));
  for (int idx = threadIdx.x; idx < CB * NZ; idx += T) {
    const int ci = idx % CB, z = idx / CB, i = i0 + ci;
    if (i < nkx) sbp[(long)z * nkx + i] = Q[ci * NZ + z];
  }
}

template <typename R, int NX, int T>
__global__ void __launch_bounds__(T) k_les4(Grid g, Bufs bf, int rk) {
  typedef typename Vec2<R>::t V;
  const int zp = blockIdx.x, j = blockIdx.y, b = blockIdx.z;
  Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + 6 * NX;
  const int nkx = g.nkx, NZ = g.mgalz;
  const int z = 2 * zp;
  const V *sbp = (const V *)bf.sbuf + ((long)b * g.my + j) * (long)NZ * nkx;
  const V zero = mk2<R>((R)0, (R)0);
  for (int idx = threadIdx.x; idx < NX; idx += T) A[idx] = zero;
  __syncthreads();
  for (int i = threadIdx.x; i < nkx; i += T) {
    V X1 = sbp[(long)z * nkx + i], X2 = sbp[(long)(z + 1) * nkx + i];
    if (i == 0) {
      X1.y = (R)0;
      X2.y = (R)0;
    }
    A[i] = mk2<R>(X1.x - X2.y, X1.y + X2.x);
    if (i > 0) A[NX - i] = mk2<R>(X1.x + X2.y, -X1.y + X2.x);
  }
  V *P = fft_batch<NX, +1, 1, T, true>(A, Bs, (const V *)tw_of<R>(bf, false));
  V *Q = (P == A) ? Bs : A;
  const R *gb = (const R *)bf.gbuf + (((long)b * g.my + j) * (NZ / 2) + zp) * 12L * NX;
  const R C = (R)g.les_c, s = (R)g.s;
  const bool neg = g.s < 0.0;
  const bool stats = (rk == 1) && M.ihist;
  R nmax = (R)0;
  double snu = 0.0, sds = 0.0;
  for (int x = threadIdx.x; x < NX; x += T) {
    const V S2 = P[x];
    R n0 = C * sqrt(fabs(S2.x)), n1 = C * sqrt(fabs(S2.y));
    if (neg) {
      n0 = -n0;
      n1 = -n1;
    }
    if (rk == 1) nmax = fmax(nmax, fmax(fabs(n0), fabs(n1)));
    if (stats) {
      snu += (double)n0 + (double)n1;
      sds += (double)n0 * (double)S2.x + (double)n1 * (double)S2.y;
    }
    // gradients: 0 ux, 1 vy, 2 wz, 3 vz+wy, 4 uy+vx, 5 uz+wx (two rows each)
    const R ux0 = gb[0 * NX + x], ux1 = gb[1 * NX + x], vy0 = gb[2 * NX + x],
            vy1 = gb[3 * NX + x], wz0 = gb[4 * NX + x], wz1 = gb[5 * NX + x],
            vz0 = gb[6 * NX + x], vz1 = gb[7 * NX + x], uy0 = gb[8 * NX + x],
            uy1 = gb[9 * NX + x], uz0 = gb[10 * NX + x], uz1 = gb[11 * NX + x];
    // T11 T12 T13 T22 T23 T33 (cross.f90:1371-1376)
    Q[0 * NX + x] = mk2<R>((R)2 * n0 * ux0, (R)2 * n1 * ux1);
    Q[1 * NX + x] = mk2<R>(n0 * (uy0 + s), n1 * (uy1 + s));
    Q[2 * NX + x] = mk2<R>(n0 * uz0, n1 * uz1);
    Q[3 * NX + x] = mk2<R>((R)2 * n0 * vy0, (R)2 * n1 * vy1);
    Q[4 * NX + x] = mk2<R>(n0 * vz0, n1 * vz1);
    Q[5 * NX + x] = mk2<R>((R)2 * n0 * wz0, (R)2 * n1 * wz1);
  }
  if (rk == 1) {
    unsigned long long bb = dbits((double)nmax);
    for (int o = 16; o > 0; o >>= 1) bb = max(bb, __shfl_xor_sync(0xffffffffu, bb, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&M.nut_bits, bb);
  }
  if (stats) {
    __shared__ double red[2][T / 32];
    for (int o = 16; o > 0; o >>= 1) {
      snu += __shfl_down_sync(0xffffffffu, snu, o);
      sds += __shfl_down_sync(0xffffffffu, sds, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = snu;
      red[1][threadIdx.x >> 5] = sds;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
      double v = 0.0;
      for (int w = 0; w < T / 32; w++) v += red[threadIdx.x][w];
      bf.lpart[(((long)b * g.my + j) * (NZ / 2) + zp) * 2 + threadIdx.x] = v;
    }
  }
  V *Rr = fft_batch<NX, -1, 6, T>(Q, P, (const V *)tw_of<R>(bf, false));
  V *tb = (V *)bf.tbuf + ((long)b * g.my + j) * (long)NZ * 6 * nkx;
  // the two rows' spectra times 2 (k_les5 takes the 1/2 with the normalisation)
  for (int idx = threadIdx.x; idx < 6 * nkx; idx += T) {
    const int f = idx / nkx, i = idx - f * nkx;
    const V zk = Rr[f * NX + i];
    const V zm = Rr[f * NX + ((NX - i) % NX)];
    tb[((long)z * 6 + f) * nkx + i] = mk2<R>(zk.x + zm.x, zk.y - zm.y);
    tb[((long)(z + 1) * 6 + f) * nkx + i] = mk2<R>(zk.y + zm.y, zm.x - zk.x);
  }
}

template <typename R, int NZ, int CB, int T>
__global__ void __launch_bounds__(T) k_les5(Grid g, Bufs bf) {
  typedef typename Vec2<R>::t V;
  const int cb = blockIdx.x, j = blockIdx.y, b = blockIdx.z;
  const Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + 6 * CB * NZ;
  const int nkx = g.nkx, mz = g.mz, nz = g.nz, i0 = cb * CB;
  const V *tb = (const V *)bf.tbuf + ((long)b * g.my + j) * (long)NZ * 6 * nkx;
  const V zero = mk2<R>((R)0, (R)0);
  for (int idx = threadIdx.x; idx < 6 * CB * NZ; idx += T) {
    const int ci = idx % CB, rem = idx / CB;
    const int f = rem % 6, z = rem / 6, i = i0 + ci;
    A[(f * CB + ci) * NZ + z] = (i < nkx) ? tb[((long)z * 6 + f) * nkx + i] : zero;
  }
  V *P = fft_batch<NZ, -1, 6 * CB, T>(A, Bs, (const V *)tw_of<R>(bf, true));
  const long pbase = (long)b * g.field + (long)j * g.plane;
  V *Dv = (V *)((R *)bf.D + pbase);
  V *Gv = (V *)((R *)bf.G + pbase);
  V *L1 = (V *)((R *)bf.L1 + pbase);
  V *L2 = (V *)((R *)bf.L2 + pbase);
  // 1/(mgalx mgalz) and the 1/2 of k_les4's row split (a power of two)
  const R norm = (R)(0.5 / (double)(g.mgalx * g.mgalz));
  for (int idx = threadIdx.x; idx < CB * mz; idx += T) {
    const int ci = idx % CB, k = idx / CB, i = i0 + ci;
    if (i >= nkx) continue;
    const int kg = kgrid(k, nz, NZ, mz);
    V t[6];
#pragma unroll
    for (int f = 0; f < 6; f++) {
      const V v = P[(f * CB + ci) * NZ + kg];
      t[f] = mk2<R>(norm * v.x, norm * v.y);
    }
    const V t11 = t[0], t12 = t[1], t13 = t[2], t22 = t[3], t23 = t[4], t33 = t[5];
    const R a = (R)(g.alp * i);
    const int kzs = (k <= nz) ? k : k - mz;
    const R gz = (R)(g.gam * kzs);
    const R a2 = a * a, g2 = gz * gz;
    // products of the imaginary wavenumbers: 2 xalp xgam, xalp xgam
    const R m2ag = -(((R)2 * a) * gz), mag = -(a * gz);
    const R ak = a2 + g2, ga = -g2 + a2;
    const long q = (long)k * nkx + i;
    // rhvc1, rhvc2, rhgc1, rhgc2 (cross.f90:1398-1403)
    const V rv1 = mk2<R>(a2 * t11.x - m2ag * t13.x + g2 * t33.x - ak * t22.x,
                         a2 * t11.y - m2ag * t13.y + g2 * t33.y - ak * t22.y);
    const V rv2 = mk2<R>((-a * t12.y) + (-gz * t23.y), (a * t12.x) + (gz * t23.x));
    const V rg1 = mk2<R>(mag * (t11.x - t33.x) + ga * t13.x, mag * (t11.y - t33.y) + ga * t13.y);
    const V rg2 = mk2<R>((-gz * t12.y) - (-a * t23.y), (gz * t12.x) - (a * t23.x));
    // dvordy - rhvc1 (cross.f90:561-564), hg + rhgc1 (cross.f90:608)
    V d = Dv[q];
    Dv[q] = mk2<R>(d.x - rv1.x, d.y - rv1.y);
    V h = Gv[q];
    Gv[q] = mk2<R>(h.x + rg1.x, h.y + rg1.y);
    L1[q] = rv2;
    L2[q] = rg2;
    if (i == 0 && k == 0) ((V *)bf.txy)[(long)b * g.my + j] = mk2<R>(t12.x, t23.x);
  }
}

// ---------------------------------------------------------------------------
// y dealiasing (iydealiasing 1, 2: dealiasing_y, operators.f90:352-467, called
// at the start of every substep, cross.f90:459-474) and the y-line transforms
// rfty / cfty (rftdoublew.F:133-158, cftdoublew.F:151-201): forward transforms
// scaled by 1/my, backward unscaled, FFTW sign conventions.
// ---------------------------------------------------------------------------
template <typename R> __device__ __forceinline__ const R *twy_of(const Bufs &bf);
template <> __device__ __forceinline__ const double *twy_of<double>(const Bufs &bf) { return bf.twy; }
template <> __device__ __forceinline__ const float *twy_of<float>(const Bufs &bf) { return bf.twyf; }

// Mean profiles u00 + i w00 of one box: 2/3 rule of their real y-spectra
// (modes m >= my23/2 and their conjugates).  With iydealiasing = 2 the first
// substep of a step wraps the offsets into one box length (cross.f90:348-351);
// every substep stores the moving-frame shift of its starting offset
// (cross.f90:459-463).
template <typename R, int MY, int T>
__global__ void __launch_bounds__(T) k_ydeal_mean(Grid g, Bufs bf, int rk) {
  typedef typename Vec2<R>::t V;
  const int b = blockIdx.x;
  Member &M = bf.mem[b];
  if (M.halted) return;
  __shared__ V A[MY], Bs[MY];
  if (threadIdx.x == 0) {
    if (g.ydeal == 2 && rk == 1) {
      M.xoffb = (M.xoffb / g.Lx - trunc(M.xoffb / g.Lx)) * g.Lx;
      M.xofft = -M.xoffb;
      M.xwb[0] = M.xoffb;
      M.xwt[0] = M.xofft;
    }
    const double xb = M.xwb[rk - 1];
    double fac = (xb / g.Lx - trunc(xb / g.Lx)) * g.Lx / g.Ly;
    if (fac < -g.Lx / g.Ly * 0.5) fac = g.Lx / g.Ly + fac;
    M.ydfac = fac;
  }
  V *mu = (V *)bf.mu + (long)b * MY;
  for (int j = threadIdx.x; j < MY; j += T) A[j] = mu[j];
  V *P = fft_batch<MY, -1, 1, T>(A, Bs, (const V *)twy_of<R>(bf));
  const int K = g.my23 / 2;
  const R dnf = (R)(1.0 / (double)MY);
  for (int m = threadIdx.x; m < MY; m += T) {
    const V z = P[m];
    P[m] = (m >= K && m <= MY - K) ? mk2<R>((R)0, (R)0) : mk2<R>(dnf * z.x, dnf * z.y);
  }
  V *Q = fft_batch<MY, +1, 1, T>(P, P == A ? Bs : A, (const V *)twy_of<R>(bf));
  for (int j = threadIdx.x; j < MY; j += T) mu[j] = Q[j];
}

// CB lines (consecutive kx at one kz) of omega_y or phi of one box: moving
// frame exp(i kx y fac) (iydealiasing 2; for 1 only kx = 0 is cut, where the
// frame is the identity), forward y-transform, the cut of dealiasing_y,
// backward transform, frame back.
template <typename R, int MY, int CB, int T>
__global__ void __launch_bounds__(T) k_ydeal(Grid g, Bufs bf) {
  typedef typename Vec2<R>::t V;
  const int k = blockIdx.y, b = blockIdx.z >> 1, fld = blockIdx.z & 1;
  const Member &M = bf.mem[b];
  if (M.halted) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + CB * MY;
  const int nkx = g.nkx, i0 = blockIdx.x * CB;
  const int ie = (g.ydeal == 1) ? 1 : nkx;
  V *f = (V *)((R *)(fld ? bf.phi : bf.vor) + (long)b * g.field) + (long)k * nkx;
  const long ps = g.plane / 2;  // complex entries per plane
  const double fac = M.ydfac;
  const bool frame = (g.ydeal == 2);
  for (int idx = threadIdx.x; idx < CB * MY; idx += T) {
    const int ci = idx % CB, j = idx / CB, i = i0 + ci;
    V v = mk2<R>((R)0, (R)0);
    if (i < ie) {
      v = f[(long)j * ps + i];
      if (frame) {
        double sn, cs;
        sincos(((g.alp * i) * ((double)j * g.dy - 0.5 * g.Ly)) * fac, &sn, &cs);
        v = mk2<R>((R)((double)v.x * cs - (double)v.y * sn), (R)((double)v.x * sn + (double)v.y * cs));
      }
    }
    A[ci * MY + j] = v;
  }
  V *P = fft_batch<MY, -1, CB, T>(A, Bs, (const V *)twy_of<R>(bf));
  const R dnf = (R)(1.0 / (double)MY);
  const double r = (double)g.ny1 / (double)(nkx - 1);
  const double LxLy = g.Lx / g.Ly;
  // The band edges are compared with integers, often exactly at an integer:
  // they are evaluated with explicitly rounded operations (no fused
  // multiply-add) so that they round as the reference's expressions do.
  auto edge = [&](double x, double di) {
    return __dmul_rn(__ddiv_rn(__dmul_rn(__dmul_rn(r, x), g.Ly), g.Lx), di);
  };
  for (int idx = threadIdx.x; idx < CB * MY; idx += T) {
    const int ci = idx / MY, j = idx % MY, i = i0 + ci;
    const double di = (double)i, dj = (double)j;
    const double xa = (g.ydeal == 1 || fac <= 0.0) ? __dsub_rn(-fac, LxLy) : __dadd_rn(-fac, LxLy);
    const double djda = edge(xa, di), djdb = edge(-fac, di);
    const double a1 = __dadd_rn((double)g.ny1, djda), a2 = __dadd_rn((double)g.ny2, djda);
    const double b1 = __dadd_rn((double)g.ny1, djdb), b2 = __dadd_rn((double)g.ny2, djdb);
    bool cut;
    if (g.ydeal == 1)
      cut = (dj > b1) && (dj < b2);
    else
      cut = ((dj >= b1) && (dj <= b2)) || ((dj > a1) && (dj < a2));
    const V z = P[idx];
    P[idx] = cut ? mk2<R>((R)0, (R)0) : mk2<R>(dnf * z.x, dnf * z.y);
  }
  V *Q = fft_batch<MY, +1, CB, T>(P, P == A ? Bs : A, (const V *)twy_of<R>(bf));
  for (int idx = threadIdx.x; idx < CB * MY; idx += T) {
    const int ci = idx % CB, j = idx / CB, i = i0 + ci;
    if (i >= ie) continue;
    V v = Q[ci * MY + j];
    if (frame) {
      double sn, cs;
      sincos(((g.alp * i) * ((double)j * g.dy - 0.5 * g.Ly)) * (-fac), &sn, &cs);
      v = mk2<R>((R)((double)v.x * cs - (double)v.y * sn), (R)((double)v.x * sn + (double)v.y * cs));
    }
    f[(long)j * ps + i] = v;
  }
}

// Standalone y-line transforms on device lines [j][line] (FP64): complex lines
// (cfty, c[2 (j ldc + l)]) or packed real lines of my + 2 rows (rfty, c[j ldc + l]).
template <int MY, int CB, int T>
__global__ void __launch_bounds__(T) k_yop(int nlines, double *c, long ldc, int iopt, int real) {
  __shared__ double2 A[CB * MY], Bs[CB * MY], tw[MY];
  for (int t = threadIdx.x; t < MY; t += T) {
    double sn, cs;
    sincospi(-2.0 * (double)t / (double)MY, &sn, &cs);
    tw[t] = make_double2(cs, sn);
  }
  const int l0 = blockIdx.x * CB;
  for (int idx = threadIdx.x; idx < CB * MY; idx += T) {
    const int ci = idx % CB, j = idx / CB, l = l0 + ci;
    double2 v = make_double2(0.0, 0.0);
    if (l < nlines) {
      if (!real) {
        v = make_double2(c[2 * ((long)j * ldc + l)], c[2 * ((long)j * ldc + l) + 1]);
      } else if (iopt < 0) {
        v = make_double2(c[(long)j * ldc + l], 0.0);
      } else {
        // Hermitian extension of the packed half spectrum; c2r ignores the
        // imaginary parts of modes 0 and my/2
        const int m = (j <= MY / 2) ? j : MY - j;
        double re = c[(long)(2 * m) * ldc + l], im = c[(long)(2 * m + 1) * ldc + l];
        if (m == 0 || 2 * m == MY) im = 0.0;
        v = make_double2(re, j <= MY / 2 ? im : -im);
      }
    }
    A[ci * MY + j] = v;
  }
  double2 *P = (iopt < 0) ? fft_batch_std<MY, -1, CB, T>(A, Bs, tw)
                           : fft_batch_std<MY, +1, CB, T>(A, Bs, tw);
  const double dnf = 1.0 / (double)MY;
  for (int idx = threadIdx.x; idx < CB * (MY + 2); idx += T) {
    const int ci = idx % CB, j = idx / CB, l = l0 + ci;
    if (l >= nlines) continue;
    if (!real) {
      if (j >= MY) continue;
      double2 v = P[ci * MY + j];
      if (iopt < 0) v = make_double2(dnf * v.x, dnf * v.y);
      c[2 * ((long)j * ldc + l)] = v.x;
      c[2 * ((long)j * ldc + l) + 1] = v.y;
    } else if (iopt < 0) {
      const double2 v = P[ci * MY + (j >> 1)];
      c[(long)j * ldc + l] = dnf * ((j & 1) ? v.y : v.x);
    } else {
      c[(long)j * ldc + l] = (j < MY) ? P[ci * MY + j].x : 0.0;
    }
  }
}

// pencil (j fastest, then kx, then kz, FP64 host layout) <-> plane-major
// device layout of storage type R, one box
template <typename R>
__global__ void k_pencil_to_plane(Grid g, const double *__restrict__ pen, R *__restrict__ dst) {
  const long n = (long)g.my * g.nkx * g.mz;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.nkx);
    const int k = (int)((t / g.nkx) % g.mz);
    const int j = (int)(t / ((long)g.nkx * g.mz));
    const long src = 2 * (((long)k * g.nkx + i) * g.my + j);
    dst[2 * t] = (R)pen[src];
    dst[2 * t + 1] = (R)pen[src + 1];
  }
}
template <typename R>
__global__ void k_plane_to_pencil(Grid g, const R *__restrict__ src, double *__restrict__ pen) {
  const long n = (long)g.my * g.nkx * g.mz;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const int j = (int)(t % g.my);
    const int i = (int)((t / g.my) % g.nkx);
    const int k = (int)(t / ((long)g.my * g.nkx));
    const long s = 2 * (((long)j * g.mz + k) * g.nkx + i);
    pen[2 * t] = (double)src[s];
    pen[2 * t + 1] = (double)src[s + 1];
  }
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
static const size_t kMaxSmem = 227 * 1024;  // opt-in shared memory per block

#if !SB_FLOAT_TU
// whether plane stage 3 with cb kx columns fits in shared memory (the
// temperature doubles its transforms)
bool plane3_fits(const Grid &g, int cb) {
  const size_t v = g.prec ? 8 : 16;
  return v * 2 * ((g.temp ? 6 : 3) * (size_t)cb * g.mgalz) <= kMaxSmem;
}
int plane_cb(int) { return 8; }
int plane_t2_default(int mgalx) {
  switch (mgalx) {
    case 32: case 48: case 80: return 64;
    case 64: case 96: case 128: return 96;
    case 160: case 192: return 128;
    default: return 256;
  }
}
int les_cb(int mgalz) { return mgalz >= 192 ? 2 : 4; }
#endif

template <typename R, int NZ, int CB, int T, int T3>
static cudaError_t launch_p13(const Grid &g, const Bufs &bf, int rk, cudaStream_t st, int which,
                              bool prep) {
  typedef typename Vec2<R>::t V;
  const size_t sm1 = sizeof(V) * 2 * (2 * CB * NZ);
  const size_t sm3 = sizeof(V) * 2 * (3 * CB * NZ), sm3t = 2 * sm3;
  if (prep) {
    cudaFuncSetAttribute(k_p1<R, NZ, CB, T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
    cudaFuncSetAttribute(k_p1<R, NZ, CB, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
    if (sm3 <= kMaxSmem)  // plane3_fits keeps the step off the blocks that do not fit
      cudaFuncSetAttribute(k_p3<R, NZ, CB, T3, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    if (sm3t <= kMaxSmem)
      cudaFuncSetAttribute(k_p3<R, NZ, CB, T3, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3t);
    return cudaGetLastError();
  }
  // stage-1 rounds: 3 field pairs, 2 more with LES, the temperature alone
  const int rounds = 3 + (g.les ? 2 : 0) + (g.temp ? 1 : 0);
  if (which == 1 && g.temp)
    k_p1<R, NZ, CB, T, true><<<dim3(g.ncb * rounds, g.my, g.B), T, sm1, st>>>(g, bf, rk);
  else if (which == 1)
    k_p1<R, NZ, CB, T, false><<<dim3(g.ncb * rounds, g.my, g.B), T, sm1, st>>>(g, bf, rk);
  else if (g.temp)
    k_p3<R, NZ, CB, T3, 6><<<dim3(g.ncb3, g.my, g.B), T3, sm3t, st>>>(g, bf);
  else
    k_p3<R, NZ, CB, T3, 3><<<dim3(g.ncb3, g.my, g.B), T3, sm3, st>>>(g, bf);
  return cudaGetLastError();
}

// plane stages 1, 3 with the tuned column block (4 or 8 kx columns)
template <typename R, int NZ>
static cudaError_t launch_p13_cb(const Grid &g, const Bufs &bf, int rk, cudaStream_t st, int which,
                                 bool prep) {
  if (prep) {
    cudaError_t e = launch_p13<R, NZ, 8, 128, 96>(g, bf, rk, st, which, true);
    return e != cudaSuccess ? e : launch_p13<R, NZ, 4, 128, 96>(g, bf, rk, st, which, true);
  }
  const int cb = (which == 1) ? g.cb1 : g.cb3;
  return cb == 4 ? launch_p13<R, NZ, 4, 128, 96>(g, bf, rk, st, which, false)
                 : launch_p13<R, NZ, 8, 128, 96>(g, bf, rk, st, which, false);
}

template <typename R, int NX, int T>
static cudaError_t launch_p2(const Grid &g, const Bufs &bf, int rk, cudaStream_t st, bool prep) {
  typedef typename Vec2<R>::t V;
  dim3 grid(g.mgalz / 2, g.my, g.B);
  const size_t sm = sizeof(V) * 2 * (6 * NX), smt = sizeof(V) * 2 * (7 * NX);
  if (prep) {
    cudaFuncSetAttribute(k_p2<R, NX, T, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_p2<R, NX, T, 7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt);
    return cudaGetLastError();
  }
  if (g.temp)
    k_p2<R, NX, T, 7><<<grid, T, smt, st>>>(g, bf, rk);
  else
    k_p2<R, NX, T, 6><<<grid, T, sm, st>>>(g, bf, rk);
  return cudaGetLastError();
}

// plane stage 2 with the tuned block size: T0 threads or 2 T0
template <typename R, int NX, int T0>
static cudaError_t launch_p2_t(const Grid &g, const Bufs &bf, int rk, cudaStream_t st, bool prep) {
  if (prep) {
    cudaError_t e = launch_p2<R, NX, T0>(g, bf, rk, st, true);
    return e != cudaSuccess ? e : launch_p2<R, NX, 2 * T0>(g, bf, rk, st, true);
  }
  return g.t2 == 2 * T0 ? launch_p2<R, NX, 2 * T0>(g, bf, rk, st, false)
                        : launch_p2<R, NX, T0>(g, bf, rk, st, false);
}

template <typename R>
static cudaError_t launch_plane_t(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st) {
  const bool prep = (stage == 0);
  if (stage == 2 || prep) {
    cudaError_t e;
    switch (g.mgalx) {
      case 32: e = launch_p2_t<R, 32, 64>(g, bf, rk, st, prep); break;
      case 48: e = launch_p2_t<R, 48, 64>(g, bf, rk, st, prep); break;
      case 64: e = launch_p2_t<R, 64, 96>(g, bf, rk, st, prep); break;
      case 80: e = launch_p2_t<R, 80, 64>(g, bf, rk, st, prep); break;
      case 96: e = launch_p2_t<R, 96, 96>(g, bf, rk, st, prep); break;
      case 128: e = launch_p2_t<R, 128, 96>(g, bf, rk, st, prep); break;
      case 160: e = launch_p2_t<R, 160, 128>(g, bf, rk, st, prep); break;
      case 192: e = launch_p2_t<R, 192, 128>(g, bf, rk, st, prep); break;
      case 256: e = launch_p2_t<R, 256, 256>(g, bf, rk, st, prep); break;
      case 320: e = launch_p2_t<R, 320, 256>(g, bf, rk, st, prep); break;
      case 384: e = launch_p2_t<R, 384, 256>(g, bf, rk, st, prep); break;
      default: return cudaErrorInvalidValue;
    }
    if (!prep || e != cudaSuccess) return e;
  }
  switch (g.mgalz) {
    case 32: return launch_p13_cb<R, 32>(g, bf, rk, st, stage, prep);
    case 48: return launch_p13_cb<R, 48>(g, bf, rk, st, stage, prep);
    case 64: return launch_p13_cb<R, 64>(g, bf, rk, st, stage, prep);
    case 80: return launch_p13_cb<R, 80>(g, bf, rk, st, stage, prep);
    case 96: return launch_p13_cb<R, 96>(g, bf, rk, st, stage, prep);
    case 128: return launch_p13_cb<R, 128>(g, bf, rk, st, stage, prep);
    case 160: return launch_p13_cb<R, 160>(g, bf, rk, st, stage, prep);
    case 192: return launch_p13_cb<R, 192>(g, bf, rk, st, stage, prep);
    case 256: return launch_p13_cb<R, 256>(g, bf, rk, st, stage, prep);
    case 384: return launch_p13_cb<R, 384>(g, bf, rk, st, stage, prep);
    default: return cudaErrorInvalidValue;
  }
}

// LES launches: stage 2..5 = k_les2..k_les5 of substep rk; stage 0 sets the
// kernels' shared-memory limits
template <typename R, int NX, int T>
static cudaError_t launch_les_x(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st,
                                bool prep) {
  typedef typename Vec2<R>::t V;
  dim3 grid(g.mgalz / 2, g.my, g.B);
  const size_t sm = sizeof(V) * 2 * (6 * NX);
  if (prep) {
    cudaFuncSetAttribute(k_les2<R, NX, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(k_les4<R, NX, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    return cudaGetLastError();
  }
  if (stage == 2)
    k_les2<R, NX, T><<<grid, T, sm, st>>>(g, bf);
  else
    k_les4<R, NX, T><<<grid, T, sm, st>>>(g, bf, rk);
  return cudaGetLastError();
}

template <typename R, int NZ, int CB>
static cudaError_t launch_les_z(const Grid &g, const Bufs &bf, int stage, cudaStream_t st,
                                bool prep) {
  typedef typename Vec2<R>::t V;
  const size_t sm3 = sizeof(V) * 2 * (8 * NZ), sm5 = sizeof(V) * 2 * (6 * CB * NZ);
  if (prep) {
    cudaFuncSetAttribute(k_les3<R, NZ, 8, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    cudaFuncSetAttribute(k_les5<R, NZ, CB, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm5);
    return cudaGetLastError();
  }
  if (stage == 3)
    k_les3<R, NZ, 8, 128><<<dim3((g.nkx + 7) / 8, g.my, g.B), 128, sm3, st>>>(g, bf);
  else
    k_les5<R, NZ, CB, 128><<<dim3(g.ncbl, g.my, g.B), 128, sm5, st>>>(g, bf);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_les_t(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st) {
  const bool prep = (stage == 0);
  if (prep || stage == 2 || stage == 4) {
    cudaError_t e;
    switch (g.mgalx) {
      case 32: e = launch_les_x<R, 32, 64>(g, bf, stage, rk, st, prep); break;
      case 48: e = launch_les_x<R, 48, 64>(g, bf, stage, rk, st, prep); break;
      case 64: e = launch_les_x<R, 64, 96>(g, bf, stage, rk, st, prep); break;
      case 96: e = launch_les_x<R, 96, 96>(g, bf, stage, rk, st, prep); break;
      case 80: e = launch_les_x<R, 80, 64>(g, bf, stage, rk, st, prep); break;
      case 128: e = launch_les_x<R, 128, 96>(g, bf, stage, rk, st, prep); break;
      case 160: e = launch_les_x<R, 160, 128>(g, bf, stage, rk, st, prep); break;
      case 192: e = launch_les_x<R, 192, 128>(g, bf, stage, rk, st, prep); break;
      case 256: e = launch_les_x<R, 256, 256>(g, bf, stage, rk, st, prep); break;
      case 320: e = launch_les_x<R, 320, 256>(g, bf, stage, rk, st, prep); break;
      case 384: e = launch_les_x<R, 384, 256>(g, bf, stage, rk, st, prep); break;
      default: return cudaErrorInvalidValue;
    }
    if (!prep || e != cudaSuccess) return e;
  }
  switch (g.mgalz) {
    case 32: return launch_les_z<R, 32, 4>(g, bf, stage, st, prep);
    case 48: return launch_les_z<R, 48, 4>(g, bf, stage, st, prep);
    case 64: return launch_les_z<R, 64, 4>(g, bf, stage, st, prep);
    case 80: return launch_les_z<R, 80, 4>(g, bf, stage, st, prep);
    case 96: return launch_les_z<R, 96, 4>(g, bf, stage, st, prep);
    case 128: return launch_les_z<R, 128, 4>(g, bf, stage, st, prep);
    case 160: return launch_les_z<R, 160, 4>(g, bf, stage, st, prep);
    case 192: return launch_les_z<R, 192, 2>(g, bf, stage, st, prep);
    case 256: return launch_les_z<R, 256, 2>(g, bf, stage, st, prep);
    case 384: return launch_les_z<R, 384, 2>(g, bf, stage, st, prep);
    default: return cudaErrorInvalidValue;
  }
}


// y dealiasing of substep rk: the mean-profile kernel (offsets, frame shift)
// then the line kernel
template <typename R, int MY>
static cudaError_t launch_ydeal_t(const Grid &g, const Bufs &bf, int rk, cudaStream_t st, bool prep) {
  typedef typename Vec2<R>::t V;
  constexpr int CB = MY <= 96 ? 16 : (MY == 192 ? 8 : 4);
  const size_t sm = sizeof(V) * 2 * CB * MY;
  if (prep) {
    cudaFuncSetAttribute(k_ydeal<R, MY, CB, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    return cudaGetLastError();
  }
  k_ydeal_mean<R, MY, 128><<<g.B, 128, 0, st>>>(g, bf, rk);
  const int nb = (g.ydeal == 1) ? 1 : (g.nkx + CB - 1) / CB;
  k_ydeal<R, MY, CB, 128><<<dim3(nb, g.mz, 2 * g.B), 128, sm, st>>>(g, bf);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_ydeal_r(const Grid &g, const Bufs &bf, int rk, cudaStream_t st, bool prep) {
  switch (g.my) {
    case 32: return launch_ydeal_t<R, 32>(g, bf, rk, st, prep);
    case 48: return launch_ydeal_t<R, 48>(g, bf, rk, st, prep);
    case 64: return launch_ydeal_t<R, 64>(g, bf, rk, st, prep);
    case 80: return launch_ydeal_t<R, 80>(g, bf, rk, st, prep);
    case 96: return launch_ydeal_t<R, 96>(g, bf, rk, st, prep);
    case 128: return launch_ydeal_t<R, 128>(g, bf, rk, st, prep);
    case 160: return launch_ydeal_t<R, 160>(g, bf, rk, st, prep);
    case 192: return launch_ydeal_t<R, 192>(g, bf, rk, st, prep);
    case 256: return launch_ydeal_t<R, 256>(g, bf, rk, st, prep);
    case 320: return launch_ydeal_t<R, 320>(g, bf, rk, st, prep);
    case 384: return launch_ydeal_t<R, 384>(g, bf, rk, st, prep);
    default: return cudaErrorInvalidValue;
  }
}

#if !SB_FLOAT_TU
bool supported_ylen(int my) {
  const int ys[] = {32, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384};
  for (int v : ys)
    if (v == my) return true;
  return false;
}

template <int MY>
static cudaError_t launch_yop_t(int nlines, double *c, long ldc, int iopt, int real, cudaStream_t st) {
  constexpr int CB = MY <= 96 ? 4 : (MY == 192 ? 2 : 1);
  k_yop<MY, CB, 128><<<(nlines + CB - 1) / CB, 128, 0, st>>>(nlines, c, ldc, iopt, real);
  return cudaGetLastError();
}

cudaError_t launch_yop(int my, int nlines, double *c, long ldc, int iopt, int real, cudaStream_t st) {
  switch (my) {
    case 32: return launch_yop_t<32>(nlines, c, ldc, iopt, real, st);
    case 48: return launch_yop_t<48>(nlines, c, ldc, iopt, real, st);
    case 64: return launch_yop_t<64>(nlines, c, ldc, iopt, real, st);
    case 80: return launch_yop_t<80>(nlines, c, ldc, iopt, real, st);
    case 96: return launch_yop_t<96>(nlines, c, ldc, iopt, real, st);
    case 128: return launch_yop_t<128>(nlines, c, ldc, iopt, real, st);
    case 160: return launch_yop_t<160>(nlines, c, ldc, iopt, real, st);
    case 192: return launch_yop_t<192>(nlines, c, ldc, iopt, real, st);
    case 256: return launch_yop_t<256>(nlines, c, ldc, iopt, real, st);
    case 320: return launch_yop_t<320>(nlines, c, ldc, iopt, real, st);
    case 384: return launch_yop_t<384>(nlines, c, ldc, iopt, real, st);
    default: return cudaErrorInvalidValue;
  }
}


// FP64 FMA throughput probe: eight independent chains per thread
__global__ void k_fp64_probe(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int it = 0; it < iters; it++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t fp64_peak(double *tflops, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 512, blocks = 2 * sms, iters = 20000;
  double *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * threads * blocks);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_probe<<<blocks, threads, 0, st>>>(d, 100, 0.999, 0.001);
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0, st);
    k_fp64_probe<<<blocks, threads, 0, st>>>(d, iters, 0.999, 0.001);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  *tflops = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3) / 1e12;
  return e;
}

bool supported_grid(int mgalx, int mgalz) {
  const int xs[] = {32, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384};
  const int zs[] = {32, 48, 64, 80, 96, 128, 160, 192, 256, 384};
  bool okx = false, okz = false;
  for (int v : xs) okx |= (v == mgalx);
  for (int v : zs) okz |= (v == mgalz);
  return okx && okz;
}
#endif  // !SB_FLOAT_TU

// ---------------------------------------------------------------------------
// Physical fields of the post-processor convh5 (hvhg_uvwp, convh5.f90:650-933)
// from the z-transforms of k_p1 run with the LES rounds (zbuf fields 0 u, 1 w,
// 2 omega_x, 3 omega_z, 4 v, 5 omega_y, 6 dv/dy, 7 i kz w, 8 2 i kz v +
// omega_x, 9 i kz u): per (plane, z row pair), the velocity with the laminar
// shear s y, the vorticity (omega_z with -s) and the nine velocity gradients
// to physical x, then the selected outputs (mask bits 0..10: u v w ox oy oz
// Q R Qs Rs Qw), each [my][mgalz][mgalx] in FP64.
// ---------------------------------------------------------------------------
template <typename R, int NX, int T>
__global__ void __launch_bounds__(T) k_phys(Grid g, Bufs bf, unsigned mask, double *out) {
  typedef typename Vec2<R>::t V;
  const int zp = blockIdx.x, j = blockIdx.y;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *A = (V *)smem_raw, *Bs = A + 15 * NX;
  const int nkx = g.nkx, NZ = g.mgalz, nzf = g.nzf;
  const int z = 2 * zp;
  const V *zb = (const V *)bf.zbuf + (long)j * NZ * nzf * nkx;
  const V zero = mk2<R>((R)0, (R)0);
  for (int idx = threadIdx.x; idx < 15 * NX; idx += T) A[idx] = zero;
  __syncthreads();
  // 0 u, 1 v, 2 w, 3 ox, 4 oy, 5 oz, 6 ux, 7 uy, 8 uz, 9 vx, 10 vy, 11 vz,
  // 12 wx, 13 wy, 14 wz (convh5.f90:801-831)
  for (int idx = threadIdx.x; idx < 15 * nkx; idx += T) {
    const int f = idx / nkx, i = idx - f * nkx;
    const R a = (R)(g.alp * i);
    V X[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const V *row = zb + (long)(z + r) * nzf * nkx;
      const V u = row[i], w = row[nkx + i], ox = row[2 * nkx + i], oz = row[3 * nkx + i],
              v = row[4 * nkx + i];
      V x;
      switch (f) {
        case 0: x = u; break;
        case 1: x = v; break;
        case 2: x = w; break;
        case 3: x = ox; break;
        case 4: x = row[5 * nkx + i]; break;
        case 5: x = oz; break;
        case 6: x = mk2<R>(-a * u.y, a * u.x); break;
        case 7: x = mk2<R>(-a * v.y - oz.x, a * v.x - oz.y); break;
        case 8: x = row[9 * nkx + i]; break;
        case 9: x = mk2<R>(-a * v.y, a * v.x); break;
        case 10: x = row[6 * nkx + i]; break;
        case 11: {
          const V t = row[8 * nkx + i];
          x = mk2<R>((R)0.5 * (t.x - ox.x), (R)0.5 * (t.y - ox.y));
          break;
        }
        case 12: x = mk2<R>(-a * w.y, a * w.x); break;
        case 13: {
          const V t = row[8 * nkx + i];
          x = mk2<R>((R)0.5 * (t.x - ox.x) + ox.x, (R)0.5 * (t.y - ox.y) + ox.y);
          break;
        }
        default: x = row[7 * nkx + i]; break;
      }
      X[r] = x;
    }
    if (i == 0) {
      X[0].y = (R)0;
      X[1].y = (R)0;
    }
    A[f * NX + i] = mk2<R>(X[0].x - X[1].y, X[0].y + X[1].x);
    if (i > 0) A[f * NX + NX - i] = mk2<R>(X[0].x + X[1].y, -X[0].y + X[1].x);
  }
  V *P = fft_batch<NX, +1, 15, T>(A, Bs, (const V *)tw_of<R>(bf, false));
  int slot[11], n = 0;
#pragma unroll
  for (int q = 0; q < 11; q++) slot[q] = (mask >> q & 1u) ? n++ : -1;
  const double s = g.s, sy = g.s * ((double)j * g.dy - 0.5 * g.Ly);
  const long pl = (long)NX * NZ;
  for (int x = threadIdx.x; x < NX; x += T) {
#pragma unroll
    for (int r = 0; r < 2; r++) {
      double U[15];
#pragma unroll
      for (int q = 0; q < 15; q++) U[q] = r ? (double)P[q * NX + x].y : (double)P[q * NX + x].x;
      U[0] += sy;  // laminar shear (convh5.f90:755-758)
      U[5] -= s;
      U[7] += s;
      const double ux = U[6], uy = U[7], uz = U[8], vx = U[9], vy = U[10], vz = U[11],
                   wx = U[12], wy = U[13], wz = U[14];
      double val[11];
#pragma unroll
      for (int q = 0; q < 6; q++) val[q] = U[q];
      val[6] = -0.5 * (ux * ux + vy * vy + wz * wz + 2.0 * (vz * wy + uy * vx + uz * wx));
      val[7] = -(ux * (vy * wz - wy * vz) - uy * (vx * wz - wx * vz) + uz * (vx * wy - wx * vy));
      const double s12 = 0.5 * (uy + vx), s23 = 0.5 * (vz + wy), s13 = 0.5 * (uz + wx);
      val[8] = -0.5 * (ux * ux + vy * vy + wz * wz) - (s12 * s12 + s13 * s13 + s23 * s23);
      val[9] = -(s12 * s23 * s13 + ux * (s12 * s12 + s13 * s13) + vy * (s12 * s12 + s23 * s23) +
                 wz * (s13 * s13 + s23 * s23) + ux * vy * wz);
      val[10] = 0.25 * (U[3] * U[3] + U[4] * U[4] + U[5] * U[5]);
#pragma unroll
      for (int q = 0; q < 11; q++)
        if (slot[q] >= 0) out[((long)slot[q] * g.my + j) * pl + (long)(z + r) * NX + x] = val[q];
    }
  }
}

template <typename R, int NX, int T>
static cudaError_t launch_phys_t(const Grid &g, const Bufs &bf, unsigned mask, double *out,
                                 cudaStream_t st) {
  typedef typename Vec2<R>::t V;
  const size_t sm = sizeof(V) * 2 * 15 * NX;
  cudaFuncSetAttribute(k_phys<R, NX, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_phys<R, NX, T><<<dim3(g.mgalz / 2, g.my), T, sm, st>>>(g, bf, mask, out);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_phys_r(const Grid &g, const Bufs &bf, unsigned mask, double *out,
                                 cudaStream_t st) {
  switch (g.mgalx) {
    case 32: return launch_phys_t<R, 32, 64>(g, bf, mask, out, st);
    case 48: return launch_phys_t<R, 48, 64>(g, bf, mask, out, st);
    case 64: return launch_phys_t<R, 64, 96>(g, bf, mask, out, st);
    case 80: return launch_phys_t<R, 80, 64>(g, bf, mask, out, st);
    case 96: return launch_phys_t<R, 96, 96>(g, bf, mask, out, st);
    case 128: return launch_phys_t<R, 128, 96>(g, bf, mask, out, st);
    case 160: return launch_phys_t<R, 160, 128>(g, bf, mask, out, st);
    case 192: return launch_phys_t<R, 192, 128>(g, bf, mask, out, st);
    case 256: return launch_phys_t<R, 256, 256>(g, bf, mask, out, st);
    case 320: return launch_phys_t<R, 320, 256>(g, bf, mask, out, st);
    case 384: return launch_phys_t<R, 384, 256>(g, bf, mask, out, st);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
static cudaError_t launch_spectra_t(const Grid &g, const Bufs &bf, cudaStream_t st) {
  const int nl = g.nkx * g.mz;
  const dim3 grid((unsigned)((nl + kSpecModes - 1) / kSpecModes), (unsigned)g.B);
  const int T = kSpecModes * kSpecSlices;
  if (g.temp)
    k_spectra<R, true><<<grid, T, 0, st>>>(g, bf);
  else
    k_spectra<R, false><<<grid, T, 0, st>>>(g, bf);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_p2p_t(const Grid &g, const double *pen, double *dst, cudaStream_t st) {
  k_pencil_to_plane<R><<<256, 256, 0, st>>>(g, pen, (R *)dst);
  return cudaGetLastError();
}
template <typename R>
static cudaError_t launch_pen_t(const Grid &g, const double *src, double *pen, cudaStream_t st) {
  k_plane_to_pencil<R><<<256, 256, 0, st>>>(g, (const R *)src, pen);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// entry points: the FP32-mixed instantiations come from the second
// compilation of this file (SB_FLOAT_TU=1), the rest from the first
// ---------------------------------------------------------------------------
cudaError_t plane_f32(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st);
cudaError_t les_f32(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st);
cudaError_t ydeal_f32(const Grid &g, const Bufs &bf, int rk, cudaStream_t st);
cudaError_t p2p_f32(const Grid &g, const double *pen, double *dst, cudaStream_t st);
cudaError_t pen_f32(const Grid &g, const double *src, double *pen, cudaStream_t st);
cudaError_t phys_f32(const Grid &g, const Bufs &bf, unsigned mask, double *out, cudaStream_t st);
cudaError_t spectra_f32(const Grid &g, const Bufs &bf, cudaStream_t st);

#if SB_FLOAT_TU
cudaError_t plane_f32(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st) {
  return launch_plane_t<float>(g, bf, stage, rk, st);
}
cudaError_t les_f32(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st) {
  return launch_les_t<float>(g, bf, stage, rk, st);
}
cudaError_t ydeal_f32(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  return launch_ydeal_r<float>(g, bf, rk, st, rk == 0);
}
cudaError_t p2p_f32(const Grid &g, const double *pen, double *dst, cudaStream_t st) {
  return launch_p2p_t<float>(g, pen, dst, st);
}
cudaError_t pen_f32(const Grid &g, const double *src, double *pen, cudaStream_t st) {
  return launch_pen_t<float>(g, src, pen, st);
}
cudaError_t phys_f32(const Grid &g, const Bufs &bf, unsigned mask, double *out, cudaStream_t st) {
  return launch_phys_r<float>(g, bf, mask, out, st);
}
cudaError_t spectra_f32(const Grid &g, const Bufs &bf, cudaStream_t st) {
  return launch_spectra_t<float>(g, bf, st);
}
#else
// stage 1..3: launch; stage 0: set the kernels' shared-memory limits (once)
cudaError_t launch_plane(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st) {
  return g.prec ? plane_f32(g, bf, stage, rk, st) : launch_plane_t<double>(g, bf, stage, rk, st);
}
cudaError_t launch_les(const Grid &g, const Bufs &bf, int stage, int rk, cudaStream_t st) {
  return g.prec ? les_f32(g, bf, stage, rk, st) : launch_les_t<double>(g, bf, stage, rk, st);
}
// rk = 1..3: launch; rk = 0: set the kernels' shared-memory limits
cudaError_t launch_ydeal(const Grid &g, const Bufs &bf, int rk, cudaStream_t st) {
  return g.prec ? ydeal_f32(g, bf, rk, st) : launch_ydeal_r<double>(g, bf, rk, st, rk == 0);
}
cudaError_t launch_pencil_to_plane(const Grid &g, const double *pen, double *dst, cudaStream_t st) {
  return g.prec ? p2p_f32(g, pen, dst, st) : launch_p2p_t<double>(g, pen, dst, st);
}
cudaError_t launch_plane_to_pencil(const Grid &g, const double *src, double *pen, cudaStream_t st) {
  return g.prec ? pen_f32(g, src, pen, st) : launch_pen_t<double>(g, src, pen, st);
}
cudaError_t launch_spectra(const Grid &g, const Bufs &bf, cudaStream_t st) {
  return g.prec ? spectra_f32(g, bf, st) : launch_spectra_t<double>(g, bf, st);
}
// one box (Grid with B = 1 and member-offset buffers): plane stage 1 with the
// extra z-transforms into g's zbuf, then the physical fields
cudaError_t launch_physical(const Grid &g, const Bufs &bf, unsigned mask, double *out,
                            cudaStream_t st) {
  cudaError_t e = launch_plane(g, bf, 1, 2, st);
  if (e != cudaSuccess) return e;
  return g.prec ? phys_f32(g, bf, mask, out, st) : launch_phys_r<double>(g, bf, mask, out, st);
}
#endif

}  // namespace sb
