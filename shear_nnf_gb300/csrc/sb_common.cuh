// sb_common.cuh -- shared device types for the shearing-box RK3 step on GB300.
//
// Device layout of one spectral field of one box ("plane-major"):
//   f[j][k][i] complex (re, im interleaved doubles), i = kx index fastest
//   (0..nkx-1), k = kz index (0..mz-1, reference ordering: 0..nz positive,
//   nz+1..mz-1 negative), j = y plane (0..my-1).  A batch of B boxes is
//   [b][j][k][i].  The y-line kernels read one double per thread per plane
//   (coalesced across kx), the plane kernels read contiguous planes, so the
//   reference's plane<->pencil transposes (change.allfac_ieor.f) disappear.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define SB_TRACE_LEN 24
#define SB_TRACE_LEN_T 29  // with the temperature: + tbmax, tner(1:4)
#define SB_NHIST_Q 15   // per-plane hist partial sums (11, then 4 of the temperature)
#define SB_MAX_NY 512
#define SB_TAIL 24      // doubles per stored shear tail

namespace sb {

struct cd {
  double x, y;
};
__host__ __device__ __forceinline__ cd mk(double a, double b) { cd z; z.x = a; z.y = b; return z; }
__host__ __device__ __forceinline__ cd operator+(cd a, cd b) { return mk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cd operator-(cd a, cd b) { return mk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cd operator*(cd a, cd b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ cd operator*(double r, cd a) { return mk(r * a.x, r * a.y); }
__host__ __device__ __forceinline__ cd cj(cd a) { return mk(a.x, -a.y); }
__host__ __device__ __forceinline__ double abs2(cd a) { return a.x * a.x + a.y * a.y; }

// Factor tables of one cyclic Hermitian heptadiagonal LDL^H factorisation with
// the shear phase factored out (see sb_factor.cpp).  Arrays are indexed
// [q * stride + line] with q the 0-based row; stride = 0 for the operators that
// are the same on every line (d/dy, d2/dy2).
struct Fac {
  const double *La, *Lb, *Lc, *Ddm1, *e, *f, *g;  // my entries each
  const double *Dd;    // my entries (rows my-8 .. my-4 are read)
  const double *sums;  // 10 entries: See Sfe Sff Sge Sgf Sgg, then a(0..3)
  const double *hf[3], *hb[3];  // segment homogeneous solutions (my entries each)
  const double *ef;             // segment border sums (9 per segment)
  // the same per row and line, interleaved for the segmented solve
  // (sb_seg.cuh): 16 doubles at rows[((row-1) * lines + line) * 16]
  const double *rows;
  long stride;                  // lines of a per-line factor (0: one for all lines)
};

// Constant per-handle parameters (passed by value to every kernel)
struct Grid {
  int B, mgalx, my, mgalz, mx, mz, nkx, nz, mgx;
  int prec;              // 0: FP64 throughout; 1: FP32-mixed (FP32 storage/transforms)
  int ncb;               // kx column blocks per plane of plane stage 1 (hist partials)
  int cb1, cb3, ncb3;    // kx columns per block of plane stages 1 and 3, stage-3 blocks
  int t2;                // threads per block of plane stage 2
  double alp, gam, Ly, s, chi, dx, dy, dz, pi;
  double rh1[7], rh2[7], pr2[7];
  long plane;            // doubles per plane of one field  (2*nkx*mz)
  long field;            // doubles per field of one box   (plane*my)
  int nlines_pad;        // component lines per member, padded to whole warps
  int nseg, slo[4], shi[4];  // segments of the banded rows of the y-solves
  int lform;             // y-line kernels of a substep: 0 k_lineA + k_lineB, 1 k_lineF
  int impl;              // 1: semi-implicit viscous terms (explicit = 0): k_hfac + k_lineI
  int ngrp;              // groups of 16 lines per member in the y-line kernels
  // Smagorinsky LES (cross.f90:1291-1406): on/off, molecular viscosity kept,
  // (Cles * Deltag)^2, fields per z row of zbuf (6, or 10 with the model),
  // kx columns per block of the LES column kernel and their count
  int les, les_visc, nzf, cbl, ncbl;
  double les_c;
  // compact y-filter (iydealiasing = 3): on/off and the symmetric 9-point
  // right-hand side frh[0..4] (filter_shear_hepta.f90:64-73)
  int ydeal;
  double frh[5];
  // y dealiasing (iydealiasing 1, 2; dealiasing_y, operators.f90:352-467):
  // 2/3-rule cut indices (initcr.f90:207-210) and Lx
  int my23, ny1, ny2;
  double Lx;
  // Boussinesq scalar of crosst (itemperature): on/off, k_p1 round of its
  // z-transform, its zbuf field, fields per z row of xbuf (3, or 6 with the
  // fluxes uT wT vT), trace record length; diffusivity and buoyancy factor
  // (zero when an LES run drops the molecular terms, crosst.f90:717-757) and
  // the mean gradient
  int temp, tround, tzf, nxf, tlen;
  double kappa, gbeta, bym;
  // window damping of the mean forcing rf0u (iadd_damping, add_damping):
  // on/off, permeability damp_up, half width aa = Lz damp_aa, Lz
  int damp;
  double damp_up, damp_a, lz;
  // body forces (iadd_force): 1, 2 the streamwise-roll force on hv(kx=0,
  // kz=1) with amplitude force_roll; -1 the inertial force xforce on rf0u
  int force;
  double force_roll, xforce;
};

// Per-member run state, owned by the device (one per box in the batch)
struct Member {
  // parameters
  double Re, nu, CFL, cflx, cfly, cflz, cflvv, vbulk, fixed_dt, uprim;
  double etime, dumptime, dtimag;
  int readflag, nhist, keep_laminar;
  // state scalars
  double time, xoffb, xofft;
  double xwb[4], xwt[4];      // image offsets: [0] at the step start, [rk] after substep rk
  double Deltat, CFLcur, CFLv;
  double umax[4];
  unsigned long long umax_bits[4];  // |u| maxima as ordered bit patterns (atomicMax)
  unsigned long long nut_bits;      // LES: max |nu_t| of this step (bit pattern)
  double max_nut;                   // LES: running maximum of |nu_t| (cross.f90:1433)
  double ydfac;                     // y dealiasing: moving-frame shift of this substep
  double cflkk;                     // temperature: thermal-diffusion CFL factor (initcr.f90:498-502)
  double tbmax;                     // temperature: max |tb| of this step
  unsigned long long tbmax_bits;
  double total_dt;                  // statistics: summed Delta t of the records (cross.f90:2072)
  int nacum;                        // statistics: records accumulated in this call
  int istop, idump, ihist, istep, halted, ntrace, trace_cap, flags;
};

enum { SBF_DIVERGED = 1, SBF_NAN = 2, SBF_LAMINAR = 4, SBF_ETIME = 8 };

// RK3 coefficients of the low-storage Spalart-Moser-Rogers scheme
// (cross.f90:17-24)
__device__ __constant__ static const double kGama[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
__device__ __constant__ static const double kZeta[3] = {-17.0 / 60.0, -5.0 / 12.0, 0.0};
__device__ __constant__ static const double kCa[3] = {8.0 / 15.0, 2.0 / 3.0, 1.0};

// Device arrays of one handle
struct Bufs {
  // spectral fields [B][field], FP64 or FP32 storage (Grid::prec); the
  // pointers are typed double for bookkeeping and cast by the kernels
  double *vor, *phi, *vorwk, *phiwk, *G, *V, *D;
  double *T, *S;                 // d/dy of the NL term and d2(phi)/dy2 between the line kernels
  double *Lv;                    // d2(omega_y)/dy2 of the next substep's starting state
  double *mu, *mwk, *mrf, *mdu;  // mean lines (u00 + i w00) [B][my] complex
  double *zbuf, *xbuf;           // plane-stage intermediates
  double *hpart;                 // hist partials [B][my][blocks of k_spectra][SB_NHIST_Q]
  double *hsum;                  // their plane sums, + hist 'p' and LES sums [B][my][SB_NHIST_Q + 5]
  double *sh_old, *sh_new;       // [B][2][nkx] complex (t then b)
  double *tl1o, *tl2o, *tl1n, *tl2n;  // shear tails of d/dy, d2/dy2 at the old and new phases [B][nkx][SB_TAIL]
  double *mf1, *mf2;             // moving-frame phases [B][my][nkx] complex
  double *trace;                 // [B][cap][SB_TRACE_LEN]
  Member *mem;                   // [B]
  const double *twz, *twx;       // FFT twiddles e^{-2 pi i t/N}, factored form (sb_fft.cuh)
  const float *twzf, *twxf;      // the same as complex values, rounded to FP32
  const float *kinvf;            // kinv rounded to FP32
  const double *ginv;            // 1/g per kz  (g = gam * kz_signed; 0 at k=0)
  const double *kinv;            // 1/(alp2+gam2) per (k,i); 0 at (0,0)
  Fac d1, d2, hz;                // d/dy, d2/dy2, Helmholtz (per line)
  Fac hi;                        // semi-implicit Helmholtz (k^2 + dtr1) per box and line
                                 // (kx, kz >= 0), then the mean line; rebuilt every substep
  Fac hit;                       // the same for the scalar of crosst (k^2 + dtr1k)
  Fac flt;                       // left-hand side of the compact y-filter
  const double *twy;             // y-transform twiddles (iydealiasing 1, 2), factored form
  const float *twyf;
  // LES buffers: physical gradient rows [B][my][mgalz/2][6][2][mgalx], |S|^2
  // x-spectra [B][my][mgalz][nkx], stress x-spectra [B][my][mgalz][6][nkx],
  // rhvc2 and rhgc2 fields, T12/T23 of the (0,0) mode [B][my] complex, plane
  // partial sums of nu_t and nu_t |S|^2 [B][my][mgalz/2][2]
  double *gbuf, *sbuf, *tbuf, *L1, *L2, *txy, *lpart;
  // temperature: tb and its RK work array, the right-hand side ht (plane
  // stage: -d(uT)/dx - d(wT)/dz - bym v, then += d(-vT)/dy), -vT, the
  // Laplacian of tb (d2/dy2 - k^2) tb; mean profile tb00 [B][my] complex (re),
  // its RK work array and d(-vT_00)/dy
  double *tb, *tbwk, *Ht, *R2, *Lt, *mt, *mtwk, *mtr;
  // statistics accumulated by hist over one call (module statistics,
  // mod.f90:94-115): stats, stats2 [B][my][23]; spectra spl, spl2
  // [B][mz][nkx][8]; temperature tstats [B][my][5], splt [B][mz][nkx][4];
  // hist 'p' partials [B][my][mgalz/2][warps of a stage-2 block][3]
  double *stats, *stats2, *spec, *spec2, *tstats, *tspec, *ppart;
};

// Asynchronous global -> shared copy of one element of NB bytes (4, 8 or 16,
// both addresses NB-aligned); with `valid` false the shared element is
// zero-filled and nothing is read.  Completed by cp_async_wait_all().
template <int NB>
__device__ __forceinline__ void cp_async(void *smem_dst, const void *gmem_src, bool valid) {
  static_assert(NB == 4 || NB == 8 || NB == 16, "cp.async element size");
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  const int n = valid ? NB : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(gmem_src),
               "n"(NB), "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

}  // namespace sb
