// sb_api.cu -- C-ABI of the shearing-box time stepper (see include/shearbox.h).
//
// Host side of the step: owns the device state of a batch of boxes, uploads
// the factor tables computed by sb_host.cpp, captures one RK3 step (sixteen
// kernel launches) in a CUDA graph and replays it.  The reference's MPI/OpenMP
// structure (cross.f90 with change.allfac_ieor.f transposes) has no
// counterpart: one handle is one GPU, one stream.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/shearbox.h"
#include "sb_common.cuh"
#include "sb_fac.h"
#include "sb_host.h"
#include "sb_kernels.h"

using namespace sb;

static thread_local std::string g_err;
namespace sb {
void set_error(const std::string &msg) { g_err = msg; }
}
static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
#define CK(x)                                                                      \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess)                                                         \
      return fail(3, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

// largest my accepted by sb_create
constexpr int kMaxMy = 448;

struct sb_handle {
  sb_params p;
  int precision;
  Grid g;
  Bufs bf;
  cudaStream_t st = nullptr;
  // side branch of the step graph: the per-box scalars and phase tables run
  // beside plane stage 3, which they do not depend on
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // the spectra of a statistics step run beside plane stages 1-2
  cudaEvent_t ev_s0 = nullptr, ev_s1 = nullptr;
  // which side work the step graph runs as a concurrent branch: bit 0 the
  // spectra, bit 1 the scalars and tables (a cleared bit puts that work on
  // the main stream in order)
  int branch = 3;
  // the host copies of phi run on the side stream beside those of omega_y
  cudaEvent_t ev_c0 = nullptr, ev_c1 = nullptr;
  cudaGraphExec_t step_exec = nullptr;
  std::vector<void *> allocs;
  // the factor tables of the y-line solves depend on the segment plan: kept
  // apart so that a new plan (sb_set_line_segments, the autotuner) can
  // replace them
  std::vector<void *> line_allocs;
  std::vector<void *> *alloc_to = nullptr;
  double *d_pen = nullptr;  // staging buffers, one pencil-layout field each
  double *d_pen2 = nullptr;
  // pinned host staging of the small per-call values (mean profiles, time and
  // offsets, the member record), so that a cross call synchronises once
  struct HostSmall {
    double mu_in[2 * kMaxMy], mu_out[2 * kMaxMy], sc_in[3], sc_out[3];
    Member m;
  } *hs = nullptr;
  int trace_cap = 0;
  std::vector<Member> mem_init;
};

namespace sb {
// handle accessors for the host code of sb_newton.cpp
const sb_params *handle_params(const sb_handle *h) { return &h->p; }
int handle_batch(const sb_handle *h) { return h->g.B; }
int handle_trace_len(const sb_handle *h) { return h->g.tlen; }
}  // namespace sb

static int dalloc(sb_handle *h, double **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, sizeof(double) * (n ? n : 1));
  if (e != cudaSuccess) return fail(4, "cudaMalloc(%zu doubles): %s", n, cudaGetErrorString(e));
  cudaMemset(q, 0, sizeof(double) * (n ? n : 1));
  (h->alloc_to ? *h->alloc_to : h->allocs).push_back(q);
  *p = (double *)q;
  return 0;
}
static int upload(sb_handle *h, const double **dst, const std::vector<double> &v) {
  double *p = nullptr;
  int rc = dalloc(h, &p, v.size());
  if (rc) return rc;
  CK(cudaMemcpy(p, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice));
  *dst = p;
  return 0;
}

static int check_params(const sb_params *p) {
  if (p && (p->ydeal < 0 || p->ydeal > 3))
    return fail(2, "iydealiasing=%d not available (0..3)", p->ydeal);
  if (p && (p->ydeal == 1 || p->ydeal == 2) && !supported_ylen(p->my))
    return fail(2, "iydealiasing=%d needs my in 32,48,64,80,96,128,160,192,256,320,384 "
                   "(y transforms)", p->ydeal);
  if (!p) return fail(1, "null parameters");
  if (p->mgalx <= 0 || p->my <= 0 || p->mgalz <= 0)
    return fail(1, "mgalx grid error %d %d %d", p->mgalx, p->my, p->mgalz);  // initcr.f90:188
  if (!supported_grid(p->mgalx, p->mgalz))
    return fail(1, "unsupported x/z grid %d x %d (transform lengths 32,48,64,80,96,128,160,192,256,"
                   "384 and for x also 320)",
                p->mgalx, p->mgalz);
  if (p->mgalz % 2) return fail(1, "mgalz must be even");
  if (p->my < 16 || p->my > kMaxMy) return fail(1, "my=%d outside 16..%d", p->my, kMaxMy);
  if (p->temperature != 0 && p->temperature != 1)
    return fail(2, "itemperature=%d not available (0, 1)", p->temperature);
  if (p->damping != 0 && p->damping != 1)
    return fail(2, "iadd_damping=%d not available (0, 1)", p->damping);
  if (p->force < -1 || p->force > 2)
    return fail(2, "iadd_force=%d not available (-1, 0, 1, 2)", p->force);
  // plane stage 3 holds 3 (6 with the temperature) columns of mgalz points
  // in shared memory, at least 4 columns per block
  if (p->temperature && p->mgalz > 256)
    return fail(2, "itemperature=1 needs mgalz <= 256 (got %d)", p->mgalz);
  if (p->implicit_visc != 0 && p->implicit_visc != 1)
    return fail(2, "implicit_visc=%d not available (0, 1)", p->implicit_visc);
  // LES with explicit = 0 stops the reference (initcr.f90:2179-2182); the
  // semi-implicit kernels cover the plain step
  if (p->implicit_visc && (p->les || p->ydeal))
    return fail(2, "implicit_visc needs les = ydeal = 0");
  if (p->implicit_visc && p->temperature && !(p->fkappa > 0.0))
    return fail(2, "implicit_visc with the temperature needs fkappa > 0");
  if (!(p->Re != 0.0) || !(p->alp > 0) || !(p->gam > 0) || !(p->Ly > 0) || !(p->CFL > 0))
    return fail(1, "invalid physical parameters");
  return 0;
}

// interleaved row records of the segmented solve (Fac::rows, sb_seg.cuh):
// row q (0-based) of line `line` of `nl` at rows[(q * nl + line) * 16] =
// La Lb Lc e f g Dm 0 | hf1 hf2 hf3 0 | hb1 hb2 hb3 0
static void pack_rows(const sbh::BaseFac &b, const sbh::SegFac &sf, size_t n, size_t nl,
                      size_t line, std::vector<double> &rows) {
  for (size_t q = 0; q < n; q++) {
    double *r = &rows[(q * nl + line) * 16];
    r[0] = b.La[q];
    r[1] = b.Lb[q];
    r[2] = b.Lc[q];
    r[3] = b.e[q];
    r[4] = b.f[q];
    r[5] = b.g[q];
    r[6] = b.Ddm1[q];
    r[7] = 0.0;
    for (int t = 0; t < 3; t++) {
      r[8 + t] = sf.hf[t][q];
      r[12 + t] = sf.hb[t][q];
    }
    r[11] = r[15] = 0.0;
  }
}

// factor tables of one band matrix, same for every line
static int upload_uniform(sb_handle *h, Fac *F, const double a[7], int n) {
  sbh::BaseFac b;
  sbh::base_factor(a, n, &b);
  sbh::SegPlan plan;
  sbh::seg_plan(n, h->g.nseg, &plan);
  sbh::SegFac sf;
  sbh::seg_factor(b, n, plan, &sf);
  int rc;
  for (int t = 0; t < 3; t++)
    if ((rc = upload(h, &F->hf[t], sf.hf[t])) || (rc = upload(h, &F->hb[t], sf.hb[t]))) return rc;
  if ((rc = upload(h, &F->ef, sf.ef))) return rc;
  if ((rc = upload(h, &F->La, b.La)) || (rc = upload(h, &F->Lb, b.Lb)) ||
      (rc = upload(h, &F->Lc, b.Lc)) || (rc = upload(h, &F->Ddm1, b.Ddm1)) ||
      (rc = upload(h, &F->Dd, b.Dd)) || (rc = upload(h, &F->e, b.e)) ||
      (rc = upload(h, &F->f, b.f)) || (rc = upload(h, &F->g, b.g)))
    return rc;
  std::vector<double> s(10);
  for (int q = 0; q < 6; q++) s[q] = b.sums[q];
  for (int q = 0; q < 4; q++) s[6 + q] = a[3 + q];
  if ((rc = upload(h, &F->sums, s))) return rc;
  std::vector<double> rows(16 * (size_t)n);
  pack_rows(b, sf, (size_t)n, 1, 0, rows);
  if ((rc = upload(h, &F->rows, rows))) return rc;
  F->stride = 0;
  return 0;
}

// The factor tables of the y-line solves for a segment plan of nseg warps per
// line: d/dy and d2/dy2 (and the y-filter), each the same for every line, and
// the Helmholtz operator (rh2 - k^2 pr2) per (kx, kz >= 0) line (lapcdy,
// diffy_shear_hepta.f90:466-525; the kz < 0 lines use the entry of -kz, the
// same k^2; line (0,0) is never solved and gets a harmless k^2 = 1).
// Replaces the tables of an earlier plan.
static int build_line_tables(sb_handle *h, int nseg) {
  Grid &g = h->g;
  Bufs &bf = h->bf;
  if (!line_segments_supported(nseg)) return fail(1, "%d warps per line solve not available", nseg);
  if ((g.my - 3) / nseg < 6) return fail(1, "my=%d too short for %d segments", g.my, nseg);
  sbh::SegPlan plan0;
  sbh::seg_plan(g.my, nseg, &plan0);
  g.nseg = plan0.nseg;
  for (int q = 0; q < plan0.nseg; q++) {
    g.slo[q] = plan0.lo[q];
    g.shi[q] = plan0.hi[q];
  }
  if (h->st) cudaStreamSynchronize(h->st);
  for (void *q : h->line_allocs) cudaFree(q);
  h->line_allocs.clear();
  h->alloc_to = &h->line_allocs;
  struct Reset {
    sb_handle *h;
    ~Reset() { h->alloc_to = nullptr; }
  } reset{h};
  sbh::Coeffs co;
  sbh::compact_coeffs(&co);
  double flhs[7], frhs[9];
  sbh::filter_coeffs(flhs, frhs);
  const double *rh2 = g.rh2;
  int rc;
  if ((rc = upload_uniform(h, &bf.d1, co.pr1, g.my)) ||
      (rc = upload_uniform(h, &bf.d2, co.pr2, g.my)) ||
      (g.ydeal == 3 && (rc = upload_uniform(h, &bf.flt, flhs, g.my))))
    return rc;
  {
    // lines (kx, kz) and (kx, -kz) share k^2 and so their factors: the table
    // holds the kz >= 0 lines only (hz_line maps a line to its entry)
    const int nlh = g.nkx * (g.nz + 1);
    const size_t n = g.my;
    std::vector<double> La(n * nlh), Lb(n * nlh), Lc(n * nlh), Dm(n * nlh), Dd(n * nlh), e(n * nlh),
        f(n * nlh), gg(n * nlh), sums(10 * (size_t)nlh);
    std::vector<double> hf[3], hb[3], ef(9 * (size_t)g.nseg * nlh), rows(16 * n * nlh);
    for (int t = 0; t < 3; t++) {
      hf[t].assign(n * nlh, 0.0);
      hb[t].assign(n * nlh, 0.0);
    }
    sbh::SegPlan plan;
    sbh::seg_plan(g.my, g.nseg, &plan);
    sbh::SegFac sfac;
    sbh::BaseFac bfac;
    for (int k = 0; k <= g.nz; k++)
      for (int i = 0; i < g.nkx; i++) {
        const size_t line = (size_t)k * g.nkx + i;
        int kzs = k;
        double gz = g.gam * kzs, a = g.alp * i;
        double k2 = (i == 0 && k == 0) ? 1.0 : gz * gz + a * a;
        double lap[7];
        for (int d = 0; d < 7; d++) lap[d] = rh2[d] - k2 * co.pr2[d];
        sbh::base_factor(lap, g.my, &bfac);
        for (size_t q = 0; q < n; q++) {
          La[q * nlh + line] = bfac.La[q];
          Lb[q * nlh + line] = bfac.Lb[q];
          Lc[q * nlh + line] = bfac.Lc[q];
          Dm[q * nlh + line] = bfac.Ddm1[q];
          Dd[q * nlh + line] = bfac.Dd[q];
          e[q * nlh + line] = bfac.e[q];
          f[q * nlh + line] = bfac.f[q];
          gg[q * nlh + line] = bfac.g[q];
        }
        for (int q = 0; q < 6; q++) sums[(size_t)q * nlh + line] = bfac.sums[q];
        for (int q = 0; q < 4; q++) sums[(size_t)(6 + q) * nlh + line] = lap[3 + q];
        sbh::seg_factor(bfac, g.my, plan, &sfac);
        for (int t = 0; t < 3; t++)
          for (size_t q = 0; q < n; q++) {
            hf[t][q * nlh + line] = sfac.hf[t][q];
            hb[t][q * nlh + line] = sfac.hb[t][q];
          }
        for (size_t q = 0; q < sfac.ef.size(); q++) ef[q * nlh + line] = sfac.ef[q];
        pack_rows(bfac, sfac, n, nlh, line, rows);
      }
    Fac &H = bf.hz;
    if ((rc = upload(h, &H.La, La)) || (rc = upload(h, &H.Lb, Lb)) || (rc = upload(h, &H.Lc, Lc)) ||
        (rc = upload(h, &H.Ddm1, Dm)) || (rc = upload(h, &H.Dd, Dd)) || (rc = upload(h, &H.e, e)) ||
        (rc = upload(h, &H.f, f)) || (rc = upload(h, &H.g, gg)) || (rc = upload(h, &H.sums, sums)) ||
        (rc = upload(h, &H.hf[0], hf[0])) || (rc = upload(h, &H.hf[1], hf[1])) ||
        (rc = upload(h, &H.hf[2], hf[2])) || (rc = upload(h, &H.hb[0], hb[0])) ||
        (rc = upload(h, &H.hb[1], hb[1])) || (rc = upload(h, &H.hb[2], hb[2])) ||
        (rc = upload(h, &H.ef, ef)) || (rc = upload(h, &H.rows, rows))) {
      return rc;
    }
    H.stride = nlh;
  }
  if (g.impl) {
    // the semi-implicit Helmholtz tables, filled by k_hfac every substep:
    // boxes x (lines (kx, kz >= 0) + the mean line)
    const size_t n = g.my, L = (size_t)g.B * (g.nkx * (g.nz + 1) + 1);
    Fac &I = bf.hi;
    double *q[17];
    const size_t cnt[17] = {n * L, n * L, n * L, n * L, n * L, n * L, n * L, n * L, 10 * L,
                            n * L, n * L, n * L, n * L, n * L, n * L, 9 * (size_t)g.nseg * L,
                            16 * n * L};
    for (int t = 0; t < 17; t++)
      if ((rc = dalloc(h, &q[t], cnt[t]))) return rc;
    I.La = q[0]; I.Lb = q[1]; I.Lc = q[2]; I.Ddm1 = q[3]; I.Dd = q[4];
    I.e = q[5]; I.f = q[6]; I.g = q[7]; I.sums = q[8];
    for (int t = 0; t < 3; t++) {
      I.hf[t] = q[9 + t];
      I.hb[t] = q[12 + t];
    }
    I.ef = q[15];
    I.rows = q[16];
    I.stride = (long)L;
    if (g.temp) {
      // the scalar's tables of crosst, same layout
      Fac &K = bf.hit;
      for (int t = 0; t < 17; t++)
        if ((rc = dalloc(h, &q[t], cnt[t]))) return rc;
      K.La = q[0]; K.Lb = q[1]; K.Lc = q[2]; K.Ddm1 = q[3]; K.Dd = q[4];
      K.e = q[5]; K.f = q[6]; K.g = q[7]; K.sums = q[8];
      for (int t = 0; t < 3; t++) {
        K.hf[t] = q[9 + t];
        K.hb[t] = q[12 + t];
      }
      K.ef = q[15];
      K.rows = q[16];
      K.stride = (long)L;
    }
  }
  if (prepare_line(g) != cudaSuccess)
    return fail(3, "line kernel attributes: %s", cudaGetErrorString(cudaGetLastError()));
  return 0;
}


static void member_defaults(const sb_params *p, const Grid &g, double Re, Member *m) {
  memset(m, 0, sizeof(Member));
  const double pi = g.pi;
  m->Re = Re;
  // without iadd_visc the LES run has no molecular viscous term (cross.f90:649)
  m->nu = (p->les && !p->les_visc) ? 0.0 : 1.0 / Re;
  m->CFL = p->CFL;
  // set_xyz_dy (initcr.f90:490-498)
  m->cflx = pi / p->CFL / g.dx;
  m->cflz = pi / p->CFL / g.dz;
  m->cfly = 2.5 / p->CFL / g.dy;
  double mm = std::fmax(std::fmax(pi * pi / g.dx / g.dx, 6.25 / g.dy / g.dy), pi * pi / g.dz / g.dz);
  m->cflvv = 1.0 / Re / p->CFL * mm;
  m->vbulk = p->vbulk;
  m->fixed_dt = p->fixed_dt;
  m->uprim = p->uprim;
  m->etime = p->etime > 0 ? p->etime : 1e10;
  m->dumptime = p->dumptime > 0 ? p->dumptime : 1e10;
  m->dtimag = p->dtimag > 0 ? p->dtimag : m->etime;
  m->readflag = p->readflag;
  m->nhist = p->nhist > 0 ? p->nhist : 1;
  m->keep_laminar = p->keep_laminar;
  // thermal diffusion CFL (initcr.f90:498-502)
  m->cflkk = p->temperature ? p->fkappa / p->CFL * mm : 0.0;
}

static int capture_step(sb_handle *h) {
  if (h->step_exec) {
    cudaGraphExecDestroy(h->step_exec);
    h->step_exec = nullptr;
  }
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int rk = 1; rk <= 3 && e == cudaSuccess; rk++) {
    if (h->g.ydeal == 3 && (e = launch_filter(h->g, h->bf, rk, h->st)) != cudaSuccess) break;
    if ((h->g.ydeal == 1 || h->g.ydeal == 2) &&
        ((e = launch_ydeal(h->g, h->bf, rk, h->st)) != cudaSuccess ||
         (e = launch_meand1(h->g, h->bf, h->st)) != cudaSuccess))
      break;
    const bool br_spec = (h->branch & 1) != 0, br_scal = (h->branch & 2) && !h->g.les;
    if (rk == 1 && !br_spec && (e = launch_spectra(h->g, h->bf, h->st)) != cudaSuccess) break;
    if (rk == 1 && br_spec &&
        ((e = cudaEventRecord(h->ev_s0, h->st)) != cudaSuccess ||
         (e = cudaStreamWaitEvent(h->side, h->ev_s0, 0)) != cudaSuccess ||
         (e = launch_spectra(h->g, h->bf, h->side)) != cudaSuccess ||
         (e = cudaEventRecord(h->ev_s1, h->side)) != cudaSuccess))
      break;
    if ((e = launch_plane(h->g, h->bf, 1, rk, h->st)) != cudaSuccess) break;
    if ((e = launch_plane(h->g, h->bf, 2, rk, h->st)) != cudaSuccess) break;
    // plane stage 3 overwrites inputs of the spectra
    if (rk == 1 && br_spec && (e = cudaStreamWaitEvent(h->st, h->ev_s1, 0)) != cudaSuccess)
      break;
    if (h->g.les)
      for (int q = 2; q <= 4 && e == cudaSuccess; q++) e = launch_les(h->g, h->bf, q, rk, h->st);
    if (e != cudaSuccess) break;
    if (br_scal) {
      // k_scalar needs stages 1-2 (statistics, |u| maxima) and k_tables needs
      // k_scalar: both run on a branch beside plane stage 3
      if ((e = cudaEventRecord(h->ev_fork, h->st)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(h->side, h->ev_fork, 0)) != cudaSuccess ||
          (e = launch_scalar(h->g, h->bf, rk, h->side)) != cudaSuccess ||
          (e = launch_tables(h->g, h->bf, rk, h->side)) != cudaSuccess ||
          (h->g.impl && (e = launch_hfac(h->g, h->bf, rk, h->side)) != cudaSuccess) ||
          (e = cudaEventRecord(h->ev_join, h->side)) != cudaSuccess ||
          (e = launch_plane(h->g, h->bf, 3, rk, h->st)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(h->st, h->ev_join, 0)) != cudaSuccess)
        break;
    } else {
      // in order on the main stream; with LES, k_scalar also takes the
      // statistics of the LES stages
      if ((e = launch_plane(h->g, h->bf, 3, rk, h->st)) != cudaSuccess) break;
      if (h->g.les && (e = launch_les(h->g, h->bf, 5, rk, h->st)) != cudaSuccess) break;
      if ((e = launch_scalar(h->g, h->bf, rk, h->st)) != cudaSuccess) break;
      if ((e = launch_tables(h->g, h->bf, rk, h->st)) != cudaSuccess) break;
      if (h->g.impl && (e = launch_hfac(h->g, h->bf, rk, h->st)) != cudaSuccess) break;
    }
    if (h->g.les && (e = launch_lineL(h->g, h->bf, h->st)) != cudaSuccess) break;
    if (h->g.impl) {
      e = launch_lineI(h->g, h->bf, rk, h->st);
      continue;
    }
    if (h->g.lform && line_fused_ok(h->g)) {
      e = launch_lineF(h->g, h->bf, rk, h->st);
      continue;
    }
    if ((e = launch_lineA(h->g, h->bf, rk, h->st)) != cudaSuccess) break;
    e = launch_lineB(h->g, h->bf, rk, h->st);
  }
  if (e == cudaSuccess) e = launch_finish(h->g, h->bf, h->st);
  cudaError_t e2 = cudaStreamEndCapture(h->st, &graph);
  if (e != cudaSuccess) return fail(3, "kernel launch during capture: %s", cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(3, "capture: %s", cudaGetErrorString(e2));
  CK(cudaGraphInstantiate(&h->step_exec, graph, 0));
  cudaGraphDestroy(graph);
  return 0;
}

static int ensure_trace(sb_handle *h, int cap) {
  if (cap <= h->trace_cap) return 0;
  cap = std::max(cap, 2 * h->trace_cap);
  // no copies in flight on either stream before the step graph is re-captured
  if (h->st) CK(cudaStreamSynchronize(h->st));
  if (h->side) CK(cudaStreamSynchronize(h->side));
  double *t;
  int rc = dalloc(h, &t, (size_t)h->g.B * cap * h->g.tlen);
  if (rc) return rc;
  h->bf.trace = t;
  h->trace_cap = cap;
  for (int b = 0; b < h->g.B; b++)
    CK(cudaMemcpy((char *)(h->bf.mem + b) + offsetof(Member, trace_cap), &cap, sizeof(int),
                  cudaMemcpyHostToDevice));
  return capture_step(h);
}

// common checks of the operator entry points
static int op_check(int my, double Ly, int nlines, const void *u, const void *out, long ldu,
                    long ldo, const double *shp, const double *shm) {
  if (my < 16 || my > SB_MAX_NY) return fail(1, "my=%d outside 16..%d", my, SB_MAX_NY);
  if (!(Ly > 0)) return fail(1, "Ly must be positive");
  if (nlines < 1) return fail(1, "nlines must be >= 1");
  if (!u || !out || !shp || !shm) return fail(1, "null argument");
  if (ldu < nlines || ldo < nlines) return fail(1, "leading dimension smaller than nlines");
  return 0;
}

extern "C" {

int sb_version(void) { return 1; }
const char *sb_last_error(void) { return g_err.c_str(); }

int sb_fft_twiddles(int n, int factored, double *out) {
  if (!out || n < 1) return fail(1, "bad argument");
  const std::vector<double> v = factored ? sbh::fft_twiddles_factored(n) : sbh::fft_twiddles(n);
  std::memcpy(out, v.data(), sizeof(double) * v.size());
  return 0;
}

int sb_sizes(const sb_params *p, int *out) {
  if (!p || !out) return fail(1, "null argument");
  int mx = 2 * (p->mgalx / 3), mz = 2 * (p->mgalz / 3) - 1;
  out[0] = mx;
  out[1] = mz;
  out[2] = mx / 2;
  out[3] = p->my;
  out[4] = (mz - 1) / 2;
  out[5] = p->mgalx;
  out[6] = p->mgalz;
  out[7] = (mx / 2) * mz * p->my;
  return 0;
}

int sb_compact_coeffs(double *pr1, double *rh1h, double *pr2, double *rh2h) {
  sbh::Coeffs c;
  sbh::compact_coeffs(&c);
  for (int d = 0; d < 7; d++) {
    pr1[d] = c.pr1[d];
    rh1h[d] = c.rh1h[d];
    pr2[d] = c.pr2[d];
    rh2h[d] = c.rh2h[d];
  }
  return 0;
}

int sb_seed_state(const sb_params *p, unsigned long long seed, double k0, double urms,
                  double *vor, double *phi, double *u00, double *w00) {
  int rc = check_params(p);
  if (rc) return rc;
  return sbh::seed_state(p->mgalx, p->my, p->mgalz, p->alp, p->gam, p->Ly, seed, k0, urms, vor,
                         phi, u00, w00);
}

int sb_create(const sb_params *p, int batch, int precision, sb_handle **out) {
  if (!out) return fail(1, "null output handle");
  *out = nullptr;
  int rc = check_params(p);
  if (rc) return rc;
  if (batch < 1) return fail(1, "batch must be >= 1");
  if (precision != SB_FP64 && precision != SB_MIXED)
    return fail(2, "precision %d not available (0: FP64, 1: FP32-mixed)", precision);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(5, "no CUDA device: the shearbox library has no CPU path");
  sb_handle *h = new sb_handle();
  h->p = *p;
  h->precision = precision;
  Grid &g = h->g;
  memset(&g, 0, sizeof(g));
  g.B = batch;
  g.prec = precision;
  g.mgalx = p->mgalx;
  g.my = p->my;
  g.mgalz = p->mgalz;
  g.mx = 2 * (p->mgalx / 3);
  g.mz = 2 * (p->mgalz / 3) - 1;
  g.nkx = g.mx / 2;
  g.nz = (g.mz - 1) / 2;
  g.mgx = p->mgalx / 2;
  g.cb1 = g.cb3 = plane_cb(p->mgalz);
  g.ncb = (g.nkx + g.cb1 - 1) / g.cb1;
  g.ncb3 = (g.nkx + g.cb3 - 1) / g.cb3;
  g.t2 = plane_t2_default(p->mgalx);
  g.pi = 4.0 * std::atan(1.0);
  g.alp = p->alp;
  g.gam = p->gam;
  g.Ly = p->Ly;
  g.s = p->s;
  g.chi = p->chi;
  g.dx = 2.0 * g.pi / p->alp / (double)g.mx;
  g.dz = 2.0 * g.pi / p->gam / (double)g.mz;
  g.dy = p->Ly / (double)p->my;
  g.les = p->les ? 1 : 0;
  g.les_visc = p->les_visc ? 1 : 0;
  g.nzf = g.les ? 10 : 6;
  // temperature (crosst): one more z-transform field after the others, the
  // three fluxes in xbuf, the longer statistics record
  g.temp = p->temperature ? 1 : 0;
  g.tround = g.les ? 5 : 3;
  g.tzf = g.nzf;
  g.nzf += g.temp;
  g.nxf = g.temp ? 6 : 3;
  g.tlen = g.temp ? SB_TRACE_LEN_T : SB_TRACE_LEN;
  // diffusion and buoyancy sit with the molecular viscous terms, which an LES
  // run without iadd_visc skips (crosst.f90:717-757)
  const bool molec = !g.les || g.les_visc;
  g.kappa = (g.temp && molec) ? p->fkappa : 0.0;
  g.gbeta = (g.temp && molec) ? p->gbeta : 0.0;
  g.bym = g.temp ? p->bym : 0.0;
  g.damp = p->damping ? 1 : 0;
  g.lz = 2.0 * g.pi / p->gam;
  g.damp_up = p->damp_up;
  g.damp_a = g.lz * p->damp_aa;
  g.force = p->force;
  g.force_roll = p->force_roll;
  g.xforce = p->xforce;
  g.cbl = les_cb(p->mgalz);
  g.ncbl = (g.nkx + g.cbl - 1) / g.cbl;
  g.ydeal = p->ydeal;
  g.impl = p->implicit_visc ? 1 : 0;
  g.my23 = 2 * (p->my / 3);  // initcr.f90:207-210
  g.ny1 = ((g.my23 - 1) - 1) / 2;
  g.ny2 = p->my - g.ny1;
  g.Lx = 2.0 * g.pi / p->alp;
  double flhs[7], frhs[9];
  sbh::filter_coeffs(flhs, frhs);
  for (int d = 0; d <= 4; d++) g.frh[d] = frhs[4 + d];
  if (g.les) {
    // Deltag = (dx dy dz)^(1/3) (initcr.f90:510); nu_t = Cles^2 Deltag^2 |S|
    const double dg = std::pow(g.dx * g.dy * g.dz, 1.0 / 3.0);
    g.les_c = p->cs * p->cs * dg * dg;
  }
  sbh::Coeffs co;
  sbh::compact_coeffs(&co);
  const double hdy = g.dy;
  double rh1[7], rh2[7];
  for (int d = 0; d < 7; d++) {
    rh1[d] = co.rh1h[d] / hdy;          // update_dy (diffy_shear_hepta.f90:562-573)
    rh2[d] = co.rh2h[d] / (hdy * hdy);
    g.rh1[d] = rh1[d];
    g.rh2[d] = rh2[d];
    g.pr2[d] = co.pr2[d];
  }
  const int nl = g.nkx * g.mz;
  g.plane = 2L * nl;
  g.field = g.plane * g.my;
  g.nlines_pad = ((2 * nl + 31) / 32) * 32;
  g.ngrp = (nl + 15) / 16;
  sbh::SegPlan plan;
  sbh::seg_plan(g.my, line_segments(), &plan);
  g.nseg = plan.nseg;
  for (int q = 0; q < plan.nseg; q++) {
    g.slo[q] = plan.lo[q];
    g.shi[q] = plan.hi[q];
  }
  g.lform = 1;  // the fused y-line kernel wherever the step allows it
  cudaError_t ce = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->ev_s0, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->ev_s1, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->ev_c0, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->ev_c1, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaMallocHost((void **)&h->hs, sizeof(sb_handle::HostSmall));
  if (ce != cudaSuccess) {
    sb_destroy(h);
    return fail(3, "stream: %s", cudaGetErrorString(ce));
  }
  Bufs &bf = h->bf;
  const size_t B = batch, F = g.field, my = g.my;
  auto A = [&](double **q, size_t n) { return dalloc(h, q, n); };
  if ((rc = A(&bf.vor, B * F)) || (rc = A(&bf.phi, B * F)) || (rc = A(&bf.vorwk, B * F)) ||
      (rc = A(&bf.phiwk, B * F)) || (rc = A(&bf.G, B * F)) || (rc = A(&bf.V, B * F)) ||
      (rc = A(&bf.D, B * F)) || (rc = A(&bf.S, B * F)) || (rc = A(&bf.T, B * F)) ||
      (rc = A(&bf.Lv, B * F)) ||
      (rc = A(&bf.tl1o, B * g.nkx * SB_TAIL)) || (rc = A(&bf.tl2o, B * g.nkx * SB_TAIL)) ||
      (rc = A(&bf.tl1n, B * g.nkx * SB_TAIL)) || (rc = A(&bf.tl2n, B * g.nkx * SB_TAIL)) ||
      (rc = A(&bf.mu, B * 2 * my)) || (rc = A(&bf.mwk, B * 2 * my)) ||
      (rc = A(&bf.mrf, B * 2 * my)) || (rc = A(&bf.mdu, B * 2 * my)) ||
      (rc = A(&bf.zbuf, B * my * g.mgalz * g.nzf * g.nkx * 2)) ||
      (rc = A(&bf.xbuf, B * my * g.mgalz * g.nxf * g.nkx * 2)) ||
      (rc = A(&bf.hpart, B * my * ((g.nkx * g.mz + 15) / 16) * SB_NHIST_Q)) ||
      (rc = A(&bf.hsum, B * my * (SB_NHIST_Q + 5))) || (rc = A(&bf.sh_old, B * 4 * g.nkx)) ||
      (rc = A(&bf.sh_new, B * 4 * g.nkx)) || (rc = A(&bf.mf1, B * my * g.nkx * 2)) ||
      (rc = A(&bf.mf2, B * my * g.nkx * 2)) || (rc = A(&h->d_pen, F)) ||
      (rc = A(&h->d_pen2, F))) {
    sb_destroy(h);
    return rc;
  }
  if ((rc = A(&bf.stats, B * my * 23)) || (rc = A(&bf.stats2, B * my * 23)) ||
      (rc = A(&bf.spec, B * g.nkx * g.mz * 8)) || (rc = A(&bf.spec2, B * g.nkx * g.mz * 8)) ||
      (rc = A(&bf.ppart, B * my * (g.mgalz / 2) * 16 * 3)) ||
      (g.temp && ((rc = A(&bf.tstats, B * my * 5)) || (rc = A(&bf.tspec, B * g.nkx * g.mz * 4))))) {
    sb_destroy(h);
    return rc;
  }
  if (g.temp &&
      ((rc = A(&bf.tb, B * F)) || (rc = A(&bf.tbwk, B * F)) || (rc = A(&bf.Ht, B * F)) ||
       (rc = A(&bf.R2, B * F)) || (rc = A(&bf.Lt, B * F)) || (rc = A(&bf.mt, B * 2 * my)) ||
       (rc = A(&bf.mtwk, B * 2 * my)) || (rc = A(&bf.mtr, B * 2 * my)))) {
    sb_destroy(h);
    return rc;
  }
  if (!plane3_fits(g, g.cb3)) {
    g.cb3 = 4;
    g.ncb3 = (g.nkx + g.cb3 - 1) / g.cb3;
  }
  if (g.les) {
    const size_t NX = g.mgalx, NZ = g.mgalz, nk = g.nkx;
    if ((rc = A(&bf.gbuf, B * my * (NZ / 2) * 12 * NX)) || (rc = A(&bf.sbuf, B * my * NZ * nk * 2)) ||
        (rc = A(&bf.tbuf, B * my * NZ * 6 * nk * 2)) || (rc = A(&bf.L1, B * F)) ||
        (rc = A(&bf.L2, B * F)) || (rc = A(&bf.txy, B * 2 * my)) ||
        (rc = A(&bf.lpart, B * my * (NZ / 2) * 2))) {
      sb_destroy(h);
      return rc;
    }
  }
  {
    void *q = nullptr;
    ce = cudaMalloc(&q, sizeof(Member) * B);
    if (ce != cudaSuccess) {
      sb_destroy(h);
      return fail(4, "cudaMalloc members: %s", cudaGetErrorString(ce));
    }
    h->allocs.push_back(q);
    bf.mem = (Member *)q;
  }
  // twiddles e^{-2 pi i t / N}
  // FFT twiddles: the complex table (FP32 storage) and the factored FP64 form
  const auto tw = sbh::fft_twiddles;
  const auto gtw = sbh::fft_twiddles_factored;
  std::vector<double> kinv((size_t)nl), ginv((size_t)g.mz);
  for (int k = 0; k < g.mz; k++) {
    int kzs = (k <= g.nz) ? k : k - g.mz;
    double gz = g.gam * kzs;
    ginv[k] = (k == 0) ? 0.0 : 1.0 / gz;
    for (int i = 0; i < g.nkx; i++) {
      double a = g.alp * i;
      double K = gz * gz + a * a;
      kinv[(size_t)k * g.nkx + i] = (i == 0 && k == 0) ? 0.0 : 1.0 / K;
    }
  }
  auto upload_f = [&](const float **dst, const std::vector<double> &v) -> int {
    std::vector<float> f(v.begin(), v.end());
    double *q;
    int r = dalloc(h, &q, (f.size() + 1) / 2);
    if (r) return r;
    cudaError_t e = cudaMemcpy(q, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(3, "upload: %s", cudaGetErrorString(e));
    *dst = (const float *)q;
    return 0;
  };
  if ((rc = upload(h, &bf.twz, gtw(g.mgalz))) || (rc = upload(h, &bf.twx, gtw(g.mgalx))) ||
      (rc = upload_f(&bf.twzf, tw(g.mgalz))) || (rc = upload_f(&bf.twxf, tw(g.mgalx))) ||
      (rc = upload_f(&bf.kinvf, kinv)) ||
      (rc = upload(h, &bf.kinv, kinv)) || (rc = upload(h, &bf.ginv, ginv)) ||
      ((g.ydeal == 1 || g.ydeal == 2) &&
       ((rc = upload(h, &bf.twy, gtw(g.my))) || (rc = upload_f(&bf.twyf, tw(g.my)))))) {
    sb_destroy(h);
    return rc;
  }
  if ((rc = build_line_tables(h, g.nseg))) {
    sb_destroy(h);
    return rc;
  }
  if (g.impl && !line_implicit_ok(g)) {
    sb_destroy(h);
    return fail(2, "implicit_visc: my=%d too large for the semi-implicit y-line block", g.my);
  }
  h->mem_init.resize(B);
  for (size_t b = 0; b < B; b++) member_defaults(p, g, p->Re, &h->mem_init[b]);
  ce = cudaMemcpy(bf.mem, h->mem_init.data(), sizeof(Member) * B, cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    sb_destroy(h);
    return fail(3, "member upload: %s", cudaGetErrorString(ce));
  }
  if (launch_plane(g, bf, 0, 0, h->st) != cudaSuccess || prepare_line(g) != cudaSuccess ||
      (g.les && launch_les(g, bf, 0, 0, h->st) != cudaSuccess) ||
      ((g.ydeal == 1 || g.ydeal == 2) && launch_ydeal(g, bf, 0, h->st) != cudaSuccess)) {
    sb_destroy(h);
    return fail(3, "kernel attributes: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if ((rc = ensure_trace(h, 64))) {
    sb_destroy(h);
    return rc;
  }
  *out = h;
  return 0;
}

int sb_destroy(sb_handle *h) {
  if (!h) return 0;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->step_exec) cudaGraphExecDestroy(h->step_exec);
  for (void *q : h->allocs) cudaFree(q);
  for (void *q : h->line_allocs) cudaFree(q);
  if (h->hs) cudaFreeHost(h->hs);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->ev_s0) cudaEventDestroy(h->ev_s0);
  if (h->ev_s1) cudaEventDestroy(h->ev_s1);
  if (h->ev_c0) cudaEventDestroy(h->ev_c0);
  if (h->ev_c1) cudaEventDestroy(h->ev_c1);
  delete h;
  return 0;
}

int sb_set_member_re(sb_handle *h, int member, double Re) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!(Re != 0.0)) return fail(1, "Re must be nonzero");
  Member m = h->mem_init[member];
  member_defaults(&h->p, h->g, Re, &m);
  h->mem_init[member].Re = m.Re;
  h->mem_init[member].nu = m.nu;
  h->mem_init[member].cflvv = m.cflvv;
  Member *d = h->bf.mem + member;
  CK(cudaMemcpy((char *)d + offsetof(Member, Re), &m.Re, sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy((char *)d + offsetof(Member, nu), &m.nu, sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy((char *)d + offsetof(Member, cflvv), &m.cflvv, sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

int sb_set_member_etime(sb_handle *h, int member, double etime) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!(etime > 0)) return fail(1, "etime must be positive");
  h->mem_init[member].etime = etime;
  CK(cudaMemcpy((char *)(h->bf.mem + member) + offsetof(Member, etime), &etime, sizeof(double),
                cudaMemcpyHostToDevice));
  return 0;
}

// State in (pencil layout -> planes) through the two staging buffers; the
// small values go through pinned host memory, so nothing here waits for the
// device unless `sync` (the public call: the caller may reuse its arrays).
static int set_state_impl(sb_handle *h, int member, const double *vor, const double *phi,
                          const double *u00, const double *w00, double time, double xoffb,
                          double xofft, bool sync) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!vor || !phi || !u00 || !w00) return fail(1, "null state array");
  const Grid &g = h->g;
  const size_t F = g.field;
  const size_t Fd = g.prec ? F / 2 : F;  // field size in doubles of the storage type
  // phi on the side stream, after the work already queued on the main one
  CK(cudaEventRecord(h->ev_c0, h->st));
  CK(cudaStreamWaitEvent(h->side, h->ev_c0, 0));
  CK(cudaMemcpyAsync(h->d_pen2, phi, sizeof(double) * F, cudaMemcpyHostToDevice, h->side));
  CK(launch_pencil_to_plane(g, h->d_pen2, h->bf.phi + member * Fd, h->side));
  CK(cudaEventRecord(h->ev_c1, h->side));
  CK(cudaMemcpyAsync(h->d_pen, vor, sizeof(double) * F, cudaMemcpyHostToDevice, h->st));
  CK(launch_pencil_to_plane(g, h->d_pen, h->bf.vor + member * Fd, h->st));
  CK(cudaStreamWaitEvent(h->st, h->ev_c1, 0));
  sb_handle::HostSmall &hs = *h->hs;
  if (g.prec) {
    float *muf = (float *)hs.mu_in;
    for (int j = 0; j < g.my; j++) {
      muf[2 * j] = (float)u00[j];
      muf[2 * j + 1] = (float)w00[j];
    }
    CK(cudaMemcpyAsync((float *)h->bf.mu + (size_t)member * 2 * g.my, muf,
                       sizeof(float) * 2 * g.my, cudaMemcpyHostToDevice, h->st));
  } else {
    for (int j = 0; j < g.my; j++) {
      hs.mu_in[2 * j] = u00[j];
      hs.mu_in[2 * j + 1] = w00[j];
    }
    CK(cudaMemcpyAsync(h->bf.mu + (size_t)member * 2 * g.my, hs.mu_in,
                       sizeof(double) * 2 * g.my, cudaMemcpyHostToDevice, h->st));
  }
  hs.sc_in[0] = time;
  hs.sc_in[1] = xoffb;
  hs.sc_in[2] = xofft;
  CK(cudaMemcpyAsync((char *)(h->bf.mem + member) + offsetof(Member, time), hs.sc_in,
                     sizeof(hs.sc_in), cudaMemcpyHostToDevice, h->st));
  // a new state restarts the LES running maximum of nu_t
  CK(cudaMemsetAsync((char *)(h->bf.mem + member) + offsetof(Member, max_nut), 0, sizeof(double),
                     h->st));
  if (sync) CK(cudaStreamSynchronize(h->st));
  return 0;
}

int sb_set_state(sb_handle *h, int member, const double *vor, const double *phi, const double *u00,
                 const double *w00, double time, double xoffb, double xofft) {
  return set_state_impl(h, member, vor, phi, u00, w00, time, xoffb, xofft, true);
}

// State out through the two staging buffers, one synchronisation; with `st`
// also the member's status from the same copy.
static void fill_status(const Member &m, sb_status *st);
static int get_state_impl(sb_handle *h, int member, double *vor, double *phi, double *u00,
                          double *w00, double *time, double *xoffb, double *xofft,
                          sb_status *st) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  const Grid &g = h->g;
  const size_t F = g.field;
  const size_t Fd = g.prec ? F / 2 : F;
  // phi on the side stream beside omega_y
  if (phi) {
    CK(cudaEventRecord(h->ev_c0, h->st));
    CK(cudaStreamWaitEvent(h->side, h->ev_c0, 0));
    CK(launch_plane_to_pencil(g, h->bf.phi + member * Fd, h->d_pen2, h->side));
    CK(cudaMemcpyAsync(phi, h->d_pen2, sizeof(double) * F, cudaMemcpyDeviceToHost, h->side));
    CK(cudaEventRecord(h->ev_c1, h->side));
  }
  if (vor) {
    CK(launch_plane_to_pencil(g, h->bf.vor + member * Fd, h->d_pen, h->st));
    CK(cudaMemcpyAsync(vor, h->d_pen, sizeof(double) * F, cudaMemcpyDeviceToHost, h->st));
  }
  if (phi) CK(cudaStreamWaitEvent(h->st, h->ev_c1, 0));
  sb_handle::HostSmall &hs = *h->hs;
  const size_t mub = (g.prec ? sizeof(float) : sizeof(double)) * 2 * g.my;
  CK(cudaMemcpyAsync(hs.mu_out, (const char *)h->bf.mu + (size_t)member * mub, mub,
                     cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(hs.sc_out, (char *)(h->bf.mem + member) + offsetof(Member, time),
                     sizeof(hs.sc_out), cudaMemcpyDeviceToHost, h->st));
  if (st)
    CK(cudaMemcpyAsync(&hs.m, h->bf.mem + member, sizeof(Member), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const float *muf = (const float *)hs.mu_out;
  for (int j = 0; j < g.my; j++) {
    const double u = g.prec ? (double)muf[2 * j] : hs.mu_out[2 * j];
    const double w = g.prec ? (double)muf[2 * j + 1] : hs.mu_out[2 * j + 1];
    if (u00) u00[j] = u;
    if (w00) w00[j] = w;
  }
  if (time) *time = hs.sc_out[0];
  if (xoffb) *xoffb = hs.sc_out[1];
  if (xofft) *xofft = hs.sc_out[2];
  if (st) fill_status(hs.m, st);
  return 0;
}

int sb_get_state(sb_handle *h, int member, double *vor, double *phi, double *u00, double *w00,
                 double *time, double *xoffb, double *xofft) {
  return get_state_impl(h, member, vor, phi, u00, w00, time, xoffb, xofft, nullptr);
}

long sb_packed_length(const sb_handle *h) { return h ? packed_length(h->g) : -1; }

int sb_set_state_packed(sb_handle *h, int member, const double *x, const double sca[3],
                        double time, double xoffb, double xofft) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!x || !sca) return fail(1, "null argument");
  if (h->g.temp) return fail(2, "packed states carry no temperature");
  if (!(sca[0] != 0.0 && sca[1] != 0.0 && sca[2] != 0.0)) return fail(1, "zero scale");
  const Grid &g = h->g;
  const size_t Fd = g.prec ? g.field / 2 : g.field;
  const size_t mud = g.prec ? (size_t)g.my : 2 * (size_t)g.my;  // doubles per member's mean line
  CK(launch_unpack(g, x, h->bf.vor + member * Fd, h->bf.phi + member * Fd,
                   h->bf.mu + member * mud, sca, h->st));
  // the pinned staging may feed an earlier copy still in flight
  CK(cudaStreamSynchronize(h->st));
  sb_handle::HostSmall &hs = *h->hs;
  hs.sc_in[0] = time;
  hs.sc_in[1] = xoffb;
  hs.sc_in[2] = xofft;
  CK(cudaMemcpyAsync((char *)(h->bf.mem + member) + offsetof(Member, time), hs.sc_in,
                     sizeof(hs.sc_in), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemsetAsync((char *)(h->bf.mem + member) + offsetof(Member, max_nut), 0, sizeof(double),
                     h->st));
  return 0;
}

int sb_packed_shift_tangent(sb_handle *h, const double *x, double *out, int dir) {
  if (!h || !x || !out) return fail(1, "null argument");
  if (dir != 0 && dir != 1) return fail(1, "dir must be 0 (x) or 1 (z)");
  CK(launch_tangent(h->g, x, out, dir, h->st));
  return 0;
}

int sb_get_state_packed(sb_handle *h, int member, double *x, const double sca[3], double shiftx,
                        double shiftz) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!x || !sca) return fail(1, "null argument");
  if (!(sca[0] != 0.0 && sca[1] != 0.0 && sca[2] != 0.0)) return fail(1, "zero scale");
  const Grid &g = h->g;
  const size_t Fd = g.prec ? g.field / 2 : g.field;
  const size_t mud = g.prec ? (size_t)g.my : 2 * (size_t)g.my;
  CK(launch_pack(g, h->bf.vor + member * Fd, h->bf.phi + member * Fd, h->bf.mu + member * mud, x,
                 sca, shiftx, shiftz, h->st));
  return 0;
}

// mean profile of one member: [my] reals <-> the re parts of a [my] complex
// device line in the storage precision
static int put_mean_re(sb_handle *h, double *dev, int member, const double *v) {
  const Grid &g = h->g;
  if (g.prec) {
    std::vector<float> f(2 * (size_t)g.my, 0.0f);
    for (int j = 0; j < g.my; j++) f[2 * j] = (float)v[j];
    CK(cudaMemcpyAsync((float *)dev + (size_t)member * 2 * g.my, f.data(), sizeof(float) * f.size(),
                       cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  } else {
    std::vector<double> d(2 * (size_t)g.my, 0.0);
    for (int j = 0; j < g.my; j++) d[2 * j] = v[j];
    CK(cudaMemcpyAsync(dev + (size_t)member * 2 * g.my, d.data(), sizeof(double) * d.size(),
                       cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return 0;
}
static int get_mean_re(sb_handle *h, const double *dev, int member, double *v) {
  const Grid &g = h->g;
  if (g.prec) {
    std::vector<float> f(2 * (size_t)g.my);
    CK(cudaMemcpyAsync(f.data(), (const float *)dev + (size_t)member * 2 * g.my,
                       sizeof(float) * f.size(), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int j = 0; j < g.my; j++) v[j] = (double)f[2 * j];
  } else {
    std::vector<double> d(2 * (size_t)g.my);
    CK(cudaMemcpyAsync(d.data(), dev + (size_t)member * 2 * g.my, sizeof(double) * d.size(),
                       cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int j = 0; j < g.my; j++) v[j] = d[2 * j];
  }
  return 0;
}

int sb_set_temperature(sb_handle *h, int member, const double *tb, const double *tb00) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!h->g.temp) return fail(2, "the handle was created without itemperature");
  if (!tb || !tb00) return fail(1, "null temperature array");
  const Grid &g = h->g;
  const size_t Fd = g.prec ? g.field / 2 : g.field;
  CK(cudaMemcpyAsync(h->d_pen, tb, sizeof(double) * g.field, cudaMemcpyHostToDevice, h->st));
  CK(launch_pencil_to_plane(g, h->d_pen, h->bf.tb + member * Fd, h->st));
  return put_mean_re(h, h->bf.mt, member, tb00);
}

int sb_get_temperature(sb_handle *h, int member, double *tb, double *tb00) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if (!h->g.temp) return fail(2, "the handle was created without itemperature");
  const Grid &g = h->g;
  const size_t Fd = g.prec ? g.field / 2 : g.field;
  if (tb) {
    CK(launch_plane_to_pencil(g, h->bf.tb + member * Fd, h->d_pen, h->st));
    CK(cudaMemcpyAsync(tb, h->d_pen, sizeof(double) * g.field, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  if (tb00) return get_mean_re(h, h->bf.mt, member, tb00);
  return 0;
}

int sb_step(sb_handle *h, int nsteps) {
  if (!h) return fail(1, "null handle");
  if (nsteps < 0) return fail(1, "nsteps < 0");
  int rc = ensure_trace(h, nsteps > 0 ? nsteps : 1);
  if (rc) return rc;
  // entry of cross(): flags and offsets, phase tables, set_conj on the state,
  // v from phi and the first derivatives (cross.f90:76-113,283-287,376-445)
  CK(launch_scalar(h->g, h->bf, 0, h->st));
  CK(launch_tables(h->g, h->bf, 0, h->st));
  CK(launch_setconj(h->g, h->bf, h->st));
  if (h->g.ydeal == 3) CK(launch_filter(h->g, h->bf, 0, h->st));
  CK(launch_lineB(h->g, h->bf, 0, h->st));
  for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(h->step_exec, h->st));
  return 0;
}

static void fill_status(const Member &m, sb_status *st) {
  st->istop = m.istop;
  st->steps_done = m.istep - 1;
  st->ntrace = m.ntrace;
  st->flags = m.flags;
  st->time = m.time;
  st->deltat = m.Deltat;
  st->xoffb = m.xoffb;
  st->xofft = m.xofft;
  st->cfl = m.CFLcur;
  st->cflv = m.CFLv;
}

int sb_get_status(sb_handle *h, int member, sb_status *st) {
  if (!h || !st || member < 0 || member >= h->g.B) return fail(1, "bad argument");
  Member m;
  CK(cudaMemcpyAsync(&m, h->bf.mem + member, sizeof(Member), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  fill_status(m, st);
  return 0;
}

int sb_get_trace(sb_handle *h, int member, double *out, int max_records, int *nrec) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad argument");
  Member m;
  CK(cudaMemcpyAsync(&m, h->bf.mem + member, sizeof(Member), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  int n = std::min(std::min(m.ntrace, h->trace_cap), max_records);
  if (n > 0 && out)
    CK(cudaMemcpy(out, h->bf.trace + (size_t)member * h->trace_cap * h->g.tlen,
                  sizeof(double) * n * h->g.tlen, cudaMemcpyDeviceToHost));
  if (nrec) *nrec = n;
  return 0;
}

int sb_cross(sb_handle *h, double *vor, double *phi, double *u00, double *w00, double *time,
             double *xoffb, double *xofft, int nstep, sb_status *st) {
  if (!h || !time || !xoffb || !xofft) return fail(1, "null argument");
  // the arrays belong to the call until it returns: one synchronisation, at
  // the end
  int rc = set_state_impl(h, 0, vor, phi, u00, w00, *time, *xoffb, *xofft, false);
  if (rc) return rc;
  if ((rc = sb_step(h, nstep))) return rc;
  return get_state_impl(h, 0, vor, phi, u00, w00, time, xoffb, xofft, st);
}

int sb_get_statistics(sb_handle *h, int member, double *stats, double *stats2, double *spec,
                      double *spec2, double *tstats, double *tspec, int *nacum,
                      double *total_dt) {
  if (!h || member < 0 || member >= h->g.B) return fail(1, "bad handle or member");
  if ((tstats || tspec) && !h->g.temp) return fail(2, "the handle has no temperature");
  const Grid &g = h->g;
  const size_t nst = (size_t)g.my * 23, nsp = (size_t)g.nkx * g.mz * 8;
  auto get = [&](double *dst, const double *src, size_t n) -> cudaError_t {
    if (!dst) return cudaSuccess;
    return cudaMemcpyAsync(dst, src + (size_t)member * n, sizeof(double) * n,
                           cudaMemcpyDeviceToHost, h->st);
  };
  CK(get(stats, h->bf.stats, nst));
  CK(get(stats2, h->bf.stats2, nst));
  CK(get(spec, h->bf.spec, nsp));
  CK(get(spec2, h->bf.spec2, nsp));
  if (g.temp) {
    CK(get(tstats, h->bf.tstats, (size_t)g.my * 5));
    CK(get(tspec, h->bf.tspec, nsp / 2));
  }
  Member m;
  CK(cudaMemcpyAsync(&m, h->bf.mem + member, sizeof(Member), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (nacum) *nacum = m.nacum;
  if (total_dt) *total_dt = m.total_dt;
  return 0;
}

int sb_crosst(sb_handle *h, double *vor, double *phi, double *u00, double *w00, double *tb,
              double *tb00, double *time, double *xoffb, double *xofft, int nstep,
              sb_status *st) {
  if (!h || !time || !xoffb || !xofft) return fail(1, "null argument");
  if (!h->g.temp) return fail(2, "crosst needs a handle created with itemperature = 1");
  int rc = sb_set_state(h, 0, vor, phi, u00, w00, *time, *xoffb, *xofft);
  if (rc || (rc = sb_set_temperature(h, 0, tb, tb00))) return rc;
  if ((rc = sb_step(h, nstep))) return rc;
  if ((rc = sb_get_state(h, 0, vor, phi, u00, w00, time, xoffb, xofft))) return rc;
  if ((rc = sb_get_temperature(h, 0, tb, tb00))) return rc;
  if (st && (rc = sb_get_status(h, 0, st))) return rc;
  return 0;
}

void *sb_get_stream(sb_handle *h) { return h ? (void *)h->st : nullptr; }

int sb_launch_stage(sb_handle *h, int stage, int rk, int count) {
  if (!h || count < 0) return fail(1, "bad argument");
  if (stage < 1 || stage > 14 || rk < 1 || rk > 3) return fail(1, "stage 1..14, rk 1..3");
  if (stage >= 7 && stage <= 11 && !h->g.les) return fail(1, "stages 7..11 need an LES handle");
  if (stage == 12 && !line_fused_ok(h->g))
    return fail(1, "stage 12 (fused y-line kernel) not available for this handle");
  if (stage >= 13 && !h->g.impl) return fail(1, "stages 13, 14 need an implicit_visc handle");
  for (int q = 0; q < count; q++) {
    cudaError_t e;
    if (stage <= 3)
      e = launch_plane(h->g, h->bf, stage, rk, h->st);
    else if (stage == 4)
      e = launch_tables(h->g, h->bf, rk, h->st);
    else if (stage == 5)
      e = launch_lineA(h->g, h->bf, rk, h->st);
    else if (stage == 6)
      e = launch_lineB(h->g, h->bf, rk, h->st);
    else if (stage <= 10)
      e = launch_les(h->g, h->bf, stage - 5, rk, h->st);
    else if (stage == 11)
      e = launch_lineL(h->g, h->bf, h->st);
    else if (stage == 12)
      e = launch_lineF(h->g, h->bf, rk, h->st);
    else if (stage == 13)
      e = launch_hfac(h->g, h->bf, rk, h->st);
    else
      e = launch_lineI(h->g, h->bf, rk, h->st);
    if (e != cudaSuccess) return fail(3, "launch: %s", cudaGetErrorString(e));
  }
  return 0;
}

// A copy of what a step changes and the next step reads: the state fields,
// the mean lines, the members' scalars (and the temperature).
struct Snapshot {
  std::vector<std::pair<void *, size_t>> parts;  // (device field, bytes)
  std::vector<void *> copies;
  int take(sb_handle *h) {
    const Grid &g = h->g;
    const size_t es = g.prec ? sizeof(float) : sizeof(double);
    const size_t Fb = es * g.field * (size_t)g.B, Mb = es * 2 * (size_t)g.my * g.B;
    parts = {{h->bf.vor, Fb}, {h->bf.phi, Fb}, {h->bf.mu, Mb},
             {h->bf.mem, sizeof(Member) * (size_t)g.B}};
    if (g.temp) {
      parts.push_back({h->bf.tb, Fb});
      parts.push_back({h->bf.mt, Mb});
    }
    for (auto &pt : parts) {
      void *q = nullptr;
      if (cudaMalloc(&q, pt.second) != cudaSuccess) {
        release();
        return fail(4, "autotune: no memory for the state snapshot");
      }
      copies.push_back(q);
      if (cudaMemcpyAsync(q, pt.first, pt.second, cudaMemcpyDeviceToDevice, h->st) != cudaSuccess)
        return fail(3, "autotune: snapshot copy failed");
    }
    return 0;
  }
  int restore(sb_handle *h) {
    for (size_t q = 0; q < copies.size(); q++)
      if (cudaMemcpyAsync(parts[q].first, copies[q], parts[q].second, cudaMemcpyDeviceToDevice,
                          h->st) != cudaSuccess)
        return fail(3, "autotune: snapshot restore failed");
    return 0;
  }
  void release() {
    for (void *q : copies) cudaFree(q);
    copies.clear();
  }
};

// the launches of one sb_step call of nsteps steps (without the trace check)
static cudaError_t launch_step_call(sb_handle *h, int nsteps) {
  cudaError_t e;
  if ((e = launch_scalar(h->g, h->bf, 0, h->st)) != cudaSuccess ||
      (e = launch_tables(h->g, h->bf, 0, h->st)) != cudaSuccess ||
      (e = launch_setconj(h->g, h->bf, h->st)) != cudaSuccess ||
      (h->g.ydeal == 3 && (e = launch_filter(h->g, h->bf, 0, h->st)) != cudaSuccess) ||
      (e = launch_lineB(h->g, h->bf, 0, h->st)) != cudaSuccess)
    return e;
  for (int s = 0; s < nsteps && e == cudaSuccess; s++) e = cudaGraphLaunch(h->step_exec, h->st);
  return e;
}

int sb_autotune(sb_handle *h, int *choice) {
  if (!h) return fail(1, "null handle");
  Grid &g = h->g;
  cudaStream_t st = h->st;
  // the derived fields of the current state, as at the entry of a call
  CK(launch_scalar(g, h->bf, 0, st));
  CK(launch_tables(g, h->bf, 0, st));
  CK(launch_setconj(g, h->bf, st));
  if (g.ydeal == 3) CK(launch_filter(g, h->bf, 0, st));
  CK(launch_lineB(g, h->bf, 0, st));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto timed = [&](int stage, float *ms) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < 2 && e == cudaSuccess; q++) e = launch_plane(g, h->bf, stage, 2, st);
    if (e != cudaSuccess) return e;
    cudaEventRecord(e0, st);
    for (int q = 0; q < 8 && e == cudaSuccess; q++) e = launch_plane(g, h->bf, stage, 2, st);
    cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    return e;
  };
  cudaError_t e = cudaSuccess;
  float best = 1e30f, t = 0.0f;
  int cb1 = g.cb1, cb3 = g.cb3, t2 = g.t2;
  for (int c : {8, 4}) {  // plane stage 1: kx columns per block
    g.cb1 = c;
    g.ncb = (g.nkx + c - 1) / c;
    if ((e = timed(1, &t)) != cudaSuccess) break;
    if (t < best) best = t, cb1 = c;
  }
  g.cb1 = cb1;
  g.ncb = (g.nkx + cb1 - 1) / cb1;
  const int t2d = plane_t2_default(g.mgalx);
  best = 1e30f;
  for (int c : {t2d, 2 * t2d}) {  // plane stage 2: threads per block
    if (e != cudaSuccess) break;
    g.t2 = c;
    if ((e = timed(2, &t)) != cudaSuccess) break;
    if (t < best) best = t, t2 = c;
  }
  g.t2 = t2;
  best = 1e30f;
  for (int c : {8, 4}) {  // plane stage 3: kx columns per block
    if (e != cudaSuccess) break;
    if (!plane3_fits(g, c)) continue;
    g.cb3 = c;
    g.ncb3 = (g.nkx + c - 1) / c;
    if ((e = timed(3, &t)) != cudaSuccess) break;
    if (t < best) best = t, cb3 = c;
  }
  g.cb3 = cb3;
  g.ncb3 = (g.nkx + cb3 - 1) / cb3;
  // the y-line tile: warps per line solve (the segment plan and its factor
  // tables), timed on whole captured steps -- the solves of a step differ in
  // kind and count per kernel, so no single kernel stands for them -- from a
  // snapshot of the state that is put back afterwards
  int nseg = g.nseg, lform = g.lform;
  best = 1e30f;
  Snapshot snap;
  int rc = snap.take(h);
  for (int c : {1, 2, 3}) {
    if (rc || e != cudaSuccess) break;
    if ((g.my - 3) / c < 6) continue;
    if ((rc = build_line_tables(h, c))) break;
    // both forms of the y-line stage where the fused one is available
    for (int f = 1; f >= 0; f--) {
      if (rc || e != cudaSuccess) break;
      if (f == 1 && !line_fused_ok(g)) continue;
      g.lform = f;
      if ((rc = capture_step(h))) break;
      for (int q = 0; q < 3 && e == cudaSuccess; q++) {
        if ((rc = snap.restore(h))) break;
        if (q) cudaEventRecord(e0, st);
        e = launch_step_call(h, 2);
        if (q) cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float tq = 0.0f;
        if (q && e == cudaSuccess) e = cudaEventElapsedTime(&tq, e0, e1);
        if (q == 1) t = tq;
        if (q == 2) t = t < tq ? t : tq;
      }
      if (!rc && e == cudaSuccess && t < best) best = t, nseg = c, lform = f;
    }
  }
  // which side work runs as a concurrent graph branch, on the chosen tile:
  // a branch that shares the SMs with short plane stages can cost more than
  // it hides (measured: the FP32-mixed 192x96x96 step is 7% faster with the
  // spectra in order, the FP64 step 1% slower)
  g.lform = lform;
  if (!rc && e == cudaSuccess && g.nseg != nseg) rc = build_line_tables(h, nseg);
  int branch = h->branch;
  best = 1e30f;
  for (int m : {3, 2, 1, 0}) {
    if (rc || e != cudaSuccess) break;
    h->branch = m;
    if ((rc = capture_step(h))) break;
    for (int q = 0; q < 3 && e == cudaSuccess; q++) {
      if ((rc = snap.restore(h))) break;
      cudaEventRecord(e0, st);
      e = launch_step_call(h, 4);
      cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float tq = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&tq, e0, e1);
      if (q == 1) t = tq;
      if (q == 2) t = t < tq ? t : tq;
    }
    if (!rc && e == cudaSuccess && t < best) best = t, branch = m;
  }
  h->branch = branch;
  if (!rc) rc = snap.restore(h);
  snap.release();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(3, "autotune: %s", cudaGetErrorString(e));
  if (choice) {
    choice[0] = g.cb1;
    choice[1] = g.cb3;
    choice[2] = g.t2;
  }
  return capture_step(h);
}

int sb_set_line_segments(sb_handle *h, int nseg) {
  if (!h) return fail(1, "null handle");
  const int rc = build_line_tables(h, nseg);
  if (rc) return rc;
  return capture_step(h);
}

int sb_set_line_form(sb_handle *h, int form) {
  if (!h) return fail(1, "null handle");
  if (form != 0 && form != 1) return fail(1, "line form %d (0 split, 1 fused)", form);
  if (form == 1 && !line_fused_ok(h->g))
    return fail(1, "fused y-line kernel not available for this handle");
  h->g.lform = form;
  return capture_step(h);
}

int sb_set_side_branch(sb_handle *h, int mask) {
  if (!h) return fail(1, "null handle");
  if (mask < 0 || mask > 3) return fail(1, "side-branch mask %d (0..3)", mask);
  h->branch = mask;
  return capture_step(h);
}

int sb_get_side_branch(sb_handle *h, int *mask) {
  if (!h || !mask) return fail(1, "null argument");
  *mask = h->branch;
  return 0;
}

int sb_get_line_form(sb_handle *h, int *form) {
  if (!h || !form) return fail(1, "null argument");
  *form = h->g.impl ? 2 : ((h->g.lform && line_fused_ok(h->g)) ? 1 : 0);
  return 0;
}

int sb_get_tuning(sb_handle *h, int *out) {
  if (!h || !out) return fail(1, "null argument");
  out[0] = h->g.cb1;
  out[1] = h->g.cb3;
  out[2] = h->g.t2;
  out[3] = h->g.nseg;
  return 0;
}

int sb_physical_fields(sb_handle *h, int member, unsigned mask, double *out) {
  if (!h || member < 0 || member >= h->g.B || !out) return fail(1, "bad argument");
  mask &= 0x7FFu;
  int nout = 0;
  for (int q = 0; q < 11; q++) nout += (mask >> q) & 1u;
  if (!nout) return 0;
  const Grid &g = h->g;
  cudaStream_t st = h->st;
  // the derived fields of the current state (v, dv/dy, d(omega_y)/dy, mean
  // derivatives), as at the entry of a call
  CK(launch_scalar(g, h->bf, 0, st));
  CK(launch_tables(g, h->bf, 0, st));
  CK(launch_setconj(g, h->bf, st));
  CK(launch_lineB(g, h->bf, 0, st));
  // one box: member-offset buffers, plane stage 1 with the extra z-transforms
  Grid gl = g;
  gl.B = 1;
  gl.les = 1;
  gl.nzf = 10;
  gl.temp = 0;
  Bufs bl = h->bf;
  const long Fd = g.prec ? g.field / 2 : g.field;
  const long Md = g.prec ? (long)g.my : 2L * g.my;
  bl.vor += member * Fd;
  bl.phi += member * Fd;
  bl.D += member * Fd;
  bl.V += member * Fd;
  bl.G += member * Fd;
  bl.mu += member * Md;
  bl.mdu += member * Md;
  bl.mem += member;
  const size_t nout_d = (size_t)nout * g.my * g.mgalz * g.mgalx;
  double *zb = nullptr, *od = nullptr;
  CK(cudaMallocAsync((void **)&zb, sizeof(double) * (size_t)g.my * g.mgalz * 10 * g.nkx * 2, st));
  CK(cudaMallocAsync((void **)&od, sizeof(double) * nout_d, st));
  bl.zbuf = zb;
  cudaError_t e = launch_physical(gl, bl, mask, od, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, od, sizeof(double) * nout_d, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(zb, st);
  cudaFreeAsync(od, st);
  if (e != cudaSuccess) return fail(3, "physical fields: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int sb_fp64_peak(sb_handle *h, double *tflops) {
  if (!h || !tflops) return fail(1, "bad argument");
  CK(fp64_peak(tflops, h->st));
  return 0;
}

int sb_sync(sb_handle *h) {
  if (!h) return fail(1, "null handle");
  CK(cudaStreamSynchronize(h->st));
  CK(cudaGetLastError());
  return 0;
}

int sb_op_derivyc(int my, double Ly, int iord, int nlines, const double *u, long ldu, double *out,
                  long ldo, const double *shp, const double *shm, void *stream) {
  int rc = op_check(my, Ly, nlines, u, out, ldu, ldo, shp, shm);
  if (rc) return rc;
  if (iord != 1 && iord != 2) return fail(1, "iord must be 1 or 2");
  cudaStream_t st = (cudaStream_t)stream;
  HostFac hf;
  double r[4];
  int anti;
  const std::vector<double> host = derivyc_block(my, Ly, iord, nlines, shp, shm, &hf, r, &anti);
  const size_t nfac = hf.buf.size();
  const long nthr = op_threads(nlines);
  double *dbuf = nullptr, *ybuf = nullptr;
  CK(cudaMallocAsync((void **)&dbuf, sizeof(double) * host.size(), st));
  CK(cudaMallocAsync((void **)&ybuf, sizeof(double) * (size_t)my * nthr, st));
  CK(cudaMemcpyAsync(dbuf, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, st));
  Fac F = fac_bind(hf, dbuf);
  cudaError_t e = launch_op_line(nlines, my, u, ldu, out, ldo, ybuf, F, dbuf + nfac,
                                 dbuf + nfac + 2 * nlines, r, anti, st);
  cudaFreeAsync(ybuf, st);
  cudaFreeAsync(dbuf, st);
  if (e != cudaSuccess) return fail(3, "launch: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int sb_op_lapcdy(int my, double Ly, int nlines, const double *u, long ldu, double *out, long ldo,
                 const double *k2, const double *shp, const double *shm, void *stream) {
  int rc = op_check(my, Ly, nlines, u, out, ldu, ldo, shp, shm);
  if (rc) return rc;
  if (!k2) return fail(1, "null k2");
  cudaStream_t st = (cudaStream_t)stream;
  sbh::Coeffs co;
  sbh::compact_coeffs(&co);
  const double dy = Ly / (double)my;
  HostFac hf;
  host_fac_init(&hf, my, nlines);
  sbh::BaseFac b;
  for (int l = 0; l < nlines; l++) {
    double lap[7];
    for (int d = 0; d < 7; d++) lap[d] = co.rh2h[d] / (dy * dy) - k2[l] * co.pr2[d];
    sbh::base_factor(lap, my, &b);
    host_fac_add(&hf, l, b, lap);
  }
  double r[4] = {co.pr2[3], co.pr2[4], co.pr2[5], co.pr2[6]};
  const size_t nfac = hf.buf.size();
  std::vector<double> host(nfac + 4 * (size_t)nlines);
  std::copy(hf.buf.begin(), hf.buf.end(), host.begin());
  std::copy(shp, shp + 2 * (size_t)nlines, host.begin() + nfac);
  std::copy(shm, shm + 2 * (size_t)nlines, host.begin() + nfac + 2 * nlines);
  const long nthr = op_threads(nlines);
  double *dbuf = nullptr, *ybuf = nullptr;
  CK(cudaMallocAsync((void **)&dbuf, sizeof(double) * host.size(), st));
  CK(cudaMallocAsync((void **)&ybuf, sizeof(double) * (size_t)my * nthr, st));
  CK(cudaMemcpyAsync(dbuf, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, st));
  Fac F = fac_bind(hf, dbuf);
  cudaError_t e = launch_op_line(nlines, my, u, ldu, out, ldo, ybuf, F, dbuf + nfac,
                                 dbuf + nfac + 2 * nlines, r, 0, st);
  cudaFreeAsync(ybuf, st);
  cudaFreeAsync(dbuf, st);
  if (e != cudaSuccess) return fail(3, "launch: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int sb_op_filterc(int my, int nlines, const double *u, long ldu, double *out, long ldo,
                  const double *shp, void *stream) {
  int rc = op_check(my, 1.0, nlines, u, out, ldu, ldo, shp, shp);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  double lhs[7], rhs[9];
  sbh::filter_coeffs(lhs, rhs);
  HostFac hf;
  host_fac_init(&hf, my, 1);
  sbh::BaseFac b;
  sbh::base_factor(lhs, my, &b);
  host_fac_add(&hf, 0, b, lhs);
  const size_t nfac = hf.buf.size();
  std::vector<double> host(nfac + 4 * (size_t)nlines);
  std::copy(hf.buf.begin(), hf.buf.end(), host.begin());
  std::copy(shp, shp + 2 * (size_t)nlines, host.begin() + nfac);
  for (int l = 0; l < nlines; l++) {  // the solve's lower image: conj(shp)
    host[nfac + 2 * nlines + 2 * l] = shp[2 * l];
    host[nfac + 2 * nlines + 2 * l + 1] = -shp[2 * l + 1];
  }
  const long nthr = op_threads(nlines);
  double *dbuf = nullptr, *ybuf = nullptr, *wbuf = nullptr;
  CK(cudaMallocAsync((void **)&dbuf, sizeof(double) * host.size(), st));
  CK(cudaMallocAsync((void **)&ybuf, sizeof(double) * (size_t)my * nthr, st));
  CK(cudaMallocAsync((void **)&wbuf, sizeof(double) * 2 * (size_t)my * nlines, st));
  CK(cudaMemcpyAsync(dbuf, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, st));
  Fac F = fac_bind(hf, dbuf);
  const double r9[5] = {rhs[4], rhs[5], rhs[6], rhs[7], rhs[8]};
  const double one[4] = {1.0, 0.0, 0.0, 0.0};
  cudaError_t e = launch_filter_rhs(nlines, my, u, ldu, wbuf, nlines, dbuf + nfac, r9, st);
  if (e == cudaSuccess)
    e = launch_op_line(nlines, my, wbuf, nlines, out, ldo, ybuf, F, dbuf + nfac,
                       dbuf + nfac + 2 * nlines, one, 0, st);
  cudaFreeAsync(wbuf, st);
  cudaFreeAsync(ybuf, st);
  cudaFreeAsync(dbuf, st);
  if (e != cudaSuccess) return fail(3, "launch: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(st));
  return 0;
}

static int yop(int my, int nlines, double *c, long ldc, int iopt, int real, void *stream) {
  if (!supported_ylen(my)) return fail(1, "my=%d: y transforms support 32,48,64,96,192,384", my);
  if (nlines < 1 || !c || ldc < nlines || iopt == 0) return fail(1, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = launch_yop(my, nlines, c, ldc, iopt, real, st);
  if (e != cudaSuccess) return fail(3, "launch: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(st));
  return 0;
}

int sb_op_cfty(int my, int nlines, double *c, long ldc, int iopt, void *stream) {
  return yop(my, nlines, c, ldc, iopt, 0, stream);
}

int sb_op_rfty(int my, int nlines, double *c, long ldc, int iopt, void *stream) {
  return yop(my, nlines, c, ldc, iopt, 1, stream);
}

int sb_op_derivyc_noalloc(int my, double Ly, int iord, int nlines, const double *u, long ldu,
                          double *out, long ldo, const double *shp, const double *shm,
                          void *stream) {
  std::string err;
  int rc = sb::noalloc_derivyc(my, Ly, iord, nlines, u, ldu, out, ldo, shp, shm, stream, &err);
  if (rc) return fail(rc, "%s", err.c_str());
  return 0;
}

}  // extern "C"
