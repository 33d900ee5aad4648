// sb_io.cpp -- restart files in the reference's binary layout (escru writer,
// readwrite.f90:1336-1398; getfil reader, readwrite.f90:72-447).
//
// The file is a Fortran unformatted sequential file: every record is framed by
// its byte length as a little-endian 32-bit integer before and after the
// payload (the gfortran/ifort default; the reference builds with
// -fconvert=little-endian).  Records, in order:
//    1  mgalx, my, mgalz, numerop                               4 int32
//    2  time, Re, alp, Ly/pi, gam, s, chi; mx, my, mz            7 float64, 3 int32
//    3  y(0:my-1)                                               my float64
//    4  xoffb, xofft, zoffb, zofft                              4 float64
//    5  u00(0:my-1), w00(0:my-1)                                2 my float64
//    6  one record per y plane: for kz, for kx (kx fastest):
//       vor.re, phi.re, vor.im, phi.im                          4 nkx mz float64
//    7  CFL, uprim, vbulk, xforce                               4 float64
//    8  irev, nopt, nparams                                     3 int32
//    9  the nopt switches (explicit, ifix_dt, iadd_force, iadd_mode, iadd_sym,
//       iadd_damping, iuse_LES, iadd_visc, idynamic)            nopt int32
//   10  the nparams parameters (Deltat, force_roll, xforce, zforce, damp_aa,
//       damp_up, Cles, Deltag, cutoffx, cutoffz, LESflt(1:3))   nparams float64
// The state arrays of the C-ABI keep the reference pencil layout
// complex(0:my1, 0:mx1, 0:mz1) (y fastest).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/shearbox.h"

namespace sb {
void set_error(const std::string &msg);  // the message sb_last_error returns (sb_api.cu)
}

namespace {

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

void put_u32(std::vector<unsigned char> &b, uint32_t v) {
  for (int q = 0; q < 4; q++) b.push_back((unsigned char)((v >> (8 * q)) & 0xffu));
}
uint32_t get_u32(const unsigned char *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
void put_i32(std::vector<unsigned char> &b, int v) { put_u32(b, (uint32_t)v); }
void put_f64(std::vector<unsigned char> &b, double v) {
  uint64_t u;
  memcpy(&u, &v, 8);
  for (int q = 0; q < 8; q++) b.push_back((unsigned char)((u >> (8 * q)) & 0xffu));
}
double get_f64(const unsigned char *p) {
  uint64_t u = 0;
  for (int q = 0; q < 8; q++) u |= (uint64_t)p[q] << (8 * q);
  double v;
  memcpy(&v, &u, 8);
  return v;
}
int get_i32(const unsigned char *p) { return (int)get_u32(p); }

bool write_record(FILE *f, const std::vector<unsigned char> &payload) {
  std::vector<unsigned char> m;
  put_u32(m, (uint32_t)payload.size());
  return fwrite(m.data(), 1, 4, f) == 4 &&
         fwrite(payload.data(), 1, payload.size(), f) == payload.size() &&
         fwrite(m.data(), 1, 4, f) == 4;
}

// reads one record; false at end of file or on a broken frame
bool read_record(FILE *f, std::vector<unsigned char> *payload, std::string *err) {
  unsigned char m[4];
  if (fread(m, 1, 4, f) != 4) return false;
  const uint32_t n = get_u32(m);
  if (n > (1u << 30)) {
    *err = "record length out of range";
    return false;
  }
  payload->resize(n);
  if (n && fread(payload->data(), 1, n, f) != n) {
    *err = "truncated record";
    return false;
  }
  unsigned char e[4];
  if (fread(e, 1, 4, f) != 4 || get_u32(e) != n) {
    *err = "record end marker mismatch";
    return false;
  }
  return true;
}

int io_fail(int code, const std::string &msg) {
  sb::set_error(msg);
  return code;
}

// Natural cubic spline through (x, y), N points: the second derivatives d2
// with zero end curvature (cubic_spline, readwrite.f90:774-812, m = 1; the
// tridiagonal sweep of the classic natural spline), and its value at c
// (interpolate, readwrite.f90:1131-1155: bisection for the bracketing knots).
void natural_spline(const double *x, const double *y, int N, double *d2) {
  std::vector<double> u((size_t)N, 0.0);
  d2[0] = 0.0;
  d2[N - 1] = 0.0;
  for (int i = 1; i < N - 1; i++) {
    const double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    const double p = sig * d2[i - 1] + 2.0;
    d2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) -
            sig * u[i - 1]) /
           p;
  }
  for (int k = N - 2; k >= 1; k--) d2[k] = d2[k] * d2[k + 1] + u[k];
}
double spline_at(double c, const double *x, const double *y, const double *d2, int N) {
  int klo = 0, khi = N - 1;
  while (khi - klo > 1) {
    const int k = (khi + klo) / 2;
    if (x[k] > c)
      khi = k;
    else
      klo = k;
  }
  const double h = x[khi] - x[klo];
  const double a = (x[khi] - c) / h, b = (c - x[klo]) / h;
  return a * y[klo] + b * y[khi] + ((a * a * a - a) * d2[klo] + (b * b * b - b) * d2[khi]) * (h * h) / 6.0;
}

}  // namespace

extern "C" {

int sb_write_restart(const char *path, const sb_params *p, const double *vor, const double *phi,
                     const double *u00, const double *w00, double time, double xoffb,
                     double xofft, double deltat) {
  if (!path || !p || !vor || !phi || !u00 || !w00) return io_fail(1, "null argument");
  const int my = p->my, mx = 2 * (p->mgalx / 3), mz = 2 * (p->mgalz / 3) - 1, nkx = mx / 2;
  if (my < 1 || nkx < 1 || mz < 1) return io_fail(1, "bad grid");
  const double pi = 4.0 * std::atan(1.0);
  File fh;
  fh.f = fopen(path, "wb");
  if (!fh.f) return io_fail(7, std::string("cannot open ") + path);
  std::vector<unsigned char> r;
  bool ok = true;
  auto flush = [&]() {
    ok = ok && write_record(fh.f, r);
    r.clear();
  };
  put_i32(r, p->mgalx); put_i32(r, my); put_i32(r, p->mgalz); put_i32(r, 1);
  flush();
  put_f64(r, time); put_f64(r, p->Re); put_f64(r, p->alp); put_f64(r, p->Ly / pi);
  put_f64(r, p->gam); put_f64(r, p->s); put_f64(r, p->chi);
  put_i32(r, mx); put_i32(r, my); put_i32(r, mz);
  flush();
  const double dy = p->Ly / (double)my;
  for (int j = 0; j < my; j++) put_f64(r, (double)j * dy - 0.5 * p->Ly);  // y (initcr.f90:486-488)
  flush();
  put_f64(r, xoffb); put_f64(r, xofft); put_f64(r, 0.0); put_f64(r, 0.0);
  flush();
  for (int j = 0; j < my; j++) put_f64(r, u00[j]);
  for (int j = 0; j < my; j++) put_f64(r, w00[j]);
  flush();
  for (int j = 0; j < my && ok; j++) {
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < nkx; i++) {
        const size_t q = 2 * (((size_t)k * nkx + i) * my + j);
        put_f64(r, vor[q]); put_f64(r, phi[q]); put_f64(r, vor[q + 1]); put_f64(r, phi[q + 1]);
      }
    flush();
  }
  put_f64(r, p->CFL); put_f64(r, p->uprim); put_f64(r, p->vbulk); put_f64(r, p->xforce);
  flush();
  put_i32(r, 1742); put_i32(r, 9); put_i32(r, 13);  // irev (mod.f90:45), nopt, nparams
  flush();
  const int opts[9] = {p->implicit_visc ? 0 : 1, p->fixed_dt > 0 ? 1 : 0, p->force, 5, 0, p->damping,
                       p->les ? 1 : 0, p->les_visc ? 1 : 0, 0};
  for (int q = 0; q < 9; q++) put_i32(r, opts[q]);
  flush();
  const double dx = 2.0 * pi / p->alp / (double)mx, dz = 2.0 * pi / p->gam / (double)mz;
  const double deltag = p->les ? std::pow(dx * dy * dz, 1.0 / 3.0) : 0.0;
  const double prm[13] = {deltat, p->force_roll, p->xforce, 0.0, p->damp_aa, p->damp_up,
                          p->les ? p->cs : 0.0, deltag, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int q = 0; q < 13; q++) put_f64(r, prm[q]);
  flush();
  if (!ok) return io_fail(7, std::string("write failed: ") + path);
  return 0;
}

int sb_read_restart_ex(const char *path, const sb_params *p, int flags, double *vor, double *phi,
                       double *u00, double *w00, sb_restart_info *info) {
  if (!path || !info) return io_fail(1, "null argument");
  memset(info, 0, sizeof(*info));
  File fh;
  fh.f = fopen(path, "rb");
  if (!fh.f) return io_fail(7, std::string("cannot open ") + path);
  std::vector<unsigned char> r;
  std::string err;
  auto need = [&](size_t n, const char *what) -> int {
    if (!read_record(fh.f, &r, &err)) return io_fail(8, std::string(what) + ": " + (err.empty() ? "missing" : err));
    if (r.size() < n) return io_fail(8, std::string(what) + ": record too short");
    return 0;
  };
  int rc;
  if ((rc = need(16, "grid record"))) return rc;
  info->mgalx = get_i32(&r[0]);
  info->my = get_i32(&r[4]);
  info->mgalz = get_i32(&r[8]);
  info->numerop = get_i32(&r[12]);
  if ((rc = need(68, "parameter record"))) return rc;
  const double pi = 4.0 * std::atan(1.0);
  info->time = get_f64(&r[0]);
  info->Re = get_f64(&r[8]);
  info->alp = get_f64(&r[16]);
  info->Ly = get_f64(&r[24]) * pi;
  info->gam = get_f64(&r[32]);
  info->s = get_f64(&r[40]);
  info->chi = get_f64(&r[48]);
  info->mx = get_i32(&r[56]);
  info->mye = get_i32(&r[60]);
  info->mz = get_i32(&r[64]);
  const int mye = info->mye, mxe = info->mx, mze = info->mz;
  if (mye < 1 || mxe < 2 || mze < 1 || mye > 1 << 16 || mxe > 1 << 16 || mze > 1 << 16)
    return io_fail(8, "sizes out of range");
  if ((rc = need(8 * (size_t)mye, "y record"))) return rc;
  std::vector<double> yfile((size_t)mye);
  for (int j = 0; j < mye; j++) yfile[j] = get_f64(&r[8 * (size_t)j]);
  if (std::fabs(info->Ly + 2.0 * get_f64(&r[0])) > 1e-9 * std::fmax(1.0, info->Ly))
    return io_fail(8, "y(0) is not -Ly/2: broken file (getfil, readwrite.f90:146-149)");
  if ((rc = need(32, "offset record"))) return rc;
  info->xoffb = get_f64(&r[0]);
  info->xofft = get_f64(&r[8]);
  info->zoffb = get_f64(&r[16]);
  info->zofft = get_f64(&r[24]);
  if ((rc = need(16 * (size_t)mye, "mean profile record"))) return rc;
  std::vector<double> m00(2 * (size_t)mye);
  for (int q = 0; q < 2 * mye; q++) m00[q] = get_f64(&r[8 * (size_t)q]);
  // the state, mapped on the caller's grid (getfil, readwrite.f90:252-305):
  // common kx modes, the klen lowest positive and negative kz modes
  const int nkxe = mxe / 2;
  std::vector<std::vector<unsigned char>> planes((size_t)mye);
  for (int j = 0; j < mye; j++) {
    if ((rc = need(32 * (size_t)nkxe * mze, "plane record"))) return rc;
    planes[j].swap(r);
  }
  // footer (optional in old files, readwrite.f90:311-323)
  if (read_record(fh.f, &r, &err) && r.size() >= 32) {
    info->CFL = get_f64(&r[0]);
    info->uprim = get_f64(&r[8]);
    info->vbulk = get_f64(&r[16]);
    info->xforce = get_f64(&r[24]);
    if (read_record(fh.f, &r, &err) && r.size() >= 12) {
      info->irev = get_i32(&r[0]);
      info->nopt = get_i32(&r[4]);
      info->nparams = get_i32(&r[8]);
      if (read_record(fh.f, &r, &err))
        for (int q = 0; q < info->nopt && q < SB_RESTART_MAXOPT && 4 * (size_t)(q + 1) <= r.size(); q++)
          info->options[q] = get_i32(&r[4 * (size_t)q]);
      if (read_record(fh.f, &r, &err))
        for (int q = 0; q < info->nparams && q < SB_RESTART_MAXOPT && 8 * (size_t)(q + 1) <= r.size(); q++)
          info->params[q] = get_f64(&r[8 * (size_t)q]);
      info->has_footer = 1;
    }
  }
  if (!p) return 0;  // header only
  if (!vor || !phi || !u00 || !w00) return io_fail(1, "null state array");
  const int my = p->my, mx = 2 * (p->mgalx / 3), mz = 2 * (p->mgalz / 3) - 1, nkx = mx / 2;
  const int nz = (mz - 1) / 2;
  const double tiny = 1e-13;  // mod.f90:41
  // x: the offsets follow a change of Lx; a doubled alp with half the x points
  // keeps the even modes of the file (ihalf, readwrite.f90:152-171)
  int iskip = 1;
  double xoffb = info->xoffb, xofft = info->xofft;
  if (info->mgalx != p->mgalx && mye != my)
    return io_fail(9, "x and y grids both change: getfil does not interpolate in my at the same "
                      "time (readwrite.f90:116-120)");
  if (info->alp != p->alp) {
    if ((int)((p->alp + 0.00001) / info->alp) == 2 && info->mgalx / p->mgalx == 2) {
      xoffb = xoffb * info->alp / p->alp * 2.0;
      xofft = xofft * info->alp / p->alp * 2.0;
      iskip = 2;
    } else {
      xoffb = xoffb * info->alp / p->alp;
      xofft = xofft * info->alp / p->alp;
    }
    if (mye != my) return io_fail(9, "alp and my both change (readwrite.f90:172-175)");
  }
  // y: the file's planes as they stand, every other one (my = mye/2), copies
  // of the box stacked in y (my = 3 or 5 mye), or a cubic spline in y
  const int ihalfy = (my == mye / 2) ? 1 : 0;
  int ncopy = 0;
  if (mye == my / 3) ncopy = 3;
  else if (mye == my / 5) ncopy = 5;
  const bool interp = (mye < my) && (ncopy == 0);
  if (interp && std::fabs(info->Ly - p->Ly) >= tiny)
    return io_fail(9, "interpolation in y needs the file's Ly (readwrite.f90:404-413)");
  const int mxm = std::min(nkx, nkxe) , mzm = std::min(mz, mze);
  if (iskip == 2 && (mxm - 1) * 2 >= nkxe) return io_fail(9, "ihalf: not enough kx modes in the file");
  memset(vor, 0, sizeof(double) * 2 * (size_t)my * nkx * mz);
  memset(phi, 0, sizeof(double) * 2 * (size_t)my * nkx * mz);
  for (int j = 0; j < my; j++) u00[j] = w00[j] = 0.0;
  const int mym = std::min(my, mye);
  for (int j = 0; j < (ihalfy ? my : mym); j++) {
    const int je = ihalfy ? 2 * j : j;
    u00[j] = m00[je];
    w00[j] = m00[(size_t)mye + je];
  }
  // modes (readwrite.f90:252-305): common kx (every iskip-th of the file),
  // the klen lowest positive and negative kz
  const int klen = (mzm + 1) / 2, kini1 = mze - klen, kini2 = mz - klen;
  const int nplanes = ihalfy ? my : mym;
  for (int j = 0; j < nplanes; j++) {
    const unsigned char *pl = planes[ihalfy ? 2 * j : j].data();
    auto put = [&](int ke, int k) {
      for (int i = 0; i < mxm; i++) {
        const unsigned char *e = pl + 32 * ((size_t)ke * nkxe + (size_t)i * iskip);
        const size_t q = 2 * (((size_t)k * nkx + i) * my + j);
        vor[q] = get_f64(e);
        phi[q] = get_f64(e + 8);
        vor[q + 1] = get_f64(e + 16);
        phi[q + 1] = get_f64(e + 24);
      }
    };
    for (int k = 0; k < klen; k++) put(k, k);
    for (int t = 1; t < klen; t++) put(kini1 + t, kini2 + t);
  }
  // set_conj on the read state (readwrite.f90:376; operators.f90:1382-1429)
  for (int k = nz + 1; k < mz; k++)
    for (int j = 0; j < my; j++) {
      const size_t dst = 2 * ((size_t)k * nkx * my + j), src = 2 * ((size_t)(mz - k) * nkx * my + j);
      vor[dst] = vor[src];
      vor[dst + 1] = -vor[src + 1];
      phi[dst] = phi[src];
      phi[dst + 1] = -phi[src + 1];
    }
  if (interp) {
    // interp_y (readwrite.f90:707-771): per mode line the file's mye planes
    // and the wrapped first plane at y = Ly/2 (times exp(-i kx xofft)), a
    // natural cubic spline through them evaluated on the run's y grid
    std::vector<double> ye((size_t)mye + 1);
    for (int j = 0; j < mye; j++) ye[j] = yfile[j];
    ye[mye] = p->Ly / 2.0;
    std::vector<double> yrun((size_t)my);
    const double dy = p->Ly / (double)my;
    for (int j = 0; j < my; j++) yrun[j] = (double)j * dy - 0.5 * p->Ly;  // initcr.f90:486-488
    const int N = mye + 1;
    std::vector<double> re(N), im(N), d2r(N), d2i(N), src(2 * (size_t)my);
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < nkx; i++) {
        const double ph = -(p->alp * i) * xofft;
        const double cr = std::cos(ph), ci = std::sin(ph);  // zexp(-xalp(i)*xofft)
        for (double *f : {vor, phi}) {
          double *line = f + 2 * ((size_t)k * nkx + i) * my;
          for (int j = 0; j < mye; j++) {
            re[j] = line[2 * j];
            im[j] = line[2 * j + 1];
          }
          re[mye] = line[0] * cr - line[1] * ci;
          im[mye] = line[0] * ci + line[1] * cr;
          natural_spline(ye.data(), re.data(), N, d2r.data());
          natural_spline(ye.data(), im.data(), N, d2i.data());
          for (int j = 0; j < my; j++) {
            src[2 * j] = spline_at(yrun[j], ye.data(), re.data(), d2r.data(), N);
            src[2 * j + 1] = spline_at(yrun[j], ye.data(), im.data(), d2i.data(), N);
          }
          std::copy(src.begin(), src.end(), line);
        }
      }
    for (double *f : {u00, w00}) {
      for (int j = 0; j < mye; j++) re[j] = f[j];
      re[mye] = f[0];
      natural_spline(ye.data(), re.data(), N, d2r.data());
      for (int j = 0; j < my; j++) src[j] = spline_at(yrun[j], ye.data(), re.data(), d2r.data(), N);
      std::copy(src.begin(), src.begin() + my, f);
    }
  } else if (mye < my && ncopy > 0) {
    // ncopy_y (readwrite.f90:449-489): the box stacked ncopy times in y, copy
    // inc shifted by exp(-i kx xofft inc); the offsets grow by ncopy
    for (int k = 0; k < mz; k++)
      for (int i = 0; i < nkx; i++)
        for (int inc = 1; inc < ncopy; inc++) {
          const double ph = -(p->alp * i) * xofft * inc;
          const double cr = std::cos(ph), ci = std::sin(ph);
          for (double *f : {vor, phi}) {
            double *line = f + 2 * ((size_t)k * nkx + i) * my;
            for (int j = 0; j < mye; j++) {
              const double a = line[2 * j], b = line[2 * j + 1];
              line[2 * (j + mye * inc)] = a * cr - b * ci;
              line[2 * (j + mye * inc) + 1] = a * ci + b * cr;
            }
          }
        }
    xofft *= (double)ncopy;
    xoffb *= (double)ncopy;
    for (int inc = 1; inc < ncopy; inc++)
      for (int j = 0; j < mye; j++) {
        u00[j + mye * inc] = u00[j];
        w00[j + mye * inc] = w00[j];
      }
  }
  // velocity scale of a changed Lz, vorticity scale of a changed Re
  // (readwrite.f90:427-442; the Newton drivers keep the vorticity as read)
  const size_t nf = 2 * (size_t)my * nkx * mz;
  if (std::fabs(info->gam - p->gam) > tiny) {
    const double f = info->gam / p->gam;
    for (int j = 0; j < my; j++) {
      u00[j] *= f;
      w00[j] *= f;
    }
    for (size_t q = 0; q < nf; q++) phi[q] *= p->gam / info->gam;
    if (!p->les)
      for (size_t q = 0; q < nf; q++) vor[q] *= f * std::sqrt(p->Re / info->Re);
  } else if (std::fabs(info->Re - p->Re) > tiny && !p->les && !(flags & SB_RESTART_KEEP_VOR)) {
    for (size_t q = 0; q < nf; q++) vor[q] *= (info->gam / p->gam) * std::sqrt(p->Re / info->Re);
  }
  info->run_xoffb = xoffb;
  info->run_xofft = xofft;
  info->ymap = interp ? 3 : (ncopy > 0 && mye < my ? 2 : (ihalfy ? 1 : 0));
  info->ncopy = ncopy > 0 && mye < my ? ncopy : 0;
  info->xskip = iskip;
  return 0;
}

int sb_read_restart(const char *path, const sb_params *p, double *vor, double *phi, double *u00,
                    double *w00, sb_restart_info *info) {
  return sb_read_restart_ex(path, p, 0, vor, phi, u00, w00, info);
}

}  // extern "C"
