// sb_host.cpp -- host-side set-up: compact coefficients, base factorisations,
// seeded initial fields.  Pure C++ (no CUDA calls).
#include "sb_host.h"

#include <cmath>
#include <complex>
#include <cstring>

namespace sbh {

// Gauss-Jordan elimination with full pivoting (the Numerical Recipes routine
// used by the reference, diffy_shear_hepta.f90:1125-1203).  a is n x n
// column-major, b is n x 1.  The pivot order follows the reference so that the
// compact coefficients come out bit-identical.
static void gauss_jordan(double *a, int n, double *b) {
  auto A = [&](int r, int c) -> double & { return a[(c - 1) * n + (r - 1)]; };
  int indxc[50], indxr[50], ipiv[50];
  int irow = 0, icol = 0;
  for (int j = 0; j < n; j++) ipiv[j] = 0;
  for (int i = 1; i <= n; i++) {
    double big = 0.0;
    for (int j = 1; j <= n; j++)
      if (ipiv[j - 1] != 1)
        for (int k = 1; k <= n; k++)
          if (ipiv[k - 1] == 0 && std::fabs(A(j, k)) >= big) {
            big = std::fabs(A(j, k));
            irow = j;
            icol = k;
          }
    ipiv[icol - 1] += 1;
    if (irow != icol) {
      for (int l = 1; l <= n; l++) std::swap(A(irow, l), A(icol, l));
      std::swap(b[irow - 1], b[icol - 1]);
    }
    indxr[i - 1] = irow;
    indxc[i - 1] = icol;
    double pivinv = 1.0 / A(icol, icol);
    A(icol, icol) = 1.0;
    for (int l = 1; l <= n; l++) A(icol, l) = A(icol, l) * pivinv;
    b[icol - 1] = b[icol - 1] * pivinv;
    for (int ll = 1; ll <= n; ll++)
      if (ll != icol) {
        double dum = A(ll, icol);
        A(ll, icol) = 0.0;
        for (int l = 1; l <= n; l++) A(ll, l) = A(ll, l) - A(icol, l) * dum;
        b[ll - 1] = b[ll - 1] - b[icol - 1] * dum;
      }
  }
  for (int l = n; l >= 1; l--)
    if (indxr[l - 1] != indxc[l - 1])
      for (int k = 1; k <= n; k++) std::swap(A(k, indxr[l - 1]), A(k, indxc[l - 1]));
}

static int ipow(int b, int e) {
  int r = 1;
  for (int q = 0; q < e; q++) r *= b;
  return r;
}

void filter_coeffs(double lhs[7], double rhs[9]) {
  // the filter's design (transfer 0 at pi, 0.72 at 6pi/9, 0.001 at 8.5pi/9,
  // 0.91 at 5.5pi/9) is fixed in the reference as decimal constants
  const double l[4] = {1.0, 0.738981897704866, 0.315003368623046, 0.053003478448814};
  const double r[5] = {0.987412035368317, 0.749052269410218, 0.309968182770373,
                       0.054442102978149, -0.000179828066167};
  for (int d = 0; d <= 3; d++) lhs[3 + d] = lhs[3 - d] = l[d];
  for (int d = 0; d <= 4; d++) rhs[4 + d] = rhs[4 - d] = r[d];
}

void compact_coeffs(Coeffs *c) {
  const int N = 3, M = 3;
  const double pi = 4.0 * std::atan(1.0);
  {  // first derivative: order conditions 1,3,5 (2N-M of them) + M spectral points
    double kap[3] = {0.5, 0.9, 0.0};
    kap[2] = 0.5 * (kap[0] + kap[1]);
    for (double &k : kap) k *= pi;
    double mat[36] = {0}, vec[6] = {0};
    auto Mt = [&](int r, int cc) -> double & { return mat[(cc - 1) * 6 + (r - 1)]; };
    for (int k = 1; k <= 2 * N - M; k++) {
      int kk = 2 * k - 1;
      for (int j = 1; j <= N; j++) {
        Mt(k, j) = (double)(kk * ipow(j, kk - 1));
        Mt(k, N + j) = -(double)ipow(j, kk);
      }
    }
    vec[0] = -0.5;
    for (int k = 1; k <= M; k++) {
      for (int j = 1; j <= N; j++) {
        Mt(2 * N - M + k, j) = kap[k - 1] * std::cos(kap[k - 1] * (double)j);
        Mt(2 * N - M + k, N + j) = -std::sin(kap[k - 1] * (double)j);
      }
      vec[2 * N - M + k - 1] = -0.5 * kap[k - 1];
    }
    gauss_jordan(mat, 2 * N, vec);
    for (int j = 1; j <= N; j++) {
      c->rh1h[3 + j] = vec[N + j - 1];
      c->rh1h[3 - j] = -vec[N + j - 1];
      c->pr1[3 + j] = vec[j - 1];
      c->pr1[3 - j] = vec[j - 1];
    }
    c->rh1h[3] = 0.0;
    c->pr1[3] = 1.0;
  }
  {  // second derivative
    double kap[3] = {0.9, 0.5, 0.0};
    kap[2] = 0.5 * (kap[0] + kap[1]);
    for (double &k : kap) k *= pi;
    double mat[49] = {0}, vec[7] = {0};
    auto Mt = [&](int r, int cc) -> double & { return mat[(cc - 1) * 7 + (r - 1)]; };
    for (int j = N + 2; j <= 2 * N + 1; j++) Mt(1, j) = 1.0;
    Mt(1, N + 1) = 0.5;
    for (int k = 2; k <= 2 * N + 1 - M; k++) {
      int kk = 2 * k - 2;
      for (int j = 1; j <= N; j++) {
        Mt(k, j) = (double)(kk * (kk - 1) * ipow(j, kk - 2));
        Mt(k, N + 1 + j) = -(double)ipow(j, kk);
      }
    }
    vec[1] = -1.0;
    for (int k = 1; k <= M; k++)
      for (int j = 1; j <= N; j++) {
        Mt(2 * N + 1 - M + k, j) = kap[k - 1] * kap[k - 1] * std::cos(kap[k - 1] * (double)j);
        Mt(2 * N + 1 - M + k, N + 1 + j) = std::cos(kap[k - 1] * (double)j);
      }
    for (int r = 2 * N + 2 - M; r <= 2 * N + 1; r++) {
      double kp = kap[r - (2 * N + 2 - M)];
      Mt(r, N + 1) = 0.5;
      vec[r - 1] = -0.5 * kp * kp;
    }
    gauss_jordan(mat, 2 * N + 1, vec);
    for (int j = 1; j <= N; j++) {
      c->rh2h[3 + j] = vec[N + j];
      c->rh2h[3 - j] = vec[N + j];
      c->pr2[3 + j] = vec[j - 1];
      c->pr2[3 - j] = vec[j - 1];
    }
    c->rh2h[3] = vec[N];
    c->pr2[3] = 1.0;
  }
}

void base_factor(const double a[7], int n, BaseFac *o) {
  // 1-based working arrays
  std::vector<double> La(n + 4, 0.0), Lb(n + 4, 0.0), Lc(n + 4, 0.0), Dd(n + 4, 0.0),
      Dm(n + 4, 0.0), e(n + 4, 0.0), f(n + 4, 0.0), g(n + 4, 0.0);
  const double a0 = a[3], a1 = a[4], a2 = a[5], a3 = a[6];
  // banded part, rows 1..n-3 (independent of the shear phase); the order of
  // the sums follows modChol7cyclic_cmplx
  for (int j = 1; j <= n - 3; j++) {
    double s = 0.0;
    if (j == 2) s = La[j] * Dd[j - 1] * La[j];
    if (j == 3) s = Lb[j] * Dd[j - 2] * Lb[j] + La[j] * Dd[j - 1] * La[j];
    if (j >= 4) s = Lc[j] * Dd[j - 3] * Lc[j] + Lb[j] * Dd[j - 2] * Lb[j] + La[j] * Dd[j - 1] * La[j];
    Dd[j] = (j == 1) ? a0 : a0 - s;
    Dm[j] = 1.0 / Dd[j];
    if (j + 1 <= n - 3) {
      double t = 0.0;
      if (j == 2) t = Lb[j + 1] * Dd[j - 1] * La[j];
      if (j >= 3) t = Lc[j + 1] * Dd[j - 2] * Lb[j] + Lb[j + 1] * Dd[j - 1] * La[j];
      La[j + 1] = (j == 1) ? Dm[j] * a1 : Dm[j] * (a1 - t);
    }
    if (j + 2 <= n - 3) Lb[j + 2] = (j == 1) ? Dm[j] * a2 : Dm[j] * (a2 - Lc[j + 2] * Dd[j - 1] * La[j]);
    if (j + 3 <= n - 3) Lc[j + 3] = Dm[j] * a3;
  }
  // border rows with the shear phase factored out
  auto rec = [&](std::vector<double> &L, int i, double rhs) {
    double t = rhs;
    if (i >= 4) t -= L[i - 3] * Dd[i - 3] * Lc[i];
    if (i >= 3) t -= L[i - 2] * Dd[i - 2] * Lb[i];
    if (i >= 2) t -= L[i - 1] * Dd[i - 1] * La[i];
    L[i] = Dm[i] * t;
  };
  for (int i = 1; i <= n - 6; i++) rec(e, i, i == 1 ? a3 : 0.0);
  for (int i = 1; i <= n - 5; i++) rec(f, i, i == 1 ? a2 : (i == 2 ? a3 : 0.0));
  for (int i = 1; i <= n - 4; i++) rec(g, i, i == 1 ? a1 : (i == 2 ? a2 : (i == 3 ? a3 : 0.0)));
  double See = 0, Sfe = 0, Sff = 0, Sge = 0, Sgf = 0, Sgg = 0;
  for (int k = 1; k <= n - 6; k++) {
    See += e[k] * e[k] * Dd[k];
    Sfe += f[k] * e[k] * Dd[k];
    Sge += g[k] * e[k] * Dd[k];
  }
  for (int k = 1; k <= n - 5; k++) {
    Sff += f[k] * f[k] * Dd[k];
    Sgf += g[k] * f[k] * Dd[k];
  }
  for (int k = 1; k <= n - 4; k++) Sgg += g[k] * g[k] * Dd[k];
  o->La.assign(n, 0.0);
  o->Lb.assign(n, 0.0);
  o->Lc.assign(n, 0.0);
  o->Dd.assign(n, 0.0);
  o->Ddm1.assign(n, 0.0);
  o->e.assign(n, 0.0);
  o->f.assign(n, 0.0);
  o->g.assign(n, 0.0);
  for (int i = 1; i <= n; i++) {
    o->La[i - 1] = La[i];
    o->Lb[i - 1] = Lb[i];
    o->Lc[i - 1] = Lc[i];
    o->Dd[i - 1] = Dd[i];
    o->Ddm1[i - 1] = Dm[i];
    o->e[i - 1] = e[i];
    o->f[i - 1] = f[i];
    o->g[i - 1] = g[i];
  }
  o->sums[0] = See;
  o->sums[1] = Sfe;
  o->sums[2] = Sff;
  o->sums[3] = Sge;
  o->sums[4] = Sgf;
  o->sums[5] = Sgg;
}

void seg_plan(int n, int nseg, SegPlan *p) {
  const int m = n - 3;  // banded rows 1..n-3
  p->nseg = nseg;
  int lo = 1;
  for (int s = 0; s < nseg; s++) {
    const int size = m / nseg + (s < m % nseg ? 1 : 0);
    p->lo[s] = lo;
    p->hi[s] = lo + size - 1;
    lo += size;
  }
}

void seg_factor(const BaseFac &b, int n, const SegPlan &p, SegFac *o) {
  auto at = [&](const std::vector<double> &v, int i) { return (i >= 1 && i <= n) ? v[i - 1] : 0.0; };
  for (int t = 0; t < 3; t++) {
    o->hf[t].assign(n, 0.0);
    o->hb[t].assign(n, 0.0);
  }
  o->ef.assign(9 * (size_t)p.nseg, 0.0);
  for (int s = 0; s < p.nseg; s++) {
    const int lo = p.lo[s], hi = p.hi[s];
    for (int t = 1; t <= 3; t++) {
      // forward: state h[lo-1], h[lo-2], h[lo-3] with h[lo-t] = 1
      std::vector<double> h(n + 8, 0.0);
      auto H = [&](int i) -> double & { return h[i + 4]; };
      H(lo - t) = 1.0;
      for (int i = lo; i <= hi; i++)
        H(i) = -at(b.Lc, i) * H(i - 3) - at(b.Lb, i) * H(i - 2) - at(b.La, i) * H(i - 1);
      double se = 0, sf = 0, sg = 0;
      for (int i = lo; i <= hi; i++) {
        o->hf[t - 1][i - 1] = H(i);
        se += at(b.e, i) * H(i);
        sf += at(b.f, i) * H(i);
        sg += at(b.g, i) * H(i);
      }
      o->ef[(s * 3 + 0) * 3 + t - 1] = se;
      o->ef[(s * 3 + 1) * 3 + t - 1] = sf;
      o->ef[(s * 3 + 2) * 3 + t - 1] = sg;
      if (s < p.nseg - 1) {
        std::vector<double> gq(n + 8, 0.0);
        auto Gq = [&](int i) -> double & { return gq[i]; };
        Gq(hi + t) = 1.0;
        for (int i = hi; i >= lo; i--)
          Gq(i) = -at(b.La, i + 1) * Gq(i + 1) - at(b.Lb, i + 2) * Gq(i + 2) -
                  at(b.Lc, i + 3) * Gq(i + 3);
        for (int i = lo; i <= hi; i++) o->hb[t - 1][i - 1] = Gq(i);
      }
    }
  }
}

// SplitMix64: counter-based so that every (seed, mode) pair has its own stream
static inline uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
static inline double u01(uint64_t seed, uint64_t ctr) {
  uint64_t r = splitmix(seed * 0x632BE59BD9B4E019ull + splitmix(ctr));
  return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

int seed_state(int mgalx, int my, int mgalz, double alp, double gam, double Ly, uint64_t seed,
               double k0, double urms, double *vor, double *phi, double *u00, double *w00) {
  typedef std::complex<double> C;
  const double pi = 4.0 * std::atan(1.0);
  const int mx = 2 * (mgalx / 3), mz = 2 * (mgalz / 3) - 1;
  const int nkx = mx / 2, nz = (mz - 1) / 2;
  const int ny = my / 3;  // y modes kept: |n| <= my/3 (no aliasing on the y grid)
  const double bet = 2.0 * pi / Ly;
  const int nyf = 2 * ny + 1;
  // 3-D spectral velocity u_hat(kx_i, ky_n, kz_k); kx >= 0 only
  std::vector<C> uh((size_t)nkx * nyf * mz * 3, C(0, 0));
  auto U = [&](int i, int n, int k, int c) -> C & {
    return uh[(((size_t)i * nyf + (n + ny)) * mz + k) * 3 + c];
  };
  auto kzv = [&](int k) { return (k <= nz) ? (double)k : -(double)(mz - k); };
  for (int i = 0; i < nkx; i++)
    for (int n = -ny; n <= ny; n++)
      for (int k = 0; k < mz; k++) {
        double kx = alp * i, ky = bet * n, kz = gam * kzv(k);
        double kk = std::sqrt(kx * kx + ky * ky + kz * kz);
        if (kk == 0.0) continue;
        if (i == 0) {
          // kx = 0 half-plane: keep (ky, kz) with kz > 0, or kz = 0 and ky > 0;
          // the rest follows from Hermitian symmetry below
          double kzs = kzv(k);
          if (kzs < 0 || (kzs == 0 && n <= 0)) continue;
        }
        uint64_t ctr = ((uint64_t)i * 4096 + (uint64_t)(n + 2048)) * 4096 + (uint64_t)k;
        double r1 = u01(seed, 4 * ctr), r2 = u01(seed, 4 * ctr + 1), r3 = u01(seed, 4 * ctr + 2);
        // amplitude: E(k) ~ k^4 exp(-2 (k/k0)^2) spread over a shell of area ~ k^2
        double ek = std::pow(kk, 4.0) * std::exp(-2.0 * (kk / k0) * (kk / k0));
        double amp = std::sqrt(ek / (kk * kk));
        // two unit vectors orthogonal to k
        double kv[3] = {kx / kk, ky / kk, kz / kk};
        double t[3] = {0, 0, 0};
        int m = (std::fabs(kv[0]) < 0.6) ? 0 : ((std::fabs(kv[1]) < 0.6) ? 1 : 2);
        t[m] = 1.0;
        double d = t[0] * kv[0] + t[1] * kv[1] + t[2] * kv[2];
        double e1[3], e2[3];
        for (int q = 0; q < 3; q++) e1[q] = t[q] - d * kv[q];
        double nrm = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        for (int q = 0; q < 3; q++) e1[q] /= nrm;
        e2[0] = kv[1] * e1[2] - kv[2] * e1[1];
        e2[1] = kv[2] * e1[0] - kv[0] * e1[2];
        e2[2] = kv[0] * e1[1] - kv[1] * e1[0];
        double th = 2.0 * pi * r3;
        C p1 = std::polar(amp, 2.0 * pi * r1), p2 = std::polar(amp, 2.0 * pi * r2);
        for (int q = 0; q < 3; q++) U(i, n, k, q) = std::cos(th) * p1 * e1[q] + std::sin(th) * p2 * e2[q];
      }
  // Hermitian completion of the kx = 0 plane: u(0,-n,-kz) = conj(u(0,n,kz))
  for (int n = -ny; n <= ny; n++)
    for (int k = 0; k < mz; k++) {
      double kzs = kzv(k);
      if (kzs < 0 || (kzs == 0 && n < 0)) {
        int kneg = (k == 0) ? 0 : mz - k;
        for (int q = 0; q < 3; q++) U(0, n, k, q) = std::conj(U(0, -n, kneg, q));
      }
    }
  // rms scaling: <u.u>/3 = urms^2 (kx > 0 modes count twice)
  double e = 0.0;
  for (int i = 0; i < nkx; i++)
    for (int n = -ny; n <= ny; n++)
      for (int k = 0; k < mz; k++)
        for (int q = 0; q < 3; q++) e += (i == 0 ? 1.0 : 2.0) * std::norm(U(i, n, k, q));
  double sc = (e > 0) ? urms / std::sqrt(e / 3.0) : 0.0;
  // synthesise y on the grid: v and omega_y = d u/dz - d w/dx; phi = lap v
  std::vector<double> y(my);
  for (int j = 0; j < my; j++) y[j] = j * (Ly / my) - 0.5 * Ly;
  std::memset(vor, 0, sizeof(double) * 2 * (size_t)my * nkx * mz);
  std::memset(phi, 0, sizeof(double) * 2 * (size_t)my * nkx * mz);
  for (int j = 0; j < my; j++) {
    u00[j] = 0.0;
    w00[j] = 0.0;
  }
  for (int k = 0; k < mz; k++)
    for (int i = 0; i < nkx; i++) {
      double kx = alp * i, kz = gam * kzv(k);
      for (int j = 0; j < my; j++) {
        C v(0, 0), om(0, 0), ph(0, 0), uu(0, 0), ww(0, 0);
        for (int n = -ny; n <= ny; n++) {
          double ky = bet * n;
          C ex = std::polar(1.0, ky * (y[j] + 0.5 * Ly));
          C uh0 = U(i, n, k, 0) * sc, uh1 = U(i, n, k, 1) * sc, uh2 = U(i, n, k, 2) * sc;
          v += uh1 * ex;
          om += (C(0, kz) * uh0 - C(0, kx) * uh2) * ex;
          ph += -(kx * kx + ky * ky + kz * kz) * uh1 * ex;
          uu += uh0 * ex;
          ww += uh2 * ex;
        }
        size_t o = 2 * ((size_t)my * ((size_t)k * nkx + i) + j);
        if (i == 0 && k == 0) {
          u00[j] = uu.real();
          w00[j] = ww.real();
          continue;  // v00 = 0 by continuity; omega_y mean = 0
        }
        vor[o] = om.real();
        vor[o + 1] = om.imag();
        phi[o] = ph.real();
        phi[o + 1] = ph.imag();
      }
    }
  return 0;
}

std::vector<double> fft_twiddles(int n) {
  const double pi = 4.0 * std::atan(1.0);
  std::vector<double> v(2 * (size_t)n);
  for (int t = 0; t < n; t++) {
    const double a = -2.0 * pi * (double)t / (double)n;
    v[2 * t] = std::cos(a);
    v[2 * t + 1] = std::sin(a);
  }
  return v;
}

std::vector<double> fft_twiddles_factored(int n) {
  const double pi = 4.0 * std::atan(1.0);
  std::vector<double> v(4 * (size_t)n);
  for (int t = 0; t < n; t++) {
    const int q = ((8 * t + n) / (2 * n)) % 4;
    const double a = pi * (double)(q * n - 4 * t) / (2.0 * (double)n);  // -2 pi t/n + q pi/2
    const double c = std::cos(a);
    const long long sw = q & 1;
    const double mx = (q <= 1) ? c : -c;
    v[4 * t] = mx;
    v[4 * t + 1] = sw ? -mx : mx;
    v[4 * t + 2] = std::sin(a) / c;
    std::memcpy(&v[4 * t + 3], &sw, sizeof(double));
  }
  return v;
}

}  // namespace sbh
