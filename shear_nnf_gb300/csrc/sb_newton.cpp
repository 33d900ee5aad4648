// sb_newton.cpp -- batched Jacobian-vector products of the period map and the
// last statistics record, on top of the C-ABI (host code).
//
// sb_jv_batch is the finite-difference product of matvec_dns_disk3d
// (gmres_shear.f90:2666-2948, iopt_matvec 1 and 2) for a whole block of
// directions: every perturbed state is one member of the handle's batch and
// the members integrate to their end time together (calc_dns_disk3d,
// gmres_shear.f90:2951-3120), so a block of Krylov directions costs one
// batched integration instead of one integration per direction.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/shearbox.h"

namespace sb {
void set_error(const std::string &msg);  // the message sb_last_error returns (sb_api.cu)
const sb_params *handle_params(const sb_handle *h);
int handle_batch(const sb_handle *h);
int handle_trace_len(const sb_handle *h);
}  // namespace sb

namespace {

int fail(int code, const std::string &msg) {
  sb::set_error(msg);
  return code;
}

double norm2(const double *v, size_t n) {
  double s = 0.0;
  for (size_t q = 0; q < n; q++) s += v[q] * v[q];
  return std::sqrt(s);
}

// state vector [vor | phi | u00 | w00]: offsets of the four parts
struct Layout {
  size_t nf, my, n;  // doubles per spectral field, my, total
};

Layout layout_of(const sb_params *p) {
  int sz[8];
  sb_sizes(p, sz);
  Layout L;
  L.nf = 2 * (size_t)sz[7];  // sz[7] = nkx*mz*my complex entries per field
  L.my = (size_t)p->my;
  L.n = 2 * L.nf + 2 * L.my;
  return L;
}

// Integrates the states (each a Layout vector) from time0 over T, up to the
// handle's batch at a time; results overwrite the states.
int integrate(sb_handle *h, std::vector<std::vector<double>> &states, const Layout &L,
              double time0, double xoffb, double xofft, double T) {
  const int B = sb::handle_batch(h);
  const sb_params *p = sb::handle_params(h);
  for (size_t q0 = 0; q0 < states.size(); q0 += (size_t)B) {
    const int nm = (int)std::min<size_t>((size_t)B, states.size() - q0);
    int rc;
    for (int m = 0; m < B; m++) {
      const double *x = states[q0 + (m < nm ? m : 0)].data();
      if ((rc = sb_set_state(h, m, x, x + L.nf, x + 2 * L.nf, x + 2 * L.nf + L.my, time0, xoffb,
                             xofft)) ||
          (rc = sb_set_member_etime(h, m, time0 + T)))
        return rc;
    }
    std::vector<int> fin((size_t)nm, 0);
    for (int it = 0;; it++) {
      if (it > (1 << 20)) return fail(6, "sb_jv_batch: end time not reached");
      if ((rc = sb_step(h, 64))) return rc;
      int all = 1;
      for (int m = 0; m < nm; m++) {
        if (fin[(size_t)m]) continue;
        sb_status st;
        if ((rc = sb_get_status(h, m, &st))) return rc;
        if ((st.flags & 3) || ((st.flags & 4) && !p->keep_laminar))
          return fail(6, "sb_jv_batch: member " + std::to_string(q0 + m) + " stopped (flags " +
                             std::to_string(st.flags) + ")");
        fin[(size_t)m] = (st.flags & 8) ? 1 : 0;
        all &= fin[(size_t)m];
      }
      if (all) break;
    }
    for (int m = 0; m < nm; m++) {
      double *x = states[q0 + m].data();
      double t, xb, xt;
      if ((rc = sb_get_state(h, m, x, x + L.nf, x + 2 * L.nf, x + 2 * L.nf + L.my, &t, &xb, &xt)))
        return rc;
    }
  }
  return 0;
}

}  // namespace

extern "C" {

int sb_stats(sb_handle *h, int member, double *uner, double *uner2) {
  if (!h || !uner || !uner2) return fail(1, "null argument");
  sb_status st;
  int rc = sb_get_status(h, member, &st);
  if (rc) return rc;
  if (st.ntrace < 1) return fail(6, "no statistics record in the last sb_step");
  const int len = sb::handle_trace_len(h);
  std::vector<double> rec((size_t)st.ntrace * (size_t)len);
  int n = 0;
  if ((rc = sb_get_trace(h, member, rec.data(), st.ntrace, &n))) return rc;
  if (n < 1) return fail(6, "no statistics record in the last sb_step");
  const double *r = rec.data() + (size_t)(n - 1) * (size_t)len;
  for (int q = 0; q < 10; q++) uner[q] = r[2 + q];
  for (int q = 0; q < 4; q++) uner2[q] = r[20 + q];
  return 0;
}

int sb_jv_batch(sb_handle *h, const double *x0, double time0, double xoffb, double xofft,
                double T, const double *dirs, int ndir, double eps_jacobi, int central,
                double *out) {
  if (!h || !x0 || !dirs || !out) return fail(1, "null argument");
  if (ndir < 1) return fail(1, "ndir must be >= 1");
  if (!(T > 0.0) || !(eps_jacobi > 0.0)) return fail(1, "T and eps_jacobi must be positive");
  const sb_params *p = sb::handle_params(h);
  if (p->temperature) return fail(2, "sb_jv_batch: the temperature variant is not supported");
  const Layout L = layout_of(p);
  const double xn = norm2(x0, L.n);
  const double eps_j = eps_jacobi * (xn > 0.0 ? xn : 1.0);
  std::vector<double> eps((size_t)ndir);
  std::vector<std::vector<double>> states;
  if (!central) states.emplace_back(x0, x0 + L.n);
  for (int q = 0; q < ndir; q++) {
    const double *d = dirs + (size_t)q * L.n;
    const double dn = norm2(d, L.n);
    if (!(dn > 0.0)) return fail(1, "sb_jv_batch: zero direction " + std::to_string(q));
    eps[(size_t)q] = eps_j / dn;
    for (int sgn = 1; sgn >= (central ? -1 : 1); sgn -= 2) {
      std::vector<double> x(L.n);
      for (size_t i = 0; i < L.n; i++) {
        // the representable step h = (x0 + eps d) - x0 (iuse_hej)
        const double hstep = (x0[i] + (sgn * eps[(size_t)q]) * d[i]) - x0[i];
        x[i] = x0[i] + hstep;
      }
      states.push_back(std::move(x));
    }
  }
  int rc = integrate(h, states, L, time0, xoffb, xofft, T);
  if (rc) return rc;
  for (int q = 0; q < ndir; q++) {
    double *o = out + (size_t)q * L.n;
    if (central) {
      const std::vector<double> &a = states[2 * (size_t)q], &b = states[2 * (size_t)q + 1];
      for (size_t i = 0; i < L.n; i++) o[i] = (a[i] - b[i]) / (2.0 * eps[(size_t)q]);
    } else {
      const std::vector<double> &a = states[1 + (size_t)q], &b = states[0];
      for (size_t i = 0; i < L.n; i++) o[i] = (a[i] - b[i]) / eps[(size_t)q];
    }
  }
  return 0;
}

}  // extern "C"
