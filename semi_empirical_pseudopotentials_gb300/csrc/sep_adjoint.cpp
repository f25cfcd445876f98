// sep_adjoint.cpp -- forward and backward entry points of the band-edge
// adjoint (dE/dtheta for the form-factor parameters theta = a0..a3 per
// species).  The reference has no gradients: it fits its parameters with a
// derivative-free Monte Carlo search (pseudopotFitting/fit.c:29-50).
//
// Forward:  theta --pot.c:35-63 + hamiltonian.c:91-94--> table v(r_k)
//           --read.c:105-108 (minus the last value)--> shifted table
//           --init.c:157-182 (GPU, sep_vbuild)--> V(r_g), installed in the context;
//           then sep_pipeline gives the Ritz pairs.
// Backward: dL/dE_k --Hellmann-Feynman (GPU)--> dL/dV(r_g) = dv sum_k dL/dE_k psi_k(r_g)^2
//           --V(r) backward (GPU)--> dL/dtable --shift adjoint--> dL/draw table
//           --transpose of the sine-transform Jacobian--> dL/da.
#include <cmath>
#include <string>
#include <vector>

#include "../../include/sep_gb300.h"
#include "sep_host.h"

namespace sep {
void set_error(const std::string& msg);
}

namespace {

constexpr int kTab = 1024;
constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.28318530717958647692;

int fail(const char* msg) {
  sep::set_error(msg);
  return SEP_ERR_ARG;
}

// Shifted tables of every type (filter/read.c:105-108 subtracts the last value).
void shifted_tables(long ntype, const double* params, double vol_per_atom, std::vector<double>& r,
                    std::vector<double>& v) {
  r.assign((size_t)ntype * kTab, 0.0);
  v.assign((size_t)ntype * kTab, 0.0);
  for (long t = 0; t < ntype; ++t) {
    double* rt = r.data() + t * kTab;
    double* vt = v.data() + t * kTab;
    sep::host::form_factor_table(params + 4 * t, vol_per_atom, rt, vt);
    const double last = vt[kTab - 1];
    for (int k = 0; k < kTab; ++k) vt[k] -= last;
  }
}

}  // namespace

extern "C" {

int sep_form_factor_backward(const double params[4], double vol_per_atom, const double* dtab,
                             double* dparams) {
  if (!params || !dtab || !dparams) return fail("sep_form_factor_backward: null argument");
  // adjoint of v_k <- v_k - v_{n-1}
  std::vector<double> d(dtab, dtab + kTab);
  double tail = 0.0;
  for (int k = 0; k < kTab - 1; ++k) tail += dtab[k];
  d[kTab - 1] = -tail;
  // q_i and r_k as the forward builds them (running sums)
  const double dq = 5.0 / (double)kTab;
  const double dr = 0.02 * kTwoPi / ((double)kTab * dq);
  std::vector<double> q(kTab), r(kTab);
  double run = 0.0;
  for (int i = 0; i < kTab; ++i, run += dq) q[i] = run;
  run = 0.0;
  for (int k = 0; k < kTab; ++k, run += dr) r[k] = run;
  // v_k = C_k sum_i q_i sin(q_i r_k) vq_i (k >= 1), v_0 = C_0 sum_i q_i^2 vq_i
  const double cube = std::pow(kTwoPi, 3.0);
  std::vector<double> wk(kTab);
  wk[0] = d[0] * (dq * 4.0 * kPi / cube);
  for (int k = 1; k < kTab; ++k) wk[k] = d[k] * (dq * 4.0 * kPi / (cube * r[k]));
  // vq_i = a0 (q^2 - a1) / (a2 e^{a3 q^2} + 1) * vol
  const double a0 = params[0], a1 = params[1], a2 = params[2], a3 = params[3];
  double g[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = 0; i < kTab; ++i) {
    double gv = wk[0] * q[i] * q[i];
    for (int k = 1; k < kTab; ++k) gv += wk[k] * q[i] * std::sin(q[i] * r[k]);
    const double q2 = q[i] * q[i];
    const double e = std::exp(a3 * q2);
    const double den = a2 * e + 1.0;
    const double num = q2 - a1;
    g[0] += gv * (num / den);
    g[1] += gv * (-a0 / den);
    g[2] += gv * (-a0 * num * e / (den * den));
    g[3] += gv * (-a0 * num * a2 * q2 * e / (den * den));
  }
  for (int j = 0; j < 4; ++j) dparams[j] = g[j] * vol_per_atom;
  return SEP_OK;
}

int sep_potential_from_params(sep_ctx* ctx, long natom, const double* xyz, const int* types,
                              const double* scale, long ntype, const double* params,
                              double vol_per_atom, const double mins[3], double* potl) {
  if (!ctx || !xyz || !types || !params || !mins || ntype < 1)
    return fail("sep_potential_from_params: bad argument");
  std::vector<double> r, v;
  shifted_tables(ntype, params, vol_per_atom, r, v);
  std::vector<long> n((size_t)ntype, kTab);
  return sep_vbuild(ctx, natom, xyz, types, scale, ntype, r.data(), v.data(), n.data(), kTab,
                    mins, potl, 1);
}

int sep_band_edge_backward(sep_ctx* ctx, long natom, const double* xyz, const int* types,
                           const double* scale, long ntype, const double* params,
                           double vol_per_atom, const double mins[3], const double* psi, long m,
                           const double* dL_dE, double* dparams) {
  if (!ctx || !xyz || !types || !params || !mins || !psi || !dL_dE || !dparams || ntype < 1 ||
      m < 1)
    return fail("sep_band_edge_backward: bad argument");
  long ngrid = 0;
  int st = sep_ctx_info(ctx, nullptr, nullptr, nullptr, &ngrid);
  if (st != SEP_OK) return st;
  std::vector<double> rho((size_t)ngrid);
  st = sep_hf_density(ctx, psi, m, dL_dE, rho.data());
  if (st != SEP_OK) return st;
  std::vector<double> r, v;
  shifted_tables(ntype, params, vol_per_atom, r, v);
  std::vector<long> n((size_t)ntype, kTab);
  std::vector<double> dtab((size_t)ntype * kTab);
  st = sep_vbuild_backward(ctx, natom, xyz, types, scale, ntype, r.data(), v.data(), n.data(), kTab,
                           mins, rho.data(), dtab.data(), nullptr);
  if (st != SEP_OK) return st;
  for (long t = 0; t < ntype; ++t) {
    st = sep_form_factor_backward(params + 4 * t, vol_per_atom, dtab.data() + t * kTab,
                                  dparams + 4 * t);
    if (st != SEP_OK) return st;
  }
  return SEP_OK;
}

}  // extern "C"
