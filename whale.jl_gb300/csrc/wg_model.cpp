// Species-tree model on the host: slice tables [ε, ϕ, ψ] from the rates, the
// survival conditioning, and the adjoints of both (the chain from the DP's
// table adjoints back to the branch rates, WGD retention rates and η).
//
//   setmodel!/setnode!/setwgdnode!/setslices!   src/model.jl:162-191
//   getα, _ϵ, _ϕ, _ψ                             src/bdputil.jl:6-11
//   geompgf                                      src/bdputil.jl:67
//   condition (Root / NonExtinct / No)           src/condition.jl:11-29
#include <cmath>

#include "wg_internal.h"

namespace wg {

namespace {

constexpr double kCriticalAtol = 1e-6;  // ΛMATOL, src/bdputil.jl:1

inline bool critical(double lam, double mu) { return std::fabs(lam - mu) <= kCriticalAtol; }

// getα (src/bdputil.jl:6-7) and its partial derivatives.
inline double alpha(double lam, double mu, double t) {
  if (critical(lam, mu)) return lam * t / (1.0 + lam * t);
  const double e = std::exp(t * (lam - mu));
  return mu * (e - 1.0) / (lam * e - mu);
}

inline void alpha_grad(double lam, double mu, double t, double& da_dlam, double& da_dmu) {
  if (critical(lam, mu)) {
    const double d = 1.0 + lam * t;
    da_dlam = t / (d * d);
    da_dmu = 0.0;
    return;
  }
  const double e = std::exp(t * (lam - mu));
  const double num = mu * (e - 1.0), den = lam * e - mu;
  const double dnum_dl = mu * t * e, dden_dl = e + lam * t * e;
  const double dnum_dm = (e - 1.0) - mu * t * e, dden_dm = -lam * t * e - 1.0;
  da_dlam = (dnum_dl * den - num * dden_dl) / (den * den);
  da_dmu = (dnum_dm * den - num * dden_dm) / (den * den);
}

inline double geompgf(double p, double s) { return p * s / (1.0 - (1.0 - p) * s); }

}  // namespace

void model_fill_tables(Model& m) {
  const int K = m.K;
  m.eps.assign(m.total_rows(), 1.0);
  m.phi.assign(m.total_rows(), 1.0);
  m.psi.assign(m.total_rows(), 1.0);
  for (int k = 0; k < K; ++k) {
    const int o = m.row_off[k];
    double* E = &m.eps[o];
    double* F = &m.phi[o];
    double* S = &m.psi[o];
    if (m.kind[k] == WG_NODE_WGD) {
      const double e = m.eps_top(m.ch0[k]);
      E[0] = m.q[k] * e * e + (1.0 - m.q[k]) * e;
    } else {
      if (m.kind[k] == WG_NODE_LEAF) {
        E[0] = m.p.empty() ? 0.0 : m.p[k];
      } else {
        E[0] = m.eps_top(m.ch0[k]) * m.eps_top(m.ch1[k]);
      }
      F[0] = 1.0;
    }
    const double lam = m.lam[k], mu = m.mu[k];
    for (int i = 1; i < m.nrow[k]; ++i) {
      const double a = alpha(lam, mu, m.slice_len[k]);
      const double b = (lam / mu) * a;
      const double e = E[i - 1];
      const double d = 1.0 - b * e;
      E[i] = (a + (1.0 - a - b) * e) / d;
      F[i] = (1.0 - a) * (1.0 - b) / (d * d);
      S[i] = (1.0 - a) * (1.0 - b) * b / (d * d * d);
    }
  }
}

double model_condition(const Model& m) {
  const int r = m.K - 1;
  switch (m.cond) {
    case WG_COND_NONE:
      return 0.0;
    case WG_COND_NONEXTINCT:
      return std::log(1.0 - geompgf(m.eta, m.eps_top(r)));
    default: {
      const double er = geompgf(m.eta, m.eps_top(r));
      const double ef = geompgf(m.eta, m.eps_top(m.ch0[r]));
      const double eg = geompgf(m.eta, m.eps_top(m.ch1[r]));
      const double p = 1.0 - ef - eg + er;
      return p > 0.0 ? std::log(p) : -INFINITY;
    }
  }
}

void model_condition_vjp(const Model& m, double scale, std::vector<double>& d_eps, double& d_eta) {
  const int r = m.K - 1;
  const double eta = m.eta;
  auto g_s = [&](double s) { const double d = 1.0 - (1.0 - eta) * s; return eta / (d * d); };
  auto g_eta = [&](double s) { const double d = 1.0 - (1.0 - eta) * s; return s * (1.0 - s) / (d * d); };
  auto top = [&](int k) { return m.row_off[k] + m.nrow[k] - 1; };
  if (m.cond == WG_COND_NONE) return;
  if (m.cond == WG_COND_NONEXTINCT) {
    const double s = m.eps_top(r);
    const double P = 1.0 - geompgf(eta, s);
    d_eps[top(r)] += scale * (-g_s(s) / P);
    d_eta += scale * (-g_eta(s) / P);
    return;
  }
  const double sr = m.eps_top(r), sf = m.eps_top(m.ch0[r]), sg = m.eps_top(m.ch1[r]);
  const double P = 1.0 - geompgf(eta, sf) - geompgf(eta, sg) + geompgf(eta, sr);
  if (!(P > 0.0)) return;
  d_eps[top(m.ch0[r])] += scale * (-g_s(sf) / P);
  d_eps[top(m.ch1[r])] += scale * (-g_s(sg) / P);
  d_eps[top(r)] += scale * (g_s(sr) / P);
  d_eta += scale * ((-g_eta(sf) - g_eta(sg) + g_eta(sr)) / P);
}

void model_tables_vjp(const Model& m, std::vector<double> d_eps, const std::vector<double>& d_phi,
                      const std::vector<double>& d_psi, std::vector<double>& d_lam,
                      std::vector<double>& d_mu, std::vector<double>& d_q, std::vector<double>& d_p) {
  const int K = m.K;
  d_lam.assign(K, 0.0);
  d_mu.assign(K, 0.0);
  d_p.assign(K, 0.0);
  if ((int)d_q.size() != K) d_q.assign(K, 0.0);
  for (int k = K - 1; k >= 0; --k) {
    const int o = m.row_off[k];
    const double lam = m.lam[k], mu = m.mu[k], t = m.slice_len[k];
    double bar_a = 0.0, bar_b = 0.0;
    double a = 0.0, b = 0.0;
    if (m.nrow[k] > 1) {
      a = alpha(lam, mu, t);
      b = (lam / mu) * a;
    }
    for (int i = m.nrow[k] - 1; i >= 1; --i) {
      const double e = m.eps[o + i - 1];
      const double d = 1.0 - b * e;
      const double u = (1.0 - a) * (1.0 - b);
      const double be = d_eps[o + i], bf = d_phi[o + i], bs = d_psi[o + i];
      const double d2 = d * d, d3 = d2 * d, d4 = d3 * d;
      // ε_i
      double de = be * (u / d2);
      bar_a += be * ((1.0 - e) / d);
      bar_b += be * (-e * (1.0 - a) * (1.0 - e) / d2);
      // ϕ_i = u / d²
      de += bf * (2.0 * u * b / d3);
      bar_a += bf * (-(1.0 - b) / d2);
      bar_b += bf * (-(1.0 - a) / d2 + 2.0 * u * e / d3);
      // ψ_i = u β / d³
      de += bs * (3.0 * u * b * b / d4);
      bar_a += bs * (-(1.0 - b) * b / d3);
      bar_b += bs * ((1.0 - a) * (1.0 - 2.0 * b) / d3 + 3.0 * u * b * e / d4);
      d_eps[o + i - 1] += de;
    }
    if (m.nrow[k] > 1) {
      // β = (λ/μ) α
      bar_a += bar_b * (lam / mu);
      d_lam[k] += bar_b * a / mu;
      d_mu[k] += -bar_b * lam * a / (mu * mu);
      double da_dl, da_dm;
      alpha_grad(lam, mu, t, da_dl, da_dm);
      d_lam[k] += bar_a * da_dl;
      d_mu[k] += bar_a * da_dm;
    }
    // bottom ε (row 0)
    const double b0 = d_eps[o];
    if (m.kind[k] == WG_NODE_WGD) {
      const int c = m.ch0[k];
      const double e = m.eps_top(c);
      d_q[k] += b0 * (e * e - e);
      d_eps[m.row_off[c] + m.nrow[c] - 1] += b0 * (2.0 * m.q[k] * e + 1.0 - m.q[k]);
    } else if (m.kind[k] == WG_NODE_LEAF) {
      d_p[k] += b0;
    } else {
      const int f = m.ch0[k], g = m.ch1[k];
      d_eps[m.row_off[f] + m.nrow[f] - 1] += b0 * m.eps_top(g);
      d_eps[m.row_off[g] + m.nrow[g] - 1] += b0 * m.eps_top(f);
    }
  }
}

}  // namespace wg
