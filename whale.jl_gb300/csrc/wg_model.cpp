// Species-tree model on the host: slice tables [ε, ϕ, ψ] from the rates, the
// survival conditioning, and the adjoints of both (the chain from the DP's
// table adjoints back to the branch rates, WGD retention rates and η).
//
//   setmodel!/setnode!/setwgdnode!/setslices!   src/model.jl:162-191
//   getα, _ϵ, _ϕ, _ψ                             src/bdputil.jl:6-11
//   geompgf                                      src/bdputil.jl:67
//   condition (Root / NonExtinct / No)           src/condition.jl:11-29
//   NowhereExtinctCondition                      src/condition.jl:31-36
//   pgf of the linear BDP, treepgf_allbinary     src/bdputil.jl:84-135
#include <cmath>
#include <vector>

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

// pgf of the linear birth-death process over time t at s (src/bdputil.jl:
// 84-99; critical form when |λ - μ| <= 1e-6) with its partials in s, λ, μ.
inline double bdp_pgf(double lam, double mu, double t, double s, double& ds, double& dlam, double& dmu) {
  if (critical(lam, mu)) {
    const double u = s - 1.0, lt = lam * t;
    const double num = 1.0 - (lt - 1.0) * u, den = 1.0 - lt * u;
    ds = (-(lt - 1.0) * den + num * lt) / (den * den);
    dlam = (-t * u * den + num * t * u) / (den * den);
    dmu = 0.0;
    return num / den;
  }
  const double rho = std::exp((mu - lam) * t);
  const double a = lam * s - mu, u = s - 1.0;
  const double num = rho * a - mu * u, den = rho * a - lam * u;
  const double drho_dl = -t * rho, drho_dm = t * rho;
  const double dnum_ds = rho * lam - mu, dden_ds = rho * lam - lam;
  const double dnum_dl = drho_dl * a + rho * s, dden_dl = drho_dl * a + rho * s - u;
  const double dnum_dm = drho_dm * a - rho - u, dden_dm = drho_dm * a - rho;
  ds = (dnum_ds * den - num * dden_ds) / (den * den);
  dlam = (dnum_dl * den - num * dden_dl) / (den * den);
  dmu = (dnum_dm * den - num * dden_dm) / (den * den);
  return num / den;
}

// NowhereExtinctCondition: log(1 - Σ_{k<last} P_k s_k) over the joint pgf P
// of the leaf counts at every binary argument and its inclusion-exclusion
// signs s (treepgf_allbinary, src/bdputil.jl:114-135; the first child's
// index varies fastest).  With grad, reverse-mode adjoints of the per-node
// natural rates λ, μ, q and of η are added, scaled by `scale`.
constexpr int kNowhereMaxLeaves = 22;

double nowhere_condition(const Model& m, bool grad, double scale, std::vector<double>* d_lam,
                         std::vector<double>* d_mu, std::vector<double>* d_q, double* d_eta) {
  if (!m.from_rates) throw Error(WG_ESTATE, "NowhereExtinctCondition needs the model's rates (wg_model_set_rates)");
  const int K = m.K, r = K - 1;
  int nleaf = 0;
  for (int k = 0; k < K; ++k) nleaf += m.kind[k] == WG_NODE_LEAF;
  if (nleaf > kNowhereMaxLeaves)
    throw Error(WG_ERANGE, "NowhereExtinctCondition over more than 22 leaves (2^leaves pgf terms)");
  // forward: x_k (product of the children's outputs; leaves: [0, 1]) and v_k
  std::vector<std::vector<double>> x(K), v(K), sg(K);
  for (int k = 0; k < K; ++k) {  // children precede parents in the model order
    if (m.kind[k] == WG_NODE_LEAF) {
      x[k] = {0.0, 1.0};
      sg[k] = {1.0, -1.0};
    } else {
      x[k] = {1.0};
      sg[k] = {1.0};
      for (int c : {m.ch0[k], m.ch1[k]}) {
        if (c < 0) continue;
        std::vector<double> nx, ns;
        nx.reserve(x[k].size() * v[c].size());
        ns.reserve(nx.capacity());
        for (size_t j = 0; j < v[c].size(); ++j)
          for (size_t i = 0; i < x[k].size(); ++i) {
            nx.push_back(x[k][i] * v[c][j]);
            ns.push_back(sg[k][i] * sg[c][j]);
          }
        x[k].swap(nx);
        sg[k].swap(ns);
      }
    }
    const bool wgd = m.kind[k] == WG_NODE_WGD;
    const double qk = wgd ? m.q[k] : 0.0, t = m.slice_len[k] * (m.nrow[k] - 1);
    v[k].resize(x[k].size());
    for (size_t i = 0; i < x[k].size(); ++i) {
      const double y = wgd ? x[k][i] * (1.0 - qk + x[k][i] * qk) : x[k][i];
      double ds, dl, dm;
      v[k][i] = k == r ? geompgf(m.eta, y) : bdp_pgf(m.lam[k], m.mu[k], t, y, ds, dl, dm);
    }
  }
  double acc = 0.0;
  for (size_t i = 0; i + 1 < v[r].size(); ++i) acc += v[r][i] * sg[r][i];
  const double c = 1.0 - acc;
  const bool ok = c > 0.0 && c < 1.0;
  const double val = ok ? std::log(c) : -INFINITY;
  if (!grad || !ok) return val;
  // reverse: bar_v of each node, parents before children
  std::vector<std::vector<double>> bv(K);
  bv[r].assign(v[r].size(), 0.0);
  for (size_t i = 0; i + 1 < v[r].size(); ++i) bv[r][i] = -sg[r][i] / c;
  for (int k = r; k >= 0; --k) {
    if (bv[k].empty()) continue;
    const bool wgd = m.kind[k] == WG_NODE_WGD;
    const double qk = wgd ? m.q[k] : 0.0, t = m.slice_len[k] * (m.nrow[k] - 1);
    std::vector<double> bx(x[k].size());
    for (size_t i = 0; i < x[k].size(); ++i) {
      const double xi = x[k][i];
      const double y = wgd ? xi * (1.0 - qk + xi * qk) : xi;
      double dvdy;
      if (k == r) {
        const double d = 1.0 - (1.0 - m.eta) * y;
        dvdy = m.eta / (d * d);
        *d_eta += scale * bv[k][i] * (y * (1.0 - y) / (d * d));
      } else {
        double dl, dm;
        bdp_pgf(m.lam[k], m.mu[k], t, y, dvdy, dl, dm);
        (*d_lam)[k] += scale * bv[k][i] * dl;
        (*d_mu)[k] += scale * bv[k][i] * dm;
      }
      const double by = bv[k][i] * dvdy;
      if (wgd) {
        (*d_q)[k] += scale * by * (xi * xi - xi);
        bx[i] = by * (1.0 - qk + 2.0 * xi * qk);
      } else {
        bx[i] = by;
      }
    }
    if (m.kind[k] == WG_NODE_LEAF) continue;
    const int c0 = m.ch0[k], c1 = m.ch1[k];
    if (c1 < 0) {
      bv[c0] = bx;  // a WGD node's only child
      continue;
    }
    const size_t n0 = v[c0].size(), n1 = v[c1].size();
    bv[c0].assign(n0, 0.0);
    bv[c1].assign(n1, 0.0);
    for (size_t j = 0; j < n1; ++j)
      for (size_t i = 0; i < n0; ++i) {
        const double b = bx[i + n0 * j];
        bv[c0][i] += b * v[c1][j];
        bv[c1][j] += b * v[c0][i];
      }
  }
  return val;
}

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
    case WG_COND_NOWHERE:
      return nowhere_condition(m, false, 0.0, nullptr, nullptr, nullptr, nullptr);
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

void model_condition_rates_vjp(const Model& m, double scale, std::vector<double>& d_lam, std::vector<double>& d_mu,
                               std::vector<double>& d_q, double& d_eta) {
  if (m.cond != WG_COND_NOWHERE) return;
  d_lam.resize(m.K, 0.0);
  d_mu.resize(m.K, 0.0);
  d_q.resize(m.K, 0.0);
  nowhere_condition(m, true, scale, &d_lam, &d_mu, &d_q, &d_eta);
}

void model_condition_vjp(const Model& m, double scale, std::vector<double>& d_eps, double& d_eta) {
  const int r = m.K - 1;
  const double eta = m.eta;
  auto g_s = [&](double s) { const double d = 1.0 - (1.0 - eta) * s; return eta / (d * d); };
  auto g_eta = [&](double s) { const double d = 1.0 - (1.0 - eta) * s; return s * (1.0 - s) / (d * d); };
  auto top = [&](int k) { return m.row_off[k] + m.nrow[k] - 1; };
  if (m.cond == WG_COND_NONE || m.cond == WG_COND_NOWHERE) return;  // the latter: model_condition_rates_vjp
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
