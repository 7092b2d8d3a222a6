// Stochastic backtracking of reconciled gene trees from one family's DP
// tables (src/track.jl:180-488): starting from the ubiquitous clade at the
// root, every latent state (species node e, clade γ, slice t) draws the event
// that produced it with probability proportional to its term in the DP
// recursion, in the reference's event order; the sampled states form a
// reconciled tree, post-processed into node heights and event labels as
// process_rectree / node_heights / getlabel do (src/track.jl:405-488).
//
// Tables: for every node k (model order), nrow[k] rows (row r = slice
// t = r + 1, t = 1 the leafward boundary) of the family's compatible clades in
// ascending clade id; incompatible clades read 0 (getl, src/ccd.jl:41-49).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <functional>
#include <sstream>
#include <string>
#include <vector>

#include "wg_internal.h"

namespace wg {

namespace {

// xoshiro256** seeded by splitmix64: uniform doubles in [0, 1)
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (auto& x : s) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      x = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

struct State {
  int e, g, t;  // g = -1: loss
};

struct RecNode {
  int g, e, t;  // clade (-1: loss), species node, slice where the branch to this node starts
  int parent;
  std::vector<int> ch;
};

class Tracker {
 public:
  Tracker(const Model& m, const CCD& c, const double* tables, const std::vector<std::vector<int>>& cols)
      : m_(m), c_(c), cols_(cols) {
    base_.resize(m.K);
    int64_t o = 0;
    for (int k = 0; k < m.K; ++k) {
      base_[k] = tables + o;
      int nc = 0;
      for (int x : cols[k]) nc += x >= 0;
      ncol_.push_back(nc);
      o += (int64_t)m.nrow[k] * nc;
    }
  }

  // getl: the family's DP value at node e, clade g, slice t (1-based)
  double L(int e, int g, int t) const {
    const int c = cols_[e][g];
    return c < 0 ? 0.0 : base_[e][(int64_t)(t - 1) * ncol_[e] + c];
  }
  double Ltop(int e, int g) const { return L(e, g, m_.nrow[e]); }
  double eps_top(int e) const { return m_.eps_top(e); }
  double phi(int e, int t) const { return m_.phi[m_.row_off[e] + t - 1]; }
  double psi(int e, int t) const { return m_.psi[m_.row_off[e] + t - 1]; }

  std::vector<RecNode> sample(Rng& rng) {
    std::vector<RecNode> nodes;
    const int root = m_.K - 1, ub = c_.n_clades - 1;
    nodes.push_back({ub, root, 1, -1, {}});
    std::vector<std::pair<State, int>> work{{{root, ub, 1}, 0}};
    while (!work.empty()) {
      auto [s, cur] = work.back();
      work.pop_back();
      if (s.g < 0) continue;  // a loss: the node was made when the state was entered
      std::vector<State> next = step(s, rng);
      // each next state hangs below `cur`: a new node when clade or branch change
      for (auto it = next.rbegin(); it != next.rend(); ++it) {
        int node = cur;
        if (it->g != nodes[cur].g || it->e != nodes[cur].e) {
          node = (int)nodes.size();
          nodes.push_back({it->g, it->e, it->t, cur, {}});
          nodes[cur].ch.push_back(node);
        }
        work.push_back({*it, node});
      }
      // children were appended in reverse order of `next`; restore it
      auto& ch = nodes[cur].ch;
      const size_t added = (size_t)std::count_if(next.begin(), next.end(), [&](const State& x) {
        return x.g != nodes[cur].g || x.e != nodes[cur].e;
      });
      std::reverse(ch.end() - (std::ptrdiff_t)added, ch.end());
    }
    return nodes;
  }

 private:
  // One backtracking step from state s: the next states (empty: a leaf).
  std::vector<State> step(const State& s, Rng& rng) {
    const int e = s.e, g = s.g, t = s.t;
    const int kind = m_.kind[e];
    if (t == 1) {  // internode (src/track.jl:205-219)
      if (kind == WG_NODE_LEAF) return {};
      const double total = L(e, g, t);
      double r = rng.uniform() * total;
      if (kind == WG_NODE_ROOT) return root_events(r, e, g, t);
      if (kind == WG_NODE_WGD) return wgd_events(r, e, g);
      return spec_events(r, e, g);
    }
    // intra-branch (src/track.jl:266-280)
    if (c_.nleaves[g] == 1) return {{e, g, 1}};
    double r = rng.uniform() * L(e, g, t);
    r -= phi(e, t) * L(e, g, t - 1);
    if (r < 0.0) return {{e, g, t - 1}};
    const double ps = psi(e, t);
    std::vector<State> last;
    for (int k = c_.split_off[g]; k < c_.split_off[g + 1]; ++k) {
      const int a = c_.g1[k], b = c_.g2[k];
      const double w = c_.p[k] * L(e, a, t - 1) * L(e, b, t - 1) * ps;
      if (w > 0.0) last = {{e, a, t - 1}, {e, b, t - 1}};
      r -= w;
      if (r < 0.0) return last;
    }
    return fallback(last, {{e, g, t - 1}});
  }

  // speciation node: sploss, then speciation (src/track.jl:223-231, 283-331)
  std::vector<State> spec_events(double r, int e, int g) {
    const int f = m_.ch0[e], h = m_.ch1[e];
    const int tf = m_.nrow[f], th = m_.nrow[h];
    std::vector<State> last;
    auto take = [&](double w, std::vector<State> nx) {
      if (w > 0.0) last = nx;
      r -= w;
      return r < 0.0;
    };
    if (take(Ltop(f, g) * eps_top(h), {{f, g, tf}, {h, -1, 0}})) return last;
    if (take(Ltop(h, g) * eps_top(f), {{h, g, th}, {f, -1, 0}})) return last;
    for (int k = c_.split_off[g]; k < c_.split_off[g + 1]; ++k) {
      const int a = c_.g1[k], b = c_.g2[k];
      if (take(c_.p[k] * Ltop(f, a) * Ltop(h, b), {{f, a, tf}, {h, b, th}})) return last;
      if (take(c_.p[k] * Ltop(h, a) * Ltop(f, b), {{h, a, th}, {f, b, tf}})) return last;
    }
    return fallback(last, {});
  }

  // WGD node: non-retention, then retention (src/track.jl:252-265, 333-357)
  std::vector<State> wgd_events(double r, int e, int g) {
    const int f = m_.ch0[e], tf = m_.nrow[f];
    const double q = m_.q[e];
    std::vector<State> last;
    const double w0 = (1.0 - q + 2.0 * q * eps_top(f)) * Ltop(f, g);
    if (w0 > 0.0) last = {{f, g, tf}};
    r -= w0;
    if (r < 0.0) return last;
    for (int k = c_.split_off[g]; k < c_.split_off[g + 1]; ++k) {
      const int a = c_.g1[k], b = c_.g2[k];
      const double w = q * c_.p[k] * Ltop(f, a) * Ltop(f, b);
      if (w > 0.0) last = {{f, a, tf}, {f, b, tf}};
      r -= w;
      if (r < 0.0) return last;
    }
    return fallback(last, {});
  }

  // root: bifurcation (stay and duplicate, or speciate), then loss
  // (src/track.jl:233-250, 359-401)
  std::vector<State> root_events(double r, int e, int g, int t) {
    const int f = m_.ch0[e], h = m_.ch1[e];
    const int tf = m_.nrow[f], th = m_.nrow[h];
    const double eta = m_.eta, eps = eps_top(e);
    const double xi = 1.0 - (1.0 - eta) * eps;
    const double cd = xi * (1.0 - eta) / eta, cs = eta * (1.0 - eps) / (xi * xi);
    std::vector<State> last;
    auto take = [&](double w, std::vector<State> nx) {
      if (w > 0.0) last = nx;
      r -= w;
      return r < 0.0;
    };
    for (int k = c_.split_off[g]; k < c_.split_off[g + 1]; ++k) {
      const int a = c_.g1[k], b = c_.g2[k];
      if (take(c_.p[k] * L(e, a, t) * L(e, b, t) * cd, {{e, a, t}, {e, b, t}})) return last;
      if (take(c_.p[k] * Ltop(f, a) * Ltop(h, b) * cs, {{f, a, tf}, {h, b, th}})) return last;
      if (take(c_.p[k] * Ltop(h, a) * Ltop(f, b) * cs, {{h, a, th}, {f, b, tf}})) return last;
    }
    if (take(Ltop(f, g) * eps_top(h) * cs, {{f, g, tf}, {h, -1, 0}})) return last;
    if (take(Ltop(h, g) * eps_top(f) * cs, {{h, g, th}, {f, -1, 0}})) return last;
    return fallback(last, {});
  }

  // The event terms sum to the drawn total up to rounding; a draw that lands
  // past the last term (the reference raises "Backtracking failed") takes
  // the last event with a positive term.
  static std::vector<State> fallback(const std::vector<State>& last, const std::vector<State>& dflt) {
    if (!last.empty()) return last;
    if (!dflt.empty()) return dflt;
    throw Error(WG_ESTATE, "backtracking found no event with positive probability");
  }

  const Model& m_;
  const CCD& c_;
  const std::vector<std::vector<int>>& cols_;
  std::vector<const double*> base_;
  std::vector<int> ncol_;
};

// Heights, labels and Newick text of a sampled reconciled tree
// (process_rectree, node_heights, getlabel: src/track.jl:414-488).
std::string to_newick(const Model& m, const CCD& c, const std::vector<RecNode>& nodes) {
  const int K = m.K;
  // species node depths Sh (distance from the root) and H = max depth
  std::vector<int> parent(K, -1);
  for (int k = 0; k < K; ++k)
    for (int ch : {m.ch0[k], m.ch1[k]})
      if (ch >= 0) parent[ch] = k;
  std::vector<double> depth(K, 0.0);
  double H = 0.0;
  for (int k = K - 1; k >= 0; --k) {  // parents after children in the order: walk it backwards
    depth[k] = parent[k] < 0 ? 0.0 : depth[parent[k]] + m.slice_len[k] * (m.nrow[k] - 1);
    H = std::max(H, depth[k]);
  }
  auto label = [&](const RecNode& n) -> std::string {
    if (n.g < 0) return "loss";
    bool dup = n.ch.size() == 2, loss = false;
    for (int x : n.ch) {
      dup = dup && nodes[x].e == n.e;
      loss = loss || nodes[x].g < 0;
    }
    const bool wgd = m.kind[n.e] == WG_NODE_WGD;
    if (n.ch.size() == 1 && wgd) return "wgdloss";
    if (!dup && !loss && wgd) return "wgd";
    if (dup) return "duplication";
    if (loss) return "sploss";
    return "speciation";
  };
  std::vector<double> h(nodes.size(), 0.0);
  std::function<void(int)> heights = [&](int i) {
    for (int x : nodes[i].ch) heights(x);
    const RecNode& n = nodes[i];
    if (n.ch.empty()) {
      h[i] = 0.0;
    } else if (label(n) == "duplication") {
      const double d = nodes[n.ch[0]].t, delta = m.slice_len[n.e];
      h[i] = H - depth[n.e] + d * delta - delta / 2.0;
    } else {
      h[i] = H - depth[n.e];
    }
  };
  heights(0);
  h[0] = H;
  std::ostringstream os;
  os.precision(17);
  std::function<void(int)> emit = [&](int i) {
    const RecNode& n = nodes[i];
    if (!n.ch.empty()) {
      os << '(';
      for (size_t j = 0; j < n.ch.size(); ++j) {
        if (j) os << ',';
        emit(n.ch[j]);
      }
      os << ')';
    }
    std::string name;
    if (n.g < 0) name = "loss";
    else if (n.ch.empty()) name = c.leaf_name.empty() || c.leaf_name[n.g].empty() ? "g" + std::to_string(n.g) : c.leaf_name[n.g];
    os << name << "[&&NHX:label=" << label(n) << ":node=" << n.e << ":clade=" << n.g << ":slice=" << n.t << ']';
    if (n.parent >= 0) os << ':' << (h[n.parent] - h[i]);
  };
  emit(0);
  os << ';';
  return os.str();
}

}  // namespace

std::string tree_newick(const Model& m, const CCD& c, const int32_t* nodes, int n) {
  if (n < 1) throw Error(WG_EINVAL, "a tree has at least its root");
  std::vector<RecNode> t((size_t)n);
  for (int i = 0; i < n; ++i) {
    const int32_t* x = nodes + 4 * (size_t)i;
    if (x[1] < 0 || x[1] >= m.K || x[0] < -1 || x[0] >= c.n_clades || x[3] >= i || (x[3] < 0) != (i == 0))
      throw Error(WG_EINVAL, "malformed tree node arrays");
    t[i] = {x[0], x[1], x[2], x[3], {}};
    if (x[3] >= 0) t[x[3]].ch.push_back(i);
  }
  // a node's children were made in one step, in reverse of the sampler's order
  for (auto& r : t) std::reverse(r.ch.begin(), r.ch.end());
  return to_newick(m, c, t);
}

std::string backtrack_family(const Model& m, const CCD& c, const double* tables, int n_samples, uint64_t seed) {
  const std::vector<std::vector<int>> cols = compat_columns(m, c);
  Tracker tr(m, c, tables, cols);
  if (!(tr.L(m.K - 1, c.n_clades - 1, 1) > 0.0))
    throw Error(WG_ESTATE, "backtracking needs a family with positive likelihood");
  Rng rng(seed);
  std::string out;
  for (int i = 0; i < n_samples; ++i) {
    out += to_newick(m, c, tr.sample(rng));
    out += '\n';
  }
  return out;
}

}  // namespace wg
