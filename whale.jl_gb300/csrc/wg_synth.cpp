// Workload generator: one gene family, simulated under the DL+WGD model and
// turned into an amalgamated CCD in ALE v0.4 text.  It stands in for the
// reference's simulator and its ALEobserve shell-out, neither of which is on
// the likelihood path:
//   randtree / dlsim!            src/simulation.jl:65-133 (geometric(η) root
//                                lineages, exponential waiting times with rate
//                                λ+μ, duplication w.p. λ/(λ+μ), WGD retention
//                                w.p. q, speciation into the children)
//   simulate_conditional         src/simulation.jl:27-46 (rejection until the
//                                root condition holds: genes on both sides)
//   get_ale_ccd / ALEobserve     src/ccd.jl:262-268 (amalgamation of a sample
//                                of unrooted trees into clade / split counts)
// The tree sample is n_trees copies of the true (unrooted) gene tree, each
// perturbed by U{0..max_nni} random nearest-neighbour interchanges.  With
// target_clades > 0 the family is redrawn until its gene count can give about
// that many clades, and perturbation stops once the count is reached.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>

#include "wg_internal.h"

namespace {

// xoshiro256** seeded by splitmix64
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (auto& x : s) {
      z += 0x9e3779b97f4a7c15ull;
      uint64_t t = z;
      t = (t ^ (t >> 30)) * 0xbf58476d1ce4e5b9ull;
      t = (t ^ (t >> 27)) * 0x94d049bb133111ebull;
      x = t ^ (t >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }  // (0, 1)
  int below(int n) { return (int)(uniform() * n); }
};

struct GeneTree {
  std::vector<int> left, right, species;  // species >= 0 for leaves (model node), -1 internal
  int add_leaf(int sp) { left.push_back(-1); right.push_back(-1); species.push_back(sp); return (int)left.size() - 1; }
  int join(int a, int b) {
    if (a < 0) return b;
    if (b < 0) return a;
    left.push_back(a); right.push_back(b); species.push_back(-1);
    return (int)left.size() - 1;
  }
};

struct Sim {
  const wg::Model& m;
  const double *lam, *mu, *q;
  Rng& rng;
  GeneTree& G;
  int budget;  // abort runaway families
  double blen(int k) const { return m.slice_len[k] * (m.nrow[k] - 1); }
  // dlsim! along the branch above node k with remaining time t
  int run(int k, double t) {
    if (--budget < 0) return -1;
    const double rate = lam[k] + mu[k];
    const double w = rate > 0 ? -std::log(rng.uniform()) / rate : INFINITY;
    if (w < t) {
      if (rng.uniform() < lam[k] / rate) {
        const int a = run(k, t - w);
        const int b = run(k, t - w);
        return G.join(a, b);
      }
      return -1;  // loss
    }
    return at_node(k);
  }
  int at_node(int k) {
    const int kind = m.kind[k];
    if (kind == WG_NODE_LEAF) return G.add_leaf(k);
    if (kind == WG_NODE_WGD) {
      const int f = m.ch0[k];
      if (rng.uniform() < q[k]) {
        const int a = run(f, blen(f));
        const int b = run(f, blen(f));
        return G.join(a, b);
      }
      return run(f, blen(f));
    }
    const int a = run(m.ch0[k], blen(m.ch0[k]));
    const int b = run(m.ch1[k], blen(m.ch1[k]));
    return G.join(a, b);
  }
};

// Unrooted binary tree as an adjacency list; leaves 0..n-1.
struct UTree {
  int n = 0;
  std::vector<std::vector<int>> adj;
};

UTree unroot(const GeneTree& G, int root, std::vector<int>& leaf_species) {
  UTree U;
  std::vector<int> id(G.left.size(), -1);
  std::vector<int> stack{root}, leaves, internals;
  // collect nodes
  std::vector<int> order;
  while (!stack.empty()) {
    int x = stack.back();
    stack.pop_back();
    order.push_back(x);
    if (G.left[x] >= 0) { stack.push_back(G.right[x]); stack.push_back(G.left[x]); }
  }
  for (int x : order) if (G.left[x] < 0) { id[x] = (int)leaves.size(); leaves.push_back(x); }
  U.n = (int)leaves.size();
  int next = U.n;
  for (int x : order) if (G.left[x] >= 0 && x != root) id[x] = next++;
  U.adj.assign(next, {});
  leaf_species.clear();
  for (int x : leaves) leaf_species.push_back(G.species[x]);
  auto link = [&](int a, int b) { U.adj[a].push_back(b); U.adj[b].push_back(a); };
  for (int x : order) {
    if (G.left[x] < 0 || x == root) continue;
    link(id[x], id[G.left[x]]);
    link(id[x], id[G.right[x]]);
  }
  // the root's two children are joined directly
  if (G.left[root] >= 0) link(id[G.left[root]], id[G.right[root]]);
  return U;
}

// One random NNI: pick an internal edge (u, v), swap a neighbour of u (not v)
// with a neighbour of v (not u).
void nni(UTree& U, Rng& rng) {
  std::vector<std::pair<int, int>> edges;
  for (int u = U.n; u < (int)U.adj.size(); ++u)
    for (int v : U.adj[u]) if (v > u) edges.emplace_back(u, v);
  if (edges.empty()) return;
  auto [u, v] = edges[rng.below((int)edges.size())];
  std::vector<int> nu, nv;
  for (int x : U.adj[u]) if (x != v) nu.push_back(x);
  for (int x : U.adj[v]) if (x != u) nv.push_back(x);
  const int a = nu[rng.below((int)nu.size())];
  const int b = nv[rng.below((int)nv.size())];
  auto repl = [&](int node, int from, int to) {
    for (int& x : U.adj[node]) if (x == from) { x = to; return; }
  };
  repl(u, a, b);
  repl(v, b, a);
  repl(a, u, v);
  repl(b, v, u);
}

using Bits = std::vector<uint64_t>;
struct BitsHash {
  size_t operator()(const Bits& v) const {
    uint64_t h = 0x84222325cbf29ce4ull;
    for (uint64_t x : v) { h ^= x; h *= 0x100000001b3ull; h ^= h >> 29; }
    return (size_t)h;
  }
};

struct Amalgam {
  int n = 0, W = 0;
  std::unordered_map<Bits, int, BitsHash> ids;  // clade -> set id
  std::vector<Bits> sets;                       // index = set id
  std::vector<int64_t> bip;
  std::vector<std::vector<std::pair<std::pair<int, int>, int64_t>>> dip;
  int get(const Bits& b) {
    auto it = ids.find(b);
    if (it != ids.end()) return it->second;
    const int id = (int)sets.size();
    ids.emplace(b, id);
    sets.push_back(b);
    bip.push_back(0);
    dip.emplace_back();
    return id;
  }
  void init(int nleaves) {
    n = nleaves;
    W = (n + 63) / 64;
    sets.assign(1, Bits(W, 0));  // id 0 unused
    bip.assign(1, 0);
    dip.assign(1, {});
    for (int i = 0; i < n; ++i) {
      Bits b(W, 0);
      b[i >> 6] |= 1ull << (i & 63);
      get(b);  // leaf i -> set id i + 1
    }
  }
  // add one unrooted tree
  void add(const UTree& U) {
    const int N = (int)U.adj.size();
    // side[x->y] = leaves on y's side of edge x-y; computed by rooting at leaf 0
    std::vector<int> parent(N, -2), order;
    std::vector<int> st{0};
    parent[0] = -1;
    while (!st.empty()) {
      int x = st.back();
      st.pop_back();
      order.push_back(x);
      for (int y : U.adj[x]) if (parent[y] == -2) { parent[y] = x; st.push_back(y); }
    }
    std::vector<Bits> down(N, Bits(W, 0));  // leaves below x (away from leaf 0)
    for (int i = (int)order.size() - 1; i >= 1; --i) {
      const int x = order[i];
      if (x < U.n) down[x][x >> 6] |= 1ull << (x & 63);
      for (int y : U.adj[x])
        if (parent[y] == x) for (int w = 0; w < W; ++w) down[x][w] |= down[y][w];
    }
    Bits all(W, 0);
    for (int i = 0; i < n; ++i) all[i >> 6] |= 1ull << (i & 63);
    auto side = [&](int x, int y) -> Bits {  // leaves on y's side of edge x - y
      if (parent[y] == x && y != 0) return down[y];
      Bits b(W);
      for (int w = 0; w < W; ++w) b[w] = all[w] & ~down[x][w];
      return b;
    };
    for (int v = U.n; v < N; ++v) {
      const auto& nb = U.adj[v];
      for (int i = 0; i < 3; ++i) {
        const int x = nb[i], y = nb[(i + 1) % 3], z = nb[(i + 2) % 3];
        (void)x;
        const Bits sy = side(v, y), sz = side(v, z);
        Bits c(W);
        for (int w = 0; w < W; ++w) c[w] = sy[w] | sz[w];
        const int cid = get(c);
        int a = get(sy), b = get(sz);
        if (a > b) std::swap(a, b);
        bip[cid] += 1;
        auto& d = dip[cid];
        bool found = false;
        for (auto& e : d) if (e.first.first == a && e.first.second == b) { e.second += 1; found = true; break; }
        if (!found) d.push_back({{a, b}, 1});
      }
    }
  }
  int n_clades() const { return (int)sets.size() - 1 + 1; }  // + ubiquitous
};

std::string newick_of(const GeneTree& G, int x, const std::vector<std::string>& names) {
  if (G.left[x] < 0) return names[x];
  return "(" + newick_of(G, G.left[x], names) + "," + newick_of(G, G.right[x], names) + ")";
}

}  // namespace

extern "C" int wg_synth_family(const wg_model* m, const double* lam, const double* mu, const double* q, double eta,
                               const char* const* species_names, uint64_t seed, int32_t n_trees, int32_t max_nni,
                               int32_t min_genes, int32_t target_clades, int32_t flags, char* out, int64_t cap,
                               int64_t* len) {
  WG_GUARD({
    if (!m || !lam || !mu || !q || !species_names || !len || n_trees < 1 || max_nni < 0)
      throw wg::Error(WG_EINVAL, "wg_synth_family: bad arguments");
    Rng rng(seed);
    const int K = m->K, r = K - 1;
    // which side of the root each leaf is on
    std::vector<int> side(K, -1);
    {
      std::vector<int> st{m->ch0[r]};
      while (!st.empty()) { int x = st.back(); st.pop_back(); side[x] = 0; if (m->ch0[x] >= 0) st.push_back(m->ch0[x]); if (m->ch1[x] >= 0) st.push_back(m->ch1[x]); }
      st = {m->ch1[r]};
      while (!st.empty()) { int x = st.back(); st.pop_back(); side[x] = 1; if (m->ch0[x] >= 0) st.push_back(m->ch0[x]); if (m->ch1[x] >= 0) st.push_back(m->ch1[x]); }
    }
    GeneTree best;
    int best_root = -1;
    double best_gap = INFINITY;
    const int max_attempts = target_clades > 0 ? 20000 : 100000;
    for (int att = 0; att < max_attempts; ++att) {
      GeneTree G;
      Sim S{*m, lam, mu, q, rng, G, 200000};
      int a = 0;
      while (rng.uniform() >= eta) ++a;  // Geometric(η) failures
      int root = -1;
      for (int i = 0; i <= a; ++i) root = G.join(root, S.at_node(r));
      if (S.budget < 0 || root < 0) continue;
      int n = 0, s0 = 0, s1 = 0;
      for (size_t x = 0; x < G.left.size(); ++x) {
        if (G.left[x] >= 0 || G.species[x] < 0) continue;
        // count only leaves reachable from root: all leaves created are kept (losses return -1)
        ++n;
        if (side[G.species[x]] == 0) ++s0; else ++s1;
      }
      if (!(s0 > 0 && s1 > 0) || n < std::max(3, (int)min_genes)) continue;
      if (target_clades <= 0) { best = G; best_root = root; break; }
      // gene count whose unperturbed tree gives 4n-5 clades and whose
      // perturbed sample can reach the target
      const double lo = 4.0 * n - 5.0;
      const double moves = (flags & WG_SYNTH_PUSH) ? (double)n_trees * max_nni : 0.5 * n_trees * max_nni;
      const double hi = (flags & WG_SYNTH_WALK) ? lo + 1.6 * moves : lo + std::min(1.6 * moves, 2.0 * n * n);
      double gap = 0.0;
      if (target_clades < lo) gap = std::log(lo / target_clades);
      else if (target_clades > hi) gap = std::log(target_clades / hi);
      if (gap < best_gap) { best_gap = gap; best = G; best_root = root; }
      if (gap == 0.0) break;
    }
    if (best_root < 0) throw wg::Error(WG_EINVAL, "could not simulate a family satisfying the root condition");
    GeneTree& G = best;
    std::vector<int> lsp;
    UTree T = unroot(G, best_root, lsp);
    const int n = T.n;
    // gene names <species>_g<i>, leaves numbered 1..n in tree order
    std::vector<std::string> gname(G.left.size());
    {
      int i = 0;
      std::vector<int> st{best_root};
      std::vector<int> lorder;
      while (!st.empty()) { int x = st.back(); st.pop_back(); if (G.left[x] < 0) lorder.push_back(x); else { st.push_back(G.right[x]); st.push_back(G.left[x]); } }
      for (int x : lorder) gname[x] = std::string(species_names[G.species[x]]) + "_g" + std::to_string(++i);
    }
    std::vector<std::string> leafname(n);
    {
      std::vector<int> st{best_root}, lorder;
      while (!st.empty()) { int x = st.back(); st.pop_back(); if (G.left[x] < 0) lorder.push_back(x); else { st.push_back(G.right[x]); st.push_back(G.left[x]); } }
      for (int i = 0; i < n; ++i) leafname[i] = gname[lorder[i]];
    }
    Amalgam AM;
    AM.init(n);
    bool reached = false;
    UTree cur = T;
    for (int t = 0; t < n_trees; ++t) {
      UTree U = (flags & WG_SYNTH_WALK) ? cur : T;
      if (!reached) {
        const int k = (flags & WG_SYNTH_PUSH) && target_clades > 0 ? max_nni : rng.below(max_nni + 1);
        for (int i = 0; i < k; ++i) nni(U, rng);
      }
      AM.add(U);
      cur = U;
      if (target_clades > 0 && AM.n_clades() >= target_clades) reached = true;
    }
    // ALE v0.4 text; set ids 1..n are the leaves, then clades in first-seen order
    std::string s;
    s.reserve(1 << 16);
    s += "#constructor_string\n" + newick_of(G, best_root, gname) + ";\n";
    s += "#observations\n" + std::to_string(n_trees) + "\n";
    s += "#Bip_counts\n";
    const int nsets = (int)AM.sets.size() - 1;
    for (int id = n + 1; id <= nsets; ++id) s += std::to_string(id) + "\t" + std::to_string(AM.bip[id]) + "\n";
    s += "#Bip_bls\n";
    for (int id = 1; id <= nsets; ++id) s += std::to_string(id) + "\t0\n";
    s += "#Dip_counts\n";
    for (int id = n + 1; id <= nsets; ++id)
      for (auto& e : AM.dip[id])
        s += std::to_string(id) + "\t" + std::to_string(e.first.first) + "\t" + std::to_string(e.first.second) + "\t" +
             std::to_string(e.second) + "\n";
    s += "#last_leafset_id\n" + std::to_string(nsets) + "\n";
    s += "#leaf-id\n";
    for (int i = 0; i < n; ++i) s += leafname[i] + "\t" + std::to_string(i + 1) + "\n";
    s += "#set-id\n";
    for (int id = 1; id <= nsets; ++id) {
      s += std::to_string(id) + "\t:";
      const Bits& b = AM.sets[id];
      for (int i = 0; i < n; ++i) if (b[i >> 6] >> (i & 63) & 1ull) s += "\t" + std::to_string(i + 1);
      s += "\n";
    }
    s += "#END\n";
    *len = (int64_t)s.size();
    if (out && cap > 0) {
      const int64_t nw = std::min<int64_t>(cap - 1, (int64_t)s.size());
      std::memcpy(out, s.data(), (size_t)nw);
      out[nw] = 0;
    }
  });
}
