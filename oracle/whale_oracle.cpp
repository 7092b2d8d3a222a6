// ============================================================================
// CPU ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, on the CPU and in plain scalar C++, the algorithm of
// Whale.jl v2.1.0 for the amalgamated reconciliation likelihood: the species
// tree model with its slice tables, the ALE (v0.4) reader and CCD layout, the
// DP over species branches x slices x clades, and the survival conditioning.
// It is the checker for the CUDA product path and the timed CPU baseline.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg call it.
// The product library never links or calls it.
//
// Every function cites the reference file:line it restates (paths relative
// to the Whale.jl project root).  Floating-point evaluation order follows the
// Julia source (left-to-right products, no FMA contraction: build with
// -ffp-contract=off) so that results track the reference to a few ulps.
//
// Third-party behaviour restated here (not vendored in the reference):
//   * NewickTree 0.3.1 (Manifest.toml:1061-1065): readnw keeps children in
//     textual order; a root without a branch length has distance NaN;
//     getleaves/postwalk visit leaves left to right.
//   * ForwardDiff 0.10.38 (Manifest.toml:630-634): forward-mode dual numbers;
//     gradients are taken with chunked duals of width WG_ORC_CHUNK (=12, the
//     default chunk that ForwardDiff picks for >= 12 inputs).
// ============================================================================
#include <algorithm>
#include <array>
#include <functional>
#include <iterator>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------------------
// Forward-mode dual number (stand-in for ForwardDiff.Dual).
// ---------------------------------------------------------------------------
#ifndef WG_ORC_CHUNK
#define WG_ORC_CHUNK 12
#endif
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0) { for (int i = 0; i < N; ++i) d[i] = 0; }
  Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0; }
};
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v; const double ib = 1.0 / (b.v * b.v);
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) * ib; return r; }
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v += a; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { Dual<N> r = -b; r.v += a; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v * b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b; return r; }
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { Dual<N> r; r.v = a * b.v; for (int i = 0; i < N; ++i) r.d[i] = a * b.d[i]; return r; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v / b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b; return r; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N> inline Dual<N> exp(const Dual<N>& a) { Dual<N> r; r.v = std::exp(a.v); for (int i = 0; i < N; ++i) r.d[i] = r.v * a.d[i]; return r; }
template <int N> inline Dual<N> log(const Dual<N>& a) { Dual<N> r; r.v = std::log(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v; return r; }
inline double val(double x) { return x; }
template <int N> inline double val(const Dual<N>& x) { return x.v; }
inline double exp(double x) { return std::exp(x); }
inline double log(double x) { return std::log(x); }

// ---------------------------------------------------------------------------
// Newick tree (NewickTree 0.3.1 semantics for the subset the reference uses).
// ---------------------------------------------------------------------------
struct TNode {
  std::string name;
  double dist = NAN;
  int parent = -1;
  std::vector<int> ch;
};

struct Tree {
  std::vector<TNode> n;
  int root = -1;
};

static void skip_ws(const std::string& s, size_t& i) { while (i < s.size() && isspace((unsigned char)s[i])) ++i; }

static int parse_subtree(const std::string& s, size_t& i, Tree& t, int parent) {
  int me = (int)t.n.size();
  t.n.push_back(TNode());
  t.n[me].parent = parent;
  skip_ws(s, i);
  if (i < s.size() && s[i] == '(') {
    ++i;
    while (true) {
      int c = parse_subtree(s, i, t, me);
      t.n[me].ch.push_back(c);
      skip_ws(s, i);
      if (i < s.size() && s[i] == ',') { ++i; continue; }
      if (i < s.size() && s[i] == ')') { ++i; break; }
      throw std::runtime_error("newick: expected ',' or ')'");
    }
  }
  skip_ws(s, i);
  std::string name;
  while (i < s.size() && s[i] != ':' && s[i] != ',' && s[i] != ')' && s[i] != ';' && s[i] != '[') name += s[i++];
  while (!name.empty() && isspace((unsigned char)name.back())) name.pop_back();
  t.n[me].name = name;
  skip_ws(s, i);
  if (i < s.size() && s[i] == '[') { while (i < s.size() && s[i] != ']') ++i; if (i < s.size()) ++i; }
  skip_ws(s, i);
  if (i < s.size() && s[i] == ':') {
    ++i;
    size_t j = i;
    while (j < s.size() && s[j] != ',' && s[j] != ')' && s[j] != ';' && s[j] != '[') ++j;
    t.n[me].dist = std::strtod(s.substr(i, j - i).c_str(), nullptr);
    i = j;
  }
  return me;
}

static Tree readnw(const std::string& s) {
  Tree t;
  size_t i = 0;
  t.root = parse_subtree(s, i, t, -1);
  return t;
}

static void postwalk(const Tree& t, int x, std::vector<int>& out) {
  for (int c : t.n[x].ch) postwalk(t, c, out);
  out.push_back(x);
}

// ---------------------------------------------------------------------------
// Model structure: src/model.jl:6-22 (Slices), :96-145 (WhaleModel ids/order),
// :32-42 (setclade!), :54 (iswgd).
// ---------------------------------------------------------------------------
enum CondKind { COND_NONE = 0, COND_ROOT = 1, COND_NONEXTINCT = 2, COND_NOWHERE = 3 };

struct MNode {
  int tn;            // index into Tree
  int id;            // reference node id (1-based)
  int wgdid;         // WGD ordinal (preorder), 0 if not a WGD
  bool wgd, leaf, root;
  std::vector<int> ch;  // children as positions in `order`
  int parent;           // position in `order` (-1 for root)
  int nrow;             // n+1 rows of the slice matrix
  double dt;            // slice length t/n (0 if n == 0)
  double leafP;         // leafℙ
  std::vector<int> clade;  // species ids (sorted)
  std::string name;
};

struct Model {
  Tree tree;
  std::vector<MNode> order;  // wm.order
  std::vector<int> index;    // id -> position in order
  int nonwgd = 0, nwgd = 0;
  std::map<std::string, int> spmap;  // leaf name -> id (last wins, src/ccd.jl:128)
  int cond = COND_ROOT;
};

static bool iswgd_name(const std::string& s) { return s.rfind("wgd", 0) == 0; }  // src/model.jl:54

// src/model.jl:16-22
static void slices_shape(double t, double Dt, int minn, int maxn, int& nrow, double& dt) {
  int n = 0;
  if (!std::isnan(t)) {
    double c = std::ceil(t / Dt);
    n = (int)std::min<double>(maxn, std::max<double>(minn, c));
  }
  nrow = n + 1;
  dt = (n == 0) ? 0.0 : t / n;
}

static Model* build_model(const std::string& nw, double Dt, int minn, int maxn, int cond) {
  auto* m = new Model();
  m->tree = readnw(nw);
  m->cond = cond;
  const Tree& T = m->tree;
  // mulgroups: leaf names occurring more than once (src/model.jl:101)
  std::vector<int> pw; postwalk(T, T.root, pw);
  std::map<std::string, int> cnt;
  for (int x : pw) if (T.n[x].ch.empty()) cnt[T.n[x].name]++;
  // walk: preorder wgd ordinals, postorder list (src/model.jl:102-121)
  std::vector<MNode> post;
  int nonwgd = 0, wgdid = 0;
  std::vector<int> tn2post(T.n.size(), -1);
  std::function<void(int)> walk = [&](int x) {
    MNode mn;
    mn.tn = x; mn.name = T.n[x].name;
    mn.wgd = iswgd_name(mn.name);
    if (mn.wgd) { wgdid += 1; mn.wgdid = wgdid; } else { nonwgd += 1; mn.wgdid = 0; }
    mn.leaf = T.n[x].ch.empty();
    mn.root = (T.n[x].parent < 0);
    auto it = cnt.find(mn.name);
    bool mul = mn.leaf && it != cnt.end() && it->second > 1;
    (void)mul;
    // leafℙ: haskey(mulgroups, name) ? 1/count : isleaf ? 1 : 0  (src/model.jl:110-111)
    if (it != cnt.end() && it->second > 1) mn.leafP = 1.0 / it->second;
    else mn.leafP = mn.leaf ? 1.0 : 0.0;
    slices_shape(T.n[x].dist, Dt, minn, maxn, mn.nrow, mn.dt);
    for (int c : T.n[x].ch) walk(c);
    tn2post[x] = (int)post.size();
    post.push_back(mn);
  };
  walk(T.root);
  // order = union(getleaves(root), postorder)  (src/model.jl:124)
  std::vector<int> ord_tn;
  std::vector<char> seen(T.n.size(), 0);
  for (int x : pw) if (T.n[x].ch.empty()) { ord_tn.push_back(x); seen[x] = 1; }
  for (int x : pw) if (!seen[x]) { ord_tn.push_back(x); seen[x] = 1; }
  std::vector<int> tn2ord(T.n.size(), -1);
  for (size_t k = 0; k < ord_tn.size(); ++k) { m->order.push_back(post[tn2post[ord_tn[k]]]); tn2ord[ord_tn[k]] = (int)k; }
  // ids (src/model.jl:122-139)
  int i = nonwgd + 1, j = 1;
  std::map<std::string, int> mulid;
  m->index.assign(m->order.size() + 1, -1);
  for (size_t k = 0; k < m->order.size(); ++k) {
    MNode& n = m->order[k];
    if (n.wgd) { n.id = i++; }
    else {
      n.id = j++;
      auto it = cnt.find(n.name);
      if (it != cnt.end() && it->second > 1) mulid[n.name] = n.id;
    }
    m->index[n.id] = (int)k;
  }
  for (size_t k = 0; k < m->order.size(); ++k) {
    MNode& n = m->order[k];
    for (int c : T.n[n.tn].ch) n.ch.push_back(tn2ord[c]);
    n.parent = T.n[n.tn].parent < 0 ? -1 : tn2ord[T.n[n.tn].parent];
  }
  // setclade! (src/model.jl:32-42)
  std::function<void(int)> setclade = [&](int k) {
    MNode& n = m->order[k];
    if (n.leaf) {
      auto it = mulid.find(n.name);
      n.clade = {it != mulid.end() ? it->second : n.id};
    } else {
      std::set<int> s;
      for (int c : n.ch) { setclade(c); for (int v : m->order[c].clade) s.insert(v); }
      n.clade.assign(s.begin(), s.end());
    }
  };
  setclade((int)m->order.size() - 1);
  m->nonwgd = nonwgd; m->nwgd = wgdid;
  // spmap: Dict(name(l)=>id(l) for l in getleaves(root(wm)))  (src/ccd.jl:128)
  for (size_t k = 0; k < m->order.size(); ++k) if (m->order[k].leaf) m->spmap[m->order[k].name] = m->order[k].id;
  return m;
}

// ---------------------------------------------------------------------------
// Rates: src/rmodels.jl:14 (getp), :31-33 (ConstantDLWGD getθ),
// :55-64 (DLWGD getθ, log-scale rates), src/model.jl:200-203 (nonwgdchild).
// ---------------------------------------------------------------------------
template <class T>
struct Rates {
  int kind = 0;            // 0 = DLWGD (log-scale λ, μ by node id), 1 = ConstantDLWGD
  std::vector<T> lam, mu;  // DLWGD: per id; Constant: one entry
  std::vector<T> q;        // per wgdid
  T eta = T(0.66);
  std::vector<double> p;   // sampling probabilities per leaf id (may be empty)
};

template <class T>
struct Theta { T lam, mu, q, eta; double p; bool nanrates; };

template <class T>
static Theta<T> getθ(const Model& m, const Rates<T>& r, int k) {
  const MNode& n = m.order[k];
  Theta<T> th; th.nanrates = false; th.q = T(NAN); th.eta = r.eta; th.p = 0.0;
  th.lam = T(NAN); th.mu = T(NAN);
  double p = (!r.p.empty() && n.leaf) ? r.p[n.id - 1] : 0.0;
  if (r.kind == 1) {
    th.lam = r.lam[0]; th.mu = r.mu[0]; th.p = p;
    if (n.wgd) th.q = r.q[n.wgdid - 1];
    return th;
  }
  if (n.wgd) {
    int c = k;
    while (m.order[c].wgd) c = m.order[c].ch[0];
    int cid = m.order[c].id;
    th.lam = exp(r.lam[cid - 1]); th.mu = exp(r.mu[cid - 1]); th.q = r.q[n.wgdid - 1];
  } else {
    if (n.id > (int)r.lam.size()) { th.nanrates = true; }
    else { th.lam = exp(r.lam[n.id - 1]); th.mu = exp(r.mu[n.id - 1]); }
    th.p = p;
  }
  return th;
}

// src/bdputil.jl:1-11
template <class T>
static T getα(const T& λ, const T& μ, double t) {
  if (std::fabs(val(λ) - val(μ)) <= 1e-6)  // isapprox(λ, μ, atol=1e-6)
    return λ * t / (1.0 + λ * t);
  return μ * (exp(t * (λ - μ)) - 1.0) / (λ * exp(t * (λ - μ)) - μ);
}
template <class T> static T _ϵ(const T& α, const T& β, const T& ϵ) { return (α + (1.0 - α - β) * ϵ) / (1.0 - β * ϵ); }
template <class T> static T _ϕ(const T& α, const T& β, const T& ϵ) { T d = 1.0 - β * ϵ; return (1.0 - α) * (1.0 - β) / (d * d); }
template <class T> static T _ψ(const T& α, const T& β, const T& ϵ) { T d = 1.0 - β * ϵ; return (1.0 - α) * (1.0 - β) * β / (d * d * d); }

// slice tables per node: columns [Δt, ε, ϕ, ψ]; rows 0..nrow-1
template <class T>
struct Tables {
  std::vector<std::vector<T>> eps, phi, psi;  // [order pos][row]
  std::vector<T> q;                            // q per order position (NaN if not wgd)
  T eta;
};

// src/model.jl:162-191 (setmodel!, setnode!, setwgdnode!, setslices!)
template <class T>
static Tables<T> setmodel(const Model& m, const Rates<T>& r) {
  Tables<T> tb;
  size_t K = m.order.size();
  tb.eps.resize(K); tb.phi.resize(K); tb.psi.resize(K); tb.q.assign(K, T(NAN));
  tb.eta = r.eta;
  for (size_t k = 0; k < K; ++k) {
    const MNode& n = m.order[k];
    Theta<T> th = getθ(m, r, (int)k);
    tb.eps[k].assign(n.nrow, T(1.0)); tb.phi[k].assign(n.nrow, T(1.0)); tb.psi[k].assign(n.nrow, T(1.0));
    if (n.wgd) {
      T ϵ = tb.eps[n.ch[0]].back();
      tb.eps[k][0] = th.q * ϵ * ϵ + (1.0 - th.q) * ϵ;
      tb.q[k] = th.q;
    } else {
      if (n.leaf) tb.eps[k][0] = T(th.p);
      else {
        // prod([c[end,2] for c in children(n)])
        T pr = tb.eps[n.ch[0]].back();
        for (size_t c = 1; c < n.ch.size(); ++c) pr = pr * tb.eps[n.ch[c]].back();
        tb.eps[k][0] = pr;
      }
      tb.phi[k][0] = T(1.0);
    }
    for (int i = 1; i < n.nrow; ++i) {
      T α = getα(th.lam, th.mu, n.dt);
      T β = (th.lam / th.mu) * α;
      T ϵ = tb.eps[k][i - 1];
      tb.eps[k][i] = _ϵ(α, β, ϵ);
      tb.phi[k][i] = _ϕ(α, β, ϵ);
      tb.psi[k][i] = _ψ(α, β, ϵ);
    }
  }
  return tb;
}

// ---------------------------------------------------------------------------
// CCD: src/ccd.jl:13-33 (Triple, Clade), :59-75 (index_and_getℓ),
// :80-121 (CCD), :139 (getspecies), :147-248 (ALE v0.4 reader).
// ---------------------------------------------------------------------------
struct Split { int g1, g2; double p; };  // 0-based clade ids
struct Clade { int id; long count; std::vector<Split> splits; std::vector<int> leaves; std::vector<int> species; };

struct CCD {
  std::vector<Clade> clades;              // size ordered, leaves first, ubiquitous last
  std::vector<std::vector<int>> compat;   // per order position: clade ids (0-based)
  std::vector<std::vector<int>> index;    // [order pos][clade] -> local column or -1
  long total = 0;
  std::string fname;
};

static std::vector<std::string> split_ws(const std::string& s) {
  std::vector<std::string> out; std::istringstream is(s); std::string w;
  while (is >> w) out.push_back(w);
  return out;
}

static std::string replace_all(std::string s, const std::string& a, const std::string& b) {
  size_t pos = 0;
  while ((pos = s.find(a, pos)) != std::string::npos) { s.replace(pos, a.size(), b); pos += b.size(); }
  return s;
}

// parse_aleobserve + addleafclades! + addubiquitous! + CCD(ale, wm, spmap)
static CCD* parse_ccd(const Model& m, const std::string& text, const std::string& fname) {
  // sections = split(alestring, "#")[2:end-1]
  std::vector<std::string> parts;
  { size_t s = 0; while (true) { size_t h = text.find('#', s); if (h == std::string::npos) { parts.push_back(text.substr(s)); break; } parts.push_back(text.substr(s, h - s)); s = h + 1; } }
  if (parts.size() < 2 || parts.size() - 2 != 8) throw std::runtime_error("Not a valid .ale file " + fname);
  long observations = 0;
  std::map<long, long> bip;                                       // Bip_counts
  std::map<long, std::vector<std::array<long, 3>>> dip;           // Dip_counts (ordered per key)
  std::map<long, std::vector<long>> set_id;
  std::map<long, std::string> leaf_id;                            // leaf number -> name
  for (size_t si = 1; si + 1 < parts.size(); ++si) {
    std::string sec = replace_all(parts[si], ":\t", "");
    std::vector<std::string> lines; { std::istringstream is(sec); std::string l; while (std::getline(is, l)) lines.push_back(l); }
    if (lines.empty()) continue;
    std::string header = replace_all(lines[0], "-", "_");
    std::vector<std::string> body; for (size_t k = 1; k < lines.size(); ++k) if (!lines[k].empty()) body.push_back(lines[k]);
    if (header == "observations") observations = std::atol(body.at(0).c_str());
    else if (header == "Bip_counts") { for (auto& l : body) { auto w = split_ws(l); bip[std::atol(w[0].c_str())] = std::atol(w[1].c_str()); } }
    else if (header == "Dip_counts") { for (auto& l : body) { auto w = split_ws(l); dip[std::atol(w[0].c_str())].push_back({std::atol(w[1].c_str()), std::atol(w[2].c_str()), std::atol(w[3].c_str())}); } }
    else if (header == "set_id") { for (auto& l : body) { auto w = split_ws(l); std::vector<long> v; for (size_t k = 1; k < w.size(); ++k) v.push_back(std::atol(w[k].c_str())); set_id[std::atol(w[0].c_str())] = v; } }
    else if (header == "leaf_id") { for (auto& l : body) { auto w = split_ws(l); leaf_id[std::atol(w[1].c_str())] = w[0]; } }
  }
  // addleafclades! (src/ccd.jl:199-216)
  std::map<long, std::string> leafclades;
  std::map<long, long> themap;
  for (auto& kv : set_id) {
    long k = kv.first; auto& v = kv.second;
    if (v.size() == 1) { bip[k] = observations; dip[k].clear(); leafclades[k] = leaf_id.at(v[0]); themap[v[0]] = k; }
    else { std::vector<long> nv; for (long x : v) nv.push_back(themap.at(x)); v = nv; }
  }
  for (auto& kv : themap) set_id[kv.second] = {kv.second};
  // addubiquitous! (src/ccd.jl:219-248)
  size_t nleaf = leafclades.size();
  long G = (long)set_id.size() + 1;
  long N = 0;
  std::vector<std::array<long, 3>> rootsplits;
  std::vector<std::vector<long>> l(G);  // l[i] sorted leaf sets (keys 1..G-1)
  for (auto& kv : set_id) { if (kv.first < 1 || kv.first >= G) throw std::runtime_error("set ids not contiguous"); auto v = kv.second; std::sort(v.begin(), v.end()); l[kv.first] = v; }
  // the reference scans all pairs i<j; each clade has at most one complement,
  // so pairs are found by hashing the complement (same pairs, same order).
  std::map<std::vector<long>, long> byset;
  for (long i = 1; i < G; ++i) byset[l[i]] = i;
  std::vector<long> all; for (auto& kv : leafclades) all.push_back(kv.first);
  std::sort(all.begin(), all.end());
  for (long i = 1; i < G; ++i) {
    if (l[i].size() >= nleaf) continue;
    std::vector<long> comp; std::set_difference(all.begin(), all.end(), l[i].begin(), l[i].end(), std::back_inserter(comp));
    if (comp.size() + l[i].size() != nleaf) continue;
    auto it = byset.find(comp);
    if (it == byset.end() || it->second <= i) continue;
    long j = it->second;
    if (bip.at(i) != bip.at(j)) throw std::runtime_error("complementary Bip counts differ");
    N += bip.at(i);
    rootsplits.push_back({i, j, bip.at(j)});
  }
  if (rootsplits.empty()) throw std::runtime_error("no root splits");
  dip[G] = rootsplits;
  bip[G] = N;
  { auto& t = rootsplits.back(); std::vector<long> u = l[t[0]]; u.insert(u.end(), l[t[1]].begin(), l[t[1]].end()); std::sort(u.begin(), u.end()); set_id[G] = u; }
  // CCD(ale, wm, spmap) (src/ccd.jl:102-121): order by (size, key)
  std::vector<std::pair<size_t, long>> ord;
  for (auto& kv : set_id) ord.push_back({kv.second.size(), kv.first});
  std::sort(ord.begin(), ord.end());
  std::map<long, int> idmap;
  for (size_t i = 0; i < ord.size(); ++i) idmap[ord[i].second] = (int)i;
  auto* c = new CCD();
  c->total = observations; c->fname = fname;
  for (size_t i = 0; i < ord.size(); ++i) {
    long k = ord[i].second;
    Clade cl; cl.id = (int)i; cl.count = bip.at(k);
    for (auto& t : dip[k]) cl.splits.push_back({idmap.at(t[0]), idmap.at(t[1]), (double)t[2] / (double)cl.count});
    std::set<int> sp;
    for (long x : set_id[k]) {
      const std::string& nm = leafclades.at(x);
      std::string pre = nm.substr(0, nm.find('_'));
      auto it = m.spmap.find(pre);
      if (it == m.spmap.end()) throw std::runtime_error("species not in tree: " + pre);
      sp.insert(it->second);
      cl.leaves.push_back((int)x);
    }
    cl.species.assign(sp.begin(), sp.end());
    c->clades.push_back(cl);
  }
  // index_and_getℓ (src/ccd.jl:59-75)
  size_t K = m.order.size();
  c->compat.resize(K); c->index.assign(K, std::vector<int>(c->clades.size(), -1));
  for (size_t k = 0; k < K; ++k) {
    const auto& cl = m.order[k].clade;
    int i = 0;
    for (auto& g : c->clades) {
      if (!std::includes(cl.begin(), cl.end(), g.species.begin(), g.species.end())) continue;
      c->compat[k].push_back(g.id);
      c->index[k][g.id] = i++;
    }
  }
  return c;
}

// ---------------------------------------------------------------------------
// The DP: src/core.jl:29-43 (logpdf!), :83-199 (whale!, whalewgd!,
// within_branch!, whaleroot!, Π*), src/ccd.jl:41-49 (getl).
// ---------------------------------------------------------------------------
template <class T>
struct Tab {  // ℓ[e] stored row-major [row][local column]
  int nrow = 0, ncol = 0;
  std::vector<T> a;
  T& at(int i, int j) { return a[(size_t)i * ncol + j]; }
};

template <class T>
static T getl(const CCD& x, std::vector<Tab<T>>& L, int e, int g, int row) {
  int j = x.index[e][g];
  return j < 0 ? T(0.0) : L[e].at(row, j);
}
template <class T>
static T getl_end(const CCD& x, std::vector<Tab<T>>& L, int e, int g) {
  int j = x.index[e][g];
  return j < 0 ? T(0.0) : L[e].at(L[e].nrow - 1, j);
}

template <class T>
static T Πspeciation(const CCD& x, const Clade& γ, std::vector<Tab<T>>& L, const MNode& n) {
  int f = n.ch[0], g = n.ch[1];
  T p = T(0.0);
  for (auto& t : γ.splits)
    p += t.p * (getl_end(x, L, f, t.g1) * getl_end(x, L, g, t.g2) + getl_end(x, L, g, t.g1) * getl_end(x, L, f, t.g2));
  return p;
}
template <class T>
static T Πloss(const CCD& x, const Clade& γ, std::vector<Tab<T>>& L, const MNode& n, const Tables<T>& tb) {
  int f = n.ch[0], g = n.ch[1];
  return getl_end(x, L, f, γ.id) * tb.eps[g].back() + getl_end(x, L, g, γ.id) * tb.eps[f].back();
}

template <class T>
static void within_branch(const CCD& x, const Clade& γ, std::vector<Tab<T>>& L, int e, int j, bool leaf, const Tables<T>& tb) {
  for (int i = 1; i < L[e].nrow; ++i) {
    L[e].at(i, j) = L[e].at(i, j) + tb.phi[e][i] * L[e].at(i - 1, j);
    if (!leaf) {
      T p = T(0.0);
      for (auto& t : γ.splits) p += t.p * getl(x, L, e, t.g1, i - 1) * getl(x, L, e, t.g2, i - 1);
      L[e].at(i, j) = L[e].at(i, j) + tb.psi[e][i] * p;
    }
  }
}

template <class T>
static T logpdf_family(const Model& m, const Tables<T>& tb, const CCD& x, std::vector<Tab<T>>* keep = nullptr) {
  size_t K = m.order.size();
  std::vector<Tab<T>> L(K);
  for (size_t k = 0; k < K; ++k) { L[k].nrow = m.order[k].nrow; L[k].ncol = (int)x.compat[k].size(); L[k].a.assign((size_t)L[k].nrow * L[k].ncol, T(0.0)); }
  for (size_t e = 0; e < K; ++e) {
    const MNode& n = m.order[e];
    if (n.wgd) {  // whalewgd!
      T q = tb.q[e];
      int f = n.ch[0];
      for (int c : x.compat[e]) {
        const Clade& γ = x.clades[c];
        int j = x.index[e][c];
        bool leaf = γ.leaves.size() == 1;
        T p = T(0.0);
        if (!leaf) {
          T s = T(0.0);
          for (auto& t : γ.splits) s += t.p * getl_end(x, L, f, t.g1) * getl_end(x, L, f, t.g2);
          p += s * q;
        }
        T lf = getl_end(x, L, f, γ.id);
        p += (1.0 - q) * lf + 2.0 * q * tb.eps[f].back() * lf;
        L[e].at(0, j) = p;
        within_branch(x, γ, L, (int)e, j, leaf, tb);
      }
    } else if (n.root) {  // whaleroot!
      T η = tb.eta;
      T ϵ = tb.eps[e].back();
      T ξ = 1.0 - (1.0 - η) * ϵ;
      for (auto& γ : x.clades) {
        bool leaf = γ.leaves.size() == 1;
        T a = T(0.0), b = T(0.0);
        T c = Πloss(x, γ, L, n, tb);
        if (!leaf) {
          T pr = T(0.0);
          for (auto& t : γ.splits) pr += t.p * getl(x, L, (int)e, t.g1, 0) * getl(x, L, (int)e, t.g2, 0);
          a += pr;
          b += Πspeciation(x, γ, L, n);
        }
        L[e].at(0, γ.id) = (1.0 - η) * ξ * a / η + (η * (1.0 - ϵ) / (ξ * ξ)) * (b + c);
      }
    } else {  // whale!
      for (int c : x.compat[e]) {
        const Clade& γ = x.clades[c];
        int j = x.index[e][c];
        bool leaf = γ.leaves.size() == 1;
        if (leaf && n.leaf) L[e].at(0, j) = T(n.leafP);
        else if (!n.leaf) L[e].at(0, j) = L[e].at(0, j) + (Πspeciation(x, γ, L, n) + Πloss(x, γ, L, n, tb));
        within_branch(x, γ, L, (int)e, j, leaf, tb);
      }
    }
  }
  int r = (int)K - 1;
  T Lr = L[r].at(0, L[r].ncol - 1);
  if (keep) *keep = L;
  return val(Lr) > 0 ? log(Lr) : T(-INFINITY);
}

// src/bdputil.jl:67
template <class T> static T geompgf(const T& p, const T& s) { return p * s / (1.0 - (1.0 - p) * s); }

// src/bdputil.jl:84-99: pgf of the linear birth-death process over time t
// (critical form when isapprox(λ, μ, atol=1e-6))
template <class T>
static T bdp_pgf(const T& λ, const T& μ, double t, const T& s) {
  if (std::fabs(val(λ) - val(μ)) <= 1e-6)
    return (1.0 - (λ * t - 1.0) * (s - 1.0)) / (1.0 - λ * t * (s - 1.0));
  T ρ = exp((μ - λ) * t);
  return (ρ * (λ * s - μ) - μ * (s - 1.0)) / (ρ * (λ * s - μ) - λ * (s - 1.0));
}

// src/bdputil.jl:114-135 (treepgf_allbinary and its inclusion-exclusion
// signs): the joint pgf of the leaf counts at every binary argument, the
// first child's index varying fastest, with the matching signs; a WGD node
// applies wgdpgf (src/bdputil.jl:104) before its branch, the root the
// geometric pgf of η.
template <class T>
static void treepgf_allbinary(const Model& m, const Rates<T>& r, int k, std::vector<T>& v, std::vector<double>& sg) {
  const MNode& n = m.order[k];
  const Theta<T> th = getθ(m, r, k);
  const double t = m.tree.n[n.tn].dist;
  std::vector<T> x;
  if (n.leaf) {
    x = {T(0.0), T(1.0)};
    sg = {1.0, -1.0};
  } else {
    x = {T(1.0)};
    sg = {1.0};
    for (int c : n.ch) {
      std::vector<T> vc;
      std::vector<double> sc;
      treepgf_allbinary(m, r, c, vc, sc);
      std::vector<T> nx;
      std::vector<double> ns;
      for (size_t j = 0; j < vc.size(); ++j)
        for (size_t i = 0; i < x.size(); ++i) {
          nx.push_back(x[i] * vc[j]);
          ns.push_back(sg[i] * sc[j]);
        }
      x.swap(nx);
      sg.swap(ns);
    }
  }
  v.resize(x.size());
  for (size_t i = 0; i < x.size(); ++i) {
    T y = n.wgd ? x[i] * (1.0 - th.q + x[i] * th.q) : x[i];
    v[i] = n.root ? geompgf(th.eta, y) : bdp_pgf(th.lam, th.mu, t, y);
  }
}

// src/condition.jl:11-36
template <class T>
static T condition(const Model& m, const Tables<T>& tb, const Rates<T>* rates = nullptr) {
  int r = (int)m.order.size() - 1;
  if (m.cond == COND_NONE) return T(0.0);
  if (m.cond == COND_NOWHERE) {
    if (!rates) throw std::runtime_error("NowhereExtinctCondition needs the rates");
    std::vector<T> v;
    std::vector<double> sg;
    treepgf_allbinary(m, *rates, r, v, sg);
    T acc(0.0);
    for (size_t i = 0; i + 1 < v.size(); ++i) acc = acc + v[i] * sg[i];
    T c = 1.0 - acc;
    return (val(c) > 0 && val(c) < 1) ? log(c) : T(-INFINITY);
  }
  T η = tb.eta;
  if (m.cond == COND_NONEXTINCT) return log(1.0 - geompgf(η, tb.eps[r].back()));
  int f = m.order[r].ch[0], g = m.order[r].ch[1];
  T ϵr = geompgf(η, tb.eps[r].back());
  T ϵf = geompgf(η, tb.eps[f].back());
  T ϵg = geompgf(η, tb.eps[g].back());
  T p = 1.0 - ϵf - ϵg + ϵr;
  return val(p) > 0 ? log(p) : T(-INFINITY);
}

}  // namespace orc

// ============================================================================
// C ABI for the tests and the CPU baseline (ctypes).
// ============================================================================
using namespace orc;

static thread_local std::string g_err;

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_model_new(const char* newick, double dt, int minn, int maxn, int cond) {
  try { return build_model(newick, dt, minn, maxn, cond); }
  catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_model_free(void* m) { delete (Model*)m; }

// per order position: id, wgdid, kind(0 leaf,1 internal,2 wgd,3 root), nrow, parent position
int orc_model_info(void* mp, int* n_nodes, int* nonwgd, int* nwgd, int* ids, int* wgdids, int* kinds, int* nrows, int* parents) {
  Model* m = (Model*)mp;
  *n_nodes = (int)m->order.size(); *nonwgd = m->nonwgd; *nwgd = m->nwgd;
  if (ids) for (size_t k = 0; k < m->order.size(); ++k) {
    auto& n = m->order[k];
    ids[k] = n.id; wgdids[k] = n.wgdid; nrows[k] = n.nrow; parents[k] = n.parent;
    kinds[k] = n.wgd ? 2 : (n.root ? 3 : (n.leaf ? 0 : 1));
  }
  return 0;
}

void* orc_ccd_new(void* mp, const char* text, const char* fname) {
  try { return parse_ccd(*(Model*)mp, text, fname ? fname : ""); }
  catch (std::exception& e) { g_err = e.what(); return nullptr; }
}
void orc_ccd_free(void* c) { delete (CCD*)c; }

// nclades, ntriples, and (optionally) per clade: count, nleaves, nsplits
int orc_ccd_info(void* cp, int* nclades, int* ntriples) {
  CCD* c = (CCD*)cp; *nclades = (int)c->clades.size(); long t = 0;
  for (auto& g : c->clades) t += (long)g.splits.size();
  *ntriples = (int)t; return 0;
}
// dump a clade table: for clade i: count, nleaves, species bitmask words (<= 2 words), splits (g1,g2,p)
int orc_ccd_clade(void* cp, int i, long* count, int* nleaves, int* nsplits, int* nspecies, int* species, int* g1, int* g2, double* p) {
  CCD* c = (CCD*)cp; auto& g = c->clades.at(i);
  *count = g.count; *nleaves = (int)g.leaves.size(); *nsplits = (int)g.splits.size(); *nspecies = (int)g.species.size();
  if (species) for (size_t k = 0; k < g.species.size(); ++k) species[k] = g.species[k];
  if (g1) for (size_t k = 0; k < g.splits.size(); ++k) { g1[k] = g.splits[k].g1; g2[k] = g.splits[k].g2; p[k] = g.splits[k].p; }
  return 0;
}

static Rates<double> make_rates(int kind, const double* lam, int nlam, const double* mu, int nmu, const double* q, int nq, double eta, const double* p, int np) {
  Rates<double> r; r.kind = kind;
  r.lam.assign(lam, lam + nlam); r.mu.assign(mu, mu + nmu); r.q.assign(q, q + nq); r.eta = eta;
  if (p && np > 0) r.p.assign(p, p + np);
  return r;
}

// Sum over families of per-family logL minus N * condition, mapped through
// ℓhood (src/core.jl:15, :58-64).  per_family[i] receives the unconditioned
// per-family logL (src/core.jl:39-43).  nthreads <= 0: all OpenMP threads.
double orc_logpdf(void* mp, int kind, const double* lam, int nlam, const double* mu, int nmu,
                  const double* q, int nq, double eta, const double* p, int np,
                  void** ccds, int nccd, double* per_family, int nthreads) {
  Model* m = (Model*)mp;
  Rates<double> r = make_rates(kind, lam, nlam, mu, nmu, q, nq, eta, p, np);
  Tables<double> tb = setmodel(*m, r);
  std::vector<double> ll(nccd);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
  for (int i = 0; i < nccd; ++i) ll[i] = logpdf_family(*m, tb, *(CCD*)ccds[i], (std::vector<Tab<double>>*)nullptr);
  double s = 0.0;
  for (int i = 0; i < nccd; ++i) { s += ll[i]; if (per_family) per_family[i] = ll[i]; }
  s = s - nccd * condition(*m, tb, &r);
  return std::isfinite(s) ? s : -INFINITY;
}

double orc_condition(void* mp, int kind, const double* lam, int nlam, const double* mu, int nmu,
                     const double* q, int nq, double eta, const double* p, int np) {
  Model* m = (Model*)mp;
  Rates<double> r = make_rates(kind, lam, nlam, mu, nmu, q, nq, eta, p, np);
  return condition(*m, setmodel(*m, r), &r);
}

// Slice tables for inspection: eps/phi/psi concatenated over order positions.
int orc_tables(void* mp, int kind, const double* lam, int nlam, const double* mu, int nmu,
               const double* q, int nq, double eta, const double* p, int np, double* eps, double* phi, double* psi) {
  Model* m = (Model*)mp;
  Rates<double> r = make_rates(kind, lam, nlam, mu, nmu, q, nq, eta, p, np);
  Tables<double> tb = setmodel(*m, r);
  size_t o = 0;
  for (size_t k = 0; k < m->order.size(); ++k)
    for (size_t i = 0; i < tb.eps[k].size(); ++i) { eps[o] = tb.eps[k][i]; phi[o] = tb.phi[k][i]; psi[o] = tb.psi[k][i]; ++o; }
  return (int)o;
}

// The DP table of one family: rows of every order position, row-major, with
// the local column order of `compat` (clade ids ascending).
int orc_family_tables(void* mp, int kind, const double* lam, int nlam, const double* mu, int nmu,
                      const double* q, int nq, double eta, const double* p, int np, void* cp, double* out, long cap) {
  Model* m = (Model*)mp;
  Rates<double> r = make_rates(kind, lam, nlam, mu, nmu, q, nq, eta, p, np);
  Tables<double> tb = setmodel(*m, r);
  std::vector<Tab<double>> keep;
  logpdf_family(*m, tb, *(CCD*)cp, &keep);
  long o = 0;
  for (auto& t : keep) for (double v : t.a) { if (o < cap) out[o] = v; ++o; }
  return (int)o;
}

// Gradient of orc_logpdf's total with respect to x = [λ (nlam), μ (nmu), q (nq), η]
// by chunked forward-mode duals (ForwardDiff.gradient stand-in).
double orc_gradient(void* mp, int kind, const double* lam, int nlam, const double* mu, int nmu,
                    const double* q, int nq, double eta, const double* p, int np,
                    void** ccds, int nccd, double* grad, int nthreads) {
  constexpr int C = WG_ORC_CHUNK;
  using D = Dual<C>;
  Model* m = (Model*)mp;
  int P = nlam + nmu + nq + 1;
  double total = 0;
  for (int c0 = 0; c0 < P; c0 += C) {
    Rates<D> r; r.kind = kind;
    auto seed = [&](int gi, double v) { D d(v); if (gi >= c0 && gi < c0 + C) d.d[gi - c0] = 1.0; return d; };
    for (int i = 0; i < nlam; ++i) r.lam.push_back(seed(i, lam[i]));
    for (int i = 0; i < nmu; ++i) r.mu.push_back(seed(nlam + i, mu[i]));
    for (int i = 0; i < nq; ++i) r.q.push_back(seed(nlam + nmu + i, q[i]));
    r.eta = seed(nlam + nmu + nq, eta);
    if (p && np > 0) r.p.assign(p, p + np);
    Tables<D> tb = setmodel(*m, r);
    std::vector<D> ll(nccd);
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
    for (int i = 0; i < nccd; ++i) ll[i] = logpdf_family(*m, tb, *(CCD*)ccds[i], (std::vector<Tab<D>>*)nullptr);
    D s(0.0);
    for (int i = 0; i < nccd; ++i) s += ll[i];
    s = s - (double)nccd * condition(*m, tb, &r);
    total = std::isfinite(s.v) ? s.v : -INFINITY;
    for (int k = 0; k < C && c0 + k < P; ++k) grad[c0 + k] = s.d[k];
  }
  return total;
}

}  // extern "C"
