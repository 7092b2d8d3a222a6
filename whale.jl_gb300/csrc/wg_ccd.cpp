// Native ALE v0.4 reader: one pass over the text into the CCD layout the DP
// uses.  Semantics follow the reference reader:
//   parse_aleobserve / parse_body   src/ccd.jl:147-185  (sections split on '#',
//                                   8 sections, ":\t" removed, '-' -> '_' in headers)
//   addleafclades!                  src/ccd.jl:199-216  (leaf sets get Bip =
//                                   observations and no splits; set ids of
//                                   leaves replace leaf ids)
//   addubiquitous!                  src/ccd.jl:219-248  (root clade split into
//                                   every complementary pair i < j, p = Bip[j]/N)
//   CCD(ale, wm, spmap)             src/ccd.jl:102-121  (clades sorted by (size,
//                                   set id); p = Dip / Bip of the parent)
//   getspecies                      src/ccd.jl:139      (species = gene-name
//                                   prefix before the first '_')
// The ubiquitous clade's complementary pairs are found by hashing each
// clade's complement instead of the reference's all-pairs scan; the pairs and
// their order (ascending i) are the same.
#include <algorithm>
#include <array>
#include <cstring>
#include <string>
#include <map>
#include <unordered_map>

#include "wg_internal.h"

namespace wg {

namespace {

struct Cursor {
  const char* p;
  const char* e;
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; }

// Split a section body into whitespace-separated tokens per line.
void tokens_of_line(const char* b, const char* e, std::vector<std::pair<const char*, size_t>>& out) {
  out.clear();
  const char* p = b;
  while (p < e) {
    while (p < e && is_space(*p)) ++p;
    const char* s = p;
    while (p < e && !is_space(*p)) ++p;
    if (p > s) out.emplace_back(s, (size_t)(p - s));
  }
}

int64_t to_i64(const std::pair<const char*, size_t>& t) {
  int64_t v = 0;
  bool neg = false;
  size_t i = 0;
  if (i < t.second && (t.first[i] == '-' || t.first[i] == '+')) { neg = t.first[i] == '-'; ++i; }
  if (i == t.second) throw Error(WG_EPARSE, "ALE: expected an integer");
  for (; i < t.second; ++i) {
    char c = t.first[i];
    if (c < '0' || c > '9') throw Error(WG_EPARSE, "ALE: expected an integer, got '" + std::string(t.first, t.second) + "'");
    v = v * 10 + (c - '0');
  }
  return neg ? -v : v;
}

struct Hash64 {
  size_t operator()(const std::vector<uint64_t>& v) const {
    uint64_t h = 1469598103934665603ull;
    for (uint64_t x : v) { h ^= x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2); }
    return (size_t)h;
  }
};

}  // namespace

CCD* parse_ale(const char* text, size_t len, const std::vector<std::string>& names, const std::vector<int>& ids) {
  // sections = split(alestring, "#")[2:end-1]
  std::vector<std::pair<const char*, const char*>> parts;
  {
    const char* s = text;
    const char* e = text + len;
    const char* p = s;
    while (true) {
      const char* h = (const char*)memchr(p, '#', (size_t)(e - p));
      if (!h) { parts.emplace_back(p, e); break; }
      parts.emplace_back(p, h);
      p = h + 1;
    }
  }
  if (parts.size() < 2 || parts.size() - 2 != 8) throw Error(WG_EPARSE, "Not a valid .ale file (expected 8 sections)");
  int64_t observations = -1;
  std::unordered_map<int64_t, int64_t> bip;
  std::unordered_map<int64_t, std::vector<std::array<int64_t, 3>>> dip;
  std::map<int64_t, std::vector<int64_t>> set_id;     // ordered by key (sort!(OrderedDict(...)))
  std::unordered_map<int64_t, std::string> leaf_id;  // leaf number -> gene name
  std::vector<std::pair<const char*, size_t>> tok;
  for (size_t si = 1; si + 1 < parts.size(); ++si) {
    const char* b = parts[si].first;
    const char* e = parts[si].second;
    const char* nl = (const char*)memchr(b, '\n', (size_t)(e - b));
    std::string header(b, nl ? nl : e);
    while (!header.empty() && (header.back() == '\r' || header.back() == ' ')) header.pop_back();
    for (char& c : header) if (c == '-') c = '_';
    const char* p = nl ? nl + 1 : e;
    while (p < e) {
      const char* le = (const char*)memchr(p, '\n', (size_t)(e - p));
      if (!le) le = e;
      // remove ":\t" (src/ccd.jl:154): it only occurs as the set-id separator
      std::string line(p, le);
      for (size_t pos = line.find(":\t"); pos != std::string::npos; pos = line.find(":\t", pos)) line.erase(pos, 2);
      tokens_of_line(line.data(), line.data() + line.size(), tok);
      p = le + (le < e ? 1 : 0);
      if (tok.empty()) continue;
      if (header == "observations") {
        observations = to_i64(tok[0]);
      } else if (header == "Bip_counts") {
        if (tok.size() < 2) throw Error(WG_EPARSE, "ALE: bad Bip_counts line");
        bip[to_i64(tok[0])] = to_i64(tok[1]);
      } else if (header == "Dip_counts") {
        if (tok.size() < 4) throw Error(WG_EPARSE, "ALE: bad Dip_counts line");
        dip[to_i64(tok[0])].push_back({to_i64(tok[1]), to_i64(tok[2]), to_i64(tok[3])});
      } else if (header == "set_id") {
        std::vector<int64_t> v;
        for (size_t k = 1; k < tok.size(); ++k) v.push_back(to_i64(tok[k]));
        set_id[to_i64(tok[0])] = std::move(v);
      } else if (header == "leaf_id") {
        if (tok.size() < 2) throw Error(WG_EPARSE, "ALE: bad leaf-id line");
        leaf_id[to_i64(tok[1])] = std::string(tok[0].first, tok[0].second);
      }
    }
  }
  if (observations < 0) throw Error(WG_EPARSE, "ALE: missing observations");
  // addleafclades!
  std::unordered_map<int64_t, std::string> leafname;  // leaf set id -> gene name
  std::unordered_map<int64_t, int64_t> themap;        // leaf id -> set id
  for (auto& kv : set_id) {
    auto& v = kv.second;
    if (v.size() == 1) {
      auto it = leaf_id.find(v[0]);
      if (it == leaf_id.end()) throw Error(WG_EPARSE, "ALE: leaf id without a name");
      bip[kv.first] = observations;
      dip[kv.first].clear();
      leafname[kv.first] = it->second;
      themap[v[0]] = kv.first;
    } else {
      for (auto& x : v) {
        auto it = themap.find(x);
        if (it == themap.end()) throw Error(WG_EPARSE, "ALE: set refers to an unknown leaf");
        x = it->second;
      }
    }
  }
  for (auto& kv : themap) set_id[kv.second] = {kv.second};
  // addubiquitous!
  const int64_t G = (int64_t)set_id.size() + 1;
  const size_t n = leafname.size();
  if (n < 2) throw Error(WG_EPARSE, "ALE: fewer than two leaves");
  if (set_id.begin()->first != 1 || set_id.rbegin()->first != G - 1)
    throw Error(WG_EPARSE, "ALE: set ids are not contiguous 1..n");
  // leaf bit index: rank of each leaf set id
  std::unordered_map<int64_t, int> leafbit;
  {
    std::vector<int64_t> ls;
    for (auto& kv : leafname) ls.push_back(kv.first);
    std::sort(ls.begin(), ls.end());
    for (size_t i = 0; i < ls.size(); ++i) leafbit[ls[i]] = (int)i;
  }
  const int W = (int)((n + 63) / 64);
  std::vector<std::vector<uint64_t>> bits(G);
  std::unordered_map<std::vector<uint64_t>, int64_t, Hash64> byset;
  for (auto& kv : set_id) {
    std::vector<uint64_t> b(W, 0);
    for (int64_t x : kv.second) {
      auto it = leafbit.find(x);
      if (it == leafbit.end()) throw Error(WG_EPARSE, "ALE: set refers to a non-leaf set");
      b[it->second >> 6] |= 1ull << (it->second & 63);
    }
    bits[kv.first] = b;
    byset.emplace(b, kv.first);
  }
  std::vector<uint64_t> all(W, 0);
  for (size_t i = 0; i < n; ++i) all[i >> 6] |= 1ull << (i & 63);
  std::vector<std::array<int64_t, 3>> rootsplits;
  int64_t N = 0;
  for (int64_t i = 1; i < G; ++i) {
    std::vector<uint64_t> c(W);
    bool empty = true;
    for (int w = 0; w < W; ++w) { c[w] = all[w] & ~bits[i][w]; empty &= c[w] == 0; }
    if (empty) continue;
    auto it = byset.find(c);
    if (it == byset.end() || it->second <= i) continue;
    const int64_t j = it->second;
    auto bi = bip.find(i), bj = bip.find(j);
    if (bi == bip.end() || bj == bip.end()) throw Error(WG_EPARSE, "ALE: missing Bip count");
    if (bi->second != bj->second) throw Error(WG_EPARSE, "ALE: complementary clades have different Bip counts");
    N += bi->second;
    rootsplits.push_back({i, j, bj->second});
  }
  if (rootsplits.empty()) throw Error(WG_EPARSE, "ALE: no complementary clade pairs for the root");
  dip[G] = rootsplits;
  bip[G] = N;
  {
    std::vector<int64_t> u = set_id[rootsplits.back()[0]];
    const auto& v = set_id[rootsplits.back()[1]];
    u.insert(u.end(), v.begin(), v.end());
    std::sort(u.begin(), u.end());
    set_id[G] = u;
  }
  // CCD(ale, wm, spmap): order by (size, key)
  std::vector<std::pair<size_t, int64_t>> ord;
  ord.reserve(set_id.size());
  for (auto& kv : set_id) ord.emplace_back(kv.second.size(), kv.first);
  std::sort(ord.begin(), ord.end());
  std::unordered_map<int64_t, int> idmap;
  for (size_t i = 0; i < ord.size(); ++i) idmap[ord[i].second] = (int)i;
  std::unordered_map<std::string, int> spmap;
  for (size_t i = 0; i < names.size(); ++i) spmap[names[i]] = ids[i];
  std::unordered_map<int64_t, int> leafsp;
  for (auto& kv : leafname) {
    const std::string& nm = kv.second;
    const std::string pre = nm.substr(0, nm.find('_'));
    auto it = spmap.find(pre);
    if (it == spmap.end()) throw Error(WG_EPARSE, "ALE: gene '" + nm + "' has no species '" + pre + "' in the tree");
    leafsp[kv.first] = it->second;
  }
  auto* c = new CCD();
  c->n_clades = (int)ord.size();
  c->observations = observations;
  c->n_genes = (int)n;
  c->sp_off.push_back(0);
  c->split_off.push_back(0);
  std::vector<int> sp;
  for (size_t i = 0; i < ord.size(); ++i) {
    const int64_t k = ord[i].second;
    auto bi = bip.find(k);
    if (bi == bip.end()) throw Error(WG_EPARSE, "ALE: clade without a Bip count");
    c->nleaves.push_back((int)ord[i].first);
    c->leaf_name.push_back(ord[i].first == 1 ? leafname.at(*set_id[k].begin()) : std::string());
    c->counts.push_back(bi->second);
    auto di = dip.find(k);
    if (di == dip.end() && ord[i].first > 1) throw Error(WG_EPARSE, "ALE: clade without Dip counts");
    if (di != dip.end()) {
      for (auto& t : di->second) {
        auto a = idmap.find(t[0]), b = idmap.find(t[1]);
        if (a == idmap.end() || b == idmap.end()) throw Error(WG_EPARSE, "ALE: split refers to an unknown set");
        c->g1.push_back(a->second);
        c->g2.push_back(b->second);
        c->p.push_back((double)t[2] / (double)bi->second);
      }
    }
    c->split_off.push_back((int)c->g1.size());
    sp.clear();
    for (int64_t x : set_id[k]) sp.push_back(leafsp.at(x));
    std::sort(sp.begin(), sp.end());
    sp.erase(std::unique(sp.begin(), sp.end()), sp.end());
    c->sp.insert(c->sp.end(), sp.begin(), sp.end());
    c->sp_off.push_back((int)c->sp.size());
  }
  return c;
}

}  // namespace wg
