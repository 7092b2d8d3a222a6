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
#include <memory>
#include <unordered_map>

#include "wg_internal.h"

namespace wg {

namespace {

struct Cursor {
  const char* p;
  const char* e;
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; }

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


// Tokens of one line [b, e) as integers or spans.  The reference deletes
// every ":\t" from a line before splitting it (src/ccd.jl:154); where each
// ':' is followed by a tab and preceded by whitespace (or starts the line),
// as in the set-id lines "12\t:\t3\t4", that equals reading ":\t" as blanks,
// which the scanner does in place.  Other lines take the literal deletion.
struct LineTokens {
  std::vector<std::pair<const char*, size_t>> tok;
  std::string buf;
  void split(const char* b, const char* e) {
    bool fast = true;  // every ':' reads as a blank
    for (const char* c = (const char*)memchr(b, ':', (size_t)(e - b)); c;
         c = c + 1 < e ? (const char*)memchr(c + 1, ':', (size_t)(e - c - 1)) : nullptr)
      if (c + 1 >= e || c[1] != '\t' || (c > b && !is_space(c[-1]))) {
        fast = false;
        break;
      }
    if (!fast) {
      buf.assign(b, e);
      for (size_t pos = buf.find(":\t"); pos != std::string::npos; pos = buf.find(":\t", pos)) buf.erase(pos, 2);
      b = buf.data();
      e = b + buf.size();
    }
    tok.clear();
    auto blank = [&](char ch) { return is_space(ch) || (fast && ch == ':'); };
    const char* p = b;
    while (p < e) {
      while (p < e && blank(*p)) ++p;
      const char* st = p;
      while (p < e && !blank(*p)) ++p;
      if (p > st) tok.emplace_back(st, (size_t)(p - st));
    }
  }
};

// A line of integers separated by blanks (and ":\t" read as a blank under
// the same rule as LineTokens) straight into `out`; false when the line has
// anything else, for the general path to handle (and report).
bool scan_ints(const char* b, const char* e, std::vector<int64_t>& out) {
  out.clear();
  const char* p = b;
  while (p < e) {
    const char ch = *p;
    if (is_space(ch)) {
      ++p;
      continue;
    }
    if (ch == ':') {
      if (p + 1 >= e || p[1] != '\t' || (p > b && !is_space(p[-1]))) return false;
      p += 2;
      continue;
    }
    bool neg = false;
    if (ch == '-' || ch == '+') neg = ch == '-', ++p;
    if (p >= e || *p < '0' || *p > '9') return false;
    int64_t v = 0;
    while (p < e && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
    if (p < e && !is_space(*p) && *p != ':') return false;
    out.push_back(neg ? -v : v);
  }
  return true;
}

int64_t count_lines(const char* b, const char* e) {
  int64_t n = 0;
  for (const char* p = b; p < e; ++p) n += *p == '\n';
  return n + 1;
}

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
  enum Kind { OTHER, OBS, BIP, DIP, SETID, LEAFID };
  struct Sec { Kind kind; const char* b; const char* e; };
  std::vector<Sec> secs;
  for (size_t si = 1; si + 1 < parts.size(); ++si) {
    const char* b = parts[si].first;
    const char* e = parts[si].second;
    const char* nl = (const char*)memchr(b, '\n', (size_t)(e - b));
    std::string header(b, nl ? nl : e);
    while (!header.empty() && (header.back() == '\r' || header.back() == ' ')) header.pop_back();
    for (char& c : header) if (c == '-') c = '_';
    const Kind k = header == "observations" ? OBS : header == "Bip_counts" ? BIP : header == "Dip_counts" ? DIP
                 : header == "set_id" ? SETID : header == "leaf_id" ? LEAFID : OTHER;
    secs.push_back({k, nl ? nl + 1 : e, e});
  }
  // Set ids must end up contiguous 1..G-1 (checked below), so every table
  // keyed by a set id is a vector over 0..G; keys outside are never read.
  int64_t set_lines = 0, leaf_lines = 0;  // leaf_lines: largest leaf number
  LineTokens lt;
  auto& tok = lt.tok;
  std::vector<std::pair<int64_t, std::string>> leaves;
  for (auto& sc : secs) {
    if (sc.kind == SETID) set_lines += count_lines(sc.b, sc.e);
    if (sc.kind != LEAFID) continue;
    for (const char* p = sc.b; p < sc.e;) {
      const char* le = (const char*)memchr(p, '\n', (size_t)(sc.e - p));
      if (!le) le = sc.e;
      lt.split(p, le);
      p = le + (le < sc.e ? 1 : 0);
      if (tok.empty()) continue;
      if (tok.size() < 2) throw Error(WG_EPARSE, "ALE: bad leaf-id line");
      const int64_t id = to_i64(tok[1]);
      if (id < 0 || id > (int64_t)1 << 31) throw Error(WG_EPARSE, "ALE: leaf id out of range");
      leaves.emplace_back(id, std::string(tok[0].first, tok[0].second));
      leaf_lines = std::max(leaf_lines, id);
    }
  }
  const int64_t cap = set_lines + 2;  // ids 0..set_lines, plus the ubiquitous clade
  int64_t observations = -1;
  std::vector<int64_t> bip(cap + 1, 0);
  std::vector<char> has_bip(cap + 1, 0), has_dip(cap + 1, 0), has_set(cap + 1, 0);
  // Dip lines in file order (parent, γ1, γ2, count); grouped by parent below
  std::vector<std::array<int64_t, 4>> diplines;
  // set-id lines: the members of set k are pool[set_off[k] .. + set_len[k])
  // (a repeated id: its last line)
  std::vector<int64_t> pool, set_off(cap + 1, 0), set_len(cap + 1, 0);
  std::vector<std::string> leaf_id(leaf_lines + 1);  // leaf number -> gene name
  std::vector<char> has_leaf(leaf_lines + 1, 0);
  for (auto& l : leaves) leaf_id[l.first] = std::move(l.second), has_leaf[l.first] = 1;
  std::vector<int64_t> ints;
  for (auto& sc : secs) {
    if (sc.kind == OTHER || sc.kind == LEAFID) continue;
    const char* p = sc.b;
    const char* e = sc.e;
    std::vector<int64_t>& v = ints;
    while (p < e) {
      const char* le = (const char*)memchr(p, '\n', (size_t)(e - p));
      if (!le) le = e;
      if (!scan_ints(p, le, v)) {  // not all integers: the general path converts (and reports)
        lt.split(p, le);
        v.clear();
        for (auto& t : tok) v.push_back(to_i64(t));
      }
      p = le + (le < e ? 1 : 0);
      if (v.empty()) continue;
      switch (sc.kind) {
        case OBS:
          observations = v[0];
          break;
        case BIP: {
          if (v.size() < 2) throw Error(WG_EPARSE, "ALE: bad Bip_counts line");
          if (v[0] >= 0 && v[0] <= cap) bip[v[0]] = v[1], has_bip[v[0]] = 1;
          break;
        }
        case DIP: {
          if (v.size() < 4) throw Error(WG_EPARSE, "ALE: bad Dip_counts line");
          if (v[0] >= 0 && v[0] <= cap) diplines.push_back({v[0], v[1], v[2], v[3]}), has_dip[v[0]] = 1;
          break;
        }
        case SETID: {
          const int64_t id = v[0];
          if (id < 1 || id >= cap) throw Error(WG_EPARSE, "ALE: set ids are not contiguous 1..n");
          set_off[id] = (int64_t)pool.size();
          set_len[id] = (int64_t)v.size() - 1;
          pool.insert(pool.end(), v.begin() + 1, v.end());
          has_set[id] = 1;
          break;
        }
        default:
          break;
      }
    }
  }
  if (observations < 0) throw Error(WG_EPARSE, "ALE: missing observations");
  // addleafclades!
  std::vector<std::string> leafname(cap + 1);  // leaf set id -> gene name
  std::vector<char> is_leafset(cap + 1, 0);
  std::vector<int64_t> themap(leaf_lines + 1, -1);  // leaf id -> set id
  for (int64_t k = 1; k < cap; ++k) {
    if (!has_set[k]) continue;
    int64_t* v = pool.data() + set_off[k];
    const int64_t len = set_len[k];
    if (len == 1) {
      const int64_t x = v[0];
      if (x < 0 || x > leaf_lines || !has_leaf[x]) throw Error(WG_EPARSE, "ALE: leaf id without a name");
      bip[k] = observations, has_bip[k] = 1;
      has_dip[k] = 1;  // leaf sets have no splits
      leafname[k] = leaf_id[x];
      is_leafset[k] = 1;
      themap[x] = k;
    } else {
      for (int64_t i = 0; i < len; ++i) {
        int64_t& x = v[i];
        if (x < 0 || x > leaf_lines || themap[x] < 0) throw Error(WG_EPARSE, "ALE: set refers to an unknown leaf");
        x = themap[x];
      }
    }
  }
  for (int64_t x = 0; x <= leaf_lines; ++x)
    if (themap[x] >= 0) pool[set_off[themap[x]]] = themap[x];
  // addubiquitous!
  int64_t nset = 0, kmin = -1, kmax = -1;
  for (int64_t k = 1; k < cap; ++k)
    if (has_set[k]) ++nset, kmax = k, kmin = kmin < 0 ? k : kmin;
  const int64_t G = nset + 1;
  size_t n = 0;
  for (int64_t k = 1; k < cap; ++k) n += is_leafset[k];
  if (n < 2) throw Error(WG_EPARSE, "ALE: fewer than two leaves");
  if (kmin != 1 || kmax != G - 1) throw Error(WG_EPARSE, "ALE: set ids are not contiguous 1..n");
  // leaf bit index: rank of each leaf set id
  std::vector<int> leafbit(cap + 1, -1);
  {
    int r = 0;
    for (int64_t k = 1; k < G; ++k)
      if (is_leafset[k]) leafbit[k] = r++;
  }
  const int W = (int)((n + 63) / 64);
  std::vector<uint64_t> bits((size_t)G * W, 0);
  auto hash_row = [W](const uint64_t* r) {
    uint64_t h = 1469598103934665603ull;
    for (int w = 0; w < W; ++w) h ^= r[w] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h;
  };
  // sets by (hash of the leaf bitset, id): the first id of equal sets wins
  // the complement lookup, as the first insert into a map keyed by the set
  std::vector<std::pair<uint64_t, int64_t>> byset;
  byset.reserve((size_t)G);
  for (int64_t k = 1; k < G; ++k) {
    uint64_t* b = bits.data() + (size_t)k * W;
    for (int64_t i = 0; i < set_len[k]; ++i) {
      const int64_t x = pool[set_off[k] + i];
      if (x < 1 || x >= G || leafbit[x] < 0) throw Error(WG_EPARSE, "ALE: set refers to a non-leaf set");
      b[leafbit[x] >> 6] |= 1ull << (leafbit[x] & 63);
    }
    byset.emplace_back(hash_row(b), k);
  }
  std::sort(byset.begin(), byset.end());
  auto find_set = [&](const uint64_t* r) -> int64_t {
    auto it = std::lower_bound(byset.begin(), byset.end(), std::make_pair(hash_row(r), (int64_t)0));
    for (; it != byset.end() && it->first == hash_row(r); ++it)
      if (std::memcmp(bits.data() + (size_t)it->second * W, r, sizeof(uint64_t) * W) == 0) return it->second;
    return -1;
  };
  std::vector<uint64_t> all(W, 0);
  for (size_t i = 0; i < n; ++i) all[i >> 6] |= 1ull << (i & 63);
  std::vector<std::array<int64_t, 3>> rootsplits;
  int64_t N = 0;
  std::vector<uint64_t> c(W);
  for (int64_t i = 1; i < G; ++i) {
    bool empty = true;
    for (int w = 0; w < W; ++w) { c[w] = all[w] & ~bits[(size_t)i * W + w]; empty &= c[w] == 0; }
    if (empty) continue;
    const int64_t j = find_set(c.data());
    if (j < 0 || j <= i) continue;
    if (!has_bip[i] || !has_bip[j]) throw Error(WG_EPARSE, "ALE: missing Bip count");
    if (bip[i] != bip[j]) throw Error(WG_EPARSE, "ALE: complementary clades have different Bip counts");
    N += bip[i];
    rootsplits.push_back({i, j, bip[j]});
  }
  if (rootsplits.empty()) throw Error(WG_EPARSE, "ALE: no complementary clade pairs for the root");
  has_dip[G] = 1;  // its splits: rootsplits (Dip lines of G are not read)
  bip[G] = N, has_bip[G] = 1;
  {
    const int64_t i = rootsplits.back()[0], j = rootsplits.back()[1];
    std::vector<int64_t> u(pool.begin() + set_off[i], pool.begin() + set_off[i] + set_len[i]);
    u.insert(u.end(), pool.begin() + set_off[j], pool.begin() + set_off[j] + set_len[j]);
    std::sort(u.begin(), u.end());
    set_off[G] = (int64_t)pool.size();
    set_len[G] = (int64_t)u.size();
    pool.insert(pool.end(), u.begin(), u.end());
  }
  // Dip lines grouped by parent, in file order within a parent
  std::vector<int64_t> dip_off(cap + 2, 0);
  for (const auto& d : diplines) ++dip_off[d[0] + 1];
  for (int64_t k = 0; k <= cap; ++k) dip_off[k + 1] += dip_off[k];
  std::vector<std::array<int64_t, 3>> dipv(diplines.size());
  {
    std::vector<int64_t> cur(dip_off.begin(), dip_off.end() - 1);
    for (const auto& d : diplines) dipv[cur[d[0]]++] = {d[1], d[2], d[3]};
  }
  // splits of set k: none for leaf sets, the complementary pairs for G
  auto splits = [&](int64_t k) -> std::pair<const std::array<int64_t, 3>*, size_t> {
    if (k == G) return {rootsplits.data(), rootsplits.size()};
    if (is_leafset[k]) return {nullptr, 0};
    return {dipv.data() + dip_off[k], (size_t)(dip_off[k + 1] - dip_off[k])};
  };
  // CCD(ale, wm, spmap): order by (size, key)
  std::vector<std::pair<size_t, int64_t>> ord;
  ord.reserve((size_t)G);
  for (int64_t k = 1; k <= G; ++k) ord.emplace_back((size_t)set_len[k], k);
  std::sort(ord.begin(), ord.end());
  std::vector<int> idmap(cap + 1, -1);
  for (size_t i = 0; i < ord.size(); ++i) idmap[ord[i].second] = (int)i;
  std::unordered_map<std::string, int> spmap;
  for (size_t i = 0; i < names.size(); ++i) spmap[names[i]] = ids[i];
  std::vector<int> leafsp(cap + 1, -1);
  for (int64_t k = 1; k < G; ++k) {
    if (!is_leafset[k]) continue;
    const std::string& nm = leafname[k];
    const std::string pre = nm.substr(0, nm.find('_'));
    auto it = spmap.find(pre);
    if (it == spmap.end()) throw Error(WG_EPARSE, "ALE: gene '" + nm + "' has no species '" + pre + "' in the tree");
    leafsp[k] = it->second;
  }
  auto* cc = new CCD();
  std::unique_ptr<CCD> guard(cc);
  cc->n_clades = (int)ord.size();
  cc->observations = observations;
  cc->n_genes = (int)n;
  {
    size_t nsplit = 0;
    for (auto& o : ord) nsplit += splits(o.second).second;
    cc->g1.reserve(nsplit), cc->g2.reserve(nsplit), cc->p.reserve(nsplit);
    for (auto* v : {&cc->nleaves, &cc->split_off, &cc->sp_off}) v->reserve(ord.size() + 1);
    cc->counts.reserve(ord.size());
    cc->leaf_name.reserve(ord.size());
    cc->sp.reserve(ord.size() * 4);
  }
  cc->sp_off.push_back(0);
  cc->split_off.push_back(0);
  std::vector<int> sp;
  // a clade's species, deduplicated by stamping (then sorted: few distinct)
  int max_sp = 0;
  for (int id : ids) {
    if (id < 0) throw Error(WG_EINVAL, "negative species id");
    max_sp = std::max(max_sp, id);
  }
  std::vector<int64_t> stamp((size_t)max_sp + 1, -1);
  for (size_t i = 0; i < ord.size(); ++i) {
    const int64_t k = ord[i].second;
    if (!has_bip[k]) throw Error(WG_EPARSE, "ALE: clade without a Bip count");
    cc->nleaves.push_back((int)ord[i].first);
    cc->leaf_name.push_back(ord[i].first == 1 ? leafname[pool[set_off[k]]] : std::string());
    cc->counts.push_back(bip[k]);
    if (!has_dip[k] && ord[i].first > 1) throw Error(WG_EPARSE, "ALE: clade without Dip counts");
    const auto sk = splits(k);
    for (size_t q = 0; q < sk.second; ++q) {
      const auto& t = sk.first[q];
      const int a = t[0] >= 0 && t[0] <= cap ? idmap[t[0]] : -1, b = t[1] >= 0 && t[1] <= cap ? idmap[t[1]] : -1;
      if (a < 0 || b < 0) throw Error(WG_EPARSE, "ALE: split refers to an unknown set");
      cc->g1.push_back(a);
      cc->g2.push_back(b);
      cc->p.push_back((double)t[2] / (double)bip[k]);
    }
    cc->split_off.push_back((int)cc->g1.size());
    sp.clear();
    for (int64_t q = 0; q < set_len[k]; ++q) {
      const int s = leafsp[pool[set_off[k] + q]];
      if (stamp[s] != k) stamp[s] = k, sp.push_back(s);
    }
    std::sort(sp.begin(), sp.end());
    cc->sp.insert(cc->sp.end(), sp.begin(), sp.end());
    cc->sp_off.push_back((int)cc->sp.size());
  }
  return guard.release();
}

}  // namespace wg
