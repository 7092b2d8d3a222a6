// Packer: turns a batch of CCDs plus the species-tree model into the device
// layout of the batched DP.
//
// What the reference does per call (src/core.jl:41, src/ccd.jl:59-75): for
// every species node e it lists the clades compatible with e (species(γ) ⊆
// clade(e), src/ccd.jl:39) in clade-id order and indexes every operand of the
// DP through index[γ, e] (getl, src/ccd.jl:41-49).  Here that indirection is
// resolved once, on the host, at batch creation:
//
//   * families are packed into groups; a group's row for node e is the
//     concatenation of its families' compatible-clade lists, so one CTA runs
//     the DP of all of them in lock step (they share the slice tables);
//   * every sum over split triples of the DP (Πduplication :178-185,
//     Πspeciation :160-170, Πwgdretention :187-194, Πroot :151-158) becomes a
//     statically scheduled "sum program" whose operands are row positions,
//     so the device never looks anything up;
//   * speciation terms that are zero in the reference because an operand
//     clade is incompatible with a child (getl returns 0) are dropped;
//   * the root's same-row dependency (Πroot reads row 1 of the root itself)
//     is ordered into levels of the split DAG.
// The transposed programs the adjoint needs are built here as well.
#include <algorithm>
#include <limits>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <exception>
#include <numeric>
#include <thread>

#include "wg_internal.h"

namespace wg {

namespace {

struct Ent {
  int a, b;
  double p;
};

using Work = std::vector<std::pair<int, std::vector<Ent>>>;  // (destination position, entries)

struct Fin {
  std::vector<std::array<int, 2>> v;  // per position: slot start, segments
};

// Statically schedule a sum program.  Lanes get contiguous runs of whole
// segments (first-fit decreasing into equal-capacity lanes); a clade's
// entries are split into ceil(s / J) segments so that no lane holds more
// than J entries.  Cost model: J * warps warp-iterations of FP64 work.
DProg schedule(const Work& work, std::vector<DEntry>& out, Fin& fin, int& nslots) {
  DProg prog;
  prog.off = (int64_t)out.size();
  int64_t W = 0;
  for (auto& w : work) W += (int64_t)w.second.size();
  nslots = 0;
  if (W == 0) return prog;
  int best_w = 1;
  int64_t best_cost = INT64_MAX;
  for (int w = 1; w <= kNT / 32; ++w) {
    const int64_t J = (W + 32 * w - 1) / (32 * w);
    const int64_t cost = J * w;
    if (cost < best_cost) { best_cost = cost; best_w = w; }
  }
  const int NB = 32 * best_w;
  int J = (int)((W + NB - 1) / NB);
  struct Seg { int item, k, begin, len; };
  std::vector<Seg> segs;
  std::vector<std::vector<int>> bins;
  while (true) {
    segs.clear();
    for (int it = 0; it < (int)work.size(); ++it) {
      const int s = (int)work[it].second.size();
      if (s == 0) continue;
      const int nseg = (s + J - 1) / J;
      const int base = s / nseg, rem = s % nseg;
      int start = 0;
      for (int k = 0; k < nseg; ++k) {
        const int len = base + (k < rem ? 1 : 0);
        segs.push_back({it, k, start, len});
        start += len;
      }
    }
    std::vector<int> order(segs.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return segs[x].len > segs[y].len; });
    bins.assign(NB, {});
    std::vector<int> load(NB, 0);
    bool ok = true;
    int first_open = 0;
    for (int si : order) {
      const int len = segs[si].len;
      int b = first_open;
      while (b < NB && load[b] + len > J) ++b;
      if (b == NB) { ok = false; break; }
      bins[b].push_back(si);
      load[b] += len;
      while (first_open < NB && load[first_open] == J) ++first_open;
    }
    if (ok) break;
    ++J;
  }
  // slots: contiguous per destination
  std::vector<int> slot_start(work.size(), 0);
  for (int it = 0; it < (int)work.size(); ++it) {
    const int s = (int)work[it].second.size();
    if (s == 0) continue;
    const int nseg = (s + J - 1) / J;
    slot_start[it] = nslots;
    fin.v[work[it].first] = {nslots, nseg};
    nslots += nseg;
  }
  if (nslots >= 65535) throw Error(WG_ERANGE, "sum program exceeds 65535 partial slots");
  int used = 0;
  for (int b = 0; b < NB; ++b) if (!bins[b].empty()) used = b + 1;
  const int nt = ((used + 31) / 32) * 32;
  prog.J = J;
  prog.nt = nt;
  out.resize(out.size() + (size_t)J * nt, DEntry{0, 0.0});
  DEntry* base = out.data() + prog.off;
  for (int t = 0; t < nt; ++t) {
    int j = 0;
    for (int si : bins[t]) {
      const Seg& sg = segs[si];
      const auto& ents = work[sg.item].second;
      const int slot = slot_start[sg.item] + sg.k;
      for (int q = 0; q < sg.len; ++q, ++j) {
        const Ent& e = ents[sg.begin + q];
        const uint64_t flags = kValid | (q == sg.len - 1 ? kEnd : 0);
        base[(size_t)j * nt + t].code = (uint64_t)e.a | ((uint64_t)e.b << 16) | ((uint64_t)slot << 32) | (flags << 48);
        base[(size_t)j * nt + t].p = e.p;
      }
    }
  }
  return prog;
}

int64_t put_fin(std::vector<int32_t>& meta, const Fin& fin) {
  if (meta.size() & 1) meta.push_back(0);
  const int64_t off = (int64_t)meta.size() / 2;  // in int2 units
  for (auto& f : fin.v) { meta.push_back(f[0]); meta.push_back(f[1]); }
  return off;
}

int64_t put_int2(std::vector<int32_t>& meta, const std::vector<std::array<int, 2>>& v) {
  if (meta.size() & 1) meta.push_back(0);
  const int64_t off = (int64_t)meta.size() / 2;
  for (auto& f : v) { meta.push_back(f[0]); meta.push_back(f[1]); }
  return off;
}

int64_t put_int(std::vector<int32_t>& meta, const std::vector<int>& v) {
  const int64_t off = (int64_t)meta.size();
  meta.insert(meta.end(), v.begin(), v.end());
  return off;
}

// Per-family compatibility of clades with species nodes (src/ccd.jl:39,59-75).
struct FamInfo {
  std::vector<std::vector<int>> idx;  // [node][clade] -> local column, -1 if incompatible
  std::vector<int> ncompat;           // [node]
};

void compat_of(const Model& m, const CCD& c, FamInfo& fi, bool want_idx) {
  const int W = m.n_words;
  std::vector<uint64_t> bits((size_t)c.n_clades * W, 0);
  for (int g = 0; g < c.n_clades; ++g)
    for (int s = c.sp_off[g]; s < c.sp_off[g + 1]; ++s) {
      const int id = c.sp[s];
      if (id < 0 || id >= 64 * W) throw Error(WG_EINVAL, "CCD species id outside the model's species range");
      bits[(size_t)g * W + (id >> 6)] |= 1ull << (id & 63);
    }
  fi.ncompat.assign(m.K, 0);
  if (want_idx) fi.idx.assign(m.K, std::vector<int>(c.n_clades, -1));
  for (int k = 0; k < m.K; ++k) {
    const uint64_t* cl = &m.clade_bits[(size_t)k * W];
    int n = 0;
    for (int g = 0; g < c.n_clades; ++g) {
      const uint64_t* b = &bits[(size_t)g * W];
      bool ok = true;
      for (int w = 0; w < W && ok; ++w) ok = (b[w] & ~cl[w]) == 0;
      if (ok) { if (want_idx) fi.idx[k][g] = n; ++n; }
    }
    fi.ncompat[k] = n;
  }
}

// Algorithmic FP64 work and bytes of one family, counted on the reference's
// data structures (every split of every compatible non-leaf clade).
void family_cost(const Model& m, const CCD& c, const FamInfo& fi, double& flops, double& bytes, double& flops_adj,
                 double& work) {
  flops = bytes = flops_adj = work = 0;
  for (int k = 0; k < m.K; ++k) {
    double T = 0, Cn = 0, Cnl = 0;
    for (int g = 0; g < c.n_clades; ++g) {
      if (fi.idx[k][g] < 0) continue;
      Cn += 1;
      if (c.nleaves[g] > 1) { Cnl += 1; T += c.split_off[g + 1] - c.split_off[g]; }
    }
    const double n = m.kind[k] == WG_NODE_ROOT ? 0 : m.nrow[k] - 1;
    flops += n * (3 * T + 2 * Cn + 2 * Cnl);
    flops_adj += n * (6 * T + 7 * Cn);
    if (m.kind[k] == WG_NODE_ROOT) { flops += 10 * T + 7 * Cn; flops_adj += 16 * T + 10 * Cn; }
    else if (m.kind[k] != WG_NODE_LEAF) { flops += 5 * T + 4 * Cn; flops_adj += 8 * T + 6 * Cn; }
    bytes += 16 * T + 8 * Cn;
    work += (n + 1) * (T + Cn);
  }
  bytes += 8.0 * 3 * m.total_rows() / 1.0 + 8;
}

// Levels of the split DAG of the root row: a clade's level is one more than
// the largest level of its split operands; clades without splits are level 0.
std::vector<int> split_levels(const CCD& c) {
  std::vector<int> lvl(c.n_clades, 0);
  for (int g = 0; g < c.n_clades; ++g) {
    int L = 0;
    for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) L = std::max(L, 1 + std::max(lvl[c.g1[s]], lvl[c.g2[s]]));
    lvl[g] = L;
  }
  return lvl;
}

}  // namespace

Packed pack_batch(const Model& m, const std::vector<const CCD*>& ccds, const PackOptions& opt) {
  Packed P;
  const int K = m.K;
  const int NF = (int)ccds.size();
  if (NF == 0) throw Error(WG_EINVAL, "empty batch");
  // ---- pass 1: sizes and work per family
  std::vector<double> work(NF), width(NF);
  for (int f = 0; f < NF; ++f) {
    FamInfo fi;
    compat_of(m, *ccds[f], fi, true);
    double fl, by, fa, w;
    family_cost(m, *ccds[f], fi, fl, by, fa, w);
    P.flops_fwd += fl;
    P.bytes_fwd += by;
    P.flops_adj += fa;
    work[f] = w;
    width[f] = ccds[f]->n_clades;
    if (ccds[f]->n_clades >= 65535) throw Error(WG_ERANGE, "CCD with 65535 or more clades");
  }
  // ---- grouping: families sorted by clade count, consecutive ones packed
  std::vector<int> ord(NF);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return width[a] > width[b]; });
  std::vector<std::vector<int>> groups;
  {
    std::vector<int> cur;
    int64_t w = 0;
    for (int f : ord) {
      if (!cur.empty() && (opt.single || w + (int64_t)width[f] > opt.group_cap || w >= opt.group_width)) {
        groups.push_back(cur);
        cur.clear();
        w = 0;
      }
      cur.push_back(f);
      w += (int64_t)width[f];
    }
    if (!cur.empty()) groups.push_back(cur);
  }
  // heaviest groups first (they start first on the device)
  std::vector<double> gwork(groups.size(), 0);
  for (size_t g = 0; g < groups.size(); ++g)
    for (int f : groups[g]) gwork[g] += work[f];
  std::vector<int> gord(groups.size());
  std::iota(gord.begin(), gord.end(), 0);
  std::stable_sort(gord.begin(), gord.end(), [&](int a, int b) { return gwork[a] > gwork[b]; });

  int max_smem = 0;
  P.fam_node0.assign(NF, 0);
  P.fam_col.assign((size_t)NF * K, 0);
  P.fam_ncol.assign((size_t)NF * K, 0);
  for (int gi : gord) {
    const auto& fams = groups[gi];
    const int nf = (int)fams.size();
    std::vector<FamInfo> info(nf);
    std::vector<std::vector<int>> lvl(nf);
    for (int i = 0; i < nf; ++i) {
      compat_of(m, *ccds[fams[i]], info[i], true);
      lvl[i] = split_levels(*ccds[fams[i]]);
    }
    // row offsets of each family in each node's row
    std::vector<std::vector<int>> off(K, std::vector<int>(nf + 1, 0));
    std::vector<int> R(K, 0);
    for (int k = 0; k < K; ++k) {
      for (int i = 0; i < nf; ++i) off[k][i + 1] = off[k][i] + info[i].ncompat[k];
      R[k] = off[k][nf];
      if (R[k] >= 65535) throw Error(WG_ERANGE, "group row wider than 65535 clades");
    }
    auto pos = [&](int i, int k, int g) -> int {
      const int j = info[i].idx[k][g];
      return j < 0 ? -1 : off[k][i] + j;
    };
    DGroup G;
    G.n_fam = nf;
    G.node0 = (int64_t)P.nodes.size();
    G.fam0 = (int64_t)P.fam_idx.size();
    G.work = gwork[gi];
    int maxw = 0, maxslot = 0;
    for (int k = 0; k < K; ++k) maxw = std::max(maxw, R[k]);
    const int r = K - 1;
    for (int i = 0; i < nf; ++i) {
      const CCD& c = *ccds[fams[i]];
      P.fam_node0[fams[i]] = G.node0;
      for (int k = 0; k < K; ++k) {
        P.fam_col[(size_t)fams[i] * K + k] = off[k][i];
        P.fam_ncol[(size_t)fams[i] * K + k] = info[i].ncompat[k];
      }
      P.fam_idx.push_back(fams[i]);
      P.fam_pos.push_back(pos(i, r, c.n_clades - 1));
    }
    for (int k = 0; k < K; ++k) {
      DNode nd;
      nd.width = R[k];
      nd.top_off = P.tops_doubles;
      P.tops_doubles += R[k];
      if (opt.keep_tables) {
        nd.tab_off = P.tab_doubles;
        P.tab_doubles += (int64_t)m.nrow[k] * R[k];
      }
      const int kind = m.kind[k];
      // ---- duplication program (rows 2.., and WGD row 1)
      const bool need_dup = (kind != WG_NODE_ROOT) && (m.nrow[k] > 1 || kind == WG_NODE_WGD);
      if (need_dup) {
        Work w;
        Work tw;
        std::vector<std::vector<Ent>> tby(opt.adjoint ? R[k] : 0);
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, k, g);
            if (pg < 0 || c.nleaves[g] <= 1) continue;
            std::vector<Ent> es;
            for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) {
              const int a = pos(i, k, c.g1[s]), b = pos(i, k, c.g2[s]);
              if (a < 0 || b < 0) throw Error(WG_EPARSE, "split operand incompatible with a compatible parent clade");
              es.push_back({a, b, c.p[s]});
              if (opt.adjoint) {
                tby[a].push_back({pg, b, c.p[s]});
                tby[b].push_back({pg, a, c.p[s]});
              }
            }
            w.emplace_back(pg, std::move(es));
          }
        }
        Fin fin;
        fin.v.assign(R[k], {0, 0});
        int ns = 0;
        nd.dup = schedule(w, P.entries, fin, ns);
        nd.nslot_dup = ns;
        maxslot = std::max(maxslot, ns);
        nd.fin_dup = put_fin(P.meta, fin);
        if (opt.adjoint) {
          for (int x = 0; x < R[k]; ++x) if (!tby[x].empty()) tw.emplace_back(x, std::move(tby[x]));
          Fin tf;
          tf.v.assign(R[k], {0, 0});
          nd.tdup = schedule(tw, P.entries, tf, ns);
          maxslot = std::max(maxslot, ns);
          nd.fin_tdup = put_fin(P.meta, tf);
        }
      }
      if (kind == WG_NODE_LEAF) {
        std::vector<std::array<int, 2>> aux(R[k], {0, 0});
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, k, g);
            if (pg >= 0 && c.nleaves[g] == 1) aux[pg] = {1, 0};
          }
        }
        nd.aux = put_int2(P.meta, aux);
      }
      if (kind == WG_NODE_WGD) {
        if (R[k] != R[m.ch0[k]]) throw Error(WG_EINVAL, "WGD node and its child differ in compatible clades");
      }
      if (kind == WG_NODE_INTERNAL || kind == WG_NODE_ROOT) {
        const int ka = m.ch0[k], kb = m.ch1[k];
        Work w;
        std::vector<std::array<int, 2>> aux(R[k], {-1, -1});
        std::vector<std::vector<Ent>> ta(opt.adjoint ? R[ka] : 0), tb(opt.adjoint ? R[kb] : 0);
        std::vector<int> inva(R[ka], -1), invb(R[kb], -1);
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, k, g);
            if (pg < 0) continue;
            const int la = pos(i, ka, g), lb = pos(i, kb, g);
            aux[pg] = {la, lb};
            if (la >= 0) inva[la] = pg;
            if (lb >= 0) invb[lb] = pg;
            if (c.nleaves[g] <= 1) continue;
            std::vector<Ent> es;
            for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) {
              const int g1 = c.g1[s], g2 = c.g2[s];
              const int a1 = pos(i, ka, g1), b2 = pos(i, kb, g2);
              const int b1 = pos(i, kb, g1), a2 = pos(i, ka, g2);
              if (a1 >= 0 && b2 >= 0) {
                es.push_back({a1, b2, c.p[s]});
                if (opt.adjoint) { ta[a1].push_back({pg, b2, c.p[s]}); tb[b2].push_back({pg, a1, c.p[s]}); }
              }
              if (b1 >= 0 && a2 >= 0) {
                es.push_back({a2, b1, c.p[s]});
                if (opt.adjoint) { ta[a2].push_back({pg, b1, c.p[s]}); tb[b1].push_back({pg, a2, c.p[s]}); }
              }
            }
            if (!es.empty()) w.emplace_back(pg, std::move(es));
          }
        }
        Fin fin;
        fin.v.assign(R[k], {0, 0});
        int ns = 0;
        nd.r1 = schedule(w, P.entries, fin, ns);
        maxslot = std::max(maxslot, ns);
        nd.fin_r1 = put_fin(P.meta, fin);
        nd.aux = put_int2(P.meta, aux);
        if (opt.adjoint) {
          Work wa, wb;
          for (int x = 0; x < R[ka]; ++x) if (!ta[x].empty()) wa.emplace_back(x, std::move(ta[x]));
          for (int x = 0; x < R[kb]; ++x) if (!tb[x].empty()) wb.emplace_back(x, std::move(tb[x]));
          Fin fa, fb;
          fa.v.assign(R[ka], {0, 0});
          fb.v.assign(R[kb], {0, 0});
          nd.tr1a = schedule(wa, P.entries, fa, ns);
          maxslot = std::max(maxslot, ns);
          nd.fin_tr1a = put_fin(P.meta, fa);
          nd.tr1b = schedule(wb, P.entries, fb, ns);
          maxslot = std::max(maxslot, ns);
          nd.fin_tr1b = put_fin(P.meta, fb);
          nd.inv_a = put_int(P.meta, inva);
          nd.inv_b = put_int(P.meta, invb);
        }
      }
      if (kind == WG_NODE_ROOT) {
        int nl = 0;
        for (int i = 0; i < nf; ++i)
          for (int v : lvl[i]) nl = std::max(nl, v + 1);
        std::vector<Work> lw(nl), tlw(nl);
        std::vector<std::vector<int>> lc(nl);
        std::vector<std::vector<Ent>> tby(opt.adjoint ? R[k] : 0);
        std::vector<int> plevel(R[k], 0);
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, k, g);
            plevel[pg] = lvl[i][g];
            lc[lvl[i][g]].push_back(pg);
            if (c.nleaves[g] <= 1) continue;
            std::vector<Ent> es;
            for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) {
              const int a = pos(i, k, c.g1[s]), b = pos(i, k, c.g2[s]);
              es.push_back({a, b, c.p[s]});
              if (opt.adjoint) { tby[a].push_back({pg, b, c.p[s]}); tby[b].push_back({pg, a, c.p[s]}); }
            }
            lw[lvl[i][g]].emplace_back(pg, std::move(es));
          }
        }
        if (opt.adjoint)
          for (int x = 0; x < R[k]; ++x) if (!tby[x].empty()) tlw[plevel[x]].emplace_back(x, std::move(tby[x]));
        Fin fin, tfin;
        fin.v.assign(R[k], {0, 0});
        tfin.v.assign(R[k], {0, 0});
        std::vector<int> lcl;
        nd.nlvl = nl;
        nd.lvl = (int64_t)P.levels.size();
        for (int L = 0; L < nl; ++L) {
          DLevel dl;
          int ns = 0;
          dl.prog = schedule(lw[L], P.entries, fin, ns);
          maxslot = std::max(maxslot, ns);
          dl.begin = (int)lcl.size();
          lcl.insert(lcl.end(), lc[L].begin(), lc[L].end());
          dl.end = (int)lcl.size();
          P.levels.push_back(dl);
        }
        nd.fin_lvl = put_fin(P.meta, fin);
        nd.lvl_clades = put_int(P.meta, lcl);
        if (opt.adjoint) {
          nd.tlvl = (int64_t)P.levels.size();
          for (int L = 0; L < nl; ++L) {
            DLevel dl;
            int ns = 0;
            dl.prog = schedule(tlw[L], P.entries, tfin, ns);
            maxslot = std::max(maxslot, ns);
            dl.begin = P.levels[nd.lvl + L].begin;
            dl.end = P.levels[nd.lvl + L].end;
            P.levels.push_back(dl);
          }
          nd.fin_tlvl = put_fin(P.meta, tfin);
        }
      }
      P.nodes.push_back(nd);
    }
    G.maxw = maxw;
    G.maxslot = maxslot;
    // shared memory: cur, nxt/X, Y, slots (+ adjoint: one more row)
    const int smem = (opt.adjoint ? 5 : 3) * maxw + maxslot + 8;
    max_smem = std::max(max_smem, smem);
    P.groups.push_back(G);
  }
  P.max_smem_doubles = max_smem;
  return P;
}

}  // namespace wg

// ===========================================================================
// Batched layout: level-synchronous (node, family group) tasks
// ===========================================================================
namespace wg {

namespace {

// A task built apart from the others: its programs' entries, int tables
// and level programs with task-local offsets.
using EntryBuf = std::vector<DEntry, UninitAlloc<DEntry>>;

struct TaskBuild {
  DTask T;
  EntryBuf entries;
  std::vector<int32_t> meta;
  std::vector<DProg2> progs;
  std::vector<int> col;  // first row position of each family of the group
  int smem_adj = 0, NT = 0;
};

struct Item {
  int c = 0;                  // output position of the finalize op
  uint32_t fin = op::FIN_DUP;
  int fa = 0xFFFF, fb = 0xFFFF;
};

// Items with their products in CSR form: item i's products are
// ents[off[i] .. off[i + 1]), in the order they were added.
struct ItemList {
  std::vector<Item> items;
  std::vector<int64_t> off{0};
  std::vector<Ent> ents;
  int size() const { return (int)items.size(); }
  int nprod(int i) const { return (int)(off[i + 1] - off[i]); }
  void open(const Item& it) { items.push_back(it); }
  void prod(int a, int b, double p) { ents.push_back({a, b, p}); }
  void close() { off.push_back((int64_t)ents.size()); }
};

// Products addressed to items by index as they arrive (the transposed
// programs of the adjoint); finish() sorts them by item, stably, so each
// item keeps its products in arrival order.
struct ScatterList {
  std::vector<Item> items;
  std::vector<int> to;
  std::vector<Ent> ents;
  explicit ScatterList(int n = 0) : items(n) {}
  void add(int x, int a, int b, double p) {
    to.push_back(x);
    ents.push_back({a, b, p});
  }
  ItemList finish() {
    ItemList L;
    const int n = (int)items.size();
    L.items = std::move(items);
    L.off.assign((size_t)n + 1, 0);
    for (int x : to) ++L.off[(size_t)x + 1];
    for (int i = 0; i < n; ++i) L.off[i + 1] += L.off[i];
    std::vector<int64_t> cur(L.off.begin(), L.off.end() - 1);
    L.ents.resize(ents.size());
    for (size_t j = 0; j < to.size(); ++j) L.ents[cur[to[j]]++] = ents[j];
    std::vector<int>().swap(to);
    std::vector<Ent>().swap(ents);
    return L;
  }
};

inline uint64_t pack_code(uint32_t f0, uint32_t f1, uint32_t f2, uint32_t opc, uint32_t kind = col::NOP) {
  return (uint64_t)(f0 & 0xFFFFu) | ((uint64_t)(f1 & 0xFFFFu) << 16) | ((uint64_t)(f2 & 0xFFFFu) << 32) |
         ((uint64_t)opc << 48) | ((uint64_t)kind << 56);
}

inline double bits_to_double(uint64_t b) {
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

// Lane programs with fused finalize.  An item (one clade) is its products
// followed by its finalize op; items longer than J ops are split into
// segments ending in FIN_PART, finished by a combine entry after a barrier.
// The columns of a warp are uniform (col::): segments go longest first (ties
// in item order) in bundles of 32, one per lane, each bundle as high as its
// longest segment with every segment ending in the bundle's last column
// (shorter ones start later; their lanes idle before); bundles stack in the
// warps first-fit (J ops per lane); J grows until they fit.  Partial slots
// are numbered from slot_base (a program run right after another without a
// barrier takes slots after the other's).
DProg2 schedule2(const ItemList& items, int ntmax, int target_j, EntryBuf& out, int slot_base = 0,
                 int comb_warp = 0) {
  DProg2 pr;
  pr.off = (int64_t)out.size();
  const int n = items.size();
  int64_t W = 0;
  int maxops = 0;
  for (int i = 0; i < n; ++i) {
    W += (int64_t)items.nprod(i) + 1;
    maxops = std::max(maxops, items.nprod(i) + 1);
  }
  if (W == 0) return pr;
  // rows are latency-bound: enough warps to bring a row to ~target_j
  // iterations, no more (idle warps issue nothing, partial ones waste FP64)
  const int best_w = (int)std::min<int64_t>(ntmax / 32, std::max<int64_t>(1, (W + 32 * target_j - 1) / (32 * target_j)));
  int J = (int)((W + 32 * best_w - 1) / (32 * best_w));
  struct Seg { int item, k, begin, len; bool split; };
  std::vector<Seg> segs;
  std::vector<int> order, cnt, bwarp, bcol, load;
  std::vector<int> nseg(n, 1);
  while (true) {
    if (maxops > J && J < 2) J = 2;
    segs.clear();
    for (int i = 0; i < n; ++i) {
      const int np = items.nprod(i);
      if (np + 1 <= J) {
        nseg[i] = 1;
        segs.push_back({i, 0, 0, np, false});
        continue;
      }
      const int per = J - 1;  // products per segment (+ FIN_PART)
      const int ns = (np + per - 1) / per;
      nseg[i] = ns;
      const int base = np / ns, rem = np % ns;
      int b = 0;
      for (int k = 0; k < ns; ++k) {
        const int len = base + (k < rem ? 1 : 0);
        segs.push_back({i, k, b, len, true});
        b += len;
      }
    }
    // longest first, stable: a counting sort (every length is below J)
    cnt.assign((size_t)J + 1, 0);
    for (const Seg& sg : segs) ++cnt[sg.len];
    for (int l = J - 1, acc = 0; l >= 0; --l) {
      const int c = cnt[l];
      cnt[l] = acc;
      acc += c;
    }
    order.resize(segs.size());
    for (int si = 0; si < (int)segs.size(); ++si) order[cnt[segs[si].len]++] = si;
    // bundles of 32 into the warps, first fit (heights do not increase)
    const int nb = (int)((order.size() + 31) / 32);
    bwarp.assign(nb, -1);
    bcol.assign(nb, 0);
    load.assign(best_w, 0);
    bool ok = true;
    for (int q = 0; q < nb && ok; ++q) {
      const int h = segs[order[(size_t)q * 32]].len + 1;
      int w = 0;
      while (w < best_w && load[w] + h > J) ++w;
      if (w == best_w) {
        ok = false;
        break;
      }
      bwarp[q] = w;
      bcol[q] = load[w];
      load[w] += h;
    }
    if (ok) break;
    ++J;
  }
  // partial slots of split items, contiguous per item
  std::vector<int> slot0(n, -1);
  int nslot = 0;
  for (int i = 0; i < n; ++i)
    if (nseg[i] > 1) { slot0[i] = slot_base + nslot; nslot += nseg[i]; }
  if (slot_base + nslot >= 65535) throw Error(WG_ERANGE, "program exceeds 65535 partial slots");
  int used = 0;
  for (int w = 0; w < best_w; ++w) if (load[w] > 0) used = w + 1;
  const int nt = 32 * used;
  pr.J = J;
  pr.nt = nt;
  pr.nslot = nslot;
  // every position is written: idle lanes and columns get NOPs carrying their
  // column's kind
  out.resize(out.size() + (size_t)J * nt);
  DEntry* base = out.data() + pr.off;
  std::vector<uint32_t> kind((size_t)J * used, col::NOP);
  const int nb = (int)bwarp.size();
  for (int q = 0; q < nb; ++q) {
    const int w = bwarp[q], h = segs[order[(size_t)q * 32]].len + 1;
    bool fin = false;
    for (int l = 0; l < 32 && (size_t)q * 32 + l < order.size(); ++l)
      fin |= !segs[order[(size_t)q * 32 + l]].split;
    for (int t = 0; t + 1 < h; ++t) kind[(size_t)(bcol[q] + t) * used + w] = col::PROD;
    kind[(size_t)(bcol[q] + h - 1) * used + w] = fin ? col::FIN : col::PART;
  }
  for (int j = 0; j < J; ++j)
    for (int t = 0; t < nt; ++t)
      base[(size_t)j * nt + t] = DEntry{pack_code(0, 0, 0, op::NOP, kind[(size_t)j * used + t / 32]), 0.0};
  for (int q = 0; q < nb; ++q) {
    const int w = bwarp[q], h = segs[order[(size_t)q * 32]].len + 1;
    const int end = bcol[q] + h - 1;  // the bundle's finalize column
    for (int l = 0; l < 32 && (size_t)q * 32 + l < order.size(); ++l) {
      const Seg& sg = segs[order[(size_t)q * 32 + l]];
      const Item& it = items.items[sg.item];
      const Ent* e = items.ents.data() + items.off[sg.item] + sg.begin;
      const int t = 32 * w + l;
      int j = end - sg.len;
      for (int x = 0; x < sg.len; ++x, ++j)
        base[(size_t)j * nt + t] = DEntry{pack_code(e[x].a, e[x].b, 0, op::PROD, col::PROD), e[x].p};
      const uint32_t k = kind[(size_t)end * used + w];
      if (sg.split)
        base[(size_t)end * nt + t] = DEntry{pack_code(0, 0, slot0[sg.item] + sg.k, op::FIN_PART, k), 0.0};
      else
        base[(size_t)end * nt + t] = DEntry{pack_code(it.c, it.fa, it.fb, it.fin, k), 0.0};
    }
  }
  // every entry fits its column's kind (the kernels take one branch per warp
  // and column; a product in a finalize column would be skipped)
  for (size_t x = 0; x < (size_t)J * nt; ++x) {
    const uint64_t code = base[x].code;
    const uint32_t o = (uint32_t)((code >> 48) & 0xFFu), kd = (uint32_t)(code >> 56);
    const bool fits = o == op::NOP || (kd == col::PROD ? o == op::PROD
                                                        : kd == col::FIN ? o != op::PROD
                                                                         : kd == col::PART && o == op::FIN_PART);
    if (!fits) throw Error(WG_ESTATE, "internal: program entry does not fit its column");
  }
  // combine entries (with comb_warp: largest first, the first nbig, those
  // of at least comb_warp partial sums, combined by a warp each); the rest
  // are combined by a thread each
  pr.comb = (int64_t)out.size();
  std::vector<int> cs;
  for (int i = 0; i < n; ++i)
    if (nseg[i] > 1) cs.push_back(i);
  int nbig = 0;
  if (comb_warp > 0) {
    std::stable_sort(cs.begin(), cs.end(), [&](int x, int y) { return nseg[x] > nseg[y]; });
    while (nbig < (int)cs.size() && nseg[cs[nbig]] >= comb_warp) ++nbig;
  }
  if (nbig > 65535) throw Error(WG_ERANGE, "program exceeds 65535 combine entries");
  pr.nbig = (uint16_t)nbig;
  for (int i : cs) {
    const Item& it = items.items[i];
    const uint64_t sl = (uint64_t)(uint32_t)slot0[i] | ((uint64_t)(uint32_t)nseg[i] << 32);
    out.push_back(DEntry{pack_code(it.c, it.fa, it.fb, it.fin), bits_to_double(sl)});
    ++pr.ncomb;
  }
  return pr;
}

}  // namespace

std::vector<std::vector<int>> compat_columns(const Model& m, const CCD& c) {
  FamInfo fi;
  compat_of(m, c, fi, true);
  return fi.idx;
}

Packed2 pack_batch2(const Model& m, const std::vector<const CCD*>& ccds, const PackOptions2& opt) {
  Packed2 P;
  const int K = m.K;
  const int NF = (int)ccds.size();
  if (NF == 0) throw Error(WG_EINVAL, "empty batch");
  const int NR = m.total_rows();
  // ---- per family: compatibility, levels, cost
  std::vector<FamInfo> info(NF);
  std::vector<std::vector<int>> lvl(NF);
  std::vector<std::array<double, 3>> cost(NF);
  // per family and node: splits of its compatible non-leaf clades plus its
  // compatible clades (the weight tasks are filled by)
  std::vector<std::vector<double>> node_w(NF);
  for (int f = 0; f < NF; ++f)
    if (ccds[f]->n_clades >= 65535) throw Error(WG_ERANGE, "CCD with 65535 or more clades");
  parallel_for(NF, opt.threads, [&](size_t f) {
    const CCD& c = *ccds[f];
    compat_of(m, c, info[f], true);
    double w;
    family_cost(m, c, info[f], cost[f][0], cost[f][1], cost[f][2], w);
    lvl[f] = split_levels(c);
    node_w[f].assign(K, 0.0);
    for (int k = 0; k < K; ++k) {
      const std::vector<int>& ix = info[f].idx[k];
      double T = 0;
      for (int g = 0; g < c.n_clades; ++g)
        if (ix[g] >= 0 && c.nleaves[g] > 1) T += c.split_off[g + 1] - c.split_off[g];
      node_w[f][k] = T + info[f].ncompat[k];
    }
  });
  for (int f = 0; f < NF; ++f) {  // summed in family order
    P.flops_fwd += cost[f][0];
    P.bytes_fwd += cost[f][1];
    P.flops_adj += cost[f][2];
  }
  // per (family, node) location of the top row, filled as tasks are built
  std::vector<int64_t> toploc((size_t)NF * K, -1);
  P.fam_tab.assign((size_t)NF * K, -1);
  P.fam_w.assign((size_t)NF * K, 0);
  P.fam_col.assign((size_t)NF * K, 0);
  P.fam_ncol.assign((size_t)NF * K, 0);
  // height levels of the species tree
  std::vector<int> height(K, 0);
  int H = 0;
  for (int k = 0; k < K; ++k) {
    if (m.ch0[k] >= 0) height[k] = std::max(height[k], height[m.ch0[k]] + 1);
    if (m.ch1[k] >= 0) height[k] = std::max(height[k], height[m.ch1[k]] + 1);
    H = std::max(H, height[k]);
  }
  P.levels.assign(H + 1, {});
  P.levels_h.assign(H + 1, {});
  P.levels_g.assign(H + 1, {});
  P.levels_gh.assign(H + 1, {});
  P.level_smem.assign(H + 1, 0);
  P.level_smem_adj.assign(H + 1, 0);
  P.level_smem_h.assign(H + 1, 0);
  P.level_smem_adj_h.assign(H + 1, 0);
  // gradient reduction contributions
  std::vector<std::vector<int64_t>> red(3 * (size_t)NR + K + 1);
  std::vector<EntryBuf> entry_chunks;
  std::vector<int64_t> entry_off;
  int64_t n_entries = 0;
  auto eps_top_row = [&](int k) { return m.row_off[k] + m.nrow[k] - 1; };

  // every node's families in task groups: compatible families, heaviest
  // first, next-fit
  std::vector<std::vector<std::vector<int>>> groups_of(K);
  std::vector<std::vector<double>> ops_of(K);
  for (int k = 0; k < K; ++k) {
    const int kind = m.kind[k];
    std::vector<std::pair<double, int>> fw;
    for (int f = 0; f < NF; ++f)
      if (info[f].ncompat[k] > 0) fw.emplace_back(node_w[f][k], f);
    std::stable_sort(fw.begin(), fw.end(), [](auto& x, auto& y) { return x.first > y.first; });
    std::vector<std::vector<int>>& groups = groups_of[k];
    std::vector<double>& group_ops = ops_of[k];
    {
      // the root row is a chain of short same-row levels, so a root task
      // takes many more families for the same per-level work
      const bool is_root = kind == WG_NODE_ROOT;
      const double tops_lim = is_root ? (double)opt.target_ops * opt.root_group : (double)opt.target_ops;
      const int64_t wlim = is_root ? opt.max_width_root : opt.max_width;
      // the adjoint keeps six rows of max(width, staged children) plus the
      // partial slots (a margin) and the branch's ϕ, ψ
      const bool bound_smem = is_root && opt.root_smem_doubles > 0;
      const int ka = m.ch0[k], kb = m.ch1[k];
      std::vector<int> cur;
      double ops = 0;
      int64_t width = 0, staged = 0;
      for (auto& [w, f] : fw) {
        const int C = info[f].ncompat[k];
        const int S = (ka >= 0 ? info[f].ncompat[ka] : 0) + (kb >= 0 ? info[f].ncompat[kb] : 0);
        const bool over_smem =
            bound_smem && 6 * std::max(width + C, staged + S) + 2 * m.nrow[k] + 1024 > opt.root_smem_doubles;
        if (!cur.empty() && (ops + w > tops_lim || width + C > wlim || over_smem)) {
          groups.push_back(cur);
          group_ops.push_back(ops);
          cur.clear();
          ops = 0;
          width = 0;
          staged = 0;
        }
        cur.push_back(f);
        ops += w;
        width += C;
        staged += S;
      }
      if (!cur.empty()) { groups.push_back(cur); group_ops.push_back(ops); }
    }
  }
  // one task per group, all nodes' tasks built in one parallel pass (largest
  // first) into task-local buffers; merged after, in node and group order
  // (global offsets and the staging maps of the children's tops set there)
  auto build = [&](int k, size_t gi, TaskBuild& tb) {
      const int kind = m.kind[k];
      const int ka = m.ch0[k], kb = m.ch1[k];
      const auto& fams = groups_of[k][gi];
      DTask& T = tb.T;
      EntryBuf& entries = tb.entries;
      std::vector<int32_t>& meta = tb.meta;
      const int nf = (int)fams.size();
      T.node = k;
      T.nfam = nf;
      const double gops = ops_of[k][gi];
      std::vector<int> col(nf + 1, 0), cola(nf + 1, 0), colb(nf + 1, 0);
      for (int i = 0; i < nf; ++i) {
        col[i + 1] = col[i] + info[fams[i]].ncompat[k];
        if (ka >= 0) cola[i + 1] = cola[i] + info[fams[i]].ncompat[ka];
        if (kb >= 0) colb[i + 1] = colb[i] + info[fams[i]].ncompat[kb];
      }
      // the root row is a chain of small same-row levels: latency-bound, so
      // root tasks stay in narrow CTAs that pack densely on the SMs; rows too
      // wide for shared memory take the wide CTAs
      const int64_t W2est = std::max<int64_t>(col[nf], (int64_t)cola[nf] + colb[nf]);
      const bool wide = (opt.adjoint ? 6 : 2) * W2est + 2 * m.nrow[k] > opt.smem_limit_doubles;
      const int NT = (!opt.light_only && kind != WG_NODE_ROOT && (gops > opt.heavy_ops || wide)) ? kNT2H : kNT2L;
      T.nt = NT;
      const int R = col[nf];
      if (R >= 32768) throw Error(WG_ERANGE, "task row wider than 32767 clades");
      T.width = R;
      T.wa = cola[nf];
      T.wb = colb[nf];
      auto pos = [&](int i, int g) { const int j = info[fams[i]].idx[k][g]; return j < 0 ? -1 : col[i] + j; };
      auto posa = [&](int i, int g) { const int j = info[fams[i]].idx[ka][g]; return j < 0 ? -1 : cola[i] + j; };
      auto posb = [&](int i, int g) { const int j = info[fams[i]].idx[kb][g]; return j < 0 ? -1 : colb[i] + j; };
      tb.col = col;
      // ---- forward programs
      const bool has_rows = kind != WG_NODE_ROOT && m.nrow[k] > 1;
      if (has_rows || (opt.adjoint && kind == WG_NODE_WGD)) {
        ItemList items;
        ScatterList titems(opt.adjoint ? R : 0);
        // row programs read both operand fields of every entry: finalize
        // entries carry their own clade in f0 and f1
        for (int x = 0; x < (int)titems.items.size(); ++x) titems.items[x] = {x, op::FIN_ADJ, x, x};
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, g);
            if (pg < 0) continue;
            items.open({pg, op::FIN_DUP, pg, pg});
            if (c.nleaves[g] > 1)
              for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) {
                const int a = pos(i, c.g1[s]), b = pos(i, c.g2[s]);
                if (a < 0 || b < 0) throw Error(WG_EPARSE, "split operand incompatible with a compatible clade");
                items.prod(a, b, c.p[s]);
                if (opt.adjoint) {
                  titems.add(a, pg, b, c.p[s]);
                  titems.add(b, pg, a, c.p[s]);
                }
              }
            items.close();
          }
        }
        if (has_rows) T.dup = schedule2(items, NT, opt.target_j, entries, 0, opt.comb_warp);
        if (opt.adjoint) T.tdup = schedule2(titems.finish(), NT, opt.target_j, entries);
      }
      if (kind == WG_NODE_LEAF) {
        std::vector<int> aux(R, 0);
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, g);
            if (pg >= 0 && c.nleaves[g] == 1) aux[pg] = 1;
          }
        }
        T.aux = put_int(meta, aux);
      } else if (kind == WG_NODE_WGD) {
        if (T.wa != R) throw Error(WG_EINVAL, "WGD node and its child differ in compatible clades");
        ItemList items;
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, g);
            if (pg < 0) continue;
            items.open({pg, op::FIN_WGD, posa(i, g), 0xFFFF});
            if (c.nleaves[g] > 1)
              for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s)
                items.prod(posa(i, c.g1[s]), posa(i, c.g2[s]), c.p[s]);
            items.close();
          }
        }
        T.init = schedule2(items, NT, opt.target_j, entries, 0, opt.comb_warp);
      } else {
        // speciation + loss (internal) or Πspec + Πloss of the root row
        ItemList items;
        std::vector<std::array<int, 2>> loss(R, {-1, -1});
        std::vector<int> inva(T.wa, -1), invb(T.wb, -1);
        ScatterList ta(opt.adjoint ? T.wa : 0), tb(opt.adjoint ? T.wb : 0);
        for (int x = 0; x < (int)ta.items.size(); ++x) ta.items[x] = {x, op::FIN_TOP, 0xFFFF, 0xFFFF};
        for (int x = 0; x < (int)tb.items.size(); ++x) tb.items[x] = {x, op::FIN_TOP, 0xFFFF, 0xFFFF};
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, g);
            if (pg < 0) continue;
            const int la = posa(i, g), lb = posb(i, g);
            loss[pg] = {la, lb};
            if (la >= 0) inva[la] = pg;
            if (lb >= 0) invb[lb] = pg;
            items.open({pg, op::FIN_SPEC, la < 0 ? 0xFFFF : la, lb < 0 ? 0xFFFF : lb});
            if (c.nleaves[g] > 1)
              for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) {
                const int g1 = c.g1[s], g2 = c.g2[s];
                const int a1 = posa(i, g1), b2 = posb(i, g2), b1 = posb(i, g1), a2 = posa(i, g2);
                if (a1 >= 0 && b2 >= 0) {
                  items.prod(a1, b2, c.p[s]);
                  if (opt.adjoint) { ta.add(a1, pg, b2, c.p[s]); tb.add(b2, pg, a1, c.p[s]); }
                }
                if (b1 >= 0 && a2 >= 0) {
                  items.prod(a2, b1, c.p[s]);
                  if (opt.adjoint) { ta.add(a2, pg, b1, c.p[s]); tb.add(b1, pg, a2, c.p[s]); }
                }
              }
            items.close();
          }
        }
        T.init = schedule2(items, NT, opt.target_j, entries, 0, opt.comb_warp);
        T.loss = put_int2(meta, loss);
        if (opt.adjoint) {
          for (int x = 0; x < T.wa; ++x) ta.items[x].fa = inva[x] < 0 ? 0xFFFF : inva[x];
          for (int x = 0; x < T.wb; ++x) tb.items[x].fa = invb[x] < 0 ? 0xFFFF : invb[x];
          T.ta = schedule2(ta.finish(), NT, opt.target_j, entries);
          // the adjoint runs tb straight after ta: disjoint partial slots
          T.tb = schedule2(tb.finish(), NT, opt.target_j, entries, T.ta.nslot);
          T.inva = put_int(meta, inva);
          T.invb = put_int(meta, invb);
        }
      }
      if (kind == WG_NODE_ROOT) {
        // Πroot (same-row recursion over split levels): the levels of all the
        // task's families in lock step, one program per level for the CTA
        int nl = 0;
        for (int i = 0; i < nf; ++i)
          for (int v : lvl[fams[i]]) nl = std::max(nl, v + 1);
        std::vector<ItemList> lw(nl), tlw(nl);
        std::vector<int> plevel(R, 0);
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) plevel[pos(i, g)] = lvl[fams[i]][g];
        }
        ScatterList tby(opt.adjoint ? R : 0);
        for (int x = 0; x < (int)tby.items.size(); ++x) tby.items[x] = {x, op::FIN_TLVL, x, x};
        for (int i = 0; i < nf; ++i) {
          const CCD& c = *ccds[fams[i]];
          for (int g = 0; g < c.n_clades; ++g) {
            const int pg = pos(i, g);
            ItemList& L = lw[plevel[pg]];
            L.open({pg, op::FIN_LVL, pg, pg});
            if (c.nleaves[g] > 1)
              for (int s = c.split_off[g]; s < c.split_off[g + 1]; ++s) {
                const int a = pos(i, c.g1[s]), b = pos(i, c.g2[s]);
                L.prod(a, b, c.p[s]);
                if (opt.adjoint) { tby.add(a, pg, b, c.p[s]); tby.add(b, pg, a, c.p[s]); }
              }
            L.close();
          }
        }
        if (opt.adjoint) {
          const ItemList t = tby.finish();
          for (int x = 0; x < R; ++x) {
            ItemList& L = tlw[plevel[x]];
            L.open(t.items[x]);
            L.ents.insert(L.ents.end(), t.ents.begin() + t.off[x], t.ents.begin() + t.off[x + 1]);
            L.close();
          }
        }
        T.nlvl = nl;
        T.lvl = (int64_t)tb.progs.size();
        for (int L = 0; L < nl; ++L)
          tb.progs.push_back(schedule2(lw[L], NT, opt.level_j, entries, 0, opt.comb_warp));
        if (opt.adjoint) {
          T.tlvl = (int64_t)tb.progs.size();
          for (int L = 0; L < nl; ++L) tb.progs.push_back(schedule2(tlw[L], NT, opt.level_j, entries));
        }
        for (const DProg2& q : tb.progs) T.rslot = std::max(T.rslot, (int32_t)q.nslot);
      }
      if (kind == WG_NODE_ROOT) {
        // log L outputs: family index and position of its ubiquitous clade
        std::vector<std::array<int, 2>> fam(nf);
        for (int i = 0; i < nf; ++i)
          fam[i] = {opt.global_ids ? (*opt.global_ids)[fams[i]] : fams[i], pos(i, ccds[fams[i]]->n_clades - 1)};
        T.fam = put_int2(meta, fam);
      }
      // shared memory: cur + nxt rows (children staged in nxt) + slots + spare
      int slots = std::max({(int)T.dup.nslot, (int)T.init.nslot, (int)T.tdup.nslot, T.ta.nslot + T.tb.nslot});
      slots = std::max(slots, T.rslot);  // root: the level programs' partial slots
      // forward: cur, nxt (children staged in nxt); adjoint: bar, barn, two
      // L rows, G; then partial slots and reduction scratch
      // row buffers of an even number of doubles (16-byte aligned rows)
      const int W2r = std::max(R, T.wa + T.wb);
      const int W2 = W2r + (W2r & 1);
      T.nslot_max = slots;
      // + the branch's ϕ and ψ rows staged in shared memory
      T.smem = 2 * W2 + slots + 2 * m.nrow[k] + 16 * (NT / 32) + 32;
      const int smem_adj = 6 * W2 + slots + 2 * m.nrow[k] + 16 * (NT / 32) + 32;
      tb.smem_adj = smem_adj;
      tb.NT = NT;
  };
  std::vector<std::vector<TaskBuild>> builds(K);
  std::vector<std::vector<std::exception_ptr>> errs(K);
  std::vector<std::pair<int, int>> jobs;
  for (int k = 0; k < K; ++k) {
    builds[k].resize(groups_of[k].size());
    errs[k].resize(groups_of[k].size());
    for (int gi = 0; gi < (int)groups_of[k].size(); ++gi) jobs.emplace_back(k, gi);
  }
  std::stable_sort(jobs.begin(), jobs.end(),
                   [&](auto& x, auto& y) { return ops_of[x.first][x.second] > ops_of[y.first][y.second]; });
  parallel_for(jobs.size(), opt.threads, [&](size_t j) {
    const auto [k, gi] = jobs[j];
    try {
      build(k, gi, builds[k][gi]);
    } catch (...) {
      errs[k][gi] = std::current_exception();
    }
  });
  for (auto& ek : errs)  // the first failing task in node and group order
    for (auto& e : ek)
      if (e) std::rethrow_exception(e);
  for (int k = 0; k < K; ++k) {
    const int kind = m.kind[k];
    const int ka = m.ch0[k], kb = m.ch1[k];
    for (size_t gi = 0; gi < groups_of[k].size(); ++gi) {
      TaskBuild& tb = builds[k][gi];
      DTask T = tb.T;
      const auto& fams = groups_of[k][gi];
      const int nf = (int)fams.size();
      const int R = T.width, NT = tb.NT, smem_adj = tb.smem_adj;
      T.top = P.tops_doubles;
      P.tops_doubles += R;
      // table rows of an even number of doubles: every row starts on a
      // 16-byte boundary (bulk copies into shared memory)
      T.tstride = R + (R & 1);
      if (opt.keep_tables) {
        T.tab = P.tab_doubles;
        P.tab_doubles += (int64_t)m.nrow[k] * T.tstride;
      }
      for (int i = 0; i < nf; ++i) {
        const size_t fk = (size_t)fams[i] * K + k;
        toploc[fk] = T.top + tb.col[i];
        P.fam_tab[fk] = T.tab;
        P.fam_w[fk] = T.tstride;
        P.fam_col[fk] = tb.col[i];
        P.fam_ncol[fk] = info[fams[i]].ncompat[k];
      }
      // staging maps of the children's top rows (final: their nodes came first)
      T.gmap = (int64_t)P.gmap.size();
      for (int ch : {ka, kb}) {
        if (ch < 0) continue;
        for (int i = 0; i < nf; ++i) {
          const int C = info[fams[i]].ncompat[ch];
          const int64_t src = toploc[(size_t)fams[i] * K + ch];
          for (int j = 0; j < C; ++j) P.gmap.push_back(src + j);
        }
      }
      // entries, level programs and int tables: task-local offsets made global
      // (entries are copied once, in parallel, after the last node)
      const int64_t eb = n_entries;
      n_entries += (int64_t)tb.entries.size();
      entry_chunks.push_back(std::move(tb.entries));
      entry_off.push_back(eb);
      for (DProg2* pr : {&T.dup, &T.init, &T.tdup, &T.ta, &T.tb}) pr->off += eb, pr->comb += eb;
      const int64_t pb = (int64_t)P.progs.size();
      for (DProg2 pr : tb.progs) {
        pr.off += eb;
        pr.comb += eb;
        P.progs.push_back(pr);
      }
      T.lvl += pb;
      T.tlvl += pb;
      if (P.meta.size() & 1) P.meta.push_back(0);  // int2 tables stay 8-byte aligned
      const int64_t mb = (int64_t)P.meta.size();
      P.meta.insert(P.meta.end(), tb.meta.begin(), tb.meta.end());
      T.aux += mb;
      T.inva += mb;
      T.invb += mb;
      T.loss += mb / 2;
      T.fam += mb / 2;
      std::vector<int32_t>().swap(tb.meta);
      if (opt.adjoint) {
        T.gout = P.gout_doubles;
        const int n = m.nrow[k];
        P.gout_doubles += 2 * (int64_t)n + 5;
        for (int r = 1; r < n && kind != WG_NODE_ROOT; ++r) {
          red[NR + m.row_off[k] + r].push_back(T.gout + 2 * r);
          red[2 * (size_t)NR + m.row_off[k] + r].push_back(T.gout + 2 * r + 1);
        }
        // row 0's slot: E_0 of the one-dot form of the row adjoints
        if (n > 1 && kind != WG_NODE_ROOT) red[NR + m.row_off[k]].push_back(T.gout);
        if (ka >= 0) red[eps_top_row(ka)].push_back(T.gout + 2 * n + 0);
        if (kb >= 0) red[eps_top_row(kb)].push_back(T.gout + 2 * n + 1);
        if (kind == WG_NODE_WGD) red[3 * (size_t)NR + k].push_back(T.gout + 2 * n + 2);
        if (kind == WG_NODE_ROOT) {
          red[3 * (size_t)NR + K].push_back(T.gout + 2 * n + 3);
          red[eps_top_row(k)].push_back(T.gout + 2 * n + 4);
        }
      }
      const int h = height[k];
      const bool heavy = NT == kNT2H;
      T.smem_adj = opt.adjoint ? smem_adj : 0;
      if (std::max(T.smem, T.smem_adj) > opt.smem_limit_doubles) {
        // working rows in device memory, one region per task
        T.scratch = P.scratch_doubles;
        P.scratch_doubles += std::max(T.smem, T.smem_adj);
        (heavy ? P.levels_gh : P.levels_g)[h].push_back((int32_t)P.tasks.size());
        P.tasks.push_back(T);
        continue;
      }
      (heavy ? P.levels_h : P.levels)[h].push_back((int32_t)P.tasks.size());
      int& sf = (heavy ? P.level_smem_h : P.level_smem)[h];
      sf = std::max(sf, T.smem);
      P.max_smem = std::max(P.max_smem, T.smem);
      if (opt.adjoint) {
        int& sa = (heavy ? P.level_smem_adj_h : P.level_smem_adj)[h];
        sa = std::max(sa, smem_adj);
        P.max_smem = std::max(P.max_smem, smem_adj);
      }
      P.tasks.push_back(T);
    }
    std::vector<TaskBuild>().swap(builds[k]);
  }
  P.entries.resize((size_t)n_entries);
  parallel_for(entry_chunks.size(), opt.threads, [&](size_t i) {
    EntryBuf& c = entry_chunks[i];
    if (!c.empty()) std::memcpy(P.entries.data() + entry_off[i], c.data(), c.size() * sizeof(DEntry));
    EntryBuf().swap(c);
  });
  // heaviest tasks first inside each launch (a root task's same-row levels
  // run one after another, each about as long as a row of six entries)
  auto task_cost = [&](const DTask& x) {
    return (int64_t)(x.dup.J + x.tdup.J) * m.nrow[x.node] + x.init.J + 6 * (int64_t)x.nlvl;
  };
  auto by_cost = [&](int a, int b) { return task_cost(P.tasks[a]) > task_cost(P.tasks[b]); };
  for (auto& L : P.levels) std::stable_sort(L.begin(), L.end(), by_cost);
  for (auto& L : P.levels_h) std::stable_sort(L.begin(), L.end(), by_cost);
  for (auto& L : P.levels_g) std::stable_sort(L.begin(), L.end(), by_cost);
  for (auto& L : P.levels_gh) std::stable_sort(L.begin(), L.end(), by_cost);
  P.red_off.assign(red.size() + 1, 0);
  for (size_t j = 0; j < red.size(); ++j) {
    P.red_off[j + 1] = P.red_off[j] + (int64_t)red[j].size();
    P.red_idx.insert(P.red_idx.end(), red[j].begin(), red[j].end());
  }
  return P;
}

Schedule persistent_schedule(const Packed2& P) {
  Schedule S;
  const size_t H = P.levels.size();
  for (size_t h = 0; h < H; ++h)
    for (const auto* lv : {&P.levels[h], &P.levels_h[h], &P.levels_g[h], &P.levels_gh[h]})
      S.order_fwd.insert(S.order_fwd.end(), lv->begin(), lv->end());
  for (size_t h = H; h-- > 0;)
    for (const auto* lv : {&P.levels[h], &P.levels_h[h], &P.levels_g[h], &P.levels_gh[h]})
      S.order_adj.insert(S.order_adj.end(), lv->begin(), lv->end());
  const int n = (int)P.tasks.size();
  if ((int)S.order_fwd.size() != n) throw Error(WG_ESTATE, "internal: a task is in no level");
  // the task owning each top-row offset
  std::vector<std::pair<int64_t, int>> tops(n);
  for (int t = 0; t < n; ++t) tops[t] = {P.tasks[t].top, t};
  std::sort(tops.begin(), tops.end());
  auto producer = [&](int64_t off) {
    auto it = std::upper_bound(tops.begin(), tops.end(), std::make_pair(off, std::numeric_limits<int>::max()));
    if (it == tops.begin()) throw Error(WG_ESTATE, "internal: staged offset before every top row");
    const int t = std::prev(it)->second;
    if (off >= P.tasks[t].top + P.tasks[t].width) throw Error(WG_ESTATE, "internal: staged offset in no top row");
    return t;
  };
  std::vector<std::vector<int>> fdep(n), adep(n);
  parallel_for((size_t)n, default_host_threads(), [&](size_t t) {
    const DTask& T = P.tasks[t];
    const int64_t ms = (int64_t)T.wa + T.wb;
    int last = -1;
    for (int64_t i = 0; i < ms; ++i) {
      const int p = producer(P.gmap[T.gmap + i]);
      if (p != last) fdep[t].push_back(p);
      last = p;
    }
    std::sort(fdep[t].begin(), fdep[t].end());
    fdep[t].erase(std::unique(fdep[t].begin(), fdep[t].end()), fdep[t].end());
  });
  for (int t = 0; t < n; ++t)
    for (int p : fdep[t]) adep[p].push_back(t);
  auto csr = [&](const std::vector<std::vector<int>>& d, std::vector<int32_t>& off, std::vector<int32_t>& idx) {
    off.assign(n + 1, 0);
    for (int t = 0; t < n; ++t) off[t + 1] = off[t] + (int32_t)d[t].size();
    idx.reserve(off[n]);
    for (int t = 0; t < n; ++t) idx.insert(idx.end(), d[t].begin(), d[t].end());
  };
  csr(fdep, S.fdep_off, S.fdep_idx);
  csr(adep, S.adep_off, S.adep_idx);
  // every wait targets an earlier ticket of its pass (no wait can block the
  // ticket it waits for)
  std::vector<int> pos_f(n), pos_a(n);
  for (int i = 0; i < n; ++i) pos_f[S.order_fwd[i]] = i, pos_a[S.order_adj[i]] = i;
  for (int t = 0; t < n; ++t) {
    for (int p : fdep[t])
      if (pos_f[p] >= pos_f[t]) throw Error(WG_ESTATE, "internal: forward order is not topological");
    for (int c : adep[t])
      if (pos_a[c] >= pos_a[t]) throw Error(WG_ESTATE, "internal: adjoint order is not topological");
  }
  return S;
}

// Checkpointed tables: the adjoint recomputes each height level's tables from
// the children's top rows (kept in the tops buffer for the whole evaluation,
// one row per species branch and family) just before it walks that level, so
// only one level's tables exist at a time.  Every level's tasks take table
// offsets from 0; the region is the largest level's.  Family table offsets
// are dropped: no family's tables outlive its level.
int64_t checkpoint_tables(Packed2& P, const Model& m) {
  int64_t need = 0;
  for (size_t h = 0; h < P.levels.size(); ++h) {
    int64_t off = 0;
    for (const auto* lv : {&P.levels[h], &P.levels_h[h], &P.levels_g[h], &P.levels_gh[h]})
      for (int t : *lv) {
        DTask& T = P.tasks[t];
        T.tab = off;
        off += (int64_t)m.nrow[T.node] * T.tstride;
      }
    need = std::max(need, off);
  }
  std::fill(P.fam_tab.begin(), P.fam_tab.end(), (int64_t)-1);
  P.tab_doubles = need;
  return need;
}

}  // namespace wg
