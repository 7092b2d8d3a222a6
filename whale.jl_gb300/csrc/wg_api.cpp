// C ABI, host-only parts: error reporting, species-tree model, CCD handles.
// The CUDA-dependent entry points (context, batch, likelihood) live in
// wg_kernels.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

#include "wg_internal.h"

namespace wg {

static thread_local std::string t_last_error;

void set_last_error(const std::string& msg) { t_last_error = msg; }

}  // namespace wg

extern "C" {

const char* wg_last_error(void) { return wg::t_last_error.c_str(); }

int wg_version(void) { return 1; }

int wg_model_create(int32_t n_nodes, const int32_t* kind, const int32_t* child0, const int32_t* child1,
                    const int32_t* nrow, const double* slice_len, const double* leaf_p,
                    const int32_t* clade_offsets, const int32_t* clade_species, int32_t condition,
                    wg_model** out) {
  WG_GUARD({
    if (!out || n_nodes < 3 || !kind || !child0 || !child1 || !nrow || !slice_len || !leaf_p || !clade_offsets ||
        !clade_species)
      throw wg::Error(WG_EINVAL, "wg_model_create: bad arguments");
    if (condition < WG_COND_NONE || condition > WG_COND_NOWHERE)
      throw wg::Error(WG_EINVAL, "wg_model_create: unknown condition");
    auto* m = new wg_model();
    m->K = n_nodes;
    m->kind.assign(kind, kind + n_nodes);
    m->ch0.assign(child0, child0 + n_nodes);
    m->ch1.assign(child1, child1 + n_nodes);
    m->nrow.assign(nrow, nrow + n_nodes);
    m->slice_len.assign(slice_len, slice_len + n_nodes);
    m->leaf_p.assign(leaf_p, leaf_p + n_nodes);
    m->cond = condition;
    m->row_off.assign(n_nodes + 1, 0);
    int maxsp = 0;
    for (int k = 0; k < n_nodes; ++k) {
      if (m->nrow[k] < 1) { delete m; throw wg::Error(WG_EINVAL, "nrow must be >= 1"); }
      m->row_off[k + 1] = m->row_off[k] + m->nrow[k];
      for (int s = clade_offsets[k]; s < clade_offsets[k + 1]; ++s) maxsp = std::max(maxsp, clade_species[s]);
      const int kd = m->kind[k];
      const bool ok = (kd == WG_NODE_LEAF && child0[k] < 0) ||
                      (kd == WG_NODE_WGD && child0[k] >= 0 && child0[k] < k) ||
                      ((kd == WG_NODE_INTERNAL || kd == WG_NODE_ROOT) && child0[k] >= 0 && child0[k] < k &&
                       child1[k] >= 0 && child1[k] < k);
      if (!ok) { delete m; throw wg::Error(WG_EINVAL, "node kinds/children not in reference order"); }
    }
    if (m->kind[n_nodes - 1] != WG_NODE_ROOT) { delete m; throw wg::Error(WG_EINVAL, "the root must be the last node"); }
    m->n_words = maxsp / 64 + 1;
    m->clade_bits.assign((size_t)n_nodes * m->n_words, 0);
    for (int k = 0; k < n_nodes; ++k)
      for (int s = clade_offsets[k]; s < clade_offsets[k + 1]; ++s) {
        const int id = clade_species[s];
        if (id < 0) { delete m; throw wg::Error(WG_EINVAL, "negative species id"); }
        m->clade_bits[(size_t)k * m->n_words + (id >> 6)] |= 1ull << (id & 63);
      }
    *out = m;
  });
}

int wg_model_destroy(wg_model* m) {
  delete m;
  return WG_OK;
}

int wg_model_set_rates(wg_model* m, const double* lam, const double* mu, const double* q, double eta,
                       const double* p) {
  WG_GUARD({
    if (!m || !lam || !mu) throw wg::Error(WG_EINVAL, "wg_model_set_rates: bad arguments");
    const int K = m->K;
    m->lam.assign(lam, lam + K);
    m->mu.assign(mu, mu + K);
    m->q.assign(K, NAN);
    if (q) m->q.assign(q, q + K);
    m->p.assign(K, 0.0);
    if (p) m->p.assign(p, p + K);
    for (int k = 0; k < K; ++k) {
      if (m->kind[k] == WG_NODE_WGD && !(m->q[k] >= 0.0 && m->q[k] <= 1.0))
        throw wg::Error(WG_EINVAL, "WGD retention rate q must lie in [0, 1]");
      if (m->kind[k] != WG_NODE_ROOT && m->nrow[k] > 1 && !(m->lam[k] >= 0.0 && m->mu[k] > 0.0))
        throw wg::Error(WG_EINVAL, "branch rates must be finite with lambda >= 0 and mu > 0");
    }
    if (!(eta > 0.0 && eta <= 1.0)) throw wg::Error(WG_EINVAL, "eta must lie in (0, 1]");
    m->eta = eta;
    wg::model_fill_tables(*m);
    m->has_params = true;
    m->from_rates = true;
    ++m->version;
  });
}

int wg_model_set_tables(wg_model* m, const double* eps, const double* phi, const double* psi, const double* q,
                        double eta) {
  WG_GUARD({
    if (!m || !eps || !phi || !psi) throw wg::Error(WG_EINVAL, "wg_model_set_tables: bad arguments");
    const int n = m->total_rows();
    m->eps.assign(eps, eps + n);
    m->phi.assign(phi, phi + n);
    m->psi.assign(psi, psi + n);
    m->q.assign(m->K, NAN);
    if (q) m->q.assign(q, q + m->K);
    m->eta = eta;
    m->has_params = true;
    m->from_rates = false;
    ++m->version;
  });
}

int wg_model_get_tables(const wg_model* m, double* eps, double* phi, double* psi) {
  WG_GUARD({
    if (!m || !m->has_params) throw wg::Error(WG_ESTATE, "model parameters not set");
    const size_t n = (size_t)m->total_rows();
    if (eps) std::memcpy(eps, m->eps.data(), n * sizeof(double));
    if (phi) std::memcpy(phi, m->phi.data(), n * sizeof(double));
    if (psi) std::memcpy(psi, m->psi.data(), n * sizeof(double));
  });
}

int wg_model_condition(const wg_model* m, double* out) {
  WG_GUARD({
    if (!m || !out) throw wg::Error(WG_EINVAL, "bad arguments");
    if (!m->has_params) throw wg::Error(WG_ESTATE, "model parameters not set");
    *out = wg::model_condition(*m);
  });
}

int wg_backtrack_tables(const wg_model* m, const wg_ccd* c, const double* tables, int64_t n_tables, int32_t n_samples,
                        uint64_t seed, char* out, int64_t cap, int64_t* needed) {
  WG_GUARD({
    if (!m || !c || !tables || n_samples < 0) throw wg::Error(WG_EINVAL, "wg_backtrack_tables: bad arguments");
    if (!m->has_params) throw wg::Error(WG_ESTATE, "model parameters not set");
    const auto cols = wg::compat_columns(*m, *c);
    int64_t need = 0;
    for (int k = 0; k < m->K; ++k) {
      int nc = 0;
      for (int x : cols[k]) nc += x >= 0;
      need += (int64_t)m->nrow[k] * nc;
    }
    if (n_tables != need) throw wg::Error(WG_EINVAL, "tables do not match the family's layout");
    const std::string text = wg::backtrack_family(*m, *c, tables, n_samples, seed);
    if (needed) *needed = (int64_t)text.size() + 1;
    if (!out) return WG_OK;
    if (cap < (int64_t)text.size() + 1) throw wg::Error(WG_ERANGE, "output buffer too small");
    std::memcpy(out, text.c_str(), text.size() + 1);
  });
}

int wg_tree_newick(const wg_model* m, const wg_ccd* c, const int32_t* nodes, int32_t n_nodes, char* out, int64_t cap,
                   int64_t* needed) {
  WG_GUARD({
    if (!m || !c || !nodes) throw wg::Error(WG_EINVAL, "wg_tree_newick: bad arguments");
    const std::string text = wg::tree_newick(*m, *c, nodes, n_nodes);
    if (needed) *needed = (int64_t)text.size() + 1;
    if (!out) return WG_OK;
    if (cap < (int64_t)text.size() + 1) throw wg::Error(WG_ERANGE, "output buffer too small");
    std::memcpy(out, text.c_str(), text.size() + 1);
  });
}

int wg_ccd_parse_ale(const char* text, size_t len, const char* const* species_names, const int32_t* species_ids,
                     int32_t n_species, wg_ccd** out) {
  WG_GUARD({
    if (!text || !out || (n_species > 0 && (!species_names || !species_ids)))
      throw wg::Error(WG_EINVAL, "wg_ccd_parse_ale: bad arguments");
    std::vector<std::string> names;
    std::vector<int> ids;
    for (int i = 0; i < n_species; ++i) { names.emplace_back(species_names[i]); ids.push_back(species_ids[i]); }
    wg::CCD* c = wg::parse_ale(text, len, names, ids);
    auto* h = new wg_ccd();
    static_cast<wg::CCD&>(*h) = std::move(*c);
    delete c;
    *out = h;
  });
}

int wg_ccd_read_ale_files(const char* const* paths, int32_t n_files, const char* const* species_names,
                          const int32_t* species_ids, int32_t n_species, int32_t threads, wg_ccd** out,
                          int32_t* failed) {
  WG_GUARD({
    if (!paths || n_files < 0 || !out || (n_species > 0 && (!species_names || !species_ids)))
      throw wg::Error(WG_EINVAL, "wg_ccd_read_ale_files: bad arguments");
    if (failed) *failed = -1;
    std::vector<std::string> names;
    std::vector<int> ids;
    for (int i = 0; i < n_species; ++i) { names.emplace_back(species_names[i]); ids.push_back(species_ids[i]); }
    std::vector<wg_ccd*> res((size_t)n_files, nullptr);
    std::mutex mu;
    int64_t bad = n_files;
    int code = WG_OK;
    std::string msg;
    wg::parallel_for((size_t)n_files, threads, [&](size_t i) {
      try {
        std::string text;
        {
          FILE* f = paths[i] ? std::fopen(paths[i], "rb") : nullptr;
          if (!f) throw wg::Error(WG_EINVAL, "cannot open file");
          char buf[1 << 16];
          for (size_t r; (r = std::fread(buf, 1, sizeof buf, f)) > 0;) text.append(buf, r);
          const bool err = std::ferror(f) != 0;
          std::fclose(f);
          if (err) throw wg::Error(WG_EINVAL, "read error");
        }
        std::unique_ptr<wg::CCD> c(wg::parse_ale(text.data(), text.size(), names, ids));
        auto* h = new wg_ccd();
        static_cast<wg::CCD&>(*h) = std::move(*c);
        res[i] = h;
      } catch (const std::exception& e) {
        const wg::Error* we = dynamic_cast<const wg::Error*>(&e);
        std::lock_guard<std::mutex> lk(mu);
        if ((int64_t)i < bad) {
          bad = (int64_t)i;
          code = we ? we->code : WG_EINVAL;
          msg = std::string(paths[i] ? paths[i] : "(null)") + ": " + e.what();
        }
      }
    });
    if (bad < n_files) {
      for (wg_ccd* h : res) delete h;
      if (failed) *failed = (int32_t)bad;
      throw wg::Error(code, msg);
    }
    std::copy(res.begin(), res.end(), out);
  });
}

int wg_ccd_create(int32_t n_clades, const int32_t* nleaves, const int32_t* species_offsets, const int32_t* species,
                  const int32_t* split_offsets, const int32_t* split_g1, const int32_t* split_g2,
                  const double* split_p, int64_t observations, wg_ccd** out) {
  WG_GUARD({
    if (!out || n_clades < 3 || !nleaves || !species_offsets || !species || !split_offsets || !split_g1 ||
        !split_g2 || !split_p)
      throw wg::Error(WG_EINVAL, "wg_ccd_create: bad arguments");
    auto* c = new wg_ccd();
    c->n_clades = n_clades;
    c->observations = observations;
    c->nleaves.assign(nleaves, nleaves + n_clades);
    c->counts.assign(n_clades, 0);
    c->sp_off.assign(species_offsets, species_offsets + n_clades + 1);
    c->sp.assign(species, species + species_offsets[n_clades]);
    c->split_off.assign(split_offsets, split_offsets + n_clades + 1);
    const int T = split_offsets[n_clades];
    c->g1.assign(split_g1, split_g1 + T);
    c->g2.assign(split_g2, split_g2 + T);
    c->p.assign(split_p, split_p + T);
    int genes = 0;
    for (int g = 0; g < n_clades; ++g) {
      if (c->nleaves[g] == 1) ++genes;
      for (int s = c->split_off[g]; s < c->split_off[g + 1]; ++s) {
        if (c->g1[s] < 0 || c->g1[s] >= g || c->g2[s] < 0 || c->g2[s] >= g) {
          delete c;
          throw wg::Error(WG_EPARSE, "split operands must be smaller clades (clades ordered by size)");
        }
      }
    }
    c->n_genes = genes;
    *out = c;
  });
}

int wg_ccd_destroy(wg_ccd* c) {
  delete c;
  return WG_OK;
}

int wg_ccd_info(const wg_ccd* c, int32_t* n_clades, int32_t* n_triples, int64_t* observations, int32_t* n_genes) {
  WG_GUARD({
    if (!c) throw wg::Error(WG_EINVAL, "null CCD");
    if (n_clades) *n_clades = c->n_clades;
    if (n_triples) *n_triples = (int32_t)c->g1.size();
    if (observations) *observations = c->observations;
    if (n_genes) *n_genes = c->n_genes;
  });
}

int wg_ccd_export(const wg_ccd* c, int32_t* nleaves, int64_t* counts, int32_t* species_offsets, int32_t* species,
                  int32_t* split_offsets, int32_t* split_g1, int32_t* split_g2, double* split_p) {
  WG_GUARD({
    if (!c) throw wg::Error(WG_EINVAL, "null CCD");
    const size_t n = (size_t)c->n_clades, T = c->g1.size();
    if (nleaves) std::memcpy(nleaves, c->nleaves.data(), n * sizeof(int32_t));
    if (counts) std::memcpy(counts, c->counts.data(), n * sizeof(int64_t));
    if (species_offsets) std::memcpy(species_offsets, c->sp_off.data(), (n + 1) * sizeof(int32_t));
    if (species) std::memcpy(species, c->sp.data(), c->sp.size() * sizeof(int32_t));
    if (split_offsets) std::memcpy(split_offsets, c->split_off.data(), (n + 1) * sizeof(int32_t));
    if (split_g1) std::memcpy(split_g1, c->g1.data(), T * sizeof(int32_t));
    if (split_g2) std::memcpy(split_g2, c->g2.data(), T * sizeof(int32_t));
    if (split_p) std::memcpy(split_p, c->p.data(), T * sizeof(double));
  });
}

// Packing options of a batch with these flags, as wg_batch_create sets them
// for a device with 228 KB of shared memory per SM (one size class).
static wg::PackOptions2 host_pack_options(uint32_t flags) {
  wg::PackOptions2 opt;
  opt.adjoint = (flags & WG_BATCH_GRAD) != 0;
  opt.keep_tables = (flags & (WG_BATCH_GRAD | WG_BATCH_TABLES)) != 0;
  if (flags & WG_BATCH_PERSISTENT) {
    const int64_t cap = (228 * 1024 / wg::pack_knob("WG_PERSIST_CTAS", 3, 1, 8) - 1024) / 8 - 64;
    opt.light_only = true;
    opt.root_smem_doubles = cap;
    opt.smem_limit_doubles = cap;
  }
  return opt;
}

int wg_pack_info(const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags, int64_t* n_groups,
                 int64_t* n_entries, int64_t* table_doubles, int64_t* smem_bytes, double* flops_fwd) {
  WG_GUARD({
    if (!m || !ccds || n_ccds <= 0) throw wg::Error(WG_EINVAL, "wg_pack_info: bad arguments");
    std::vector<const wg::CCD*> cs(ccds, ccds + n_ccds);
    const wg::PackOptions2 opt = host_pack_options(flags);
    wg::Packed2 P = wg::pack_batch2(*m, cs, opt);
    // the persistent schedule is checked here too (topological ticket orders)
    if (flags & WG_BATCH_PERSISTENT) (void)wg::persistent_schedule(P);
    // the per-level table region of a checkpointed gradient layout
    if ((flags & WG_BATCH_CHECKPOINT) && opt.adjoint && !(flags & WG_BATCH_TABLES)) wg::checkpoint_tables(P, *m);
    if (n_groups) *n_groups = (int64_t)P.tasks.size();
    if (n_entries) *n_entries = (int64_t)P.entries.size();
    if (table_doubles) *table_doubles = P.tab_doubles;
    if (smem_bytes) *smem_bytes = (int64_t)P.max_smem * 8;
    if (flops_fwd) *flops_fwd = P.flops_fwd;
  });
}

int wg_pack_tasks(const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags, int32_t* out,
                  int64_t cap, int64_t* n_tasks) {
  WG_GUARD({
    if (!m || !ccds || n_ccds <= 0 || !n_tasks) throw wg::Error(WG_EINVAL, "wg_pack_tasks: bad arguments");
    std::vector<const wg::CCD*> cs(ccds, ccds + n_ccds);
    wg::Packed2 P = wg::pack_batch2(*m, cs, host_pack_options(flags));
    *n_tasks = (int64_t)P.tasks.size();
    if (!out) return WG_OK;
    std::vector<int> level(P.tasks.size(), 0);
    for (size_t L = 0; L < P.levels.size(); ++L)
      for (const auto* lv : {&P.levels[L], &P.levels_h[L], &P.levels_g[L], &P.levels_gh[L]})
        for (int t : *lv) level[t] = (int)L;
    for (size_t t = 0; t < P.tasks.size() && (int64_t)(t + 1) * 12 <= cap; ++t) {
      const wg::DTask& T = P.tasks[t];
      int32_t* o = out + 12 * t;
      o[0] = T.node; o[1] = level[t]; o[2] = T.width; o[3] = T.nfam;
      o[4] = T.dup.J; o[5] = T.dup.nt; o[6] = T.init.J; o[7] = T.init.nt;
      o[8] = T.tdup.J; o[9] = T.tdup.nt; o[10] = T.nlvl; o[11] = T.smem;
    }
  });
}

}  // extern "C"
