// Internal declarations shared by the host C++ and the CUDA translation units
// of libwhalegpu.  Nothing here is part of the public ABI (include/whalegpu.h).
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <exception>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/whalegpu.h"

namespace wg {

// Error carried to the C ABI as (status, message).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

// Host threads of the packer: WG_PACK_THREADS when set, else 0 (every core).
inline int default_host_threads() {
  const char* e = std::getenv("WG_PACK_THREADS");
  return e ? std::atoi(e) : 0;
}

// A packing knob from the environment (WG_PACK_TARGET_OPS, WG_PACK_TARGET_J,
// WG_PACK_ROOT_GROUP, WG_PACK_HEAVY_OPS: what the autotuner varies), else
// its default; values outside [lo, hi] are refused.
inline int64_t pack_knob(const char* name, int64_t dflt, int64_t lo, int64_t hi) {
  const char* e = std::getenv(name);
  if (!e || !*e) return dflt;
  char* end = nullptr;
  const long long v = std::strtoll(e, &end, 10);
  if (end == e || *end != '\0') throw Error(WG_EINVAL, std::string(name) + " is not an integer");
  if (v < lo || v > hi) throw Error(WG_EINVAL, std::string(name) + " out of range");
  return (int64_t)v;
}

// fn(i) for i < n on up to `threads` host threads (0: all cores); the first
// exception is rethrown here.
template <class F>
void parallel_for(size_t n, int threads, F fn) {
  unsigned nt = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
  nt = (unsigned)std::min<size_t>({(size_t)nt, (size_t)64, n});
  if (nt <= 1) {
    for (size_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::exception_ptr> err(nt);
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      try {
        for (size_t i; (i = next.fetch_add(1)) < n;) fn(i);
      } catch (...) {
        err[t] = std::current_exception();
        next = n;
      }
    });
  for (auto& th : pool) th.join();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
}

// ---------------------------------------------------------------------------
// Species-tree model: the node order, per-node slice shapes and species sets
// of a WhaleModel, and the current slice tables [ε, ϕ, ψ] (src/model.jl).
// ---------------------------------------------------------------------------
struct Model {
  int K = 0;                         // nodes, in the reference order
  std::vector<int> kind, ch0, ch1;   // WG_NODE_*, children (order positions)
  std::vector<int> nrow, row_off;    // rows per node, prefix offsets (size K+1)
  std::vector<double> slice_len, leaf_p;
  int n_words = 0;                   // species bitset words
  std::vector<uint64_t> clade_bits;  // K * n_words
  int cond = WG_COND_ROOT;
  // parameters of the current evaluation
  bool has_params = false;
  bool from_rates = false;           // tables were derived from rates (gradient maps back to rates)
  std::vector<double> lam, mu, q, p; // per node (natural scale)
  double eta = 0.66;
  std::vector<double> eps, phi, psi; // per row, sum(nrow)
  uint64_t version = 0;              // bumped on every parameter change
  int total_rows() const { return row_off.empty() ? 0 : row_off[K]; }
  double eps_top(int k) const { return eps[row_off[k] + nrow[k] - 1]; }
};

// Slice tables from rates (setmodel!, src/model.jl:162-191).
void model_fill_tables(Model& m);
// Condition value (src/condition.jl:11-29).
double model_condition(const Model& m);
// Adjoint of the condition w.r.t. the tables: adds -scale * d cond to the
// adjoints of the top ε of the root's children / root and to d_eta.
void model_condition_vjp(const Model& m, double scale, std::vector<double>& d_eps, double& d_eta);
// NowhereExtinctCondition depends on the rates directly: adds scale * d cond
// to the adjoints of the per-node natural rates λ, μ, q and to d_eta (no-op
// for the other conditions).
void model_condition_rates_vjp(const Model& m, double scale, std::vector<double>& d_lam, std::vector<double>& d_mu,
                               std::vector<double>& d_q, double& d_eta);
// Adjoint of setmodel!: given adjoints of every table entry (eps/phi/psi per
// row) and of q per node, accumulates adjoints of lam, mu, q, p per node.
void model_tables_vjp(const Model& m, std::vector<double> d_eps, const std::vector<double>& d_phi,
                      const std::vector<double>& d_psi, std::vector<double>& d_lam,
                      std::vector<double>& d_mu, std::vector<double>& d_q, std::vector<double>& d_p);

// ---------------------------------------------------------------------------
// Conditional clade distribution in the reference layout (src/ccd.jl:80-121):
// clades ordered by (size, ALE set id), leaves first, ubiquitous clade last.
// ---------------------------------------------------------------------------
struct CCD {
  int n_clades = 0;
  int64_t observations = 0;
  int n_genes = 0;
  std::vector<int> nleaves;
  std::vector<int64_t> counts;
  std::vector<int> sp_off, sp;           // species ids per clade (CSR)
  std::vector<int> split_off, g1, g2;    // splits per clade (CSR), 0-based clade ids
  std::vector<double> p;                 // Dip / Bip
  std::vector<std::string> leaf_name;    // gene name of each single-gene clade ("" otherwise)
};

CCD* parse_ale(const char* text, size_t len, const std::vector<std::string>& names,
               const std::vector<int>& ids);

// ---------------------------------------------------------------------------
// Packed device layout.  Families are packed into groups; one CTA evaluates
// one group as a block-diagonal union of its families' CCDs.  For every
// (group, node) the host emits statically scheduled "sum programs": lane t
// of the CTA executes entries [j * nt + t], j < J, each accumulating
// p * A[a] * B[b] into a running sum that is flushed to a partial slot at a
// segment end.  A finalize pass then combines the partial slots of each clade.
// ---------------------------------------------------------------------------
constexpr int kNT = 128;           // threads per CTA of the batched kernels
constexpr uint64_t kValid = 1;     // entry flags (bits 48..63 of code)
constexpr uint64_t kEnd = 2;

struct alignas(16) DEntry {
  uint64_t code;  // plain programs: a | b << 16 | dst << 32 | flags << 48; batched programs:
                  // f0 | f1 << 16 | f2 << 32 | op << 48 | column kind << 56
  double p;
};

// Allocator whose resize() leaves trivial elements uninitialised: large
// buffers that are filled right after (in parallel) are not first zeroed on
// one thread.
template <class T>
struct UninitAlloc : std::allocator<T> {
  template <class U>
  struct rebind { using other = UninitAlloc<U>; };
  UninitAlloc() = default;
  template <class U>
  UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept { ::new ((void*)p) U; }
  template <class U, class... A>
  void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};

struct DProg {
  int64_t off = 0;  // first entry
  int32_t J = 0;    // iterations
  int32_t nt = 0;   // lanes (multiple of 32, <= kNT)
};

struct DNode {
  int32_t width = 0;     // row width R (sum of compatible clades over the group's families)
  int32_t nslot_dup = 0;
  int64_t top_off = 0;   // doubles: top row in the tops buffer
  int64_t tab_off = -1;  // doubles: row 0 of this node's table (-1: tables not kept)
  DProg dup;             // duplication sum over the previous row (also WGD row 1)
  int64_t fin_dup = 0;   // int2 per clade: (slot start, n segments) of dup
  DProg r1;              // speciation sum over the children's top rows
  int64_t fin_r1 = 0;    // int2 per clade for r1
  int64_t aux = 0;       // int2 per clade: loss map (pos in child0, pos in child1) or leaf flag
  // adjoint programs (transposed), see the adjoint kernel
  DProg tdup;            // per clade x: sum over (parent γ, sibling) of p * bar[γ] * row[sib]
  int64_t fin_tdup = 0;
  DProg tr1a;            // per clade of child0: sum over entries of p * bar[γ] * top1[sib]
  int64_t fin_tr1a = 0;
  DProg tr1b;            // per clade of child1
  int64_t fin_tr1b = 0;
  int64_t inv_a = 0;     // int per child0 clade: position in this row (loss term), -1 if none
  int64_t inv_b = 0;     // int per child1 clade
  // root only: clade-size levels of the same-row recursion (Πroot)
  int32_t nlvl = 0;
  int32_t _pad = 0;
  int64_t lvl = 0;       // first DLevel
  int64_t fin_lvl = 0;   // int2 per clade (slots inside its level's program)
  int64_t lvl_clades = 0;  // ints: clade positions sorted by level
  int64_t tlvl = 0;        // first DLevel of the transposed level programs (adjoint)
  int64_t fin_tlvl = 0;
};

struct DLevel {
  DProg prog;
  int32_t begin = 0, end = 0;  // range in lvl_clades
};

struct DGroup {
  int32_t n_fam = 0;
  int32_t maxw = 0;       // max row width over nodes
  int32_t maxslot = 0;    // max partial slots over programs
  int32_t _pad = 0;
  int64_t node0 = 0;      // first DNode (K per group)
  int64_t fam0 = 0;       // first entry of fam_idx / fam_pos
  double work = 0;        // estimated DP work (for ordering)
};

struct Packed {
  std::vector<DGroup> groups;
  std::vector<DNode> nodes;
  std::vector<DEntry> entries;
  std::vector<int32_t> meta;   // int2 arrays are stored as pairs of int32
  std::vector<DLevel> levels;
  std::vector<int32_t> fam_idx, fam_pos;
  // per original family f and node k (index f * K + k): first DNode of the
  // family's group, column offset of the family in the group row, columns
  std::vector<int64_t> fam_node0;
  std::vector<int32_t> fam_col, fam_ncol;
  int64_t tops_doubles = 0;
  int64_t tab_doubles = 0;
  int32_t max_smem_doubles = 0;
  double flops_fwd = 0, bytes_fwd = 0, flops_adj = 0;
};

struct PackOptions {
  int64_t group_width = 1024;   // target sum of clade counts per group
  int64_t group_cap = 4096;     // hard cap on the row width of a group
  bool keep_tables = false;     // allocate table space (adjoint / logpdf!)
  bool adjoint = false;         // build transposed programs
  bool single = false;          // one family per group (plain path)
};

Packed pack_batch(const Model& m, const std::vector<const CCD*>& ccds, const PackOptions& opt);

// ---------------------------------------------------------------------------
// Batched layout (level-synchronous tasks).  A task is one species node for a
// group of families; the tasks of one height level of the species tree are
// independent and run in one launch, one CTA per task.  Every task runs
// host-scheduled lane programs whose entries are either products
// (acc += p * A[a] * B[b]) or finalize ops that consume acc and write a row
// value; clades too long for one lane are split into partial slots that a
// short combine pass (after one barrier) finishes.
// ---------------------------------------------------------------------------
// Kind of a program column (bits 56-63 of an entry's code), the same for the
// 32 lanes of a warp: PROD columns hold products (or idle lanes), FIN columns
// finalize ops (or partial-sum stores, or idle lanes), PART columns only
// partial-sum stores, NOP columns nothing.  A warp then never runs two FP64
// paths for one column.
namespace col {
enum : uint32_t { NOP = 0, PROD = 1, FIN = 2, PART = 3 };
}

namespace op {
enum : uint32_t {
  PROD = 0,
  FIN_DUP = 1,     // out[c] = ψ·acc + ϕ·in[c]
  FIN_SPEC = 2,    // out[c] = acc + (A[a]·εb + B[b]·εa)
  FIN_WGD = 3,     // out[c] = q·acc + ((1-q)·A[a] + 2qεf·A[a])
  FIN_LVL = 4,     // cur[c] = ca·acc + cb·cur[c]            (root, in place)
  FIN_PART = 5,    // part[slot] = acc
  FIN_ADJ = 6,     // barn[c] = ψ·acc + ϕ·bar[c]; dϕ += bar[c]·L[c]; dψ += acc·L[c]
  FIN_TOP = 7,     // bartop[c] = acc + (bar[a]·ε)             (speciation/loss adjoint)
  FIN_WGDADJ = 8,  // bartop[c] = ((1-q) + 2qεf)·bar[c] + q·acc; dq, dεf
  FIN_TLVL = 9,    // bar[c] += ca·acc; dca += acc·L[c]/2     (root levels, reverse)
  NOP = 15,
};
}

struct DProg2 {
  int64_t off = 0;      // entries [j * nt + lane]
  int32_t J = 0;
  int32_t nt = 0;       // lanes used (multiple of 32)
  int64_t comb = 0;     // combine entries (one per split clade)
  int32_t ncomb = 0;
  uint16_t nslot = 0;   // partial slots (host: shared-memory sizing)
  uint16_t nbig = 0;    // leading combine entries a warp each combines (the rest: a thread each)
};

struct DTask {
  int32_t node = 0;     // model order position
  int32_t width = 0;    // R: row width (sum of compatible clades of its families)
  int32_t wa = 0, wb = 0;  // staged widths of child 0 / child 1 top rows
  int32_t nfam = 0;     // families (root tasks: log L outputs)
  int32_t smem = 0;     // shared doubles needed (forward)
  int32_t nt = 0;       // threads of the CTA that runs the task
  int32_t nslot_max = 0;  // partial slots of the largest program (shared-memory layout)
  int64_t tab = -1;     // DP table base, task-major [row][R] (-1: not kept)
  int64_t top = 0;      // top row base in the tops buffer
  int64_t gmap = 0;     // int64 per staged position (wa + wb): offset in tops
  int64_t aux = 0;      // leaf tasks: int per clade, 1 for leaf clades
  int64_t loss = 0;     // int2 per clade: positions in stage A / stage B (-1)
  int64_t inva = 0;     // int per stage-A position: row position of that clade (-1)
  int64_t invb = 0;     // int per stage-B position
  DProg2 dup, init;     // forward: rows >= 1, row 0
  DProg2 tdup;          // adjoint of rows >= 1 (and WGD row 0)
  DProg2 ta, tb;        // adjoint of the speciation row 0, per child
  int32_t nlvl = 0;     // root: levels of the same-row recursion
  int32_t rslot = 0;    // root: partial slots of the level programs
  int64_t lvl = 0;      // root: first DProg2 of the level programs (forward)
  int64_t tlvl = 0;     // root: first DProg2 of the level programs (adjoint)
  int64_t fam = 0;      // root: int2 per family (family index, ubiquitous position)
  int64_t gout = 0;     // adjoint: per-task outputs, 2 * nrow + 5 doubles
  int64_t scratch = -1;  // rows wider than shared memory: offset of the task's working rows in the
                         // batch's device scratch (doubles); -1: the rows live in shared memory
  int32_t smem_adj = 0;  // shared doubles needed (adjoint)
  int32_t tstride = 0;   // doubles between the DP-table rows: width rounded up to even (rows start 16-byte aligned)
};

struct Packed2 {
  std::vector<DTask> tasks;
  std::vector<DEntry, UninitAlloc<DEntry>> entries;  // filled in parallel after sizing
  std::vector<int32_t> meta;
  std::vector<int64_t> gmap;
  std::vector<DProg2> progs;               // level programs
  // task indices per launch level, for light (kNT2L threads) and heavy
  // (kNT2H threads) tasks, with the largest shared memory of each launch
  std::vector<std::vector<int32_t>> levels, levels_h;
  std::vector<int32_t> level_smem, level_smem_adj, level_smem_h, level_smem_adj_h;
  // tasks whose rows exceed shared memory (working rows in device scratch),
  // per level: 128-thread (root) and 256-thread CTAs
  std::vector<std::vector<int32_t>> levels_g, levels_gh;
  int64_t scratch_doubles = 0;
  int64_t tops_doubles = 0, tab_doubles = 0, gout_doubles = 0;
  // gradient reduction: for every output j (3 NR + K + 1), the gout indices
  // that contribute, in a fixed order (CSR)
  std::vector<int64_t> red_off, red_idx;
  // per family f and node k (f * K + k): table base, row width, column, columns
  std::vector<int64_t> fam_tab;
  std::vector<int32_t> fam_w, fam_col, fam_ncol;
  double flops_fwd = 0, bytes_fwd = 0, flops_adj = 0;
  int32_t max_smem = 0;
};

constexpr int kNT2L = 128;   // threads per CTA of light tasks
constexpr int kNT2H = 256;   // threads per CTA of heavy (single large family) tasks

struct PackOptions2 {
  int64_t target_ops = pack_knob("WG_PACK_TARGET_OPS", 480, 32, 1 << 16);  // forward product + finalize ops per row per task
  int64_t heavy_ops = pack_knob("WG_PACK_HEAVY_OPS", 1024, 32, 1 << 20);  // non-root tasks above this many ops per row get kNT2H threads
  int64_t max_width = 6144;   // cap on a task's row width
  // Root tasks run their same-row levels one after another, each short and
  // latency-bound, so they take target_ops * root_group ops (all levels
  // together), up to max_width_root clades (their adjoint keeps six rows).
  int root_group = (int)pack_knob("WG_PACK_ROOT_GROUP", 16, 1, 256);
  int64_t max_width_root = 1536;
  // tasks needing more shared doubles than this keep their working rows in
  // device memory (L2-resident) instead
  int64_t smem_limit_doubles = 227 * 1024 / 8;
  int target_j = (int)pack_knob("WG_PACK_TARGET_J", 3, 1, 16);  // iterations per row the lane scheduler aims for
  // iterations per same-row level of a root task the lane scheduler aims for
  // (levels within one warp synchronize that warp only)
  int level_j = (int)pack_knob("WG_PACK_LEVEL_J", 3, 1, 32);
  // split clades of the forward programs with at least this many partial
  // sums are combined by a warp each (0: every one by a thread; adjoint
  // programs always combine by thread).  Measured on 5,000 config-1
  // families: 24 gives 1.510 ms per gradient evaluation, 0 1.517 ms.
  int comb_warp = (int)pack_knob("WG_PACK_COMB_WARP", 24, 0, 1 << 16);
  // persistent launches: every task takes kNT2L threads, and a root task's
  // families are grouped so that its adjoint rows fit in this many shared
  // doubles (0: no such bound)
  bool light_only = false;
  int64_t root_smem_doubles = 0;
  bool keep_tables = false;
  bool adjoint = false;
  const std::vector<int>* global_ids = nullptr;  // family index written to log L outputs
  int threads = default_host_threads();  // host threads building tasks; the layout does not depend on it
};

Packed2 pack_batch2(const Model& m, const std::vector<const CCD*>& ccds, const PackOptions2& opt);

// Schedule of a layout run as one persistent launch per pass: the tickets'
// task order of the forward (height levels upwards, each level in launch
// order) and of the adjoint (levels downwards), and per task the tasks it
// waits for: in the forward the producers of the children's top rows it
// stages, in the adjoint the tasks that stage its own top row (they write its
// top-row adjoints).  CSR, task indices of the layout.
struct Schedule {
  std::vector<int32_t> order_fwd, order_adj;
  std::vector<int32_t> fdep_off, fdep_idx, adep_off, adep_idx;
};
Schedule persistent_schedule(const Packed2& P);

// Re-lays a gradient layout's tables for per-level recomputation (every
// height level's tasks share one region from offset 0); returns the doubles
// that region needs.
int64_t checkpoint_tables(Packed2& P, const Model& m);

// For every node (model order) and clade: the clade's column among the
// node's compatible clades (ascending clade id), -1 if incompatible.
std::vector<std::vector<int>> compat_columns(const Model& m, const CCD& c);

// Samples n reconciled trees of a family from its DP tables (the layout of
// wg_logpdf_tables); one extended-Newick line per tree.
std::string backtrack_family(const Model& m, const CCD& c, const double* tables, int n_samples, uint64_t seed);

// One sampled tree given as node arrays (clade, species node, slice, parent;
// nodes in the sampler's creation order) in the extended Newick of
// backtrack_family.
std::string tree_newick(const Model& m, const CCD& c, const int32_t* nodes, int n);

}  // namespace wg

// Public opaque handles are the internal types.
struct wg_model : wg::Model {};
struct wg_ccd : wg::CCD {};

// Run `body`, mapping exceptions to (status, wg_last_error()).
#define WG_GUARD(...)                                           \
  try {                                                         \
    __VA_ARGS__;                                                \
    return WG_OK;                                               \
  } catch (const wg::Error& e) {                                \
    wg::set_last_error(e.what());                               \
    return e.code;                                              \
  } catch (const std::bad_alloc&) {                             \
    wg::set_last_error("host allocation failed");              \
    return WG_ENOMEM;                                           \
  } catch (const std::exception& e) {                           \
    wg::set_last_error(e.what());                               \
    return WG_EINVAL;                                           \
  }

