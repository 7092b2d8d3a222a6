/*
 * whalegpu.h -- C ABI of the GB300 (sm_103a) implementation of Whale.jl's
 * amalgamated reconciliation likelihood: the ALE DP over gene-family CCDs
 * under the duplication-loss + WGD model, its survival conditioning, and its
 * gradient.
 *
 * Every entry point returns an int status (WG_OK == 0, negative on error);
 * no C++ exception crosses this boundary.  The message of the last failure
 * on the calling thread is returned by wg_last_error().  Buffers are plain
 * host pointers owned by the caller; device memory is owned by the handles.
 * Calls on one wg_ctx are synchronous at return (one CUDA stream per
 * context) except the wg_enqueue_* / wg_fetch pair.
 *
 * Reference interfaces replaced (Whale.jl v2.1.0, paths in its project):
 *   wg_model_*        WhaleModel / (m::WhaleModel)(θ) / setmodel!     src/model.jl:71-191
 *                     getα, _ϵ, _ϕ, _ψ                                 src/bdputil.jl:6-11
 *   wg_model_condition condition(wm) (Root / NonExtinct / No)          src/condition.jl:11-29
 *   wg_ccd_*          read_ale / parse_aleobserve / CCD(ale, wm, spmap) src/ccd.jl:102-248
 *                     (wg_ccd_read_ale_files: many files on all host threads)
 *   wg_batch_*        index_and_getℓ + per-call table allocation       src/ccd.jl:59-75, src/core.jl:41
 *   wg_logpdf         logpdf(wm, xs::Vector{CCD})                      src/core.jl:58-64
 *   wg_logpdf_grad    ForwardDiff.gradient of the above                test/runtests.jl:36-38
 *   wg_logpdf_plain   logpdf(wm, x::CCD), one family per launch        src/core.jl:39-43
 *   wg_logpdf_tables  logpdf!(wm, x) (tables kept for backtracking)    src/core.jl:29-37
 */
#ifndef WHALEGPU_H
#define WHALEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WG_OK 0
#define WG_EINVAL (-1)   /* bad argument */
#define WG_EPARSE (-2)   /* malformed ALE / inconsistent CCD */
#define WG_ECUDA (-3)    /* CUDA runtime error */
#define WG_ENOMEM (-4)   /* host or device allocation failed */
#define WG_ESTATE (-5)   /* call out of order (e.g. rates not set) */
#define WG_ERANGE (-6)   /* size beyond a documented limit */

/* node kinds, in the reference's node order (wm.order, src/model.jl:121-139) */
#define WG_NODE_LEAF 0
#define WG_NODE_INTERNAL 1
#define WG_NODE_WGD 2
#define WG_NODE_ROOT 3

/* survival conditioning (src/condition.jl:1-29) */
#define WG_COND_NONE 0
#define WG_COND_ROOT 1
#define WG_COND_NONEXTINCT 2
#define WG_COND_NOWHERE 3  /* NowhereExtinctCondition (needs wg_model_set_rates; <= 22 leaves) */

/* wg_batch_create flags */
#define WG_BATCH_GRAD 1u   /* keep device space for the adjoint's DP tables */
#define WG_BATCH_TABLES 2u /* keep device space to return every DP table (logpdf!) */
/* Every task keeps its working rows in device memory, as the tasks too wide
 * for shared memory always do (a testing aid for that path; slower). */
#define WG_BATCH_SCRATCH_ROWS 4u
/* Per-branch checkpoint/recompute of the adjoint's DP tables in every size
 * class: only the children's top rows are kept through the evaluation and
 * each species-tree height level's tables are recomputed just before the
 * adjoint walks that level, so the device holds one level's tables at a
 * time.  Without this flag a gradient batch does this by itself for its
 * largest size classes when storing every table would exceed the table
 * budget (WG_TABLE_BUDGET_BYTES in the environment, else the device memory
 * free at creation less the batch's other buffers and a 1 GiB reserve).
 * Ignored with WG_BATCH_TABLES (logpdf! returns every table). */
#define WG_BATCH_CHECKPOINT 8u
/* One persistent launch per pass (forward, adjoint) over every task of the
 * batch instead of one launch per species-tree height level and size class:
 * CTAs take tasks in a topological order and wait (bounded) for the tasks
 * whose rows they read.  A wait that runs out of polls makes the call return
 * WG_ECUDA.  Not with WG_BATCH_CHECKPOINT (that layout keeps level launches). */
#define WG_BATCH_PERSISTENT 16u

typedef struct wg_ctx wg_ctx;
typedef struct wg_model wg_model;
typedef struct wg_ccd wg_ccd;
typedef struct wg_batch wg_batch;

const char* wg_last_error(void);
int wg_version(void);

/* ---- context: one CUDA device and stream ------------------------------- */
int wg_ctx_create(int device, wg_ctx** out);
int wg_ctx_destroy(wg_ctx* ctx);
void* wg_ctx_stream(wg_ctx* ctx); /* the cudaStream_t all work is issued on */
/* Per-kernel device timing (CUDA events on the context stream) of the last
 * evaluation: forward, adjoint and group-reduction kernels, milliseconds.
 * A size class's adjoint starts when its own forward is done (unless
 * WG_ADJ_OVERLAP=0 when the batch is created), so in a gradient evaluation
 * the split between the first two is where the last class's forward ended;
 * their sum is the evaluation's device time. */
int wg_ctx_set_timing(wg_ctx* ctx, int enable);
int wg_ctx_timings(wg_ctx* ctx, float* forward_ms, float* adjoint_ms, float* reduce_ms);
/* Measured FP64 FMA throughput of this device (TFLOP/s), from a short
 * register-resident DFMA loop; the roofline denominator for the DP kernels. */
int wg_probe_fp64(wg_ctx* ctx, double* tflops);

/* ---- species-tree model (WhaleModel, src/model.jl:96-145) --------------
 * Nodes are given in the reference order wm.order: leaves first, then the
 * internal and WGD nodes in postorder, the root last.  child0/child1 are
 * order positions (-1 when absent; a WGD node has one child).  nrow = number
 * of slices + 1 (src/model.jl:16-22), slice_len = t/n (0 when n == 0),
 * leaf_p = leafℙ (1 for a leaf, 1/k for a k-fold MUL leaf, 0 otherwise).
 * clade_offsets[n_nodes+1]/clade_species give each node's species set (the
 * species ids the CCDs use, src/model.jl:32-42). */
int wg_model_create(int32_t n_nodes, const int32_t* kind, const int32_t* child0, const int32_t* child1,
                    const int32_t* nrow, const double* slice_len, const double* leaf_p,
                    const int32_t* clade_offsets, const int32_t* clade_species, int32_t condition,
                    wg_model** out);
int wg_model_destroy(wg_model* m);
/* Per-node natural-scale rates as getθ returns them (src/rmodels.jl:31-33,
 * :55-64): lam/mu[n_nodes] (a WGD node carries its non-WGD child's rates; the
 * root's may be NaN), q[n_nodes] (read for WGD nodes only), eta, and the
 * leaf sampling probability p[n_nodes] (NULL = all 0).  Fills the slice
 * tables as setmodel! does (src/model.jl:162-191). */
int wg_model_set_rates(wg_model* m, const double* lam, const double* mu, const double* q, double eta,
                       const double* p);
/* Slice tables given directly: eps/phi/psi of every node's rows, node after
 * node in model order (sum of nrow entries each), q[n_nodes], eta.  The
 * gradient of wg_logpdf_grad is then returned w.r.t. these tables only. */
int wg_model_set_tables(wg_model* m, const double* eps, const double* phi, const double* psi,
                        const double* q, double eta);
int wg_model_get_tables(const wg_model* m, double* eps, double* phi, double* psi);
int wg_model_condition(const wg_model* m, double* out);

/* ---- conditional clade distributions (src/ccd.jl:13-248) ---------------
 * Parse ALE v0.4 text.  Gene names map to species by the prefix before the
 * first '_' (src/ccd.jl:139) through species_names -> species_ids. */
int wg_ccd_parse_ale(const char* text, size_t len, const char* const* species_names,
                     const int32_t* species_ids, int32_t n_species, wg_ccd** out);
/* read_ale over many files (src/ccd.jl:126-137): reads and parses n_files
 * ALE files on up to `threads` host threads (0: every core); out[i] receives
 * the CCD of paths[i].  If any file fails, no CCD is returned, *failed (if
 * non-null) is the index of the first failing file and the error message
 * names it. */
int wg_ccd_read_ale_files(const char* const* paths, int32_t n_files, const char* const* species_names,
                          const int32_t* species_ids, int32_t n_species, int32_t threads, wg_ccd** out,
                          int32_t* failed);
/* Build a CCD from arrays already in the reference layout: clades ordered by
 * size with leaves first and the ubiquitous clade last; splits (g1, g2, p) with
 * 0-based clade ids and p = Dip/Bip. */
int wg_ccd_create(int32_t n_clades, const int32_t* nleaves, const int32_t* species_offsets,
                  const int32_t* species, const int32_t* split_offsets, const int32_t* split_g1,
                  const int32_t* split_g2, const double* split_p, int64_t observations, wg_ccd** out);
int wg_ccd_destroy(wg_ccd* c);
int wg_ccd_info(const wg_ccd* c, int32_t* n_clades, int32_t* n_triples, int64_t* observations,
                int32_t* n_genes);
/* Export the clade table (any pointer may be NULL). */
int wg_ccd_export(const wg_ccd* c, int32_t* nleaves, int64_t* counts, int32_t* species_offsets,
                  int32_t* species, int32_t* split_offsets, int32_t* split_g1, int32_t* split_g2,
                  double* split_p);

/* ---- device-resident batch of families --------------------------------
 * The batch keeps pointers to its CCDs (wg_logpdf_plain and wg_track_device
 * build their own layouts from them on first use): destroy the batch before
 * its CCDs.  Limits (WG_ERANGE beyond them): a family's clades compatible
 * with one species node below 32,768 and a CCD below 65,535 clades (16-bit
 * program fields; the reference has no such limit), a program's partial sums
 * below 65,535. */
int wg_batch_create(wg_ctx* ctx, const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags,
                    wg_batch** out);
int wg_batch_destroy(wg_batch* b);
/* n_groups: tasks (CTAs over all launches); device_bytes: device memory held;
 * flops_fwd / bytes_fwd: algorithmic FP64 flops and bytes of one forward
 * (counted from the packed layout). */
int wg_batch_info(const wg_batch* b, int32_t* n_families, int32_t* n_groups, int64_t* device_bytes,
                  double* flops_fwd, double* bytes_fwd, double* flops_adj);

/* NowhereExtinctCondition (src/condition.jl:31-36, src/bdputil.jl:84-135)
 * of model m's tree and rates, evaluated on the device (2^leaves pgf
 * arguments, at most 22 leaves): value = log P(every leaf keeps a copy),
 * -inf when P is not in (0, 1).  With any of d_lam, d_mu, d_q, d_eta
 * non-null, also ∂value/∂ of the per-node natural rates λ, μ (K each), the
 * WGD retention rates q (K, zero at other nodes) and η.  Synchronous on the
 * context stream.  A batch whose model carries this condition evaluates it
 * the same way, beside the DP. */
int wg_nowhere_condition(wg_ctx* ctx, const wg_model* m, double* value, double* d_lam, double* d_mu, double* d_q,
                         double* d_eta);

/* Table layout of a gradient batch: size classes, how many of them recompute
 * their tables per level (WG_BATCH_CHECKPOINT), the doubles every table
 * would take and the doubles the device holds for tables.  Not in the
 * reference (its tables are allocated per call, src/core.jl:41). */
int wg_batch_tables_layout(const wg_batch* b, int32_t* classes, int32_t* checkpointed, int64_t* full_doubles,
                           int64_t* kept_doubles);

/* Kernel launches in one evaluation of the batch as last recorded: forward
 * only, and forward + adjoint + gradient reduction (0 before the first call
 * of that kind).  Not in the reference (a measurement aid). */
int wg_batch_launches(const wg_batch* b, int32_t* forward, int32_t* gradient);

/* Pack a batch on the host only (no device needed) and report its layout:
 * tasks (CTAs over all launches), program entries, DP-table doubles kept for
 * the adjoint (with WG_BATCH_GRAD | WG_BATCH_CHECKPOINT: the one-level region
 * of the per-level recomputation), largest shared memory per CTA (bytes) and
 * the algorithmic forward FLOPs.  All families form one size class here.
 * With WG_BATCH_PERSISTENT the layout (and its persistent schedule, which is
 * checked) is packed as that flag packs it. */
int wg_pack_info(const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags, int64_t* n_groups,
                 int64_t* n_entries, int64_t* table_doubles, int64_t* smem_bytes, double* flops_fwd);

/* Per-task schedule of the packed layout (tuning aid): 12 ints per task:
 * node, level, width, families, rows-program J and lanes, row-0 program J and
 * lanes, adjoint rows-program J and lanes, root levels, shared doubles. */
int wg_pack_tasks(const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags, int32_t* out,
                  int64_t cap, int64_t* n_tasks);

/* ---- likelihood -------------------------------------------------------
 * per_family[i] = log L_i (-Inf when L_i <= 0) without conditioning
 * (src/core.jl:39-43); total = sum_i per_family[i] - N * condition, non-finite
 * mapped to -Inf (src/core.jl:15, :58-64).  Either pointer may be NULL. */
int wg_logpdf(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total);
/* As wg_logpdf plus the gradient of total w.r.t. the per-node natural-scale
 * lam, mu, q (n_nodes each) and eta given to wg_model_set_rates.  After
 * wg_model_set_tables, d_eps/d_phi/d_psi (sum of nrow each) receive the
 * gradient w.r.t. the tables instead (any output pointer may be NULL). */
int wg_logpdf_grad(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total,
                   double* d_lam, double* d_mu, double* d_q, double* d_eta,
                   double* d_eps, double* d_phi, double* d_psi);
/* Weighted form: total = sum_i weights[i] * per_family[i] - cond_scale *
 * condition (terms with weight 0 dropped) and its gradient, the adjoint of
 * family i seeded with weights[i] (weights: one per family, in batch order).
 * The building block of MixtureModel (src/core.jl:66-75: weights = each
 * family's posterior component weight, cond_scale = their sum) and ModelArray
 * (src/core.jl:77-78: unconditioned, cond_scale = 0); the reference has no C
 * counterpart. */
int wg_logpdf_grad_weighted(wg_ctx* ctx, wg_model* m, wg_batch* b, const double* weights, double cond_scale,
                            double* per_family, double* total, double* d_lam, double* d_mu, double* d_q,
                            double* d_eta, double* d_eps, double* d_phi, double* d_psi);
/* One family per launch: the plain per-family path (src/core.jl:39-43). */
int wg_logpdf_plain(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total);
/* logpdf! (src/core.jl:29-37): also returns family i's DP tables.  out holds,
 * node after node in model order, the node's rows (nrow x ncompat, row-major,
 * compatible clades in ascending clade id).  cap = doubles available; the
 * needed size is returned in *needed (call with out == NULL to query).
 * The batch must have been created with WG_BATCH_TABLES. */
int wg_logpdf_tables(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t family, double* out, int64_t cap,
                     int64_t* needed, double* logl);

/* The DP tables of family i as the batch's last fetched evaluation left them
 * (wg_logpdf, wg_logpdf_grad[_weighted], wg_fetch, wg_logpdf_tables), in the
 * wg_logpdf_tables layout, and its log L; no evaluation here.  One batched
 * logpdf! then one download per family: the order src/track.jl:18-21 names
 * as the faster one for TreeTracker.  The batch must have WG_BATCH_TABLES;
 * WG_ESTATE when no fetched evaluation holds the tables (none yet, one
 * pending, or wg_logpdf_noalloc since).  *needed as wg_logpdf_tables. */
int wg_batch_tables(wg_ctx* ctx, wg_batch* b, int32_t family, double* out, int64_t cap, int64_t* needed,
                    double* logl);

/* Forward evaluation that allocates nothing (no counterpart in the reference).
 * For callers that cannot allocate device memory when they evaluate: hosts
 * whose device memory is owned by another allocator or pool, and sampler
 * loops that must not enter the allocator between steps (cudaMalloc can
 * synchronise the device and fail under memory pressure).  Same results
 * as wg_logpdf on a batch created beforehand (any flags).  The scratch it
 * needs -- the top row of every (node, family group) task -- lives in one
 * fixed device array of 1 << 20 doubles (8 MiB) that every GPU loading the
 * library holds until exit; batches needing more are rejected with WG_ERANGE.
 * wg_ctx_create looks up that array's device address once (the library's
 * kernels are loaded by then, so the lookup allocates nothing); this call
 * only uses it.  An evaluation enqueued by wg_enqueue must be fetched first
 * (WG_ESTATE otherwise).  All calls share the array and it keeps the last
 * call's contents: calls whose work overlaps on the GPU (two host threads,
 * two contexts on one device) race on it. */
int wg_logpdf_noalloc(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total);

/* backtrack (src/track.jl:180-488): samples n_samples reconciled gene trees
 * of family i from its DP tables (the batch must have WG_BATCH_TABLES; the
 * batch is evaluated first, as logpdf! then backtrack).  out receives one
 * extended-Newick line per tree, NUL-terminated: nodes carry
 * [&&NHX:label=<speciation|duplication|wgd|wgdloss|sploss|loss>:node=<model
 * order position>:clade=<0-based clade, -1 for a loss>:slice=<t>], leaves the
 * gene name (or "loss"), branch lengths from the reference's node heights.
 * The same seed gives the same trees; *needed = bytes including the NUL (call
 * with out == NULL to query).  Randomness is this library's xoshiro256**
 * stream, not Julia's: trees match the reference in distribution. */
int wg_backtrack(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t family, int32_t n_samples, uint64_t seed, char* out,
                 int64_t cap, int64_t* needed);
/* The same sampling from DP tables the caller already holds (host only, no
 * device): tables in the wg_logpdf_tables layout for model m (its slice
 * tables set) and CCD c; n_tables = their length. */
int wg_backtrack_tables(const wg_model* m, const wg_ccd* c, const double* tables, int64_t n_tables, int32_t n_samples,
                        uint64_t seed, char* out, int64_t cap, int64_t* needed);

/* TreeTracker's sampling on the device (src/track.jl:180-414, :30-40): tree i
 * of family families[i] is drawn with seed seeds[i] by one GPU thread from the
 * DP tables of the batch's last fetched evaluation (as wg_batch_tables: the
 * batch has WG_BATCH_TABLES), with the host sampler's event order, arithmetic
 * and random stream, so a tree equals wg_backtrack_tables' for the same seed
 * (n_samples = 1).  offsets[n_trees + 1] receives the prefix sums of the trees'
 * node counts; the nodes stay in the batch until wg_track_nodes copies them.
 * Nothing but these node arrays crosses to the host.  m: the batch's model
 * (its structure maps clades to table columns on the first call). */
int wg_track_device(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t n_trees, const int32_t* families,
                    const uint64_t* seeds, int64_t* offsets);
/* The last wg_track_device call's nodes, 4 ints each: clade (-1: loss),
 * species node (model-order position), slice where its branch starts,
 * parent node (-1 at the root), trees one after another, nodes in the
 * sampler's order.  cap = nodes the buffer holds. */
int wg_track_nodes(const wg_batch* b, int32_t* nodes, int64_t cap);
/* One tree's node arrays (as wg_track_nodes gives them) as wg_backtrack's
 * extended Newick line, NUL-terminated; *needed as there. */
int wg_tree_newick(const wg_model* m, const wg_ccd* c, const int32_t* nodes, int32_t n_nodes, char* out, int64_t cap,
                   int64_t* needed);

/* Asynchronous pair for device-side timing: enqueue the evaluation on the
 * context stream (inputs already resident), then fetch the results (this
 * synchronises).  with_grad selects the adjoint. */
int wg_enqueue(wg_ctx* ctx, wg_model* m, wg_batch* b, int with_grad);
int wg_fetch(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total, double* d_lam,
             double* d_mu, double* d_q, double* d_eta);

/* ---- workload generator (stand-in for the reference's simulate + ALEobserve,
 * src/simulation.jl:14-133, src/ccd.jl:262-268) ----------------------------
 * Simulates one gene family under the DL+WGD model on the given model and
 * rates (root condition: genes on both sides of the root), perturbs its
 * gene tree with random NNIs over n_trees samples and amalgamates them into
 * ALE v0.4 text.  Writes at most cap bytes to out (NUL-terminated), returns
 * the needed length in *len.  species_names[i] names the leaf at order
 * position i (empty for non-leaves).  flags: WG_SYNTH_WALK = each sample
 * perturbs the previous one (otherwise the true tree); WG_SYNTH_PUSH = while
 * fewer than target_clades clades exist, samples take max_nni moves. */
#define WG_SYNTH_WALK 1
#define WG_SYNTH_PUSH 2
int wg_synth_family(const wg_model* m, const double* lam, const double* mu, const double* q, double eta,
                    const char* const* species_names, uint64_t seed, int32_t n_trees, int32_t max_nni,
                    int32_t min_genes, int32_t target_clades, int32_t flags, char* out, int64_t cap,
                    int64_t* len);

#ifdef __cplusplus
}
#endif
#endif /* WHALEGPU_H */
