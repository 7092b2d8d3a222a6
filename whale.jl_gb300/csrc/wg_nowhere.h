// NowhereExtinctCondition on the device (src/condition.jl:31-36,
// src/bdputil.jl:84-135).
//
// log P(every leaf keeps a copy) = log(1 - Σ_{i<last} s_i P(x_i)), the
// inclusion-exclusion over the joint pgf P of the leaf counts at all 2^L
// binary arguments x_i (leaf bits of i: 0 or 1), s_i = (-1)^popcount(i).
// Every node k holds a vector v_k over the 2^{L_k} arguments of its own
// leaves (the first child's leaves in the low bits, as in the reference's
// treepgf_allbinary):
//   x_k = v_{c0} ⊗ v_{c1} (binary), v_{c0} (WGD), the leaf bit (leaf)
//   y_k = x_k (1 - q + x_k q) at a WGD node, x_k otherwise
//   v_k = pgf of the linear birth-death process over the branch at y_k
//         (critical form when |λ - μ| <= 1e-6), or at the root the
//         geometric prior ηy / (1 - (1-η)y),
// each evaluated in the reference's own arithmetic.
//
// Kernels: one CTA computes the vectors of every node below the root
// (postorder, a barrier per height); the root's 2^L entries are tiled over
// the grid, which also starts the reverse sweep (adjoint seed -s_i, tile
// partial sums for the children's adjoints); one CTA finishes the reverse
// sweep (preorder) and writes, per node, the adjoints of λ, μ and q.  The
// host sums the root tiles in a fixed order.  Everything is deterministic.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <vector>

#include "wg_internal.h"

namespace wg {

struct NwTopo {
  int kind, c0, c1;  // WG_NODE_*, children (-1: none)
  int L, L0;         // leaves below the node and below its first child
  int pad;
  int64_t off;       // offset of the node's vector in v / bv
};

struct NwPlan {
  int device = 0;
  int K = 0, root = -1;
  std::vector<int> kind, ch0, ch1;  // the tree the plan was built for
  // root tiles: T0 x T1 entries (first child's index fastest), nt0 x nt1 tiles
  int T0 = 1, T1 = 1, lT0 = 0, lT1 = 0, nt0 = 1, nt1 = 1, ntiles = 1;
  int n_fwd_lv = 0, n_rev_lv = 0, n_fwd = 0, n_rev = 0;
  int64_t nv = 0;    // doubles of all node vectors
  int64_t pq_n = 0;  // doubles per reduction array of the reverse sweep
  bool pq_smem = false;
  int n_out = 0;     // ntiles Σ s_i v | ntiles ∂/∂η | 3·K node adjoints
  double* d_coef = nullptr;  // 6 per node: λ (η at the root) μ t ρ q mode
  NwTopo* d_topo = nullptr;
  int* d_lists = nullptr;    // forward nodes | offsets | reverse nodes | offsets
  double* d_v = nullptr;
  double* d_bv = nullptr;
  double* d_pq = nullptr;
  double* d_part = nullptr;  // root tiles' partial sums: rows [nt1][n0] | cols [nt0][n1]
  double* d_out = nullptr;
  double* h_coef = nullptr;  // pinned
  double* h_out = nullptr;   // pinned
  cudaStream_t s = nullptr;  // side stream of the batched evaluation
  cudaEvent_t fork = nullptr, done = nullptr;
  NwPlan() = default;
  NwPlan(const NwPlan&) = delete;
  NwPlan& operator=(const NwPlan&) = delete;
  ~NwPlan();
};

struct NwResult {
  double value = 0.0;  // log P; -inf when P is not in (0, 1)
  bool ok = false;
  std::vector<double> d_lam, d_mu, d_q;  // per node, ∂ value / ∂ natural rate
  double d_eta = 0.0;
};

// Plan for model m's tree; WG_ERANGE above 22 leaves.
std::unique_ptr<NwPlan> nw_plan_create(const Model& m, int device);
bool nw_plan_matches(const NwPlan& p, const Model& m);
// Coefficients of m's current rates into the pinned staging buffer.
void nw_stage(NwPlan& p, const Model& m);
// Coefficient upload, kernels and result download on stream s (capturable);
// returns the kernel launches.
int nw_record(NwPlan& p, cudaStream_t s, bool grad);
// After the recorded work completed: value and, with grad, the adjoints.
NwResult nw_result(const NwPlan& p, const Model& m, bool grad);

}  // namespace wg
