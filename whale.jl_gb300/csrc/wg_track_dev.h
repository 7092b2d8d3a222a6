// Device backtracking (wg_track_dev.cu): the arguments of one launch that
// samples one reconciled tree per thread from a batch's DP tables.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/whalegpu.h"

namespace wg {

// per-tree status written instead of a node count
constexpr int kTrackOverflow = -1;      // more nodes than the tree's capacity
constexpr int kTrackNoEvent = -2;       // a state with no event of positive weight
constexpr int kTrackNoLikelihood = -3;  // the family's likelihood is not positive

struct TrackArgs {
  // model
  int K = 0, NR = 0;
  const int4* mnode = nullptr;    // kind, child0, child1, nrow per node
  const int* row_off = nullptr;   // K + 1
  const double* params = nullptr; // eps | phi | psi (NR each) | q (K) | eta
  // families
  const double* const* ftabs = nullptr;  // per family: the table buffer of its size class
  const int64_t* fk_tab = nullptr;       // per (family, node): first double of the task's table
  const int* fk_w = nullptr;             // row width of that table
  const int* fk_col = nullptr;           // column of the family's first compatible clade
  const int64_t* fclade = nullptr;       // per family: its first clade in the clade arrays
  const int* fnclade = nullptr;
  const int64_t* fcol = nullptr;         // per family: its first entry of cols
  const int16_t* cols = nullptr;         // per (family, node, clade): column among the compatible clades, -1
  const int64_t* csplit = nullptr;       // per clade (all families) + 1: first split
  const int* g1 = nullptr;               // splits: clade ids within the family
  const int* g2 = nullptr;
  const double* sp = nullptr;            // split probabilities
  const unsigned char* cleaf = nullptr;  // per clade: 1 for a single-gene clade
  // trees
  int n = 0;
  const int* fam = nullptr;
  const uint64_t* seed = nullptr;
  const int64_t* cap_off = nullptr;      // per tree: first node slot; [n] = total slots
  int4* nodes = nullptr;                 // (clade, species node, slice, parent) per node
  int4* stack = nullptr;                 // work stack (same slots)
  int* count = nullptr;                  // per tree: nodes, or a negative status
};

cudaError_t track_launch(const TrackArgs& A, cudaStream_t s);
cudaError_t track_compact(const int4* nodes, const int64_t* cap_off, const int64_t* off, int4* out, int n,
                          cudaStream_t s);

}  // namespace wg
