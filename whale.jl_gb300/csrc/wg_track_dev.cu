// Backtracking on the device (src/track.jl:180-414): one thread samples one
// reconciled gene tree of one family from the DP tables a batched logpdf!
// left in device memory.  The event order, the arithmetic (every product and
// difference rounded on its own, as the host sampler compiled without FMA
// contraction) and the random stream (xoshiro256** seeded by splitmix64) are
// those of the host sampler (wg_track.cpp), so a tree equals the host's for
// the same seed; the host formats the compact node arrays as text.
#include <cuda_runtime.h>

#include "wg_track_dev.h"

namespace wg {
namespace {

struct DRng {
  uint64_t s[4];
  __device__ explicit DRng(uint64_t seed) {
    for (int i = 0; i < 4; ++i) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s[i] = z ^ (z >> 31);
    }
  }
  __device__ static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  __device__ uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  __device__ double uniform() { return __dmul_rn((double)(next() >> 11), 0x1.0p-53); }
};

struct St {
  int e, g, t;
};

// The model, the family and its tables as one thread sees them.
struct Fam {
  const TrackArgs* A;
  int f;
  int nc;
  const double* tab;
  __device__ int col(int e, int g) const { return A->cols[A->fcol[f] + (int64_t)e * nc + g]; }
  __device__ double L(int e, int g, int t) const {
    const int c = col(e, g);
    if (c < 0) return 0.0;
    const int64_t fk = (int64_t)f * A->K + e;
    return tab[A->fk_tab[fk] + (int64_t)(t - 1) * A->fk_w[fk] + A->fk_col[fk] + c];
  }
  __device__ int nrow(int e) const { return A->mnode[e].w; }
  __device__ double Ltop(int e, int g) const { return L(e, g, nrow(e)); }
  __device__ double eps_top(int e) const { return A->params[A->row_off[e] + nrow(e) - 1]; }
  __device__ double phi(int e, int t) const { return A->params[A->NR + A->row_off[e] + t - 1]; }
  __device__ double psi(int e, int t) const { return A->params[2 * A->NR + A->row_off[e] + t - 1]; }
  __device__ int64_t split0(int g) const { return A->csplit[A->fclade[f] + g]; }
  __device__ int64_t split1(int g) const { return A->csplit[A->fclade[f] + g + 1]; }
  __device__ bool leafclade(int g) const { return A->cleaf[A->fclade[f] + g] != 0; }
};

// Event selection: r falls through the terms in the reference's order; the
// last term with a positive weight is kept for a draw that rounding pushes
// past the end (the host sampler's fallback).
struct Pick {
  double r;
  int n = 0, lastn = 0;
  St out[2], last[2];
  // true when the draw falls in this term
  __device__ bool take(double w, int k, St a, St b) {
    if (w > 0.0) {
      lastn = k;
      last[0] = a;
      last[1] = b;
    }
    r = __dsub_rn(r, w);
    if (r < 0.0) {
      n = lastn;
      out[0] = last[0];
      out[1] = last[1];
      return true;
    }
    return false;
  }
};

// One step from state s: 0, 1 or 2 next states in out; -1 when no event has
// a positive weight.
__device__ int step(const Fam& F, St s, DRng& rng, St* out) {
  const int e = s.e, g = s.g, t = s.t;
  const int4 mn = F.A->mnode[e];
  if (t == 1) {  // internode (src/track.jl:205-219)
    if (mn.x == WG_NODE_LEAF) return 0;
    Pick P;
    P.r = __dmul_rn(rng.uniform(), F.L(e, g, t));
    if (mn.x == WG_NODE_ROOT) {  // bifurcation, then loss (src/track.jl:233-250, 359-401)
      const int f = mn.y, h = mn.z;
      const int tf = F.nrow(f), th = F.nrow(h);
      const double eta = F.A->params[3 * F.A->NR + F.A->K], eps = F.eps_top(e);
      const double xi = __dsub_rn(1.0, __dmul_rn(__dsub_rn(1.0, eta), eps));
      const double cd = __ddiv_rn(__dmul_rn(xi, __dsub_rn(1.0, eta)), eta);
      const double cs = __ddiv_rn(__dmul_rn(eta, __dsub_rn(1.0, eps)), __dmul_rn(xi, xi));
      for (int64_t k = F.split0(g); k < F.split1(g); ++k) {
        const int a = F.A->g1[k], b = F.A->g2[k];
        const double p = F.A->sp[k];
        if (P.take(__dmul_rn(__dmul_rn(__dmul_rn(p, F.L(e, a, t)), F.L(e, b, t)), cd), 2, St{e, a, t}, St{e, b, t}))
          break;
        if (P.take(__dmul_rn(__dmul_rn(__dmul_rn(p, F.Ltop(f, a)), F.Ltop(h, b)), cs), 2, St{f, a, tf},
                   St{h, b, th}))
          break;
        if (P.take(__dmul_rn(__dmul_rn(__dmul_rn(p, F.Ltop(h, a)), F.Ltop(f, b)), cs), 2, St{h, a, th},
                   St{f, b, tf}))
          break;
      }
      if (P.r >= 0.0 && !P.take(__dmul_rn(__dmul_rn(F.Ltop(f, g), F.eps_top(h)), cs), 2, St{f, g, tf}, St{h, -1, 0}))
        P.take(__dmul_rn(__dmul_rn(F.Ltop(h, g), F.eps_top(f)), cs), 2, St{h, g, th}, St{f, -1, 0});
    } else if (mn.x == WG_NODE_WGD) {  // non-retention, then retention (src/track.jl:252-265, 333-357)
      const int f = mn.y, tf = F.nrow(f);
      const double q = F.A->params[3 * F.A->NR + e];
      const double w0 =
          __dmul_rn(__dadd_rn(__dsub_rn(1.0, q), __dmul_rn(__dmul_rn(2.0, q), F.eps_top(f))), F.Ltop(f, g));
      if (!P.take(w0, 1, St{f, g, tf}, St{0, 0, 0}))
        for (int64_t k = F.split0(g); k < F.split1(g); ++k) {
          const int a = F.A->g1[k], b = F.A->g2[k];
          const double w = __dmul_rn(__dmul_rn(__dmul_rn(q, F.A->sp[k]), F.Ltop(f, a)), F.Ltop(f, b));
          if (P.take(w, 2, St{f, a, tf}, St{f, b, tf})) break;
        }
    } else {  // speciation node: sploss, then speciation (src/track.jl:223-231, 283-331)
      const int f = mn.y, h = mn.z;
      const int tf = F.nrow(f), th = F.nrow(h);
      if (!P.take(__dmul_rn(F.Ltop(f, g), F.eps_top(h)), 2, St{f, g, tf}, St{h, -1, 0}) &&
          !P.take(__dmul_rn(F.Ltop(h, g), F.eps_top(f)), 2, St{h, g, th}, St{f, -1, 0}))
        for (int64_t k = F.split0(g); k < F.split1(g); ++k) {
          const int a = F.A->g1[k], b = F.A->g2[k];
          const double p = F.A->sp[k];
          if (P.take(__dmul_rn(__dmul_rn(p, F.Ltop(f, a)), F.Ltop(h, b)), 2, St{f, a, tf}, St{h, b, th})) break;
          if (P.take(__dmul_rn(__dmul_rn(p, F.Ltop(h, a)), F.Ltop(f, b)), 2, St{h, a, th}, St{f, b, tf})) break;
        }
    }
    if (P.r >= 0.0) {  // past the last term
      if (P.lastn == 0) return -1;
      P.n = P.lastn;
      P.out[0] = P.last[0];
      P.out[1] = P.last[1];
    }
    out[0] = P.out[0];
    out[1] = P.out[1];
    return P.n;
  }
  // intra-branch (src/track.jl:266-280)
  if (F.leafclade(g)) {
    out[0] = St{e, g, 1};
    return 1;
  }
  double r = __dmul_rn(rng.uniform(), F.L(e, g, t));
  r = __dsub_rn(r, __dmul_rn(F.phi(e, t), F.L(e, g, t - 1)));
  if (r < 0.0) {
    out[0] = St{e, g, t - 1};
    return 1;
  }
  const double ps = F.psi(e, t);
  Pick P;
  P.r = r;
  for (int64_t k = F.split0(g); k < F.split1(g); ++k) {
    const int a = F.A->g1[k], b = F.A->g2[k];
    const double w = __dmul_rn(__dmul_rn(__dmul_rn(F.A->sp[k], F.L(e, a, t - 1)), F.L(e, b, t - 1)), ps);
    if (P.take(w, 2, St{e, a, t - 1}, St{e, b, t - 1})) {
      out[0] = P.out[0];
      out[1] = P.out[1];
      return 2;
    }
  }
  if (P.lastn) {
    out[0] = P.last[0];
    out[1] = P.last[1];
    return 2;
  }
  out[0] = St{e, g, t - 1};
  return 1;
}

__global__ void __launch_bounds__(128) k_track(const TrackArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const int f = A.fam[i];
  Fam F{&A, f, A.fnclade[f], A.ftabs[f]};
  const int64_t base = A.cap_off[i];
  const int cap = (int)(A.cap_off[i + 1] - base);
  int4* nodes = A.nodes + base;
  int4* stack = A.stack + base;
  const int root = A.K - 1, ub = F.nc - 1;
  if (!(F.L(root, ub, 1) > 0.0)) {
    A.count[i] = kTrackNoLikelihood;
    return;
  }
  DRng rng(A.seed[i]);
  int cnt = 1, sp = 1;
  nodes[0] = make_int4(ub, root, 1, -1);
  stack[0] = make_int4(root, ub, 1, 0);
  while (sp > 0) {
    const int4 s = stack[--sp];
    if (s.y < 0) continue;  // a loss: its node was made when the state was entered
    St nx[2];
    const int k = step(F, St{s.x, s.y, s.z}, rng, nx);
    if (k < 0) {
      A.count[i] = kTrackNoEvent;
      return;
    }
    const int cur = s.w;
    for (int j = k - 1; j >= 0; --j) {  // next states in reverse: the host sampler's node order
      int node = cur;
      if (nx[j].g != nodes[cur].x || nx[j].e != nodes[cur].y) {
        if (cnt >= cap) {
          A.count[i] = kTrackOverflow;
          return;
        }
        node = cnt++;
        nodes[node] = make_int4(nx[j].g, nx[j].e, nx[j].t, cur);
      }
      if (sp >= cap) {
        A.count[i] = kTrackOverflow;
        return;
      }
      stack[sp++] = make_int4(nx[j].e, nx[j].g, nx[j].t, node);
    }
  }
  A.count[i] = cnt;
}

// Compaction: tree i's nodes to out + off[i] (one CTA per tree).
__global__ void k_track_compact(const int4* __restrict__ nodes, const int64_t* __restrict__ cap_off,
                                const int64_t* __restrict__ off, int4* __restrict__ out, int n) {
  const int i = blockIdx.x;
  if (i >= n) return;
  const int64_t m = off[i + 1] - off[i];
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) out[off[i] + j] = nodes[cap_off[i] + j];
}

}  // namespace

cudaError_t track_launch(const TrackArgs& A, cudaStream_t s) {
  if (A.n <= 0) return cudaSuccess;
  k_track<<<(A.n + 127) / 128, 128, 0, s>>>(A);
  return cudaGetLastError();
}

cudaError_t track_compact(const int4* nodes, const int64_t* cap_off, const int64_t* off, int4* out, int n,
                          cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_track_compact<<<n, 128, 0, s>>>(nodes, cap_off, off, out, n);
  return cudaGetLastError();
}

}  // namespace wg
