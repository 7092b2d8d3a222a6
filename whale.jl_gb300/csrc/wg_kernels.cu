// CUDA kernels (sm_103a) and the device-side C ABI of libwhalegpu.
//
// The DP (src/core.jl:83-199) runs per group of families, one CTA per group:
// for every species node in the reference order the CTA builds row 1 of the
// node's table from its children's top rows (leaf / speciation+loss / WGD
// retention+loss / root), then advances the rows of the branch,
//     ℓ[i, γ] = ϕ_i ℓ[i-1, γ] + ψ_i Σ_{(γ1,γ2,p) ∈ S(γ)} p ℓ[i-1, γ1] ℓ[i-1, γ2]
// (within_branch!/Πduplication, src/core.jl:121-128, :178-185), entirely in
// shared memory.  Each Σ over split triples is a host-scheduled sum program
// (see wg_pack.cpp).  Everything is FP64.
//
// The adjoint kernel walks the nodes in reverse and back-propagates
// ∂ Σ_f log L_f through the same rows (read back from the tables the forward
// stored), producing per-group adjoints of every slice-table entry [ε, ϕ, ψ],
// of q and of η; a second kernel sums them over groups in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>

#include "wg_internal.h"
#include "wg_nowhere.h"
#include "wg_track_dev.h"

using namespace wg;

namespace {

// ---------------------------------------------------------------------------
// device side
// ---------------------------------------------------------------------------
struct KArgs {
  const DGroup* groups;
  const DNode* nodes;
  const DEntry* entries;
  const int* meta;
  const DLevel* levels;
  const int* fam_idx;
  const int* fam_pos;
  const int4* mnode;     // kind, child0, child1, nrow
  const int* row_off;    // K + 1
  const double* leafp;   // K
  const double* params;  // eps | phi | psi (NR each) | q (K) | eta | ca | cb
  double* tops;
  double* tabs;
  double* bartops;
  double* logl;
  int K;
  int NR;
};

__device__ __forceinline__ const int2* meta2(const KArgs& A, int64_t off) {
  return reinterpret_cast<const int2*>(A.meta) + off;
}

// One sum program: lane executes entries [j * nt + lane], j < J.
__device__ __forceinline__ void run_prog(const DEntry* __restrict__ E, const DProg pr, int lane,
                                         const double* A, const double* B, double* part) {
  if (lane >= pr.nt) return;
  const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + pr.off) + lane;
  double acc = 0.0;
  for (int j = 0; j < pr.J; ++j, e += pr.nt) {
    const ulonglong2 raw = __ldg(e);
    const unsigned fl = (unsigned)(raw.x >> 48);
    if (fl & 1u) {
      const unsigned a = (unsigned)(raw.x & 0xFFFFu);
      const unsigned b = (unsigned)((raw.x >> 16) & 0xFFFFu);
      acc = fma(__longlong_as_double((long long)raw.y) * A[a], B[b], acc);
      if (fl & 2u) {
        part[(unsigned)((raw.x >> 32) & 0xFFFFu)] = acc;
        acc = 0.0;
      }
    }
  }
}

__device__ __forceinline__ double slot_sum(const double* part, int2 f) {
  double s = 0.0;
  for (int k = 0; k < f.y; ++k) s += part[f.x + k];
  return s;
}

__device__ __forceinline__ double eps_top(const KArgs& A, int k) {
  return A.params[A.row_off[k] + A.mnode[k].w - 1];
}

template <bool TABLES>
__global__ void __launch_bounds__(kNT) k_forward(const KArgs A) {
  extern __shared__ double sm[];
  const DGroup G = A.groups[blockIdx.x];
  const int tid = threadIdx.x;
  const int mw = G.maxw;
  double* const B0 = sm;
  double* const B1 = sm + mw;
  double* const Y = sm + 2 * mw;
  double* const part = sm + 3 * mw;
  const double* phi = A.params + A.NR;
  const double* psi = A.params + 2 * A.NR;
  const double* qv = A.params + 3 * A.NR;
  for (int k = 0; k < A.K; ++k) {
    const DNode& nd = A.nodes[G.node0 + k];
    const int4 mn = A.mnode[k];
    const int R = nd.width;
    const int roff = A.row_off[k];
    const int lane = (tid + 32 * (int)((blockIdx.x + k) & 3)) & (kNT - 1);
    double* cur = B0;
    double* nxt = B1;
    if (mn.x == WG_NODE_LEAF) {
      const int2* aux = meta2(A, nd.aux);
      const double lp = A.leafp[k];
      for (int c = tid; c < R; c += kNT) cur[c] = aux[c].x ? lp : 0.0;
    } else if (mn.x == WG_NODE_WGD) {
      const DNode& nc = A.nodes[G.node0 + mn.y];
      const double* top = A.tops + nc.top_off;
      for (int c = tid; c < R; c += kNT) nxt[c] = top[c];
      __syncthreads();
      run_prog(A.entries, nd.dup, lane, nxt, nxt, part);
      __syncthreads();
      const double q = qv[k];
      const double ef = eps_top(A, mn.y);
      const int2* fin = meta2(A, nd.fin_dup);
      for (int c = tid; c < R; c += kNT) {
        const double x = nxt[c];
        cur[c] = q * slot_sum(part, fin[c]) + ((1.0 - q) * x + 2.0 * q * ef * x);
      }
    } else {
      const DNode& na = A.nodes[G.node0 + mn.y];
      const DNode& nb = A.nodes[G.node0 + mn.z];
      const double* ta = A.tops + na.top_off;
      const double* tb = A.tops + nb.top_off;
      for (int c = tid; c < na.width; c += kNT) nxt[c] = ta[c];
      for (int c = tid; c < nb.width; c += kNT) Y[c] = tb[c];
      __syncthreads();
      run_prog(A.entries, nd.r1, lane, nxt, Y, part);
      __syncthreads();
      const double ea = eps_top(A, mn.y), eb = eps_top(A, mn.z);
      const int2* fin = meta2(A, nd.fin_r1);
      const int2* aux = meta2(A, nd.aux);
      for (int c = tid; c < R; c += kNT) {
        const int2 l = aux[c];
        const double la = l.x >= 0 ? nxt[l.x] : 0.0;
        const double lb = l.y >= 0 ? Y[l.y] : 0.0;
        cur[c] = slot_sum(part, fin[c]) + (la * eb + lb * ea);
      }
      if (mn.x == WG_NODE_ROOT) {
        // whaleroot! (src/core.jl:130-149): ℓ[γ] = A·Πroot(γ) + B·(Πspec + Πloss),
        // Πroot reading smaller clades of the same row: level by level.
        __syncthreads();
        const double eta = A.params[3 * A.NR + A.K];
        const double er = eps_top(A, k);
        const double xi = 1.0 - (1.0 - eta) * er;
        const double ca = (1.0 - eta) * xi / eta;
        const double cb = eta * (1.0 - er) / (xi * xi);
        const int2* finl = meta2(A, nd.fin_lvl);
        const int* lc = A.meta + nd.lvl_clades;
        for (int L = 0; L < nd.nlvl; ++L) {
          const DLevel lv = A.levels[nd.lvl + L];
          if (lv.prog.J > 0) {
            run_prog(A.entries, lv.prog, lane, cur, cur, part);
            __syncthreads();
          }
          for (int i = lv.begin + tid; i < lv.end; i += kNT) {
            const int c = lc[i];
            cur[c] = fma(ca, slot_sum(part, finl[c]), cb * cur[c]);
          }
          __syncthreads();
        }
      }
    }
    __syncthreads();
    if (TABLES) {
      double* t0 = A.tabs + nd.tab_off;
      for (int c = tid; c < R; c += kNT) t0[c] = cur[c];
    }
    if (mn.x != WG_NODE_ROOT) {
      const int2* fin = meta2(A, nd.fin_dup);
      for (int r = 1; r < mn.w; ++r) {
        const double ph = phi[roff + r], ps = psi[roff + r];
        run_prog(A.entries, nd.dup, lane, cur, cur, part);
        __syncthreads();
        double* tr = TABLES ? A.tabs + nd.tab_off + (int64_t)r * R : nullptr;
        for (int c = tid; c < R; c += kNT) {
          const double v = fma(ps, slot_sum(part, fin[c]), ph * cur[c]);
          nxt[c] = v;
          if (TABLES) tr[c] = v;
        }
        __syncthreads();
        double* t = cur;
        cur = nxt;
        nxt = t;
      }
    }
    double* top = A.tops + nd.top_off;
    for (int c = tid; c < R; c += kNT) top[c] = cur[c];
    __syncthreads();
  }
  // log L per family (src/core.jl:35-36): the ubiquitous clade of the root row
  for (int f = tid; f < G.n_fam; f += kNT) {
    const double L = B0[A.fam_pos[G.fam0 + f]];
    A.logl[A.fam_idx[G.fam0 + f]] = L > 0.0 ? log(L) : -INFINITY;
  }
}

// FP64 FMA throughput probe: 8 independent register-resident DFMA chains per
// thread; 2 flops per DFMA.
__global__ void __launch_bounds__(256) k_fp64_probe(double* out, int iters, double a, double b) {
  double x[8];
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
  for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 12345.678) out[0] = s;  // keeps the loop alive; never true for the inputs used
}

// ===========================================================================
// Batched kernels: one CTA per (species node, family group) task; the tasks
// of one height level of the species tree run in one launch.
// ===========================================================================

struct KArgs2 {
  const DTask* tasks;
  const DEntry* entries;
  const int* meta;
  const int64_t* gmap;
  const DProg2* progs;
  const int4* mnode;     // kind, child0, child1, nrow
  const int* row_off;
  const double* leafp;
  const double* params;  // eps | phi | psi (NR each) | q (K) | eta | ca | cb
  double* tops;
  double* tabs;
  double* bartops;
  double* gout;
  double* logl;
  double* scratch;  // working rows of the tasks too wide for shared memory
  const double* famw;  // adjoint seed weight per family (null: 1)
  int* err;            // error bits of the evaluation (bit 1: a bulk-copy wait ran out)
  int NR, K;
};

struct Raw {
  unsigned f0, f1, f2, opc, kind;
  double p;
};

__device__ __forceinline__ Raw decode(const ulonglong2 r) {
  Raw x;
  x.f0 = (unsigned)(r.x & 0xFFFFu);
  x.f1 = (unsigned)((r.x >> 16) & 0xFFFFu);
  x.f2 = (unsigned)((r.x >> 32) & 0xFFFFu);
  x.opc = (unsigned)((r.x >> 48) & 0xFFu);
  x.kind = (unsigned)(r.x >> 56);
  x.p = __longlong_as_double((long long)r.y);
  return x;
}

// 1-D bulk copies (the TMA engine) from this GPU's memory into the CTA's own
// shared memory, each completing on an mbarrier with its byte count.  Both
// addresses are 16-byte aligned and the size a multiple of 16.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* mb) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mb)) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* mb) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(mb)) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// shared memory the generic proxy touched, ordered before the bulk copies' writes
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_row_g2s(void* dst, const void* src, unsigned bytes, uint64_t* mb) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(mb))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mb, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for a phase of an mbarrier; false (and the error bit 2 set)
// when the poll limit ran out.
constexpr int kMbarPolls = 1 << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* mb, unsigned parity, int* err) {
  for (int i = 0; i < kMbarPolls; ++i)
    if (mbar_try_wait(mb, parity)) return true;
  if (err) atomicOr(err, 2);
  return false;
}

// L1 prefetch of a lane's entries of a program (and of the thread's first
// combine entry), issued at task start so that the phases that read them
// later do not each wait a full memory latency.
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void prefetch_prog(const DEntry* __restrict__ E, const DProg2& pr, int lane) {
  if (lane < pr.nt)
    for (int j = 0; j < pr.J; ++j) prefetch_l1(E + pr.off + (size_t)j * pr.nt + lane);
  if ((int)threadIdx.x < pr.ncomb) prefetch_l1(E + pr.comb + threadIdx.x);
}

// L2 prefetch of a root task's level programs: the same-row levels run one
// after another with a barrier between them and each loads the next level's
// entries, so a DRAM latency per level would otherwise sit on the chain.  The
// levels' entries (lane entries then combine entries, level after level) and
// their descriptors are each one contiguous range; warp 0 issues bulk L2
// prefetches of 16 KB pieces of both.
__device__ __forceinline__ void bulk_prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
static_assert(sizeof(DEntry) == 16 && sizeof(DProg2) % 16 == 0, "bulk prefetch pieces are multiples of 16 bytes");
__device__ __forceinline__ void prefetch_levels(const DEntry* __restrict__ E, const DProg2* __restrict__ progs, int nl) {
  if (nl <= 0 || threadIdx.x >= 32) return;
  constexpr int64_t kPiece = 16384;
  const DProg2 a = progs[0], b = progs[nl - 1];
  const char* lo = reinterpret_cast<const char*>(E + a.off);
  const int64_t bytes = (b.comb + b.ncomb - a.off) * (int64_t)sizeof(DEntry);
  for (int64_t o = (int64_t)threadIdx.x * kPiece; o < bytes; o += 32 * kPiece)
    bulk_prefetch_l2(lo + o, (uint32_t)min(kPiece, bytes - o));
  const int64_t dbytes = (int64_t)nl * (int64_t)sizeof(DProg2);
  for (int64_t o = (int64_t)threadIdx.x * kPiece; o < dbytes; o += 32 * kPiece)
    bulk_prefetch_l2(reinterpret_cast<const char*>(progs) + o, (uint32_t)min(kPiece, dbytes - o));
}

// General lane program: products accumulate, finalize ops call fin().
// Entries are fetched four at a time ahead of their use.
template <class Fin>
__device__ __forceinline__ void run_any(const DEntry* __restrict__ E, const DProg2& pr, int lane, const double* A,
                                        const double* B, double* part, Fin fin) {
  if (lane >= pr.nt) return;
  const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + pr.off) + lane;
  const ulonglong2 nop = make_ulonglong2(0, (uint64_t)op::NOP << 48);
  double acc = 0.0;
  for (int j0 = 0; j0 < pr.J; j0 += 4) {
    ulonglong2 r[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) r[u] = j0 + u < pr.J ? __ldg(e + (size_t)(j0 + u) * pr.nt) : nop;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const Raw x = decode(r[u]);
      if (x.opc == op::PROD) {
        acc = fma(x.p * A[x.f0], B[x.f1], acc);
      } else if (x.opc == op::FIN_PART) {
        part[x.f2] = acc;
        acc = 0.0;
      } else if (x.opc != op::NOP) {
        fin(x.opc, x.f0, x.f1, x.f2, acc);
        acc = 0.0;
      }
    }
  }
}

// One combine entry: the partial sums of a split clade (two interleaved
// chains), handed to fin().
template <class Fin>
__device__ __forceinline__ void comb_one(const ulonglong2 raw, const double* part, Fin fin) {
  const Raw x = decode(raw);
  const unsigned s0 = (unsigned)(raw.y & 0xFFFFFFFFu), n = (unsigned)(raw.y >> 32);
  double s = part[s0], t = 0.0;
  unsigned k = 1;
  for (; k + 1 < n; k += 2) {
    s += part[s0 + k];
    t += part[s0 + k + 1];
  }
  if (k < n) s += part[s0 + k];
  fin(x.opc, x.f0, x.f1, x.f2, s + t);
}

// The first pr.nbig combine entries (split clades with many partial sums):
// one warp each, lanes summing strided partials (two chains), then
// a shuffle tree; lane 0 hands the sum to fin().  tix: the thread's index
// among the NTG threads that share the pass.
template <int NTG, class Fin>
__device__ __forceinline__ void comb_big(const DEntry* __restrict__ E, const DProg2& pr, const double* part, Fin& fin,
                                         int tix) {
  const int l = tix & 31;
  for (int i = tix >> 5; i < (int)pr.nbig; i += NTG / 32) {
    const ulonglong2 raw = __ldg(reinterpret_cast<const ulonglong2*>(E + pr.comb + i));
    const unsigned s0 = (unsigned)(raw.y & 0xFFFFFFFFu), n = (unsigned)(raw.y >> 32);
    double s = 0.0, t = 0.0;
    unsigned k = (unsigned)l;
    for (; k + 32 < n; k += 64) {
      s += part[s0 + k];
      t += part[s0 + k + 32];
    }
    if (k < n) s += part[s0 + k];
    s += t;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (l == 0) {
      const Raw x = decode(raw);
      fin(x.opc, x.f0, x.f1, x.f2, s);
    }
  }
}

// Combine pass for split clades: with BIG the first pr.nbig a warp each,
// the rest one thread each.  (Adjoint programs have no warp-combined
// entries: their passes leave the warp code out of the row loops.)
template <int NT, bool BIG, class Fin>
__device__ __forceinline__ void run_comb(const DEntry* __restrict__ E, const DProg2& pr, const double* part,
                                         Fin fin) {
  if constexpr (BIG) comb_big<NT>(E, pr, part, fin, (int)threadIdx.x);
  for (int i = pr.nbig + threadIdx.x; i < pr.ncomb; i += NT)
    comb_one(__ldg(reinterpret_cast<const ulonglong2*>(E + pr.comb + i)), part, fin);
}

// A thread's first one-thread combine entry of a program, held in registers
// while the program repeats (rows of a branch) or runs later (next root
// level).
struct CombReg {
  ulonglong2 raw;
};
// tix: the thread's index among the NT threads that share the program.
__device__ __forceinline__ CombReg load_comb(const DEntry* __restrict__ E, const DProg2& pr,
                                             int tix = (int)threadIdx.x) {
  CombReg c;
  const int i = pr.nbig + tix;
  c.raw = i < pr.ncomb ? __ldg(reinterpret_cast<const ulonglong2*>(E + pr.comb + i)) : make_ulonglong2(0, 0);
  return c;
}
template <int NT, bool BIG, class Fin>
__device__ __forceinline__ void run_comb_reg(const DEntry* __restrict__ E, const DProg2& pr, const CombReg& cr,
                                             const double* part, Fin fin, int tix = (int)threadIdx.x) {
  if constexpr (BIG) comb_big<NT>(E, pr, part, fin, tix);
  const int i0 = pr.nbig + tix;
  if (i0 < pr.ncomb) comb_one(cr.raw, part, fin);
  for (int i = i0 + NT; i < pr.ncomb; i += NT)
    comb_one(__ldg(reinterpret_cast<const ulonglong2*>(E + pr.comb + i)), part, fin);
}

// One entry of a lane program, by its column's kind (the same for the warp's
// 32 lanes, so a warp takes one branch).  PROD column: acc = fma(p·A[f0],
// B[f1], acc) on lanes holding a product (idle lanes keep acc); FIN column:
// the finalize op FIN (entries with f0 = f1 = c) v = fma(ψ, acc, ϕ·A[c]),
// handed to onfin(c, v, acc), or FIN_PART part[f2] = acc; PART column:
// partial sums only.  Every finalize column clears acc.
template <unsigned FIN, class OnFin>
__device__ __forceinline__ void lane_step(unsigned kind, unsigned f0, unsigned f1, unsigned f2, unsigned opc,
                                          double p, const double* A, const double* B, double* part, double ph,
                                          double ps, OnFin& onfin, double& acc) {
  if (kind == col::PROD) {
    const double v = fma(p * A[f0], B[f1], acc);
    acc = opc == op::PROD ? v : acc;
  } else if (kind == col::FIN) {
    const double v = fma(ps, acc, ph * A[f0]);
    if (opc == FIN) onfin(f0, v, acc);
    else if (opc == op::FIN_PART) part[f2] = acc;
    acc = 0.0;
  } else if (kind == col::PART) {
    if (opc == op::FIN_PART) part[f2] = acc;
    acc = 0.0;
  }
}

// Entries j0..J-1 of a lane's program streamed from memory (e: the lane's
// entry 0, nt: the program's lanes), four at a time with the next four's
// loads in flight while the four before them run.
template <unsigned FIN, class OnFin>
__device__ __forceinline__ void stream_steps(const ulonglong2* __restrict__ e, int nt, int j0, int J, const double* A,
                                             const double* B, double* part, double ph, double ps, OnFin& onfin,
                                             double& acc) {
  const ulonglong2 nop = make_ulonglong2(0, 0);  // column kind NOP: no work
  ulonglong2 c[4], nx[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) c[u] = j0 + u < J ? __ldg(e + (size_t)(j0 + u) * nt) : nop;
  for (int j = j0; j < J; j += 4) {
#pragma unroll
    for (int u = 0; u < 4; ++u) nx[u] = j + 4 + u < J ? __ldg(e + (size_t)(j + 4 + u) * nt) : nop;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const Raw x = decode(c[u]);
      lane_step<FIN>(x.kind, x.f0, x.f1, x.f2, x.opc, x.p, A, B, part, ph, ps, onfin, acc);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) c[u] = nx[u];
  }
}

// Row program of the branch recursion streamed from memory (programs deeper
// than the register-resident instantiations): entries as in lane_step.
//   PROD:    acc = fma(p·cur[a], cur[b], acc)
//   FIN_DUP: out[c] = fma(ψ, acc, ϕ·cur[c])     (entry has a = b = c)
template <bool STORE>
__device__ __forceinline__ void run_rows(const DEntry* __restrict__ E, const DProg2& pr, int lane, const double* cur,
                                         double* out, double* part, double ph, double ps, double* tab) {
  if (lane >= pr.nt) return;
  const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + pr.off) + lane;
  auto onfin = [&](unsigned c, double v, double) {
    out[c] = v;
    if (STORE) tab[c] = v;
  };
  double acc = 0.0;
  stream_steps<op::FIN_DUP>(e, pr.nt, 0, pr.J, cur, cur, part, ph, ps, onfin, acc);
}

// A lane's share of a row program held in registers for all rows of a node:
// (f0 | f1 << 16, f2 | op << 16 | column kind << 24, p) per iteration.  Rows
// then issue no entry loads; operand loads of every iteration are known up
// front.
template <int MAXJ>
struct LaneProg {
  uint32_t ab[MAXJ];
  uint32_t om[MAXJ];
  double p[MAXJ];
  int J;
};

template <int MAXJ>
__device__ __forceinline__ void load_lane_prog(const DEntry* __restrict__ E, const DProg2& pr, int lane,
                                               LaneProg<MAXJ>& lp) {
  lp.J = lane < pr.nt ? pr.J : 0;
  const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + pr.off) + lane;
#pragma unroll
  for (int j = 0; j < MAXJ; ++j) {
    if (j < lp.J) {
      const ulonglong2 r = __ldg(e + (size_t)j * pr.nt);
      lp.ab[j] = (uint32_t)(r.x & 0xFFFFFFFFu);
      lp.om[j] = (uint32_t)((r.x >> 32) & 0xFFFFu) | ((uint32_t)((r.x >> 48) & 0xFFu) << 16) |
                 ((uint32_t)(r.x >> 56) << 24);
      lp.p[j] = __longlong_as_double((long long)r.y);
    } else {
      lp.ab[j] = 0;
      lp.om[j] = (uint32_t)op::NOP << 16 | (uint32_t)col::NOP << 24;
      lp.p[j] = 0.0;
    }
  }
}

// The register-resident entries of a lane program (the first min(J, MAXJ)).
template <int MAXJ, unsigned FIN, class OnFin>
__device__ __forceinline__ void reg_steps(const LaneProg<MAXJ>& lp, const double* A, const double* B, double* part,
                                          double ph, double ps, OnFin& onfin, double& acc) {
#pragma unroll
  for (int j = 0; j < MAXJ; ++j)
    if (j < lp.J)
      lane_step<FIN>(lp.om[j] >> 24, lp.ab[j] & 0xFFFFu, lp.ab[j] >> 16, lp.om[j] & 0xFFFFu, (lp.om[j] >> 16) & 0xFFu,
                     lp.p[j], A, B, part, ph, ps, onfin, acc);
}

// One row from a register-resident program.
template <int MAXJ, unsigned FIN, class OnFin>
__device__ __forceinline__ void rows_reg(const LaneProg<MAXJ>& lp, const double* A, const double* B, double* part,
                                         double ph, double ps, OnFin onfin) {
  double acc = 0.0;
  reg_steps<MAXJ, FIN>(lp, A, B, part, ph, ps, onfin, acc);
}

// A lane's first MAXJ entries of a level program as loaded (decoded where
// they are used): the loads of the next level are issued while the current
// one runs and nothing waits for them until that level starts.
template <int MAXJ>
struct LaneRaw {
  ulonglong2 r[MAXJ];
  int J;
};
template <int MAXJ>
__device__ __forceinline__ void load_lane_raw(const DEntry* __restrict__ E, const DProg2& pr, int lane,
                                              LaneRaw<MAXJ>& lr) {
  lr.J = lane < pr.nt ? pr.J : 0;
  const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + pr.off) + lane;
#pragma unroll
  for (int j = 0; j < MAXJ; ++j)
    lr.r[j] = j < lr.J ? __ldg(e + (size_t)j * pr.nt) : make_ulonglong2(0, (uint64_t)op::NOP << 48);
}
template <int MAXJ, unsigned FIN, class OnFin>
__device__ __forceinline__ void raw_steps(const LaneRaw<MAXJ>& lr, const double* A, const double* B, double* part,
                                          double ph, double ps, OnFin& onfin, double& acc) {
#pragma unroll
  for (int j = 0; j < MAXJ; ++j)
    if (j < lr.J) {
      const Raw x = decode(lr.r[j]);
      lane_step<FIN>(x.kind, x.f0, x.f1, x.f2, x.opc, x.p, A, B, part, ph, ps, onfin, acc);
    }
}

// The same-row levels of a root row (Πroot), run by the NTG threads of the
// CTA for all the task's families in lock step: level after level with a
// barrier between them; entries as in lane_step (products and the
// finalize op FIN).  Levels are short and latency-bound, so each level's
// first kLvlJ entries per lane and its first combine entry per thread are
// loaded while the level before it runs (held as loaded, decoded at use) and
// the descriptor two levels ahead; entries past kLvlJ are prefetched to L1
// then.  comb(opc, c, fa, fb, s) finishes split clades after a barrier.
// wl: lane in the program, tix: thread index among the NTG.
constexpr int kLvlJ = 4;
template <int NTG, bool REVERSE, unsigned FIN, class OnFin, class Comb>
__device__ __forceinline__ void chain_levels(const DEntry* __restrict__ E, const DProg2* __restrict__ progs, int nlvl,
                                             int wl, int tix, const double* A, const double* B, double* part,
                                             double ph, double ps, OnFin onfin, Comb comb) {
  // Threads a level's work occupies: its lanes, its one-thread combines and
  // its warp combines.  wl and tix are unrotated (lane l is thread l), so a
  // level within 32 threads is warp 0's alone, and a barrier between two such
  // levels (or inside one) is that warp's; the other warps pass them and wait
  // at the next CTA barrier, which every thread reaches in the same order.
  auto width = [](const DProg2& p) {
    return max(max(p.nt, p.ncomb - (int)p.nbig), 32 * min((int)p.nbig, NTG / 32));
  };
  auto sync = [](bool narrow) {
    if (NTG == 32 || narrow) __syncwarp();
    else __syncthreads();
  };
  if (nlvl <= 0) return;
  auto at = [&](int i) { return REVERSE ? nlvl - 1 - i : i; };
  DProg2 cur = progs[at(0)];
  DProg2 nxt = nlvl > 1 ? progs[at(1)] : cur;
  LaneRaw<kLvlJ> lp;
  load_lane_raw<kLvlJ>(E, cur, wl, lp);
  CombReg cr = load_comb(E, cur, tix);
  for (int i = 0; i < nlvl; ++i) {
    const bool more = i + 1 < nlvl;
    LaneRaw<kLvlJ> lpn;
    CombReg crn = cr;
    DProg2 nn = nxt;
    if (more) {
      load_lane_raw<kLvlJ>(E, nxt, wl, lpn);
      crn = load_comb(E, nxt, tix);
      if (i + 2 < nlvl) nn = progs[at(i + 2)];
      if (wl < nxt.nt)  // the next level's entries past the registers, to L1
        for (int j = kLvlJ; j < nxt.J; ++j) prefetch_l1(E + nxt.off + (size_t)j * nxt.nt + wl);
    }
    if (wl < cur.nt) {
      double acc = 0.0;
      raw_steps<kLvlJ, FIN>(lp, A, B, part, ph, ps, onfin, acc);
      // (one entry at a time past the registers: the root kernels' register
      // budget has no room for a streaming window)
      const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + cur.off) + wl;
      for (int j = kLvlJ; j < cur.J; ++j) {
        const Raw x = decode(__ldg(e + (size_t)j * cur.nt));
        lane_step<FIN>(x.kind, x.f0, x.f1, x.f2, x.opc, x.p, A, B, part, ph, ps, onfin, acc);
      }
    }
    const bool narrow = width(cur) <= 32;
    if (cur.ncomb) {
      sync(narrow);
      run_comb_reg<NTG, !REVERSE>(E, cur, cr, part, comb, tix);
    }
    sync(narrow && more && width(nxt) <= 32);  // (the last level ends on a CTA barrier)
    if (more) {
      cur = nxt;
      nxt = nn;
      lp = lpn;
      cr = crn;
    }
  }
}

__device__ __forceinline__ double eps_top2(const KArgs2& A, int k) {
  return A.params[A.row_off[k] + A.mnode[k].w - 1];
}

// Rows 1..n-1 of a branch with the lane program in registers: J is the
// instantiated depth, the program's own depth (lp.J <= J) bounds the
// iterations.  cur/nxt are swapped row by row.
template <int NT, bool TABLES, int J>
__device__ __forceinline__ void fwd_rows(const DEntry* __restrict__ E, const DTask& T, int lane, int n, int R,
                                         const double* phs, const double* pss, double*& cur, double*& nxt,
                                         double* part, double* tab0) {
  const DProg2 dup = T.dup;  // held in registers: the rows store to global memory
  LaneProg<J> lp;
  load_lane_prog<J>(E, dup, lane, lp);
  const CombReg cr = load_comb(E, dup);
  const bool active = lane < dup.nt;
  for (int r = 1; r < n; ++r) {
    const double ph = phs[r], ps = pss[r];
    double* tr = TABLES ? tab0 + (int64_t)r * R : nullptr;
    double* o = nxt;
    if (active)
      rows_reg<J, op::FIN_DUP>(lp, cur, cur, part, ph, ps, [&](unsigned c, double v, double) {
        o[c] = v;
        if (TABLES) tr[c] = v;
      });
    if (dup.ncomb) {
      __syncthreads();
      const double* cc = cur;
      run_comb_reg<NT, true>(E, dup, cr, part, [&](unsigned, unsigned c, unsigned, unsigned, double s) {
        const double v = fma(ps, s, ph * cc[c]);
        o[c] = v;
        if (TABLES) tr[c] = v;
      });
    }
    __syncthreads();
    double* t = cur;
    cur = nxt;
    nxt = t;
  }
}

template <int NT, bool TABLES>
__device__ __forceinline__ void fwd_rows_generic(const DEntry* __restrict__ E, const DTask& T, int lane, int n, int R,
                                                 const double* phs, const double* pss, double*& cur, double*& nxt,
                                                 double* part, double* tab0) {
  const DProg2 dup = T.dup;
  const CombReg cr = load_comb(E, dup);
  for (int r = 1; r < n; ++r) {
    const double ph = phs[r], ps = pss[r];
    double* tr = TABLES ? tab0 + (int64_t)r * R : nullptr;
    run_rows<TABLES>(E, dup, lane, cur, nxt, part, ph, ps, tr);
    if (dup.ncomb) {
      __syncthreads();
      const double* cc = cur;
      double* o = nxt;
      run_comb_reg<NT, true>(E, dup, cr, part, [&](unsigned, unsigned c, unsigned, unsigned, double s) {
        const double v = fma(ps, s, ph * cc[c]);
        o[c] = v;
        if (TABLES) tr[c] = v;
      });
    }
    __syncthreads();
    double* t = cur;
    cur = nxt;
    nxt = t;
  }
}

// Row loops are instantiated for a few program depths only (a program of
// depth j runs in the smallest instantiation J >= j; the lanes' padding
// iterations are skipped by a CTA-uniform test): fewer copies of the
// unrolled loops keep the kernels' instruction footprint small (measured:
// steps of 2 for the forward rows and 4 for the adjoint rows beat every
// depth in its own copy by ~5% per evaluation).
constexpr int kFwdJStep = 2, kAdjJStep = 4;

template <int NT, bool TABLES, int J = kFwdJStep>
__device__ __forceinline__ bool fwd_rows_dispatch(int j, const DEntry* __restrict__ E, const DTask& T, int lane, int n,
                                                  int R, const double* phs, const double* pss, double*& cur,
                                                  double*& nxt, double* part, double* tab0) {
  constexpr int MAXJ = NT == kNT2L ? 8 : 12;
  if constexpr (J > MAXJ) {
    return false;
  } else {
    constexpr int NEXT = (J + kFwdJStep > MAXJ && J < MAXJ) ? MAXJ : J + kFwdJStep;
    if (j <= J) {
      fwd_rows<NT, TABLES, J>(E, T, lane, n, R, phs, pss, cur, nxt, part, tab0);
      return true;
    }
    return fwd_rows_dispatch<NT, TABLES, NEXT>(j, E, T, lane, n, R, phs, pss, cur, nxt, part, tab0);
  }
}

// Top rows (forward) and their adjoints (reverse) written by other CTAs of
// the same launch are read through L2 only (ld.global.cg): the SM's L1 is not
// coherent with other SMs' stores and may hold an older copy of the line.
template <bool CG>
__device__ __forceinline__ double ld_shared_row(const double* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}

// dst[i] = src[gm[i]] for i < n over the CTA's NT threads: each gather is two
// dependent global loads, so every thread has four indices and then four
// values in flight at a time rather than one of each.
template <int NT, bool CG>
__device__ __forceinline__ void gather_rows(double* dst, const double* src, const int64_t* __restrict__ gm, int n) {
  for (int i0 = (int)threadIdx.x; i0 < n; i0 += 4 * NT) {
    int64_t g[4];
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) g[u] = i0 + u * NT < n ? __ldg(gm + i0 + u * NT) : 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = i0 + u * NT < n ? ld_shared_row<CG>(src + g[u]) : 0.0;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + u * NT < n) dst[i0 + u * NT] = v[u];
  }
}

// One forward task (one species node for a group of families).  rot rotates
// the lane assignment by warps (spreads the lanes' programs over the warps of
// successive CTAs); CG: the children's top rows were written in this launch.
template <bool TABLES, int NT, bool ROOT, bool GLOBAL, bool CG>
__device__ __forceinline__ void fwd_task(const KArgs2& A, const DTask& T, int rot, double* smem_dyn) {
  double* const sm = GLOBAL ? A.scratch + T.scratch : smem_dyn;
  const int k = T.node;
  const int4 mn = A.mnode[k];
  const int R = T.width;
  const int W2 = (max(R, T.wa + T.wb) + 1) & ~1;  // even: 16-byte aligned row buffers
  const int tid = threadIdx.x;
  const int lane = (tid + 32 * (int)(rot & (NT / 32 - 1))) & (NT - 1);
  double* cur = sm;
  double* nxt = sm + W2;
  double* part = sm + 2 * W2;
  const int roff = A.row_off[k];
  const int NR = A.NR;
  const DEntry* E = A.entries;
  if (!ROOT) {
    prefetch_prog(E, T.dup, lane);
    prefetch_prog(E, T.init, lane);
    for (int r = tid; r < mn.w; r += NT) {
      prefetch_l1(A.params + NR + roff + r);
      prefetch_l1(A.params + 2 * NR + roff + r);
    }
  } else {
    prefetch_levels(E, A.progs + T.lvl, T.nlvl);
    prefetch_prog(E, T.init, lane);
  }
  if (!ROOT && mn.x == WG_NODE_LEAF) {
    const int* aux = A.meta + T.aux;
    const double lp = A.leafp[k];
    for (int c = tid; c < R; c += NT) cur[c] = aux[c] ? lp : 0.0;
  } else {
    const int64_t* gm = A.gmap + T.gmap;
    gather_rows<NT, CG>(nxt, A.tops, gm, T.wa + T.wb);
    __syncthreads();
    const double* X = nxt;
    const double* Y = nxt + T.wa;
    if (!ROOT && mn.x == WG_NODE_WGD) {
      const double q = A.params[3 * NR + k];
      const double ef = eps_top2(A, mn.y);
      auto fin = [&](unsigned, unsigned c, unsigned fa, unsigned, double acc) {
        const double x = X[fa];
        cur[c] = q * acc + ((1.0 - q) * x + 2.0 * q * ef * x);
      };
      run_any(E, T.init, lane, X, X, part, fin);
      if (T.init.ncomb) {
        __syncthreads();
        run_comb<NT, true>(E, T.init, part, fin);
      }
    } else {
      const double ea = eps_top2(A, mn.y), eb = eps_top2(A, mn.z);
      auto fin = [&](unsigned, unsigned c, unsigned fa, unsigned fb, double acc) {
        const double la = fa != 0xFFFFu ? X[fa] : 0.0;
        const double lb = fb != 0xFFFFu ? Y[fb] : 0.0;
        cur[c] = acc + (la * eb + lb * ea);
      };
      run_any(E, T.init, lane, X, Y, part, fin);
      if (T.init.ncomb) {
        __syncthreads();
        run_comb<NT, true>(E, T.init, part, fin);
      }
      if (ROOT) {
        // whaleroot! (src/core.jl:130-149), Πroot over smaller clades of the
        // same row: level by level, in place
        __syncthreads();
        const double ca = A.params[3 * NR + A.K + 1], cb = A.params[3 * NR + A.K + 2];
        auto lcomb = [&](unsigned, unsigned c, unsigned, unsigned, double acc) { cur[c] = fma(ca, acc, cb * cur[c]); };
        auto lfin = [&](unsigned c, double v, double) { cur[c] = v; };
        chain_levels<NT, false, op::FIN_LVL>(E, A.progs + T.lvl, T.nlvl, tid, tid, cur, cur, part, cb, ca, lfin,
                                             lcomb);
      }
    }
  }
  __syncthreads();
  if (TABLES)
    for (int c = tid; c < R; c += NT) A.tabs[T.tab + c] = cur[c];
  if (!ROOT && mn.w > 1) {
    double* phs = part + T.nslot_max;  // ϕ, ψ of this branch's rows
    double* pss = phs + mn.w;
    for (int r = tid; r < mn.w; r += NT) {
      phs[r] = A.params[NR + roff + r];
      pss[r] = A.params[2 * NR + roff + r];
    }
    __syncthreads();
    double* tab0 = TABLES ? A.tabs + T.tab : nullptr;
    // (the row loops use the width only as the tables' row stride)
    if (!fwd_rows_dispatch<NT, TABLES>(T.dup.J, E, T, lane, mn.w, T.tstride, phs, pss, cur, nxt, part, tab0))
      fwd_rows_generic<NT, TABLES>(E, T, lane, mn.w, T.tstride, phs, pss, cur, nxt, part, tab0);
  }
  double* top = A.tops + T.top;
  for (int c = tid; c < R; c += NT) top[c] = cur[c];
  if (ROOT) {
    const int2* fam = reinterpret_cast<const int2*>(A.meta) + T.fam;
    for (int f = tid; f < T.nfam; f += NT) {
      const int2 fp = fam[f];
      const double L = cur[fp.y];
      A.logl[fp.x] = L > 0.0 ? log(L) : -INFINITY;
    }
  }
}

// ROOT: the launch of the top level, whose tasks are all root tasks; the other
// launches hold no root task.  Separate instantiations keep the root-row
// machinery out of the register budget of the branch kernels.
// GLOBAL: the tasks of the launch keep their working rows in device memory
// (A.scratch + T.scratch, L2-resident) because they do not fit in shared
// memory; the code is otherwise the same.
template <bool TABLES, int NT, bool ROOT = false, bool GLOBAL = false>
__global__ void __launch_bounds__(NT) k_fwd2(const KArgs2 A, const int* __restrict__ list) {
  extern __shared__ __align__(128) double smem_dyn[];
  fwd_task<TABLES, NT, ROOT, GLOBAL, false>(A, A.tasks[list[blockIdx.x]], (int)blockIdx.x, smem_dyn);
}

// ---- adjoint helpers -------------------------------------------------------
// Warp reduce-scatter of 16 values per lane (v[0..7] and w[0..7]): afterwards
// the lanes with bit 0 clear hold the warp sum of value index idx(lane).
__device__ __forceinline__ double reduce_scatter16(double (&v)[8], double (&w)[8], int lane, int& idx) {
  const unsigned FULL = 0xffffffffu;
  double a[8];
  const bool hi16 = lane & 16;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double send = hi16 ? v[i] : w[i];
    const double keep = hi16 ? w[i] : v[i];
    a[i] = keep + __shfl_xor_sync(FULL, send, 16);
  }
  const bool hi8 = lane & 8;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double send = hi8 ? a[i] : a[i + 4];
    const double keep = hi8 ? a[i + 4] : a[i];
    a[i] = keep + __shfl_xor_sync(FULL, send, 8);
  }
  const bool hi4 = lane & 4;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double send = hi4 ? a[i] : a[i + 2];
    const double keep = hi4 ? a[i + 2] : a[i];
    a[i] = keep + __shfl_xor_sync(FULL, send, 4);
  }
  const bool hi2 = lane & 2;
  {
    const double send = hi2 ? a[0] : a[1];
    const double keep = hi2 ? a[1] : a[0];
    a[0] = keep + __shfl_xor_sync(FULL, send, 2);
  }
  a[0] += __shfl_xor_sync(FULL, a[0], 1);
  idx = (hi16 ? 8 : 0) + (hi8 ? 4 : 0) + (hi4 ? 2 : 0) + (hi2 ? 1 : 0);
  return a[0];
}

// Warp reduce-scatter of 8 values per lane: afterwards every lane holds the
// warp sum of value index idx(lane) (lanes differing only in bits 0-1 agree).
__device__ __forceinline__ double reduce_scatter8(double (&v)[8], int lane, int& idx) {
  const unsigned FULL = 0xffffffffu;
  double a[4];
  const bool hi16 = lane & 16;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double send = hi16 ? v[i] : v[i + 4];
    const double keep = hi16 ? v[i + 4] : v[i];
    a[i] = keep + __shfl_xor_sync(FULL, send, 16);
  }
  const bool hi8 = lane & 8;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double send = hi8 ? a[i] : a[i + 2];
    const double keep = hi8 ? a[i + 2] : a[i];
    a[i] = keep + __shfl_xor_sync(FULL, send, 8);
  }
  const bool hi4 = lane & 4;
  {
    const double send = hi4 ? a[0] : a[1];
    const double keep = hi4 ? a[1] : a[0];
    a[0] = keep + __shfl_xor_sync(FULL, send, 4);
  }
  a[0] += __shfl_xor_sync(FULL, a[0], 2);
  a[0] += __shfl_xor_sync(FULL, a[0], 1);
  idx = (hi16 ? 4 : 0) + (hi8 ? 2 : 0) + (hi4 ? 1 : 0);
  return a[0];
}

// Rows with ψ below this take the two-dot form of the row adjoints (the
// one-dot form divides a difference of two sums by ψ).
constexpr double kPsiOneDot = 1e-6;

template <int NT>
__device__ __forceinline__ void block_sum4(double (&v)[4], double* red) {
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int i = 0; i < 4; ++i) red[4 * w + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    double s = 0.0;
    for (int q = 0; q < NT / 32; ++q) s += red[4 * q + i];
    v[i] = s;
  }
}

// Reverse sweep of one task.  Per-task outputs (gout + T.gout):
// [2r] ∂/∂ϕ_r, [2r+1] ∂/∂ψ_r (rows r >= 1; a branch in the one-dot form of
// adj_rows writes E_r to [2r] for r = 0..n-1 instead), [2n] ∂/∂ε_top(child 0),
// [2n+1] ∂/∂ε_top(child 1), [2n+2] ∂/∂q, [2n+3] ∂/∂η, [2n+4] ∂/∂ε_top(own).
// Reverse rows n-1 .. 1 of a branch.  J > 0: lane program in registers (an
// instantiation of depth J for programs of depth <= J); J == 0: entries
// streamed from memory.  Per row:
// G[x] = Σ p·bar[γ]·L[sib], bar_{r-1}[x] = ϕ bar[x] + ψ G[x]; then
// ∂/∂ϕ_r = Σ bar_r·L_{r-1} and ∂/∂ψ_r = ½ Σ G·L_{r-1} (each split counted
// twice).  The row step is homogeneous of degree 1 in ϕ-terms and 2 in
// ψ-terms, so with E_r = Σ bar_r·L_r:
//   E_r = ϕ_r ∂ϕ_r + ψ_r ∂ψ_r,   E_{r-1} = ϕ_r ∂ϕ_r + 2 ψ_r ∂ψ_r,
// i.e. ∂ψ_r = (E_{r-1} - E_r)/ψ_r and ∂ϕ_r = (2E_r - E_{r-1})/ϕ_r: one dot
// per row (E_{r-1} = Σ bar_{r-1}·L_{r-1}) instead of two, reduced 8 rows at
// a time by a register-ring reduce-scatter.  The task writes E_r to out[2r]
// (r = 0..n-1); the pairs are linear, ϕ and ψ are the node's, so the host
// forms the row adjoints after the sum over tasks.  Branches with a row whose
// ψ is below kPsiOneDot (or ϕ = 0) take both dots directly (ONEDOT false,
// entries streamed) and write ∂/∂ϕ_r, ∂/∂ψ_r to out[2r], out[2r + 1].
// GMEM: the task's rows live in device memory (plain copies, no bulk copies).
// Otherwise each table row goes to its shared buffer as one 1-D bulk copy
// (TMA) issued by thread 0 and completed on that buffer's mbarrier (mb[NB]).
template <int NT, int J, bool ONEDOT, bool GMEM>
__device__ __forceinline__ void adj_rows(const DEntry* __restrict__ E, const DTask& T, int lane, int n, int R,
                                         const double* phs, const double* pss, double*& bar, double*& barn,
                                         double* Lb, int W2, double* Gs, double* part, double* red,
                                         const double* tab0, double* out, uint64_t* mb, int* err) {
  const int tid = threadIdx.x, wid = tid >> 5, wl = tid & 31;
  const int S = T.tstride;  // table row stride (even: rows 16-byte aligned)
  double rp[8], rs[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) rp[i] = rs[i] = 0.0;
  const DProg2 td = T.tdup;  // held in registers: the loop stores to global memory
  LaneProg<(J > 0 ? J : 1)> lp;
  if (J > 0) load_lane_prog<(J > 0 ? J : 1)>(E, td, lane, lp);
  const bool active = lane < td.nt;
  // table-row buffers: four (copies three rows ahead) in the one-dot form,
  // which leaves G unused and takes its row as the fourth; three otherwise
  constexpr int NB = ONEDOT ? 4 : 3;
  if constexpr (!GMEM) {
    // the buffers may hold what generic stores left (an earlier task's rows)
    fence_proxy_async_smem();
    if (tid == 0) {
      for (int i = 0; i < NB; ++i) mbar_init(mb + i);
      mbar_init_fence();
    }
    __syncthreads();
  }
  // Row r reads table row r-1 from buffer (n-1-r) mod NB (buffer i at Lb +
  // i·W2); the copies run NB-1 rows ahead (none past row 1).  par: bit i is
  // the phase parity of buffer i's next completion.
  unsigned par = 0;
  auto fetch = [&](int rr, int buf) {
    if (rr < 1) return;
    const double* src = tab0 + (int64_t)(rr - 1) * S;
    double* dst = Lb + buf * W2;
    if constexpr (GMEM) {
      for (int c = tid; c < R; c += NT) dst[c] = src[c];
    } else if (tid == 0) {
      bulk_row_g2s(dst, src, (unsigned)S * 8u, mb + buf);
    }
  };
  auto landed = [&](int buf) {  // buffer buf's copy has arrived (every thread waits)
    if constexpr (!GMEM) {
      mbar_wait(mb + buf, (par >> buf) & 1u, err);
      par ^= 1u << buf;
    }
  };
  constexpr int NW = NT / 32;
  if constexpr (ONEDOT) {  // E_{n-1} = Σ bar_{n-1}·L_{n-1}
    const double* Ltop = tab0 + (int64_t)(n - 1) * S;
    double e = 0.0;
    for (int c = tid; c < R; c += NT) e = fma(bar[c], Ltop[c], e);
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (wl == 0) red[wid] = e;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < NW; ++q) t += red[q];
      out[2 * (n - 1)] = t;
    }
  }
  // One row's program and split-clade combines: bar_{r-1} into bn from bar_r
  // (bb) and table row r-1 (Lp).
  auto row = [&](int r, const double* Lp, const double* bb, double* bn) {
    const double ph = phs[r], ps = pss[r];
    if (J > 0) {
      if (active)
        rows_reg<(J > 0 ? J : 1), op::FIN_ADJ>(lp, bb, Lp, part, ph, ps, [&](unsigned c, double v, double g) {
          bn[c] = v;
          if constexpr (!ONEDOT) Gs[c] = g;  // G is read by the two-dot form only
        });
    } else if (active) {
      const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + td.off) + lane;
      double acc = 0.0;
      auto onfin = [&](unsigned c, double v, double g) {
        bn[c] = v;
        if constexpr (!ONEDOT) Gs[c] = g;
      };
      stream_steps<op::FIN_ADJ>(e, td.nt, 0, td.J, bb, Lp, part, ph, ps, onfin, acc);
    }
    if (td.ncomb) {
      __syncthreads();
      // (combine entries stream from memory here: registers are the limit)
      run_comb<NT, false>(E, td, part, [&](unsigned, unsigned c, unsigned, unsigned, double g) {
        bn[c] = fma(ps, g, ph * bb[c]);
        if constexpr (!ONEDOT) Gs[c] = g;
      });
    }
  };
  int bi = 0;
  for (int i = 0; i + 1 < NB; ++i) fetch(n - 1 - i, i);
  if constexpr (ONEDOT) {
    // One CTA barrier per row: it follows the program (bar_{r-1} complete)
    // once the next row's table row has landed.  The dot reads only
    // bar_{r-1} and row r-1, which the next program does not write, and a
    // buffer is refilled only after the barrier that follows its last reader
    // (the dot of the row above: row r+1's buffer takes table row r-NB).
    landed(0);
    __syncthreads();
    for (int r = n - 1; r >= 1; --r) {
      double* Lp = Lb + bi * W2;
      double* bn = barn;
      row(r, Lp, bar, bn);
      if (r >= 2) landed(bi + 1 == NB ? 0 : bi + 1);
      __syncthreads();
      fetch(r - (NB - 1), bi == 0 ? NB - 1 : bi - 1);
      bi = bi + 1 == NB ? 0 : bi + 1;
      const int slot = (n - 1 - r) & 7;
      double e = 0.0;  // this lane's share of E_{r-1}
      for (int c = tid; c < R; c += NT) e = fma(bn[c], Lp[c], e);
#pragma unroll
      for (int i = 0; i < 8; ++i) rp[i] = (i == slot) ? e : rp[i];
      if (slot == 7 || r == 1) {
        int idx;
        const double v = reduce_scatter8(rp, wl, idx);
        if ((wl & 3) == 0) red[8 * wid + idx] = v;
        __syncthreads();
        if (tid <= slot) {  // batch slot tid holds E_{rr-1}, rr its row
          double sum = 0.0;
          for (int q = 0; q < NW; ++q) sum += red[8 * q + tid];
          out[2 * (r + slot - tid - 1)] = sum;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) rp[i] = 0.0;
      }
      double* t = bar;
      bar = barn;
      barn = t;
    }
  } else {
    for (int r = n - 1; r >= 1; --r) {
      double* Lp = Lb + bi * W2;
      landed(bi);
      __syncthreads();
      // every thread is past row r+1, whose buffer takes table row r-NB
      fetch(r - (NB - 1), bi == 0 ? NB - 1 : bi - 1);
      bi = bi + 1 == NB ? 0 : bi + 1;
      const double* bb = bar;
      row(r, Lp, bb, barn);
      __syncthreads();
      const int slot = (n - 1 - r) & 7;
      double dphi = 0.0, dpsi = 0.0;
      for (int c = tid; c < R; c += NT) {
        const double l = Lp[c];
        dphi = fma(bb[c], l, dphi);
        dpsi = fma(Gs[c], l, dpsi);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        rp[i] = (i == slot) ? dphi : rp[i];
        rs[i] = (i == slot) ? dpsi : rs[i];
      }
      if (slot == 7 || r == 1) {
        int idx;
        const double v = reduce_scatter16(rp, rs, wl, idx);
        if ((wl & 1) == 0) red[16 * wid + idx] = v;
        __syncthreads();
        if (tid < 16) {
          double sum = 0.0;
          for (int q = 0; q < NT / 32; ++q) sum += red[16 * q + tid];
          const int i = tid & 7;
          const int rr = r + slot - i;  // row of batch slot i
          if (i <= slot) out[2 * rr + (tid >> 3)] = (tid >> 3) ? 0.5 * sum : sum;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) rp[i] = rs[i] = 0.0;
      }
      double* t = bar;
      bar = barn;
      barn = t;
    }
  }
  if constexpr (!GMEM) {  // every copy was waited for; row 0 reuses the buffers
    __syncthreads();
    if (tid == 0)
      for (int i = 0; i < NB; ++i) mbar_inval(mb + i);
  }
}

template <int NT, bool GMEM, int J = kAdjJStep>
__device__ __forceinline__ bool adj_rows_dispatch(int j, const DEntry* __restrict__ E, const DTask& T, int lane, int n,
                                                  int R, const double* phs, const double* pss, double*& bar,
                                                  double*& barn, double* Lb, int W2, double* Gs, double* part,
                                                  double* red, const double* tab0, double* out, uint64_t* mb,
                                                  int* err) {
  constexpr int MAXJ = NT == kNT2L ? 8 : 12;
  if constexpr (J > MAXJ) {
    return false;
  } else {
    constexpr int NEXT = (J + kAdjJStep > MAXJ && J < MAXJ) ? MAXJ : J + kAdjJStep;
    if (j <= J) {
      adj_rows<NT, J, true, GMEM>(E, T, lane, n, R, phs, pss, bar, barn, Lb, W2, Gs, part, red, tab0, out, mb, err);
      return true;
    }
    return adj_rows_dispatch<NT, GMEM, NEXT>(j, E, T, lane, n, R, phs, pss, bar, barn, Lb, W2, Gs, part, red, tab0, out,
                                             mb, err);
  }
}

// One adjoint task; rot and CG as for fwd_task (CG: the task's own top-row
// adjoints were written by its parents' tasks in this launch).
template <int NT, bool ROOT, bool GLOBAL, bool CG>
__device__ __forceinline__ void adj_task(const KArgs2& A, const DTask& T, int rot, double* smem_dyn) {
  double* const sm = GLOBAL ? A.scratch + T.scratch : smem_dyn;
  const int k = T.node;
  const int4 mn = A.mnode[k];
  const int R = T.width;
  const int W2 = (max(R, T.wa + T.wb) + 1) & ~1;  // even: 16-byte aligned row buffers
  const int tid = threadIdx.x;
  const int lane = (tid + 32 * (int)(rot & (NT / 32 - 1))) & (NT - 1);
  const int NR = A.NR;
  const int roff = A.row_off[k];
  const int n = mn.w;
  double* bar = sm;
  double* barn = sm + W2;
  double* L0 = sm + 2 * W2;  // L0, L1, a third and (one-dot form) G's row: table rows of the branch
  double* L1 = sm + 3 * W2;
  double* Gs = sm + 5 * W2;
  double* part = sm + 6 * W2;
  double* red = part + T.nslot_max;  // 16 * warps doubles
  double* out = A.gout + T.gout;
  const DEntry* E = A.entries;
  const int64_t* gm = A.gmap + T.gmap;
  if (!ROOT) {
    prefetch_prog(E, T.tdup, lane);
    prefetch_prog(E, T.ta, lane);
    prefetch_prog(E, T.tb, lane);
    for (int r = tid; r < n; r += NT) {
      prefetch_l1(A.params + NR + roff + r);
      prefetch_l1(A.params + 2 * NR + roff + r);
    }
  } else {
    prefetch_levels(E, A.progs + T.tlvl, T.nlvl);
    prefetch_prog(E, T.init, lane);
    prefetch_prog(E, T.ta, lane);
    prefetch_prog(E, T.tb, lane);
  }
  if (ROOT) {
    const double* row0 = A.tabs + T.tab;
    for (int c = tid; c < R; c += NT) {
      L0[c] = row0[c];
      bar[c] = 0.0;
    }
    __syncthreads();
    const int2* fam = reinterpret_cast<const int2*>(A.meta) + T.fam;
    for (int f = tid; f < T.nfam; f += NT) {
      const double L = L0[fam[f].y];
      const double w = A.famw ? A.famw[fam[f].x] : 1.0;  // ∂(Σ w log L)/∂L
      bar[fam[f].y] = L > 0.0 ? w / L : 0.0;
    }
    __syncthreads();
    const double ca = A.params[3 * NR + A.K + 1], cb = A.params[3 * NR + A.K + 2];
    double acc4[4] = {0.0, 0.0, 0.0, 0.0};  // dca, dcb, dea, deb
    for (int c = tid; c < R; c += NT) Gs[c] = 0.0;
    __syncthreads();
    auto tcomb = [&](unsigned, unsigned c, unsigned, unsigned, double g) {
      bar[c] = fma(ca, g, bar[c]);
      Gs[c] = g;
    };
    auto tfin = [&](unsigned c, double v, double g) {
      bar[c] = v;
      Gs[c] = g;
    };
    chain_levels<NT, true, op::FIN_TLVL>(E, A.progs + T.tlvl, T.nlvl, tid, tid, bar, L0, part, 1.0, ca, tfin,
                                         tcomb);
    // ∂/∂ca = Σ bar[γ]·Πroot(γ) = ½ Σ_x G[x]·L[x] (each split counted twice)
    for (int c = tid; c < R; c += NT) acc4[0] += 0.5 * Gs[c] * L0[c];
    // stage the children's tops, recompute Πspec + Πloss for ∂/∂cb
    double* X = barn;
    double* Y = barn + T.wa;
    gather_rows<NT, false>(barn, A.tops, gm, T.wa + T.wb);
    __syncthreads();
    const double ea = eps_top2(A, mn.y), eb = eps_top2(A, mn.z);
    double* bbc = L1;  // cb · bar, the adjoint of Πspec + Πloss
    const int2* loss = reinterpret_cast<const int2*>(A.meta) + T.loss;
    auto sfin = [&](unsigned, unsigned c, unsigned fa, unsigned fb, double acc) {
      const double la = fa != 0xFFFFu ? X[fa] : 0.0;
      const double lb = fb != 0xFFFFu ? Y[fb] : 0.0;
      const double bc = acc + (la * eb + lb * ea);
      acc4[1] += bar[c] * bc;
    };
    run_any(E, T.init, lane, X, Y, part, sfin);
    if (T.init.ncomb) {
      __syncthreads();
      run_comb<NT, true>(E, T.init, part, sfin);
    }
    for (int c = tid; c < R; c += NT) {
      const double b = cb * bar[c];
      bbc[c] = b;
      const int2 l = loss[c];
      acc4[2] += b * (l.y >= 0 ? Y[l.y] : 0.0);
      acc4[3] += b * (l.x >= 0 ? X[l.x] : 0.0);
    }
    __syncthreads();
    auto afin = [&](unsigned, unsigned x, unsigned fa, unsigned, double acc) {
      A.bartops[gm[x]] = acc + (fa != 0xFFFFu ? bbc[fa] * eb : 0.0);
    };
    // ta and tb have disjoint partial slots: one combine phase after both
    run_any(E, T.ta, lane, bbc, Y, part, afin);
    auto bfin = [&](unsigned, unsigned x, unsigned fa, unsigned, double acc) {
      A.bartops[gm[T.wa + x]] = acc + (fa != 0xFFFFu ? bbc[fa] * ea : 0.0);
    };
    run_any(E, T.tb, lane, bbc, X, part, bfin);
    if (T.ta.ncomb || T.tb.ncomb) {
      __syncthreads();
      run_comb<NT, false>(E, T.ta, part, afin);
      run_comb<NT, false>(E, T.tb, part, bfin);
    }
    block_sum4<NT>(acc4, red);
    if (tid == 0) {
      const double eta = A.params[3 * NR + A.K];
      const double er = eps_top2(A, k);
      const double xi = 1.0 - (1.0 - eta) * er;
      const double dxi_deta = er, dxi_der = -(1.0 - eta);
      const double dca_deta = (-xi + (1.0 - eta) * dxi_deta) / eta - (1.0 - eta) * xi / (eta * eta);
      const double dca_der = (1.0 - eta) * dxi_der / eta;
      const double xi2 = xi * xi, xi3 = xi2 * xi;
      const double dcb_deta = (1.0 - er) / xi2 - 2.0 * eta * (1.0 - er) * dxi_deta / xi3;
      const double dcb_der = -eta / xi2 - 2.0 * eta * (1.0 - er) * dxi_der / xi3;
      out[2 * n + 3] = acc4[0] * dca_deta + acc4[1] * dcb_deta;
      out[2 * n + 4] = acc4[0] * dca_der + acc4[1] * dcb_der;
      out[2 * n + 0] = acc4[2];
      out[2 * n + 1] = acc4[3];
    }
    return;
  }
  // ---- rows n-1 .. 1 of the branch (within_branch!)
  for (int c = tid; c < R; c += NT) bar[c] = ld_shared_row<CG>(A.bartops + T.top + c);
  if (n > 1) {
    double* phs = red + 16 * (NT / 32);  // ϕ, ψ of this branch's rows
    double* pss = phs + n;
    for (int r = tid; r < n; r += NT) {
      phs[r] = A.params[NR + roff + r];
      pss[r] = A.params[2 * NR + roff + r];
    }
    __syncthreads();
    const double* tab0 = A.tabs + T.tab;
    // one-dot row adjoints unless a row's ψ is tiny (uniform over the CTA)
    bool ok = true;
    for (int r = 1 + tid; r < n; r += NT) ok &= pss[r] >= kPsiOneDot && phs[r] > 0.0;
    __shared__ __align__(8) uint64_t mb[4];  // the table-row buffers' mbarriers
    if (!__syncthreads_and(ok))
      adj_rows<NT, 0, false, GLOBAL>(E, T, lane, n, R, phs, pss, bar, barn, L0, W2, Gs, part, red, tab0, out, mb,
                                     A.err);
    else if (!adj_rows_dispatch<NT, GLOBAL>(T.tdup.J, E, T, lane, n, R, phs, pss, bar, barn, L0, W2, Gs, part, red,
                                           tab0, out, mb, A.err))
      adj_rows<NT, 0, true, GLOBAL>(E, T, lane, n, R, phs, pss, bar, barn, L0, W2, Gs, part, red, tab0, out, mb,
                                    A.err);
  }
  __syncthreads();
  // ---- row 0
  if (mn.x == WG_NODE_WGD) {
    double* X = L0;
    gather_rows<NT, false>(X, A.tops, gm, T.wa);
    __syncthreads();
    const double q = A.params[3 * NR + k];
    const double ef = eps_top2(A, mn.y);
    double acc4[4] = {0.0, 0.0, 0.0, 0.0};  // dq, def
    auto wfin = [&](unsigned, unsigned c, unsigned, unsigned, double g) {
      const double b = bar[c], xv = X[c];
      A.bartops[gm[c]] = ((1.0 - q) + 2.0 * q * ef) * b + q * g;
      acc4[0] += b * (2.0 * ef * xv - xv) + 0.5 * g * xv;
      acc4[1] += b * 2.0 * q * xv;
    };
    // the row-0 retention term uses the duplication triples of this node
    // (transposed program over the staged child row)
    if (lane < T.tdup.nt) {
      const ulonglong2* e = reinterpret_cast<const ulonglong2*>(E + T.tdup.off) + lane;
      double acc = 0.0;
      for (int j = 0; j < T.tdup.J; ++j, e += T.tdup.nt) {
        const Raw x = decode(__ldg(e));
        if (x.opc == op::PROD) acc = fma(x.p * bar[x.f0], X[x.f1], acc);
        else if (x.opc == op::FIN_PART) { part[x.f2] = acc; acc = 0.0; }
        else if (x.opc == op::FIN_ADJ) { wfin(0, x.f0, 0, 0, acc); acc = 0.0; }
      }
    }
    if (T.tdup.ncomb) {
      __syncthreads();
      run_comb<NT, false>(E, T.tdup, part, wfin);
    }
    block_sum4<NT>(acc4, red);
    if (tid == 0) {
      out[2 * n + 2] = acc4[0];
      out[2 * n + 0] = acc4[1];
    }
  } else if (mn.x == WG_NODE_INTERNAL) {
    double* X = L0;
    double* Y = L0 + T.wa;
    gather_rows<NT, false>(L0, A.tops, gm, T.wa + T.wb);
    __syncthreads();
    const double ea = eps_top2(A, mn.y), eb = eps_top2(A, mn.z);
    auto afin = [&](unsigned, unsigned x, unsigned fa, unsigned, double acc) {
      A.bartops[gm[x]] = acc + (fa != 0xFFFFu ? bar[fa] * eb : 0.0);
    };
    // ta and tb have disjoint partial slots: one combine phase after both
    run_any(E, T.ta, lane, bar, Y, part, afin);
    auto bfin = [&](unsigned, unsigned x, unsigned fa, unsigned, double acc) {
      A.bartops[gm[T.wa + x]] = acc + (fa != 0xFFFFu ? bar[fa] * ea : 0.0);
    };
    run_any(E, T.tb, lane, bar, X, part, bfin);
    if (T.ta.ncomb || T.tb.ncomb) {
      __syncthreads();
      run_comb<NT, false>(E, T.ta, part, afin);
      run_comb<NT, false>(E, T.tb, part, bfin);
    }
    double acc4[4] = {0.0, 0.0, 0.0, 0.0};  // dea, deb
    const int2* loss = reinterpret_cast<const int2*>(A.meta) + T.loss;
    for (int c = tid; c < R; c += NT) {
      const int2 l = loss[c];
      const double b = bar[c];
      acc4[0] += b * (l.y >= 0 ? Y[l.y] : 0.0);
      acc4[1] += b * (l.x >= 0 ? X[l.x] : 0.0);
    }
    block_sum4<NT>(acc4, red);
    if (tid == 0) {
      out[2 * n + 0] = acc4[0];
      out[2 * n + 1] = acc4[1];
    }
  }
}

// ROOT as for k_fwd2.  Four 128-thread CTAs per SM leave the adjoint its
// ~110 registers: at five or six the spills cost more than the occupancy
// gains (the rows are latency-bound, not FP64-bound).
template <int NT, bool ROOT = false, bool GLOBAL = false>
__global__ void __launch_bounds__(NT, NT == 128 && !GLOBAL ? 4 : (GLOBAL ? 1 : 2))
    k_adj2(const KArgs2 A, const int* __restrict__ list) {
  extern __shared__ __align__(128) double smem_dyn[];
  adj_task<NT, ROOT, GLOBAL, false>(A, A.tasks[list[blockIdx.x]], (int)blockIdx.x, smem_dyn);
}

// Gradient reduction: out[j] = Σ gout[idx] over the fixed contributor list of
// j; one warp per output, lane-strided partial sums and a fixed butterfly.
__global__ void k_reduce2(const double* __restrict__ gout, const int64_t* __restrict__ off,
                          const int64_t* __restrict__ idx, int P, double* __restrict__ out) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= P) return;
  double s = 0.0;
  for (int64_t i = off[j] + lane; i < off[j + 1]; i += 32) s += gout[idx[i]];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[j] = s;
}

// ===========================================================================
// Persistent launches: one kernel per pass over every task of a layout.
// CTAs take tickets in a topological order of the pass (an atomic counter);
// a task waits until the tasks it depends on have published their results,
// runs, and publishes its own.  A task's dependencies hold earlier tickets,
// so each is finished or held by a running CTA: the unfinished task with the
// lowest ticket can always proceed and the waits cannot deadlock.  Every wait
// is bounded: past the poll limit the CTA sets an error bit (which the host
// turns into WG_ECUDA), skips the task's work and still publishes it, so the
// launch ends in bounded time.
// ===========================================================================
struct PArgs {
  const int* order;    // ticket -> task
  const int* dep_off;  // per task: the tasks it waits for (CSR)
  const int* dep_idx;
  int* done;           // per task: 1 once published in this pass; [n] is never set
  int* ticket;         // next ticket of this pass
  int* err;            // bit 0: a dependency wait gave up
  int n;
  int spin_cap;        // polls per dependency before giving up
  int wait_unset;      // test aid: every task also waits on done[n], which nothing sets
};

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Bounded wait of one flag; false when the poll limit ran out.
__device__ __forceinline__ bool wait_flag(const int* f, int cap) {
  for (int polls = 0; ld_acquire_gpu(f) == 0; ++polls) {
    if (polls >= cap) return false;
    __nanosleep(200);
  }
  return true;
}

// Every thread waits for a share of the task's dependencies; true when all
// were published (a CTA barrier orders the waits before the task's reads).
__device__ __forceinline__ bool wait_deps(const PArgs& P, int task) {
  bool ok = true;
  const int b = P.dep_off[task], e = P.dep_off[task + 1];
  for (int i = b + (int)threadIdx.x; i < e && ok; i += blockDim.x) ok = wait_flag(P.done + P.dep_idx[i], P.spin_cap);
  if (P.wait_unset && threadIdx.x == 0) ok = ok && wait_flag(P.done + P.n, P.spin_cap);
  const bool all = __syncthreads_and(ok) != 0;
  if (!all && threadIdx.x == 0) atomicOr(P.err, 1);
  return all;
}

// Publishes a finished task: the barrier orders every thread's stores before
// thread 0's release.
__device__ __forceinline__ void publish(const PArgs& P, int task) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release_gpu(P.done + task, 1);
  }
}

// Persistent forward: any task of the layout (root or branch, rows in shared
// or device memory) with kNT2L threads; the dynamic shared memory is the
// largest of the layout's shared-memory tasks.  Bounded for three CTAs per
// SM (the default WG_PERSIST_CTAS): the four variants held at once fit ~165
// registers without spills; the grid follows the occupancy it compiles to.
template <bool TABLES>
__global__ void __launch_bounds__(kNT2L, 3) k_fwd_persist(const KArgs2 A, const PArgs P) {
  extern __shared__ __align__(128) double smem_dyn[];
  __shared__ int s_t;
  for (;;) {
    if (threadIdx.x == 0) s_t = atomicAdd(P.ticket, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= P.n) return;
    const int task = P.order[t];
    if (wait_deps(P, task)) {  // (its barrier also lets s_t be rewritten)
      const DTask& T = A.tasks[task];
      const bool root = A.mnode[T.node].x == WG_NODE_ROOT;
      if (root && T.scratch >= 0) fwd_task<TABLES, kNT2L, true, true, true>(A, T, t, smem_dyn);
      else if (root) fwd_task<TABLES, kNT2L, true, false, true>(A, T, t, smem_dyn);
      else if (T.scratch >= 0) fwd_task<TABLES, kNT2L, false, true, true>(A, T, t, smem_dyn);
      else fwd_task<TABLES, kNT2L, false, false, true>(A, T, t, smem_dyn);
    }
    publish(P, task);
  }
}

// Persistent adjoint, tickets from the root level down.
__global__ void __launch_bounds__(kNT2L, 3) k_adj_persist(const KArgs2 A, const PArgs P) {
  extern __shared__ __align__(128) double smem_dyn[];
  __shared__ int s_t;
  for (;;) {
    if (threadIdx.x == 0) s_t = atomicAdd(P.ticket, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= P.n) return;
    const int task = P.order[t];
    if (wait_deps(P, task)) {
      const DTask& T = A.tasks[task];
      const bool root = A.mnode[T.node].x == WG_NODE_ROOT;
      if (root && T.scratch >= 0) adj_task<kNT2L, true, true, true>(A, T, t, smem_dyn);
      else if (root) adj_task<kNT2L, true, false, true>(A, T, t, smem_dyn);
      else if (T.scratch >= 0) adj_task<kNT2L, false, true, true>(A, T, t, smem_dyn);
      else adj_task<kNT2L, false, false, true>(A, T, t, smem_dyn);
    }
    publish(P, task);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(WG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
T* dalloc(size_t n, int64_t& bytes) {
  if (n == 0) n = 1;
  void* p = nullptr;
  const cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(WG_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  bytes += (int64_t)(n * sizeof(T));
  return static_cast<T*>(p);
}

template <class T, class A>
void h2d(T* d, const std::vector<T, A>& h, cudaStream_t s) {
  if (!h.empty()) ck(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
}

}  // namespace

struct wg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // heavy tasks of a level run here, joined back per level
  cudaEvent_t fork = nullptr, join = nullptr;
  int n_sm = 0;
  size_t smem_optin = 0;
  size_t smem_sm = 0;  // shared memory of one SM
  bool timing = false;
  bool timed = false;  // events of the last evaluation were recorded
  bool timed_grad = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float last_ms[3] = {0, 0, 0};
  std::unique_ptr<NwPlan> nw;  // wg_nowhere_condition's plan
  double* noalloc_tops = nullptr;  // device address of wg_logpdf_noalloc's fixed scratch on this device
};

namespace {

void free_all(int device, std::initializer_list<void*> dptrs, std::initializer_list<void*> hptrs) {
  cudaSetDevice(device);
  for (void* p : dptrs)
    if (p) cudaFree(p);
  for (void* p : hptrs)
    if (p) cudaFreeHost(p);
}

// Slice tables, q and η of the current rates into a pinned staging buffer
// (eps | phi | psi | q | eta) and on to the device.
void upload_params(const wg_model* m, int NR, int K, double* h, double* d, cudaStream_t s) {
  std::memcpy(h, m->eps.data(), NR * sizeof(double));
  std::memcpy(h + NR, m->phi.data(), NR * sizeof(double));
  std::memcpy(h + 2 * NR, m->psi.data(), NR * sizeof(double));
  for (int k = 0; k < K; ++k) h[3 * NR + k] = std::isnan(m->q[k]) ? 0.0 : m->q[k];
  h[3 * NR + K] = m->eta;
  ck(cudaMemcpyAsync(d, h, sizeof(double) * (3 * NR + K + 1), cudaMemcpyHostToDevice, s), "params upload");
}

}  // namespace

// Plain path: one family per launch (v1 single-CTA kernel).
struct PlainBatch {
  wg_ctx* ctx = nullptr;
  int K = 0, NR = 0, NF = 0, n_groups = 0, P = 0;
  size_t smem_fwd = 0;
  DGroup* d_groups = nullptr;
  DNode* d_nodes = nullptr;
  DEntry* d_entries = nullptr;
  int* d_meta = nullptr;
  DLevel* d_levels = nullptr;
  int* d_famidx = nullptr;
  int* d_fampos = nullptr;
  int4* d_mnode = nullptr;
  int* d_rowoff = nullptr;
  double* d_leafp = nullptr;
  double* d_params = nullptr;
  double* d_tops = nullptr;
  double* d_logl = nullptr;
  double* d_gred = nullptr;
  double* h_params = nullptr;
  double* h_logl = nullptr;
  double* h_gred = nullptr;
  bool grad_pending = false;
  int64_t device_bytes = 0;
  ~PlainBatch() {
    if (ctx)
      free_all(ctx->device, {d_groups, d_nodes, d_entries, d_meta, d_levels, d_famidx, d_fampos, d_mnode, d_rowoff,
                             d_leafp, d_params, d_tops, d_logl},
               {h_params, h_logl});
  }
};

// Batched path: families split into size classes; each class is a layout of
// level-synchronous (node, family group) tasks on its own pair of streams, so
// the classes overlap on the device and every launch sizes its shared memory
// for tasks of one size class.
struct SubBatch {
  int device = 0;
  int n_tasks = 0;
  std::vector<int> fam;  // global family index of each local family
  std::vector<int> lvl_off, lvl_n, lvlh_off, lvlh_n;
  std::vector<size_t> lvl_smem, lvl_smem_adj, lvlh_smem, lvlh_smem_adj;
  std::vector<int> lvlg_off, lvlg_n, lvlgh_off, lvlgh_n;  // tasks with rows in device scratch
  double* d_scratch = nullptr;
  std::vector<int64_t> fam_tab;
  std::vector<int32_t> fam_w, fam_col, fam_ncol;
  DTask* d_tasks = nullptr;
  DEntry* d_entries = nullptr;
  int* d_meta = nullptr;
  int64_t* d_gmap = nullptr;
  DProg2* d_progs = nullptr;
  int* d_lists = nullptr;
  int64_t* d_red_off = nullptr;
  int64_t* d_red_idx = nullptr;
  double* d_tops = nullptr;
  double* d_tabs = nullptr;
  double* d_bartops = nullptr;
  double* d_gout = nullptr;
  double* d_gred = nullptr;
  int64_t gout_doubles = 0;
  int64_t tops_doubles = 0;
  bool checkpoint = false;  // tables recomputed level by level in the adjoint (one level's tables held)
  // persistent launches (one kernel per pass): ticket orders, dependency
  // lists, per-task flags and the ticket / error counters
  bool persist = false;
  int n_pdep_f = 0, n_pdep_a = 0;
  int* d_porder = nullptr;  // forward order (n_tasks) then adjoint order
  int* d_pdep = nullptr;    // forward CSR (n_tasks + 1 offsets, indices) then adjoint CSR
  int* d_pdone = nullptr;   // n_tasks + 1 flags
  int* d_pctl = nullptr;    // [0] ticket, [1] error bits
  size_t psmem_f = 0, psmem_a = 0;
  int pgrid_f = 0, pgrid_a = 0;
  cudaStream_t s = nullptr, s2 = nullptr;
  cudaStream_t sa = nullptr, sa2 = nullptr;  // adjoint streams when the adjoint follows the class's own forward
  cudaEvent_t fork = nullptr, join = nullptr, done = nullptr;
  ~SubBatch() {
    free_all(device, {d_tasks, d_entries, d_meta, d_gmap, d_progs, d_lists, d_red_off, d_red_idx, d_tops, d_tabs,
                      d_bartops, d_gout, d_gred, d_scratch, d_porder, d_pdep, d_pdone, d_pctl},
             {});
    for (cudaEvent_t e : {fork, join, done})
      if (e) cudaEventDestroy(e);
    if (s2) cudaStreamDestroy(s2);
    if (s) cudaStreamDestroy(s);
    if (sa2) cudaStreamDestroy(sa2);
    if (sa) cudaStreamDestroy(sa);
  }
};

// Device copy of the families' structure for backtracking on the device
// (built on the first wg_track_device call of a batch), and the buffers of
// the last call.
struct TrackData {
  int device = 0;
  int64_t* d_fk_tab = nullptr;
  int* d_fk_w = nullptr;
  int* d_fk_col = nullptr;
  int64_t* d_fclade = nullptr;
  int* d_fnclade = nullptr;
  int64_t* d_fcol = nullptr;
  int16_t* d_cols = nullptr;
  int64_t* d_csplit = nullptr;
  int* d_g1 = nullptr;
  int* d_g2 = nullptr;
  double* d_sp = nullptr;
  unsigned char* d_cleaf = nullptr;
  const double** d_ftabs = nullptr;
  std::vector<int64_t> cap;  // per family: node slots of one tree (an upper bound)
  // per-call buffers, grown as needed
  int* d_fam = nullptr;
  uint64_t* d_seed = nullptr;
  int64_t* d_capoff = nullptr;
  int64_t* d_off = nullptr;
  int* d_count = nullptr;
  int4* d_nodes = nullptr;
  int4* d_stack = nullptr;
  int4* d_out = nullptr;
  size_t n_trees_cap = 0, slots_cap = 0, out_cap = 0;
  std::vector<int32_t> last_nodes;  // the last call's trees (4 ints per node)
  ~TrackData() {
    free_all(device, {d_fk_tab, d_fk_w, d_fk_col, d_fclade, d_fnclade, d_fcol, d_cols, d_csplit, d_g1, d_g2, d_sp,
                      d_cleaf, (void*)d_ftabs, d_fam, d_seed, d_capoff, d_off, d_count, d_nodes, d_stack, d_out},
             {});
  }
};

struct wg_batch {
  wg_ctx* ctx = nullptr;
  int K = 0, NR = 0, NF = 0, P = 0, n_tasks = 0;
  uint32_t flags = 0;
  int64_t device_bytes = 0;
  double flops_fwd = 0, bytes_fwd = 0, flops_adj = 0;
  int64_t tab_full = 0, tab_kept = 0;  // table doubles: every table / held on the device
  // 2 (default): each size class's adjoint follows its own forward on
  // streams of the class's priority, overlapping the other classes' forwards
  // (1.62 against 1.66 ms per config-1 gradient evaluation); 1 (3): the same
  // at the lowest (highest) stream priority; 0: the adjoint starts once every
  // class's forward is done (WG_ADJ_OVERLAP)
  int adj_overlap = 2;
  bool persist = false;                // persistent launches (WG_BATCH_PERSISTENT)
  int* d_err = nullptr;                // error bits of an evaluation: 1 dependency wait, 2 bulk-copy wait
  int* h_perr = nullptr;               // the last evaluation's error bits (pinned)
  int persist_spin_cap = 1 << 22, persist_wait_unset = 0;
  int n_checkpointed = 0;              // size classes that recompute their tables per level
  std::vector<std::unique_ptr<SubBatch>> subs;
  std::vector<int> fam_sub, fam_local;
  std::vector<int> nrow;
  int4* d_mnode = nullptr;
  int* d_rowoff = nullptr;
  double* d_leafp = nullptr;
  double* d_params = nullptr;
  double* d_logl = nullptr;
  double* h_params = nullptr;
  double* h_logl = nullptr;
  double* h_gred = nullptr;  // P per sub-batch
  bool grad_pending = false;
  bool pending = false;  // an enqueued evaluation has not been fetched yet
  bool tables_fresh = false;  // d_tabs and h_logl hold the last fetched evaluation (WG_BATCH_TABLES)
  int launches[2] = {0, 0};  // kernels per recorded sequence: [forward only, with gradient]
  std::vector<wg_ccd*> ccds;  // not owned; for the lazily built plain layout
  std::unique_ptr<PlainBatch> plain;
  // per-family adjoint weights (wg_logpdf_grad_weighted)
  double* d_famw = nullptr;
  double* h_famw = nullptr;
  bool weighted_pending = false;
  double cond_scale = 0.0;  // of the pending weighted evaluation
  // NowhereExtinctCondition on the device, forked beside the DP
  std::unique_ptr<NwPlan> nw;
  bool nw_pending = false;
  std::unique_ptr<TrackData> track;  // device backtracking (wg_track_device)
  // captured launch sequences: [with gradient][with tables][weighted][nowhere]
  cudaGraphExec_t graph[2][2][2][2] = {};
  void drop_graphs(int nowhere) {
    for (auto& g3 : graph)
      for (auto& g2 : g3)
        for (auto& g1 : g2)
          if (g1[nowhere]) {
            cudaGraphExecDestroy(g1[nowhere]);
            g1[nowhere] = nullptr;
          }
  }
  ~wg_batch() {
    drop_graphs(0);
    drop_graphs(1);
    nw.reset();
    track.reset();
    if (ctx) free_all(ctx->device, {d_famw}, {h_famw});
    plain.reset();
    subs.clear();
    if (ctx)
      free_all(ctx->device, {d_mnode, d_rowoff, d_leafp, d_params, d_logl, d_err}, {h_params, h_logl, h_gred, h_perr});
  }
};

namespace {

template <class B>
void upload_model_static(B* b, const wg_model* m, cudaStream_t s) {
  int64_t& by = b->device_bytes;
  b->d_mnode = dalloc<int4>(m->K, by);
  b->d_rowoff = dalloc<int>(m->K + 1, by);
  b->d_leafp = dalloc<double>(m->K, by);
  std::vector<int4> mn(m->K);
  for (int k = 0; k < m->K; ++k) mn[k] = make_int4(m->kind[k], m->ch0[k], m->ch1[k], m->nrow[k]);
  h2d(b->d_mnode, mn, s);
  h2d(b->d_rowoff, m->row_off, s);
  h2d(b->d_leafp, m->leaf_p, s);
}

std::unique_ptr<PlainBatch> build_plain(wg_ctx* ctx, const wg_model* m, wg_ccd* const* ccds, int n) {
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  std::vector<const CCD*> cs(ccds, ccds + n);
  PackOptions opt;
  opt.single = true;
  Packed P = pack_batch(*m, cs, opt);
  auto b = std::make_unique<PlainBatch>();
  b->ctx = ctx;
  b->K = m->K;
  b->NR = m->total_rows();
  b->NF = n;
  b->n_groups = (int)P.groups.size();
  b->P = 3 * b->NR + b->K + 1;
  b->smem_fwd = (size_t)P.max_smem_doubles * sizeof(double);
  if (b->smem_fwd > ctx->smem_optin) throw Error(WG_ERANGE, "a family needs more shared memory than one CTA holds");
  cudaStream_t s = ctx->stream;
  int64_t& by = b->device_bytes;
  b->d_groups = dalloc<DGroup>(P.groups.size(), by);
  b->d_nodes = dalloc<DNode>(P.nodes.size(), by);
  b->d_entries = dalloc<DEntry>(P.entries.size(), by);
  b->d_meta = dalloc<int>(P.meta.size(), by);
  b->d_levels = dalloc<DLevel>(P.levels.size(), by);
  b->d_famidx = dalloc<int>(P.fam_idx.size(), by);
  b->d_fampos = dalloc<int>(P.fam_pos.size(), by);
  b->d_params = dalloc<double>(b->P, by);
  b->d_tops = dalloc<double>(P.tops_doubles, by);
  b->d_logl = dalloc<double>(n, by);
  h2d(b->d_groups, P.groups, s);
  h2d(b->d_nodes, P.nodes, s);
  h2d(b->d_entries, P.entries, s);
  h2d(b->d_meta, P.meta, s);
  h2d(b->d_levels, P.levels, s);
  h2d(b->d_famidx, P.fam_idx, s);
  h2d(b->d_fampos, P.fam_pos, s);
  upload_model_static(b.get(), m, s);
  ck(cudaMallocHost(&b->h_params, sizeof(double) * b->P), "cudaMallocHost");
  ck(cudaMallocHost(&b->h_logl, sizeof(double) * n), "cudaMallocHost");
  ck(cudaStreamSynchronize(s), "plain batch upload");
  return b;
}

KArgs plain_args(const PlainBatch* b) {
  KArgs A;
  A.groups = b->d_groups;
  A.nodes = b->d_nodes;
  A.entries = b->d_entries;
  A.meta = b->d_meta;
  A.levels = b->d_levels;
  A.fam_idx = b->d_famidx;
  A.fam_pos = b->d_fampos;
  A.mnode = b->d_mnode;
  A.row_off = b->d_rowoff;
  A.leafp = b->d_leafp;
  A.params = b->d_params;
  A.tops = b->d_tops;
  A.tabs = nullptr;
  A.bartops = nullptr;
  A.logl = b->d_logl;
  A.K = b->K;
  A.NR = b->NR;
  return A;
}

// Size classes by clade count (upper bounds); one layout per non-empty class.
// Families are split by clade count into size classes, each packed on its
// own and run on its own pair of streams: the levels of one class do not wait
// for the levels of another.  Larger classes carry the critical paths and get
// higher stream priorities, so their CTAs are dispatched first.
// (192, 512, 1536): measured best of 13 bound sets on config 1 with each
// class's adjoint on its own forward's heels (1.570 ms per gradient
// evaluation against 1.615 ms for (128, 256, 512, 1024, 1536)).
constexpr int kClassBounds[] = {192, 512, 1536, 1 << 30};

// The size classes' upper bounds: WG_CLASS_BOUNDS (increasing clade counts,
// comma-separated, at most 7; a last class takes the rest), else the above.
std::vector<int> class_bounds() {
  const char* e = std::getenv("WG_CLASS_BOUNDS");
  if (!e || !*e) return std::vector<int>(std::begin(kClassBounds), std::end(kClassBounds));
  std::vector<int> v;
  const char* p = e;
  while (*p) {
    char* end = nullptr;
    const long x = std::strtol(p, &end, 10);
    if (end == p || x < 1 || x >= (1 << 30) || (!v.empty() && x <= v.back()))
      throw Error(WG_EINVAL, "WG_CLASS_BOUNDS is not an increasing list of clade counts");
    v.push_back((int)x);
    p = end;
    if (*p == ',') ++p;
    else if (*p) throw Error(WG_EINVAL, "WG_CLASS_BOUNDS is not an increasing list of clade counts");
  }
  if (v.size() > 7) throw Error(WG_EINVAL, "WG_CLASS_BOUNDS: at most 7 bounds");
  v.push_back(1 << 30);
  return v;
}

// Device bytes of a packed class other than its tables.
int64_t class_other_bytes(const Packed2& P, bool adjoint, int P_params) {
  int64_t by = (int64_t)(P.tasks.size() * sizeof(DTask) + P.entries.size() * sizeof(DEntry) +
                         P.meta.size() * sizeof(int32_t) + P.gmap.size() * sizeof(int64_t) +
                         P.progs.size() * sizeof(DProg2) + P.tasks.size() * sizeof(int32_t));
  by += 8 * (P.tops_doubles + P.scratch_doubles);
  if (adjoint)
    by += 8 * (P.tops_doubles + P.gout_doubles + P_params) +
          (int64_t)(P.red_off.size() + P.red_idx.size()) * (int64_t)sizeof(int64_t);
  return by;
}

// Table budget of a gradient batch: WG_TABLE_BUDGET_BYTES, else the device
// memory free now less the batch's other buffers and a 1 GiB reserve.
int64_t table_budget(int64_t other_bytes) {
  const char* e = std::getenv("WG_TABLE_BUDGET_BYTES");
  if (e && *e) {
    char* end = nullptr;
    const long long v = std::strtoll(e, &end, 10);
    if (end == e || *end != '\0' || v < 0) throw Error(WG_EINVAL, "WG_TABLE_BUDGET_BYTES is not a byte count");
    return (int64_t)v;
  }
  size_t fr = 0, tot = 0;
  ck(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
  return (int64_t)fr - other_bytes - ((int64_t)1 << 30);
}

std::unique_ptr<wg_batch> build_batch(wg_ctx* ctx, const wg_model* m, wg_ccd* const* ccds, int n, uint32_t flags) {
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  for (int i = 0; i < n; ++i)
    if (!ccds[i]) throw Error(WG_EINVAL, "null CCD in batch");
  auto b = std::make_unique<wg_batch>();
  b->ctx = ctx;
  b->K = m->K;
  b->NR = m->total_rows();
  b->NF = n;
  b->flags = flags;
  b->P = 3 * b->NR + b->K + 1;
  b->nrow = m->nrow;
  b->fam_sub.assign(n, -1);
  b->fam_local.assign(n, -1);
  cudaStream_t s = ctx->stream;
  int64_t& by = b->device_bytes;
  const bool adjoint = (flags & WG_BATCH_GRAD) != 0;
  const bool keep = (flags & (WG_BATCH_GRAD | WG_BATCH_TABLES)) != 0;
  // ---- pack every size class on the host
  struct Cls {
    int cls;
    std::vector<int> ids;
    Packed2 P;
    bool checkpoint = false;
  };
  std::vector<Cls> cl;
  int lo = 0;
  int cls = -1;
  // persistent launches: one layout of 128-thread tasks whose shared memory
  // fits WG_PERSIST_CTAS (default 3) CTAs per SM; wider tasks keep their rows
  // in device memory
  b->persist = (flags & WG_BATCH_PERSISTENT) != 0;
  b->adj_overlap = (int)pack_knob("WG_ADJ_OVERLAP", 2, 0, 3);
  const int64_t pctas = pack_knob("WG_PERSIST_CTAS", 3, 1, 8);
  // (an SM's shared memory split over pctas CTAs, less the 1 KB the
  // hardware reserves per CTA and a margin for the kernels' static variables)
  const int64_t pcap = std::min<int64_t>((int64_t)ctx->smem_optin, (int64_t)ctx->smem_sm / pctas - 1024) /
                           (int64_t)sizeof(double) - 64;
  b->persist_spin_cap = (int)pack_knob("WG_PERSIST_SPIN_CAP", 1 << 22, 0, 1 << 30);
  b->persist_wait_unset = (int)pack_knob("WG_PERSIST_TEST_UNSET_WAIT", 0, 0, 1);
  std::vector<int> bounds = b->persist ? std::vector<int>{1 << 30} : class_bounds();
  for (const int bound : bounds) {
    ++cls;
    std::vector<int> ids;
    for (int i = 0; i < n; ++i)
      if (ccds[i]->n_clades > lo && ccds[i]->n_clades <= bound) ids.push_back(i);
    lo = bound;
    if (ids.empty()) continue;
    std::vector<const CCD*> cs;
    for (int i : ids) cs.push_back(ccds[i]);
    PackOptions2 opt;
    opt.adjoint = adjoint;
    opt.keep_tables = keep;
    opt.global_ids = &ids;
    // (a little below the opt-in size: the kernels' static shared variables)
    opt.smem_limit_doubles = (flags & WG_BATCH_SCRATCH_ROWS) ? 0 : (int64_t)(ctx->smem_optin / sizeof(double)) - 32;
    // per-class threshold of the 256-thread tasks (WG_PACK_HEAVY_OPS_C<class>)
    opt.heavy_ops = pack_knob(("WG_PACK_HEAVY_OPS_C" + std::to_string(cls)).c_str(), opt.heavy_ops, 32, 1 << 20);
    if (b->persist) {
      opt.light_only = true;
      opt.root_smem_doubles = pcap;
      if (!(flags & WG_BATCH_SCRATCH_ROWS)) opt.smem_limit_doubles = pcap;
    }
    Cls c;
    c.cls = cls;
    c.P = pack_batch2(*m, cs, opt);
    c.ids = std::move(ids);
    if ((size_t)c.P.max_smem * sizeof(double) > ctx->smem_optin)
      throw Error(WG_ERANGE, "a task needs more shared memory than one CTA can hold");
    cl.push_back(std::move(c));
  }
  // ---- per-branch checkpoint/recompute where the tables would not fit
  b->tab_full = 0;
  for (auto& c : cl) b->tab_full += c.P.tab_doubles;
  if (adjoint && !(flags & WG_BATCH_TABLES)) {
    if (flags & WG_BATCH_CHECKPOINT) {
      for (auto& c : cl) {
        c.checkpoint = true;
        checkpoint_tables(c.P, *m);
      }
    } else {
      int64_t other = 0, tabs = 0;
      for (auto& c : cl) {
        other += class_other_bytes(c.P, adjoint, b->P);
        tabs += 8 * c.P.tab_doubles;
      }
      const int64_t budget = table_budget(other);
      if (tabs > budget) {
        // largest tables first, until the rest fit
        std::vector<size_t> order(cl.size());
        for (size_t i = 0; i < cl.size(); ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](size_t x, size_t y) { return cl[x].P.tab_doubles > cl[y].P.tab_doubles; });
        for (size_t i : order) {
          if (tabs <= budget) break;
          Cls& c = cl[i];
          const int64_t full = c.P.tab_doubles;
          c.checkpoint = true;
          const int64_t kept = checkpoint_tables(c.P, *m);
          tabs -= 8 * (full - kept);
        }
      }
    }
  }
  int prio_lo = 0, prio_hi = 0;
  ck(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi), "priority range");
  for (auto& c : cl) {
    Packed2& P = c.P;
    const std::vector<int>& ids = c.ids;
    auto sb = std::make_unique<SubBatch>();
    sb->device = ctx->device;
    sb->checkpoint = c.checkpoint;
    sb->fam = ids;
    sb->n_tasks = (int)P.tasks.size();
    sb->fam_tab = P.fam_tab;
    sb->fam_w = P.fam_w;
    sb->fam_col = P.fam_col;
    sb->fam_ncol = P.fam_ncol;
    b->n_tasks += sb->n_tasks;
    b->flops_fwd += P.flops_fwd;
    b->bytes_fwd += P.bytes_fwd;
    b->flops_adj += P.flops_adj;
    b->tab_kept += P.tab_doubles;
    if (c.checkpoint) ++b->n_checkpointed;
    for (size_t i = 0; i < ids.size(); ++i) {
      b->fam_sub[ids[i]] = (int)b->subs.size();
      b->fam_local[ids[i]] = (int)i;
    }
    if ((!P.levels_h.empty() && !P.levels_h.back().empty()) || (!P.levels_gh.empty() && !P.levels_gh.back().empty()))
      throw Error(WG_ESTATE, "internal: heavy task at the root level");
    for (size_t L = 0; L < P.levels.size(); ++L)
      for (auto* lv : {&P.levels[L], &P.levels_g[L]})
        for (int t : *lv)
          if ((m->kind[P.tasks[t].node] == WG_NODE_ROOT) != (L + 1 == P.levels.size()))
            throw Error(WG_ESTATE, "internal: root tasks must form the top level");
    std::vector<int> lists;
    for (size_t L = 0; L < P.levels.size(); ++L) {
      sb->lvl_off.push_back((int)lists.size());
      sb->lvl_n.push_back((int)P.levels[L].size());
      sb->lvl_smem.push_back((size_t)P.level_smem[L] * sizeof(double));
      sb->lvl_smem_adj.push_back((size_t)P.level_smem_adj[L] * sizeof(double));
      lists.insert(lists.end(), P.levels[L].begin(), P.levels[L].end());
      sb->lvlh_off.push_back((int)lists.size());
      sb->lvlh_n.push_back((int)P.levels_h[L].size());
      sb->lvlh_smem.push_back((size_t)P.level_smem_h[L] * sizeof(double));
      sb->lvlh_smem_adj.push_back((size_t)P.level_smem_adj_h[L] * sizeof(double));
      lists.insert(lists.end(), P.levels_h[L].begin(), P.levels_h[L].end());
      sb->lvlg_off.push_back((int)lists.size());
      sb->lvlg_n.push_back((int)P.levels_g[L].size());
      lists.insert(lists.end(), P.levels_g[L].begin(), P.levels_g[L].end());
      sb->lvlgh_off.push_back((int)lists.size());
      sb->lvlgh_n.push_back((int)P.levels_gh[L].size());
      lists.insert(lists.end(), P.levels_gh[L].begin(), P.levels_gh[L].end());
    }
    if (P.scratch_doubles > 0) sb->d_scratch = dalloc<double>(P.scratch_doubles, by);
    sb->d_tasks = dalloc<DTask>(P.tasks.size(), by);
    sb->d_entries = dalloc<DEntry>(P.entries.size(), by);
    sb->d_meta = dalloc<int>(P.meta.size(), by);
    sb->d_gmap = dalloc<int64_t>(P.gmap.size(), by);
    sb->d_progs = dalloc<DProg2>(P.progs.size(), by);
    sb->d_lists = dalloc<int>(lists.size(), by);
    sb->d_tops = dalloc<double>(P.tops_doubles, by);
    sb->tops_doubles = P.tops_doubles;
    if (keep) sb->d_tabs = dalloc<double>(P.tab_doubles, by);
    if (adjoint) {
      sb->d_bartops = dalloc<double>(P.tops_doubles, by);
      sb->gout_doubles = P.gout_doubles;
      sb->d_gout = dalloc<double>(P.gout_doubles, by);
      sb->d_gred = dalloc<double>(b->P, by);
      sb->d_red_off = dalloc<int64_t>(P.red_off.size(), by);
      sb->d_red_idx = dalloc<int64_t>(P.red_idx.size(), by);
      h2d(sb->d_red_off, P.red_off, s);
      h2d(sb->d_red_idx, P.red_idx, s);
    }
    h2d(sb->d_tasks, P.tasks, s);
    h2d(sb->d_entries, P.entries, s);
    h2d(sb->d_meta, P.meta, s);
    h2d(sb->d_gmap, P.gmap, s);
    h2d(sb->d_progs, P.progs, s);
    h2d(sb->d_lists, lists, s);
    // persistent launches need every table kept (a checkpointed class keeps
    // its level launches)
    sb->persist = b->persist && !c.checkpoint;
    if (sb->persist) {
      const Schedule S = persistent_schedule(P);
      const int nt = sb->n_tasks;
      std::vector<int> ord(S.order_fwd.begin(), S.order_fwd.end());
      ord.insert(ord.end(), S.order_adj.begin(), S.order_adj.end());
      std::vector<int> dep(S.fdep_off.begin(), S.fdep_off.end());
      dep.insert(dep.end(), S.fdep_idx.begin(), S.fdep_idx.end());
      sb->n_pdep_f = (int)dep.size();
      dep.insert(dep.end(), S.adep_off.begin(), S.adep_off.end());
      dep.insert(dep.end(), S.adep_idx.begin(), S.adep_idx.end());
      sb->n_pdep_a = (int)dep.size() - sb->n_pdep_f;
      sb->d_porder = dalloc<int>(ord.size(), by);
      sb->d_pdep = dalloc<int>(dep.size(), by);
      sb->d_pdone = dalloc<int>((size_t)nt + 1, by);
      sb->d_pctl = dalloc<int>(2, by);
      h2d(sb->d_porder, ord, s);
      h2d(sb->d_pdep, dep, s);
      ck(cudaMemsetAsync(sb->d_pdone, 0, sizeof(int) * ((size_t)nt + 1), s), "memset");
      ck(cudaMemsetAsync(sb->d_pctl, 0, sizeof(int) * 2, s), "memset");
      int sf = 0, sa = 0;
      for (const DTask& T : P.tasks)
        if (T.scratch < 0) {
          sf = std::max(sf, T.smem);
          sa = std::max(sa, T.smem_adj);
        }
      sb->psmem_f = (size_t)sf * sizeof(double);
      sb->psmem_a = (size_t)sa * sizeof(double);
      int nbf = 0, nba = 0;
      ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbf, k_fwd_persist<true>, kNT2L, sb->psmem_f), "occupancy");
      ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nba, k_adj_persist, kNT2L, sb->psmem_a), "occupancy");
      if (nbf < 1 || (adjoint && nba < 1)) throw Error(WG_ERANGE, "persistent launch does not fit on an SM");
      sb->pgrid_f = std::min(nt, nbf * ctx->n_sm);
      sb->pgrid_a = std::min(nt, std::max(nba, 1) * ctx->n_sm);
    }
    {
      // priority grows (numerically falls) with the class
      const int pr = std::max(prio_hi, prio_lo - c.cls);
      ck(cudaStreamCreateWithPriority(&sb->s, cudaStreamNonBlocking, pr), "cudaStreamCreate");
      ck(cudaStreamCreateWithPriority(&sb->s2, cudaStreamNonBlocking, pr), "cudaStreamCreate");
      if (b->adj_overlap) {
        const int pa = b->adj_overlap == 1 ? prio_lo : b->adj_overlap == 3 ? prio_hi : pr;
        ck(cudaStreamCreateWithPriority(&sb->sa, cudaStreamNonBlocking, pa), "cudaStreamCreate");
        ck(cudaStreamCreateWithPriority(&sb->sa2, cudaStreamNonBlocking, pa), "cudaStreamCreate");
      }
    }
    for (cudaEvent_t* e : {&sb->fork, &sb->join, &sb->done})
      ck(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
    // the host copy of this class is no longer needed once its uploads landed
    ck(cudaStreamSynchronize(s), "batch upload");
    std::vector<DTask>().swap(P.tasks);
    decltype(P.entries)().swap(P.entries);
    std::vector<int64_t>().swap(P.gmap);
    b->subs.push_back(std::move(sb));
  }
  b->d_params = dalloc<double>(b->P + 2, by);
  b->d_logl = dalloc<double>(n, by);
  b->d_err = dalloc<int>(1, by);
  ck(cudaMemsetAsync(b->d_err, 0, sizeof(int), s), "memset");
  upload_model_static(b.get(), m, s);
  ck(cudaMallocHost(&b->h_params, sizeof(double) * (b->P + 2)), "cudaMallocHost");
  ck(cudaMallocHost(&b->h_logl, sizeof(double) * n), "cudaMallocHost");
  if (adjoint) ck(cudaMallocHost(&b->h_gred, sizeof(double) * b->P * b->subs.size()), "cudaMallocHost");
  ck(cudaMallocHost(&b->h_perr, sizeof(int)), "cudaMallocHost");
  *b->h_perr = 0;
  ck(cudaStreamSynchronize(s), "batch upload");
  b->ccds.assign(ccds, ccds + n);
  return b;
}

KArgs2 sub_args(const wg_batch* b, const SubBatch* sb) {
  KArgs2 A;
  A.tasks = sb->d_tasks;
  A.entries = sb->d_entries;
  A.meta = sb->d_meta;
  A.gmap = sb->d_gmap;
  A.progs = sb->d_progs;
  A.mnode = b->d_mnode;
  A.row_off = b->d_rowoff;
  A.leafp = b->d_leafp;
  A.params = b->d_params;
  A.tops = sb->d_tops;
  A.tabs = sb->d_tabs;
  A.bartops = sb->d_bartops;
  A.gout = sb->d_gout;
  A.logl = b->d_logl;
  A.scratch = sb->d_scratch;
  A.famw = nullptr;
  A.err = b->d_err;
  A.NR = b->NR;
  A.K = b->K;
  return A;
}

template <class B>
void check_model(const B* b, const wg_model* m) {
  if (!m->has_params) throw Error(WG_ESTATE, "model parameters not set (wg_model_set_rates / wg_model_set_tables)");
  if (m->K != b->K || m->total_rows() != b->NR) throw Error(WG_EINVAL, "batch was built for a different model");
}

// One level of one size class: heavy tasks on the class's second stream,
// light ones on its first, joined before the next level (each side also
// launches its tasks whose rows live in device scratch).
template <class Light, class Heavy>
void run_level(SubBatch* sb, int L, Light light, Heavy heavy, cudaStream_t s1 = nullptr, cudaStream_t s2 = nullptr) {
  if (!s1) s1 = sb->s, s2 = sb->s2;
  const bool h = sb->lvlh_n[L] + sb->lvlgh_n[L] > 0, l = sb->lvl_n[L] + sb->lvlg_n[L] > 0;
  if (h && l) {
    ck(cudaEventRecord(sb->fork, s1), "event");
    ck(cudaStreamWaitEvent(s2, sb->fork, 0), "wait");
    heavy(s2);
    light(s1);
    ck(cudaEventRecord(sb->join, s2), "event");
    ck(cudaStreamWaitEvent(s1, sb->join, 0), "wait");
  } else if (h) {
    heavy(s1);
  } else if (l) {
    light(s1);
  }
}

// The context stream forks to every size class and joins them again.
void fork_subs(wg_batch* b) {
  wg_ctx* ctx = b->ctx;
  ck(cudaEventRecord(ctx->fork, ctx->stream), "event");
  for (auto& sb : b->subs) ck(cudaStreamWaitEvent(sb->s, ctx->fork, 0), "wait");
}
void join_subs(wg_batch* b) {
  wg_ctx* ctx = b->ctx;
  for (auto& sb : b->subs) {
    ck(cudaEventRecord(sb->done, sb->s), "event");
    ck(cudaStreamWaitEvent(ctx->stream, sb->done, 0), "wait");
  }
}

// Parameters of one evaluation in the pinned staging buffer: ε, ϕ, ψ per row,
// q per node, η, then the root-row constants of whaleroot! (src/core.jl:
// 130-149) ca = (1-η)ξ/η and cb = η(1-ε)/ξ² with ξ = 1-(1-η)ε, ε the top ε of
// the root, which every root task would otherwise recompute.
void stage_params(wg_batch* b, const wg_model* m) {
  const int NR = b->NR, K = b->K;
  double* h = b->h_params;
  std::memcpy(h, m->eps.data(), NR * sizeof(double));
  std::memcpy(h + NR, m->phi.data(), NR * sizeof(double));
  std::memcpy(h + 2 * NR, m->psi.data(), NR * sizeof(double));
  for (int k = 0; k < K; ++k) h[3 * NR + k] = std::isnan(m->q[k]) ? 0.0 : m->q[k];
  const double eta = m->eta;
  h[3 * NR + K] = eta;
  int root = -1;
  for (int k = 0; k < K; ++k)
    if (m->kind[k] == WG_NODE_ROOT) root = k;
  const double er = root >= 0 ? m->eps_top(root) : 0.0;
  const double xi = 1.0 - (1.0 - eta) * er;
  h[3 * NR + K + 1] = (1.0 - eta) * xi / eta;
  h[3 * NR + K + 2] = eta * (1.0 - er) / (xi * xi);
}

// Every class's forward levels (and the reverse levels of the adjoint plus
// its gradient reduction), forked from and joined back to the context stream.
void record_sequence(wg_batch* b, bool grad, bool tables, bool weighted, bool nowhere) {
  wg_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  int& nl = b->launches[grad ? 1 : 0];
  nl = 0;
  ck(cudaMemcpyAsync(b->d_params, b->h_params, sizeof(double) * (b->P + 2), cudaMemcpyHostToDevice, s),
     "params upload");
  ck(cudaMemsetAsync(b->d_err, 0, sizeof(int), s), "memset");
  if (nowhere) {  // the condition depends on the rates only: beside the DP
    NwPlan& p = *b->nw;
    ck(cudaEventRecord(p.fork, s), "event");
    ck(cudaStreamWaitEvent(p.s, p.fork, 0), "wait");
    nl += nw_record(p, p.s, grad);
    ck(cudaEventRecord(p.done, p.s), "event");
  }
  auto join_nw = [&] {
    if (nowhere) ck(cudaStreamWaitEvent(s, b->nw->done, 0), "wait");
  };
  if (weighted)
    ck(cudaMemcpyAsync(b->d_famw, b->h_famw, sizeof(double) * b->NF, cudaMemcpyHostToDevice, s), "weights upload");
  if (grad)
    for (auto& sb : b->subs)
      ck(cudaMemsetAsync(sb->d_gout, 0, sizeof(double) * (size_t)sb->gout_doubles, s), "memset");
  // the forward launches of one height level of one class; tab: the tasks
  // store their DP tables
  auto fwd_level = [&](SubBatch* sb, const KArgs2& A, int L, bool tab) {
    const int top = (int)sb->lvl_n.size() - 1;  // the root level
    const int* ll = sb->d_lists + sb->lvl_off[L];
    const int* lh = sb->d_lists + sb->lvlh_off[L];
    run_level(
        sb, L,
        [&](cudaStream_t st) {
          const dim3 g(sb->lvl_n[L]), gg(sb->lvlg_n[L]);
          const size_t sm = sb->lvl_smem[L];
          const int* lg = sb->d_lists + sb->lvlg_off[L];
          if (sb->lvl_n[L] > 0) {
            ++nl;
            if (L == top && tab) k_fwd2<true, kNT2L, true><<<g, kNT2L, sm, st>>>(A, ll);
            else if (L == top) k_fwd2<false, kNT2L, true><<<g, kNT2L, sm, st>>>(A, ll);
            else if (tab) k_fwd2<true, kNT2L><<<g, kNT2L, sm, st>>>(A, ll);
            else k_fwd2<false, kNT2L><<<g, kNT2L, sm, st>>>(A, ll);
          }
          if (sb->lvlg_n[L] > 0) {
            ++nl;
            if (L == top && tab) k_fwd2<true, kNT2L, true, true><<<gg, kNT2L, 0, st>>>(A, lg);
            else if (L == top) k_fwd2<false, kNT2L, true, true><<<gg, kNT2L, 0, st>>>(A, lg);
            else if (tab) k_fwd2<true, kNT2L, false, true><<<gg, kNT2L, 0, st>>>(A, lg);
            else k_fwd2<false, kNT2L, false, true><<<gg, kNT2L, 0, st>>>(A, lg);
          }
        },
        [&](cudaStream_t st) {
          const int* lgh = sb->d_lists + sb->lvlgh_off[L];
          if (sb->lvlh_n[L] > 0) {
            ++nl;
            if (tab) k_fwd2<true, kNT2H><<<sb->lvlh_n[L], kNT2H, sb->lvlh_smem[L], st>>>(A, lh);
            else k_fwd2<false, kNT2H><<<sb->lvlh_n[L], kNT2H, sb->lvlh_smem[L], st>>>(A, lh);
          }
          if (sb->lvlgh_n[L] > 0) {
            ++nl;
            if (tab) k_fwd2<true, kNT2H, false, true><<<sb->lvlgh_n[L], kNT2H, 0, st>>>(A, lgh);
            else k_fwd2<false, kNT2H, false, true><<<sb->lvlgh_n[L], kNT2H, 0, st>>>(A, lgh);
          }
        });
  };
  // one persistent pass of a class: flags and ticket cleared, then the kernel
  auto persist_args = [&](SubBatch* sb, bool adj) {
    PArgs P;
    P.order = sb->d_porder + (adj ? sb->n_tasks : 0);
    P.dep_off = sb->d_pdep + (adj ? sb->n_pdep_f : 0);
    P.dep_idx = P.dep_off + sb->n_tasks + 1;
    P.done = sb->d_pdone;
    P.ticket = sb->d_pctl;
    P.err = b->d_err;
    P.n = sb->n_tasks;
    P.spin_cap = b->persist_spin_cap;
    P.wait_unset = b->persist_wait_unset;
    ck(cudaMemsetAsync(sb->d_pdone, 0, sizeof(int) * ((size_t)sb->n_tasks + 1), sb->s), "memset");
    ck(cudaMemsetAsync(sb->d_pctl, 0, sizeof(int), sb->s), "memset");
    return P;
  };
  ck(cudaEventRecordWithFlags(ctx->ev[0], s, cudaEventRecordExternal), "event");
  fork_subs(b);
  for (auto& sbp : b->subs) {
    SubBatch* sb = sbp.get();
    KArgs2 A = sub_args(b, sb);
    A.famw = weighted ? b->d_famw : nullptr;
    if (sb->persist) {
      const PArgs P = persist_args(sb, false);
      ++nl;
      if (tables) k_fwd_persist<true><<<sb->pgrid_f, kNT2L, sb->psmem_f, sb->s>>>(A, P);
      else k_fwd_persist<false><<<sb->pgrid_f, kNT2L, sb->psmem_f, sb->s>>>(A, P);
      continue;
    }
    // a checkpointed class keeps no tables in the forward: its adjoint
    // recomputes them level by level
    for (int L = 0; L < (int)sb->lvl_n.size(); ++L) fwd_level(sb, A, L, tables && !sb->checkpoint);
  }
  ck(cudaGetLastError(), "forward launch");
  // a class's adjoint on its own forward's heels (adj_overlap): its adjoint
  // streams wait for its forward only
  const bool ovl = grad && b->adj_overlap > 0;
  if (ovl)
    for (auto& sb : b->subs)
      if (sb->sa && !sb->persist && !sb->checkpoint) {
        ck(cudaEventRecord(sb->done, sb->s), "event");
        ck(cudaStreamWaitEvent(sb->sa, sb->done, 0), "wait");
      }
  join_subs(b);
  if (!grad) join_nw();
  ck(cudaEventRecordWithFlags(ctx->ev[1], s, cudaEventRecordExternal), "event");
  if (grad) {
    fork_subs(b);
    for (auto& sbp : b->subs) {
      SubBatch* sb = sbp.get();
      KArgs2 A = sub_args(b, sb);
      A.famw = weighted ? b->d_famw : nullptr;
      const int top = (int)sb->lvl_n.size() - 1;
      const bool own = ovl && sb->sa && !sb->persist && !sb->checkpoint;
      cudaStream_t a1 = own ? sb->sa : sb->s, a2 = own ? sb->sa2 : sb->s2;
      if (sb->persist) {
        const PArgs P = persist_args(sb, true);
        ++nl;
        k_adj_persist<<<sb->pgrid_a, kNT2L, sb->psmem_a, sb->s>>>(A, P);
      }
      for (int L = sb->persist ? -1 : (int)sb->lvl_n.size() - 1; L >= 0; --L) {
        const int* ll = sb->d_lists + sb->lvl_off[L];
        const int* lh = sb->d_lists + sb->lvlh_off[L];
        // checkpointed class: this level's tables again, from the children's
        // top rows, into the region the level above has finished with
        if (sb->checkpoint) fwd_level(sb, A, L, true);
        run_level(
            sb, L,
            [&](cudaStream_t st) {
              const int* lg = sb->d_lists + sb->lvlg_off[L];
              if (sb->lvl_n[L] > 0) {
                ++nl;
                if (L == top) k_adj2<kNT2L, true><<<sb->lvl_n[L], kNT2L, sb->lvl_smem_adj[L], st>>>(A, ll);
                else k_adj2<kNT2L><<<sb->lvl_n[L], kNT2L, sb->lvl_smem_adj[L], st>>>(A, ll);
              }
              if (sb->lvlg_n[L] > 0) {
                ++nl;
                if (L == top) k_adj2<kNT2L, true, true><<<sb->lvlg_n[L], kNT2L, 0, st>>>(A, lg);
                else k_adj2<kNT2L, false, true><<<sb->lvlg_n[L], kNT2L, 0, st>>>(A, lg);
              }
            },
            [&](cudaStream_t st) {
              const int* lgh = sb->d_lists + sb->lvlgh_off[L];
              if (sb->lvlh_n[L] > 0) {
                ++nl;
                k_adj2<kNT2H><<<sb->lvlh_n[L], kNT2H, sb->lvlh_smem_adj[L], st>>>(A, lh);
              }
              if (sb->lvlgh_n[L] > 0) {
                ++nl;
                k_adj2<kNT2H, false, true><<<sb->lvlgh_n[L], kNT2H, 0, st>>>(A, lgh);
              }
            },
            a1, a2);
      }
      ++nl;
      k_reduce2<<<(b->P * 32 + 255) / 256, 256, 0, a1>>>(sb->d_gout, sb->d_red_off, sb->d_red_idx, b->P, sb->d_gred);
      if (own) {  // back onto the class's stream for the join
        ck(cudaEventRecord(sb->join, a1), "event");
        ck(cudaStreamWaitEvent(sb->s, sb->join, 0), "wait");
      }
    }
    ck(cudaGetLastError(), "adjoint launch");
    join_subs(b);
    join_nw();
    ck(cudaEventRecordWithFlags(ctx->ev[2], s, cudaEventRecordExternal), "event");
    ck(cudaEventRecordWithFlags(ctx->ev[3], s, cudaEventRecordExternal), "event");
  }
  // results to the pinned host buffers, inside the graph: fetch only waits
  ck(cudaMemcpyAsync(b->h_logl, b->d_logl, sizeof(double) * b->NF, cudaMemcpyDeviceToHost, s), "logl download");
  ck(cudaMemcpyAsync(b->h_perr, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "error download");
  if (grad)
    for (size_t i = 0; i < b->subs.size(); ++i)
      ck(cudaMemcpyAsync(b->h_gred + i * b->P, b->subs[i]->d_gred, sizeof(double) * b->P, cudaMemcpyDeviceToHost, s),
         "grad download");
}

// Stage the parameters on the host and replay the captured launch sequence
// (captured into a CUDA graph on first use).
void enqueue(wg_batch* b, const wg_model* m, bool grad, const double* weights = nullptr, double cond_scale = 0.0) {
  check_model(b, m);
  wg_ctx* ctx = b->ctx;
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (grad && !(b->flags & WG_BATCH_GRAD)) throw Error(WG_ESTATE, "batch was created without WG_BATCH_GRAD");
  for (auto& e : ctx->ev)
    if (!e) ck(cudaEventCreate(&e), "cudaEventCreate");
  // the pinned parameter buffer is read by the previous launch's copy
  if (b->pending) ck(cudaStreamSynchronize(ctx->stream), "pending evaluation");
  b->tables_fresh = false;
  stage_params(b, m);
  const bool weighted = weights != nullptr;
  if (weighted) {
    if (!grad) throw Error(WG_EINVAL, "family weights apply to the gradient");
    if (!b->d_famw) {
      ck(cudaMalloc(&b->d_famw, sizeof(double) * b->NF), "cudaMalloc");
      ck(cudaMallocHost(&b->h_famw, sizeof(double) * b->NF), "cudaMallocHost");
    }
    std::memcpy(b->h_famw, weights, sizeof(double) * b->NF);
  }
  b->weighted_pending = weighted;
  b->cond_scale = weighted ? cond_scale : (double)b->NF;
  const bool nowhere = m->cond == WG_COND_NOWHERE;
  if (nowhere) {
    if (!b->nw || !nw_plan_matches(*b->nw, *m)) {
      b->drop_graphs(1);
      b->nw.reset();
      b->nw = nw_plan_create(*m, ctx->device);
    }
    nw_stage(*b->nw, *m);
  }
  b->nw_pending = nowhere;
  const bool tables = grad || (b->flags & WG_BATCH_TABLES);
  cudaGraphExec_t& ge = b->graph[grad][tables][weighted][nowhere];
  cudaStream_t s = ctx->stream;
  if (!ge) {
    ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
      record_sequence(b, grad, tables, weighted, nowhere);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    cudaGraph_t g = nullptr;
    ck(cudaStreamEndCapture(s, &g), "end capture");
    // kernel nodes keep the priorities of the streams they were captured on
    const cudaError_t e = cudaGraphInstantiate(&ge, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    ck(e, "graph instantiate");
  }
  ck(cudaGraphLaunch(ge, s), "graph launch");
  b->pending = true;
  ctx->timed = ctx->timing;
  ctx->timed_grad = grad;
  b->grad_pending = grad;
}

void finish_timing(wg_ctx* ctx) {
  if (!ctx->timed) return;
  ck(cudaEventElapsedTime(&ctx->last_ms[0], ctx->ev[0], ctx->ev[1]), "event time");
  ctx->last_ms[1] = ctx->last_ms[2] = 0.0f;
  if (ctx->timed_grad) {
    ck(cudaEventElapsedTime(&ctx->last_ms[1], ctx->ev[1], ctx->ev[2]), "event time");
    ck(cudaEventElapsedTime(&ctx->last_ms[2], ctx->ev[2], ctx->ev[3]), "event time");
  }
  ctx->timed = false;
}

// The adjoint writes, for a branch whose rows all take the one-dot form,
// E_r = Σ bar_r·L_r per row (summed over tasks into the ∂/∂ϕ slots); the row
// adjoints follow from consecutive E: ∂ϕ_r = (2E_r - E_{r-1})/ϕ_r and
// ∂ψ_r = (E_{r-1} - E_r)/ψ_r.  The choice of form repeats the kernel's test.
void rows_from_sums(const wg_model* m, std::vector<double>& gred) {
  const int NR = m->total_rows();
  for (int k = 0; k < m->K; ++k) {
    const int n = m->nrow[k], o = m->row_off[k];
    if (m->kind[k] == WG_NODE_ROOT || n < 2) continue;
    bool onedot = true;
    for (int r = 1; r < n; ++r) onedot &= m->psi[o + r] >= kPsiOneDot && m->phi[o + r] > 0.0;
    if (!onedot) continue;
    double* dp = gred.data() + NR + o;
    double* ds = gred.data() + 2 * NR + o;
    for (int r = n - 1; r >= 1; --r) {
      const double ehi = dp[r], elo = dp[r - 1];
      dp[r] = (2.0 * ehi - elo) / m->phi[o + r];
      ds[r] = (elo - ehi) / m->psi[o + r];
    }
    dp[0] = 0.0;
  }
}

// Per-family log L, the conditioned total and (for a gradient evaluation) the
// chain from the table adjoints to the rates, on the host.
// Σ w_f log L_f - c·condition and its gradient; unweighted: w = 1, c = N
// (src/core.jl:15, :58-64).
void finish(const wg_model* m, int NF, const double* logl, const double* gred, bool grad, double* per_family,
            double* total, double* d_lam, double* d_mu, double* d_q, double* d_eta, double* d_eps, double* d_phi,
            double* d_psi, const double* weights = nullptr, double cond_scale = -1.0,
            const NwResult* nw = nullptr) {
  double sum = 0.0;
  for (int i = 0; i < NF; ++i) sum += weights ? (weights[i] != 0.0 ? weights[i] * logl[i] : 0.0) : logl[i];
  const double cond = nw ? nw->value : model_condition(*m);
  const double cs = cond_scale < 0 ? (double)NF : cond_scale;
  double tot = sum - cs * cond;
  if (!std::isfinite(tot)) tot = -INFINITY;
  if (per_family) std::memcpy(per_family, logl, sizeof(double) * NF);
  if (total) *total = tot;
  if (!grad) return;
  const int NR = m->total_rows(), K = m->K;
  std::vector<double> de(gred, gred + NR), dp(gred + NR, gred + 2 * NR), ds(gred + 2 * NR, gred + 3 * NR),
      dq(gred + 3 * NR, gred + 3 * NR + K);
  double deta = gred[3 * NR + K];
  model_condition_vjp(*m, -cs, de, deta);
  if (d_eps) std::memcpy(d_eps, de.data(), NR * sizeof(double));
  if (d_phi) std::memcpy(d_phi, dp.data(), NR * sizeof(double));
  if (d_psi) std::memcpy(d_psi, ds.data(), NR * sizeof(double));
  if (m->from_rates) {
    std::vector<double> dl, dm, dpp;
    if (d_lam || d_mu || d_q) model_tables_vjp(*m, de, dp, ds, dl, dm, dq, dpp);
    // a condition on the rates themselves (NowhereExtinct) adds its own adjoints
    if (nw) {
      if (nw->ok) {
        dl.resize(K, 0.0);
        dm.resize(K, 0.0);
        dq.resize(K, 0.0);
        for (int k = 0; k < K; ++k) {
          dl[k] -= cs * nw->d_lam[k];
          dm[k] -= cs * nw->d_mu[k];
          dq[k] -= cs * nw->d_q[k];
        }
        deta -= cs * nw->d_eta;
      }
    } else {
      model_condition_rates_vjp(*m, -cs, dl, dm, dq, deta);
    }
    if (d_lam) std::memcpy(d_lam, dl.data(), K * sizeof(double));
    if (d_mu) std::memcpy(d_mu, dm.data(), K * sizeof(double));
  }
  if (d_eta) *d_eta = deta;
  if (d_q) std::memcpy(d_q, dq.data(), K * sizeof(double));
}

void fetch(wg_batch* b, const wg_model* m, double* per_family, double* total, double* d_lam, double* d_mu,
           double* d_q, double* d_eta, double* d_eps, double* d_phi, double* d_psi) {
  cudaStream_t s = b->ctx->stream;
  const bool grad = b->grad_pending;
  ck(cudaStreamSynchronize(s), "evaluation");  // the graph ends with the result downloads
  b->pending = false;
  if (const int e = *b->h_perr) {
    *b->h_perr = 0;
    throw Error(WG_ECUDA, std::string(e & 1 ? "persistent pass: a wait for a dependency ran out of polls"
                                            : "adjoint: a wait for a bulk copy ran out of polls") +
                              "; the results are invalid");
  }
  b->tables_fresh = (b->flags & WG_BATCH_TABLES) != 0;
  finish_timing(b->ctx);
  std::vector<double> gred;
  if (grad) {  // size classes summed in class order
    gred.assign(b->h_gred, b->h_gred + b->P);
    for (size_t i = 1; i < b->subs.size(); ++i)
      for (int j = 0; j < b->P; ++j) gred[j] += b->h_gred[i * b->P + j];
    rows_from_sums(m, gred);
  }
  NwResult nw;
  if (b->nw_pending) {
    if (m->cond != WG_COND_NOWHERE || !nw_plan_matches(*b->nw, *m))
      throw Error(WG_ESTATE, "the model's condition changed since the evaluation was enqueued");
    nw = nw_result(*b->nw, *m, grad);
  }
  finish(m, b->NF, b->h_logl, gred.data(), grad, per_family, total, d_lam, d_mu, d_q, d_eta, d_eps, d_phi, d_psi,
         b->weighted_pending ? b->h_famw : nullptr, b->cond_scale, b->nw_pending ? &nw : nullptr);
}

void fetch_plain(PlainBatch* b, const wg_model* m, double* per_family, double* total) {
  cudaStream_t s = b->ctx->stream;
  ck(cudaMemcpyAsync(b->h_logl, b->d_logl, sizeof(double) * b->NF, cudaMemcpyDeviceToHost, s), "logl download");
  ck(cudaStreamSynchronize(s), "evaluation");
  finish_timing(b->ctx);
  finish(m, b->NF, b->h_logl, nullptr, false, per_family, total, nullptr, nullptr, nullptr, nullptr, nullptr,
         nullptr, nullptr);
}

// Fixed device scratch of wg_logpdf_noalloc (the top row of every task):
// 1 << 20 doubles (8 MiB), held by every device that loads the library.
constexpr int64_t kNoAllocMaxTops = (int64_t)1 << 20;
__device__ __align__(256) double g_noalloc_tops[kNoAllocMaxTops];

// In host code g_noalloc_tops names a host-side stand-in, not device memory:
// its device address is looked up with the context's device current, when
// the context is created (the module holding it is loaded by then, so the
// lookup allocates nothing), and kept in the context.  A context created
// after a device reset looks it up again.
void noalloc_resolve(wg_ctx* c) {
  void* p = nullptr;
  ck(cudaGetSymbolAddress(&p, g_noalloc_tops), "cudaGetSymbolAddress(g_noalloc_tops)");
  c->noalloc_tops = static_cast<double*>(p);
}

}  // namespace

extern "C" {

int wg_ctx_create(int device, wg_ctx** out) {
  WG_GUARD({
    if (!out) throw Error(WG_EINVAL, "null output");
    int n = 0;
    ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (device < 0 || device >= n) throw Error(WG_EINVAL, "no such CUDA device");
    ck(cudaSetDevice(device), "cudaSetDevice");
    auto c = std::make_unique<wg_ctx>();
    c->device = device;
    ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    int v = 0;
    ck(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device), "attr");
    c->n_sm = v;
    ck(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device), "attr");
    c->smem_sm = (size_t)v;
    ck(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "attr");
    c->smem_optin = (size_t)v;
    ck(cudaFuncSetAttribute(k_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v), "attr");
    ck(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming), "cudaEventCreate");
    // the largest dynamic shared memory every kernel may request: the
    // opt-in size less its own static shared variables
    auto set_dyn_max = [&](const void* fn) {
      cudaFuncAttributes fa;
      ck(cudaFuncGetAttributes(&fa, fn), "attr");
      ck(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, v - (int)fa.sharedSizeBytes), "attr");
    };
    set_dyn_max((const void*)k_fwd2<false, kNT2L>);
    set_dyn_max((const void*)k_fwd2<true, kNT2L>);
    set_dyn_max((const void*)k_fwd2<false, kNT2H>);
    set_dyn_max((const void*)k_fwd2<true, kNT2H>);
    set_dyn_max((const void*)k_fwd2<false, kNT2L, true>);
    set_dyn_max((const void*)k_fwd2<true, kNT2L, true>);
    set_dyn_max((const void*)k_adj2<kNT2L>);
    set_dyn_max((const void*)k_adj2<kNT2L, true>);
    set_dyn_max((const void*)k_adj2<kNT2H>);
    set_dyn_max((const void*)k_fwd_persist<true>);
    set_dyn_max((const void*)k_fwd_persist<false>);
    set_dyn_max((const void*)k_adj_persist);
    noalloc_resolve(c.get());
    *out = c.release();
  });
}

int wg_ctx_destroy(wg_ctx* ctx) {
  if (!ctx) return WG_OK;
  cudaSetDevice(ctx->device);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->fork) cudaEventDestroy(ctx->fork);
  if (ctx->join) cudaEventDestroy(ctx->join);
  if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return WG_OK;
}

void* wg_ctx_stream(wg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int wg_ctx_set_timing(wg_ctx* ctx, int enable) {
  WG_GUARD({
    if (!ctx) throw Error(WG_EINVAL, "null context");
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    for (auto& e : ctx->ev)
      if (!e) ck(cudaEventCreate(&e), "cudaEventCreate");
    ctx->timing = enable != 0;
  });
}

int wg_ctx_timings(wg_ctx* ctx, float* forward_ms, float* adjoint_ms, float* reduce_ms) {
  WG_GUARD({
    if (!ctx) throw Error(WG_EINVAL, "null context");
    if (forward_ms) *forward_ms = ctx->last_ms[0];
    if (adjoint_ms) *adjoint_ms = ctx->last_ms[1];
    if (reduce_ms) *reduce_ms = ctx->last_ms[2];
  });
}

int wg_probe_fp64(wg_ctx* ctx, double* tflops) {
  WG_GUARD({
    if (!ctx || !tflops) throw Error(WG_EINVAL, "bad arguments");
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    double* d = nullptr;
    ck(cudaMalloc(&d, sizeof(double)), "cudaMalloc");
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    const int blocks = ctx->n_sm * 8, threads = 256, iters = 4096;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      ck(cudaEventRecord(e0, ctx->stream), "event");
      k_fp64_probe<<<blocks, threads, 0, ctx->stream>>>(d, iters, 0.999999, 1e-9);
      ck(cudaEventRecord(e1, ctx->stream), "event");
      ck(cudaEventSynchronize(e1), "probe");
      float ms = 0;
      ck(cudaEventElapsedTime(&ms, e0, e1), "event");
      if (rep > 0) best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
  });
}

int wg_batch_create(wg_ctx* ctx, const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags,
                    wg_batch** out) {
  WG_GUARD({
    if (!ctx || !m || !ccds || n_ccds <= 0 || !out) throw Error(WG_EINVAL, "wg_batch_create: bad arguments");
    *out = build_batch(ctx, m, ccds, n_ccds, flags).release();
  });
}

int wg_batch_destroy(wg_batch* b) {
  delete b;
  return WG_OK;
}

int wg_batch_info(const wg_batch* b, int32_t* n_families, int32_t* n_groups, int64_t* device_bytes,
                  double* flops_fwd, double* bytes_fwd, double* flops_adj) {
  WG_GUARD({
    if (!b) throw Error(WG_EINVAL, "null batch");
    if (n_families) *n_families = b->NF;
    if (n_groups) *n_groups = b->n_tasks;
    if (device_bytes) *device_bytes = b->device_bytes;
    if (flops_fwd) *flops_fwd = b->flops_fwd;
    if (bytes_fwd) *bytes_fwd = b->bytes_fwd;
    if (flops_adj) *flops_adj = b->flops_adj;
  });
}

int wg_nowhere_condition(wg_ctx* ctx, const wg_model* m, double* value, double* d_lam, double* d_mu, double* d_q,
                         double* d_eta) {
  WG_GUARD({
    if (!ctx || !m || !value) throw Error(WG_EINVAL, "wg_nowhere_condition: bad arguments");
    if (!m->has_params) throw Error(WG_ESTATE, "model parameters not set");
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (!ctx->nw || !nw_plan_matches(*ctx->nw, *m)) {
      ctx->nw.reset();
      ctx->nw = nw_plan_create(*m, ctx->device);
    }
    NwPlan& p = *ctx->nw;
    const bool grad = d_lam || d_mu || d_q || d_eta;
    nw_stage(p, *m);
    nw_record(p, ctx->stream, grad);
    ck(cudaStreamSynchronize(ctx->stream), "condition");
    const NwResult r = nw_result(p, *m, grad);
    *value = r.value;
    for (int k = 0; grad && k < m->K; ++k) {
      if (d_lam) d_lam[k] = r.ok ? r.d_lam[k] : 0.0;
      if (d_mu) d_mu[k] = r.ok ? r.d_mu[k] : 0.0;
      if (d_q) d_q[k] = r.ok ? r.d_q[k] : 0.0;
    }
    if (d_eta) *d_eta = r.ok ? r.d_eta : 0.0;
  });
}

int wg_batch_tables_layout(const wg_batch* b, int32_t* classes, int32_t* checkpointed, int64_t* full_doubles,
                           int64_t* kept_doubles) {
  WG_GUARD({
    if (!b) throw Error(WG_EINVAL, "null batch");
    if (classes) *classes = (int32_t)b->subs.size();
    if (checkpointed) *checkpointed = b->n_checkpointed;
    if (full_doubles) *full_doubles = b->tab_full;
    if (kept_doubles) *kept_doubles = b->tab_kept;
  });
}

int wg_batch_launches(const wg_batch* b, int32_t* forward, int32_t* gradient) {
  WG_GUARD({
    if (!b) throw Error(WG_EINVAL, "null batch");
    if (forward) *forward = b->launches[0];
    if (gradient) *gradient = b->launches[1];
  });
}

int wg_logpdf(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf: bad arguments");
    enqueue(b, m, false);
    fetch(b, m, per_family, total, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  });
}

int wg_logpdf_grad(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total, double* d_lam,
                   double* d_mu, double* d_q, double* d_eta, double* d_eps, double* d_phi, double* d_psi) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf_grad: bad arguments");
    enqueue(b, m, true);
    fetch(b, m, per_family, total, d_lam, d_mu, d_q, d_eta, d_eps, d_phi, d_psi);
  });
}

int wg_logpdf_grad_weighted(wg_ctx* ctx, wg_model* m, wg_batch* b, const double* weights, double cond_scale,
                            double* per_family, double* total, double* d_lam, double* d_mu, double* d_q,
                            double* d_eta, double* d_eps, double* d_phi, double* d_psi) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx || !weights) throw Error(WG_EINVAL, "wg_logpdf_grad_weighted: bad arguments");
    if (!(cond_scale >= 0.0)) throw Error(WG_EINVAL, "wg_logpdf_grad_weighted: condition scale must be >= 0");
    enqueue(b, m, true, weights, cond_scale);
    fetch(b, m, per_family, total, d_lam, d_mu, d_q, d_eta, d_eps, d_phi, d_psi);
  });
}

int wg_logpdf_plain(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf_plain: bad arguments");
    if (!b->plain) b->plain = build_plain(ctx, m, b->ccds.data(), b->NF);
    PlainBatch* pb = b->plain.get();
    check_model(pb, m);
    cudaStream_t s = ctx->stream;
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    upload_params(m, pb->NR, pb->K, pb->h_params, pb->d_params, s);
    KArgs A = plain_args(pb);
    const DGroup* g0 = pb->d_groups;
    for (int g = 0; g < pb->n_groups; ++g) {  // one family per launch
      A.groups = g0 + g;
      k_forward<false><<<1, kNT, pb->smem_fwd, s>>>(A);
    }
    ck(cudaGetLastError(), "plain launch");
    fetch_plain(pb, m, per_family, total);
  });
}

int wg_logpdf_tables(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t family, double* out, int64_t cap,
                     int64_t* needed, double* logl) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf_tables: bad arguments");
    if (family < 0 || family >= b->NF) throw Error(WG_EINVAL, "family index out of range");
    if (!(b->flags & WG_BATCH_TABLES)) throw Error(WG_ESTATE, "batch was created without WG_BATCH_TABLES");
    const int K = b->K;
    const SubBatch* sb = b->subs[b->fam_sub[family]].get();
    const size_t lf = (size_t)b->fam_local[family];
    int64_t need = 0;
    for (int k = 0; k < K; ++k) need += (int64_t)b->nrow[k] * sb->fam_ncol[lf * K + k];
    if (needed) *needed = need;
    if (!out) return WG_OK;
    if (cap < need) throw Error(WG_ERANGE, "output buffer too small");
    enqueue(b, m, false);
    fetch(b, m, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (logl) *logl = b->h_logl[family];
    cudaStream_t s = ctx->stream;
    int64_t o = 0;
    for (int k = 0; k < K; ++k) {
      const size_t fk = lf * K + k;
      const int nc = sb->fam_ncol[fk];
      if (nc > 0)
        ck(cudaMemcpy2DAsync(out + o, nc * sizeof(double), sb->d_tabs + sb->fam_tab[fk] + sb->fam_col[fk],
                             (size_t)sb->fam_w[fk] * sizeof(double), nc * sizeof(double), b->nrow[k],
                             cudaMemcpyDeviceToHost, s),
           "table download");
      o += (int64_t)b->nrow[k] * nc;
    }
    ck(cudaStreamSynchronize(s), "table download");
  });
}

int wg_batch_tables(wg_ctx* ctx, wg_batch* b, int32_t family, double* out, int64_t cap, int64_t* needed,
                    double* logl) {
  WG_GUARD({
    if (!ctx || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_batch_tables: bad arguments");
    if (family < 0 || family >= b->NF) throw Error(WG_EINVAL, "family index out of range");
    if (!(b->flags & WG_BATCH_TABLES)) throw Error(WG_ESTATE, "batch was created without WG_BATCH_TABLES");
    const int K = b->K;
    const SubBatch* sb = b->subs[b->fam_sub[family]].get();
    const size_t lf = (size_t)b->fam_local[family];
    int64_t need = 0;
    for (int k = 0; k < K; ++k) need += (int64_t)b->nrow[k] * sb->fam_ncol[lf * K + k];
    if (needed) *needed = need;
    if (!out) return WG_OK;
    if (cap < need) throw Error(WG_ERANGE, "output buffer too small");
    if (b->pending || !b->tables_fresh)
      throw Error(WG_ESTATE, "no fetched evaluation of this batch holds its tables (evaluate it first)");
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (logl) *logl = b->h_logl[family];
    cudaStream_t s = ctx->stream;
    int64_t o = 0;
    for (int k = 0; k < K; ++k) {
      const size_t fk = lf * K + k;
      const int nc = sb->fam_ncol[fk];
      if (nc > 0)
        ck(cudaMemcpy2DAsync(out + o, nc * sizeof(double), sb->d_tabs + sb->fam_tab[fk] + sb->fam_col[fk],
                             (size_t)sb->fam_w[fk] * sizeof(double), nc * sizeof(double), b->nrow[k],
                             cudaMemcpyDeviceToHost, s),
           "table download");
      o += (int64_t)b->nrow[k] * nc;
    }
    ck(cudaStreamSynchronize(s), "table download");
  });
}

}  // extern "C"

namespace {

// Species-tree height in nodes (root to deepest leaf, WGD nodes counted).
int tree_height(const wg_model* m) {
  std::vector<int> h(m->K, 0);
  for (int k = 0; k < m->K; ++k)  // children precede parents in the order
    for (int c : {m->ch0[k], m->ch1[k]})
      if (c >= 0) h[k] = std::max(h[k], h[c] + 1);
  return h[m->K - 1];
}

template <class T>
T* upload_vec(const std::vector<T>& v, cudaStream_t s) {
  int64_t by = 0;
  T* d = dalloc<T>(v.size(), by);
  h2d(d, v, s);
  return d;
}

std::unique_ptr<TrackData> build_track(wg_batch* b, const wg_model* m) {
  const int K = b->K, NF = b->NF;
  cudaStream_t s = b->ctx->stream;
  auto td = std::make_unique<TrackData>();
  td->device = b->ctx->device;
  std::vector<int64_t> fk_tab((size_t)NF * K), fclade(NF), fcol(NF), csplit;
  std::vector<int> fk_w((size_t)NF * K), fk_col((size_t)NF * K), fnclade(NF), g1, g2;
  std::vector<int16_t> cols;
  std::vector<double> sp;
  std::vector<unsigned char> cleaf;
  std::vector<const double*> ftabs(NF);
  const int H = tree_height(m);
  td->cap.resize(NF);
  int64_t nsplit = 0;
  for (int f = 0; f < NF; ++f) {
    const SubBatch* sb = b->subs[b->fam_sub[f]].get();
    const size_t lf = (size_t)b->fam_local[f];
    const CCD& c = *b->ccds[f];
    ftabs[f] = sb->d_tabs;
    for (int k = 0; k < K; ++k) {
      const size_t fk = (size_t)f * K + k, lk = lf * K + k;
      fk_tab[fk] = sb->fam_tab[lk];
      fk_w[fk] = sb->fam_w[lk];
      fk_col[fk] = sb->fam_col[lk];
    }
    fclade[f] = (int64_t)cleaf.size();
    fnclade[f] = c.n_clades;
    fcol[f] = (int64_t)cols.size();
    const auto cc = compat_columns(*m, c);
    for (int k = 0; k < K; ++k)
      for (int g = 0; g < c.n_clades; ++g) cols.push_back((int16_t)cc[k][g]);
    for (int g = 0; g < c.n_clades; ++g) {
      csplit.push_back(nsplit + c.split_off[g]);
      cleaf.push_back(c.nleaves[g] == 1 ? 1 : 0);
    }
    nsplit += c.split_off[c.n_clades];
    g1.insert(g1.end(), c.g1.begin(), c.g1.end());
    g2.insert(g2.end(), c.g2.begin(), c.g2.end());
    sp.insert(sp.end(), c.p.begin(), c.p.end());
    // every gene-tree edge crosses at most H + 1 species nodes, each crossing
    // at most one node and one loss
    td->cap[f] = 2 * (2 * (int64_t)std::max(c.n_genes, 1)) * (H + 1) + 8;
  }
  csplit.push_back(nsplit);
  td->d_fk_tab = upload_vec(fk_tab, s);
  td->d_fk_w = upload_vec(fk_w, s);
  td->d_fk_col = upload_vec(fk_col, s);
  td->d_fclade = upload_vec(fclade, s);
  td->d_fnclade = upload_vec(fnclade, s);
  td->d_fcol = upload_vec(fcol, s);
  td->d_cols = upload_vec(cols, s);
  td->d_csplit = upload_vec(csplit, s);
  td->d_g1 = upload_vec(g1, s);
  td->d_g2 = upload_vec(g2, s);
  td->d_sp = upload_vec(sp, s);
  td->d_cleaf = upload_vec(cleaf, s);
  td->d_ftabs = upload_vec(ftabs, s);
  ck(cudaStreamSynchronize(s), "track upload");
  return td;
}

}  // namespace

extern "C" {

int wg_track_device(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t n_trees, const int32_t* families,
                    const uint64_t* seeds, int64_t* offsets) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx || n_trees < 0 || (n_trees > 0 && (!families || !seeds)) || !offsets)
      throw Error(WG_EINVAL, "wg_track_device: bad arguments");
    if (!(b->flags & WG_BATCH_TABLES)) throw Error(WG_ESTATE, "batch was created without WG_BATCH_TABLES");
    if (m->K != b->K || m->total_rows() != b->NR) throw Error(WG_EINVAL, "batch was built for a different model");
    if (b->pending || !b->tables_fresh)
      throw Error(WG_ESTATE, "no fetched evaluation of this batch holds its tables (evaluate it first)");
    for (int i = 0; i < n_trees; ++i)
      if (families[i] < 0 || families[i] >= b->NF) throw Error(WG_EINVAL, "family index out of range");
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t s = ctx->stream;
    if (!b->track) b->track = build_track(b, m);
    TrackData& td = *b->track;
    const size_t n = (size_t)n_trees;
    std::vector<int64_t> cap_off(n + 1, 0);
    for (size_t i = 0; i < n; ++i) cap_off[i + 1] = cap_off[i] + td.cap[families[i]];
    int64_t by = 0;
    if (n + 1 > td.n_trees_cap) {
      free_all(td.device, {td.d_fam, td.d_seed, td.d_count, td.d_capoff, td.d_off}, {});
      td.d_fam = nullptr, td.d_seed = nullptr, td.d_count = nullptr, td.d_capoff = nullptr, td.d_off = nullptr;
      td.d_fam = dalloc<int>(n + 1, by);
      td.d_seed = dalloc<uint64_t>(n + 1, by);
      td.d_count = dalloc<int>(n + 1, by);
      td.d_capoff = dalloc<int64_t>(n + 1, by);
      td.d_off = dalloc<int64_t>(n + 1, by);
      td.n_trees_cap = n + 1;
    }
    const size_t slots = (size_t)std::max<int64_t>(cap_off[n], 1);
    if (slots > td.slots_cap) {
      free_all(td.device, {td.d_nodes, td.d_stack}, {});
      td.d_nodes = nullptr, td.d_stack = nullptr;
      td.d_nodes = dalloc<int4>(slots, by);
      td.d_stack = dalloc<int4>(slots, by);
      td.slots_cap = slots;
    }
    ck(cudaMemcpyAsync(td.d_fam, families, sizeof(int) * n, cudaMemcpyHostToDevice, s), "upload");
    ck(cudaMemcpyAsync(td.d_seed, seeds, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, s), "upload");
    ck(cudaMemcpyAsync(td.d_capoff, cap_off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s), "upload");
    TrackArgs A;
    A.K = b->K;
    A.NR = b->NR;
    A.mnode = b->d_mnode;
    A.row_off = b->d_rowoff;
    A.params = b->d_params;
    A.ftabs = td.d_ftabs;
    A.fk_tab = td.d_fk_tab;
    A.fk_w = td.d_fk_w;
    A.fk_col = td.d_fk_col;
    A.fclade = td.d_fclade;
    A.fnclade = td.d_fnclade;
    A.fcol = td.d_fcol;
    A.cols = td.d_cols;
    A.csplit = td.d_csplit;
    A.g1 = td.d_g1;
    A.g2 = td.d_g2;
    A.sp = td.d_sp;
    A.cleaf = td.d_cleaf;
    A.n = n_trees;
    A.fam = td.d_fam;
    A.seed = td.d_seed;
    A.cap_off = td.d_capoff;
    A.nodes = td.d_nodes;
    A.stack = td.d_stack;
    A.count = td.d_count;
    ck(track_launch(A, s), "track launch");
    std::vector<int> count(n);
    ck(cudaMemcpyAsync(count.data(), td.d_count, sizeof(int) * n, cudaMemcpyDeviceToHost, s), "download");
    ck(cudaStreamSynchronize(s), "track");
    offsets[0] = 0;
    for (size_t i = 0; i < n; ++i) {
      if (count[i] == kTrackOverflow) throw Error(WG_ERANGE, "a sampled tree exceeds its node capacity");
      if (count[i] == kTrackNoEvent) throw Error(WG_ESTATE, "backtracking found no event with positive probability");
      if (count[i] == kTrackNoLikelihood) throw Error(WG_ESTATE, "backtracking needs a family with positive likelihood");
      offsets[i + 1] = offsets[i] + count[i];
    }
    const size_t total = (size_t)offsets[n];
    if (std::max<size_t>(total, 1) > td.out_cap) {
      free_all(td.device, {td.d_out}, {});
      td.d_out = nullptr;
      td.d_out = dalloc<int4>(std::max<size_t>(total, 1), by);
      td.out_cap = std::max<size_t>(total, 1);
    }
    ck(cudaMemcpyAsync(td.d_off, offsets, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s), "upload");
    ck(track_compact(td.d_nodes, td.d_capoff, td.d_off, td.d_out, n_trees, s), "track compaction");
    td.last_nodes.resize(4 * total);
    if (total)
      ck(cudaMemcpyAsync(td.last_nodes.data(), td.d_out, sizeof(int4) * total, cudaMemcpyDeviceToHost, s),
         "download");
    ck(cudaStreamSynchronize(s), "track");
  });
}

int wg_track_nodes(const wg_batch* b, int32_t* nodes, int64_t cap) {
  WG_GUARD({
    if (!b || !nodes) throw Error(WG_EINVAL, "wg_track_nodes: bad arguments");
    if (!b->track) throw Error(WG_ESTATE, "no wg_track_device call on this batch");
    const auto& v = b->track->last_nodes;
    if (cap < (int64_t)(v.size() / 4)) throw Error(WG_ERANGE, "output buffer too small");
    if (!v.empty()) std::memcpy(nodes, v.data(), v.size() * sizeof(int32_t));
  });
}

int wg_backtrack(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t family, int32_t n_samples, uint64_t seed, char* out,
                 int64_t cap, int64_t* needed) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx || n_samples < 0) throw Error(WG_EINVAL, "wg_backtrack: bad arguments");
    if (family < 0 || family >= b->NF) throw Error(WG_EINVAL, "family index out of range");
    int64_t need = 0;
    int rc = wg_logpdf_tables(ctx, m, b, family, nullptr, 0, &need, nullptr);
    if (rc != WG_OK) throw Error(rc, wg_last_error());
    std::vector<double> tab((size_t)std::max<int64_t>(need, 1));
    rc = wg_logpdf_tables(ctx, m, b, family, tab.data(), need, &need, nullptr);
    if (rc != WG_OK) throw Error(rc, wg_last_error());
    const std::string text = backtrack_family(*m, *b->ccds[family], tab.data(), n_samples, seed);
    if (needed) *needed = (int64_t)text.size() + 1;
    if (!out) return WG_OK;
    if (cap < (int64_t)text.size() + 1) throw Error(WG_ERANGE, "output buffer too small");
    std::memcpy(out, text.c_str(), text.size() + 1);
  });
}

int wg_enqueue(wg_ctx* ctx, wg_model* m, wg_batch* b, int with_grad) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_enqueue: bad arguments");
    enqueue(b, m, with_grad != 0);
  });
}

int wg_fetch(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total, double* d_lam, double* d_mu,
             double* d_q, double* d_eta) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_fetch: bad arguments");
    fetch(b, m, per_family, total, d_lam, d_mu, d_q, d_eta, nullptr, nullptr, nullptr);
  });
}

}  // extern "C"

// ===========================================================================
// Forward evaluation that allocates nothing.
//
// Some callers cannot call cudaMalloc at the time they evaluate the
// likelihood: hosts whose device memory is owned by another allocator or pool,
// and sampler loops that must not enter the allocator between steps
// (cudaMalloc can synchronise the device and can fail under memory pressure).
// wg_logpdf allocates nothing per call either,
// but its first call on a batch instantiates a CUDA graph, which does.  This
// entry point runs the same forward task kernel with its scratch (the top
// row of every task, read by the parent tasks) in the file-scope array
// g_noalloc_tops (its device address looked up when the context was created)
// instead of the batch's own buffer, and launches the levels directly.
// ===========================================================================
extern "C" int wg_logpdf_noalloc(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf_noalloc: bad arguments");
    check_model(b, m);
    int64_t need = 0;
    for (auto& sb : b->subs) need += sb->tops_doubles;
    if (need > kNoAllocMaxTops)
      throw Error(WG_ERANGE, "wg_logpdf_noalloc: the batch needs " + std::to_string(need) +
                                 " doubles of scratch, more than the fixed " + std::to_string(kNoAllocMaxTops) +
                                 " (split the families over smaller batches)");
    // an enqueued evaluation owns the batch's result buffers until wg_fetch
    if (b->pending) throw Error(WG_ESTATE, "wg_logpdf_noalloc: an enqueued evaluation of this batch is not fetched yet");
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    double* scratch = ctx->noalloc_tops;
    if (!scratch) throw Error(WG_ESTATE, "wg_logpdf_noalloc: context has no scratch address");
    cudaStream_t s = ctx->stream;
    b->tables_fresh = false;  // writes no tables; h_logl becomes this call's
    stage_params(b, m);
    ck(cudaMemcpyAsync(b->d_params, b->h_params, sizeof(double) * (b->P + 2), cudaMemcpyHostToDevice, s),
       "params upload");
    // every top row is written by its task before a parent reads it, so the
    // scratch needs no clearing; it keeps the last call's rows afterwards
    int64_t off = 0;
    for (auto& sbp : b->subs) {
      SubBatch* sb = sbp.get();
      KArgs2 A = sub_args(b, sb);
      A.tops = scratch + off;
      A.tabs = nullptr;
      off += sb->tops_doubles;
      for (int L = 0; L < (int)sb->lvl_n.size(); ++L) {
        const bool top = L + 1 == (int)sb->lvl_n.size();
        if (sb->lvlgh_n[L] > 0)
          k_fwd2<false, kNT2H, false, true><<<sb->lvlgh_n[L], kNT2H, 0, s>>>(A, sb->d_lists + sb->lvlgh_off[L]);
        if (sb->lvlg_n[L] > 0 && top)
          k_fwd2<false, kNT2L, true, true><<<sb->lvlg_n[L], kNT2L, 0, s>>>(A, sb->d_lists + sb->lvlg_off[L]);
        else if (sb->lvlg_n[L] > 0)
          k_fwd2<false, kNT2L, false, true><<<sb->lvlg_n[L], kNT2L, 0, s>>>(A, sb->d_lists + sb->lvlg_off[L]);
        if (sb->lvlh_n[L] > 0)
          k_fwd2<false, kNT2H><<<sb->lvlh_n[L], kNT2H, sb->lvlh_smem[L], s>>>(A, sb->d_lists + sb->lvlh_off[L]);
        if (sb->lvl_n[L] > 0 && L + 1 == (int)sb->lvl_n.size())
          k_fwd2<false, kNT2L, true><<<sb->lvl_n[L], kNT2L, sb->lvl_smem[L], s>>>(A, sb->d_lists + sb->lvl_off[L]);
        else if (sb->lvl_n[L] > 0)
          k_fwd2<false, kNT2L><<<sb->lvl_n[L], kNT2L, sb->lvl_smem[L], s>>>(A, sb->d_lists + sb->lvl_off[L]);
      }
    }
    ck(cudaGetLastError(), "forward launch");
    ck(cudaMemcpyAsync(b->h_logl, b->d_logl, sizeof(double) * b->NF, cudaMemcpyDeviceToHost, s), "logl download");
    ck(cudaStreamSynchronize(s), "evaluation");
    finish(m, b->NF, b->h_logl, nullptr, false, per_family, total, nullptr, nullptr, nullptr, nullptr, nullptr,
           nullptr, nullptr);
  });
}
