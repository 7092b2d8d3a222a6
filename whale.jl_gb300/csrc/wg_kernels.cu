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
#include <mutex>

#include "wg_internal.h"

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
  const double* params;  // eps | phi | psi (NR each) | q (K) | eta
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

// Warp butterfly sum of two values (every lane ends with the sums).
__device__ __forceinline__ void warp_sum2(double& a, double& b) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
}

// Block sum of two values in a fixed order; red needs 2 * kNT/32 doubles.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* red) {
  warp_sum2(a, b);
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    red[2 * w] = a;
    red[2 * w + 1] = b;
  }
  __syncthreads();
  a = 0.0;
  b = 0.0;
  for (int i = 0; i < kNT / 32; ++i) {
    a += red[2 * i];
    b += red[2 * i + 1];
  }
}

// Reverse sweep.  gout (per group, P = 3 NR + K + 1 doubles, zeroed):
// [0, NR) d eps, [NR, 2 NR) d phi, [2 NR, 3 NR) d psi, [3 NR, 3 NR + K) d q, [3 NR + K] d eta.
__global__ void __launch_bounds__(kNT) k_adjoint(const KArgs A, double* gbuf, int P) {
  extern __shared__ double sm[];
  const DGroup G = A.groups[blockIdx.x];
  const int tid = threadIdx.x;
  const int mw = G.maxw;
  double* const Bb = sm;
  double* const Bn = sm + mw;
  double* const Lp = sm + 2 * mw;
  double* const X = sm + 3 * mw;
  double* const Y = sm + 4 * mw;
  double* const part = sm + 5 * mw;
  double* const red = part + G.maxslot;  // 2 * 2 * (kNT/32) doubles
  double* out = gbuf + (int64_t)blockIdx.x * P;
  const int NR = A.NR;
  const double* phi = A.params + NR;
  const double* psi = A.params + 2 * NR;
  const double* qv = A.params + 3 * NR;
  for (int k = A.K - 1; k >= 0; --k) {
    const DNode& nd = A.nodes[G.node0 + k];
    const int4 mn = A.mnode[k];
    const int R = nd.width;
    const int roff = A.row_off[k];
    const int lane = (tid + 32 * (int)((blockIdx.x + k) & 3)) & (kNT - 1);
    double* bar = Bb;
    double* barn = Bn;
    if (mn.x == WG_NODE_ROOT) {
      const double* row0 = A.tabs + nd.tab_off;
      for (int c = tid; c < R; c += kNT) {
        Lp[c] = row0[c];
        bar[c] = 0.0;
      }
      __syncthreads();
      for (int f = tid; f < G.n_fam; f += kNT) {
        const int pos = A.fam_pos[G.fam0 + f];
        const double L = Lp[pos];
        bar[pos] = L > 0.0 ? 1.0 / L : 0.0;
      }
      __syncthreads();
      const double eta = A.params[3 * NR + A.K];
      const double er = eps_top(A, k);
      const double xi = 1.0 - (1.0 - eta) * er;
      const double ca = (1.0 - eta) * xi / eta;
      const double cb = eta * (1.0 - er) / (xi * xi);
      double dca = 0.0, dcb = 0.0;
      const int2* tfin = meta2(A, nd.fin_tlvl);
      const int* lc = A.meta + nd.lvl_clades;
      for (int L = nd.nlvl - 1; L >= 0; --L) {
        const DLevel tl = A.levels[nd.tlvl + L];
        if (tl.prog.J > 0) {
          run_prog(A.entries, tl.prog, lane, bar, Lp, part);
          __syncthreads();
          for (int i = tl.begin + tid; i < tl.end; i += kNT) {
            const int c = lc[i];
            const double g = slot_sum(part, tfin[c]);
            bar[c] += ca * g;
            dca += 0.5 * g * Lp[c];
          }
        }
        __syncthreads();
      }
      // recompute Πspec + Πloss of the root row for d cb, then its adjoint
      const DNode& na = A.nodes[G.node0 + mn.y];
      const DNode& nb = A.nodes[G.node0 + mn.z];
      const double* ta = A.tops + na.top_off;
      const double* tb = A.tops + nb.top_off;
      for (int c = tid; c < na.width; c += kNT) X[c] = ta[c];
      for (int c = tid; c < nb.width; c += kNT) Y[c] = tb[c];
      __syncthreads();
      run_prog(A.entries, nd.r1, lane, X, Y, part);
      __syncthreads();
      const double ea = eps_top(A, mn.y), eb = eps_top(A, mn.z);
      double dea = 0.0, deb = 0.0;
      {
        const int2* fin = meta2(A, nd.fin_r1);
        const int2* aux = meta2(A, nd.aux);
        for (int c = tid; c < R; c += kNT) {
          const int2 l = aux[c];
          const double la = l.x >= 0 ? X[l.x] : 0.0;
          const double lb = l.y >= 0 ? Y[l.y] : 0.0;
          const double bc = slot_sum(part, fin[c]) + (la * eb + lb * ea);
          dcb += bar[c] * bc;
          const double bbc = cb * bar[c];
          barn[c] = bbc;
          dea += bbc * lb;
          deb += bbc * la;
        }
      }
      __syncthreads();
      {
        run_prog(A.entries, nd.tr1a, lane, barn, Y, part);
        __syncthreads();
        const int2* fin = meta2(A, nd.fin_tr1a);
        const int* inv = A.meta + nd.inv_a;
        double* o = A.bartops + na.top_off;
        for (int x = tid; x < na.width; x += kNT) {
          const int iv = inv[x];
          o[x] = slot_sum(part, fin[x]) + (iv >= 0 ? barn[iv] * eb : 0.0);
        }
        __syncthreads();
        run_prog(A.entries, nd.tr1b, lane, barn, X, part);
        __syncthreads();
        const int2* finb = meta2(A, nd.fin_tr1b);
        const int* invb = A.meta + nd.inv_b;
        double* ob = A.bartops + nb.top_off;
        for (int x = tid; x < nb.width; x += kNT) {
          const int iv = invb[x];
          ob[x] = slot_sum(part, finb[x]) + (iv >= 0 ? barn[iv] * ea : 0.0);
        }
      }
      block_sum2(dca, dcb, red);
      block_sum2(dea, deb, red + 2 * (kNT / 32));
      if (tid == 0) {
        // ca = (1-η) ξ / η, cb = η (1-ε) / ξ², ξ = 1 - (1-η) ε
        const double dxi_deta = er, dxi_der = -(1.0 - eta);
        const double dca_deta = (-xi + (1.0 - eta) * dxi_deta) / eta - (1.0 - eta) * xi / (eta * eta);
        const double dca_der = (1.0 - eta) * dxi_der / eta;
        const double xi2 = xi * xi, xi3 = xi2 * xi;
        const double dcb_deta = (1.0 - er) / xi2 - 2.0 * eta * (1.0 - er) * dxi_deta / xi3;
        const double dcb_der = -eta / xi2 - 2.0 * eta * (1.0 - er) * dxi_der / xi3;
        out[3 * NR + A.K] += dca * dca_deta + dcb * dcb_deta;
        out[roff + mn.w - 1] += dca * dca_der + dcb * dcb_der;
        out[A.row_off[mn.y] + A.mnode[mn.y].w - 1] += dea;
        out[A.row_off[mn.z] + A.mnode[mn.z].w - 1] += deb;
      }
      __syncthreads();
      continue;
    }
    // ---- non-root: rows nrow-1 .. 1 (within_branch!)
    {
      const double* bt = A.bartops + nd.top_off;
      for (int c = tid; c < R; c += kNT) bar[c] = bt[c];
    }
    __syncthreads();
    const int2* tfin = meta2(A, nd.fin_tdup);
    for (int r = mn.w - 1; r >= 1; --r) {
      const double* lr = A.tabs + nd.tab_off + (int64_t)(r - 1) * R;
      for (int c = tid; c < R; c += kNT) Lp[c] = lr[c];
      __syncthreads();
      const double ph = phi[roff + r], ps = psi[roff + r];
      run_prog(A.entries, nd.tdup, lane, bar, Lp, part);
      __syncthreads();
      double dphi = 0.0, dpsi = 0.0;
      for (int c = tid; c < R; c += kNT) {
        const double g = slot_sum(part, tfin[c]);
        const double b = bar[c], l = Lp[c];
        barn[c] = fma(ps, g, ph * b);
        dphi += b * l;
        dpsi += g * l;
      }
      block_sum2(dphi, dpsi, red);
      if (tid == 0) {
        out[NR + roff + r] += dphi;
        out[2 * NR + roff + r] += 0.5 * dpsi;
      }
      double* t = bar;
      bar = barn;
      barn = t;
    }
    __syncthreads();
    // ---- row 1
    if (mn.x == WG_NODE_WGD) {
      const DNode& nc = A.nodes[G.node0 + mn.y];
      const double* top = A.tops + nc.top_off;
      for (int c = tid; c < R; c += kNT) X[c] = top[c];
      __syncthreads();
      run_prog(A.entries, nd.tdup, lane, bar, X, part);
      __syncthreads();
      const double q = qv[k];
      const double ef = eps_top(A, mn.y);
      double dq = 0.0, def = 0.0;
      double* o = A.bartops + nc.top_off;
      for (int x = tid; x < R; x += kNT) {
        const double g = slot_sum(part, tfin[x]);
        const double b = bar[x], xv = X[x];
        o[x] = ((1.0 - q) + 2.0 * q * ef) * b + q * g;
        dq += b * (2.0 * ef * xv - xv) + 0.5 * g * xv;
        def += b * 2.0 * q * xv;
      }
      block_sum2(dq, def, red);
      if (tid == 0) {
        out[3 * NR + k] += dq;
        out[A.row_off[mn.y] + A.mnode[mn.y].w - 1] += def;
      }
    } else if (mn.x == WG_NODE_INTERNAL) {
      const DNode& na = A.nodes[G.node0 + mn.y];
      const DNode& nb = A.nodes[G.node0 + mn.z];
      const double* ta = A.tops + na.top_off;
      const double* tb = A.tops + nb.top_off;
      for (int c = tid; c < na.width; c += kNT) X[c] = ta[c];
      for (int c = tid; c < nb.width; c += kNT) Y[c] = tb[c];
      __syncthreads();
      const double ea = eps_top(A, mn.y), eb = eps_top(A, mn.z);
      run_prog(A.entries, nd.tr1a, lane, bar, Y, part);
      __syncthreads();
      {
        const int2* fin = meta2(A, nd.fin_tr1a);
        const int* inv = A.meta + nd.inv_a;
        double* o = A.bartops + na.top_off;
        for (int x = tid; x < na.width; x += kNT) {
          const int iv = inv[x];
          o[x] = slot_sum(part, fin[x]) + (iv >= 0 ? bar[iv] * eb : 0.0);
        }
      }
      __syncthreads();
      run_prog(A.entries, nd.tr1b, lane, bar, X, part);
      __syncthreads();
      {
        const int2* fin = meta2(A, nd.fin_tr1b);
        const int* inv = A.meta + nd.inv_b;
        double* o = A.bartops + nb.top_off;
        for (int x = tid; x < nb.width; x += kNT) {
          const int iv = inv[x];
          o[x] = slot_sum(part, fin[x]) + (iv >= 0 ? bar[iv] * ea : 0.0);
        }
      }
      double dea = 0.0, deb = 0.0;
      const int2* aux = meta2(A, nd.aux);
      for (int c = tid; c < R; c += kNT) {
        const int2 l = aux[c];
        const double b = bar[c];
        deb += b * (l.x >= 0 ? X[l.x] : 0.0);
        dea += b * (l.y >= 0 ? Y[l.y] : 0.0);
      }
      block_sum2(dea, deb, red);
      if (tid == 0) {
        out[A.row_off[mn.y] + A.mnode[mn.y].w - 1] += dea;
        out[A.row_off[mn.z] + A.mnode[mn.z].w - 1] += deb;
      }
    }
    __syncthreads();
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

// Sum the per-group adjoints in group order (deterministic).
__global__ void k_reduce_groups(const double* gbuf, int n_groups, int P, double* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= P) return;
  double s = 0.0;
  for (int g = 0; g < n_groups; ++g) s += gbuf[(int64_t)g * P + j];
  out[j] = s;
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

template <class T>
void h2d(T* d, const std::vector<T>& h, cudaStream_t s) {
  if (!h.empty()) ck(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
}

}  // namespace

struct wg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int n_sm = 0;
  size_t smem_optin = 0;
  bool timing = false;
  bool timed = false;      // events of the last evaluation were recorded
  bool timed_grad = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float last_ms[3] = {0, 0, 0};
};

struct wg_batch {
  wg_ctx* ctx = nullptr;
  int K = 0, NR = 0, NF = 0, n_groups = 0, P = 0;
  uint32_t flags = 0;
  int64_t device_bytes = 0;
  size_t smem_fwd = 0, smem_adj = 0;
  double flops_fwd = 0, bytes_fwd = 0, flops_adj = 0;
  // layout (host copies needed to address tables)
  std::vector<int64_t> fam_node0;
  std::vector<int32_t> fam_col, fam_ncol;
  std::vector<DNode> nodes;
  std::vector<int> nrow;
  // device
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
  double* d_tabs = nullptr;
  double* d_bartops = nullptr;
  double* d_logl = nullptr;
  double* d_gbuf = nullptr;
  double* d_gred = nullptr;
  // pinned host staging
  double* h_params = nullptr;
  double* h_logl = nullptr;
  double* h_gred = nullptr;
  bool grad_pending = false;
  // one-family-per-launch layout (plain path), built on first use
  std::unique_ptr<wg_batch> plain;
  std::vector<wg_ccd*> ccds;  // not owned; kept for the lazy plain layout
  ~wg_batch();
};

wg_batch::~wg_batch() {
  void* dptrs[] = {d_groups, d_nodes, d_entries, d_meta, d_levels, d_famidx, d_fampos, d_mnode, d_rowoff,
                   d_leafp, d_params, d_tops, d_tabs, d_bartops, d_logl, d_gbuf, d_gred};
  if (ctx) cudaSetDevice(ctx->device);
  for (void* p : dptrs)
    if (p) cudaFree(p);
  if (h_params) cudaFreeHost(h_params);
  if (h_logl) cudaFreeHost(h_logl);
  if (h_gred) cudaFreeHost(h_gred);
}

namespace {

KArgs make_args(const wg_batch* b) {
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
  A.tabs = b->d_tabs;
  A.bartops = b->d_bartops;
  A.logl = b->d_logl;
  A.K = b->K;
  A.NR = b->NR;
  return A;
}

std::unique_ptr<wg_batch> build_batch(wg_ctx* ctx, const wg_model* m, wg_ccd* const* ccds, int n, uint32_t flags,
                                      bool single) {
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  std::vector<const CCD*> cs;
  for (int i = 0; i < n; ++i) {
    if (!ccds[i]) throw Error(WG_EINVAL, "null CCD in batch");
    cs.push_back(ccds[i]);
  }
  PackOptions opt;
  opt.adjoint = (flags & WG_BATCH_GRAD) != 0;
  opt.keep_tables = (flags & (WG_BATCH_GRAD | WG_BATCH_TABLES)) != 0;
  opt.single = single;
  Packed P = pack_batch(*m, cs, opt);
  auto b = std::make_unique<wg_batch>();
  b->ctx = ctx;
  b->K = m->K;
  b->NR = m->total_rows();
  b->NF = n;
  b->flags = flags;
  b->n_groups = (int)P.groups.size();
  b->P = 3 * b->NR + b->K + 1;
  b->flops_fwd = P.flops_fwd;
  b->bytes_fwd = P.bytes_fwd;
  b->flops_adj = P.flops_adj;
  b->fam_node0 = P.fam_node0;
  b->fam_col = P.fam_col;
  b->fam_ncol = P.fam_ncol;
  b->nodes = P.nodes;
  b->nrow = m->nrow;
  b->smem_fwd = (size_t)P.max_smem_doubles * sizeof(double);
  b->smem_adj = b->smem_fwd + 2 * 2 * (kNT / 32) * sizeof(double) + 64;
  if (b->smem_adj > ctx->smem_optin)
    throw Error(WG_ERANGE, "a group needs more shared memory than one CTA can hold");
  cudaStream_t s = ctx->stream;
  int64_t& by = b->device_bytes;
  b->d_groups = dalloc<DGroup>(P.groups.size(), by);
  b->d_nodes = dalloc<DNode>(P.nodes.size(), by);
  b->d_entries = dalloc<DEntry>(P.entries.size(), by);
  b->d_meta = dalloc<int>(P.meta.size(), by);
  b->d_levels = dalloc<DLevel>(P.levels.size(), by);
  b->d_famidx = dalloc<int>(P.fam_idx.size(), by);
  b->d_fampos = dalloc<int>(P.fam_pos.size(), by);
  b->d_mnode = dalloc<int4>(m->K, by);
  b->d_rowoff = dalloc<int>(m->K + 1, by);
  b->d_leafp = dalloc<double>(m->K, by);
  b->d_params = dalloc<double>(3 * b->NR + b->K + 1, by);
  b->d_tops = dalloc<double>(P.tops_doubles, by);
  if (opt.keep_tables) b->d_tabs = dalloc<double>(P.tab_doubles, by);
  if (opt.adjoint) {
    b->d_bartops = dalloc<double>(P.tops_doubles, by);
    b->d_gbuf = dalloc<double>((size_t)b->n_groups * b->P, by);
    b->d_gred = dalloc<double>(b->P, by);
  }
  b->d_logl = dalloc<double>(n, by);
  h2d(b->d_groups, P.groups, s);
  h2d(b->d_nodes, P.nodes, s);
  h2d(b->d_entries, P.entries, s);
  h2d(b->d_meta, P.meta, s);
  h2d(b->d_levels, P.levels, s);
  h2d(b->d_famidx, P.fam_idx, s);
  h2d(b->d_fampos, P.fam_pos, s);
  std::vector<int4> mn(m->K);
  for (int k = 0; k < m->K; ++k) mn[k] = make_int4(m->kind[k], m->ch0[k], m->ch1[k], m->nrow[k]);
  h2d(b->d_mnode, mn, s);
  h2d(b->d_rowoff, m->row_off, s);
  h2d(b->d_leafp, m->leaf_p, s);
  ck(cudaMallocHost(&b->h_params, sizeof(double) * (3 * b->NR + b->K + 1)), "cudaMallocHost");
  ck(cudaMallocHost(&b->h_logl, sizeof(double) * n), "cudaMallocHost");
  if (opt.adjoint) ck(cudaMallocHost(&b->h_gred, sizeof(double) * b->P), "cudaMallocHost");
  ck(cudaStreamSynchronize(s), "batch upload");
  b->ccds.assign(ccds, ccds + n);
  return b;
}

void check_model(const wg_batch* b, const wg_model* m) {
  if (!m->has_params) throw Error(WG_ESTATE, "model parameters not set (wg_model_set_rates / wg_model_set_tables)");
  if (m->K != b->K || m->total_rows() != b->NR) throw Error(WG_EINVAL, "batch was built for a different model");
}

// Stage the slice tables, q and η and launch the forward (and adjoint).
void enqueue(wg_batch* b, const wg_model* m, bool grad) {
  check_model(b, m);
  wg_ctx* ctx = b->ctx;
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int NR = b->NR, K = b->K;
  std::memcpy(b->h_params, m->eps.data(), NR * sizeof(double));
  std::memcpy(b->h_params + NR, m->phi.data(), NR * sizeof(double));
  std::memcpy(b->h_params + 2 * NR, m->psi.data(), NR * sizeof(double));
  for (int k = 0; k < K; ++k) b->h_params[3 * NR + k] = std::isnan(m->q[k]) ? 0.0 : m->q[k];
  b->h_params[3 * NR + K] = m->eta;
  cudaStream_t s = ctx->stream;
  ck(cudaMemcpyAsync(b->d_params, b->h_params, sizeof(double) * (3 * NR + K + 1), cudaMemcpyHostToDevice, s),
     "params upload");
  const KArgs A = make_args(b);
  const bool tm = ctx->timing;
  if (grad && !(b->flags & WG_BATCH_GRAD)) throw Error(WG_ESTATE, "batch was created without WG_BATCH_GRAD");
  if (grad) ck(cudaMemsetAsync(b->d_gbuf, 0, sizeof(double) * (size_t)b->n_groups * b->P, s), "memset");
  if (tm) ck(cudaEventRecord(ctx->ev[0], s), "event");
  if (grad || (b->flags & WG_BATCH_TABLES))
    k_forward<true><<<b->n_groups, kNT, b->smem_fwd, s>>>(A);
  else
    k_forward<false><<<b->n_groups, kNT, b->smem_fwd, s>>>(A);
  ck(cudaGetLastError(), "forward launch");
  if (tm) ck(cudaEventRecord(ctx->ev[1], s), "event");
  if (grad) {
    k_adjoint<<<b->n_groups, kNT, b->smem_adj, s>>>(A, b->d_gbuf, b->P);
    ck(cudaGetLastError(), "adjoint launch");
    if (tm) ck(cudaEventRecord(ctx->ev[2], s), "event");
    k_reduce_groups<<<(b->P + 127) / 128, 128, 0, s>>>(b->d_gbuf, b->n_groups, b->P, b->d_gred);
    ck(cudaGetLastError(), "reduce launch");
    if (tm) ck(cudaEventRecord(ctx->ev[3], s), "event");
  }
  ctx->timed = tm;
  ctx->timed_grad = grad;
  b->grad_pending = grad;
}

void fetch(wg_batch* b, const wg_model* m, double* per_family, double* total, double* d_lam, double* d_mu,
           double* d_q, double* d_eta, double* d_eps, double* d_phi, double* d_psi) {
  cudaStream_t s = b->ctx->stream;
  ck(cudaMemcpyAsync(b->h_logl, b->d_logl, sizeof(double) * b->NF, cudaMemcpyDeviceToHost, s), "logl download");
  const bool grad = b->grad_pending;
  if (grad) ck(cudaMemcpyAsync(b->h_gred, b->d_gred, sizeof(double) * b->P, cudaMemcpyDeviceToHost, s), "grad download");
  ck(cudaStreamSynchronize(s), "evaluation");
  wg_ctx* ctx = b->ctx;
  if (ctx->timed) {
    ck(cudaEventElapsedTime(&ctx->last_ms[0], ctx->ev[0], ctx->ev[1]), "event time");
    ctx->last_ms[1] = ctx->last_ms[2] = 0.0f;
    if (ctx->timed_grad) {
      ck(cudaEventElapsedTime(&ctx->last_ms[1], ctx->ev[1], ctx->ev[2]), "event time");
      ck(cudaEventElapsedTime(&ctx->last_ms[2], ctx->ev[2], ctx->ev[3]), "event time");
    }
    ctx->timed = false;
  }
  // sum over families minus N * condition, ℓhood (src/core.jl:15, :58-64)
  double sum = 0.0;
  for (int i = 0; i < b->NF; ++i) sum += b->h_logl[i];
  const double cond = model_condition(*m);
  double tot = sum - b->NF * cond;
  if (!std::isfinite(tot)) tot = -INFINITY;
  if (per_family) std::memcpy(per_family, b->h_logl, sizeof(double) * b->NF);
  if (total) *total = tot;
  if (!grad) return;
  const int NR = b->NR, K = b->K;
  std::vector<double> de(b->h_gred, b->h_gred + NR), dp(b->h_gred + NR, b->h_gred + 2 * NR),
      ds(b->h_gred + 2 * NR, b->h_gred + 3 * NR), dq(b->h_gred + 3 * NR, b->h_gred + 3 * NR + K);
  double deta = b->h_gred[3 * NR + K];
  model_condition_vjp(*m, -(double)b->NF, de, deta);
  if (d_eps) std::memcpy(d_eps, de.data(), NR * sizeof(double));
  if (d_phi) std::memcpy(d_phi, dp.data(), NR * sizeof(double));
  if (d_psi) std::memcpy(d_psi, ds.data(), NR * sizeof(double));
  if (d_eta) *d_eta = deta;
  if (m->from_rates && (d_lam || d_mu || d_q)) {
    std::vector<double> dl, dm, dpp;
    model_tables_vjp(*m, de, dp, ds, dl, dm, dq, dpp);
    if (d_lam) std::memcpy(d_lam, dl.data(), K * sizeof(double));
    if (d_mu) std::memcpy(d_mu, dm.data(), K * sizeof(double));
  }
  if (d_q) std::memcpy(d_q, dq.data(), K * sizeof(double));
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
    ck(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "attr");
    c->smem_optin = (size_t)v;
    ck(cudaFuncSetAttribute(k_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v), "attr");
    ck(cudaFuncSetAttribute(k_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v), "attr");
    ck(cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, v), "attr");
    *out = c.release();
  });
}

int wg_ctx_destroy(wg_ctx* ctx) {
  if (!ctx) return WG_OK;
  cudaSetDevice(ctx->device);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return WG_OK;
}

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

void* wg_ctx_stream(wg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int wg_batch_create(wg_ctx* ctx, const wg_model* m, wg_ccd* const* ccds, int32_t n_ccds, uint32_t flags,
                    wg_batch** out) {
  WG_GUARD({
    if (!ctx || !m || !ccds || n_ccds <= 0 || !out) throw Error(WG_EINVAL, "wg_batch_create: bad arguments");
    *out = build_batch(ctx, m, ccds, n_ccds, flags, false).release();
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
    if (n_groups) *n_groups = b->n_groups;
    if (device_bytes) *device_bytes = b->device_bytes;
    if (flops_fwd) *flops_fwd = b->flops_fwd;
    if (bytes_fwd) *bytes_fwd = b->bytes_fwd;
    if (flops_adj) *flops_adj = b->flops_adj;
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

int wg_logpdf_plain(wg_ctx* ctx, wg_model* m, wg_batch* b, double* per_family, double* total) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf_plain: bad arguments");
    if (!b->plain) b->plain = build_batch(ctx, m, b->ccds.data(), b->NF, 0, true);
    wg_batch* pb = b->plain.get();
    check_model(pb, m);
    // one launch per family, in family order, on the context stream
    const int NR = pb->NR, K = pb->K;
    std::memcpy(pb->h_params, m->eps.data(), NR * sizeof(double));
    std::memcpy(pb->h_params + NR, m->phi.data(), NR * sizeof(double));
    std::memcpy(pb->h_params + 2 * NR, m->psi.data(), NR * sizeof(double));
    for (int k = 0; k < K; ++k) pb->h_params[3 * NR + k] = std::isnan(m->q[k]) ? 0.0 : m->q[k];
    pb->h_params[3 * NR + K] = m->eta;
    cudaStream_t s = ctx->stream;
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    ck(cudaMemcpyAsync(pb->d_params, pb->h_params, sizeof(double) * (3 * NR + K + 1), cudaMemcpyHostToDevice, s),
       "params upload");
    KArgs A = make_args(pb);
    const DGroup* g0 = pb->d_groups;
    for (int g = 0; g < pb->n_groups; ++g) {
      A.groups = g0 + g;
      k_forward<false><<<1, kNT, pb->smem_fwd, s>>>(A);
    }
    ck(cudaGetLastError(), "plain launch");
    pb->grad_pending = false;
    fetch(pb, m, per_family, total, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  });
}

int wg_logpdf_tables(wg_ctx* ctx, wg_model* m, wg_batch* b, int32_t family, double* out, int64_t cap,
                     int64_t* needed, double* logl) {
  WG_GUARD({
    if (!ctx || !m || !b || b->ctx != ctx) throw Error(WG_EINVAL, "wg_logpdf_tables: bad arguments");
    if (family < 0 || family >= b->NF) throw Error(WG_EINVAL, "family index out of range");
    if (!(b->flags & WG_BATCH_TABLES)) throw Error(WG_ESTATE, "batch was created without WG_BATCH_TABLES");
    const int K = b->K;
    int64_t need = 0;
    for (int k = 0; k < K; ++k) need += (int64_t)b->nrow[k] * b->fam_ncol[(size_t)family * K + k];
    if (needed) *needed = need;
    if (!out) return WG_OK;
    if (cap < need) throw Error(WG_ERANGE, "output buffer too small");
    enqueue(b, m, false);
    fetch(b, m, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (logl) *logl = b->h_logl[family];
    cudaStream_t s = ctx->stream;
    int64_t o = 0;
    for (int k = 0; k < K; ++k) {
      const DNode& nd = b->nodes[b->fam_node0[family] + k];
      const int nc = b->fam_ncol[(size_t)family * K + k];
      const int col = b->fam_col[(size_t)family * K + k];
      if (nc > 0)
        ck(cudaMemcpy2DAsync(out + o, nc * sizeof(double), b->d_tabs + nd.tab_off + col, (size_t)nd.width * sizeof(double),
                             nc * sizeof(double), b->nrow[k], cudaMemcpyDeviceToHost, s),
           "table download");
      o += (int64_t)b->nrow[k] * nc;
    }
    ck(cudaStreamSynchronize(s), "table download");
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
