// NowhereExtinctCondition on the device: the 2^L-term inclusion-exclusion
// over the joint pgf of the leaf counts (src/condition.jl:31-36,
// treepgf_allbinary src/bdputil.jl:114-135) and its reverse-mode adjoint.
// The layout and the kernels are described in wg_nowhere.h.
#include <cmath>
#include <cstring>
#include <string>

#include "wg_nowhere.h"

namespace wg {

namespace {

constexpr int kNwMaxLeaves = 22;       // 2^22 root arguments
constexpr int kNwThreads = 512;        // the single-CTA sweeps
constexpr int kNwTileThreads = 256;    // root tiles: up to 1024 entries each
constexpr double kNwCriticalAtol = 1e-6;  // ΛMATOL, src/bdputil.jl:1

void nck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(WG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

struct NwArgs {
  const double* coef;  // per node: λ (η at the root), μ, t, ρ = e^{(μ-λ)t}, q, mode
  const NwTopo* topo;
  const int* fwd;
  const int* fwd_off;
  const int* rev;
  const int* rev_off;
  int n_fwd_lv, n_rev_lv;
  double* v;
  double* bv;
  double* pq;  // reverse reduction arrays in device memory (pq_smem == 0)
  int64_t pq_n;
  int pq_smem;
  double* rowpart;  // [nt1][n0]
  double* colpart;  // [nt0][n1]
  double* out;      // ntiles Σ s_i v | ntiles ∂/∂η | 3·K node adjoints (λ, μ, q)
  int root, T0, T1, lT0, nt0, nt1, ntiles;
};

enum { kNwBdp = 0, kNwCritical = 1, kNwRoot = 2 };

// The node's pgf at y, in the reference's own arithmetic (src/bdputil.jl:
// 67, 93-99; no contraction into FMAs, so every vector entry is the value
// the reference's expression rounds to):
//   bdp       (ρ(λy - μ) - μ(y - 1)) / (ρ(λy - μ) - λ(y - 1))
//   critical  (1 - (λt - 1)(y - 1)) / (1 - λt(y - 1))
//   root      ηy / (1 - (1 - η)y)
__device__ __forceinline__ double nw_pgf(const double* c, double y) {
  const int mode = (int)c[5];
  if (mode == kNwRoot) return __ddiv_rn(__dmul_rn(c[0], y), __dsub_rn(1.0, __dmul_rn(__dsub_rn(1.0, c[0]), y)));
  const double u = __dsub_rn(y, 1.0);
  if (mode == kNwCritical) {
    const double lt = __dmul_rn(c[0], c[2]);
    return __ddiv_rn(__dsub_rn(1.0, __dmul_rn(__dsub_rn(lt, 1.0), u)), __dsub_rn(1.0, __dmul_rn(lt, u)));
  }
  const double ra = __dmul_rn(c[3], __dsub_rn(__dmul_rn(c[0], y), c[1]));
  return __ddiv_rn(__dsub_rn(ra, __dmul_rn(c[1], u)), __dsub_rn(ra, __dmul_rn(c[0], u)));
}

// WGD retention before the branch (wgdpgf, src/bdputil.jl:104): x(1 - q + xq).
__device__ __forceinline__ double nw_wgd(double x, double q) {
  return __dmul_rn(x, __dadd_rn(__dsub_rn(1.0, q), __dmul_rn(x, q)));
}

// Partial derivatives of the node's pgf at y with value v: ∂/∂y, ∂/∂λ (∂/∂η
// at the root) and ∂/∂μ (quotient rule on the expressions above).
__device__ __forceinline__ void nw_pgf_grad(const double* c, double y, double v, double& dy, double& d0, double& d1) {
  const int mode = (int)c[5];
  if (mode == kNwRoot) {
    const double eta = c[0], d = 1.0 - (1.0 - eta) * y, i2 = 1.0 / (d * d);
    dy = eta * i2;
    d0 = y * (1.0 - y) * i2;
    d1 = 0.0;
    return;
  }
  const double lam = c[0], mu = c[1], t = c[2], u = y - 1.0;
  if (mode == kNwCritical) {
    const double lt = lam * t, inv = 1.0 / (1.0 - lt * u);
    dy = (v * lt - (lt - 1.0)) * inv;
    d0 = t * u * (v - 1.0) * inv;
    d1 = 0.0;
    return;
  }
  const double rho = c[3], a = lam * y - mu, ra = rho * a, tr = t * rho;
  const double inv = 1.0 / (ra - lam * u);
  dy = ((rho * lam - mu) - v * (rho * lam - lam)) * inv;
  const double nl = -tr * a + rho * y;  // ∂num/∂λ; ∂den/∂λ = nl - u
  d0 = (nl - v * (nl - u)) * inv;
  const double nm = tr * a - rho - u;  // ∂num/∂μ; ∂den/∂μ = tr a - ρ
  d1 = (nm - v * (tr * a - rho)) * inv;
}

// Argument x_k of node k at index i (leaf bit, the WGD child's value, or the
// product of the children's values); x0, x1 return the children's values.
__device__ __forceinline__ double nw_arg(const NwTopo& t, int64_t i, const double* v0, const double* v1, double& x0,
                                         double& x1) {
  x0 = x1 = 0.0;
  if (t.kind == WG_NODE_LEAF) return (double)i;
  if (t.c1 < 0) return v0[i];
  x0 = v0[i & (((int64_t)1 << t.L0) - 1)];
  x1 = v1[i >> t.L0];
  return __dmul_rn(x0, x1);
}

// Block sum of NV values per thread (fixed butterfly, warps summed in
// order); the result is valid in thread 0.  red: 32·NV doubles.
template <int NV>
__device__ __forceinline__ void nw_block_sum(double (&s)[NV], double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int j = 0; j < NV; ++j) s[j] += __shfl_xor_sync(0xffffffffu, s[j], o);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) red[w * NV + j] = s[j];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double t = 0.0;
      for (int q = 0; q < nw; ++q) t += red[q * NV + j];
      s[j] = t;
    }
}

// Vectors of every node below the root, children before parents: one height
// of the species tree per barrier.
__global__ void __launch_bounds__(kNwThreads) k_nw_fwd(const NwArgs a) {
  for (int h = 0; h < a.n_fwd_lv; ++h) {
    for (int j = a.fwd_off[h]; j < a.fwd_off[h + 1]; ++j) {
      const int k = a.fwd[j];
      const NwTopo t = a.topo[k];
      const double* cf = a.coef + 6 * k;
      const double* v0 = t.c0 >= 0 ? a.v + a.topo[t.c0].off : nullptr;
      const double* v1 = t.c1 >= 0 ? a.v + a.topo[t.c1].off : nullptr;
      const int64_t n = (int64_t)1 << t.L;
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double x0, x1;
        const double x = nw_arg(t, i, v0, v1, x0, x1);
        a.v[t.off + i] = nw_pgf(cf, t.kind == WG_NODE_WGD ? nw_wgd(x, cf[4]) : x);
      }
    }
    __syncthreads();
  }
}

// The root's 2^L arguments in T0 x T1 tiles: Σ s_i v_r(i) over i < last per
// tile and, with GRAD, the reverse sweep's start: adjoint seed -s_i (the
// 1/P factor is applied on the host), the tile's sum for ∂/∂η, and its
// partial sums of the children's adjoints
//   bv_{c0}[i0] = Σ_{i1} bx[i0 + n0 i1] v_{c1}[i1],  bv_{c1}[i1] = Σ_{i0} bx[..] v_{c0}[i0].
template <bool GRAD>
__global__ void __launch_bounds__(kNwTileThreads) k_nw_root(const NwArgs a) {
  __shared__ double P[1024], Q[1024];
  __shared__ double red[32 * 2];
  const NwTopo t = a.topo[a.root];
  const double* cf = a.coef + 6 * a.root;
  const int64_t n0 = (int64_t)1 << t.L0, n1 = (int64_t)1 << (t.L - t.L0), last = ((int64_t)1 << t.L) - 1;
  const double* v0 = a.v + a.topo[t.c0].off;
  const double* v1 = a.v + a.topo[t.c1].off;
  const int ti0 = blockIdx.x % a.nt0, ti1 = blockIdx.x / a.nt0;
  const int E = a.T0 * a.T1;
  double s[2] = {0.0, 0.0};
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    const int64_t i0 = (int64_t)ti0 * a.T0 + (e & (a.T0 - 1));
    const int64_t i1 = (int64_t)ti1 * a.T1 + (e >> a.lT0);
    const int64_t i = i0 + (i1 << t.L0);
    const double x0 = v0[i0], x1 = v1[i1], x = __dmul_rn(x0, x1);
    const double v = nw_pgf(cf, x);
    const double sg = (__popcll((unsigned long long)i) & 1) ? -1.0 : 1.0;
    const double b = i == last ? 0.0 : -sg;
    s[0] -= b * v;  // s_i v over i < last
    if (GRAD) {
      double dy, de, d1;
      nw_pgf_grad(cf, x, v, dy, de, d1);
      s[1] += b * de;
      const double bx = b * dy;
      P[e] = bx * x1;
      Q[e] = bx * x0;
    }
  }
  nw_block_sum<2>(s, red);
  if (threadIdx.x == 0) {
    a.out[blockIdx.x] = s[0];
    a.out[a.ntiles + blockIdx.x] = s[1];
  }
  if (!GRAD) return;
  __syncthreads();
  // rows: sum over the tile's i1 (stride T0); columns: over its i0
  for (int st = a.T1 >> 1; st >= 1; st >>= 1) {
    for (int e = threadIdx.x; e < a.T0 * st; e += blockDim.x) P[e] += P[e + a.T0 * st];
    __syncthreads();
  }
  for (int st = a.T0 >> 1; st >= 1; st >>= 1) {
    for (int u = threadIdx.x; u < a.T1 * st; u += blockDim.x) {
      const int l1 = u / st, l0 = u - l1 * st;
      Q[l0 + a.T0 * l1] += Q[l0 + st + a.T0 * l1];
    }
    __syncthreads();
  }
  for (int l0 = threadIdx.x; l0 < a.T0; l0 += blockDim.x)
    a.rowpart[(int64_t)ti1 * n0 + (int64_t)ti0 * a.T0 + l0] = P[l0];
  for (int l1 = threadIdx.x; l1 < a.T1; l1 += blockDim.x)
    a.colpart[(int64_t)ti0 * n1 + (int64_t)ti1 * a.T1 + l1] = Q[a.T0 * l1];
}

// Reverse sweep below the root, parents before children: the root's
// children's adjoints from the tiles' partial sums, then per node the
// adjoints of λ, μ, q and its children's adjoints (tree sums over the other
// child's index bits, in shared or device memory).
__global__ void __launch_bounds__(kNwThreads, 1) k_nw_rev(const NwArgs a) {
  extern __shared__ double nw_smem[];
  __shared__ double red[32 * 3];
  double* P = a.pq_smem ? nw_smem : a.pq;
  double* Q = P + a.pq_n;
  const int tid = threadIdx.x, NT = blockDim.x;
  {
    const NwTopo t = a.topo[a.root];
    const int64_t n0 = (int64_t)1 << t.L0, n1 = (int64_t)1 << (t.L - t.L0);
    double* b0 = a.bv + a.topo[t.c0].off;
    double* b1 = a.bv + a.topo[t.c1].off;
    for (int64_t i0 = tid; i0 < n0; i0 += NT) {
      double s = 0.0;
      for (int u = 0; u < a.nt1; ++u) s += a.rowpart[(int64_t)u * n0 + i0];
      b0[i0] = s;
    }
    for (int64_t i1 = tid; i1 < n1; i1 += NT) {
      double s = 0.0;
      for (int u = 0; u < a.nt0; ++u) s += a.colpart[(int64_t)u * n1 + i1];
      b1[i1] = s;
    }
  }
  __syncthreads();
  double* nout = a.out + 2 * a.ntiles;
  for (int d = 0; d < a.n_rev_lv; ++d) {
    for (int j = a.rev_off[d]; j < a.rev_off[d + 1]; ++j) {
      const int k = a.rev[j];
      const NwTopo t = a.topo[k];
      const double* cf = a.coef + 6 * k;
      const double q = cf[4];
      const double* v0 = t.c0 >= 0 ? a.v + a.topo[t.c0].off : nullptr;
      const double* v1 = t.c1 >= 0 ? a.v + a.topo[t.c1].off : nullptr;
      const double* vk = a.v + t.off;
      const double* bk = a.bv + t.off;
      const bool wgd = t.kind == WG_NODE_WGD, binary = t.kind != WG_NODE_LEAF && t.c1 >= 0;
      const int64_t n = (int64_t)1 << t.L;
      double s[3] = {0.0, 0.0, 0.0};
      for (int64_t i = tid; i < n; i += NT) {
        double x0, x1;
        const double x = nw_arg(t, i, v0, v1, x0, x1);
        const double y = wgd ? nw_wgd(x, q) : x;
        const double b = bk[i];
        double dy, dl, dm;
        nw_pgf_grad(cf, y, vk[i], dy, dl, dm);
        s[0] += b * dl;
        s[1] += b * dm;
        const double by = b * dy;
        double bx = by;
        if (wgd) {
          s[2] += by * (x * x - x);
          bx = by * (1.0 - q + 2.0 * q * x);
        }
        if (t.kind == WG_NODE_LEAF) continue;
        if (!binary) {
          a.bv[a.topo[t.c0].off + i] = bx;
        } else {
          P[i] = bx * x1;
          Q[i] = bx * x0;
        }
      }
      nw_block_sum<3>(s, red);
      if (tid == 0) {
        nout[3 * k] = s[0];
        nout[3 * k + 1] = s[1];
        nout[3 * k + 2] = s[2];
      }
      __syncthreads();
      if (binary) {
        const int64_t n0 = (int64_t)1 << t.L0, n1 = n >> t.L0;
        for (int64_t st = n1 >> 1; st >= 1; st >>= 1) {
          for (int64_t e = tid; e < n0 * st; e += NT) P[e] += P[e + n0 * st];
          __syncthreads();
        }
        for (int64_t st = n0 >> 1; st >= 1; st >>= 1) {
          for (int64_t u = tid; u < n1 * st; u += NT) {
            const int64_t l1 = u / st, l0 = u - l1 * st;
            Q[l0 + n0 * l1] += Q[l0 + st + n0 * l1];
          }
          __syncthreads();
        }
        double* b0 = a.bv + a.topo[t.c0].off;
        double* b1 = a.bv + a.topo[t.c1].off;
        for (int64_t i0 = tid; i0 < n0; i0 += NT) b0[i0] = P[i0];
        for (int64_t i1 = tid; i1 < n1; i1 += NT) b1[i1] = Q[n0 * i1];
        __syncthreads();
      }
    }
  }
}

NwArgs nw_args(const NwPlan& p) {
  NwArgs a;
  a.coef = p.d_coef;
  a.topo = p.d_topo;
  a.fwd = p.d_lists;
  a.fwd_off = p.d_lists + p.n_fwd;
  a.rev = a.fwd_off + p.n_fwd_lv + 1;
  a.rev_off = a.rev + p.n_rev;
  a.n_fwd_lv = p.n_fwd_lv;
  a.n_rev_lv = p.n_rev_lv;
  a.v = p.d_v;
  a.bv = p.d_bv;
  a.pq = p.d_pq;
  a.pq_n = p.pq_n;
  a.pq_smem = p.pq_smem ? 1 : 0;
  a.rowpart = p.d_part;
  a.colpart = p.d_part + (int64_t)p.nt1 * ((int64_t)p.T0 * p.nt0);
  a.out = p.d_out;
  a.root = p.root;
  a.T0 = p.T0;
  a.T1 = p.T1;
  a.lT0 = p.lT0;
  a.nt0 = p.nt0;
  a.nt1 = p.nt1;
  a.ntiles = p.ntiles;
  return a;
}

}  // namespace

NwPlan::~NwPlan() {
  cudaSetDevice(device);
  for (void* d : {(void*)d_coef, (void*)d_topo, (void*)d_lists, (void*)d_v, (void*)d_bv, (void*)d_pq, (void*)d_part,
                  (void*)d_out})
    if (d) cudaFree(d);
  for (void* h : {(void*)h_coef, (void*)h_out})
    if (h) cudaFreeHost(h);
  if (fork) cudaEventDestroy(fork);
  if (done) cudaEventDestroy(done);
  if (s) cudaStreamDestroy(s);
}

bool nw_plan_matches(const NwPlan& p, const Model& m) {
  return p.K == m.K && p.kind == m.kind && p.ch0 == m.ch0 && p.ch1 == m.ch1;
}

std::unique_ptr<NwPlan> nw_plan_create(const Model& m, int device) {
  const int K = m.K;
  auto p = std::make_unique<NwPlan>();
  p->device = device;
  p->K = K;
  p->kind = m.kind;
  p->ch0 = m.ch0;
  p->ch1 = m.ch1;
  std::vector<NwTopo> topo(K);
  std::vector<int> height(K, 0), depth(K, 0);
  int root = -1;
  for (int k = 0; k < K; ++k) {  // children precede parents in the model order
    NwTopo& t = topo[k];
    t.kind = m.kind[k];
    t.c0 = t.kind == WG_NODE_LEAF ? -1 : m.ch0[k];
    t.c1 = t.kind == WG_NODE_LEAF ? -1 : m.ch1[k];
    t.pad = 0;
    if (t.kind == WG_NODE_LEAF) {
      t.L = 1, t.L0 = 0;
    } else {
      if (t.c0 < 0 || t.c0 >= k || t.c1 >= k) throw Error(WG_EINVAL, "NowhereExtinctCondition: malformed tree");
      t.L0 = topo[t.c0].L;
      t.L = t.L0 + (t.c1 >= 0 ? topo[t.c1].L : 0);
      height[k] = 1 + std::max(height[t.c0], t.c1 >= 0 ? height[t.c1] : 0);
    }
    if (t.kind == WG_NODE_ROOT) root = k;
  }
  if (root != K - 1 || topo[root].c1 < 0) throw Error(WG_EINVAL, "NowhereExtinctCondition: the root must be binary and last");
  if (topo[root].L > kNwMaxLeaves)
    throw Error(WG_ERANGE, "NowhereExtinctCondition over more than 22 leaves (2^leaves pgf terms)");
  p->root = root;
  int64_t off = 0, pq = 1;
  for (int k = 0; k < K; ++k) {
    topo[k].off = off;
    off += (int64_t)1 << topo[k].L;
    if (k != root && topo[k].kind != WG_NODE_LEAF && topo[k].c1 >= 0) pq = std::max<int64_t>(pq, (int64_t)1 << topo[k].L);
  }
  p->nv = off;
  p->pq_n = pq;
  p->pq_smem = 2 * pq * (int64_t)sizeof(double) <= 40 * 1024;  // + static: under 48 KB
  for (int k = K - 1; k >= 0; --k)
    if (topo[k].kind != WG_NODE_LEAF) {
      depth[topo[k].c0] = depth[k] + 1;
      if (topo[k].c1 >= 0) depth[topo[k].c1] = depth[k] + 1;
    }
  // forward nodes by height, reverse nodes by depth (the root excluded)
  std::vector<int> lists;
  int H = 0, Dp = 0;
  for (int k = 0; k < K; ++k)
    if (k != root) H = std::max(H, height[k] + 1), Dp = std::max(Dp, depth[k]);
  std::vector<int> fo(1, 0), ro(1, 0);
  for (int h = 0; h < H; ++h) {
    for (int k = 0; k < K; ++k)
      if (k != root && height[k] == h) lists.push_back(k);
    fo.push_back((int)lists.size());
  }
  p->n_fwd = (int)lists.size();
  p->n_fwd_lv = H;
  lists.insert(lists.end(), fo.begin(), fo.end());
  const size_t rev0 = lists.size();
  for (int d = 1; d <= Dp; ++d) {
    for (int k = 0; k < K; ++k)
      if (k != root && depth[k] == d) lists.push_back(k);
    ro.push_back((int)(lists.size() - rev0));
  }
  p->n_rev = (int)(lists.size() - rev0);
  p->n_rev_lv = Dp;
  lists.insert(lists.end(), ro.begin(), ro.end());
  // root tiles
  const int L0 = topo[root].L0, L1 = topo[root].L - L0;
  p->lT0 = std::min(L0, 5);
  p->lT1 = std::min(L1, 10 - p->lT0);
  p->T0 = 1 << p->lT0;
  p->T1 = 1 << p->lT1;
  p->nt0 = 1 << (L0 - p->lT0);
  p->nt1 = 1 << (L1 - p->lT1);
  p->ntiles = p->nt0 * p->nt1;
  p->n_out = 2 * p->ntiles + 3 * K;
  const int64_t npart = ((int64_t)1 << L0) * p->nt1 + ((int64_t)1 << L1) * p->nt0;
  nck(cudaSetDevice(device), "cudaSetDevice");
  auto dal = [](void** d, size_t bytes) { nck(cudaMalloc(d, bytes ? bytes : 8), "cudaMalloc (condition)"); };
  dal((void**)&p->d_coef, sizeof(double) * 6 * K);
  dal((void**)&p->d_topo, sizeof(NwTopo) * K);
  dal((void**)&p->d_lists, sizeof(int) * lists.size());
  dal((void**)&p->d_v, sizeof(double) * p->nv);
  dal((void**)&p->d_bv, sizeof(double) * p->nv);
  if (!p->pq_smem) dal((void**)&p->d_pq, sizeof(double) * 2 * p->pq_n);
  dal((void**)&p->d_part, sizeof(double) * npart);
  dal((void**)&p->d_out, sizeof(double) * p->n_out);
  nck(cudaMallocHost((void**)&p->h_coef, sizeof(double) * 6 * K), "cudaMallocHost");
  nck(cudaMallocHost((void**)&p->h_out, sizeof(double) * p->n_out), "cudaMallocHost");
  nck(cudaMemcpy(p->d_topo, topo.data(), sizeof(NwTopo) * K, cudaMemcpyHostToDevice), "upload");
  nck(cudaMemcpy(p->d_lists, lists.data(), sizeof(int) * lists.size(), cudaMemcpyHostToDevice), "upload");
  nck(cudaStreamCreateWithFlags(&p->s, cudaStreamNonBlocking), "cudaStreamCreate");
  nck(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming), "cudaEventCreate");
  nck(cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming), "cudaEventCreate");
  return p;
}

void nw_stage(NwPlan& p, const Model& m) {
  if (!m.from_rates) throw Error(WG_ESTATE, "NowhereExtinctCondition needs the model's rates (wg_model_set_rates)");
  for (int k = 0; k < p.K; ++k) {
    double* c = p.h_coef + 6 * k;
    if (k == p.root) {
      c[0] = m.eta, c[1] = c[2] = c[3] = 0.0, c[5] = kNwRoot;
    } else {
      const double lam = m.lam[k], mu = m.mu[k], t = m.slice_len[k] * (m.nrow[k] - 1);
      c[0] = lam, c[1] = mu, c[2] = t, c[3] = std::exp((mu - lam) * t);
      c[5] = std::fabs(lam - mu) <= kNwCriticalAtol ? kNwCritical : kNwBdp;
    }
    c[4] = m.kind[k] == WG_NODE_WGD ? m.q[k] : 0.0;
  }
}

int nw_record(NwPlan& p, cudaStream_t s, bool grad) {
  nck(cudaMemcpyAsync(p.d_coef, p.h_coef, sizeof(double) * 6 * p.K, cudaMemcpyHostToDevice, s), "upload");
  const NwArgs a = nw_args(p);
  k_nw_fwd<<<1, kNwThreads, 0, s>>>(a);
  int n = 2;
  if (grad) {
    k_nw_root<true><<<p.ntiles, kNwTileThreads, 0, s>>>(a);
    k_nw_rev<<<1, kNwThreads, p.pq_smem ? 2 * p.pq_n * sizeof(double) : 0, s>>>(a);
    ++n;
  } else {
    k_nw_root<false><<<p.ntiles, kNwTileThreads, 0, s>>>(a);
  }
  nck(cudaGetLastError(), "condition launch");
  const int nout = grad ? p.n_out : p.ntiles;
  nck(cudaMemcpyAsync(p.h_out, p.d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost, s), "download");
  return n;
}

NwResult nw_result(const NwPlan& p, const Model& m, bool grad) {
  NwResult r;
  const double* o = p.h_out;
  double acc = 0.0;
  for (int b = 0; b < p.ntiles; ++b) acc += o[b];
  const double c = 1.0 - acc;
  r.ok = c > 0.0 && c < 1.0;
  r.value = r.ok ? std::log(c) : -INFINITY;
  if (!grad || !r.ok) return r;
  const int K = p.K;
  r.d_lam.assign(K, 0.0);
  r.d_mu.assign(K, 0.0);
  r.d_q.assign(K, 0.0);
  const double sc = 1.0 / c;  // ∂ log(1 - acc) with the kernels' seed -s_i
  double ge = 0.0;
  for (int b = 0; b < p.ntiles; ++b) ge += o[p.ntiles + b];
  r.d_eta = sc * ge;
  const double* nd = o + 2 * p.ntiles;
  for (int k = 0; k < K; ++k) {
    if (k == p.root) continue;
    r.d_lam[k] = sc * nd[3 * k];
    r.d_mu[k] = sc * nd[3 * k + 1];
    if (m.kind[k] == WG_NODE_WGD) r.d_q[k] = sc * nd[3 * k + 2];
  }
  return r;
}

}  // namespace wg
