"""The likelihood API: ``logpdf``, ``logpdf_inplace`` (``logpdf!``),
``loglikelihood`` and the gradient, evaluated on one GB300 by libwhalegpu.

Reference semantics (src/core.jl):
  logpdf(wm, x::CCD)            :39-43  per-family log L, no conditioning,
                                        -Inf when L <= 0
  logpdf(wm, xs::Vector{CCD})   :58-64  Σ log L - N·condition(wm), non-finite
                                        mapped to -Inf (ℓhood, :15)
  logpdf!(wm, x / xs)           :29-37, :46-56  same values; the DP tables are
                                        kept in ccd.ℓ for backtracking
  loglikelihood(wm, x)          :17, :81
The gradient replaces ForwardDiff.gradient over the rates struct
(test/runtests.jl:36-38): it is computed by the hand-written adjoint kernel.

Families are uploaded once per distinct list of CCDs and stay resident on the
device; every call re-uploads only the slice tables of the current rates.
There is no CPU path: without a CUDA device these functions raise.
"""
from __future__ import annotations

import threading
import weakref
from typing import Dict, List, Sequence, Tuple, Union

import numpy as np

from . import _native as N
from .ccd import CCD
from .model import ConstantDLWGD, DLWGD, WhaleModel


class Context:
    """One CUDA device and stream (wg_ctx)."""

    def __init__(self, device: int = 0):
        h = N.vp()
        N.check(N.lib().wg_ctx_create(int(device), N.C.byref(h)))
        self.h = h
        self.device = device

    @property
    def stream(self) -> int:
        return N.lib().wg_ctx_stream(self.h) or 0

    def __del__(self):
        if getattr(self, "h", None) and N._lib is not None:
            N._lib.wg_ctx_destroy(self.h)
            self.h = None


_ctx_lock = threading.Lock()
_default_ctx: Context = None


def default_context() -> Context:
    global _default_ctx
    with _ctx_lock:
        if _default_ctx is None:
            _default_ctx = Context(0)
        return _default_ctx


def nowhere_condition(wm: WhaleModel, grad: bool = False, ctx: Context = None):
    """NowhereExtinctCondition of ``wm``'s tree and rates, on the device
    (src/condition.jl:31-36, src/bdputil.jl:84-135): log P(every leaf keeps
    a copy).  With ``grad``, also its derivatives on the per-node natural
    rates λ, μ, q (positions of ``wm.order``) and on η, as a dict.  Batched
    evaluations of a model carrying this condition compute it the same way."""
    wm.load()
    ctx = ctx or default_context()
    v = N.dbl()
    L = N.lib()
    if not grad:
        N.check(L.wg_nowhere_condition(ctx.h, wm._struct.h, N.C.byref(v), None, None, None, None))
        return v.value
    K = len(wm.order)
    dl, dm, dq, de = np.zeros(K), np.zeros(K), np.zeros(K), np.zeros(1)
    N.check(L.wg_nowhere_condition(ctx.h, wm._struct.h, N.C.byref(v), N.dptr(dl), N.dptr(dm), N.dptr(dq),
                                   N.dptr(de)))
    return v.value, {"λ": dl, "μ": dm, "q": dq, "η": float(de[0])}


class Batch:
    """Device-resident packed families (wg_batch) for one model structure."""

    def __init__(self, wm: WhaleModel, ccds: Sequence[CCD], grad: bool = False, tables: bool = False,
                 ctx: Context = None, scratch_rows: bool = False, checkpoint: bool = False,
                 persistent: bool = False):
        """scratch_rows: every task keeps its working rows in device memory,
        as tasks too wide for shared memory always do (testing aid).
        checkpoint: the adjoint recomputes each height level's DP tables from
        the children's top rows instead of keeping every table (a gradient
        batch does this by itself for its largest size classes when the
        tables would exceed the device-memory budget).
        persistent: one persistent launch per pass over every task, CTAs
        taking tasks in a topological order (bounded dependency waits)."""
        self.ctx = ctx or default_context()
        self.ccds = list(ccds)
        self.n = len(self.ccds)
        flags = ((N.BATCH_GRAD if grad else 0) | (N.BATCH_TABLES if tables else 0)
                 | (N.BATCH_SCRATCH_ROWS if scratch_rows else 0) | (N.BATCH_CHECKPOINT if checkpoint else 0)
                 | (N.BATCH_PERSISTENT if persistent else 0))
        arr = (N.C.c_void_p * self.n)(*[c._h for c in self.ccds])
        h = N.vp()
        N.check(N.lib().wg_batch_create(self.ctx.h, wm._struct.h, arr, self.n, flags, N.C.byref(h)))
        self.h = h
        self.struct = wm._struct
        self.grad = grad
        self.tables = tables
        nf, ng = N.i32(), N.i32()
        by = N.i64()
        ff, fb, fa = N.dbl(), N.dbl(), N.dbl()
        N.check(N.lib().wg_batch_info(self.h, N.C.byref(nf), N.C.byref(ng), N.C.byref(by), N.C.byref(ff),
                                      N.C.byref(fb), N.C.byref(fa)))
        self.n_groups, self.device_bytes = ng.value, by.value
        self.flops_fwd, self.bytes_fwd, self.flops_adj = ff.value, fb.value, fa.value

    def tables_layout(self):
        """(size classes, classes recomputing their tables per level, doubles
        every table would take, doubles of tables held on the device)."""
        c, k = N.i32(), N.i32()
        full, kept = N.i64(), N.i64()
        N.check(N.lib().wg_batch_tables_layout(self.h, N.C.byref(c), N.C.byref(k), N.C.byref(full),
                                               N.C.byref(kept)))
        return c.value, k.value, full.value, kept.value

    def __del__(self):
        if getattr(self, "h", None) and N._lib is not None:
            N._lib.wg_batch_destroy(self.h)
            self.h = None

    # ---- evaluation
    def logpdf(self, wm: WhaleModel, per_family: bool = False):
        wm.load()
        per = np.zeros(self.n)
        tot = N.dbl()
        N.check(N.lib().wg_logpdf(self.ctx.h, wm._struct.h, self.h, N.dptr(per), N.C.byref(tot)))
        return (tot.value, per) if per_family else tot.value

    def logpdf_plain(self, wm: WhaleModel):
        wm.load()
        per = np.zeros(self.n)
        tot = N.dbl()
        N.check(N.lib().wg_logpdf_plain(self.ctx.h, wm._struct.h, self.h, N.dptr(per), N.C.byref(tot)))
        return tot.value, per

    def grad_nodes(self, wm: WhaleModel):
        """Total, per-family logL and the adjoints of the per-node natural rates."""
        if not self.grad:
            raise ValueError("batch was created without gradient support")
        wm.load()
        K = len(wm.order)
        per = np.zeros(self.n)
        dl, dm, dq = np.zeros(K), np.zeros(K), np.zeros(K)
        de = N.dbl()
        tot = N.dbl()
        N.check(N.lib().wg_logpdf_grad(self.ctx.h, wm._struct.h, self.h, N.dptr(per), N.C.byref(tot), N.dptr(dl),
                                       N.dptr(dm), N.dptr(dq), N.C.byref(de), None, None, None))
        return tot.value, per, dl, dm, dq, de.value

    def grad_nodes_weighted(self, wm: WhaleModel, weights, cond_scale: float):
        """As grad_nodes for Σ_i weights[i]·log L_i - cond_scale·condition."""
        if not self.grad:
            raise ValueError("batch was created without gradient support")
        wm.load()
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.shape != (self.n,):
            raise ValueError(f"need {self.n} family weights")
        K = len(wm.order)
        per = np.zeros(self.n)
        dl, dm, dq = np.zeros(K), np.zeros(K), np.zeros(K)
        de = N.dbl()
        tot = N.dbl()
        N.check(N.lib().wg_logpdf_grad_weighted(self.ctx.h, wm._struct.h, self.h, N.dptr(w), float(cond_scale),
                                                N.dptr(per), N.C.byref(tot), N.dptr(dl), N.dptr(dm), N.dptr(dq),
                                                N.C.byref(de), None, None, None))
        return tot.value, per, dl, dm, dq, de.value

    def grad_tables(self, wm: WhaleModel):
        """Adjoints of the slice tables (ε, ϕ, ψ per row), q per node and η."""
        wm.load()
        NR = wm._struct.total_rows
        K = len(wm.order)
        de, dp, ds, dq = np.zeros(NR), np.zeros(NR), np.zeros(NR), np.zeros(K)
        deta, tot = N.dbl(), N.dbl()
        N.check(N.lib().wg_logpdf_grad(self.ctx.h, wm._struct.h, self.h, None, N.C.byref(tot), None, None,
                                       N.dptr(dq), N.C.byref(deta), N.dptr(de), N.dptr(dp), N.dptr(ds)))
        return tot.value, de, dp, ds, dq, deta.value

    def family_tables(self, wm: WhaleModel, i: int):
        wm.load()
        need = N.i64()
        N.check(N.lib().wg_logpdf_tables(self.ctx.h, wm._struct.h, self.h, i, None, 0, N.C.byref(need), None))
        out = np.zeros(max(need.value, 1))
        ll = N.dbl()
        N.check(N.lib().wg_logpdf_tables(self.ctx.h, wm._struct.h, self.h, i, N.dptr(out), need.value,
                                         N.C.byref(need), N.C.byref(ll)))
        return ll.value, out[: need.value]

    def last_tables(self, i: int):
        """Family i's log L and DP tables as the last fetched evaluation of
        this batch left them (no evaluation here; ``family_tables`` layout)."""
        need = N.i64()
        N.check(N.lib().wg_batch_tables(self.ctx.h, self.h, i, None, 0, N.C.byref(need), None))
        out = np.zeros(max(need.value, 1))
        ll = N.dbl()
        N.check(N.lib().wg_batch_tables(self.ctx.h, self.h, i, N.dptr(out), need.value, N.C.byref(need),
                                        N.C.byref(ll)))
        return ll.value, out[: need.value]


# cache of device batches keyed by the model structure and the CCD objects
_batches: Dict[Tuple, Batch] = {}
_batch_lock = threading.Lock()


def get_batch(wm: WhaleModel, ccds: Sequence[CCD], grad: bool = False, tables: bool = False) -> Batch:
    key = (id(wm._struct), tuple(id(c) for c in ccds), grad, tables)
    with _batch_lock:
        b = _batches.get(key)
        if b is not None and b.struct is wm._struct and all(x is y for x, y in zip(b.ccds, ccds)):
            return b
        if len(_batches) > 16:
            _batches.clear()
        b = Batch(wm, ccds, grad=grad, tables=tables)
        _batches[key] = b
        return b


def logpdf(wm: WhaleModel, x: Union[CCD, Sequence[CCD]]) -> float:
    """``logpdf(wm, x)``: a single CCD gives its unconditioned log L; a vector
    gives Σ log L - N·condition (src/core.jl:39-43, :58-64).  A MixtureModel
    or ModelArray dispatches to its own form (src/core.jl:66-79)."""
    from . import mixture

    if isinstance(wm, mixture.MixtureModel):
        return mixture.logpdf(wm, x)
    if isinstance(wm, mixture.ModelArray):
        return mixture.modelarray_logpdf(wm, x)
    if isinstance(x, CCD):
        _, per = get_batch(wm, [x]).logpdf(wm, per_family=True)
        return float(per[0])
    return get_batch(wm, list(x)).logpdf(wm)


def loglikelihood(wm: WhaleModel, x) -> float:
    return logpdf(wm, x)


def logpdf_inplace(wm: WhaleModel, x: Union[CCD, Sequence[CCD]]) -> float:
    """``logpdf!``: as logpdf, and every family's DP tables are stored in
    ``ccd.ℓ`` (one (nslices+1) x ncompat array per node, in node order)."""
    single = isinstance(x, CCD)
    xs = [x] if single else list(x)
    b = get_batch(wm, xs, tables=True)
    tot, per = b.logpdf(wm, per_family=True)
    for i, c in enumerate(xs):
        _, flat = b.family_tables(wm, i)
        c.ℓ = _split_tables(wm, c, flat)
    return float(per[0]) if single else tot


def _split_tables(wm, c, flat):
    out = []
    o = 0
    nrow = wm._struct.nrow
    sizes = _ncompat(wm, c)
    for k in range(len(wm.order)):
        n = int(nrow[k]) * sizes[k]
        out.append(flat[o:o + n].reshape(int(nrow[k]), sizes[k]))
        o += n
    return out


def _ncompat(wm, c):
    a = c.arrays()
    spo, sp = a["species_offsets"], a["species"]
    res = []
    for m in wm.order:
        cl = set(m.clade)
        n = 0
        for g in range(c.n_clades):
            if all(int(s) in cl for s in sp[spo[g]:spo[g + 1]]):
                n += 1
        res.append(n)
    return res


def logpdf_plain(wm: WhaleModel, xs: Sequence[CCD]):
    """One family per launch (the plain per-family GPU path)."""
    return get_batch(wm, list(xs)).logpdf_plain(wm)


def logpdf_gradient(wm: WhaleModel, xs: Sequence[CCD]):
    """Σ log L - N·condition and its gradient w.r.t. the rates struct:
    for DLWGD a dict with 'λ', 'μ' (log-scale, by node id), 'q', 'η'; for
    ConstantDLWGD scalars 'λ', 'μ', vector 'q' and 'η'.  A MixtureModel
    returns (total, [gradient per component], d/d prior); a ModelArray
    returns (total, [(model, gradient) per distinct model])."""
    from . import mixture

    if isinstance(wm, mixture.MixtureModel):
        return mixture.logpdf_gradient(wm, xs)
    if isinstance(wm, mixture.ModelArray):
        return mixture.modelarray_logpdf_gradient(wm, xs)
    b = get_batch(wm, list(xs), grad=True)
    tot, per, dl, dm, dq, deta = b.grad_nodes(wm)
    return tot, map_gradient(wm, dl, dm, dq, deta)


def map_gradient(wm: WhaleModel, dl, dm, dq, deta):
    """Chain per-node natural-rate adjoints to the rates struct's fields
    (getθ, src/rmodels.jl:31-33, :55-64)."""
    r = wm.rates
    lam, mu, _, _, _ = wm.node_rates()
    gq = np.zeros(r.q.size)
    for m in wm.order:
        if m.wgdid > 0:
            gq[m.wgdid - 1] += dq[m.pos]
    if isinstance(r, ConstantDLWGD):
        ok = ~np.isnan(lam)
        return {"λ": float(np.sum(dl[ok])), "μ": float(np.sum(dm[ok])), "q": gq, "η": deta}
    gl = np.zeros(r.λ.size)
    gm = np.zeros(r.μ.size)
    for m in wm.order:
        k = m.pos
        if np.isnan(lam[k]):
            continue
        tgt = wm.order[wm.nonwgdchild(k)].id if m.kind == N.NODE_WGD else m.id
        gl[tgt - 1] += dl[k] * lam[k]
        gm[tgt - 1] += dm[k] * mu[k]
    return {"λ": gl, "μ": gm, "q": gq, "η": deta}


def gradient(wm: WhaleModel, xs: Sequence[CCD]) -> np.ndarray:
    """Flat gradient in the order of the reference's test vector
    x = [λ; μ; q; η] (test/runtests.jl:36-37)."""
    _, g = logpdf_gradient(wm, xs)
    if isinstance(wm.rates, ConstantDLWGD):
        return np.concatenate([[g["λ"], g["μ"]], g["q"], [g["η"]]])
    return np.concatenate([g["λ"], g["μ"], g["q"], [g["η"]]])
