"""CPU oracle loader -- TEST INFRASTRUCTURE ONLY.

ctypes front end for ``whale_oracle.cpp``, the plain C++ restatement of
Whale.jl's likelihood (src/core.jl, src/model.jl, src/bdputil.jl,
src/condition.jl, src/rmodels.jl, src/ccd.jl).  Only the tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module; the product package never does.

Rates are passed exactly as the reference's parameter structs hold them:
``kind="DLWGD"`` takes log-scale branch rates indexed by node id
(src/rmodels.jl:55-64), ``kind="ConstantDLWGD"`` takes one natural-scale
λ and μ (src/rmodels.jl:31-33).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libwhale_oracle.so")
_lib = None

COND = {"none": 0, "root": 1, "nonextinct": 2, "nowhere": 3}


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, no FMA contraction, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_last_error.restype = C.c_char_p
        L.orc_model_new.restype = vp
        L.orc_model_new.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_int, C.c_int]
        L.orc_model_free.argtypes = [vp]
        L.orc_model_info.argtypes = [vp, ip, ip, ip, ip, ip, ip, ip, ip]
        L.orc_ccd_new.restype = vp
        L.orc_ccd_new.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.orc_ccd_free.argtypes = [vp]
        L.orc_ccd_info.argtypes = [vp, ip, ip]
        L.orc_ccd_clade.argtypes = [vp, C.c_int, C.POINTER(C.c_long), ip, ip, ip, ip, ip, ip, dp]
        rate_args = [vp, C.c_int, dp, C.c_int, dp, C.c_int, dp, C.c_int, C.c_double, dp, C.c_int]
        L.orc_logpdf.restype = C.c_double
        L.orc_logpdf.argtypes = rate_args + [C.POINTER(vp), C.c_int, dp, C.c_int]
        L.orc_gradient.restype = C.c_double
        L.orc_gradient.argtypes = rate_args + [C.POINTER(vp), C.c_int, dp, C.c_int]
        L.orc_condition.restype = C.c_double
        L.orc_condition.argtypes = rate_args
        L.orc_tables.restype = C.c_int
        L.orc_tables.argtypes = rate_args + [dp, dp, dp]
        L.orc_family_tables.restype = C.c_int
        L.orc_family_tables.argtypes = rate_args + [vp, dp, C.c_long]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleModel:
    """WhaleModel restatement: tree with WGD nodes given as unary Newick nodes."""

    def __init__(self, newick: str, dt: float, minn: int = 5, maxn: int = 10000, condition: str = "root"):
        L = lib()
        self._h = L.orc_model_new(newick.encode(), dt, minn, maxn, COND[condition])
        if not self._h:
            raise ValueError(L.orc_last_error().decode())
        n, nw, ng = C.c_int(), C.c_int(), C.c_int()
        L.orc_model_info(self._h, C.byref(n), C.byref(nw), C.byref(ng), None, None, None, None, None)
        self.n_nodes, self.nonwgd, self.nwgd = n.value, nw.value, ng.value
        arrs = [np.zeros(self.n_nodes, np.int32) for _ in range(5)]
        ptr = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs]
        L.orc_model_info(self._h, C.byref(n), C.byref(nw), C.byref(ng), *ptr)
        self.ids, self.wgdids, self.kinds, self.nrows, self.parents = arrs

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_model_free(self._h)
            self._h = None

    def _rates(self, kind, lam, mu, q, eta, p):
        lam = np.ascontiguousarray(np.atleast_1d(np.asarray(lam, np.float64)))
        mu = np.ascontiguousarray(np.atleast_1d(np.asarray(mu, np.float64)))
        q = np.ascontiguousarray(np.asarray(q if q is not None else [], np.float64).reshape(-1))
        p = np.ascontiguousarray(np.asarray(p if p is not None else [], np.float64).reshape(-1))
        k = 0 if kind == "DLWGD" else 1
        keep = (lam, mu, q, p)
        return keep, [self._h, k, _dp(lam), lam.size, _dp(mu), mu.size, _dp(q), q.size, float(eta), _dp(p), p.size]

    def logpdf(self, ccds, lam, mu, q=None, eta=0.66, p=None, kind="DLWGD", nthreads=0):
        """Returns (total, per_family) as in src/core.jl:39-64."""
        keep, args = self._rates(kind, lam, mu, q, eta, p)
        arr = (C.c_void_p * len(ccds))(*[c._h for c in ccds])
        per = np.zeros(len(ccds))
        tot = lib().orc_logpdf(*args, arr, len(ccds), _dp(per), nthreads)
        return tot, per

    def gradient(self, ccds, lam, mu, q=None, eta=0.66, p=None, kind="DLWGD", nthreads=0):
        """Returns (total, grad) with grad over [λ..., μ..., q..., η]."""
        keep, args = self._rates(kind, lam, mu, q, eta, p)
        arr = (C.c_void_p * len(ccds))(*[c._h for c in ccds])
        P = keep[0].size + keep[1].size + keep[2].size + 1
        g = np.zeros(P)
        tot = lib().orc_gradient(*args, arr, len(ccds), _dp(g), nthreads)
        return tot, g

    def condition(self, lam, mu, q=None, eta=0.66, p=None, kind="DLWGD"):
        keep, args = self._rates(kind, lam, mu, q, eta, p)
        return lib().orc_condition(*args)

    def tables(self, lam, mu, q=None, eta=0.66, p=None, kind="DLWGD"):
        keep, args = self._rates(kind, lam, mu, q, eta, p)
        tot = int(self.nrows.sum())
        e, f, s = np.zeros(tot), np.zeros(tot), np.zeros(tot)
        lib().orc_tables(*args, _dp(e), _dp(f), _dp(s))
        return e, f, s

    def family_tables(self, ccd, lam, mu, q=None, eta=0.66, p=None, kind="DLWGD"):
        keep, args = self._rates(kind, lam, mu, q, eta, p)
        n = lib().orc_family_tables(*args, ccd._h, None, 0)
        out = np.zeros(n)
        lib().orc_family_tables(*args, ccd._h, _dp(out), n)
        return out


class OracleCCD:
    """CCD restatement parsed from ALE v0.4 text (src/ccd.jl:102-248)."""

    def __init__(self, model: OracleModel, text: str, fname: str = ""):
        L = lib()
        self._h = L.orc_ccd_new(model._h, text.encode(), fname.encode())
        if not self._h:
            raise ValueError(L.orc_last_error().decode())
        nc, nt = C.c_int(), C.c_int()
        L.orc_ccd_info(self._h, C.byref(nc), C.byref(nt))
        self.n_clades, self.n_triples = nc.value, nt.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_ccd_free(self._h)
            self._h = None

    def clade(self, i):
        L = lib()
        cnt = C.c_long()
        nl, ns, nsp = C.c_int(), C.c_int(), C.c_int()
        L.orc_ccd_clade(self._h, i, C.byref(cnt), C.byref(nl), C.byref(ns), C.byref(nsp), None, None, None, None)
        sp = np.zeros(max(nsp.value, 1), np.int32)
        g1 = np.zeros(max(ns.value, 1), np.int32)
        g2 = np.zeros(max(ns.value, 1), np.int32)
        p = np.zeros(max(ns.value, 1))
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        L.orc_ccd_clade(self._h, i, C.byref(cnt), C.byref(nl), C.byref(ns), C.byref(nsp), ip(sp), ip(g1), ip(g2), _dp(p))
        return dict(count=cnt.value, nleaves=nl.value, species=sp[: nsp.value].tolist(),
                    splits=list(zip(g1[: ns.value].tolist(), g2[: ns.value].tolist(), p[: ns.value].tolist())))


def read_ale_files(model: OracleModel, paths):
    out = []
    for pth in paths:
        with open(pth) as fh:
            out.append(OracleCCD(model, fh.read(), os.path.basename(pth)))
    return out


def parse_texts(model: OracleModel, texts, threads: int = 0):
    """OracleCCDs of many ALE texts, parsed on host threads (ctypes releases
    the GIL during each parse); results in input order."""
    from concurrent.futures import ThreadPoolExecutor

    n = threads or os.cpu_count() or 1
    with ThreadPoolExecutor(max_workers=n) as ex:
        return list(ex.map(lambda s: OracleCCD(model, s), texts))
