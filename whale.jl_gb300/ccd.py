"""Conditional clade distributions: ``read_ale`` and the ``CCD`` type.

``read_ale(path, wm)`` (src/ccd.jl:126-137) accepts a single ``.ale`` file, a
directory (all entries, sorted, as Julia's readdir gives them) or a text file
listing paths; lines starting with '#' are skipped.  Parsing is done by the
native reader (wg_ccd_parse_ale), which restates parse_aleobserve,
addleafclades!, addubiquitous! and CCD(ale, wm, spmap) (src/ccd.jl:102-248).
"""
from __future__ import annotations

import os
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N


class CCD:
    """One gene family's CCD in the reference layout: clades ordered by size
    (leaves first, ubiquitous clade last), splits (γ1, γ2, p = Dip/Bip)."""

    def __init__(self, handle, fname: str = ""):
        self._h = handle
        self.fname = fname
        nc, nt, ng = N.i32(), N.i32(), N.i32()
        obs = N.i64()
        N.check(N.lib().wg_ccd_info(self._h, N.C.byref(nc), N.C.byref(nt), N.C.byref(obs), N.C.byref(ng)))
        self.n_clades, self.n_triples, self.total, self.n_genes = nc.value, nt.value, obs.value, ng.value
        self.ℓ: Optional[list] = None  # DP tables after logpdf_inplace (logpdf!)

    def __len__(self) -> int:
        return self.n_clades

    def __del__(self):
        if getattr(self, "_h", None) and N._lib is not None:
            N._lib.wg_ccd_destroy(self._h)
            self._h = None

    def __repr__(self) -> str:
        return f"CCD(Γ={self.n_clades}, 𝓛={self.n_genes})"

    def arrays(self):
        """Clade table: nleaves, counts, species CSR, split CSR (g1, g2, p)."""
        n, T = self.n_clades, self.n_triples
        nleaves = np.zeros(n, np.int32)
        counts = np.zeros(n, np.int64)
        spo = np.zeros(n + 1, np.int32)
        N.check(N.lib().wg_ccd_export(self._h, N.iptr(nleaves), N.lptr(counts), N.iptr(spo), None, None, None,
                                      None, None))
        sp = np.zeros(max(int(spo[-1]), 1), np.int32)
        so = np.zeros(n + 1, np.int32)
        g1 = np.zeros(max(T, 1), np.int32)
        g2 = np.zeros(max(T, 1), np.int32)
        p = np.zeros(max(T, 1), np.float64)
        N.check(N.lib().wg_ccd_export(self._h, None, None, None, N.iptr(sp), N.iptr(so), N.iptr(g1), N.iptr(g2),
                                      N.dptr(p)))
        return dict(nleaves=nleaves, counts=counts, species_offsets=spo, species=sp[: spo[-1]],
                    split_offsets=so, g1=g1[:T], g2=g2[:T], p=p[:T])

    @classmethod
    def from_arrays(cls, nleaves, species_offsets, species, split_offsets, g1, g2, p, observations=0, fname=""):
        a = [np.ascontiguousarray(x, dtype=np.int32) for x in (nleaves, species_offsets, species, split_offsets, g1, g2)]
        pp = np.ascontiguousarray(p, dtype=np.float64)
        h = N.vp()
        N.check(N.lib().wg_ccd_create(len(a[0]), *[N.iptr(x) for x in a], N.dptr(pp), int(observations),
                                      N.C.byref(h)))
        return cls(h, fname)


def _spmap_arrays(wm):
    names = list(wm.spmap.keys())
    ids = np.array([wm.spmap[k] for k in names], np.int32)
    enc = (N.C.c_char_p * len(names))(*[k.encode() for k in names])
    return enc, ids


def parse_ale_text(text: str, wm, fname: str = "") -> CCD:
    enc, ids = _spmap_arrays(wm)
    b = text.encode()
    h = N.vp()
    N.check(N.lib().wg_ccd_parse_ale(b, len(b), enc, N.iptr(ids), len(ids), N.C.byref(h)))
    return CCD(h, fname)


def read_ale(path: str, wm, threads: int = 0) -> List[CCD]:
    """``read_ale(s, wm)`` (src/ccd.jl:126-137): one file, a directory (its
    files in sorted order) or a file listing paths.  The files are read and
    parsed natively on ``threads`` host threads (0: every core)."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"Not a file nor directory `{path}`")
    if os.path.isfile(path) and path.endswith(".ale"):
        files = [path]
    else:
        if os.path.isfile(path):
            with open(path) as fh:
                files = [l.rstrip("\n") for l in fh]
        else:
            files = [os.path.join(path, f) for f in sorted(os.listdir(path))]
        files = [f for f in files if not f.startswith("#")]
    enc, ids = _spmap_arrays(wm)
    n = len(files)
    paths = (N.C.c_char_p * max(n, 1))(*[f.encode() for f in files])
    out = (N.vp * max(n, 1))()
    failed = N.C.c_int32(-1)
    N.check(N.lib().wg_ccd_read_ale_files(paths, n, enc, N.iptr(ids), len(ids), int(threads), out,
                                          N.C.byref(failed)))
    return [CCD(N.vp(out[i]), os.path.basename(f)) for i, f in enumerate(files)]
