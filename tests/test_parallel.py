"""Family sharding across ranks with one all-reduce, on world-size-2 gloo CPU
ranks.  Each rank evaluates its shard with the oracle (no GPU here); the
reduced total and gradient must equal the single-process values."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import sys

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    import __graft_entry__
    import oracle as O

    W = __graft_entry__.load_package()
    from whale_gb300 import parallel, synth

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = synth.config0(seed=4, n_families=24)
    wm = wl.model
    ccds = wl.ccds()
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    occ = [O.OracleCCD(om, s) for s in wl.ale]
    by_id = {id(c): oc for c, oc in zip(ccds, occ)}
    r = wm.rates

    def evaluate(model, xs):
        return om.gradient([by_id[id(x)] for x in xs], [r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD",
                           nthreads=1)

    tot, g = parallel.distributed_logpdf_gradient(wm, ccds, evaluate=evaluate)
    if rank == 0:
        np.save(out_path, np.r_[tot, g])
    dist.barrier()
    dist.destroy_process_group()


def test_shard_is_a_partition(W):
    from whale_gb300.parallel import shard_families

    w = np.random.default_rng(0).lognormal(size=101)
    sh = shard_families(w, 4)
    assert sorted(i for s in sh for i in s) == list(range(101))
    loads = [w[s].sum() for s in sh]
    assert max(loads) - min(loads) <= w.max()


def test_two_rank_allreduce_equals_single_process(tmp_path, W, O):
    import torch.multiprocessing as mp

    out = str(tmp_path / "res.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    from whale_gb300 import synth

    wl = synth.config0(seed=4, n_families=24)
    wm = wl.model
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    r = wm.rates
    tot, g = om.gradient([O.OracleCCD(om, s) for s in wl.ale], [r.λ], [r.μ], q=r.q, eta=r.η,
                         kind="ConstantDLWGD")
    assert got[0] == pytest.approx(tot, rel=1e-12)
    assert np.allclose(got[1:], g, rtol=1e-10, atol=1e-10)
