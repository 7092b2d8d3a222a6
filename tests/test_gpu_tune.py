"""The packing autotuner on the device: it times its candidates and returns
the fastest setting with its batch, which evaluates like the default layout
(per-family log L and gradient equal to rounding)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tuned_batch_evaluates_like_the_default(W):
    from whale_gb300 import synth

    wl = synth.config1(n_families=80)
    wm, ccds = wl.model, wl.ccds()
    neighbours = {"target_ops": (320, 480), "target_j": (3,), "root_group": (16,), "heavy_ops": (1024,)}
    best, b, log = W.tune(wm, ccds, steps=2, warmup=1, neighbours=neighbours, rounds=1)
    assert best["target_ops"] in (320, 480) and b is not None
    assert len(log) == 2 and all(ms > 0 for _, ms in log)
    ref = W.Batch(wm, ccds, grad=True)
    t0, p0, dl0, dm0, dq0, de0 = ref.grad_nodes(wm)
    t1, p1, dl1, dm1, dq1, de1 = b.grad_nodes(wm)
    assert np.allclose(p1, p0, rtol=1e-12, atol=0.0)
    for x, y in ((dl1, dl0), (dm1, dm0), (dq1, dq0), (de1, de0)):
        assert np.allclose(x, y, rtol=1e-9, atol=1e-12)
