"""Order of the size classes' launches: a class's adjoint after its own
forward (at the class's stream priority, the lowest or the highest) or after every
class's forward.  Only the order of independent work changes, so log L and
the gradient are bit-identical across the three, and the default (the
adjoint on its own forward's heels) agrees with the oracle on the golden
families."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_overlap_modes_are_bit_identical(W, monkeypatch):
    from whale_gb300 import synth

    wl = synth.config1(seed=4, n_families=300)
    wm, ccds = wl.model, wl.ccds()
    out = []
    for mode in ("0", "1", "2", "3"):
        monkeypatch.setenv("WG_ADJ_OVERLAP", mode)
        b = W.Batch(wm, ccds, grad=True)
        out.append(b.grad_nodes(wm))
        del b
    for other in out[1:]:
        for x, y in zip(out[0], other):
            assert np.array_equal(np.asarray(x), np.asarray(y))
    monkeypatch.setenv("WG_ADJ_OVERLAP", "4")
    with pytest.raises(W.WhaleError, match="out of range"):
        W.Batch(wm, ccds, grad=True)
