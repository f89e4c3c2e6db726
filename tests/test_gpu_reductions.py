"""Reductions and the sampler at sizes with many 2^16-element chunks.

Exact mode: the warp-specialised chain kernels keep the reference's serial
f64 order (src/sample.rs:38-108, src/state.rs:143-156, :599-626), so
norm_sqr, prob_one and every sampled index equal the oracle's bit for bit,
including partial CTAs (chunk counts not a multiple of 32) and draws that
resolve by replaying one recorded stage.

Fast mode: parallel double-float sums. Values agree with the oracle to
~1e-13 relative; a sampled index may differ only where its draw falls within
rounding distance of a cumulative boundary, so almost all indices agree and
every index drawn has nonzero probability.
"""

import numpy as np
import pytest

from helpers import rand_state

pytestmark = pytest.mark.gpu


def pair(zc, oracle, n, prec, amps, flags):
    g = zc.CudaBackend(n, prec, flags)
    g.load_state(amps)
    o = oracle.State(n, prec)
    o.load(amps)
    return g, o


@pytest.mark.parametrize("prec", (64, 32))
def test_exact_many_chunks(zc, oracle, prec):
    for n, shots in ((21, 3000), (23, 20000)):  # 32 and 128 chunks
        amps = rand_state(n, 900 + n, normalize=True)
        g, o = pair(zc, oracle, n, prec, amps, zc.FLAG_EXACT)
        assert g.norm_sqr() == o.norm_sqr()
        for q in (0, 5, 16, n - 1):
            assert g.prob_one(q) == o.prob_one(q), (n, q)
        a, b = g.sample(shots, 11), o.sample(shots, 11)
        assert np.array_equal(a, b), (n, int(np.sum(a != b)))
        g.close()


def test_exact_skewed_state(zc, oracle):
    """Mass concentrated in a few chunks: many draws per chunk, early stops."""
    n = 20
    amps = rand_state(n, 77) * 1e-3
    amps[(3 << 16) + 100:(3 << 16) + 140] = 1.0
    amps[(9 << 16) + 65000] = 2.0
    amps /= np.linalg.norm(amps)
    for prec in (64, 32):
        g, o = pair(zc, oracle, n, prec, amps, zc.FLAG_EXACT)
        a, b = g.sample(30000, 3), o.sample(30000, 3)
        assert np.array_equal(a, b)
        g.close()


@pytest.mark.parametrize("prec", (64, 32))
def test_fast_reductions_and_sampler(zc, oracle, prec):
    for n in (10, 17, 21):
        amps = rand_state(n, 300 + n, normalize=True)
        g, o = pair(zc, oracle, n, prec, amps, zc.FLAG_FAST)
        ref = o.norm_sqr()
        assert abs(g.norm_sqr() - ref) <= 1e-13 * ref
        for q in (0, n // 2, n - 1):
            p = o.prob_one(q)
            assert abs(g.prob_one(q) - p) <= 1e-13 * p, (n, q)
        shots = 8192
        a, b = g.sample(shots, 5), o.sample(shots, 5)
        assert np.all(np.diff(a.astype(np.int64)) >= 0)
        assert np.mean(a == b) >= 0.999, (n, int(np.sum(a != b)))
        probs = np.abs(o.statevector()) ** 2
        assert np.all(probs[a.astype(np.int64)] > 0)
        g.close()


def test_fast_sparse_state(zc, oracle):
    n = 18
    amps = np.zeros(1 << n, complex)
    amps[5] = 0.6
    amps[(1 << 17) + 3] = 0.8j
    for prec in (64, 32):
        g, o = pair(zc, oracle, n, prec, amps, zc.FLAG_FAST)
        a = g.sample(10000, 9)
        assert set(np.unique(a)) <= {5, (1 << 17) + 3}
        assert abs(np.mean(a == 5) - 0.36) < 0.03
        g.close()
