"""The sampling entry point that allocates nothing (zc_sample_noalloc).

It exists for callers that cannot let the library allocate device memory
when they sample (a runtime owning all device memory in its own pool, a
loop that must not stall on cudaMalloc/cudaFree, a stream capture in
progress). Through the C ABI it must draw exactly the indices zc_sample
draws, on two calls in a row sharing its fixed scratch array. Collected
last so that a failure here leaves every other test already run.
"""

import numpy as np
import pytest

from helpers import rand_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", (64, 32))
def test_noalloc_sampler_matches_sampler(zc, prec):
    n = 18
    be = zc.CudaBackend(n, prec)
    be.load_state(rand_state(n, 123, normalize=True))
    be.finish()
    for shots, seed in ((5000, 7), (3000, 8)):  # two calls in a row, same scratch
        want = be.sample(shots, seed)
        got = be.sample_noalloc(shots, seed)
        assert np.array_equal(got, want), (prec, shots, seed)
    be.close()


def test_noalloc_sampler_after_gates_and_limits(zc):
    n = 16  # large enough that ops are queued for sweeps
    be = zc.CudaBackend(n, 64)
    be.apply_unitary([3], np.array([[1, 1], [1, -1]]) / np.sqrt(2))
    be.apply_cx(3, 7)
    with pytest.raises(zc.ZenoCudaError, match="zc_finish"):
        be.sample_noalloc(10, 1)
    be.finish()
    a = be.sample_noalloc(2000, 5)
    assert np.array_equal(a, be.sample(2000, 5))
    assert set(np.unique(a)) <= {0, (1 << 3) | (1 << 7)}
    with pytest.raises(zc.ZenoCudaError, match="16384 shots"):
        be.sample_noalloc(16385, 1)
    be.close()
