"""The sampling entry point that allocates nothing (zc_sample_noalloc).

It exists for callers that cannot let the library allocate device memory
when they sample: a runtime that owns all device memory in its own pool, or
a loop that must not stall on cudaMalloc/cudaFree. Through the C ABI it
must draw exactly the indices zeno's sampler draws — exact-mode zc_sample's
— on two calls in a row sharing its fixed scratch array, on states of
either arithmetic flag, without changing the device's free memory. Collected
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


@pytest.mark.parametrize("prec", (64, 32))
def test_noalloc_on_fast_state_draws_exact_mode_indices(zc, prec):
    """On a ZC_FLAG_FAST state the call still draws exact-mode indices: the
    same amplitudes loaded into an exact-mode state sample identically."""
    n = 19
    fast = zc.CudaBackend(n, prec, zc.FLAG_FAST)
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    rng = np.random.default_rng(5)
    for q in range(n):
        th, ph, la = rng.uniform(0, 2 * np.pi, 3)
        u = np.array([[np.cos(th / 2), -np.exp(1j * la) * np.sin(th / 2)],
                      [np.exp(1j * ph) * np.sin(th / 2), np.exp(1j * (ph + la)) * np.cos(th / 2)]])
        fast.apply_unitary([q], u)
        fast.apply_unitary([(q + 3) % n], h)
    fast.finish()
    amps = fast.statevector()
    exact = zc.CudaBackend(n, prec, zc.FLAG_EXACT)
    exact.load_state(amps)
    exact.finish()
    assert np.array_equal(exact.statevector(), amps)
    for shots, seed in ((8192, 11), (4096, 12)):
        assert np.array_equal(fast.sample_noalloc(shots, seed), exact.sample(shots, seed)), (prec, seed)
    fast.close()
    exact.close()


def test_noalloc_sampler_allocates_nothing(zc):
    """A fresh 20-qubit state samples through the entry point twice without
    any change in the device's free memory (zc_sample would grow its
    buffers on the first call). A first call on another state loads the
    kernels and resolves the scratch address before the measurement."""
    import torch

    warm = zc.CudaBackend(12, 64)
    warm.sample_noalloc(64, 1)
    warm.close()
    be = zc.CudaBackend(20, 64)
    be.load_state(rand_state(20, 77, normalize=True))
    be.finish()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    a = be.sample_noalloc(16384, 3)
    b = be.sample_noalloc(1000, 4)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(a, be.sample(16384, 3)) and np.array_equal(b, be.sample(1000, 4))
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
