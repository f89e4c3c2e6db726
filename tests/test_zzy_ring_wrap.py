"""The device parameter ring wrapping in the middle of a program.

Op tables are staged through a 32 MiB pinned-host -> device ring right
before the kernel that reads them; when the ring is full the stream is
synchronised and staging restarts at its front. A k = 6 unitary on an f64
state stages 64 KiB (split re / im), so 700 of them wrap the ring once while
the program runs; exact mode must stay bit-identical to the oracle.
"""

import numpy as np
import pytest

from helpers import bits_equal, rand_matrix, rand_state

pytestmark = pytest.mark.gpu


def test_parameter_ring_wraps_mid_program(zc, oracle):
    n = 8
    amps = rand_state(n, 5, normalize=True)
    g = zc.CudaBackend(n, 64, zc.FLAG_EXACT)
    g.load_state(amps)
    o = oracle.State(n, 64)
    o.load(amps)
    mats = [np.linalg.qr(rand_matrix(64, 1000 + i))[0] for i in range(8)]  # unitary: magnitudes stay bounded
    rng = np.random.default_rng(9)
    for i in range(700):
        qs = sorted(int(x) for x in rng.choice(n, 6, replace=False))
        g.apply_unitary(qs, mats[i % 8])
        o.apply_unitary(qs, mats[i % 8])
    a, b = g.statevector(), o.statevector()
    g.close()
    assert bits_equal(a, b), "max |d| = %g" % np.abs(a - b).max()
