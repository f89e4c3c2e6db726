"""Dense k-qubit blocks on tensor cores (3xTF32, FP32 accumulation) for f32
states, against the FP64 oracle: max |d amp| and TVD at f32 level."""

import numpy as np
import pytest

from helpers import rand_matrix, rand_state
from zeno_gb300 import circuit as C

pytestmark = pytest.mark.gpu


def unitary(d, seed):
    return np.linalg.qr(rand_matrix(d, seed))[0]


@pytest.mark.parametrize("k", (3, 4, 5, 6, 7))
def test_tc_block_matches_fp64(zc, oracle, k):
    n = 14
    amps = rand_state(n, 30 + k, normalize=True)
    for si, qs in enumerate(([0, 2, 3, 5, 8, 9, 13][:k], list(range(n - k, n)), list(range(k)))):
        u = unitary(1 << k, 100 * k + si)
        g = zc.CudaBackend(n, 32, zc.FLAG_TENSOR | zc.FLAG_FAST)
        g.load_state(amps)
        g.apply_unitary(sorted(qs), u)
        o = oracle.State(n, 64)
        o.load(amps)
        o.apply_unitary(sorted(qs), u)
        want = o.statevector()
        got = g.statevector()
        assert np.abs(got - want).max() < 2e-6, (k, qs, np.abs(got - want).max())
        g.close()


def test_fused_circuit_on_tensor_cores(zc, oracle):
    """Gate-mix circuit fused to 7-qubit blocks, f32 state on tensor cores,
    against the FP64 oracle on the unfused circuit."""
    n = 18
    p = C.mixed_circuit(n, 20, 3).to_program()
    prog = zc.compile(p, 7)
    widths = [len(op.qubits) for op in prog.ops if op.kind == zc.OP_UNITARY]
    assert max(widths) == 7 and sum(w >= 3 for w in widths) > 10, widths
    r = zc.run(p, shots=0, precision=32, statevector=True, flags=zc.FLAG_TENSOR | zc.FLAG_FAST, program=prog)
    _, _, sv, _ = oracle.run(p, prec=64, shots=0, fusion=1, statevector=True)
    d = np.abs(r.statevector - sv).max()
    tvd = 0.5 * np.abs(np.abs(r.statevector) ** 2 - np.abs(sv) ** 2).sum()
    assert d < 1e-5 and tvd < 1e-5, (d, tvd)
