"""Bit-exact parity of every CUDA kernel with the oracle's scalar kernels.

The model is the reference's own `to_bits` sweep (src/state.rs:1385-1574):
random states, every target qubit and sorted support, n = 1..12, both
precisions. In exact mode the GPU must reproduce the oracle's state bit for
bit; prob_one / norm_sqr / sampled indices follow the same f64 summation
order and must match exactly too.
"""

import numpy as np
import pytest

from helpers import as_precision, bits_equal, rand_matrix, rand_state, supports

pytestmark = pytest.mark.gpu

PRECS = (64, 32)


def pair(zc, oracle, n, prec, amps):
    g = zc.CudaBackend(n, prec)
    g.load_state(amps)
    o = oracle.State(n, prec)
    o.load(amps)
    return g, o


def same(g, o, ctx=""):
    a, b = g.statevector(), o.statevector()
    assert bits_equal(a, b), "%s: max |d| = %g" % (ctx, np.abs(a - b).max())


@pytest.mark.parametrize("prec", PRECS)
def test_1q_every_qubit(zc, oracle, prec):
    for n in range(1, 13):
        amps = rand_state(n, 100 + n)
        for q in range(n):
            m = rand_matrix(2, 1000 * n + q)
            g, o = pair(zc, oracle, n, prec, amps)
            g.apply_unitary([q], m)
            o.apply_unitary([q], m)
            same(g, o, "1q n=%d q=%d f%d" % (n, q, prec))
            g.close()


@pytest.mark.parametrize("prec", PRECS)
def test_diag_every_support(zc, oracle, prec):
    for n in range(1, 11):
        amps = rand_state(n, 200 + n)
        for k in range(1, min(n, 6) + 1):
            d = rand_state(k, 50 * n + k)
            sups = supports(n, k)
            for si, qs in enumerate(sups):
                if n > 8 and si % 7:
                    continue
                g, o = pair(zc, oracle, n, prec, amps)
                g.apply_diagonal(qs, d)
                o.apply_diagonal(qs, d)
                same(g, o, "diag n=%d qs=%s f%d" % (n, qs, prec))
                g.close()


@pytest.mark.parametrize("prec", PRECS)
def test_wide_diagonal(zc, oracle, prec):
    n = 14
    amps = rand_state(n, 7)
    for qs in ([0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11], [2, 3, 5, 7, 8, 9, 10, 11, 12, 13], [13]):
        d = rand_state(len(qs), len(qs))
        g, o = pair(zc, oracle, n, prec, amps)
        g.apply_diagonal(qs, d)
        o.apply_diagonal(qs, d)
        same(g, o, "wide diag %s" % qs)
        g.close()


@pytest.mark.parametrize("prec", PRECS)
def test_kq_supports(zc, oracle, prec):
    for n in range(2, 13):
        amps = rand_state(n, 300 + n)
        for k in range(2, min(n, 7) + 1):
            m = rand_matrix(1 << k, 77 * n + k)
            sups = supports(n, k)
            pick = [s for i, s in enumerate(sups) if i % max(1, len(sups) // 6) == 0 or i == len(sups) - 1]
            for qs in pick:
                g, o = pair(zc, oracle, n, prec, amps)
                g.apply_unitary(qs, m)
                o.apply_unitary(qs, m)
                same(g, o, "kq n=%d qs=%s f%d" % (n, qs, prec))
                g.close()


@pytest.mark.parametrize("prec", PRECS)
def test_cx_and_swap_every_pair(zc, oracle, prec):
    swap = np.zeros((4, 4), complex)
    for c in range(4):
        swap[((c & 1) << 1) | ((c >> 1) & 1), c] = 1
    for n in (2, 3, 5, 9):
        amps = rand_state(n, 400 + n)
        for a in range(n):
            for b in range(n):
                if a == b:
                    continue
                g, o = pair(zc, oracle, n, prec, amps)
                g.apply_cx(a, b)
                o.apply_cx(a, b)
                same(g, o, "cx %d %d" % (a, b))
                if a < b:
                    g.apply_swap(a, b)
                    o.apply_unitary([a, b], swap)
                    same(g, o, "swap %d %d" % (a, b))
                g.close()


@pytest.mark.parametrize("prec", PRECS)
def test_reductions_and_measure(zc, oracle, prec):
    for n in (1, 3, 8, 16, 18):
        amps = rand_state(n, 500 + n, normalize=True)
        g, o = pair(zc, oracle, n, prec, amps)
        assert g.norm_sqr() == o.norm_sqr()
        for q in sorted({0, n // 2, n - 1}):
            assert g.prob_one(q) == o.prob_one(q), (n, q)
        for q, u in ((n - 1, 0.3), (0, 0.7)):
            assert g.measure(q, u) == o.measure(q, u)
            same(g, o, "collapse n=%d q=%d" % (n, q))
        g.reset_all()
        o.reset_all()
        same(g, o, "reset")
        g.close()


@pytest.mark.parametrize("prec", PRECS)
def test_sampler_bit_exact(zc, oracle, prec):
    for n, shots, seed in ((1, 100, 1), (4, 1000, 2), (12, 4096, 3), (17, 8192, 4), (20, 50000, 5)):
        amps = rand_state(n, 600 + n, normalize=True)
        g, o = pair(zc, oracle, n, prec, amps)
        a, b = g.sample(shots, seed), o.sample(shots, seed)
        assert np.array_equal(a, b), (n, shots)
        assert np.all(np.diff(a.astype(np.int64)) >= 0)
        g.close()


def test_sampler_sparse_state(zc, oracle):
    """Zero-probability chunks and the unresolved-draw fallback paths."""
    n = 18
    amps = np.zeros(1 << n, complex)
    amps[5] = 0.6
    amps[(1 << 17) + 3] = 0.8j
    for prec in PRECS:
        g, o = pair(zc, oracle, n, prec, amps)
        a, b = g.sample(10000, 9), o.sample(10000, 9)
        assert np.array_equal(a, b)
        assert set(np.unique(a)) <= {5, (1 << 17) + 3}
        g.close()


def test_fast_mode_tolerance(zc, oracle):
    """FMA-contracted arithmetic stays within 1e-12 (f64) / 1e-5 (f32)."""
    n = 12
    amps = rand_state(n, 9, normalize=True)
    for prec, tol in ((64, 1e-12), (32, 1e-5)):
        g = zc.CudaBackend(n, prec, zc.FLAG_FAST)
        g.load_state(amps)
        o = oracle.State(n, prec)
        o.load(amps)
        for q in range(n):
            m = np.linalg.qr(rand_matrix(2, q))[0]
            g.apply_unitary([q], m)
            o.apply_unitary([q], m)
        m = np.linalg.qr(rand_matrix(16, 3))[0]
        g.apply_unitary([1, 4, 7, 9], m)
        o.apply_unitary([1, 4, 7, 9], m)
        assert np.abs(g.statevector() - o.statevector()).max() < tol
        g.close()


def test_invalid_arguments(zc):
    g = zc.CudaBackend(4, 64)
    with pytest.raises(zc.ZenoCudaError):
        g.apply_unitary([4], np.eye(2))
    with pytest.raises(zc.ZenoCudaError):
        g.apply_unitary([2, 1], np.eye(4))
    with pytest.raises(zc.ZenoCudaError):
        g.apply_cx(1, 1)
    with pytest.raises(zc.ZenoCudaError):
        g.apply_diagonal([0, 1, 2, 3, 4], np.ones(32))
    g.close()


def test_capacity_refusal(zc):
    """A state beyond the HBM budget is refused with mem::plan's message."""
    with pytest.raises(zc.ZenoCudaError) as e:
        zc.CudaBackend(40, 64)
    assert e.value.code == zc.ZC_ERR_MEMORY and "max 33 qubits" in str(e.value)


def test_device_info_report(zc):
    from zeno_gb300 import info

    r = info.report()
    assert r["sms"] >= 100 and r["hbm_bytes"] > 100e9 and r["l2_bytes"] > 50e6
    assert r["budget_bytes"] == int(r["hbm_bytes"] * 0.75) or "ZENO_MEM_BYTES" in __import__("os").environ
    f64 = r["precisions"]["f64"]
    assert f64["state_bytes"] <= r["budget_bytes"] < f64["next_qubit_bytes"]
