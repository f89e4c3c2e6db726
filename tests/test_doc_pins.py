"""Counts pinned to the seeded runs printed in zeno's own documentation.

These outputs come from the Rust binary (`zeno run ... --seed S` and
`zeno demo`): they fix the whole random path end to end — rand_xoshiro 0.6
`seed_from_u64`, the executor's `splitmix64(seed)` (src/exec.rs:436), rand
0.8's `gen::<f64>` and the sampler's draw/sort/route order
(src/sample.rs:29-111) — which the oracle and the library restate from the
crates' published algorithms.

  * README.md:112-123 and docs/TUTORIAL.md:161-171: bell, 1000 shots, seed 42
  * docs/TUTORIAL.md:182-192: the same with `h` on q[1]
  * docs/TUTORIAL.md:214-226: ghz3, 1000 shots, seed 42
  * docs/TUTORIAL.md:235-245: bell, default 1024 shots, seed 42
    (`--statevector`; the sampled counts are printed beside the amplitudes)
  * docs/TUTORIAL.md:257-268: bell, 10 shots, seed 42 (5/5) and seed 45
    (an 8/2 split; the page does not say which key gets 8, so only the
    split is pinned)
  * docs/TUTORIAL.md:53-80 and :104: `zeno demo` (bell, 1000 shots by default,
    src/main.rs:114-116) at seed 0x701a0d019f1a425e

The CPU tests pin the oracle; the GPU tests pin the CUDA backend's exact
path twice: through the host pipeline (`zc_run`) and through the trait-level
entry points the Rust shim binds (apply ops, then `zc_sample(shots,
splitmix64(seed))`, as run_sampled does).
"""

import pytest

from zeno_gb300 import circuit as C
from zeno_gb300.rng import splitmix64


def _bell(hq=0):
    c = C.Circuit(2)
    c.h(hq)
    c.cx(0, 1)
    c.measure_all()
    return c.to_program()


def _ghz3():
    c = C.Circuit(3)
    c.h(0)
    c.cx(0, 1)
    c.cx(1, 2)
    c.measure_all()
    return c.to_program()


# (name, program, shots, seed, expected counts or None for the 8/2 split)
CASES = [
    ("bell_seed42", _bell, 1000, 42, {"00": 502, "11": 498}),
    ("bell_h_on_q1", lambda: _bell(1), 1000, 42, {"00": 502, "10": 498}),
    ("ghz3_seed42", _ghz3, 1000, 42, {"000": 502, "111": 498}),
    ("bell_1024_seed42", _bell, 1024, 42, {"00": 517, "11": 507}),
    ("bell_10_seed42", _bell, 10, 42, {"00": 5, "11": 5}),
    ("bell_10_seed45", _bell, 10, 45, None),
    ("demo_bell", _bell, 1000, 0x701A0D019F1A425E, {"00": 507, "11": 493}),
]


def _check(name, counts, want):
    if want is None:
        assert sorted(counts.values()) == [2, 8] and set(counts) <= {"00", "11"}, (name, counts)
    else:
        assert counts == want, (name, counts)


@pytest.mark.parametrize("name,make,shots,seed,want", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("fusion", (0, 1))
def test_oracle_matches_documented_runs(oracle, name, make, shots, seed, want, fusion):
    counts, _, _, _ = oracle.run(make(), prec=64, shots=shots, seed=seed, fusion=fusion)
    _check(name, counts, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,shots,seed,want", CASES, ids=[c[0] for c in CASES])
def test_cuda_run_matches_documented_runs(zc, name, make, shots, seed, want):
    """zc_run, exact f64 (the drop-in's default arithmetic)."""
    r = zc.run(make(), shots=shots, seed=seed, precision=64, flags=zc.FLAG_EXACT)
    assert r.backend == "cuda-f64"
    _check(name, r.counts, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,shots,seed,want", CASES, ids=[c[0] for c in CASES])
def test_cuda_trait_sample_matches_documented_runs(zc, name, make, shots, seed, want):
    """The trait-level path: apply the compiled ops one by one, then
    `zc_sample(shots, splitmix64(seed))` and the histogram of run_sampled
    (src/exec.rs:436-447; every qubit is measured into its own clbit)."""
    p = make()
    prog = zc.compile(p, 1)
    be = zc.CudaBackend(p.n_qubits, 64, zc.FLAG_EXACT)
    try:
        for op in prog.ops:
            if op.kind == zc.OP_UNITARY:
                be.apply_unitary(op.qubits, op.data)
            elif op.kind == zc.OP_DIAG:
                be.apply_diagonal(op.qubits, op.data)
            elif op.kind == zc.OP_CX:
                be.apply_cx(op.a, op.b)
            elif op.kind == zc.OP_SWAP:
                be.apply_swap(op.a, op.b)
        idx = be.sample(shots, splitmix64(seed))
    finally:
        be.close()
    counts = {}
    for i in idx:
        key = C.format_key(int(i), p.cregs)
        counts[key] = counts.get(key, 0) + 1
    _check(name, counts, want)
