"""Dynamic circuits (mid-circuit measure, reset, classically conditioned
ops) as batched trajectories: one launch for all shots, each shot a
trajectory with its own Philox stream and classical bits. Counts agree
with zeno's per-shot replay (src/exec.rs:459-619) in distribution; the
per-shot path itself (f64, or ZC_FLAG_PER_SHOT) stays bit-exact."""

import pytest

from helpers import program_from_json
from helpers_dynamic import dynamic_program

pytestmark = pytest.mark.gpu


def tvd(a, b):
    na, nb = sum(a.values()), sum(b.values())
    keys = set(a) | set(b)
    return 0.5 * sum(abs(a.get(k, 0) / na - b.get(k, 0) / nb) for k in keys)


def test_teleport_batched(zc, examples):
    p = program_from_json(examples["teleport"])
    r = zc.run(p, shots=20000, seed=3, precision=32)
    assert r.batched and sum(r.counts.values()) == 20000
    assert all(k.startswith("1 ") for k in r.counts), r.counts  # the teleported |1> always arrives
    assert len(r.counts) == 4 and min(r.counts.values()) > 4000


def test_dynamic_distribution_matches_per_shot_oracle(zc, oracle):
    p = dynamic_program(4, 3, 11)
    shots = 100000
    mine = zc.run(p, shots=shots, seed=5, precision=32)
    assert mine.batched and mine.launches <= 2
    ref = oracle.run(p, prec=64, shots=shots, seed=5)[0]
    assert tvd(mine.counts, ref) < 0.05, tvd(mine.counts, ref)


def test_dynamic_with_noise_matches_per_shot_oracle(zc, oracle):
    noise = zc.NoiseModel(depolarizing_1q=0.01, depolarizing_2q=0.03, amplitude_damping=0.02,
                          bit_flip=0.01, phase_flip=0.01, readout_flip_0to1=0.02, readout_flip_1to0=0.03)
    p = dynamic_program(4, 3, 12)
    shots = 100000
    mine = zc.run(p, shots=shots, seed=6, precision=32, noise=noise)
    assert mine.batched
    ref = oracle.run(p, prec=64, shots=shots, seed=6, noise=noise)[0]
    assert tvd(mine.counts, ref) < 0.05, tvd(mine.counts, ref)


def test_dynamic_batched_is_deterministic_and_per_shot_flag_is_exact(zc, oracle):
    p = dynamic_program(5, 4, 13)
    a = zc.run(p, shots=3000, seed=9, precision=32)
    b = zc.run(p, shots=3000, seed=9, precision=32)
    assert a.counts == b.counts
    r = zc.run(p, shots=300, seed=9, precision=32, flags=zc.FLAG_PER_SHOT)
    assert not r.batched
    assert r.counts == oracle.run(p, prec=32, shots=300, seed=9)[0]
