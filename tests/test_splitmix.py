"""CPU: the SplitMix64 restatement that checks the device uniform stream of
the sampled-expectation pipeline, pinned to the generator's published
known answer (seed 1234567)."""
import numpy as np

from helpers import splitmix64, splitmix_uniforms

# First five outputs of SplitMix64 from seed 1234567, as published with the
# generator's reference implementation.
KAT_SEED = 1234567
KAT = [6457827717110365317, 3203168211198807973, 9817491932198370423, 4593380528125082431,
       16408922859458223821]


def _scalar(seed, k):
    """Plain-integer restatement (one state update per output)."""
    m = (1 << 64) - 1
    x, out = seed, []
    for _ in range(k):
        x = (x + 0x9E3779B97F4A7C15) & m
        z = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        out.append(z ^ (z >> 31))
    return out


def test_splitmix_known_answer():
    assert [int(v) for v in splitmix64(KAT_SEED, 0, 5)] == KAT
    assert _scalar(KAT_SEED, 5) == KAT


def test_splitmix_offsets_and_wraparound():
    for seed in (0, 1, 2**63 + 5, 2**64 - 1):
        full = [int(v) for v in splitmix64(seed, 0, 40)]
        assert full == _scalar(seed, 40)
        assert [int(v) for v in splitmix64(seed, 17, 23)] == full[17:]


def test_uniforms_in_unit_interval():
    u = splitmix_uniforms(99, 100000)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    np.testing.assert_array_equal(splitmix_uniforms(KAT_SEED, 5), [(v >> 11) * 2.0 ** -53 for v in KAT])
