"""Cross-checks among the oracle families and against numpy (CPU only)."""
import numpy as np
import pytest

import afquantumsim_gb300 as aq
from oracle import oracle
from tests import _kat


@pytest.mark.parametrize("n,seed", [(3, 1), (4, 2), (5, 3), (6, 4), (7, 5)])
def test_reference_algorithm_matches_per_gate(n, seed):
    """The faithful restatement (dense Kronecker / CSR operators) and the
    per-gate oracles agree on random circuits over every gate kind."""
    ops = _kat.random_circuit(n, 40, seed)
    v = _kat.random_state(n, seed)
    ref = oracle.ref32_apply(v.astype(np.complex64), n, ops)
    f32 = oracle.apply_f32(v.astype(np.complex64), ops)
    f64 = oracle.apply_f64(v.copy(), ops)
    assert np.max(np.abs(ref - f64)) < 1e-5
    assert np.max(np.abs(f32 - f64)) < 1e-5


def _bitrev(x, n):
    idx = np.arange(1 << n)
    r = np.zeros_like(idx)
    for b in range(n):
        r |= ((idx >> b) & 1) << (n - 1 - b)
    return x[r]


@pytest.mark.parametrize("n", [2, 5, 8, 10])
def test_qft_is_inverse_dft_of_bit_reversed_input(n):
    """aqs::fourier_transform(n) (quantum_algo.cpp:103-114, no swaps) maps v
    to sqrt(N) * ifft(bitrev(v)); with the final swaps the output is
    bit-reversed as well.  Pins bit order and sign convention."""
    v = _kat.random_state(n, 11 + n)
    N = 1 << n
    out = oracle.apply_f64(v.copy(), aq.fourier_transform(n))
    want = np.fft.ifft(_bitrev(v, n)) * np.sqrt(N)
    assert np.max(np.abs(out - want)) < 1e-6  # float angles pi/2^k
    out_s = oracle.apply_f64(v.copy(), aq.fourier_transform(n, swaps=True))
    assert np.max(np.abs(out_s - _bitrev(want, n))) < 1e-6


def philox4x32_10(c, k0, k1):
    """Philox4x32-10 (Salmon et al., SC'11), the engine's device generator."""
    c = list(c)
    M = 0xFFFFFFFF
    for r in range(10):
        if r:
            k0, k1 = (k0 + 0x9E3779B9) & M, (k1 + 0xBB67AE85) & M
        p0, p1 = 0xD2511F53 * c[0], 0xCD9E8D57 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k0, p1 & M, (p0 >> 32) ^ c[3] ^ k1, p0 & M]
    return c


def philox_uniform(seed, shot):
    """The engine's uniform for (seed, shot): 53 bits of the first two words."""
    c = philox4x32_10([shot & 0xFFFFFFFF, shot >> 32, 0, 0], seed & 0xFFFFFFFF, seed >> 32)
    return (((c[0] >> 5) << 26) | (c[1] >> 6)) / 9007199254740992.0


def test_philox_known_answers():
    """Published Philox4x32-10 known-answer vectors (Random123 kat_vectors)."""
    assert philox4x32_10([0, 0, 0, 0], 0, 0) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox4x32_10([0xFFFFFFFF] * 4, 0xFFFFFFFF, 0xFFFFFFFF) == \
        [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], 0xA4093822, 0x299F31D0) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_profile_measure_semantics():
    """profile_measure_all's sort/countByKey histogram (quantum.cpp:467-501)
    equals a per-shot first-index draw; u above the total is 'unmatched'."""
    n = 5
    v = _kat.random_state(n, 7, np.complex64)
    u = np.random.default_rng(1).random(2000).astype(np.float32)
    counts, un = oracle.ref32_profile_measure_all(v, u)
    p = oracle.probs(v)
    want = np.zeros(1 << n, dtype=np.int64)
    for x in u:
        want[oracle.ref32_peek_measure_all(v, float(x))] += 1
    assert un == 0 and np.array_equal(counts, want)
