"""Index arithmetic of the whole-sector diagonal pass (k_diag1_blk in
afquantumsim_gb300/csrc/gate_kernels.cu), restated on the CPU: for a phase
pattern that fixes index bit 0 or 1 (complex64; bit 0 for complex128), the
kernel expands block u over the pattern's other fixed bits and changes the
elements j of the block with (j & lowmask) == lowval.  Every block must be
aligned and inside the register, and the changed elements must be exactly
the indices of the pattern, each once.  The kernels themselves are checked
against the oracle on the GPU (every gate at every placement)."""
import pytest


def expand(k, pos, val):
    for p in pos:
        lo = k & ((1 << p) - 1)
        k = ((k - lo) << 1) | lo
    return k | val


@pytest.mark.parametrize("blk", [4, 2])  # amplitudes per 32-byte sector: complex64, complex128
def test_blocks_cover_the_pattern_once(blk):
    low = blk - 1
    for n in range(1, 8):
        N = 1 << n
        if N < blk:
            continue
        for mask in range(1, N):
            if not mask & low:
                continue
            for val in range(N):
                if val & ~mask:
                    continue
                pos = [b for b in range(n) if (mask & ~low) >> b & 1]
                blocks = (N >> len(pos)) // blk
                got = []
                for u in range(blocks):
                    i = expand(u * blk, pos, val & ~low)
                    assert i % blk == 0 and i + blk <= N
                    got += [i + j for j in range(blk) if (j & mask & low) == (val & low)]
                assert len(got) == len(set(got))
                assert sorted(got) == [i for i in range(N) if (i & mask) == val]
