"""The index arithmetic of the batched scatter launches, replayed on the CPU.

formoniq_gb300/csrc/fq_batch.cu pads each mesh's slot range to a multiple of 32
in the batch index space; every launch shape (tps = 1, 2, 4 threads per slot,
or warp-staged) must skip the padding, keep every slot_ptr / perm / value
access inside its mesh and write every real slot exactly once. This replays the
kernels' index computations (grid-stride loops, binary search over the
entries, the padding test) for random batches and grid sizes.

This checks the index scheme, written out again in Python, not the compiled
kernels; the GPU batch tests (every member against fq_assemble and the oracle)
pin the kernels themselves.
"""
import random

import pytest

def entries(rng):
    ents, begin = [], 0
    for _ in range(rng.randint(1, 9)):
        n = rng.choice([0, 1, 5, 31, 32, 33, 64, 100, rng.randint(0, 300)])
        ents.append((begin, n)); begin += (n + 31) & ~31
    return ents, begin

def find(ents, g):
    lo, hi = 0, len(ents) - 1
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if ents[mid][0] <= g: lo = mid
        else: hi = mid - 1
    return lo

def tps_kernel(ents, total, tps, blocks, threads=256):
    writes = {}
    gpg = blocks * (threads // tps)
    for bx in range(blocks):
        base = bx * (threads // tps)
        while base < total:
            for tx in range(threads):
                g = base + tx // tps; lane = tx % tps
                valid = g < total
                if not valid: continue
                lo = find(ents, g); b, n = ents[lo]
                assert b <= g
                live = g - b < n
                if live:
                    s = g - b
                    assert 0 <= s and s + 1 <= n   # slot_ptr[s], slot_ptr[s+1] within n+1 entries
                    if lane == 0:
                        writes[(lo, s)] = writes.get((lo, s), 0) + 1
            base += gpg
    return writes

def warp_kernel(ents, total, blocks, threads=256):
    writes = {}
    wpg = blocks * 8
    for bx in range(blocks):
        for warp in range(8):
            w = bx * 8 + warp
            while w * 32 < total:
                g0 = w * 32
                lo = find(ents, g0); b, n = ents[lo]
                s0 = g0 - b
                if s0 < n:
                    slast = min(s0 + 32, n)
                    assert slast <= n
                    for lane in range(32):
                        s = s0 + lane
                        if s < n:
                            assert s + 1 <= n
                            writes[(lo, s)] = writes.get((lo, s), 0) + 1
                w += wpg
    return writes



@pytest.mark.parametrize("seed", range(6))
def test_batch_scatter_index_arithmetic(seed):
    rng = random.Random(seed)
    for _ in range(50):
        ents, total = entries(rng)
        want = {(i, s): 1 for i, (_, n) in enumerate(ents) for s in range(n)}
        for tps in (1, 2, 4):
            need = (total * tps + 255) // 256
            for grid in (0, 1, 3):
                blocks = need if grid == 0 else min(grid, need)
                if blocks:
                    assert tps_kernel(ents, total, tps, blocks) == want, (ents, tps, grid)
        need = (total + 255) // 256
        for grid in (0, 1, 2):
            blocks = need if grid == 0 else min(grid, need)
            if blocks:
                assert warp_kernel(ents, total, blocks) == want, (ents, grid)
