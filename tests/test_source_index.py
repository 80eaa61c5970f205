"""The staging index arithmetic of the source-load cell kernel, replayed on the CPU.

formoniq_gb300/csrc/fq_source.cuh stages the cell-major values [ncells][nq][cin]
of a block's cells through shared memory, a chunk of nodes at a time, with a
padded odd row stride; fq_source.cu picks chunk = max(1, min(nq, 47 // cin))
and stride = (chunk * cin) | 1 for 128-thread blocks. This replays the kernel's
loops (grid-stride over 128-cell blocks, the chunk loop, the cooperative copy
and each thread's reads) and checks every global read is inside the values
array, every shared-memory index inside 128 * stride doubles, and that each
thread reads exactly its own cell's values, each once, in node order.

This checks the index scheme, written out again in Python, not the compiled
kernel; the GPU source-load tests against the oracle pin the kernel itself.
"""
import random

import pytest

THREADS, STAGE = 128, 47


def replay(ncells, nq, cin, grid):
    chunk = max(1, min(nq, STAGE // cin))
    stride = (chunk * cin) | 1
    assert stride <= STAGE, (chunk, cin)
    per = nq * cin
    total = ncells * per
    reads = {}  # cell -> list of global indices read through its row
    base = 0
    for bx in range(grid):
        base = bx * THREADS
        while base < ncells:
            nb = min(THREADS, ncells - base)
            for q0 in range(0, nq, chunk):
                qn = min(chunk, nq - q0)
                run = qn * cin
                smem = {}
                for tid in range(THREADS):  # cooperative copy, stride blockDim
                    for i in range(tid, nb * run, THREADS):
                        c = i // run
                        sidx = c * stride + (i - c * run)
                        gidx = (base + c) * per + q0 * cin + (i - c * run)
                        assert 0 <= sidx < THREADS * stride
                        assert 0 <= gidx < total
                        assert sidx not in smem
                        smem[sidx] = gidx
                for tid in range(THREADS):
                    cell = base + tid
                    if cell >= ncells:
                        continue
                    for q in range(qn):
                        for c in range(cin):
                            sidx = tid * stride + q * cin + c
                            assert sidx in smem
                            reads.setdefault(cell, []).append(smem[sidx])
            base += grid * THREADS
    for cell in range(ncells):
        assert reads[cell] == list(range(cell * per, (cell + 1) * per)), cell


@pytest.mark.parametrize("nq,cin", [(1, 1), (5, 3), (6, 6), (21, 6), (56, 6), (66, 1), (15, 4), (4, 10)])
def test_staging_reads_each_value_once(nq, cin):
    rng = random.Random(nq * 100 + cin)
    for ncells in (1, 127, 128, 129, 300, rng.randint(1, 700)):
        for grid in (1, 2, 3):
            replay(ncells, nq, cin, grid)
