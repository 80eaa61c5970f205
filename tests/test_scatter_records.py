"""The symmetric scatter's 16-byte slot records, replayed on the CPU.

formoniq_gb300/csrc/fq_assembly.cu encodes, per upper slot u with contributions
up_perm[up_ptr[u] .. up_ptr[u+1]), a record (slot, mirror, p0, p1): p0 the first
contribution, p1 the second when there are exactly two, -1 when there is one,
-(2 + up_ptr[u] + 1) when there are more (the rest read from up_perm up to
up_ptr[u+1]). The scatter decodes it. This replays both and checks that every
slot sums exactly its contributions, in plan order.

This checks the encoding scheme, written out again in Python, not the compiled
kernel: a change to the kernel alone would still pass here. The GPU parity
tests (every assembled matrix against the oracle) pin the kernel itself.
"""
import random


def encode(up_ptr, up_perm, u):
    b, e = up_ptr[u], up_ptr[u + 1]
    p0 = up_perm[b] if e > b else -1
    p1 = up_perm[b + 1] if e - b == 2 else (-(2 + (b + 1)) if e - b > 2 else -1)
    return p0, p1


def decode(rec, up_ptr, up_perm, u, unroll=4):
    p0, p1 = rec
    seen = [p0] if p0 >= 0 else []
    if p1 >= 0:
        seen.append(p1)
    elif p1 < -1:
        e = up_ptr[u + 1]
        t = -(p1 + 2)
        while t < e:
            for k in range(unroll):
                if t + k < e:
                    seen.append(up_perm[t + k])
            t += unroll
    return seen


def test_records_visit_every_contribution_in_order():
    rng = random.Random(7)
    for _ in range(200):
        counts = [rng.choice([1, 1, 1, 2, 2, 3, 4, 5, 6, 9]) for _ in range(rng.randint(1, 60))]
        up_ptr = [0]
        for c in counts:
            up_ptr.append(up_ptr[-1] + c)
        up_perm = [rng.randrange(10 ** 6) for _ in range(up_ptr[-1])]
        for u in range(len(counts)):
            rec = encode(up_ptr, up_perm, u)
            assert decode(rec, up_ptr, up_perm, u) == up_perm[up_ptr[u]:up_ptr[u + 1]]


def multi_slot_rounds(nup, grid_threads, U):
    """The slots each thread of scatter_sym_multi_kernel handles, round by
    round, and the record loads it issues (current and prefetched): the
    kernel's index scheme, written out again in Python."""
    handled, loads = [], []
    T = grid_threads
    for tid in range(T):
        nxt = [tid + i * T for i in range(U)]
        loads += [u for u in nxt if u < nup]
        t0 = tid
        while t0 < nup:
            cur = nxt
            t1 = t0 + U * T
            if t1 < nup:
                nxt = [t1 + i * T for i in range(U)]
                loads += [u for u in nxt if u < nup]
            handled += [u for u in cur if u < nup]
            t0 = t1
    return handled, loads


def test_multi_slot_rounds_cover_every_slot_once():
    """Every upper slot is handled exactly once, every record load is in
    bounds, and no record is loaded twice, for U in 1, 2, 4, 8 over grids
    smaller and larger than one round."""
    rng = random.Random(7)
    for _ in range(300):
        U = rng.choice([1, 2, 4, 8])
        nup = rng.randint(0, 3000)
        T = 256 * rng.randint(1, 6)
        handled, loads = multi_slot_rounds(nup, T, U)
        assert sorted(handled) == list(range(nup))
        assert sorted(loads) == list(range(nup))
