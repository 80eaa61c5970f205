"""The leapfrog's parity blocks, replayed on the CPU.

formoniq_gb300/csrc/fq_leapfrog.cu places the mass CSR of every grade of one
parity on the diagonal of one block CSR: row pointers shifted by the block's
entry offset, column indices by its row offset (lf_block_csr, one thread per
index up to max(nrows + 1, nnz)). This replays that kernel on random CSRs and
checks the block equals scipy's block_diag of the grades' matrices.

This checks the index scheme, written out again in Python, not the compiled
kernel; the GPU leapfrog tests against the oracle pin the kernel itself.
"""
import random

import numpy as np
import scipy.sparse as sp


def lf_block_csr(rp, ci, nrows, nnz, row_off, nnz_off, rp_out, ci_out):
    for i in range(max(nrows + 1, nnz)):
        if i <= nrows:
            rp_out[row_off + i] = rp[i] + nnz_off
        if i < nnz:
            ci_out[nnz_off + i] = ci[i] + row_off


def test_parity_block_is_the_block_diagonal():
    rng = random.Random(3)
    for _ in range(50):
        mats = []
        for _ in range(rng.randint(1, 3)):
            n = rng.randint(1, 30)
            m = sp.random(n, n, density=rng.uniform(0.05, 0.5), random_state=rng.randint(0, 10 ** 6), format="csr")
            m = (m + sp.eye(n)).tocsr()
            m.sort_indices()
            mats.append(m)
        rows = sum(m.shape[0] for m in mats)
        nnz = sum(m.nnz for m in mats)
        rp_out = np.full(rows + 1, -1, np.int64)
        ci_out = np.full(nnz, -1, np.int64)
        val = np.concatenate([m.data for m in mats])
        r0 = z0 = 0
        for m in mats:
            lf_block_csr(m.indptr, m.indices, m.shape[0], m.nnz, r0, z0, rp_out, ci_out)
            r0 += m.shape[0]
            z0 += m.nnz
        assert (rp_out >= 0).all() and (ci_out >= 0).all()
        got = sp.csr_matrix((val, ci_out, rp_out), shape=(rows, rows))
        want = sp.block_diag(mats, format="csr")
        assert abs(got - want).max() == 0
