"""Every launch shape of the symmetric scatter (fq_ctx_set_scatter_shape) gives
the same values, bit for bit, as one thread per upper slot: each slot sums the
same contributions in the same order whatever the shape. Checked in the three
precision modes on 2D-4D forms, including slots with more than two
contributions (the diagonal ones) and a grid too small for one round."""
import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

SHAPES = [(-1, 0), (1, 0), (2, 0), (4, 0), (8, 0), (2, 1), (4, 2)]


@pytest.mark.parametrize("precision", [fq.FQ_FP64, fq.FQ_FP64_IEEE, fq.FQ_FP32])
@pytest.mark.parametrize("dim,nb,forms", [(2, 9, (("mass", 1), ("dif_both", 2))),
                                          (3, 7, (("mass", 1), ("mass", 2), ("dif_both", 2), ("dif_both", 3))),
                                          (4, 3, (("mass", 2), ("dif_both", 3)))])
def test_scatter_shapes_bit_identical(ctx, precision, dim, nb, forms):
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    wc = fq.WhitneyComplex(mesh, precision=precision)
    mesh.kuhn_lengths(jitter=0.1, seed=9)
    mats = [getattr(wc, name)(k) for name, k in forms]
    try:
        # the values of two different length sets, one thread per upper slot
        ctx.set_scatter_shape(0)
        want = {}
        for seed in (9, 10):
            mesh.kuhn_lengths(jitter=0.1, seed=seed)
            fq.Matrix.reassemble_many(mats)
            want[seed] = [m.host_arrays()[2].copy() for m in mats]
        for spt, bps in SHAPES:
            # the first length set with the reference shape, then the second with
            # the shape under test: a slot the shape skipped keeps a stale value
            ctx.set_scatter_shape(0)
            mesh.kuhn_lengths(jitter=0.1, seed=9)
            fq.Matrix.reassemble_many(mats)
            ctx.set_scatter_shape(spt, bps)
            mesh.kuhn_lengths(jitter=0.1, seed=10)
            fq.Matrix.reassemble_many(mats)
            for (name, k), m, w in zip(forms, mats, want[10]):
                got = m.host_arrays()[2]
                assert np.array_equal(got.view(np.uint8), w.view(np.uint8)), (spt, bps, name, k)
    finally:
        ctx.set_scatter_shape(-1)
        for m in mats:
            m.close()
        mesh.close()


def test_scatter_shape_rejects_unknown_shapes(ctx):
    with pytest.raises(fq.FqError):
        ctx.set_scatter_shape(3)
    with pytest.raises(fq.FqError):
        ctx.set_scatter_shape(2, 9)
    ctx.set_scatter_shape(-1)
