"""Batched assembly against per-mesh assembly and the oracle."""
import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu


def meshes_of(ctx, specs):
    out = []
    for i, (dim, nb) in enumerate(specs):
        m = fq.Mesh.kuhn_cube(ctx, dim, nb)
        m.kuhn_lengths(jitter=0.1, seed=40 + i)
        out.append(m)
    return out


SPECS = [(2, 9), (3, 4), (4, 2), (2, 17), (3, 6), (4, 3), (3, 5), (2, 4)]
GRADES = [1, 2, 3, 0, 1, 2, 3, 2]


@pytest.mark.parametrize("form", [fq.FQ_BATCH_HDIF, fq.FQ_BATCH_MASS])
def test_batch_equals_per_mesh_assembly_bit_for_bit(ctx, form):
    meshes = meshes_of(ctx, SPECS)
    batch = fq.Batch(ctx, meshes, GRADES, form)
    batch.assemble()
    info = batch.info()
    assert info["classes"] == len({(d, k) for (d, _), k in zip(SPECS, GRADES)})
    for i, (m, k) in enumerate(zip(meshes, GRADES)):
        wc = fq.WhitneyComplex(m)
        single = (wc.hdif_gram(k) if form == fq.FQ_BATCH_HDIF else wc.mass(k)).to_scipy()
        got = batch.to_scipy(i)
        np.testing.assert_array_equal(got.indptr, single.indptr)
        np.testing.assert_array_equal(got.indices, single.indices)
        np.testing.assert_array_equal(got.data, single.data)
    # the per-mesh launches of the same kernels give the same values
    ref = [batch.to_scipy(i).data.copy() for i in range(len(meshes))]
    batch.assemble_per_mesh()
    for i in range(len(meshes)):
        np.testing.assert_array_equal(batch.to_scipy(i).data, ref[i])
    batch.close()
    for m in meshes:
        m.close()


def test_tuned_batch_stays_within_roundoff(ctx):
    meshes = meshes_of(ctx, SPECS)
    batch = fq.Batch(ctx, meshes, GRADES, fq.FQ_BATCH_HDIF)
    batch.assemble()
    ref = [batch.to_scipy(i) for i in range(len(meshes))]
    batch.tune(reps=2)
    batch.assemble()
    info = batch.info()
    assert info["scatter_threads_per_slot"] in (-1, 0, 1, 2, 4)
    for i in range(len(meshes)):
        a, b = batch.to_scipy(i), ref[i]
        assert np.abs(a.data - b.data).max() <= 1e-14 * np.abs(b.data).max()
    # every launch shape the tuner may pick
    for tps in (-1, 0, 1, 2, 4):
        for eg, sg in ((0, 0), (152, 304), (1216, 2432)):
            batch.set_launch(eg, tps, sg)
            batch.assemble()
            for i in range(len(meshes)):
                a, b = batch.to_scipy(i), ref[i]
                assert np.abs(a.data - b.data).max() <= 1e-14 * np.abs(b.data).max(), (tps, eg, sg)
    batch.close()
    for m in meshes:
        m.close()


def test_batch_matches_the_oracle(oracle, ctx):
    specs, grades = [(2, 5), (3, 3)], [1, 2]
    cxs, meshes = [], []
    for i, (dim, nb) in enumerate(specs):
        cx, coords = oracle.cartesian_unit(dim, nb)
        lengths = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, 70 + i, 0.1))
        m = fq.Mesh.kuhn_cube(ctx, dim, nb)
        m.set_lengths_sq(lengths)
        cxs.append((cx, lengths))
        meshes.append(m)
    batch = fq.Batch(ctx, meshes, grades, fq.FQ_BATCH_HDIF)
    batch.assemble()
    for i, ((cx, lengths), k) in enumerate(zip(cxs, grades)):
        want = oracle.WhitneyComplex(cx, lengths).hdif_gram(k).toarray()
        got = batch.to_scipy(i).toarray()
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    batch.close()
    for m in meshes:
        m.close()


def test_fused_element_launch_equals_per_class_launches(ctx):
    """One fused element launch over every (dimension, grade) class gives the
    per-class launches' values bit for bit (the same programs on the same
    cells); other forms are refused."""
    specs = SPECS + [(4, 2)]
    grades = GRADES + [4]
    meshes = meshes_of(ctx, specs)
    batch = fq.Batch(ctx, meshes, grades, fq.FQ_BATCH_HDIF)
    batch.assemble()
    ref = [batch.to_scipy(i).data.copy() for i in range(len(meshes))]
    assert batch.fused_registers() > 0
    for grid in (0, 2 * 152):
        batch.set_element_launch(True, grid)
        batch.assemble()
        for i in range(len(meshes)):
            np.testing.assert_array_equal(batch.to_scipy(i).data, ref[i])
    batch.set_element_launch(False)
    batch.close()
    mass = fq.Batch(ctx, meshes, grades, fq.FQ_BATCH_MASS)
    with pytest.raises(fq.FqError) as e:
        mass.set_element_launch(True)
    assert e.value.name == "FQ_UNSUPPORTED"
    mass.close()
    for m in meshes:
        m.close()
