"""The device leapfrog (fq_leapfrog_*) against the oracle's time::Leapfrog
(exact block solves): the same trajectory, and the staggered energy conserved
(formoniq/src/time.rs:401-420), on the full (natural) and relative (PEC)
complexes."""
import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,nb", [(2, 6), (3, 3)])
@pytest.mark.parametrize("relative", [False, True])
def test_leapfrog_matches_oracle(oracle, ctx, dim, nb, relative):
    import torch

    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, 2, 0.1)
    lengths = cx.edge_lengths_sq(coords)
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(dim, nb))
    mesh.set_lengths_sq(lengths)
    dt = 0.05 / nb
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    off, mb, olf = oracle.leapfrog_for(owc, dt)
    lf = fq.Leapfrog(mesh, fq.FQ_RELATIVE if relative else fq.FQ_ABSOLUTE, dt)
    np.testing.assert_array_equal(lf.offsets(), off)
    y0 = np.random.default_rng(7).standard_normal(int(off[-1]))
    yd = torch.tensor(y0, device="cuda")
    yo = y0.copy()
    for _ in range(10):
        yo = olf.step(yo)
    lf.step(yd, 10)
    got = yd.cpu().numpy()
    assert np.linalg.norm(got - yo) <= 1e-10 * np.linalg.norm(yo)
    e_o = olf.conserved_energy(yo)
    e, c = lf.energy(yd)
    assert abs(c - e_o) <= 1e-10 * abs(e_o)
    assert abs(e - 0.5 * yo @ (mb @ yo)) <= 1e-10 * abs(e)


def test_leapfrog_conserves_the_staggered_energy(oracle, ctx):
    import torch

    dim, nb = 3, 4
    cx, coords = oracle.cartesian_unit(dim, nb)
    lengths = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, 3, 0.1))
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(dim, nb))
    mesh.set_lengths_sq(lengths)
    lf = fq.Leapfrog(mesh, fq.FQ_RELATIVE, 0.05 / nb)
    n = int(lf.offsets()[-1])
    y = torch.tensor(np.random.default_rng(9).standard_normal(n), device="cuda")
    _, c0 = lf.energy(y)
    lf.step(y, 100)
    _, c1 = lf.energy(y)
    assert abs(c1 - c0) <= 1e-10 * abs(c0), (c0, c1)
