"""The source load on the GPU (fq_source_nodes / fq_source_assemble) against
the oracle's restatement of SourceForm::element (formoniq/src/operators.rs:598-635)
and assemble_vector (galerkin.rs:279-312), and the reference's law that the
load of a Whitney form is a mass column (galerkin.rs:334-371)."""
import math

import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def setup(oracle, ctx, dim, nb, seed=5):
    import torch

    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, seed, 0.1)
    lengths = cx.edge_lengths_sq(coords)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(lengths)
    return cx, coords, lengths, mesh, torch.tensor(coords, device="cuda")


@pytest.mark.parametrize("dim,nb", [(1, 9), (2, 5), (3, 3), (4, 2)])
def test_reference_frame_values_match_oracle(oracle, ctx, dim, nb):
    import torch

    cx, coords, lengths, mesh, _ = setup(oracle, ctx, dim, nb)
    rng = np.random.default_rng(dim)
    for k in range(dim + 1):
        for degree in (1, 3):
            nq = len(oracle.gm_rule(dim, degree)[1])
            vals = rng.standard_normal((cx.ncells(), nq, math.comb(dim, k)))
            dvals = torch.tensor(vals, device="cuda")
            for bc in (fq.FQ_ABSOLUTE, fq.FQ_RELATIVE):
                want = oracle.source_form(cx, lengths, k, vals, degree, relative=bc == fq.FQ_RELATIVE)
                got = fq.source_form(mesh, k, dvals, degree, bc=bc).cpu().numpy()
                assert got.shape == want.shape
                assert rel(got, want) < TOL, (k, degree, bc)


@pytest.mark.parametrize("dim,nb", [(2, 5), (3, 3), (4, 2)])
def test_flat_ambient_form_matches_oracle(oracle, ctx, dim, nb):
    """A polynomial ambient form, evaluated by the caller at the device's nodes
    and pulled back cell by cell (Pullback::identity)."""
    import torch

    cx, coords, lengths, mesh, dcoords = setup(oracle, ctx, dim, nb)
    bary, _ = oracle.gm_rule(dim, 3)
    nodes_o = np.einsum("qv,cva->cqa", bary, coords[cx.simplices(dim)])
    nodes = fq.source_nodes(mesh, 3, dcoords)
    assert np.abs(nodes.cpu().numpy() - nodes_o).max() < 1e-15
    assert np.abs(fq.source_nodes(mesh, 3).cpu().numpy() - bary).max() == 0.0
    for k in range(dim + 1):
        ncomp = math.comb(dim, k)

        def field(x, xp):
            return xp.stack([1.0 + (c + 1) * x[..., c % dim] * x[..., (c + 1) % dim] - 0.5 * x[..., 0] ** 2
                             for c in range(ncomp)], -1)

        want = oracle.source_form(cx, lengths, k, field(nodes_o, np), 3, coords=coords)
        got = fq.source_form(mesh, k, lambda x: field(x, torch), 3, coords=dcoords).cpu().numpy()
        assert rel(got, want) < TOL, k


def test_embedded_surface_pullback(oracle, ctx):
    """A 2D mesh embedded in 3D (adim > n): the pulled-back ambient 1- and
    2-forms against the oracle."""
    import torch

    nb = 4
    cx, c2 = oracle.cartesian_unit(2, nb)
    c2 = oracle.jitter_coords(c2, nb, 7, 0.1)
    coords = np.concatenate([c2, (0.3 * c2[:, 0] ** 2 - 0.2 * c2[:, 1])[:, None]], 1)
    lengths = cx.edge_lengths_sq(coords)
    mesh = fq.Mesh.kuhn_cube(ctx, 2, nb)
    mesh.set_lengths_sq(lengths)
    dcoords = torch.tensor(coords, device="cuda")
    rng = np.random.default_rng(3)
    for k in (0, 1, 2):
        nq = len(oracle.gm_rule(2, 2)[1])
        vals = rng.standard_normal((cx.ncells(), nq, math.comb(3, k)))
        want = oracle.source_form(cx, lengths, k, vals, 2, coords=coords)
        got = fq.source_form(mesh, k, torch.tensor(vals, device="cuda"), 2, coords=dcoords).cpu().numpy()
        assert rel(got, want) < TOL, k


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_load_of_a_whitney_form_is_a_mass_column(oracle, ctx, dim):
    import torch

    cx, coords = oracle.cartesian_unit(dim, 2)
    lengths = cx.edge_lengths_sq(coords)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, 2)
    mesh.set_lengths_sq(lengths)
    gwc = fq.WhitneyComplex(mesh)
    bary = fq.source_nodes(mesh, 4).cpu().numpy()
    for k in range(dim + 1):
        nd = cx.nsimplices(k)
        basis = np.zeros(nd)
        basis[nd // 2] = 1.0
        vals = torch.tensor(oracle.whitney_interpolant_values(cx, k, basis, bary), device="cuda")
        load = fq.source_form(mesh, k, vals, 4).cpu().numpy()
        col = gwc.mass(k).to_scipy() @ basis
        assert rel(load, col) < TOL, k


@pytest.mark.parametrize("dim,nb,k,degree", [(4, 2, 2, 7), (1, 12, 1, 21), (3, 2, 1, 9)])
def test_high_degree_rules_stage_in_chunks(oracle, ctx, dim, nb, k, degree):
    """Rules with more nodes than one shared-memory chunk holds."""
    import torch

    cx, coords, lengths, mesh, _ = setup(oracle, ctx, dim, nb)
    nq = len(oracle.gm_rule(dim, degree)[1])
    assert nq == ctx.L.fq_source_npoints(dim, degree)
    vals = np.random.default_rng(9).standard_normal((cx.ncells(), nq, math.comb(dim, k)))
    want = oracle.source_form(cx, lengths, k, vals, degree)
    got = fq.source_form(mesh, k, torch.tensor(vals, device="cuda"), degree).cpu().numpy()
    assert rel(got, want) < TOL


def test_argument_and_cell_errors(oracle, ctx):
    import torch

    cx, coords, lengths, mesh, dcoords = setup(oracle, ctx, 2, 3)
    nq = ctx.L.fq_source_npoints(2, 1)
    vals = torch.zeros((cx.ncells(), nq, 2), dtype=torch.float64, device="cuda")
    with pytest.raises(fq.FqError):
        fq.source_form(mesh, 3, vals, 1)  # grade above the dimension
    with pytest.raises(fq.FqError):
        fq.source_form(mesh, 1, vals, 22)  # no rule of that degree
    with pytest.raises(fq.FqError):
        fq.source_form(mesh, 1, vals[:, :, :1], 1)  # wrong component count
    flat = fq.Mesh.kuhn_cube(ctx, 2, 3)
    flat.set_lengths_sq(np.zeros(cx.nsimplices(1)))  # every cell collapsed to a point
    with pytest.raises(fq.FqError) as e:
        fq.source_form(flat, 1, vals, 1)
    assert e.value.name == "FQ_DEGENERATE_CELL"
