"""The oracle's restatement of time::Leapfrog (formoniq/src/time.rs:292-420)
against the reference's own laws (CPU only): the grade-parity colouring makes
the mass block-diagonal and A block-antidiagonal, A = dif - delta is skew, the
staggered energy is conserved to roundoff under the CFL condition, and a step
is second-order consistent with the exact flow exp(dt M^-1 A)."""
import numpy as np
import pytest
import scipy.linalg as sla


def setup(oracle, dim, nb, relative, dt_scale=0.05):
    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, 2, 0.1)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords), relative=relative)
    return wc, oracle.leapfrog_for(wc, dt_scale / nb)


@pytest.mark.parametrize("relative", [False, True])
def test_colouring_and_skew_generator(oracle, relative):
    wc, (off, mb, lf) = setup(oracle, 3, 2, relative)
    _, _, a = oracle.dirac_signed(wc, -1.0)
    assert abs(a + a.T).max() == 0.0
    color = oracle.grade_parity_coloring(off)
    m = mb.tocoo()
    assert np.all(color[m.row] == color[m.col])
    c = a.tocoo()
    assert np.all(color[c.row] != color[c.col])


@pytest.mark.parametrize("relative", [False, True])
def test_staggered_energy_is_conserved(oracle, relative):
    wc, (off, mb, lf) = setup(oracle, 3, 2, relative)
    y = np.random.default_rng(1).standard_normal(int(off[-1]))
    e0 = lf.conserved_energy(y)
    for _ in range(200):
        y = lf.step(y)
    assert abs(lf.conserved_energy(y) - e0) <= 1e-12 * abs(e0)


def test_step_is_second_order(oracle):
    wc, (off, mb, lf0) = setup(oracle, 2, 2, True)
    _, _, a = oracle.dirac_signed(wc, -1.0)
    gen = np.linalg.solve(mb.toarray(), a.toarray())
    y0 = np.random.default_rng(3).standard_normal(int(off[-1]))
    errs = []
    for dt in (0.02, 0.01):
        lf = oracle.Leapfrog(mb, a, oracle.grade_parity_coloring(off), dt)
        errs.append(np.linalg.norm(lf.step(y0) - sla.expm(dt * gen) @ y0))
    # local error O(dt^3)
    assert errs[0] / errs[1] > 6.0, errs
