"""The serving loop: results alone and in the mix, against direct solves,
admission by HBM budget and resident meshes."""
import math

import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

# A request's result is the same alone and in the mix: the kernels are
# deterministic, so the stated tolerance is exact equality.
MIX_TOL = 0.0
SOLVE_TOL = 1e-8


def small_requests():
    reqs = []
    seed = 100
    for dim, nb in ((2, 6), (3, 3), (4, 2)):
        for k in range(dim + 1):
            for bc in (fq.FQ_ABSOLUTE, fq.FQ_RELATIVE):
                reqs.append(dict(kind=fq.FQ_REQ_HODGE, dim=dim, nbox=nb, grade=k, bc=bc, jitter=0.1, seed=seed))
                seed += 1
    # Lorentzian Dirac: sizes where MINRES converges (the source problem on the
    # spacetime box is near-resonant and MINRES stalls on larger boxes)
    for nb in (2, 3):
        reqs.append(dict(kind=fq.FQ_REQ_DIRAC, dim=3, nbox=nb, minkowski=True, jitter=0.05, seed=seed,
                         mass_term=1.5))
        seed += 1
    return reqs


def ndofs(req):
    from oracle import cartesian_unit

    cx, _ = cartesian_unit(req["dim"], req["nbox"])
    if req["kind"] == fq.FQ_REQ_DIRAC:
        return sum(cx.nsimplices(j) for j in range(req["dim"] + 1))
    k = req["grade"]
    return (cx.nsimplices(k - 1) if k >= 1 else 0) + cx.nsimplices(k)


def run_all(server, reqs, opts, concurrent):
    sols, res = [], []
    if concurrent:
        tickets = []
        for r in reqs:
            sol = np.zeros(ndofs(r))
            sols.append(sol)
            tickets.append(server.submit(**r, solution=sol, opts=opts))
        res = [server.wait(t) for t in tickets]
    else:
        for r in reqs:
            sol = np.zeros(ndofs(r))
            sols.append(sol)
            res.append(server.wait(server.submit(**r, solution=sol, opts=opts)))
    return sols, res


def test_results_are_the_same_alone_and_in_the_mix(oracle):
    reqs = small_requests()
    opts = fq.SolveOpts.default(rtol=1e-10)
    with fq.Server(lanes=1, cache=False) as alone:
        sa, ra = run_all(alone, reqs, opts, concurrent=False)
    with fq.Server(lanes=4, cache=True) as mix:
        # twice: the second pass runs on resident meshes
        sm, rm = run_all(mix, reqs + reqs, opts, concurrent=True)
        st = mix.stats()
    assert st["completed"] == 2 * len(reqs) and st["cache_hits"] >= len(reqs)
    assert len({r["lane"] for r in rm}) > 1
    for i, r in enumerate(reqs):
        assert ra[i]["status"] == 0 and rm[i]["status"] == 0, (r, ra[i], rm[i])
        for sol in (sm[i], sm[i + len(reqs)]):
            err = np.abs(sol - sa[i]).max() / max(np.abs(sa[i]).max(), 1e-300)
            assert err <= MIX_TOL, (r, err)


def test_overlap_happens_across_lanes(oracle):
    reqs = [dict(kind=fq.FQ_REQ_HODGE, dim=3, nbox=10, grade=1, bc=fq.FQ_ABSOLUTE, jitter=0.1, seed=s)
            for s in range(8)]
    with fq.Server(lanes=4, cache=True) as srv:
        ts = [srv.submit(**r) for r in reqs]
        res = [srv.wait(t) for t in ts]
    spans = sorted((r["start_ms"], r["end_ms"]) for r in res)
    overlaps = sum(1 for a, b in zip(spans, spans[1:]) if b[0] < a[1])
    assert overlaps >= 1, spans
    assert all(r["status"] == 0 and r["report"].converged for r in res)


def test_budget_admits_one_at_a_time_when_tight(oracle):
    reqs = [dict(kind=fq.FQ_REQ_HODGE, dim=3, nbox=6, grade=1, bc=fq.FQ_ABSOLUTE, jitter=0.1, seed=s)
            for s in range(5)]
    # budget below two requests' estimates: no two may run together
    with fq.Server(lanes=4, cache=False, budget_bytes=60 << 20) as srv:
        ts = [srv.submit(**r) for r in reqs]
        res = [srv.wait(t) for t in ts]
    spans = sorted((r["start_ms"], r["end_ms"]) for r in res)
    for a, b in zip(spans, spans[1:]):
        assert b[0] >= a[1], spans
    assert all(r["status"] == 0 for r in res)


def test_served_hodge_matches_the_direct_solve(oracle):
    dim, nb, k = 2, 6, 1
    cx, coords = oracle.cartesian_unit(dim, nb)
    lengths = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, 9, 0.1))
    src = np.random.default_rng(4).standard_normal(cx.nsimplices(k))
    owc = oracle.WhitneyComplex(cx, lengths)
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, k, oracle.harmonics(owc, k))
    x = oracle.direct_solve(a, rhs)
    sol = np.zeros(ns + nu)
    with fq.Server(lanes=2) as srv:
        for prec in (fq.FQ_FP64, fq.FQ_FP32):
            opts = fq.SolveOpts.default(rtol=1e-10 if prec == fq.FQ_FP64 else 1e-5, precision=prec,
                                        refine_rtol=1e-11)
            r = srv.wait(srv.submit(fq.FQ_REQ_HODGE, dim, nb, grade=k, lengths=lengths, source=src, solution=sol,
                                    opts=opts))
            assert r["status"] == 0, r
            assert np.linalg.norm(sol - x[:ns + nu]) / np.linalg.norm(x) < SOLVE_TOL, prec


def test_served_dirac_matches_the_direct_solve(oracle):
    dim, nb = 3, 3
    cx, coords, signs = oracle.minkowski(dim, nb)
    lengths = cx.edge_lengths_sq(coords, signs)
    lengths = lengths * (1.0 + 0.05 * oracle.uniform_pm1(8, np.arange(len(lengths), dtype=np.uint64)))
    nfull = sum(cx.nsimplices(j) for j in range(dim + 1))
    load = np.random.default_rng(6).standard_normal(nfull)
    x_ref = oracle.dirac_solve_source(cx, lengths, 1.5, load, np.zeros(nfull))
    sol = np.zeros(nfull)
    with fq.Server(lanes=2) as srv:
        r = srv.wait(srv.submit(fq.FQ_REQ_DIRAC, dim, nb, minkowski=True, lengths=lengths, source=load,
                                solution=sol, mass_term=1.5, opts=fq.SolveOpts.default(rtol=1e-12)))
    assert r["status"] == 0, r
    assert np.linalg.norm(sol - x_ref) / np.linalg.norm(x_ref) < SOLVE_TOL


def test_a_failing_request_does_not_stop_the_server(oracle):
    with fq.Server(lanes=2) as srv:
        bad = srv.submit(fq.FQ_REQ_HODGE, 2, 4, grade=5)
        good = srv.submit(fq.FQ_REQ_HODGE, 2, 4, grade=1, seed=3)
        rb, rg = srv.wait(bad), srv.wait(good)
    assert rb["status"] != 0 and rg["status"] == 0
