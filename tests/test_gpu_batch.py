"""Batched design evaluations (mg_batch_*): many SIMP cantilevers of uneven grid
sizes with 1-4 load cases each, solved together by the mixed-precision
multi-problem solver, against the FP64 oracle.

Bars: FP64 residual <= 1e-8 per problem; compliance and sensitivities within
1e-6 relative of the oracle; a problem's results are bitwise the same alone and
inside any batch (each problem's multigrid hierarchy, reductions and phase
sequence depend on that problem only).
"""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu


def opts(**kw):
    base = dict(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3, timeout_s=300.0)
    base.update(kw)
    return M.default_opts(**base)


def small_designs(seed=5):
    rng = np.random.default_rng(seed)
    shapes = [((8, 4, 4), [(0, 4), (2, 3)]), ((16, 8, 8), [(0, 8)]), ((12, 6, 6), [(1, 5), (6, 6), (0, 2)]),
              ((24, 12, 12), [(3, 9), (0, 12)])]
    return [dict(nx=s[0], ny=s[1], nz=s[2], rho=rng.uniform(0.01, 1.0, s[0] * s[1] * s[2]), spans=sp)
            for s, sp in shapes]


def oracle_case(d, span):
    nx, ny, nz = d["nx"], d["ny"], d["nz"]
    desc = O.simp_desc(nx, ny, nz, load_y0=span[0], load_y1=span[1], rtol=1e-12, maxit=10 ** 6)
    u, dc, rep = O.simp_solve(desc, d["rho"])
    return u, dc, rep.compliance


def test_batch_matches_oracle():
    des = small_designs()
    with M.Batch(des) as b:
        assert b.n_designs == 4 and b.n_problems == 8
        rc, reps = b.solve(opts())
        for r in reps:
            assert r.status == 0 and r.relres <= 1e-8, (r.status, r.relres)
        for d, dd in enumerate(des):
            comp, dc, u = b.results(d, want_u=True)
            for c, span in enumerate(dd["spans"]):
                u_ref, dc_ref, c_ref = oracle_case(dd, span)
                assert abs(comp[c] - c_ref) / abs(c_ref) < 1e-6, (d, c, comp[c], c_ref)
                assert np.abs(dc[c] - dc_ref).max() / np.abs(dc_ref).max() < 1e-6, (d, c)
                assert np.linalg.norm(u[c] - u_ref) / np.linalg.norm(u_ref) < 1e-6, (d, c)


def test_batch_result_is_independent_of_batch_composition():
    des = small_designs()
    with M.Batch(des) as b:
        b.solve(opts())
        mixed = [b.results(d, want_u=True) for d in range(len(des))]
    for d in (0, 2, 3):
        with M.Batch([des[d]]) as b1:
            b1.solve(opts())
            comp, dc, u = b1.results(0, want_u=True)
        assert np.array_equal(comp, mixed[d][0]), d
        assert np.array_equal(dc, mixed[d][1]), d
        assert np.array_equal(u, mixed[d][2]), d


def test_batch_subset_solve_leaves_other_problems():
    des = small_designs()
    with M.Batch(des) as b:
        b.solve(opts())
        before = [b.results(d) for d in range(len(des))]
        rho2 = np.clip(des[1]["rho"] + np.random.default_rng(9).normal(0, 0.02, des[1]["rho"].size), 0.01, 1.0)
        b.set_design(1, rho2)
        active = np.zeros(b.n_problems, np.uint8)
        active[2] = 1  # design 1 is problem 2 (design 0 has two cases)
        rc, reps = b.solve(opts(warm_start=1), active=active)
        assert reps[2].status == 0 and reps[2].relres <= 1e-8
        for d in (0, 2, 3):
            c, dc, _ = b.results(d)
            assert np.array_equal(c, before[d][0]) and np.array_equal(dc, before[d][1])
        c1, dc1, _ = b.results(1)
    _, dc_ref, c_ref = oracle_case(dict(des[1], rho=rho2), des[1]["spans"][0])
    assert abs(c1[0] - c_ref) / c_ref < 1e-6
    assert np.abs(dc1[0] - dc_ref).max() / np.abs(dc_ref).max() < 1e-6


def test_batch_warm_start_cuts_iterations():
    d = small_designs()[3]
    with M.Batch([d]) as b:
        _, cold = b.solve(opts())
        rho2 = np.clip(d["rho"] + np.random.default_rng(2).normal(0, 0.02, d["rho"].size), 0.01, 1.0)
        b.set_design(0, rho2)
        _, warm = b.solve(opts(warm_start=1))
        c_warm, dc_warm, _ = b.results(0)
    assert all(r.status == 0 and r.relres <= 1e-8 for r in warm)
    assert sum(r.krylov_iterations for r in warm) < sum(r.krylov_iterations for r in cold)
    _, dc_ref, c_ref = oracle_case(dict(d, rho=rho2), d["spans"][0])
    assert abs(c_warm[0] - c_ref) / c_ref < 1e-6


def test_batch_jacobi_and_bf16_forms_converge():
    des = small_designs()[:2]
    for o in (opts(preconditioner=M.PC_JACOBI), opts(precision=M.MIXED_BF16X3)):
        with M.Batch(des) as b:
            rc, reps = b.solve(o)
            assert all(r.status == 0 and r.relres <= 1e-8 for r in reps)
            comp, dc, _ = b.results(1)
        _, dc_ref, c_ref = oracle_case(des[1], des[1]["spans"][0])
        assert abs(comp[0] - c_ref) / c_ref < 1e-6


def test_autotune_picks_a_converging_schedule_and_caches_it():
    des = small_designs()
    with M.Batch(des) as b:
        o, secs = b.autotune(opts(), max_trials=6)
        assert secs > 0
        o2, secs2 = b.autotune(opts(), max_trials=6)  # cache hit: same schedule, no trials
        assert (o2.precision, o2.smooth_degree, o2.coarse_degree, o2.graph_chunk) == \
               (o.precision, o.smooth_degree, o.coarse_degree, o.graph_chunk)
        assert secs2 == secs
        rc, reps = b.solve(o)
        assert all(r.status == 0 and r.relres <= 1e-8 for r in reps)
        comp, dc, _ = b.results(2)
    _, dc_ref, c_ref = oracle_case(des[2], des[2]["spans"][1])
    assert abs(comp[1] - c_ref) / c_ref < 1e-6


def test_batch_rejects_plain_precision_and_bad_design_index():
    with M.Batch(small_designs()[:1]) as b:
        rc, _ = b.solve(opts(precision=M.PLAIN_FP64), raise_on_error=False)
        assert rc == M.MG_ENOTSUP
        assert M.lib().mg_batch_results(b.h, 5, None, None, None) == M.MG_EINVAL
        assert M.lib().mg_batch_results(b.h, -1, None, None, None) == M.MG_EINVAL
