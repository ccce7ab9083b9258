"""Request loop (mg_server_*): continuous batching of design evaluations.

Checks: every result equals the one the same request gets when its chain is
served alone (bitwise: each problem's solve depends on that problem only), and
matches the FP64 oracle within 1e-6; requests of different chains overlap on
the GPU; chains beyond the device-memory cap are evicted and come back; a chain
that cannot fit alone is answered with MG_ENOMEM.
"""
import numpy as np
import pytest

import mastgpu as M
import oracle as O

pytestmark = pytest.mark.gpu

CHAINS = [((8, 4, 4), [(0, 4)]), ((16, 8, 8), [(0, 8), (2, 5)]), ((12, 6, 6), [(3, 6)]),
          ((16, 8, 8), [(4, 8)]), ((24, 12, 12), [(0, 12)])]


def opts():
    return M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3, timeout_s=300.0)


def chain_requests(n_per_chain=3, seed=11):
    """Per chain: a list of density fields, each the previous plus N(0, 0.02) noise."""
    rng = np.random.default_rng(seed)
    out = []
    for (nx, ny, nz), spans in CHAINS:
        cur = rng.uniform(0.01, 1.0, nx * ny * nz)
        seq = []
        for _ in range(n_per_chain):
            cur = np.clip(cur + rng.normal(0.0, 0.02, cur.size), 0.01, 1.0)
            seq.append(cur.copy())
        out.append(seq)
    return out


def serve(chain_ids, reqs, interleave=True, **kw):
    """Submit the requests of the given chains (all at once) and collect results by (chain, k)."""
    res = {}
    with M.Server(opts(), **kw) as s:
        order = []
        n = max(len(reqs[c]) for c in chain_ids)
        if interleave:
            for k in range(n):
                for c in chain_ids:
                    order.append((c, k))
        else:
            order = [(c, k) for c in chain_ids for k in range(len(reqs[c]))]
        for tag, (c, k) in enumerate(order):
            (nx, ny, nz), spans = CHAINS[c]
            res[(c, k)] = s.submit(tag, c, nx, ny, nz, reqs[c][k], spans)
        s.drain(timeout_s=600.0)
        done = {}
        while True:
            got = s.poll(1024)
            if not got:
                break
            for cpl in got:
                done[cpl.tag] = cpl
        st = s.stats()
    assert len(done) == len(order)
    for tag, (c, k) in enumerate(order):
        assert done[tag].status == 0 and done[tag].relres <= 1e-8, (c, k, done[tag].status, done[tag].relres)
    return res, st, done


def test_each_result_is_the_same_alone_and_in_the_mix():
    reqs = chain_requests()
    ids = list(range(len(CHAINS)))
    mixed, st, _ = serve(ids, reqs)
    assert st["completed"] == 15 and st["failed"] == 0
    assert st["peak_inflight"] >= 2  # requests of different chains shared the solver launches
    for c in ids:
        alone, _, _ = serve([c], reqs)
        for k in range(len(reqs[c])):
            assert np.array_equal(mixed[(c, k)][0], alone[(c, k)][0]), (c, k)
            assert np.array_equal(mixed[(c, k)][1], alone[(c, k)][1]), (c, k)
    # and both match the FP64 oracle
    for c in ids:
        (nx, ny, nz), spans = CHAINS[c]
        for i, (j0, j1) in enumerate(spans):
            desc = O.simp_desc(nx, ny, nz, load_y0=j0, load_y1=j1, rtol=1e-12, maxit=10 ** 6)
            _, dc_ref, rep = O.simp_solve(desc, reqs[c][-1])
            comp, dc = mixed[(c, len(reqs[c]) - 1)]
            assert abs(comp[i] - rep.compliance) / rep.compliance < 1e-6
            assert np.abs(dc[i] - dc_ref).max() / np.abs(dc_ref).max() < 1e-6


def test_warm_start_from_the_chain_cuts_iterations():
    reqs = chain_requests(n_per_chain=4)
    _, _, done = serve([4], reqs, interleave=False)
    its = [done[t].krylov_iterations for t in sorted(done)]
    assert its[1] < its[0] and its[-1] < its[0], its


def test_memory_cap_evicts_and_readmits():
    reqs = chain_requests(n_per_chain=2)
    # room for about the two largest chains (24x12x12: 1.35 MB, 16x8x8 with two
    # load cases: 0.84 MB of resident tables) out of 2.9 MB in all
    cap = 2_300_000
    res, st, _ = serve(list(range(len(CHAINS))), reqs, hbm_cap_bytes=cap)
    assert st["evictions"] > 0 and st["failed"] == 0
    assert st["peak_resident_bytes"] <= cap * 1.5
    ref, _, _ = serve(list(range(len(CHAINS))), reqs)
    for key in ref:  # a re-admitted chain restarts cold: same answer within the tolerance
        assert np.allclose(res[key][0], ref[key][0], rtol=1e-6, atol=0)


def test_chain_larger_than_the_cap_is_rejected():
    rng = np.random.default_rng(0)
    with M.Server(opts(), hbm_cap_bytes=1 << 20) as s:
        s.submit(1, 0, 24, 12, 12, rng.uniform(0.01, 1, 24 * 12 * 12), [(0, 12)])
        s.drain(timeout_s=120.0)
        got = s.poll(8)
    assert len(got) == 1 and got[0].status == M.MG_ENOMEM


def test_malformed_requests_are_refused():
    with M.Server(opts()) as s:
        with pytest.raises(M.MastGpuError):
            s.submit(1, 0, 8, 4, 4, np.full(128, 2.0), [(0, 4)])  # density > 1
        with pytest.raises(M.MastGpuError):
            s.submit(2, 0, 8, 4, 4, np.full(128, 0.5), [(0, 9)])  # span beyond the edge
        s.submit(3, 0, 8, 4, 4, np.full(128, 0.5), [(0, 4)])
        try:  # contradicts chain 0's grid: refused at submit or answered with MG_EINVAL
            s.submit(4, 0, 8, 4, 8, np.full(256, 0.5), [(0, 4)])
            refused = False
        except M.MastGpuError as e:
            assert e.status == M.MG_EINVAL
            refused = True
        s.drain(timeout_s=120.0)
        got = {c.tag: c.status for c in s.poll(8)}
    assert got[3] == 0
    assert refused or got[4] == M.MG_EINVAL


def test_synthetic_stream_reports_latency_percentiles():
    with M.Server(opts()) as s:
        st, comp = s.run_synthetic(40, rate=400.0, n_chains=6, sizes=[(8, 4, 4), (16, 8, 8)],
                                   big_fraction=0.0, max_cases=2, seed=3)
    assert st["completed"] == 40 and st["failed"] == 0
    assert 0 < st["p50_s"] <= st["p99_s"] <= st["max_s"]
    assert st["solves_per_s"] > 0 and st["peak_inflight"] >= 2
    assert np.all(comp[:, 0] > 0)


def test_synthetic_stream_results_match_the_oracle():
    """Served completions of the synthetic Poisson stream, checked one by one: each sampled
    request's densities and load spans are regenerated from the stream's seed
    (mg_server_synthetic_request) and solved by the FP64 oracle; compliance within 1e-6."""
    sizes = ((8, 4, 4), (16, 8, 8), (12, 6, 6))
    kw = dict(n_chains=6, sizes=sizes, big_fraction=0.0, max_cases=3, seed=5)
    with M.Server(opts()) as s:
        st, comp = s.run_synthetic(40, rate=400.0, **kw)
    assert st["completed"] == 40 and st["failed"] == 0
    desc = M.synthetic_desc(40, 400.0, **kw)
    for i in (0, 7, 19, 33, 39):
        r = M.synthetic_request(desc, i)
        nx, ny, nz = r["grid"]
        for k, (j0, j1) in enumerate(r["spans"]):
            _, _, ref = O.simp_solve(O.simp_desc(nx, ny, nz, load_y0=j0, load_y1=j1, rtol=1e-12,
                                                 maxit=10 ** 6), r["rho"], want_sens=False)
            assert abs(comp[i, k] - ref.compliance) <= 1e-6 * abs(ref.compliance), (i, k)
        assert np.all(comp[i, len(r["spans"]):] == 0.0)
