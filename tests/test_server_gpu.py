"""The query server (GPU): continuous batching gives every query the values of
a solo run, whatever it shares its batch with; FIFO mode is the plain engine;
the budget is enforced; cancellation and statistics work."""
import numpy as np
import pytest

import ascetic_gb300 as A
import oracle

pytestmark = pytest.mark.gpu
PR_TOL = 1e-6


def _graphs():
    ga = A.rmat_csr(12, 16, 41, weights=(1, 63))
    gb = A.rmat_csr(11, 8, 42, weights=(1, 63))
    return [ga, gb]


@pytest.mark.parametrize("mode", [A.SERVE_BATCHED, A.SERVE_FIFO])
def test_mixed_queries_equal_solo_runs(mode):
    data = _graphs()
    graphs = [A.Graph.from_csr(p, adj, budget=A.make_budget(frac=0.25)) for p, adj in data]
    rng = np.random.default_rng(3)
    std32 = A.make_params(pr_mode=A.PR_STD, precision=A.F32)
    with A.Server(mode=mode) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        plan = []
        for i in range(150):
            gi = int(rng.integers(0, 2))
            r = rng.random()
            V = graphs[gi].V
            if r < 0.5:
                plan.append((gi, "bfs", int(rng.integers(0, V)), None))
            elif r < 0.8:
                plan.append((gi, "sssp", int(rng.integers(0, V)), None))
            elif r < 0.9:
                plan.append((gi, "cc", 0, None))
            else:
                plan.append((gi, "pr", 0, std32))
        tickets = [srv.submit(ids[gi], algo, src, params=p) for gi, algo, src, p in plan]
        results = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(plan) and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    sssp_cache = {}
    for (gi, algo, src, p), (out, info) in zip(plan, results):
        ptr, adj = data[gi]
        col = adj[:, 0]
        assert info["status"] == A.OK
        if algo == "bfs":
            assert np.array_equal(out, oracle.bfs(ptr, col, src))
        elif algo == "sssp":
            key = (gi, src)
            if key not in sssp_cache:
                sssp_cache[key] = oracle.sssp(ptr, adj, src)
            assert np.array_equal(out, sssp_cache[key])
        elif algo == "cc":
            assert np.array_equal(out, oracle.cc(ptr, col))
        else:
            cptr, ccol, od = A.formats.transpose(ptr, col)
            exp, _, _ = oracle.pr_std(cptr, ccol, od)
            assert np.abs(out.astype(np.float64) - exp).max() <= PR_TOL
    for g in graphs:
        g.close()


def test_batched_query_alone_equals_in_the_mix():
    ptr, adj = A.rmat_csr(12, 16, 43, weights=(1, 63))
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=0.25)) as g:
        with A.Server() as srv:
            gid = srv.add_graph(g)
            alone, _ = srv.wait(srv.submit(gid, "bfs", 17))
            alone_s, _ = srv.wait(srv.submit(gid, "sssp", 17))
            ts = [srv.submit(gid, "bfs", int(s)) for s in range(100, 160)]
            mid = srv.submit(gid, "bfs", 17)      # joins a running batch
            mid_s = srv.submit(gid, "sssp", 17)
            ts += [srv.submit(gid, "sssp", int(s)) for s in range(200, 230)]
            mixed, info = srv.wait(mid)
            mixed_s, _ = srv.wait(mid_s)
            for t in ts:
                srv.wait(t)
    assert np.array_equal(alone, mixed) and np.array_equal(alone_s, mixed_s)
    assert np.array_equal(alone, oracle.bfs(ptr, adj[:, 0], 17))


def test_budget_and_cancel():
    ptr, adj = A.rmat_csr(10, 8, 44, weights=(1, 63))
    with A.Graph.from_csr(ptr, adj) as g:
        with pytest.raises(A.AscError) as e:
            with A.Server(budget_bytes=1024) as srv:
                srv.add_graph(g)
        assert e.value.status == A.ERR_BUDGET
        # room for the graph and its single-query state (the server's estimate)
        # but not for a batch (about 45 bytes per vertex): BFS queries fall back
        # to whole runs and still answer correctly
        V, E = g.V, g.E
        base = g.info.device_edge_bytes + 4 * (V + 1)
        ws = 4 * V + 12 * (V // 32 + 2) + 8 * V + 8 * (E // 256 + 1024) + 4096
        with A.Server(budget_bytes=base + ws + 20000) as srv:
            gid = srv.add_graph(g)
            out, info = srv.wait(srv.submit(gid, "bfs", 3))
            assert np.array_equal(out, oracle.bfs(ptr, adj[:, 0], 3))
        with A.Server(mode=A.SERVE_FIFO) as srv:
            gid = srv.add_graph(g)
            ts = [srv.submit(gid, "pr", 0) for _ in range(20)]
            srv.cancel(ts[-1])
            outs = [srv.wait(t) for t in ts]
            st = srv.stats()
            assert st["completed"] + st["cancelled"] == 20


@pytest.mark.parametrize("extra", [1_000_000, 2_500_000, 5_000_000, 10_000_000])
def test_tight_shared_budget_completes(extra):
    """Several graphs under a budget too small for all their batch engines at
    once, every query submitted at t=0: engines take turns (idle ones and unused
    single-query state are freed for waiting queries, and queries that cannot
    get batch memory run whole), every query completes with the solo values."""
    data = [A.rmat_csr(13, 16, 51, weights=(1, 63)), A.rmat_csr(12, 16, 52, weights=(1, 63)),
            A.rmat_csr(11, 16, 53, weights=(1, 63))]
    graphs = [A.Graph.from_csr(p, adj, budget=A.make_budget(frac=0.25)) for p, adj in data]
    base = sum(g.info.device_edge_bytes + 4 * (g.V + 1) for g in graphs)
    rng = np.random.default_rng(extra)
    std32 = A.make_params(pr_mode=A.PR_STD, precision=A.F32)
    plan = []
    for i in range(120):
        gi = int(rng.integers(0, 3))
        r = rng.random()
        algo = "bfs" if r < 0.5 else "sssp" if r < 0.8 else "cc" if r < 0.9 else "pr"
        src = int(rng.integers(0, graphs[gi].V)) if algo in ("bfs", "sssp") else 0
        plan.append((gi, algo, src))
    with A.Server(budget_bytes=base + extra) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        tickets = [srv.submit(ids[gi], algo, src, params=std32 if algo == "pr" else None)
                   for gi, algo, src in plan]
        results = [srv.wait(t, timeout_ms=120000) for t in tickets]
        st = srv.stats()
        assert st["device_bytes"] <= base + extra
    assert st["completed"] == len(plan) and st["failed"] == 0
    for (gi, algo, src), (out, info) in zip(plan, results):
        ptr, adj = data[gi]
        if algo == "bfs":
            assert np.array_equal(out, oracle.bfs(ptr, adj[:, 0], src))
        elif algo == "sssp":
            assert np.array_equal(out, oracle.sssp(ptr, adj, src))
        elif algo == "cc":
            assert np.array_equal(out, oracle.cc(ptr, adj[:, 0]))
    for g in graphs:
        g.close()


@pytest.mark.parametrize("max_batch", [12, 32])
def test_narrow_sssp_batches_equal_solo_runs(max_batch):
    """A server whose max_batch is at most 32 (or whose budget cannot hold 64
    distance columns of a graph) runs SSSP batches with rows of 16 or 32
    sources; every query still gets the solo values."""
    ptr, adj = A.rmat_csr(13, 16, 61, weights=(1, 63))
    deg = np.diff(ptr)
    rng = np.random.default_rng(max_batch)
    srcs = rng.choice(np.nonzero(deg)[0], size=70, replace=False).tolist()
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=0.25)) as g:
        with A.Server(max_batch=max_batch) as srv:
            gid = srv.add_graph(g)
            tickets = [srv.submit(gid, "sssp", s) for s in srcs]
            results = [srv.wait(t, timeout_ms=120000) for t in tickets]
            st = srv.stats()
    assert st["completed"] == len(srcs) and st["failed"] == 0
    for s, (out, info) in zip(srcs, results):
        assert info["status"] == A.OK and 1 <= info["batch_size"] <= max_batch
        assert np.array_equal(out, oracle.sssp(ptr, adj, s)), s
