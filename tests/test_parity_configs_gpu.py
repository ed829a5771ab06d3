"""Parity at the benchmark configurations and of the budget split (GPU).

* The plain BFS configuration as written: RMAT scale 16, edge factor 16
  (a=.57 b=.19 c=.19), seed 1, BFS from vertex 0, no device cap, levels
  bit-exact against the serial oracle.
* The static split: for every reference run in the golden manifest, the same
  edge cap gives the engine the reference's own static prefix
  (max_partition_size after rounding, GraphMeta.cuh:341-365) and the same set
  of edges owned by static vertices (max_static_node); at a mid-size graph the
  engine's prefix equals the oracle's restatement of that rule for every
  budget mode that caps the prefix.
* Reference-mode PageRank (FP64, 0.15 + 0.85 * sum, per-vertex stop at
  |delta| <= 0.001, gpu_kernels.cuh:533-594) at RMAT scale 16 against the
  oracle: max-abs and relative error per vertex.
"""
import json
import os

import numpy as np
import pytest

import ascetic_gb300 as A
import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
PR_TOL = 1e-6       # max-abs per vertex against the FP64 oracle
PR_REL_TOL = 1e-9   # relative per vertex, reference mode (FP64 sums; ranks are >= 0.15)


@pytest.fixture(scope="module", autouse=True)
def _engine():
    A.lib()
    if A.device_count() == 0:
        pytest.fail("no CUDA device: the engine has no CPU fallback")


def test_plain_bfs_configuration_scale16_seed1_source0():
    ptr, col = A.rmat_csr(16, 16, 1)
    assert len(ptr) - 1 == 65536 and int(ptr[-1]) == 1048576
    with A.Graph.from_csr(ptr, col, budget=A.make_budget()) as g:
        assert g.info.static_edges == g.E           # no cap: the whole graph is resident
        got, st = g.run("bfs", 0)
    exp = oracle.bfs(ptr, col, 0)
    assert np.array_equal(got, exp)
    assert st["ondemand_edges"] == 0
    assert st["reached_edges"] == oracle.reached_edges(ptr, exp, len(ptr))


def _check_split_against_reference_rule(g, ptr, cap):
    """Engine prefix and static vertices against the oracle's restatement of
    the reference rule for an edge cap."""
    flags, mps, in_static = oracle.static_split(ptr, cap)
    S, st = int(g.info.static_vertices), int(g.info.static_edges)
    assert st == mps, (cap, st, mps)
    assert int(ptr[S]) == in_static, (cap, S, in_static)
    deg = np.diff(ptr.astype(np.int64))
    # every vertex that owns an edge is static in both or in neither
    mine = np.zeros(len(deg), bool)
    mine[:S] = True
    assert np.array_equal(mine & (deg > 0), flags.astype(bool) & (deg > 0))


def _graph_arrays(z, algo):
    if algo == "bfs":
        return z["ptr"], z["col"], None
    if algo == "sssp":
        return z["ptr"], z["adj"], None
    if algo == "cc":
        return z["sptr"], z["scol"], None
    return z["cptr"], z["ccol"], z["outdeg"]


@pytest.mark.parametrize("graph", sorted(MANIFEST["graphs"]))
def test_static_split_equals_reference_runs(graph):
    """The cap each golden run gave the reference yields the reference's own
    static prefix, and the vertices above its max_static_node that the engine
    counts as static own no edges."""
    z = np.load(os.path.join(GOLDEN, graph + ".npz"))
    seen = set()
    for r in MANIFEST["graphs"][graph]["runs"]:
        key = (r["algo"], r["static_edges"])
        if key in seen:
            continue
        seen.add(key)
        ptr, edges, od = _graph_arrays(z, r["algo"])
        with A.Graph.from_csr(ptr, edges, outdeg=od, budget=A.make_budget(edges=r["static_edges"])) as g:
            assert g.info.static_edges == r["ref_static_edges"], r["key"]
            S = int(g.info.static_vertices)
            m = r["max_static_node"]
            deg = np.diff(np.asarray(ptr, np.int64))
            if S > 0:
                assert m < S and not deg[m + 1:S].any(), r["key"]
            else:
                assert m == 0, r["key"]          # the reference's initial value: no static vertex
            _check_split_against_reference_rule(g, np.asarray(ptr, np.uint64), r["static_edges"])


@pytest.mark.parametrize("packing", ["1", "0"])
def test_static_split_modes_follow_reference_rule(packing, monkeypatch):
    """RMAT scale 16: fraction, byte and edge caps all end in the reference's
    rounding (a multiple of 4096 edges, at most E) and static-vertex rule,
    with 32-bit edge words and with the bit stream (whose narrower edges fit
    more of them in the same bytes)."""
    monkeypatch.setenv("ASC_EDGE_PACKING", packing)
    ptr, col = A.rmat_csr(16, 16, 1)
    E = int(ptr[-1])
    ptr64 = ptr.astype(np.uint64)
    # a byte budget also holds the first in-edge of every vertex (bottom-up
    # BFS steps) when edges stay on demand; the prefix cap is what remains
    for frac in (0.0, 0.05, 0.25, 0.5, 0.999, 1.0):
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
            eb = g.info.edge_bits / 8.0
            heads = g.info.in_head_bytes
            cap = E if frac * 4.0 >= eb else int((frac * float(E) * 4.0 - heads) / eb)
            _check_split_against_reference_rule(g, ptr64, cap)
            assert g.info.static_edges % 4096 == 0
            assert g.info.device_edge_bytes <= max(frac * E * 4.0, 4.0 * E) or frac < 1
    for nbytes in (0, 4095, 1 << 20, 3_000_001, 10 << 20):
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(nbytes=nbytes)) as g:
            eb = g.info.edge_bits / 8.0
            heads = g.info.in_head_bytes
            cap = E if nbytes / eb >= E else int((nbytes - heads) / eb)
            _check_split_against_reference_rule(g, ptr64, cap)
            assert g.info.device_edge_bytes <= max(nbytes, 4.0 * E)
    for edges in (1, 4095, 4096, 123_457, E - 1, E, E + 5):
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(edges=edges)) as g:
            _check_split_against_reference_rule(g, ptr64, min(edges, E))
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(advise_k=0.001)) as g:
        assert g.info.static_edges % 4096 == 0 and g.info.static_edges <= E


@pytest.mark.parametrize("scale,frac", [(16, 1.0), (16, 0.3), (16, 0.0), (20, 0.3)])
def test_reference_pagerank_at_scale(scale, frac):
    """Reference PageRank's per-vertex stop (|delta| <= 0.001, vertices stay
    inactive) makes a wrong pass count visible: the engine's pass count and
    every rank match the oracle's at RMAT scale 16 and 20 (1 M vertices)."""
    cptr, ccol, od = A.rmat_csr(scale, 16, 3, transpose=True)
    exp, passes = oracle.pr_ref(cptr, ccol, od)
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=frac)) as g:
        got, st = g.run("pr")
    err = np.abs(got - exp)
    rel = err / np.abs(exp)
    assert err.max() <= PR_TOL, err.max()
    assert rel.max() <= PR_REL_TOL, rel.max()
    assert st["iterations"] == passes


@pytest.mark.parametrize("frac", [1.0, 0.3, 0.0])
def test_standard_pagerank_scale16_fp32_and_fp64(frac):
    """Standard PageRank (damping 0.85, uniform start, dangling mass spread
    uniformly, stop at FP64 L1 residual < 1e-9) at RMAT scale 16 against the
    FP64 oracle: FP64 within 1e-12 relative per vertex in the oracle's pass
    count; FP32 contributions within 1e-6 max-abs and 1e-5 relative, converged
    below the 1e-9 residual well inside the 100-pass cap (a few passes after
    FP64 while the last FP32 contributions settle)."""
    cptr, ccol, od = A.rmat_csr(16, 16, 3, transpose=True)
    exp, passes, _ = oracle.pr_std(cptr, ccol, od)
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=frac)) as g:
        for prec, rel_tol in ((A.F64, 1e-12), (A.F32, 1e-5)):
            got, st = g.run("pr", params=A.make_params(pr_mode=A.PR_STD, precision=prec))
            err = np.abs(got.astype(np.float64) - exp)
            assert err.max() <= PR_TOL, (prec, err.max())
            assert (err / exp).max() <= rel_tol, (prec, (err / exp).max())
            assert st["residual"] < 1e-9
            if prec == A.F64:
                assert st["iterations"] == passes
            else:
                assert st["iterations"] <= passes + 10, (st["iterations"], passes)


def test_batched_configuration_scale26_rows_equal_oracle():
    """The batched multi-source configuration: RMAT scale 26, edge factor 16,
    seed 4, weights uniform in [1, 63], static region 25% of edge bytes; 64
    seeded sources with out-degree > 0 as one 64-wide BFS batch and one batched
    SSSP; four rows of each (first, last, two between) bit-exact against the
    oracle (the reference frontier scheme on all host threads)."""
    ptr, adj = A.rmat_csr(26, 16, 4, weights=(1, 63))
    assert len(ptr) - 1 == 1 << 26 and int(ptr[-1]) == 1 << 30
    deg = np.diff(ptr)
    rng = np.random.default_rng(4)
    srcs = [int(x) for x in rng.choice(np.nonzero(deg > 0)[0], size=64, replace=False)]
    del deg
    check = [0, 21, 42, 63]
    threads = os.cpu_count() or 1
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=0.25)) as g:
        assert 0 < g.info.static_edges < g.E
        for algo, mode in (("bfs", 0), ("sssp", 1)):
            rows, st = g.run_batch(algo, srcs)
            assert st["ondemand_edges"] > 0
            kept = {i: rows[i].copy() for i in check}
            del rows
            col = adj[:, 0].copy() if algo == "bfs" else adj
            for i in check:
                exp, _ = oracle.relax_mt(mode, ptr, col, srcs[i], threads)
                assert np.array_equal(kept[i], exp), (algo, i, srcs[i])
            del col, kept
