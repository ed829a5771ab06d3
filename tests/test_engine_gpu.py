"""CUDA engine against the oracle and the reference golden vectors (GPU).

Every value array is compared bit for bit (BFS, SSSP, CC) or within 1e-6
max-abs per vertex (PageRank), across static/on-demand splits from
all-on-demand to all-static, through the C ABI.
"""
import json
import os
import tempfile

import numpy as np
import pytest

import ascetic_gb300 as A
import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
PR_TOL = 1e-6   # max-abs per vertex against the FP64 oracle


@pytest.fixture(scope="module", autouse=True)
def _engine():
    A.lib()
    if A.device_count() == 0:
        pytest.fail("no CUDA device: the engine has no CPU fallback")


@pytest.mark.parametrize("graph", sorted(MANIFEST["graphs"]))
def test_golden_vectors(graph):
    """Same graph, same static prefix size as the reference run, same result."""
    z = np.load(os.path.join(GOLDEN, graph + ".npz"))
    cache = {}
    for r in MANIFEST["graphs"][graph]["runs"]:
        algo = r["algo"]
        key = (algo, r["static_edges"])
        if key not in cache:
            b = A.make_budget(edges=r["static_edges"])
            if algo in ("bfs",):
                cache[key] = A.Graph.from_csr(z["ptr"], z["col"], budget=b)
            elif algo == "sssp":
                cache[key] = A.Graph.from_csr(z["ptr"], z["adj"], budget=b)
            elif algo == "cc":
                cache[key] = A.Graph.from_csr(z["sptr"], z["scol"], budget=b)
            else:
                cache[key] = A.Graph.from_csr(z["cptr"], z["ccol"], outdeg=z["outdeg"], budget=b)
        g = cache[key]
        exp = z[r["key"]]
        if algo == "pr_ref":
            got, _ = g.run("pr")
            assert np.abs(got - exp).max() <= PR_TOL, r["key"]
        else:
            got, _ = g.run(algo, r["source"])
            assert np.array_equal(got, exp), r["key"]
    for g in cache.values():
        g.close()


FRACS = [1.0, 0.5, 0.25, 0.05, 0.0]
# the iteration loop runs as a CUDA graph by default; the host-driven loop and
# the per-region timed launches must give the same values
LOOPS = [0, A.RUN_HOST_LOOP, A.RUN_PHASE_TIMING]


@pytest.mark.parametrize("frac", FRACS)
def test_bfs_matches_oracle(frac):
    ptr, col = A.rmat_csr(14, 16, 11)
    deg = np.diff(ptr)
    srcs = [0, int(np.nonzero(deg)[0][-1]), int(np.nonzero(deg == 0)[0][0]) if (deg == 0).any() else 5]
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
        for s in srcs:
            exp = oracle.bfs(ptr, col, s)
            iters = set()
            for flags in LOOPS:
                got, st = g.run("bfs", s, params=A.make_params(flags=flags))
                assert np.array_equal(got, exp), (frac, s, flags)
                assert st["reached_edges"] == oracle.reached_edges(ptr, exp, len(ptr))
                assert st["reached_vertices"] == int((exp != len(ptr)).sum())
                if g.info.static_edges < g.E and st["reached_vertices"] > 1000:
                    assert st["ondemand_edges"] > 0
                iters.add(st["iterations"])
            # BFS runs one level per iteration whatever drives the loop
            assert len(iters) == 1


@pytest.mark.parametrize("frac", FRACS)
def test_sssp_matches_oracle(frac):
    ptr, adj = A.rmat_csr(13, 16, 12, weights=(1, 63))
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=frac)) as g:
        for s in (0, 77):
            exp = oracle.sssp(ptr, adj, s)
            for flags in LOOPS:
                got, _ = g.run("sssp", s, params=A.make_params(flags=flags))
                assert np.array_equal(got, exp), (frac, s, flags)


@pytest.mark.parametrize("frac", FRACS)
def test_cc_matches_oracle(frac):
    ptr, col = A.rmat_csr(13, 8, 13, symmetric=True)
    exp = oracle.cc(ptr, col)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
        for flags in LOOPS:
            got, _ = g.run("cc", params=A.make_params(flags=flags))
            assert np.array_equal(got, exp), flags


@pytest.mark.parametrize("frac", [1.0, 0.25, 0.0])
def test_batch_bfs_rows_equal_single_source(frac):
    ptr, col = A.rmat_csr(13, 16, 31)
    deg = np.diff(ptr)
    rng = np.random.default_rng(5)
    srcs = rng.choice(np.nonzero(deg)[0], size=62, replace=False).tolist() + [0, 0]   # duplicates allowed
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
        got, st = g.run_batch("bfs", srcs)
        for i, s in enumerate(srcs):
            assert np.array_equal(got[i], oracle.bfs(ptr, col, s)), (frac, i, s)
        one, _ = g.run_batch("bfs", [srcs[3]])
        assert np.array_equal(one[0], got[3])


@pytest.mark.parametrize("n_src", [3, 6, 40])
@pytest.mark.parametrize("frac", [1.0, 0.25, 0.0])
def test_batch_sssp_rows_equal_single_source(frac, n_src):
    """Rows of a batched SSSP equal single-source runs: 3 sources take the
    per-source loads, 6 the 16-byte quads, 40 (+3) the lane groups per edge."""
    ptr, adj = A.rmat_csr(12, 16, 32, weights=(1, 63))
    deg = np.diff(ptr)
    rng = np.random.default_rng(6)
    srcs = rng.choice(np.nonzero(deg)[0], size=n_src, replace=False).tolist()
    if n_src > 8:
        srcs += [7, 7, int(np.nonzero(deg == 0)[0][0])]
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=frac)) as g:
        got, st = g.run_batch("sssp", srcs)
        for i, s in enumerate(srcs):
            assert np.array_equal(got[i], oracle.sssp(ptr, adj, s)), (frac, i, s)


def test_packed_and_unpacked_weighted_edges():
    """Weighted edges are stored packed (dst << bits | weight, bits the width of
    the largest weight: 13 + 6 = 19-bit words here, stored as a bit stream) when
    they fit, AoS otherwise; both give the oracle's distances, and a byte budget
    holds 64/19 times the edges when packed."""
    ptr, adj = A.rmat_csr(13, 8, 36, weights=(1, 63))
    big = adj.copy()
    big[:, 1] = (big[:, 1].astype(np.uint64) * 40000).astype(np.uint32)   # needs > 19 weight bits
    for arr, packed in ((adj, True), (big, False)):
        with A.Graph.from_csr(ptr, arr, budget=A.make_budget(frac=0.2)) as g:
            assert (g.info.weight_bits == 6) == packed and (g.info.weight_bits > 0) == packed
            assert g.info.edge_bytes == (4 if packed else 8)
            assert g.info.edge_bits == (19 if packed else 64)
            frac_edges = g.info.static_edges / g.E
            # the byte budget also holds the first in-edge of every vertex
            expect = (0.2 * 8 * g.E - g.info.in_head_bytes) / (g.info.edge_bits / 8) / g.E
            assert abs(frac_edges - expect) < 0.05, (frac_edges, expect)
            for s in (0, 41):
                got, _ = g.run("sssp", s)
                assert np.array_equal(got, oracle.sssp(ptr, arr, s)), (packed, s)
                got, _ = g.run("bfs", s)
                assert np.array_equal(got, oracle.bfs(ptr, arr[:, 0].copy(), s))
            rows, _ = g.run_batch("sssp", [0, 41])
            assert np.array_equal(rows[1], oracle.sssp(ptr, arr, 41))
            # more sources than the few-source path takes: lanes per source
            many = [0, 41] + list(range(100, 1400, 100))
            rows, _ = g.run_batch("sssp", many)
            for i in (0, 1, 7, len(many) - 1):
                assert np.array_equal(rows[i], oracle.sssp(ptr, arr, many[i])), (packed, many[i])


def test_cc_directed_is_min_ancestor():
    ptr, col = A.rmat_csr(12, 4, 14)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=0.3)) as g:
        got, _ = g.run("cc")
    assert np.array_equal(got, oracle.cc(ptr, col))


@pytest.mark.parametrize("frac", [1.0, 0.3, 0.0])
def test_pagerank_ref_and_std(frac):
    cptr, ccol, od = A.rmat_csr(13, 16, 15, transpose=True)
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=frac)) as g:
        got, st = g.run("pr")
        exp, it = oracle.pr_ref(cptr, ccol, od)
        assert np.abs(got - exp).max() <= PR_TOL
        exp, it, res = oracle.pr_std(cptr, ccol, od)
        for prec in (A.F64, A.F32):
            got, st = g.run("pr", params=A.make_params(pr_mode=A.PR_STD, precision=prec))
            err = np.abs(got.astype(np.float64) - exp).max()
            assert err <= PR_TOL, (prec, err)
            if prec == A.F64:
                assert st["iterations"] == it
            else:
                # exact sums of the FP32 contributions: the FP64 residual meets
                # the stop tolerance within a few passes of the FP64 run's
                assert st["residual"] < 1e-9 and st["iterations"] <= it + 10, (st["residual"], st["iterations"], it)


@pytest.mark.parametrize("weighted", [False, True])
def test_pagerank_scatter_on_out_edge_graphs(weighted):
    """CSR graphs (bcsr / bwcsr) run PageRank by scatter over out-edges; the
    values equal the oracle's on the transposed (in-edge) arrays."""
    ptr, col = A.rmat_csr(12, 16, 33)
    edges = A.rmat_csr(12, 16, 33, weights=(1, 63))[1] if weighted else col
    cptr, ccol, od = A.formats.transpose(ptr, col)
    with A.Graph.from_csr(ptr, edges, budget=A.make_budget(frac=0.25)) as g:
        got, _ = g.run("pr")
        assert np.abs(got - oracle.pr_ref(cptr, ccol, od)[0]).max() <= PR_TOL
        exp, it, _ = oracle.pr_std(cptr, ccol, od)
        for prec in (A.F64, A.F32):
            got, st = g.run("pr", params=A.make_params(pr_mode=A.PR_STD, precision=prec))
            assert np.abs(got.astype(np.float64) - exp).max() <= PR_TOL, prec
            assert st["residual"] < 1e-9 and st["iterations"] <= it + 10, (prec, st["residual"], st["iterations"], it)


@pytest.mark.parametrize("huge,seg,div,delta", [(32, 256, 1, 1), (64, 4096, 0, 0), (4096, 1024, 16, 64),
                                                (512, 2048, 2, 1000)])
def test_tunables_do_not_change_results(huge, seg, div, delta):
    ptr, adj = A.rmat_csr(13, 16, 34, weights=(1, 63))
    col = adj[:, 0].copy()
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(frac=0.3)) as g:
        g.set_tuning(huge_degree=huge, segment_edges=seg, dense_div=div, delta=delta)
        assert g.get_tuning()["huge_degree"] == huge
        for s in (0, 99):
            got, _ = g.run("bfs", s)
            assert np.array_equal(got, oracle.bfs(ptr, col, s))
            got, _ = g.run("sssp", s)
            assert np.array_equal(got, oracle.sssp(ptr, adj, s))
        got, _ = g.run_batch("bfs", [0, 99, 5])
        assert np.array_equal(got[1], oracle.bfs(ptr, col, 99))


def test_autotuner_picks_a_working_setting(tmp_path, monkeypatch):
    monkeypatch.setenv("ASC_TUNE_CACHE", str(tmp_path / "tune.txt"))
    ptr, col = A.rmat_csr(14, 16, 35)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=0.25)) as g:
        best = g.tune("bfs", [0, 5])
        assert best["ms"] > 0 and best["huge_degree"] >= 32
        got, _ = g.run("bfs", 5)
        assert np.array_equal(got, oracle.bfs(ptr, col, 5))
        again = g.tune("bfs", [0, 5])          # served from the cache
        assert again["ms"] == -1 and again["huge_degree"] == best["huge_degree"]


def test_huge_vertices_and_segments():
    """A star whose hub list is far above the segment threshold, mostly on demand."""
    V = 50000
    src = np.concatenate([np.zeros(V - 1, np.int64), np.arange(1, V), [7] * 3000])
    dst = np.concatenate([np.arange(1, V), np.zeros(V - 1, np.int64), np.arange(3000) + 100])
    ptr, col = A.formats.csr_from_edges(V, src, dst)
    for frac in (0.0, 0.02, 1.0):
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
            for s in (0, 5, 7):
                got, _ = g.run("bfs", s)
                assert np.array_equal(got, oracle.bfs(ptr, col, s)), (frac, s)
            got, _ = g.run("cc")
            assert np.array_equal(got, oracle.cc(ptr, col))


def test_file_formats_and_reference_entry_points():
    ptr, col = A.rmat_csr(11, 8, 16)
    _, adj = A.rmat_csr(11, 8, 16, weights=(1, 63))
    cptr, ccol, od = A.rmat_csr(11, 8, 16, transpose=True)
    d = tempfile.mkdtemp()
    files = {"g.bcsr": (A.FMT_BCSR, ptr, col, None), "g.bwcsr": (A.FMT_BWCSR, ptr, adj, None),
             "g.bcsc": (A.FMT_BCSC, cptr, ccol, od), "g.bcsr32": (A.FMT_BCSR32, ptr, col, None)}
    for name, (fmt, p, e, o) in files.items():
        A.write_graph(os.path.join(d, name), fmt, p, e, o)
    got, st = A.bfs_opt(os.path.join(d, "g.bcsr"), 3, 0.5)
    assert np.array_equal(got, oracle.bfs(ptr, col, 3))
    got, _ = A.sssp_opt(os.path.join(d, "g.bwcsr"), 3, 0.0)
    assert np.array_equal(got, oracle.sssp(ptr, adj, 3))
    got, _ = A.cc_opt(os.path.join(d, "g.bcsr"))
    assert np.array_equal(got, oracle.cc(ptr, col))
    got, _ = A.pr_opt(os.path.join(d, "g.bcsc"))
    assert np.abs(got - oracle.pr_ref(cptr, ccol, od)[0]).max() <= PR_TOL
    with A.Graph.open(os.path.join(d, "g.bcsr32"), budget=A.make_budget(frac=0.25)) as g:
        got, _ = g.run("bfs", 3)
        assert np.array_equal(got, oracle.bfs(ptr, col, 3))


def test_errors_are_statuses():
    ptr, col = A.rmat_csr(8, 4, 17)
    with A.Graph.from_csr(ptr, col) as g:
        with pytest.raises(A.AscError) as e:
            g.run("bfs", 1 << 20)
        assert e.value.status == A.ERR_INVALID
        with pytest.raises(A.AscError) as e:
            g.run("sssp", 0)
        assert e.value.status == A.ERR_UNSUPPORTED
    bad = col.copy()
    bad[5] = 1 << 20
    with pytest.raises(A.AscError) as e:
        A.Graph.from_csr(ptr, bad)
    assert e.value.status == A.ERR_INVALID or e.value.status == A.ERR_BAD_FILE


def test_iteration_cap_returns_timeout():
    V = 2000
    s = np.arange(V - 1)
    ptr, col = A.formats.csr_from_edges(V, s, s + 1)   # a chain: V-1 levels
    with A.Graph.from_csr(ptr, col) as g:
        for flags in (0, A.RUN_HOST_LOOP):
            with pytest.raises(A.AscError) as e:
                g.run("bfs", 0, params=A.make_params(max_iterations=10, flags=flags))
            assert e.value.status == A.ERR_TIMEOUT
            got, st = g.run("bfs", 0, params=A.make_params(flags=flags))
            assert got[-1] == V and st["iterations"] == V


def test_single_vertex_and_isolated_source():
    with A.Graph.from_csr(np.array([0, 1], np.uint64), np.array([0], np.uint32)) as g:
        got, _ = g.run("bfs", 0)
        assert got.tolist() == [1]
        got, _ = g.run("cc")
        assert got.tolist() == [0]
    ptr, col = A.formats.csr_from_edges(10, np.array([1, 2]), np.array([2, 3]))
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=0.0)) as g:
        got, st = g.run("bfs", 0)
        assert got.tolist() == [1] + [11] * 9
        assert st["reached_vertices"] == 1 and st["reached_edges"] == 0


def test_ptgraph_cli_matches_oracle():
    """The drop-in command line: reference flags, values written with --output."""
    import subprocess
    d = tempfile.mkdtemp()
    ptr, col = A.rmat_csr(12, 8, 37)
    _, adj = A.rmat_csr(12, 8, 37, weights=(1, 63))
    cptr, ccol, od = A.rmat_csr(12, 8, 37, transpose=True)
    A.write_graph(os.path.join(d, "g.bcsr"), A.FMT_BCSR, ptr, col)
    A.write_graph(os.path.join(d, "g.bwcsr"), A.FMT_BWCSR, ptr, adj)
    A.write_graph(os.path.join(d, "g.bcsc"), A.FMT_BCSC, cptr, ccol, od)
    cases = [("bfs", "g.bcsr", ["--source", "5"], oracle.bfs(ptr, col, 5)),
             ("sssp", "g.bwcsr", ["--source", "5"], oracle.sssp(ptr, adj, 5)),
             ("cc", "g.bcsr", [], oracle.cc(ptr, col)),
             ("pr", "g.bcsc", [], oracle.pr_ref(cptr, ccol, od)[0])]
    for algo, f, extra, exp in cases:
        out = os.path.join(d, algo + ".out")
        cmd = [A.PTGRAPH_PATH, "--input", os.path.join(d, f), "--type", algo, "--adviseK", "0.3",
               "--method", "1", "--output", out, "--json", "1"] + extra
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert "move overload size" in r.stdout
        got = np.fromfile(out, dtype=np.float64 if algo == "pr" else np.uint32)
        if algo == "pr":
            assert np.abs(got - exp).max() <= PR_TOL
        else:
            assert np.array_equal(got, exp), algo
    r = subprocess.run([A.PTGRAPH_PATH, "--input", os.path.join(d, "missing.bcsr")], capture_output=True, text=True)
    assert r.returncode == 2 and "bad graph file" in r.stderr


def test_managed_comparison_engine():
    """The UVM comparison engine (edges in managed memory, no static region)
    computes the same values as the split engine."""
    ptr, adj = A.rmat_csr(13, 16, 41, weights=(1, 63))
    col = adj[:, 0].copy()
    cptr, ccol, od = A.formats.transpose(ptr, col)
    with A.Graph.from_csr(ptr, adj, budget=A.make_budget(managed=True)) as g:
        assert g.info.static_edges == 0
        for s in (0, 77):
            for _ in range(2):  # first touch migrates pages; the second run reads them on the GPU
                got, _ = g.run("bfs", s)
                assert np.array_equal(got, oracle.bfs(ptr, col, s))
            got, _ = g.run("sssp", s)
            assert np.array_equal(got, oracle.sssp(ptr, adj, s))
        got, _ = g.run_batch("bfs", [0, 77])
        assert np.array_equal(got[1], oracle.bfs(ptr, col, 77))
    with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(managed=True)) as g:
        got, _ = g.run("pr")
        assert np.abs(got - oracle.pr_ref(cptr, ccol, od)[0]).max() <= PR_TOL


def test_converted_edge_list_runs(tmp_path):
    """asc-convert output opens in every layout and runs like the oracle on
    the edge list (CSR / CSC built by the oracle's converter restatement)."""
    import subprocess
    rng = np.random.default_rng(7)
    n, V = 20000, 3000
    src, dst = rng.integers(0, V, n), rng.integers(0, V, n)
    path = tmp_path / "g.txt"
    path.write_text("# edge list\n" + "\n".join("%d %d" % e for e in zip(src, dst)) + "\n")
    r = subprocess.run([A.CONVERT_PATH, str(path), "--to", "bcsr,bwcsr,bcsc,bcsr32"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    Vc, ptr, order, outdeg = oracle.converter(src, dst)
    col = dst.astype(np.uint32)[order]
    w = oracle.converter_ref_weights(n)[order]
    adj = np.stack([col, w], axis=1)
    _, cptr, corder, _ = oracle.converter(src, dst, by_dst=True)
    ccol = src.astype(np.uint32)[corder]
    stem = str(tmp_path / "g")
    for ext in ("bcsr", "bcsr32"):
        with A.Graph.open(stem + "." + ext, budget=A.make_budget(frac=0.3)) as g:
            got, _ = g.run("bfs", int(src[0]))
            assert np.array_equal(got, oracle.bfs(ptr, col, int(src[0])))
    with A.Graph.open(stem + ".bwcsr", budget=A.make_budget(frac=0.3)) as g:
        got, _ = g.run("sssp", int(src[0]))
        assert np.array_equal(got, oracle.sssp(ptr, adj, int(src[0])))
    with A.Graph.open(stem + ".bcsc", budget=A.make_budget(frac=0.3)) as g:
        got, _ = g.run("pr")
        assert np.abs(got - oracle.pr_ref(cptr, ccol, outdeg)[0]).max() <= PR_TOL


@pytest.mark.parametrize("frac", [0.25, 0.0, 1.0])
def test_bit_packed_edges_match_32_bit_edges(frac, monkeypatch):
    """Unweighted edges are stored as a bit stream of bits(max id) per edge
    (more static edges per budget byte, fewer link bytes); results equal the
    32-bit layout's and the oracle's."""
    ptr, col = A.rmat_csr(14, 16, 61)
    cptr, ccol, od = A.formats.transpose(ptr, col)
    sptr, scol = A.formats.symmetrize(ptr, col)
    runs = {}
    for packing in ("1", "0"):
        monkeypatch.setenv("ASC_EDGE_PACKING", packing)
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
            info = g.info
            assert info.edge_bits == (14 if packing == "1" else 32)
            out = {"static": info.static_edges}
            for s in (0, 1234):
                out["bfs", s] = g.run("bfs", s)[0]
            out["batch"] = g.run_batch("bfs", [0, 1234, 77])[0]
            out["pr_push"] = g.run("pr")[0]
        with A.Graph.from_csr(sptr, scol, budget=A.make_budget(frac=frac)) as g:
            out["cc"] = g.run("cc")[0]
        with A.Graph.from_csr(cptr, ccol, outdeg=od, budget=A.make_budget(frac=frac)) as g:
            out["pr"] = g.run("pr")[0]
            out["pr_std"] = g.run("pr", params=A.make_params(pr_mode=A.PR_STD, precision=A.F32))[0]
        runs[packing] = out
    p, u = runs["1"], runs["0"]
    if 0 < frac < 1:
        # the same budget bytes hold 32/14 times the edges (down to whole fragments)
        assert p["static"] > 2 * u["static"]
    for s in (0, 1234):
        exp = oracle.bfs(ptr, col, s)
        assert np.array_equal(p["bfs", s], exp) and np.array_equal(u["bfs", s], exp)
    assert np.array_equal(p["batch"][1], oracle.bfs(ptr, col, 1234))
    assert np.array_equal(p["cc"], oracle.cc(sptr, scol)) and np.array_equal(u["cc"], p["cc"])
    ref = oracle.pr_ref(cptr, ccol, od)[0]
    assert np.abs(p["pr"] - ref).max() <= PR_TOL and np.abs(p["pr_push"] - ref).max() <= PR_TOL
    std = oracle.pr_std(cptr, ccol, od)[0]
    assert np.abs(p["pr_std"].astype(np.float64) - std).max() <= PR_TOL


@pytest.mark.parametrize("V", [2, 3, 5, 33, 1000, 70000, (1 << 20) + 3])
def test_bit_stream_widths(V):
    """Bit streams of every width class (1 bit for ids {0, 1} up to 21 bits),
    with edges straddling word boundaries, split at several budgets."""
    rng = np.random.default_rng(V)
    E = min(40 * V, 400000)
    src = np.sort(rng.integers(0, V, E))
    dst = rng.integers(0, V, E)
    dst[-1] = V - 1  # the widest id is present
    ptr, col = A.formats.csr_from_edges(V, src, dst)
    bits = max(1, int(V - 1).bit_length())
    for frac in (0.0, 0.3, 1.0):
        with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
            assert g.info.edge_bits == bits
            for s in (0, V - 1, V // 2):
                got, _ = g.run("bfs", s)
                assert np.array_equal(got, oracle.bfs(ptr, col, s)), (V, frac, s)
            got, _ = g.run("cc")
            assert np.array_equal(got, oracle.cc(ptr, col)), (V, frac)


def test_link_probe_runs():
    """The run-length link probe measures a positive rate and rejects bad sizes."""
    assert A.link_probe_runs(64, nbytes=4 << 20, iters=1) > 0
    assert A.link_probe_runs(4096, nbytes=4 << 20, iters=1) > 0
    for bad in (2, 6, 1 << 20):
        with pytest.raises(A.AscError):
            A.link_probe_runs(bad, nbytes=4 << 20, iters=1)


def test_fragment_counts_add_up():
    """Per-fragment read counters sum to the edges the runs processed, and
    counting leaves the values unchanged."""
    ptr, col = A.rmat_csr(13, 16, 71)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=0.3)) as g:
        prm = A.make_params(flags=A.RUN_FRAGMENT_COUNTS)
        total = 0
        for s in (0, 5):
            got, st = g.run("bfs", s, params=prm)
            assert np.array_equal(got, oracle.bfs(ptr, col, s))
            total += st["edges_processed"]
        got, st = g.run("cc", params=prm)
        total += st["edges_processed"]
        c = g.fragment_counts(reset=True)
        assert len(c) == (g.E + 4095) // 4096 and int(c.sum()) == total
        assert g.fragment_counts().sum() == 0  # the reset cleared them
        g.run("bfs", 0)  # without the flag nothing is counted
        assert g.fragment_counts().sum() == 0


def test_pinned_result_buffer():
    """asc_run fills a page-locked buffer from asc_host_alloc like any other."""
    ptr, col = A.rmat_csr(12, 16, 81)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=0.3)) as g:
        buf = A.PinnedArray(g.V, np.uint32)
        for s in (0, 9):
            g.run("bfs", s, out=buf.array)
            assert np.array_equal(buf.array, oracle.bfs(ptr, col, s))
        buf.close()


def test_graph_without_edges():
    """A graph with vertices and no edges: every source reaches only itself."""
    V = 5
    ptr = np.zeros(V + 1, np.uint64)
    with A.Graph.from_csr(ptr, np.zeros(0, np.uint32), budget=A.make_budget(frac=0.25)) as g:
        got, st = g.run("bfs", 2)
        assert got.tolist() == [V + 1, V + 1, 1, V + 1, V + 1] and st["reached_edges"] == 0
        got, _ = g.run("cc")
        assert got.tolist() == list(range(V))
        rows, _ = g.run_batch("bfs", [0, 4])
        assert rows[1].tolist() == [V + 1] * 4 + [1]
    with A.Graph.from_csr(ptr, np.zeros((0, 2), np.uint32)) as g:
        got, _ = g.run("sssp", 3)
        assert got.tolist() == [V + 1, V + 1, V + 1, 1, V + 1]


@pytest.mark.parametrize("frac", [0.0, 0.3])
def test_gather_copy_engine_matches(frac):
    """The gather-and-copy comparison engine (on-demand edges gathered on the
    host and copied each iteration) gives the same values, for every stored
    layout: bit stream, packed weighted words, {dst, weight} pairs."""
    ptr, adj = A.rmat_csr(13, 16, 91, weights=(1, 63))
    col = adj[:, 0].copy()
    big = adj.copy()
    big[:, 1] = (big[:, 1].astype(np.uint64) * 40000).astype(np.uint32)   # too wide to pack: pairs
    gat = A.make_params(flags=A.RUN_GATHER_COPY)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(frac=frac)) as g:
        for s in (0, 321):
            got, st = g.run("bfs", s, params=gat)
            assert np.array_equal(got, oracle.bfs(ptr, col, s))
            if frac == 0.0 and st["reached_vertices"] > 1000:
                assert st["ondemand_edges"] > 0
        got, _ = g.run("cc", params=gat)
        assert np.array_equal(got, oracle.cc(ptr, col))
    for arr in (adj, big):
        with A.Graph.from_csr(ptr, arr, budget=A.make_budget(frac=frac)) as g:
            for s in (0, 321):
                got, _ = g.run("sssp", s, params=gat)
                assert np.array_equal(got, oracle.sssp(ptr, arr, s))


@pytest.mark.parametrize("frac", [0.25, 0.1, 0.0])
@pytest.mark.parametrize("layout", ["csc", "csr", "csr_weighted"])
def test_staged_pagerank_equals_zero_copy(frac, layout):
    """Standard PageRank on a graph with staging buffers copies the on-demand
    edges in chunks every pass (two 8 KiB buffers here: 10 to 26 chunks, long
    lists cut between chunks); the ranks equal the zero-copy run's and the
    oracle's, and the buffers come out of the byte budget."""
    ptr, col = A.rmat_csr(13, 16, 71)
    cptr, ccol, od = A.formats.transpose(ptr, col)
    exp, it, _ = oracle.pr_std(cptr, ccol, od)
    if layout == "csc":
        args = (cptr, ccol)
        kw = {"outdeg": od}
    elif layout == "csr":
        args, kw = (ptr, col), {}
    else:
        args, kw = (ptr, A.rmat_csr(13, 16, 71, weights=(1, 63))[1]), {}
    stage = 16 << 10
    # a zero budget holds no staging either: every edge is then read in place
    budget = A.make_budget(frac=frac, stage_bytes=stage) if frac else A.make_budget(nbytes=stage,
                                                                                   stage_bytes=stage)
    file_bytes = 8 if layout == "csr_weighted" else 4
    with A.Graph.from_csr(*args, budget=budget, **kw) as g:
        info = g.info
        assert info.staging_bytes == stage and (info.static_edges == 0 or frac)
        assert info.device_edge_bytes <= max(frac * g.E * file_bytes, stage) + 8
        for tuning in ({}, {"huge_degree": 32, "segment_edges": 256}):
            if tuning:
                g.set_tuning(**tuning)
            for prec in (A.F32, A.F64):
                zc, st0 = g.run("pr", params=A.make_params(pr_mode=A.PR_STD, precision=prec,
                                                            flags=A.RUN_NO_STAGING))
                got, st = g.run("pr", params=A.make_params(pr_mode=A.PR_STD, precision=prec))
                assert st0["staged_chunks"] == 0 and st["staged_chunks"] >= 5 * st["iterations"], st
                assert np.abs(got.astype(np.float64) - exp).max() <= PR_TOL, (prec, tuning)
                # FP32 partials are summed in FP32 within a warp, so tiles cut
                # at other vertices round differently (relative 1e-7 level)
                rel = np.abs(got.astype(np.float64) - zc.astype(np.float64)) / exp
                assert rel.max() <= (1e-5 if prec == A.F32 else 1e-12), (prec, tuning, rel.max())
                assert abs(st["iterations"] - st0["iterations"]) <= 5
                assert st["residual"] < 1e-9


@pytest.mark.parametrize("frac", [1.0, 0.25, 0.0])
@pytest.mark.parametrize("bu_div", [0, 16, 1 << 30])
def test_bottom_up_bfs_levels_equal_top_down(frac, bu_div):
    """Direction-optimizing BFS: iterations whose frontier holds more than
    V / bu_div vertices step bottom-up over the in-edges (1 << 30: every
    iteration, the first included; 0: never). Levels equal the oracle's under
    the CUDA-graph loop and the host loop, on plain and weighted graphs."""
    ptr, col = A.rmat_csr(14, 16, 81)
    _, adj = A.rmat_csr(14, 16, 81, weights=(1, 63))
    deg = np.diff(ptr)
    srcs = [0, int(np.nonzero(deg)[0][-1]), int(np.nonzero(deg == 0)[0][0])]
    for edges in (col, adj):
        with A.Graph.from_csr(ptr, edges, budget=A.make_budget(frac=frac)) as g:
            g.set_tuning(bu_div=bu_div)
            assert g.get_tuning()["bu_div"] == bu_div
            for s in srcs:
                exp = oracle.bfs(ptr, col, s)
                for flags in (0, A.RUN_HOST_LOOP):
                    got, st = g.run("bfs", s, params=A.make_params(flags=flags))
                    assert np.array_equal(got, exp), (frac, bu_div, s, flags)
                    assert st["reached_edges"] == oracle.reached_edges(ptr, exp, len(ptr))
                    assert st["reached_vertices"] == int((exp != len(ptr)).sum())


@pytest.mark.parametrize("frac", [0.25, 0.0])
def test_partition_copy_engine_matches(frac):
    """The whole-partition comparison engine (the reference's baseline: every
    partition holding a frontier vertex copied whole each iteration) gives the
    oracle's values; with a zero budget it is the reference's configuration
    (every edge in partitions, no static region)."""
    stage = 64 << 10
    mk = (lambda: A.make_budget(frac=frac, stage_bytes=stage)) if frac else \
        (lambda: A.make_budget(nbytes=stage, stage_bytes=stage))
    prm = A.make_params(flags=A.RUN_PARTITION_COPY)
    ptr, adj = A.rmat_csr(13, 16, 91, weights=(1, 63))
    col = adj[:, 0].copy()
    sptr, scol = A.formats.symmetrize(ptr, col)
    with A.Graph.from_csr(ptr, col, budget=mk()) as g:
        assert g.info.staging_bytes == stage and (frac or g.info.static_edges == 0)
        for s in (0, 1000):
            got, st = g.run("bfs", s, params=prm)
            assert np.array_equal(got, oracle.bfs(ptr, col, s)), s
            assert st["staged_chunks"] > 0 and st["ondemand_bytes"] > 0
    with A.Graph.from_csr(ptr, adj, budget=mk()) as g:
        got, _ = g.run("sssp", 5, params=prm)
        assert np.array_equal(got, oracle.sssp(ptr, adj, 5))
    with A.Graph.from_csr(sptr, scol, budget=mk()) as g:
        got, _ = g.run("cc", params=prm)
        assert np.array_equal(got, oracle.cc(sptr, scol))


def test_partition_copy_rejects_a_list_longer_than_a_partition():
    V = 12000
    ptr = np.zeros(V + 1, np.uint64)
    ptr[1:] = V - 1                     # vertex 0 points at every other vertex
    col = np.arange(1, V, dtype=np.uint32)
    with A.Graph.from_csr(ptr, col, budget=A.make_budget(nbytes=8 << 10, stage_bytes=8 << 10)) as g:
        with pytest.raises(A.AscError) as e:
            g.run("bfs", 0, params=A.make_params(flags=A.RUN_PARTITION_COPY))
        assert e.value.status == A.ERR_BUDGET
