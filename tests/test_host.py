"""Host-side checks that need no GPU: the C-ABI library loads and exports every
declared symbol, the RMAT generator is deterministic and well formed, file
round trips, and the command line exists. No compute call reaches a GPU."""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import ascetic_gb300 as A
from ascetic_gb300 import formats as F

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not os.path.exists(A.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()


def test_header_symbols_are_exported():
    hdr = open(os.path.join(ROOT, "include", "ascetic.h")).read()
    declared = set(re.findall(r"^(?:const\s+)?\w+\s*\*?\s*(asc_\w+)\(", hdr, re.M))
    assert declared == set(A.EXPORTED)
    L = A.lib()
    for name in declared:
        assert hasattr(L, name), name
    assert b"sm_103a" in L.asc_version()
    assert L.asc_status_string(A.ERR_BUDGET) == b"device budget exceeded"


def test_rmat_is_deterministic_and_well_formed():
    p1, c1 = A.rmat_csr(12, 8, 5)
    p2, c2 = A.rmat_csr(12, 8, 5)
    assert np.array_equal(p1, p2) and np.array_equal(c1, c2)
    V = 1 << 12
    assert len(p1) == V + 1 and p1[-1] == V * 8
    assert (np.diff(p1.astype(np.int64)) >= 0).all() and (c1 < V).all()
    deg = np.diff(p1)
    assert deg[0] == deg.max()            # a=.57: vertex 0 is the top hub
    p3, c3 = A.rmat_csr(12, 8, 6)
    assert not np.array_equal(c1, c3)


def test_rmat_weights_symmetric_transpose_agree():
    p, c = A.rmat_csr(10, 16, 3)
    pw, adj = A.rmat_csr(10, 16, 3, weights=(1, 63))
    assert np.array_equal(p, pw) and np.array_equal(adj[:, 0], c)
    assert adj[:, 1].min() >= 1 and adj[:, 1].max() <= 63
    ps, cs = A.rmat_csr(10, 16, 3, symmetric=True)
    sp, sc = F.symmetrize(p, c)
    assert np.array_equal(ps, sp)
    for v in range(0, 1024, 7):
        assert sorted(cs[ps[v]:ps[v + 1]]) == sorted(sc[sp[v]:sp[v + 1]])
    pc, cc, od = A.rmat_csr(10, 16, 3, transpose=True)
    tp, tc, tod = F.transpose(p, c)
    assert np.array_equal(pc, tp) and np.array_equal(od, tod)
    for v in range(0, 1024, 7):
        assert sorted(cc[pc[v]:pc[v + 1]]) == sorted(tc[tp[v]:tp[v + 1]])


@pytest.mark.parametrize("fmt", [A.FMT_BCSR, A.FMT_BWCSR, A.FMT_BCSC, A.FMT_BCSR32])
def test_write_and_read_back(fmt):
    d = tempfile.mkdtemp()
    path = os.path.join(d, "g")
    if fmt == A.FMT_BWCSR:
        p, e = A.rmat_csr(9, 4, 1, weights=(1, 63))
        A.write_graph(path, fmt, p, e)
        back = F.read(path, fmt)
        assert np.array_equal(back["adj"], e)
    elif fmt == A.FMT_BCSC:
        p, e, od = A.rmat_csr(9, 4, 1, transpose=True)
        A.write_graph(path, fmt, p, e, od)
        back = F.read(path, fmt)
        assert np.array_equal(back["col"], e) and np.array_equal(back["outdeg"], od)
    else:
        p, e = A.rmat_csr(9, 4, 1)
        A.write_graph(path, fmt, p, e)
        back = F.read(path, fmt)
        assert np.array_equal(back["col"], e)
    assert np.array_equal(back["ptr"], p)


def test_graph_calls_without_a_device_return_a_status():
    if A.device_count() > 0:
        pytest.skip("a GPU is present")
    p, c = A.rmat_csr(6, 4, 1)
    with pytest.raises(A.AscError) as e:
        A.Graph.from_csr(p, c)
    assert e.value.status == A.ERR_NO_DEVICE


def test_invalid_generator_arguments():
    with pytest.raises(A.AscError) as e:
        A.rmat_csr(0, 4, 1)
    assert e.value.status == A.ERR_INVALID
    with pytest.raises(A.AscError):
        A.rmat_csr(8, 4, 1, a=0.9, b=0.2, c=0.1)


def test_ptgraph_cli_prints_usage():
    r = subprocess.run([A.PTGRAPH_PATH], capture_output=True, text=True)
    assert r.returncode == 1 and "usage: ptgraph" in r.stderr


def _write_small(path, fmt):
    p, e = A.rmat_csr(8, 4, 9)
    A.write_graph(path, fmt, p, e)
    return p, e


def test_malformed_files_are_rejected_before_any_device_work():
    """A short file, a header that matches no layout, and an ambiguous size all
    return ASC_ERR_BAD_FILE (checked on the host, no GPU needed)."""
    d = tempfile.mkdtemp()
    path = os.path.join(d, "g.bcsr")
    _write_small(path, A.FMT_BCSR)
    raw = open(path, "rb").read()
    for name, data in [("short.bcsr", raw[:-40]), ("tiny.bcsr", raw[:6]), ("junk.bcsr", b"\xff" * 64)]:
        bad = os.path.join(d, name)
        open(bad, "wb").write(data)
        with pytest.raises(A.AscError) as e:
            A.Graph.open(bad)
        assert e.value.status == A.ERR_BAD_FILE, name
    # explicit layout that does not match the size
    with pytest.raises(A.AscError) as e:
        A.Graph.open(path, fmt=A.FMT_BWCSR)
    assert e.value.status == A.ERR_BAD_FILE
    with pytest.raises(A.AscError) as e:
        A.Graph.open(os.path.join(d, "missing.bcsr"))
    assert e.value.status == A.ERR_BAD_FILE


def _replica_worker(rank, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": "2", "LOCAL_RANK": str(rank), "CUDA_VISIBLE_DEVICES": "4,5"})
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.replica_setup()
    bench.replica_barrier(w)
    edges, secs = bench.replica_reduce(1000 * (rank + 1), 0.5 + rank, w)
    q.put((r, w, edges, secs, os.environ["CUDA_VISIBLE_DEVICES"]))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_bench_replicas_gloo_world2():
    """bench.py under torchrun runs one replica per GPU: a gloo group gives the
    barrier, whole-job edges (sum) and time (slowest replica). Two CPU ranks."""
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:4] for r in res] == [(0, 2, 3000.0, 1.5), (1, 2, 3000.0, 1.5)]
    assert [r[4] for r in res] == ["4", "5"]   # one device per replica, by local rank


def test_bench_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` runs the reference's frontier/atomic-min
    scheme on the host cores (no GPU) and prints one JSON line with the
    reference-arm keys."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "12",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GTEPS" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["scale"] == 12
