"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs the reference emulation library (oracle/_ref/libascref.so: the reference's
own gpu_kernels.cuh kernels and GraphMeta.cuh budget/gather/partition code,
compiled for the CPU by oracle/refemu/Makefile from the reference tree) on small
graphs written in the reference's file formats, and stores its result arrays.

Each graph goes into <name>.npz (graph arrays plus one result array per run);
manifest.json lists the runs. For every run two results are stored:

* ``<key>``       the reference with staticNodePointer[max_static_node] set to
                  its intended value (hazard_mode 1): what the oracle and the
                  CUDA engine must reproduce bit for bit;
* ``<key>_asis``  the reference as it behaves on real inputs, where that entry
                  stays zero (hazard_mode 0, GraphMeta.cuh:230-233).

Usage (needs the reference tree, so it runs only where the fixtures are made):
    make -C oracle/refemu REF=<reference tree> && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ascetic_gb300 import formats as F  # noqa: E402

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libascref.so")


class RefStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("max_static_node", ctypes.c_uint32),
                ("static_edges", ctypes.c_uint64), ("staging_edges", ctypes.c_uint64),
                ("moved_edges", ctypes.c_uint64), ("node_sum", ctypes.c_uint64),
                ("parts", ctypes.c_uint64)]


def load_ref():
    lib = ctypes.CDLL(REF_LIB)
    lib.asc_ref_run.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint64,
                                ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                ctypes.POINTER(RefStats)]
    lib.asc_ref_run.restype = ctypes.c_int
    return lib


PARAM_SIZE = {0: 13, 1: 15, 2: 13, 3: 17}   # CalculateOpt.cu:20, :215, :388, :553
EDGE_BYTES = {0: 4, 1: 8, 2: 4, 3: 4}


def ref_run(lib, algo, path, V, source, static_edges, staging_edges, hazard_mode):
    """Sizes cudaMemGetInfo and --adviseK so that the reference's own
    getMaxPartitionSize (GraphMeta.cuh:310-372) picks static_edges for the
    static prefix and staging_edges for the on-demand buffer."""
    total = static_edges + staging_edges
    avail = PARAM_SIZE[algo] * 4 * V + total * EDGE_BYTES[algo]
    advise = static_edges / total if static_edges else 1e-9
    out = np.zeros(max(V, 1), np.float64 if algo == 3 else np.uint32)
    st = RefStats()
    rc = lib.asc_ref_run(algo, path.encode(), source, avail, advise, hazard_mode,
                         out.ctypes.data, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("reference run failed rc=%d" % rc)
    return out[:V], st


def rmat_edges(scale, ef, seed, a=0.57, b=0.19, c=0.19):
    rng = np.random.default_rng(seed)
    V = 1 << scale
    E = V * ef
    src = np.zeros(E, np.int64)
    dst = np.zeros(E, np.int64)
    for _ in range(scale):
        u = rng.random(E)
        sb = (u >= a + b).astype(np.int64)
        db = (((u >= a) & (u < a + b)) | (u >= a + b + c)).astype(np.int64)
        src = src * 2 + sb
        dst = dst * 2 + db
    w = rng.integers(1, 64, size=E)
    return V, src, dst, w


def edge_case_graphs():
    """Small hand-built graphs covering the edge cases of the reference path."""
    g = {}
    # chain 0->1->...->99 with a long weighted tail
    V = 100
    s = np.arange(V - 1)
    g["chain"] = (V, s, s + 1, np.full(V - 1, 63))
    # star: hub 0 to all, plus spokes back; self-loops and duplicate edges
    V = 300
    s = np.concatenate([np.zeros(V - 1, np.int64), np.arange(1, V), [5, 5, 5, 7, 7]])
    d = np.concatenate([np.arange(1, V), np.zeros(V - 1, np.int64), [5, 5, 9, 7, 8]])
    g["star_loops_dups"] = (V, s, d, (np.arange(len(s)) % 63) + 1)
    # zero-degree head and tail vertices (vertex 0 at offset 0 with degree 0,
    # which the reference's u64 static test wraps), an isolated middle vertex
    V = 64
    s = np.array([3, 3, 4, 5, 6, 10, 10, 11, 40, 41, 41, 50])
    d = np.array([4, 5, 6, 6, 3, 11, 12, 13, 41, 40, 50, 3])
    g["zero_degree_ends"] = (V, s, d, np.array([1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12]))
    # two components with a one-way bridge (directed CC = min ancestor id)
    V = 40
    s = np.array([30, 31, 32, 33, 5, 6, 7, 31])
    d = np.array([31, 32, 33, 30, 6, 7, 5, 6])
    g["oneway_bridge"] = (V, s, d, np.array([2, 2, 2, 2, 1, 1, 1, 9]))
    # a single vertex with a self-loop
    g["single"] = (1, np.array([0]), np.array([0]), np.array([1]))
    return g


def main():
    if not os.path.exists(REF_LIB):
        sys.exit("build the reference emulation first: make -C oracle/refemu REF=<reference tree>")
    lib = load_ref()
    tmp = tempfile.mkdtemp()
    manifest = {"graphs": {}}
    graphs = {}
    for scale, ef, seed in [(10, 16, 1), (11, 8, 2)]:
        graphs["rmat_s%d_ef%d_seed%d" % (scale, ef, seed)] = rmat_edges(scale, ef, seed)
    graphs.update(edge_case_graphs())

    for name, (V, src, dst, w) in graphs.items():
        arrays = {}
        runs = []
        ptr, col = F.csr_from_edges(V, src, dst)
        _, adj = F.csr_from_edges(V, src, dst, w)
        sptr, scol = F.symmetrize(ptr, col)
        cptr, ccol, outdeg = F.transpose(ptr, col)
        arrays.update(ptr=ptr, col=col, adj=adj, sptr=sptr, scol=scol, cptr=cptr, ccol=ccol,
                      outdeg=outdeg)
        files = {}
        for key, writer, args in [("bcsr", F.write_bcsr, (ptr, col)), ("bwcsr", F.write_bwcsr, (ptr, adj)),
                                  ("sym", F.write_bcsr, (sptr, scol)),
                                  ("bcsc", F.write_bcsc, (cptr, ccol, outdeg))]:
            files[key] = os.path.join(tmp, "%s.%s" % (name, key))
            writer(files[key], *args)
        E = int(ptr[-1])
        deg = np.diff(ptr)
        nz = np.nonzero(deg)[0]
        rng = np.random.default_rng(7)
        sources = sorted(set([0] + [int(x) for x in rng.choice(nz, size=min(3, len(nz)), replace=False)]))
        if name == "zero_degree_ends":
            sources = [0, 3, 40]          # 0 has no out-edges
        splits = sorted(set([0, 4096, 8192, ((E + 4095) // 4096) * 4096]))
        for algo, aname, fkey, srcs in [(0, "bfs", "bcsr", sources), (1, "sssp", "bwcsr", sources[:2]),
                                        (2, "cc", "sym", [0]), (3, "pr_ref", "bcsc", [0])]:
            e_alg = E * (2 if algo == 2 else 1)
            for s in srcs:
                for st_edges in splits:
                    if st_edges > ((e_alg + 4095) // 4096) * 4096:
                        continue
                    staging = max(4096, ((e_alg + 4095) // 4096) * 4096)
                    for staging_edges in sorted(set([staging, 4096])):
                        key = "%s_s%d_st%d_sg%d" % (aname, s, st_edges, staging_edges)
                        try:
                            good, st = ref_run(lib, algo, files[fkey], V, s, st_edges, staging_edges, 1)
                            asis, _ = ref_run(lib, algo, files[fkey], V, s, st_edges, staging_edges, 0)
                        except RuntimeError:
                            continue       # planner would not terminate for this staging size
                        arrays[key] = good
                        arrays[key + "_asis"] = asis
                        runs.append({"key": key, "algo": aname, "source": s, "static_edges": st_edges,
                                     "staging_edges": staging_edges, "iterations": st.iterations,
                                     "moved_edges": int(st.moved_edges), "parts": int(st.parts),
                                     "ref_static_edges": int(st.static_edges),
                                     "max_static_node": int(st.max_static_node),
                                     "asis_differs": int((asis != good).sum())})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        manifest["graphs"][name] = {"V": int(V), "E": E, "runs": runs}
        print(name, "V=%d E=%d runs=%d" % (V, E, len(runs)))
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
