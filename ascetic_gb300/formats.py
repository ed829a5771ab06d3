"""Reader and writer for the reference's binary graph files (host side, numpy).

Layouts (GraphMeta.cuh:151-171 reads them; converter/converter.cpp:77-420 writes them):

* ``.bcsr``   u64 V, u64 E, u64 ptr[V], u32 col[E]
* ``.bwcsr``  u64 V, u64 E, u64 ptr[V], {u32 dst, u32 weight}[E]
* ``.bcsc``   u64 V, u64 E, u32 outDeg[V], u64 ptr[V], u32 src[E] (in-edges)
* ``.bcsr32`` u32 V, u32 E, u32 ptr[V], u32 col[E]  (legacy layout, bfs.cu:14-23)

Only V row offsets are stored; in memory we keep V+1 with ptr[V] = E, which
gives the reference's degree rule deg[V-1] = E - ptr[V-1] (GraphMeta.cuh:216-226).
The C++ library reads the same files natively (asc_graph_open); this module is
for tools and tests that build small graphs in Python.
"""
from __future__ import annotations

import numpy as np

FMT_AUTO, FMT_BCSR, FMT_BWCSR, FMT_BCSC, FMT_BCSR32 = 0, 1, 2, 3, 4


def csr_from_edges(V, src, dst, weights=None):
    """Stable counting sort of an edge list by source: returns ptr (V+1, u64)
    and col (u32) or adj ((E, 2) u32 with dst, weight). Each vertex keeps its
    edges in input order; self-loops and duplicates are kept."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.uint32)
    order = np.argsort(src, kind="stable")
    counts = np.bincount(src, minlength=V) if len(src) else np.zeros(V, np.int64)
    ptr = np.zeros(V + 1, np.uint64)
    ptr[1:] = np.cumsum(counts, dtype=np.uint64)
    if weights is None:
        return ptr, dst[order]
    adj = np.empty((len(src), 2), np.uint32)
    adj[:, 0] = dst[order]
    adj[:, 1] = np.asarray(weights, dtype=np.uint32)[order]
    return ptr, adj


def transpose(ptr, col):
    """CSC (in-edge) arrays of a CSR graph, and the out-degree of each vertex.
    In-edges of v are ordered by source id, then by position in the source's list."""
    ptr = np.asarray(ptr, dtype=np.uint64)
    V = len(ptr) - 1
    deg = np.diff(ptr).astype(np.int64)
    srcs = np.repeat(np.arange(V, dtype=np.uint32), deg)
    cptr, ccol = csr_from_edges(V, np.asarray(col, dtype=np.int64), srcs)
    return cptr, ccol, deg.astype(np.uint32)


def symmetrize(ptr, col):
    """Adds the reverse of every edge: the list is all original edges in CSR
    order followed by all reversed edges, stably sorted by source."""
    ptr = np.asarray(ptr, dtype=np.uint64)
    V = len(ptr) - 1
    deg = np.diff(ptr).astype(np.int64)
    s = np.repeat(np.arange(V, dtype=np.int64), deg)
    d = np.asarray(col, dtype=np.int64)
    return csr_from_edges(V, np.concatenate([s, d]), np.concatenate([d, s]))


def write_bcsr(path, ptr, col):
    ptr = np.asarray(ptr, dtype=np.uint64)
    V = len(ptr) - 1
    with open(path, "wb") as f:
        np.array([V, ptr[-1]], dtype=np.uint64).tofile(f)
        ptr[:V].tofile(f)
        np.asarray(col, dtype=np.uint32).tofile(f)


def write_bwcsr(path, ptr, adj):
    ptr = np.asarray(ptr, dtype=np.uint64)
    V = len(ptr) - 1
    with open(path, "wb") as f:
        np.array([V, ptr[-1]], dtype=np.uint64).tofile(f)
        ptr[:V].tofile(f)
        np.asarray(adj, dtype=np.uint32).reshape(-1).tofile(f)


def write_bcsc(path, cptr, ccol, outdeg):
    cptr = np.asarray(cptr, dtype=np.uint64)
    V = len(cptr) - 1
    with open(path, "wb") as f:
        np.array([V, cptr[-1]], dtype=np.uint64).tofile(f)
        np.asarray(outdeg, dtype=np.uint32).tofile(f)
        cptr[:V].tofile(f)
        np.asarray(ccol, dtype=np.uint32).tofile(f)


def write_bcsr32(path, ptr, col):
    ptr = np.asarray(ptr, dtype=np.uint64)
    V = len(ptr) - 1
    with open(path, "wb") as f:
        np.array([V, ptr[-1]], dtype=np.uint32).tofile(f)
        ptr[:V].astype(np.uint32).tofile(f)
        np.asarray(col, dtype=np.uint32).tofile(f)


def read(path, fmt=FMT_BCSR):
    """Returns a dict with ptr (V+1, u64) and col / adj / (col, outdeg)."""
    raw = np.fromfile(path, dtype=np.uint8)
    if fmt == FMT_BCSR32:
        V, E = (int(x) for x in raw[:8].view(np.uint32))
        off = 8
        ptr = np.empty(V + 1, np.uint64)
        ptr[:V] = raw[off:off + 4 * V].view(np.uint32)
        ptr[V] = E
        off += 4 * V
        return {"ptr": ptr, "col": raw[off:off + 4 * E].view(np.uint32).copy()}
    V, E = (int(x) for x in raw[:16].view(np.uint64))
    off = 16
    out = {}
    if fmt == FMT_BCSC:
        out["outdeg"] = raw[off:off + 4 * V].view(np.uint32).copy()
        off += 4 * V
    ptr = np.empty(V + 1, np.uint64)
    ptr[:V] = raw[off:off + 8 * V].view(np.uint64)
    ptr[V] = E
    off += 8 * V
    out["ptr"] = ptr
    if fmt == FMT_BWCSR:
        out["adj"] = raw[off:off + 8 * E].view(np.uint32).reshape(E, 2).copy()
    else:
        out["col"] = raw[off:off + 4 * E].view(np.uint32).copy()
    return out
