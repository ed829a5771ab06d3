"""CPU oracle for the out-of-GPU-memory iteration engine (test infrastructure).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` import it.
It wraps ``oracle.c`` (a plain-C restatement of what the reference computes on
its hot path) through ctypes, and, where it was built, the reference emulation
library ``oracle/_ref/libascref.so`` (the reference's own ``gpu_kernels.cuh`` and
``GraphMeta.cuh`` compiled for the CPU; see ``oracle/refemu``).

Every graph here is given as numpy arrays: ``ptr`` (uint64, V+1 entries with
ptr[V] = E) and ``col`` (uint32 destinations) or ``adj`` (uint32 pairs
dst, weight).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB_PATH = os.path.join(REF_DIR, "libascref.so")

_lib = None
_ref = None

_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (gcc, no GPU needed)."""
    src = os.path.join(HERE, "oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(LIB_PATH)
    u64 = ctypes.c_uint64
    u32 = ctypes.c_uint32
    i32p = ctypes.POINTER(ctypes.c_int32)
    lib.orc_bfs.argtypes = [u64, _u64p, _u32p, u32, _u32p]
    lib.orc_sssp.argtypes = [u64, _u64p, _u32p, u32, _u32p]
    lib.orc_cc.argtypes = [u64, _u64p, _u32p, _u32p]
    lib.orc_pr_ref.argtypes = [u64, _u64p, _u32p, _u32p, _f64p, i32p]
    lib.orc_pr_std.argtypes = [u64, _u64p, _u32p, _u32p, ctypes.c_double, ctypes.c_double,
                               ctypes.c_int32, _f64p, i32p, ctypes.POINTER(ctypes.c_double)]
    lib.orc_pr_std_mt.argtypes = [u64, _u64p, _u32p, _u32p, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int32, ctypes.c_int, _f64p, i32p, ctypes.POINTER(ctypes.c_double)]
    lib.orc_static_split.argtypes = [u64, _u64p, u64, _u8p, ctypes.POINTER(u64), ctypes.POINTER(u64)]
    lib.orc_reached_edges.argtypes = [u64, _u64p, _u32p, u32]
    lib.orc_reached_edges.restype = u64
    lib.orc_relax_mt.argtypes = [ctypes.c_int, u64, _u64p, _u32p, u32, ctypes.c_int, _u32p, i32p]
    for f in ("orc_bfs", "orc_sssp", "orc_cc", "orc_pr_ref", "orc_pr_std", "orc_pr_std_mt", "orc_static_split",
              "orc_relax_mt"):
        getattr(lib, f).restype = ctypes.c_int
    _lib = lib
    return lib


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed with code %d" % (what, rc))


def _ptr(ptr):
    return np.ascontiguousarray(ptr, dtype=np.uint64)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def bfs(ptr, col, src):
    ptr, col = _ptr(ptr), _u32(col)
    V = len(ptr) - 1
    out = np.empty(V, np.uint32)
    _check(_load().orc_bfs(V, ptr, col if len(col) else np.zeros(1, np.uint32), src, out), "bfs")
    return out


def sssp(ptr, adj, src):
    """adj: uint32 array of 2E entries (dst, weight) or an (E, 2) array."""
    ptr, adj = _ptr(ptr), _u32(np.asarray(adj).reshape(-1))
    V = len(ptr) - 1
    out = np.empty(V, np.uint32)
    _check(_load().orc_sssp(V, ptr, adj if len(adj) else np.zeros(2, np.uint32), src, out), "sssp")
    return out


def cc(ptr, col):
    ptr, col = _ptr(ptr), _u32(col)
    V = len(ptr) - 1
    out = np.empty(V, np.uint32)
    _check(_load().orc_cc(V, ptr, col if len(col) else np.zeros(1, np.uint32), out), "cc")
    return out


def pr_ref(ptr, col, outdeg):
    """Reference PageRank over CSC arrays; returns (ranks, passes)."""
    ptr, col, outdeg = _ptr(ptr), _u32(col), _u32(outdeg)
    V = len(ptr) - 1
    out = np.empty(V, np.float64)
    it = ctypes.c_int32(0)
    _check(_load().orc_pr_ref(V, ptr, col if len(col) else np.zeros(1, np.uint32), outdeg, out,
                              ctypes.byref(it)), "pr_ref")
    return out, it.value


def pr_std(ptr, col, outdeg, damping=0.85, tol=1e-9, max_iter=100):
    """Standard PageRank over CSC arrays; returns (ranks, passes, l1_residual)."""
    ptr, col, outdeg = _ptr(ptr), _u32(col), _u32(outdeg)
    V = len(ptr) - 1
    out = np.empty(V, np.float64)
    it = ctypes.c_int32(0)
    res = ctypes.c_double(0)
    _check(_load().orc_pr_std(V, ptr, col if len(col) else np.zeros(1, np.uint32), outdeg,
                              damping, tol, max_iter, out, ctypes.byref(it), ctypes.byref(res)),
           "pr_std")
    return out, it.value, res.value


def pr_std_mt(ptr, col, outdeg, nthreads, damping=0.85, tol=1e-9, max_iter=100):
    """pr_std on host threads (same per-vertex sums; the dangling mass and the
    residual are combined from per-thread partials); returns (ranks, passes,
    l1_residual)."""
    ptr, col, outdeg = _ptr(ptr), _u32(col), _u32(outdeg)
    V = len(ptr) - 1
    out = np.empty(max(V, 1), np.float64)
    it = ctypes.c_int32(0)
    res = ctypes.c_double(0)
    _check(_load().orc_pr_std_mt(V, ptr, col if len(col) else np.zeros(1, np.uint32), outdeg,
                                 damping, tol, max_iter, int(nthreads), out, ctypes.byref(it), ctypes.byref(res)),
           "pr_std_mt")
    return out[:V], it.value, res.value


def static_split(ptr, static_edges_cap):
    """Reference static-region rule; returns (is_static uint8[V], mps, edges_in_static)."""
    ptr = _ptr(ptr)
    V = len(ptr) - 1
    flags = np.empty(max(V, 1), np.uint8)
    mps = ctypes.c_uint64(0)
    ins = ctypes.c_uint64(0)
    _check(_load().orc_static_split(V, ptr, static_edges_cap, flags, ctypes.byref(mps),
                                    ctypes.byref(ins)), "static_split")
    return flags[:V], mps.value, ins.value


def reached_edges(ptr, val, unreached):
    ptr, val = _ptr(ptr), _u32(val)
    return int(_load().orc_reached_edges(len(ptr) - 1, ptr, val, unreached))


def relax_mt(mode, ptr, edges, src, nthreads):
    """Reference iteration scheme on host threads (mode 0 BFS, 1 SSSP, 2 CC)."""
    ptr, edges = _ptr(ptr), _u32(np.asarray(edges).reshape(-1))
    V = len(ptr) - 1
    out = np.empty(max(V, 1), np.uint32)
    it = ctypes.c_int32(0)
    _check(_load().orc_relax_mt(mode, V, ptr, edges if len(edges) else np.zeros(2, np.uint32), src,
                                nthreads, out, ctypes.byref(it)), "relax_mt")
    return out[:V], it.value


def converter(src, dst, by_dst=False, compat=False):
    """The reference converter's CSR/CSC build, restated (converter/converter.cpp).

    V = largest id + 1 over both endpoints (converter.cpp:102-125); offsets are
    the running degree sum, stepped back by one once it reaches E
    (converter.cpp:131-138) when ``compat``; each list keeps the edges in input
    order (converter.cpp:143-164; :246-268 for CSC, keyed by destination and
    storing the source). Pure Python loops: small inputs only. Returns
    (V, ptr uint64[V+1] with ptr[V] = E, order int64[E] = input index of each
    placed edge, outdeg uint32[V]).
    """
    src = [int(x) for x in src]
    dst = [int(x) for x in dst]
    E = len(src)
    V = max([max(s, d) + 1 for s, d in zip(src, dst)] or [0])
    key = dst if by_dst else src
    deg = [0] * V
    for k in key:
        deg[k] += 1
    ptr = [0] * (V + 1)
    t = 0
    for v in range(V):
        ptr[v] = t
        t += deg[v]
        if compat and t == E and E:
            t -= 1
    ptr[V] = E
    exact = [0] * V
    t = 0
    for v in range(V):
        exact[v] = t
        t += deg[v]
    anchor = [0] * V
    order = [0] * E
    for i, k in enumerate(key):
        order[exact[k] + anchor[k]] = i
        anchor[k] += 1
    outdeg = [0] * V
    for s in src:
        outdeg[s] += 1
    return V, np.array(ptr, np.uint64), np.array(order, np.int64), np.array(outdeg, np.uint32)


def converter_ref_weights(n):
    """convertByteToBWCSR's weights (converter.cpp:303-306, :396): srand(0), then
    rand() % 20 per edge in input order, drawn from this host's C library."""
    libc = ctypes.CDLL(None)
    libc.srand(0)
    return np.array([libc.rand() % 20 for _ in range(n)], np.uint32)
