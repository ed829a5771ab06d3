"""ascetic_gb300: GB300-native out-of-GPU-memory graph iteration engine.

A thin ctypes mirror of the C ABI in include/ascetic.h (libascetic_gb300.so,
built in-tree by ascetic_gb300/build.py). The reference's host drivers
bfs_opt / cc_opt / sssp_opt / pr_opt (CalculateOpt.cuh:11-14) map to
``bfs_opt`` ... ``pr_opt`` here; ``Graph`` mirrors GraphMeta (GraphMeta.cuh:52-149).

The library loads lazily: importing this package never touches the GPU, and
every call that needs the engine raises ``EngineUnavailable`` when the shared
library has not been built. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import formats  # noqa: F401  (re-exported helper module)

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libascetic_gb300.so")
PTGRAPH_PATH = os.path.join(_PKG, "_lib", "ptgraph")
CONVERT_PATH = os.path.join(_PKG, "_lib", "asc-convert")

# enums (include/ascetic.h)
OK, ERR_INVALID, ERR_BAD_FILE, ERR_BUDGET, ERR_CUDA, ERR_TIMEOUT, ERR_CANCELLED, ERR_UNSUPPORTED, \
    ERR_NO_DEVICE, ERR_NOMEM, ERR_BUSY = range(11)
FMT_AUTO, FMT_BCSR, FMT_BWCSR, FMT_BCSC, FMT_BCSR32 = range(5)
BFS, SSSP, CC, PR = range(4)
BUDGET_ALL, BUDGET_FRAC, BUDGET_BYTES, BUDGET_ADVISE_K, BUDGET_EDGES, BUDGET_MANAGED = range(6)
PR_REF, PR_STD = 0, 1
F64, F32 = 0, 1
RUN_NO_OUTPUT, RUN_DEVICE_OUT, RUN_PHASE_TIMING, RUN_HOST_LOOP, RUN_FRAGMENT_COUNTS, RUN_GATHER_COPY = 1, 2, 4, 8, 16, 32
RUN_NO_STAGING, RUN_PARTITION_COPY = 64, 128
RMAT_WEIGHTS, RMAT_SYMMETRIC, RMAT_TRANSPOSE = 1, 2, 4
ALGOS = {"bfs": BFS, "sssp": SSSP, "cc": CC, "pr": PR}

# every symbol include/ascetic.h declares
EXPORTED = ["asc_status_string", "asc_last_error", "asc_version", "asc_device_count", "asc_budget_default",
            "asc_graph_open", "asc_graph_from_csr", "asc_graph_info_get", "asc_graph_close",
            "asc_params_default", "asc_run", "asc_bfs_opt", "asc_cc_opt", "asc_sssp_opt", "asc_pr_opt",
            "asc_rmat_csr", "asc_graph_rmat", "asc_write_graph", "asc_link_probe",
            "asc_bfs_device_noalloc", "asc_run_batch", "asc_server_config_default", "asc_server_create",
            "asc_server_add_graph", "asc_server_submit", "asc_server_wait", "asc_server_cancel",
            "asc_server_stats_get", "asc_server_destroy", "asc_graph_get_tuning", "asc_graph_set_tuning",
            "asc_graph_tune", "asc_device_memory", "asc_link_probe_runs", "asc_graph_fragment_counts",
            "asc_host_alloc", "asc_host_free"]
TUNE_NO_CACHE = 1
SERVE_BATCHED, SERVE_FIFO = 0, 1


class EngineUnavailable(RuntimeError):
    pass


class AscError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_status_name(status), msg))
        self.status = status


class Budget(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_uint32), ("fragment_edges", ctypes.c_uint32), ("value", ctypes.c_double),
                ("stage_bytes", ctypes.c_uint64)]


class GraphInfo(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_uint64), ("edges", ctypes.c_uint64), ("edge_bytes", ctypes.c_uint32),
                ("is_csc", ctypes.c_uint32), ("static_edges", ctypes.c_uint64),
                ("static_vertices", ctypes.c_uint64), ("device_edge_bytes", ctypes.c_uint64),
                ("device_vertex_bytes", ctypes.c_uint64), ("host_pinned_bytes", ctypes.c_uint64),
                ("max_degree", ctypes.c_uint32), ("max_weight", ctypes.c_uint32),
                ("weight_bits", ctypes.c_uint32), ("edge_bits", ctypes.c_uint32),
                ("staging_bytes", ctypes.c_uint64), ("in_head_bytes", ctypes.c_uint64)]


class Tuning(ctypes.Structure):
    _fields_ = [("huge_degree", ctypes.c_uint32), ("segment_edges", ctypes.c_uint32),
                ("dense_div", ctypes.c_uint32), ("ctas_per_sm", ctypes.c_uint32), ("delta", ctypes.c_uint32),
                ("bu_div", ctypes.c_uint32), ("ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("device_budget_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_uint32),
                ("queue_capacity", ctypes.c_uint32), ("mode", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class QueryInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("iterations", ctypes.c_int32), ("batch_size", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("cancelled", ctypes.c_uint64), ("batch_iterations", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("queries_per_s", ctypes.c_double),
                ("span_s", ctypes.c_double), ("engines_created", ctypes.c_uint64),
                ("engines_freed", ctypes.c_uint64), ("workspaces_freed", ctypes.c_uint64),
                ("memory_waits", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Params(ctypes.Structure):
    _fields_ = [("pr_mode", ctypes.c_uint32), ("precision", ctypes.c_uint32), ("damping", ctypes.c_double),
                ("tolerance", ctypes.c_double), ("max_iterations", ctypes.c_int32), ("flags", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("status_detail", ctypes.c_int32),
                ("frontier_vertices", ctypes.c_uint64), ("ondemand_vertices", ctypes.c_uint64),
                ("edges_processed", ctypes.c_uint64),
                ("ondemand_edges", ctypes.c_uint64), ("ondemand_bytes", ctypes.c_uint64),
                ("reached_vertices", ctypes.c_uint64), ("reached_edges", ctypes.c_uint64),
                ("ms_total", ctypes.c_double), ("ms_static", ctypes.c_double), ("ms_ondemand", ctypes.c_double),
                ("ms_copyout", ctypes.c_double), ("residual", ctypes.c_double),
                ("kernel_launches", ctypes.c_uint32), ("staged_chunks", ctypes.c_uint32),
                ("bottom_up_edges", ctypes.c_uint64), ("ms_bottom_up", ctypes.c_double),
                ("bottom_up_vertices", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k not in ("reserved", "status_detail")}


_lib = None


def _status_name(s):
    names = ["OK", "ERR_INVALID", "ERR_BAD_FILE", "ERR_BUDGET", "ERR_CUDA", "ERR_TIMEOUT", "ERR_CANCELLED",
             "ERR_UNSUPPORTED", "ERR_NO_DEVICE", "ERR_NOMEM", "ERR_BUSY"]
    return names[s] if 0 <= s < len(names) else "status %d" % s


def lib():
    """Loads libascetic_gb300.so; raises EngineUnavailable when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise EngineUnavailable("%s is not built: run ascetic_gb300/build.py (nvcc, sm_103a)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    c_u32, c_u64, c_dbl, c_vp = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p
    gpp = P(c_vp)
    sig = {
        "asc_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "asc_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_size_t),
        "asc_version": ([], ctypes.c_char_p),
        "asc_device_count": ([], ctypes.c_int),
        "asc_device_memory": ([P(c_u64), P(c_u64)], ctypes.c_int),
        "asc_host_alloc": ([c_u64, P(c_vp)], ctypes.c_int),
        "asc_host_free": ([c_vp], ctypes.c_int),
        "asc_budget_default": ([P(Budget)], None),
        "asc_graph_open": ([ctypes.c_char_p, ctypes.c_int, P(Budget), gpp], ctypes.c_int),
        "asc_graph_from_csr": ([c_u64, c_u64, c_vp, c_vp, c_u32, c_vp, P(Budget), gpp], ctypes.c_int),
        "asc_graph_info_get": ([c_vp, P(GraphInfo)], ctypes.c_int),
        "asc_graph_close": ([c_vp], ctypes.c_int),
        "asc_params_default": ([P(Params)], None),
        "asc_run": ([c_vp, ctypes.c_int, c_u32, P(Params), c_vp, P(Stats)], ctypes.c_int),
        "asc_bfs_opt": ([ctypes.c_char_p, c_u32, c_dbl, c_vp, P(Stats)], ctypes.c_int),
        "asc_cc_opt": ([ctypes.c_char_p, c_dbl, c_vp, P(Stats)], ctypes.c_int),
        "asc_sssp_opt": ([ctypes.c_char_p, c_u32, c_dbl, c_vp, P(Stats)], ctypes.c_int),
        "asc_pr_opt": ([ctypes.c_char_p, c_dbl, c_vp, P(Stats)], ctypes.c_int),
        "asc_rmat_csr": ([c_u32, c_u32, c_u64, c_dbl, c_dbl, c_dbl, c_u32, c_u32, c_u32, c_vp, c_vp, c_vp],
                         ctypes.c_int),
        "asc_graph_rmat": ([c_u32, c_u32, c_u64, c_dbl, c_dbl, c_dbl, c_u32, c_u32, c_u32, P(Budget), gpp],
                           ctypes.c_int),
        "asc_write_graph": ([ctypes.c_char_p, ctypes.c_int, c_u64, c_u64, c_vp, c_vp, c_vp], ctypes.c_int),
        "asc_link_probe": ([c_u64, ctypes.c_int, P(c_dbl), P(c_dbl)], ctypes.c_int),
        "asc_link_probe_runs": ([c_u64, c_u32, ctypes.c_int, P(c_dbl)], ctypes.c_int),
        "asc_graph_fragment_counts": ([c_vp, c_vp, c_u64, P(c_u64), ctypes.c_int], ctypes.c_int),
        "asc_bfs_device_noalloc": ([c_u64, c_u64, c_vp, c_vp, c_u32, c_vp, c_vp], ctypes.c_int),
        "asc_run_batch": ([c_vp, ctypes.c_int, c_vp, c_u32, P(Params), c_vp, P(Stats)], ctypes.c_int),
        "asc_server_config_default": ([P(ServerConfig)], None),
        "asc_graph_get_tuning": ([c_vp, P(Tuning)], ctypes.c_int),
        "asc_graph_set_tuning": ([c_vp, P(Tuning)], ctypes.c_int),
        "asc_graph_tune": ([c_vp, ctypes.c_int, c_vp, c_u32, c_u32, P(Tuning)], ctypes.c_int),
        "asc_server_create": ([P(ServerConfig), gpp], ctypes.c_int),
        "asc_server_add_graph": ([c_vp, c_vp, P(c_u32)], ctypes.c_int),
        "asc_server_submit": ([c_vp, c_u32, ctypes.c_int, c_u32, P(Params), c_vp, P(c_u64)], ctypes.c_int),
        "asc_server_wait": ([c_vp, c_u64, ctypes.c_int64, P(QueryInfo)], ctypes.c_int),
        "asc_server_cancel": ([c_vp, c_u64], ctypes.c_int),
        "asc_server_stats_get": ([c_vp, P(ServerStats)], ctypes.c_int),
        "asc_server_destroy": ([c_vp], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().asc_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _check(status):
    if status != OK:
        raise AscError(status, last_error())


def device_count():
    return lib().asc_device_count()


class PinnedArray:
    """A numpy array over page-locked host memory (asc_host_alloc), for result
    buffers that asc_run fills at the copy engine's full rate. Keep the object
    alive while the array is in use; close() frees the memory."""

    def __init__(self, n, dtype=np.uint32):
        dtype = np.dtype(dtype)
        self._p = ctypes.c_void_p()
        _check(lib().asc_host_alloc(max(1, n * dtype.itemsize), ctypes.byref(self._p)))
        buf = (ctypes.c_char * max(1, n * dtype.itemsize)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=n)

    def close(self):
        if self._p and self._p.value:
            self.array = None
            lib().asc_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_free_bytes():
    free, total = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(lib().asc_device_memory(ctypes.byref(free), ctypes.byref(total)))
    return free.value


def make_budget(frac=None, nbytes=None, edges=None, advise_k=None, fragment_edges=4096, managed=False,
                stage_bytes=0):
    """Static-region budget. managed=True selects the UVM comparison engine
    (no static region, edges in CUDA managed memory). stage_bytes of the budget
    become two staging buffers for dense on-demand passes (standard PageRank)."""
    b = Budget()
    lib().asc_budget_default(ctypes.byref(b))
    b.fragment_edges = fragment_edges
    b.stage_bytes = int(stage_bytes)
    if managed:
        b.mode, b.value = BUDGET_MANAGED, 0.0
    elif frac is not None:
        b.mode, b.value = BUDGET_FRAC, float(frac)
    elif nbytes is not None:
        b.mode, b.value = BUDGET_BYTES, float(nbytes)
    elif edges is not None:
        b.mode, b.value = BUDGET_EDGES, float(edges)
    elif advise_k is not None:
        b.mode, b.value = BUDGET_ADVISE_K, float(advise_k)
    return b


def make_params(pr_mode=PR_REF, precision=F64, damping=0.85, tolerance=1e-9, max_iterations=0, flags=0):
    p = Params()
    lib().asc_params_default(ctypes.byref(p))
    p.pr_mode, p.precision, p.damping, p.tolerance = pr_mode, precision, damping, tolerance
    p.max_iterations, p.flags = max_iterations, flags
    return p


class Graph:
    """A graph resident as a device static prefix plus a pinned host copy."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)
        info = GraphInfo()
        _check(lib().asc_graph_info_get(self._h, ctypes.byref(info)))
        self.info = info
        self.V = info.vertices
        self.E = info.edges

    @classmethod
    def open(cls, path, fmt=FMT_AUTO, budget=None):
        h = ctypes.c_void_p()
        b = budget if budget is not None else make_budget()
        _check(lib().asc_graph_open(path.encode(), fmt, ctypes.byref(b), ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def from_csr(cls, ptr, edges, outdeg=None, budget=None):
        """ptr: V+1 offsets; edges: u32 destinations, or (E, 2) u32 (dst, weight)."""
        ptr = np.ascontiguousarray(ptr, dtype=np.uint64)
        edges = np.ascontiguousarray(edges, dtype=np.uint32)
        V = len(ptr) - 1
        E = int(ptr[-1])
        eb = 8 if edges.ndim == 2 else 4
        if edges.size == 0:
            edges = np.zeros(2, np.uint32)
        od = None
        if outdeg is not None:
            od = np.ascontiguousarray(outdeg, dtype=np.uint32)
        b = budget if budget is not None else make_budget()
        h = ctypes.c_void_p()
        _check(lib().asc_graph_from_csr(V, E, ptr.ctypes.data, edges.ctypes.data, eb,
                                        od.ctypes.data if od is not None else None, ctypes.byref(b),
                                        ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def rmat(cls, scale, edge_factor=16, seed=1, a=0.57, b=0.19, c=0.19, weights=None, symmetric=False,
             transpose=False, budget=None):
        flags = (RMAT_WEIGHTS if weights else 0) | (RMAT_SYMMETRIC if symmetric else 0) | \
            (RMAT_TRANSPOSE if transpose else 0)
        wmin, wmax = weights if weights else (0, 0)
        bud = budget if budget is not None else make_budget()
        h = ctypes.c_void_p()
        _check(lib().asc_graph_rmat(scale, edge_factor, seed, a, b, c, wmin, wmax, flags, ctypes.byref(bud),
                                    ctypes.byref(h)))
        return cls(h.value)

    def close(self):
        if self._h:
            lib().asc_graph_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def fragment_counts(self, reset=False):
        """Edges read per 4096-edge fragment by the runs made with
        RUN_FRAGMENT_COUNTS since the last reset (uint64 array)."""
        n = ctypes.c_uint64(0)
        _check(lib().asc_graph_fragment_counts(self._h, None, 0, ctypes.byref(n), 0))
        out = np.zeros(max(n.value, 1), np.uint64)
        _check(lib().asc_graph_fragment_counts(self._h, out.ctypes.data, n.value, None, 1 if reset else 0))
        return out[:n.value]

    def refresh_info(self):
        _check(lib().asc_graph_info_get(self._h, ctypes.byref(self.info)))
        return self.info

    def run(self, algo, source=0, params=None, out=None, no_output=False):
        """Runs one query; returns (values, stats dict)."""
        if isinstance(algo, str):
            algo = ALGOS[algo]
        p = params if params is not None else make_params()
        if no_output:
            p.flags |= RUN_NO_OUTPUT
        if out is None and not no_output:
            if algo == PR:
                out = np.empty(self.V, np.float32 if (p.precision == F32 and p.pr_mode == PR_STD) else np.float64)
            else:
                out = np.empty(self.V, np.uint32)
        st = Stats()
        _check(lib().asc_run(self._h, algo, source, ctypes.byref(p),
                             out.ctypes.data if out is not None else None, ctypes.byref(st)))
        return out, st.as_dict()


def _run_batch(self, algo, sources, params=None, out=None, no_output=False):
    """Runs up to 64 BFS/SSSP sources together; returns ((n, V) values, stats)."""
    if isinstance(algo, str):
        algo = ALGOS[algo]
    src = np.ascontiguousarray(sources, dtype=np.uint32)
    p = params if params is not None else make_params()
    if no_output:
        p.flags |= RUN_NO_OUTPUT
    if out is None and not no_output:
        out = np.empty((len(src), self.V), np.uint32)
    st = Stats()
    _check(lib().asc_run_batch(self._h, algo, src.ctypes.data, len(src), ctypes.byref(p),
                               out.ctypes.data if out is not None else None, ctypes.byref(st)))
    return out, st.as_dict()


Graph.run_batch = _run_batch


def _tune(self, algo, sources=(), cache=True):
    """Autotunes the engine's thresholds for this graph; returns the setting."""
    if isinstance(algo, str):
        algo = ALGOS[algo]
    src = np.ascontiguousarray(list(sources) or [0], dtype=np.uint32)
    t = Tuning()
    _check(lib().asc_graph_tune(self._h, algo, src.ctypes.data, len(src), 0 if cache else TUNE_NO_CACHE,
                                ctypes.byref(t)))
    return t.as_dict()


def _get_tuning(self):
    t = Tuning()
    _check(lib().asc_graph_get_tuning(self._h, ctypes.byref(t)))
    return t.as_dict()


def _set_tuning(self, huge_degree=512, segment_edges=2048, dense_div=64, ctas_per_sm=0, delta=0, bu_div=64):
    t = Tuning(huge_degree, segment_edges, dense_div, ctas_per_sm, delta, bu_div, 0.0)
    _check(lib().asc_graph_set_tuning(self._h, ctypes.byref(t)))


Graph.tune = _tune
Graph.get_tuning = _get_tuning
Graph.set_tuning = _set_tuning


class Server:
    """Query server over resident graphs (continuous batching or FIFO).

    budget_bytes caps every device allocation the server makes (0: no cap);
    max_batch (1..64) caps the sources of one batch, and an SSSP batch of at
    most 16 or 32 sources keeps distance rows of that width, as it does when
    64 columns of a graph could never fit the budget."""

    def __init__(self, budget_bytes=0, mode=SERVE_BATCHED, max_batch=64):
        cfg = ServerConfig()
        lib().asc_server_config_default(ctypes.byref(cfg))
        cfg.device_budget_bytes, cfg.mode, cfg.max_batch = int(budget_bytes), mode, max_batch
        h = ctypes.c_void_p()
        _check(lib().asc_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._graphs = []
        self._out = {}

    def add_graph(self, graph):
        gid = ctypes.c_uint32()
        _check(lib().asc_server_add_graph(self._h, graph._h, ctypes.byref(gid)))
        self._graphs.append(graph)
        return gid.value

    def submit(self, graph_id, algo, source=0, params=None, out=None):
        if isinstance(algo, str):
            algo = ALGOS[algo]
        p = params if params is not None else make_params()
        if out is None:
            g = self._graphs[graph_id]
            dt = np.uint32 if algo != PR else (np.float32 if (p.pr_mode == PR_STD and p.precision == F32)
                                                 else np.float64)
            out = np.empty(g.V, dt)
        t = ctypes.c_uint64()
        _check(lib().asc_server_submit(self._h, graph_id, algo, source, ctypes.byref(p), out.ctypes.data,
                                       ctypes.byref(t)))
        self._out[t.value] = out
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        info = QueryInfo()
        st = lib().asc_server_wait(self._h, ticket, timeout_ms, ctypes.byref(info))
        out = self._out.pop(ticket, None)
        if st not in (OK, ERR_CANCELLED):
            raise AscError(st, last_error())
        return out, {k: getattr(info, k) for k, _ in info._fields_ if k != "reserved"}

    def cancel(self, ticket):
        _check(lib().asc_server_cancel(self._h, ticket))

    def stats(self):
        st = ServerStats()
        _check(lib().asc_server_stats_get(self._h, ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if self._h:
            lib().asc_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rmat_csr(scale, edge_factor=16, seed=1, a=0.57, b=0.19, c=0.19, weights=None, symmetric=False,
             transpose=False):
    """Host-only RMAT generator (no GPU needed): returns ptr, edges[, outdeg]."""
    V = 1 << scale
    E = V * edge_factor * (2 if symmetric else 1)
    flags = (RMAT_WEIGHTS if weights else 0) | (RMAT_SYMMETRIC if symmetric else 0) | \
        (RMAT_TRANSPOSE if transpose else 0)
    wmin, wmax = weights if weights else (0, 0)
    ptr = np.empty(V + 1, np.uint64)
    edges = np.empty((E, 2) if weights else E, np.uint32)
    outdeg = np.empty(V, np.uint32) if transpose else None
    _check(lib().asc_rmat_csr(scale, edge_factor, seed, a, b, c, wmin, wmax, flags, ptr.ctypes.data,
                              edges.ctypes.data, outdeg.ctypes.data if outdeg is not None else None))
    return (ptr, edges, outdeg) if transpose else (ptr, edges)


def link_probe(nbytes=1 << 30, iters=5):
    """(pinned H2D copy-engine GB/s, SM zero-copy read GB/s)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(lib().asc_link_probe(nbytes, iters, ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def link_probe_runs(run_bytes, nbytes=1 << 30, iters=3):
    """Host-link GB/s when warps read runs of run_bytes at random offsets."""
    g = ctypes.c_double()
    _check(lib().asc_link_probe_runs(nbytes, run_bytes, iters, ctypes.byref(g)))
    return g.value


def write_graph(path, fmt, ptr, edges, outdeg=None):
    ptr = np.ascontiguousarray(ptr, dtype=np.uint64)
    edges = np.ascontiguousarray(edges, dtype=np.uint32)
    od = np.ascontiguousarray(outdeg, dtype=np.uint32) if outdeg is not None else None
    _check(lib().asc_write_graph(path.encode(), fmt, len(ptr) - 1, int(ptr[-1]), ptr.ctypes.data,
                                 edges.ctypes.data, od.ctypes.data if od is not None else None))


def _opt(fn, path, *args, out_dtype=np.uint32, want_output=True):
    V = int(np.fromfile(path, dtype=np.uint64, count=1)[0])
    out = np.empty(V, out_dtype) if want_output else None
    st = Stats()
    _check(fn(path.encode(), *args, out.ctypes.data if out is not None else None, ctypes.byref(st)))
    return out, st.as_dict()


def bfs_opt(path, source, advise_rate=0.0):
    return _opt(lib().asc_bfs_opt, path, source, advise_rate)


def cc_opt(path, advise_rate=0.0):
    return _opt(lib().asc_cc_opt, path, advise_rate)


def sssp_opt(path, source, advise_rate=0.0):
    return _opt(lib().asc_sssp_opt, path, source, advise_rate)


def pr_opt(path, advise_rate=0.0):
    return _opt(lib().asc_pr_opt, path, advise_rate, out_dtype=np.float64)
