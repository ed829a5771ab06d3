"""The allocation-free BFS entry point (asc_bfs_device_noalloc) through the C ABI.

It is for callers that cannot allocate device memory at query time (their
device memory belongs to another allocator, or cudaMalloc/cudaFree are not
allowed in their loop); its scratch is a fixed device array inside the library.
The test checks it against the regular entry point (asc_run) and against the
CPU oracle on the same graph, bit for bit, on two calls in a row (the first on
the default stream, the second on a stream of the caller's), plus its limit and
input checks. The graph is placed in device memory with torch, which stands in
for the caller's own allocator. This file is collected last.
"""
import numpy as np
import pytest

import ascetic_gb300 as A
import oracle

pytestmark = pytest.mark.gpu


def _device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def test_noalloc_bfs_matches_asc_run_on_two_calls():
    torch = pytest.importorskip("torch")
    ptr, col = A.rmat_csr(15, 16, 21)
    V, E = len(ptr) - 1, int(ptr[-1])
    sources = [0, int(np.nonzero(np.diff(ptr))[0][-1])]
    with A.Graph.from_csr(ptr, col) as g:
        expected = [g.run("bfs", s)[0] for s in sources]
    d_ptr = _device(torch, ptr.astype(np.uint32))
    d_col = _device(torch, col)
    d_out = torch.empty(V, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    # the second call runs on a stream of the caller's (its cudaStream_t handle)
    streams = [None, torch.cuda.Stream()]
    for s, exp, stream in zip(sources, expected, streams):
        handle = None if stream is None else stream.cuda_stream
        rc = A.lib().asc_bfs_device_noalloc(V, E, d_ptr.data_ptr(), d_col.data_ptr(), s, d_out.data_ptr(), handle)
        torch.cuda.synchronize()
        assert rc == A.OK, A.last_error()
        got = d_out.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, exp), s
        assert np.array_equal(got, oracle.bfs(ptr, col, s)), s


def test_noalloc_rejects_sizes_and_bad_csr():
    torch = pytest.importorskip("torch")
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = A.lib().asc_bfs_device_noalloc((1 << 20) + 1, 4, d.data_ptr(), d.data_ptr(), 0, d.data_ptr(), None)
    assert rc == A.ERR_BUDGET and "scratch limit" in A.last_error()
    ptr = np.array([0, 2, 3, 3], np.uint32)
    col = np.array([1, 7, 2], np.uint32)          # 7 >= V
    d_ptr, d_col = _device(torch, ptr), _device(torch, col)
    out = torch.empty(3, dtype=torch.int32, device="cuda")
    rc = A.lib().asc_bfs_device_noalloc(3, 3, d_ptr.data_ptr(), d_col.data_ptr(), 0, out.data_ptr(), None)
    assert rc == A.ERR_INVALID
    col[1] = 2
    d_col = _device(torch, col)
    rc = A.lib().asc_bfs_device_noalloc(3, 3, d_ptr.data_ptr(), d_col.data_ptr(), 0, out.data_ptr(), None)
    assert rc == A.OK
    assert out.cpu().numpy().tolist() == [1, 2, 2]
