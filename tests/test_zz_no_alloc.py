"""qg_search_batch_noalloc: the search entry point for callers that cannot allocate device
memory (code running while a CUDA graph is captured, or a serving process that fixes its
device memory at start-up). It must give exactly what qg_search_batch gives, call after call,
from its file-scope scratch array, and refuse sizes that do not fit that array.

This file is named so that pytest collects it last; it passes alone in a fresh process and
after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from cases import SEARCH_CASES
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr() if t is not None else 0)


def test_no_alloc_search_matches_the_allocating_entry_point(cuda):
    torch = cuda
    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    lib = N.load()
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    space = RabitqSpace(128, g["center"])
    index = OursIndex(space, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    q = torch.from_numpy(Q).cuda()
    nq, k = q.shape[0], 10

    ids_a = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    d_a = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    st_a = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
    index.search_into(q, ids_a, d_a, k=k, l_value=40, stats_out=st_a)
    torch.cuda.synchronize()

    params = N.SearchParams(k, 40, 1, 1.9, 100, 0, 0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):  # two calls in a row share (and must re-clear) the scratch array
        ids_b = torch.full((nq, k), 7, dtype=torch.int32, device="cuda")
        d_b = torch.zeros((nq, k), dtype=torch.float32, device="cuda")
        st_b = torch.zeros((nq, 9), dtype=torch.int64, device="cuda")
        rc = lib.qg_search_batch_noalloc(index.handle, _ptr(q), nq, C.byref(params), None, None, k,
                                         _ptr(ids_b), _ptr(d_b), _ptr(st_b), stream)
        assert rc == N.QG_OK, N.last_error()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ids_b.cpu().numpy(), ids_a.cpu().numpy())
        np.testing.assert_array_equal(d_b.cpu().numpy().view(np.uint32), d_a.cpu().numpy().view(np.uint32))
        np.testing.assert_array_equal(st_b.cpu().numpy(), st_a.cpu().numpy())
    # the reference's own results, as a final anchor
    np.testing.assert_array_equal(ids_b.cpu().numpy().astype(np.uint32), g["ids_L40_k10"])


def test_no_alloc_search_rejects_sizes_beyond_its_scratch(cuda):
    torch = cuda
    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    lib = N.load()
    g = load_golden("search_c1")
    space = RabitqSpace(128, g["center"])
    index = OursIndex(space, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    nq = (N.QG_NOALLOC_SCRATCH_BYTES // (128 * 5)) + 1  # prepared queries alone exceed the array
    q = torch.zeros((nq, 128), dtype=torch.float32, device="cuda")
    ids = torch.empty((nq, 10), dtype=torch.int32, device="cuda")
    d = torch.empty((nq, 10), dtype=torch.float32, device="cuda")
    params = N.SearchParams(10, 40, 1, 1.9, 100, 0, 0)
    rc = lib.qg_search_batch_noalloc(index.handle, _ptr(q), nq, C.byref(params), None, None, 10, _ptr(ids),
                                     _ptr(d), None, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 1  # QG_ERR_INVALID
    assert "do not fit" in N.last_error()


def _noalloc_call(lib, N, index, q, k, params, torch, d_l=None):
    nq = q.shape[0]
    ids = torch.full((nq, k), 7, dtype=torch.int32, device="cuda")
    d = torch.zeros((nq, k), dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.qg_search_batch_noalloc(index.handle, _ptr(q), nq, C.byref(params), None, _ptr(d_l), k, _ptr(ids),
                                     _ptr(d), None, stream)
    assert rc == N.QG_OK, N.last_error()
    return ids, d, lib.qg_search_noalloc_status(stream)


def test_no_alloc_status_reports_what_the_kernels_saw(cuda):
    """A neighbour id outside the graph gives UINT32_MAX ids and QG_ERR_GRAPH, a per-query L above
    the call's pool capacity gives QG_ERR_INVALID, exactly as qg_search_batch + qg_search_status
    report them; a clean call afterwards reads QG_OK again."""
    torch = cuda
    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    lib = N.load()
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    q = torch.from_numpy(Q[:32]).cuda()
    space = RabitqSpace(128, g["center"])
    params = N.SearchParams(10, 40, 1, 1.9, 100, 0, 0)

    edges = g["edges"].copy()
    edges[0, 0] = 10 ** 6  # node 0 (the start of every query) names a node outside the graph
    bad = OursIndex(space, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], edges)
    ids, _, st = _noalloc_call(lib, N, bad, q, 10, params, torch)
    assert st == 4, N.STATUS_NAMES.get(st)  # QG_ERR_GRAPH
    assert (ids.cpu().numpy().astype(np.uint32) == np.uint32(0xFFFFFFFF)).all()
    with pytest.raises(RuntimeError, match="QG_ERR_GRAPH"):  # the allocating path agrees
        bad.search(q, k=10, l_value=40)

    good = OursIndex(space, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    big_l = torch.full((q.shape[0],), 80, dtype=torch.int32, device="cuda")  # above params.l_value = 40
    _, _, st = _noalloc_call(lib, N, good, q, 10, params, torch, d_l=big_l)
    assert st == 1, N.STATUS_NAMES.get(st)  # QG_ERR_INVALID: clamped to 40
    ids, d, st = _noalloc_call(lib, N, good, q, 10, params, torch)
    assert st == N.QG_OK
    np.testing.assert_array_equal(ids.cpu().numpy().astype(np.uint32), g["ids_L40_k10"][:32])
