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
