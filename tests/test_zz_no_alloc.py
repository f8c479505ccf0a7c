"""lj_gpu_morton_sort_noalloc -- the Morton sort for callers that cannot
allocate device memory when they call it (an application whose GPU memory is
handed out by its own fixed arena, or a loop that must not pay for the
synchronisation an allocation can cause).  It works in a fixed array inside
the library instead of allocating, so it must give exactly the results of
lj_gpu_morton_sort, call after call, whatever the previous call left in that
array.  The outputs are integers, so "the same" means bit-identical.

This file is collected last on purpose: it also has to pass after every other
test of the session (and alone in a fresh process)."""
import ctypes as C

import numpy as np
import pytest
import torch

from lajolla_public_gb300 import abi, gpu, scenes

pytestmark = pytest.mark.gpu


def _noalloc():
    L = gpu.lib()
    f = L.lj_gpu_morton_sort_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _tris(seed, n):
    pos, idx = scenes.triangle_soup(seed, n)
    return torch.from_numpy(pos[idx].reshape(-1, 9).copy()).cuda()


def _run_noalloc(tri, stream=None):
    n = tri.shape[0]
    codes = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    order = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    handle = None if stream is None else stream.cuda_stream
    if stream is not None:
        stream.wait_stream(torch.cuda.current_stream())
    rc = _noalloc()(tri.data_ptr(), n, codes.data_ptr(), order.data_ptr(), handle)
    assert rc == abi.LJ_OK, rc
    torch.cuda.synchronize()
    return codes.cpu().numpy(), order.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_two_calls_in_a_row(ctx):
    # a large call first, then a smaller one that must not see its leftovers
    for seed, n in ((11, abi.LJ_NOALLOC_MORTON_MAX_TRIANGLES), (12, 4099)):
        tri = _tris(seed, n)
        got_codes, got_order = _run_noalloc(tri)
        want_codes, want_order = ctx.morton_sort(tri)
        np.testing.assert_array_equal(got_codes, want_codes.cpu().numpy())
        np.testing.assert_array_equal(got_order, want_order.cpu().numpy())


def test_noalloc_rejects_sizes_beyond_its_fixed_scratch(ctx):
    n = abi.LJ_NOALLOC_MORTON_MAX_TRIANGLES + 1
    tri = torch.zeros((n, 9), dtype=torch.float32, device="cuda")
    codes = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    order = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    rc = _noalloc()(tri.data_ptr(), n, codes.data_ptr(), order.data_ptr(), None)
    assert rc == abi.LJ_ERR_SIZE_LIMIT
    torch.cuda.synchronize()
    assert bool((codes == 7).all()) and bool((order == 7).all())


def test_noalloc_smallest_sizes_and_a_side_stream(ctx):
    # n = 1 skips the sort (only the codes and the identity order are
    # written), n = 2 sorts one pair; then a call on a stream of its own
    side = torch.cuda.Stream()
    for seed, n, stream in ((21, 1, None), (22, 2, None), (23, 2, None), (24, 5000, side), (25, 1, side)):
        tri = _tris(seed, n)
        got_codes, got_order = _run_noalloc(tri, stream)
        want_codes, want_order = ctx.morton_sort(tri)
        np.testing.assert_array_equal(got_codes, want_codes.cpu().numpy())
        np.testing.assert_array_equal(got_order, want_order.cpu().numpy())
