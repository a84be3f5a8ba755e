"""The counting sort entry point that allocates nothing, for callers that may
not allocate GPU memory while they run (an engine that budgets all device
memory at level load, where a cudaMalloc or cudaFree mid-frame could
synchronise the device; a host whose allocator policy rejects allocations
outside its pool).  It must give exactly what the allocating entry point
gives -- integer output, so bit for bit -- on consecutive calls that reuse
its fixed scratch array.  The file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(fn_name, keys, num_cells):
    import torch
    from lustrine_gb300 import _lib
    lib = _lib.load()
    k = torch.from_numpy(np.ascontiguousarray(keys, np.int32)).cuda()
    counts = torch.full((num_cells + 1,), -1, dtype=torch.int32, device="cuda")
    out = torch.full((len(keys),), -1, dtype=torch.int32, device="cuda")
    rc = getattr(lib, fn_name)(C.c_void_p(counts.data_ptr()), C.c_void_p(k.data_ptr()), len(keys),
                               num_cells, C.c_void_p(out.data_ptr()), None)
    return rc, counts.cpu().numpy(), out.cpu().numpy()


def test_noalloc_counting_sort_matches_allocating_entry_point_twice():
    rng = np.random.default_rng(99)
    # two calls in a row with different sizes: the second finds the first
    # call's data in the shared scratch and must clear what it relies on
    cases = [(rng.integers(0, 5000, 200_000).astype(np.int32), 5000),
             (rng.integers(0, 1 << 20, 1 << 20).astype(np.int32), 1 << 20)]
    for keys, cells in cases:
        rc_a, counts_a, perm_a = _call("lustrine_counting_sort", keys, cells)
        rc_b, counts_b, perm_b = _call("lustrine_counting_sort_noalloc", keys, cells)
        assert rc_a == 0 and rc_b == 0
        assert np.array_equal(perm_b, perm_a)
        assert np.array_equal(counts_b, counts_a)
        assert np.array_equal(perm_b, np.argsort(keys, kind="stable"))


def test_noalloc_counting_sort_rejects_sizes_beyond_its_limit():
    from lustrine_gb300 import _lib
    too_many = np.zeros((1 << 20) + 1, np.int32)
    rc, _, _ = _call("lustrine_counting_sort_noalloc", too_many, 4)
    assert rc == 10 and _lib.ERRORS[rc] == "LUSTRINE_ERR_TOO_LARGE"
    rc, _, _ = _call("lustrine_counting_sort_noalloc", np.zeros(8, np.int32), (1 << 20) + 1)
    assert rc == 10
