"""Python side of the GPU counting sort (Sorting::counting_sort,
src/neighbors/Sorting.cpp:12-34) exported by liblustrine_gb300.so.

Arrays are device pointers (ints); torch tensors are the convenient holder:

    counts = torch.empty(num_cells + 1, dtype=torch.int32, device="cuda")
    sorted_ = torch.empty(n, dtype=torch.int32, device="cuda")
    counting_sort(counts, keys, num_cells, sorted_)
"""
from __future__ import annotations

import ctypes as C

from . import _lib


def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(getattr(stream, "cuda_stream", stream))


def counting_sort(counts, keys, num_cells: int, sorted_indices, stream=None) -> None:
    """Stable counting sort of device int32 keys; fills sorted_indices (input
    indices in key order) and counts (the first output slot of every key,
    then n).  Raises LustrineError on a key outside [0, num_cells)."""
    lib = _lib.load()
    _lib.check(lib.lustrine_counting_sort(C.c_void_p(counts.data_ptr()), C.c_void_p(keys.data_ptr()),
                                          keys.numel(), int(num_cells),
                                          C.c_void_p(sorted_indices.data_ptr()), _stream_ptr(stream)),
               "lustrine_counting_sort")
