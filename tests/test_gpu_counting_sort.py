"""GPU counting sort against the reference's unit test (golden vector written
by Sorting::counting_sort itself, experiments/unit_tests/main.cpp:46-89) and
against a stable argsort at larger sizes."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _sort(keys, num_cells):
    import torch
    from lustrine_gb300.sorting import counting_sort
    k = torch.from_numpy(np.ascontiguousarray(keys, np.int32)).cuda()
    counts = torch.full((num_cells + 1,), -7, dtype=torch.int32, device="cuda")
    out = torch.full((len(keys),), -7, dtype=torch.int32, device="cuda")
    counting_sort(counts, k, num_cells, out)
    return counts.cpu().numpy(), out.cpu().numpy()


def test_counting_sort_matches_reference_unit_test():
    g = golden("counting_sort.npz")
    counts, perm = _sort(g["keys"], int(g["num_cells"]))
    assert np.array_equal(perm, g["perm"])
    # the reference leaves each key's first output slot in counts, then n
    hist = np.bincount(g["keys"], minlength=int(g["num_cells"]))
    assert np.array_equal(counts[:-1], np.cumsum(hist) - hist) and counts[-1] == len(perm)


@pytest.mark.parametrize("n,cells,seed", [(1, 1, 0), (1000, 7, 1), (300_000, 1_000_003, 2),
                                          (2_000_000, 4096, 3)])
def test_counting_sort_stable_argsort(n, cells, seed):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, cells, n).astype(np.int32)
    counts, perm = _sort(keys, cells)
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))
    hist = np.bincount(keys, minlength=cells)
    assert counts[-1] == n and np.array_equal(counts[:-1], np.cumsum(hist) - hist)


def test_counting_sort_empty_and_bad_keys():
    from lustrine_gb300 import LustrineError
    counts, perm = _sort(np.zeros(0, np.int32), 5)
    assert len(perm) == 0 and np.array_equal(counts, np.zeros(6, np.int32))
    with pytest.raises(LustrineError):
        _sort(np.array([0, 5, 1], np.int32), 5)


@pytest.mark.parametrize("case", ["all_equal_65536", "thresholds", "merge_passes", "mixed_sizes"])
def test_counting_sort_skewed_keys_stable(case):
    """Skewed key distributions: the members of a cell of more than 32 keys
    are ordered by a block-wide sort (bitonic in shared memory up to 2,048,
    merged runs beyond), so a cell of k keys costs O(k log k), not O(k^2)."""
    rng = np.random.default_rng(7)
    if case == "all_equal_65536":
        keys, cells = np.zeros(65536, np.int32), 3
    elif case == "thresholds":
        # cells of exactly 32, 33, 2048 and 2049 members, interleaved
        sizes = {0: 32, 1: 33, 2: 2048, 3: 2049, 4: 1}
        keys = np.concatenate([np.full(k, c, np.int32) for c, k in sizes.items()])
        keys = keys[rng.permutation(len(keys))]
        cells = 5
    elif case == "merge_passes":
        # one cell of 20,000 keys (runs of 2,048 merged over four passes) among uniform keys
        keys = np.concatenate([np.full(20_000, 11, np.int32), rng.integers(0, 64, 5000).astype(np.int32)])
        keys = keys[rng.permutation(len(keys))]
        cells = 64
    else:
        # log-uniform cell sizes up to 5,000 over 200 cells
        sizes = np.exp(rng.uniform(0, np.log(5000), 200)).astype(int) + 1
        keys = np.repeat(np.arange(200, dtype=np.int32), sizes)
        keys = keys[rng.permutation(len(keys))]
        cells = 200
    counts, perm = _sort(keys, cells)
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))
    hist = np.bincount(keys, minlength=cells)
    assert counts[-1] == len(keys) and np.array_equal(counts[:-1], np.cumsum(hist) - hist)
