"""MagicaVoxel (.vox) grids through the wrapper's init_grid_magikavoxel and
create_grid (no GPU): small files written from the published chunk format
(tests/golden/vox/) against what the reference's loader made of them
(tests/golden/vox_ref.npz), and -- where the reference tree is mounted --
the reference's own .vox assets against its loader run here."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, HAVE_REF, REF, golden
FILES = ("box", "empty_first", "dup")


def _load(path, position=(0.0, 0.0, 0.0)):
    from lustrine_gb300 import wrapper as W
    g = W.init_grid_magikavoxel(path, position)
    status = W.last_status()
    try:
        cells, colors = W.grid_arrays(g) if g.cells else (None, None)
        meta = dict(X=g.X, Y=g.Y, Z=g.Z, occupied=g.num_occupied_grid_cells, type=g.type,
                    per_cell=bool(g.has_one_color_per_cell), position=(g.position.x, g.position.y, g.position.z))
    finally:
        W.free_grid(g)
    return status, cells, colors, meta


@pytest.mark.parametrize("name", FILES)
def test_vox_grid_matches_reference_loader(name):
    g = golden("vox_ref.npz")
    status, cells, colors, meta = _load(os.path.join(GOLDEN, "vox", f"{name}.vox"), (1.0, 2.0, 3.0))
    assert status == 0
    assert np.array_equal(cells, g[f"{name}_cells"])
    assert np.array_equal(colors, g[f"{name}_colors"])
    assert meta["occupied"] == int(g[f"{name}_occupied"]) == int((cells != 0).sum())
    assert meta["type"] == 0 and meta["per_cell"] and meta["position"] == (1.0, 2.0, 3.0)


def test_vox_reader_semantics():
    """The empty first model is skipped, a voxel listed twice keeps its last
    colour, colour index 255 names palette entry 254."""
    g = golden("vox_ref.npz")
    assert g["empty_first_cells"].shape == (4, 2, 3)
    cells = g["dup_cells"]
    assert cells.shape == (3, 3, 2) and cells[0, 0, 0] == 9 and cells[1, 2, 1] == 255
    assert np.array_equal(g["dup_colors"][1, 2, 1], g["dup_rgba"][254].astype(np.float32) / np.float32(255))


@pytest.mark.parametrize("name", FILES)
def test_create_grid_cells_and_double_colours(name):
    from lustrine_gb300 import wrapper as W
    g = golden("vox_ref.npz")
    grid = W.create_grid(os.path.join(GOLDEN, "vox", f"{name}.vox"), type_=1)
    try:
        assert W.last_status() == 0
        cells, colors = W.grid_arrays(grid)
        assert grid.type == 1 and grid.num_occupied_grid_cells == int(g[f"{name}_occupied"])
    finally:
        W.free_grid(grid)
    ref = g[f"{name}_cells"]
    assert np.array_equal(cells, (ref != 0).astype(np.int32))
    # LustrineWrapper.cpp:608-611: voxel_color.r / 255.0 in double, stored as float
    rgba = g[f"{name}_rgba"]
    want = np.zeros(ref.shape + (4,), np.float32)
    occ = ref != 0
    want[occ] = (rgba[(ref[occ] + 255) & 255].astype(np.float64) / 255.0).astype(np.float32)
    assert np.array_equal(colors, want)


def test_vox_errors(tmp_path):
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import write_vox
    from lustrine_gb300 import wrapper as W
    from lustrine_gb300._lib import GridWrapper
    status, cells, _, _ = _load(str(tmp_path / "missing.vox"))
    assert status == 1 and cells is None  # LUSTRINE_ERR_ARGS, grid untouched
    bad = tmp_path / "bad.vox"
    bad.write_bytes(b"NOTAVOXFILE.....")
    assert _load(str(bad))[0] == 1
    empty = tmp_path / "empty.vox"
    write_vox(str(empty), [((2, 2, 2), [])], np.zeros((256, 4), np.uint8))
    assert _load(str(empty))[0] == 1  # no model with a voxel
    # no RGBA chunk: the cells, zero colours and "unsupported" (the default palette is not carried)
    nopal = tmp_path / "nopal.vox"
    data = bytearray(open(os.path.join(GOLDEN, "vox", "dup.vox"), "rb").read())
    i = data.find(b"RGBA")
    nopal.write_bytes(bytes(data[:i]))
    status, cells, colors, _ = _load(str(nopal))
    assert status == 6 and cells[0, 0, 0] == 9 and not colors.any()
    assert isinstance(GridWrapper(), GridWrapper) and W is not None


@pytest.mark.skipif(not HAVE_REF, reason="LUSTRINE_REFERENCE_DIR not set")
def test_reference_assets_load_like_the_reference(orc):
    path = orc.build_ref(REF)
    R = orc.Reference(path)
    files = sorted(glob.glob(os.path.join(REF, "experiments", "**", "*.vox"), recursive=True))
    assert files
    for f in files:
        cells, colors, occ = R.load_vox(f)
        status, c2, col2, meta = _load(f)
        assert status == 0, f
        assert np.array_equal(c2, cells) and np.array_equal(col2, colors), f
        assert meta["occupied"] == occ, f
