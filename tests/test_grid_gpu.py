"""Device neighbour-grid rebuild against the reference's NeighborGrid
outputs (tests/golden/neighbor_grid.npz) and the oracle.  Integer outputs,
so every comparison is exact."""
import ctypes
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG_NAME, load_golden

pytestmark = pytest.mark.gpu


def _mod():
    return importlib.import_module(PKG_NAME + ".solvers.neighbor_grid")


def _xm(pos, dev):
    xm = torch.zeros((pos.shape[0], 4), dtype=torch.float32, device=dev)
    xm[:, :3] = torch.tensor(pos, dtype=torch.float32, device=dev)
    return xm


def _check(grid, g, name):
    assert grid.ngas == int(g[f"{name}_ngas"]), name
    np.testing.assert_array_equal(grid.gsort.cpu().numpy(), g[f"{name}_gsort"])
    np.testing.assert_array_equal(grid.cell_start.cpu().numpy(), g[f"{name}_cell_start"])
    assert (grid.nx, grid.ny, grid.nz) == tuple(int(v) for v in g[f"{name}_dims"]), name
    assert grid.lo == tuple(float(v) for v in g[f"{name}_lo"]), name
    assert grid.inv_cell == float(g[f"{name}_inv_cell"]), name


@pytest.mark.parametrize("name", ["disk", "disk_all", "tiny_h", "lattice", "zero_h", "single_gas"])
def test_rebuild_matches_reference(cuda_dev, name):
    ng = _mod()
    g = load_golden("neighbor_grid")
    pos, h = g[f"{name}_pos"], g[f"{name}_h"]
    grid = ng.NeighborGrid(pos.shape[0], min_radius=float(g[f"{name}_min_radius"]), device=cuda_dev)
    hs = torch.tensor(h, dtype=torch.float32, device=cuda_dev)
    star = g.get(f"{name}_is_star")
    st = torch.tensor(star, dtype=torch.int32, device=cuda_dev) if star is not None else None
    grid.rebuild(_xm(pos, cuda_dev), hs, st)
    _check(grid, g, name)
    # A second rebuild of the same input gives the same outputs.
    grid.rebuild(_xm(pos, cuda_dev), hs, st)
    _check(grid, g, name)
    grid.close()


def test_rebuild_without_gas_keeps_previous_grid(cuda_dev):
    ng = _mod()
    g = load_golden("neighbor_grid")
    pos, h = g["disk_pos"], g["disk_h"]
    grid = ng.NeighborGrid(pos.shape[0], device=cuda_dev)
    xm = _xm(pos, cuda_dev)
    hs = torch.tensor(h, dtype=torch.float32, device=cuda_dev)
    grid.rebuild(xm, hs, torch.tensor(g["disk_is_star"], dtype=torch.int32, device=cuda_dev))
    _check(grid, g, "disk")
    assert grid.rebuild(xm, hs, torch.tensor(g["nogas_is_star"], dtype=torch.int32, device=cuda_dev)) == 0
    _check(grid, g, "nogas")
    grid.close()


def test_rebuild_1m_matches_oracle(cuda_dev, orc):
    """N = 1,000,000 exponential disk, 30% stars: every output equal to the
    oracle's, gsort a stable cell ordering of the gas indices."""
    ng = _mod()
    ic = importlib.import_module(PKG_NAME + ".ic")
    n = 1_000_000
    pos, _, _ = ic.exponential_disk(n, seed=5)
    pos = pos.astype(np.float32).astype(np.float64)
    rng = np.random.default_rng(6)
    h = rng.lognormal(np.log(0.05), 0.5, n).astype(np.float32)
    star = (rng.random(n) < 0.3).astype(np.int32)
    grid = ng.NeighborGrid(n, min_radius=0.02, device=cuda_dev)
    ngas = grid.rebuild(_xm(pos, cuda_dev), torch.tensor(h, device=cuda_dev),
                        torch.tensor(star, device=cuda_dev))
    ref = orc.grid_rebuild(pos, h.astype(np.float64), star, 0.02)
    assert ngas == ref["ngas"] == int((star == 0).sum())
    gs = grid.gsort.cpu().numpy()
    cs = grid.cell_start.cpu().numpy()
    np.testing.assert_array_equal(gs, ref["gsort"])
    np.testing.assert_array_equal(cs, ref["cell_start"])
    assert (grid.nx, grid.ny, grid.nz) == tuple(int(v) for v in ref["dims"])
    assert grid.inv_cell == ref["inv_cell"]
    nc = grid.nx * grid.ny * grid.nz
    assert np.all(np.diff(cs[:nc + 1]) >= 0) and cs[nc] == ngas and not cs[nc + 1:].any()
    assert np.array_equal(np.sort(gs[:ngas]), np.nonzero(star == 0)[0])
    grid.close()


def test_nonfinite_and_empty_inputs(cuda_dev):
    ng = _mod()
    pkg = importlib.import_module(PKG_NAME)
    lib_mod = importlib.import_module(PKG_NAME + "._lib")
    pos = np.random.default_rng(2).normal(size=(100, 3))
    pos[7, 1] = np.nan
    grid = ng.NeighborGrid(100, device=cuda_dev)
    with pytest.raises(pkg.GravityError):
        grid.rebuild_all(_xm(pos, cuda_dev), torch.full((100,), 0.1, device=cuda_dev))
    grid.close()
    # n = 0: nothing to bin.
    h = ctypes.c_void_p()
    lib_mod.call("gb_grid_create", ctypes.byref(h), 0, 0.0)
    info = lib_mod.GridInfo()
    lib_mod.call("gb_grid_rebuild", h, None, None, None, None, None, ctypes.byref(info),
                 torch.cuda.current_stream().cuda_stream)
    assert info.ngas == 0 and lib_mod.load().gb_grid_max_cells(h) == 64
    lib_mod.load().gb_grid_destroy(h)
