"""Host side of the slab partition: layouts (adv_slab_layout, no GPU), the
ghost-layer exchange between gloo ranks (world size 2 and 3, CPU tensors) and
the cross-rank reductions.  Every rank cuts its local vector out of the same
global vector with its owned layers only; after the exchange every ghost face
layer must hold the neighbouring cells' values of the global vector."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from advection_miniapp_gb300 import make_config
from advection_miniapp_gb300.distributed import SlabLayout, TorchExchange, slab_ranges

CASES = {
    "periodic-k3": dict(degree=3, n_cells=(3, 2, 5), periodic=1),
    "dirichlet-k2": dict(degree=2, n_cells=(2, 3, 4), periodic=0),
    "sipg-k2": dict(degree=2, n_cells=(2, 2, 4), periodic=0, velocity_type=1, diffusion=1e-3, boundary_value=0),
}


def test_slab_ranges():
    assert slab_ranges(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert slab_ranges(4, 4) == [(0, 1), (1, 2), (2, 3), (3, 4)]
    with pytest.raises(ValueError):
        slab_ranges(2, 3)


@pytest.mark.parametrize("case", sorted(CASES))
def test_layouts_tile_the_mesh(adv_lib, case):
    cfg = make_config(**CASES[case])
    nz, n = cfg.n_cells[2], cfg.degree + 1
    cells = cfg.n_cells[0] * cfg.n_cells[1]
    for ws in (1, 2, nz):
        owned = 0
        for zb, ze in slab_ranges(nz, ws):
            lay = SlabLayout(cfg, zb, ze)
            assert lay.layer_cells == cells and lay.dofs_per_cell == n ** 3
            assert lay.ghost_lo == (bool(cfg.periodic) or zb > 0)
            assert lay.ghost_hi == (bool(cfg.periodic) or ze < nz)
            assert lay.layers == (ze - zb) + lay.ghost_lo + lay.ghost_hi
            assert lay.n_dofs == lay.layers * cells * n ** 3
            assert lay.owned_begin == lay.ghost_lo * cells * n ** 3
            assert lay.zoff == zb - lay.ghost_lo
            assert lay.halo_values == (n ** 3 if cfg.diffusion else n ** 2)
            owned += lay.owned_dofs
        assert owned == nz * cells * n ** 3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, case, errors):
    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
        cfg = make_config(**CASES[case])
        nz, n = cfg.n_cells[2], cfg.degree + 1
        zb, ze = slab_ranges(nz, ws)[rank]
        lay = SlabLayout(cfg, zb, ze)
        per_cell = n ** 3
        glob = torch.from_numpy(np.random.default_rng(11).standard_normal(nz * lay.layer_cells * per_cell))
        loc = torch.full((lay.n_dofs,), float("nan"), dtype=torch.float64)
        lay.owned(loc).copy_(glob[zb * lay.layer_cells * per_cell:ze * lay.layer_cells * per_cell])
        ex = TorchExchange(rank, ws, bool(cfg.periodic))
        ex.update_ghost_values(lay, loc)
        ref = lay.from_global(glob)
        g = loc.view(lay.layers, lay.layer_cells, n, n * n)
        r = ref.view(lay.layers, lay.layer_cells, n, n * n)
        if lay.ghost_lo:
            sel = slice(None) if lay.full_cells else n - 1
            assert torch.equal(g[0, :, sel], r[0, :, sel]), "ghost layer below"
        if lay.ghost_hi:
            sel = slice(None) if lay.full_cells else 0
            assert torch.equal(g[-1, :, sel], r[-1, :, sel]), "ghost layer above"
        assert torch.equal(lay.owned(loc), lay.owned(ref))
        # reductions: sums of squares of the owned parts, minimum of the slab starts
        s = ex.all_reduce([float((lay.owned(loc) ** 2).sum()), 1.0])
        assert abs(s[0] - float((glob ** 2).sum())) <= 1e-12 * s[0] and s[1] == ws
        m = ex.all_reduce([float(zb)], op="min")
        assert m[0] == 0.0
        dist.barrier()
        dist.destroy_process_group()
    except BaseException as e:  # reported to the parent
        errors.put(f"rank {rank}: {type(e).__name__}: {e}")
        raise


@pytest.mark.parametrize("ws", [2, 3])
@pytest.mark.parametrize("case", sorted(CASES))
def test_gloo_ghost_exchange(adv_lib, case, ws):
    if CASES[case]["n_cells"][2] < ws:
        pytest.skip("fewer layers than ranks")
    ctx = mp.get_context("spawn")
    errors = ctx.Queue()
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    mp.start_processes(_rank_main, args=(ws, _free_port(), case, errors), nprocs=ws, join=True,
                       start_method="spawn")
    assert errors.empty()


def test_single_rank_periodic_wraps_to_itself(adv_lib):
    cfg = make_config(**CASES["periodic-k3"])
    lay = SlabLayout(cfg, 0, cfg.n_cells[2])
    n = cfg.degree + 1
    glob = torch.from_numpy(np.random.default_rng(2).standard_normal(cfg.n_cells[2] * lay.layer_cells * n ** 3))
    loc = torch.zeros(lay.n_dofs, dtype=torch.float64)
    lay.owned(loc).copy_(glob)
    TorchExchange(0, 1, True).update_ghost_values(lay, loc)
    ref = lay.from_global(glob)
    g = loc.view(lay.layers, -1, n, n * n)
    r = ref.view(lay.layers, -1, n, n * n)
    assert torch.equal(g[0, :, n - 1], r[0, :, n - 1]) and torch.equal(g[-1, :, 0], r[-1, :, 0])
