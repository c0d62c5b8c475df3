"""Host-side logic without a GPU: synthetic workload generation and the
multi-GPU bin partition (exercised over gloo with two ranks)."""
import os

import numpy as np
import pytest


def test_workload_shapes(synth):
    w = synth.WORKLOADS["cfg3"]
    lines = synth.readout_lines(w)
    assert lines.shape == (3072, 2)
    k = synth.wave_trajectory(w)
    assert k.shape == (3072 * 512, 3)
    u = k * (np.array(w.grid) - 1)
    # readouts span the grid along x; the outermost phase-encode lines wave
    # past the grid edge by up to the wave amplitude (those taps are dropped)
    assert u[:, 0].min() >= 0 and u[:, 0].max() < w.grid[0]
    assert u[:, 1:].min() >= -w.wave_cells - 1e-9
    assert (u[:, 1:].max(axis=0) <= np.array(w.grid[1:]) + w.wave_cells).all()


def test_breathing_bins_uneven_occupancy(synth):
    bins = synth.breathing_bins(3072, 16)
    occ = np.array([len(b) for b in bins]) / 3072
    assert np.isclose(occ.sum(), 1.0)
    assert occ.min() >= 0.025 and occ.max() <= 0.125
    assert occ.max() / occ.min() > 3
    allr = np.sort(np.concatenate(bins))
    assert np.array_equal(allr, np.arange(3072))


def test_coil_maps_normalised(synth):
    m = synth.coil_maps((16, 12, 8), 6)
    assert np.allclose(np.sum(np.abs(m) ** 2, axis=0), 1.0, atol=1e-5)


def test_phantom_seeded(synth):
    a = synth.phantom((16, 16, 16))
    b = synth.phantom((16, 16, 16))
    assert np.array_equal(a, b) and np.abs(a).max() > 0


def test_partition_balanced():
    import importlib
    dist = importlib.import_module("4d_lung_gb300.dist")
    sizes = [5, 9, 3, 12, 7, 7, 4, 10]
    parts = dist.partition_bins(sizes, 3)
    assert sorted(sum(parts, [])) == list(range(8))
    loads = [sum(sizes[b] for b in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)


def _rank_main(rank, world, port, sizes, q):
    import importlib

    import torch
    import torch.distributed as dist_
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist_.init_process_group("gloo", rank=rank, world_size=world)
    d = importlib.import_module("4d_lung_gb300.dist")
    mine = d.partition_bins(sizes, world)[rank]
    t = torch.zeros(len(sizes), dtype=torch.int64)
    for b in mine:
        t[b] += 1
    dist_.all_reduce(t)
    load = torch.tensor([sum(sizes[b] for b in mine)], dtype=torch.int64)
    loads = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist_.all_gather(loads, load)
    if rank == 0:
        q.put((t.tolist(), [int(x.item()) for x in loads]))
    dist_.destroy_process_group()


def test_partition_two_ranks_gloo():
    """Every bin is solved by exactly one rank; no data-path collective is
    needed (the check itself uses one all_reduce)."""
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    sizes = [int(x) for x in np.random.default_rng(0).integers(50, 200, 16)]
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    counts, loads = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert counts == [1] * 16
    assert abs(loads[0] - loads[1]) <= max(sizes)


def test_roofline_byte_model(synth):
    """bench.stage_bytes: each stage reads its input and writes its output
    once; with sample-support pruning the x passes count only the listed
    columns, the forward y pass (listed rows) only their rows, and the
    spreading gather its stores, row offsets, taps and sample values."""
    import importlib
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    bench = importlib.import_module("bench")
    w = synth.scaled(synth.WORKLOADS["cfg1"], (8, 8, 4), (16, 16, 8), n_ch=2, read_os=2)
    Ix, Iy, Iz = w.img
    Gx, Gy, Gz = w.grid
    Ni, Nl, C8 = Ix * Iy * Iz, Ix * Iy, 8 * w.n_ch
    sizes = [10, 30]
    full = bench.stage_bytes(w, sizes)
    assert full["fwd_z"] == 2 * (8 * Ni + C8 * Nl * Gz) + C8 * Ni   # coil maps once (L2 across bins)
    assert full["fwd_y"] == 2 * C8 * (Nl * Gz + Ix * Gy * Gz)
    assert full["fwd_x"] == C8 * 2 * Gy * Gz * (Ix + Gx)
    assert full["adj_x"] == full["fwd_x"] and full["adj_y"] == full["fwd_y"]
    assert full["adj_z"] == 2 * (C8 * Nl * Gz + 8 * Ni) + C8 * Ni
    cols, tiles = [40, 60], [3, 5]
    pruned = bench.stage_bytes(w, sizes, (cols, tiles), matrix=(500, 100 * Gx), y_listed=True)
    assert pruned["fwd_x"] == C8 * 100 * (Ix + Gx)
    assert pruned["fwd_y"] == C8 * (2 * Nl * Gz + Ix * 100)
    assert pruned["spread"] == C8 * 100 * Gx + 4 * 100 * Gx + 8 * 500 + 40 * C8
    assert pruned["interp"] == C8 * 100 * Gx + 40 * (64 + 4 + C8)
    assert bench.apply_bytes(w, sizes) == sum(full.values())
    # the spreading fused with the adjoint x pass: one stage that reads the
    # matrix and the samples and writes the x pass's Ix output rows
    fused = bench.stage_bytes(w, sizes, (cols, tiles), matrix=(500, 100 * Gx), y_listed=True, fused=True)
    assert list(fused) == bench.STAGES_FUSED
    assert fused["spread_adjx"] == 4 * 100 * Gx + 8 * 500 + 40 * C8 + C8 * 100 * Ix
    assert all(fused[k] == pruned[k] for k in fused if k != "spread_adjx")
    assert (bench.apply_bytes(w, sizes, (cols, tiles), (500, 100 * Gx), True, True) ==
            bench.apply_bytes(w, sizes, (cols, tiles), (500, 100 * Gx), True) - C8 * 100 * Gx * 2)
