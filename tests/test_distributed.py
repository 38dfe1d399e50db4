"""Two-rank (gloo, CPU) test of the multi-process host logic: every rank images
its own strip of the grid with the FP64 oracle, no data-path collective; the
strips assembled equal the single-process image, and the timing reduction
returns the maximum over ranks."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from sar_cambrianaccelerationcard_gb300 import replicas, scenes


def _scene():
    s = scenes.config1(np_=64, ns=512, n_img=8, snr_db=None)
    s.grid = scenes.centred_grid(s.radar, 24, 150, 0.5)
    return s


def _worker(rank, world, port, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as orc
    orc.set_threads(1)
    s = _scene()
    rc = orc.range_compress(s, orc.echo(s, noise=False))
    sub = replicas.grid_strip(s.grid, rank, world)
    g = s.grid
    img = orc.backproject_raw(rc, s.apc, sub.origin, sub.ux, sub.uy, (0, 0, sub.nx, sub.ny), s.radar.fc, s.radar.c,
                              s.layout.t0_bins, s.layout.bin_rate)
    np.save(os.path.join(outdir, f"strip{rank}.npy"), img)
    m = replicas.max_over_ranks(10.0 + rank, dist)
    np.save(os.path.join(outdir, f"max{rank}.npy"), np.array([m]))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_strip_bounds_cover_grid():
    for ny in (1, 63, 64, 150, 4096):
        for world in (1, 2, 3, 8):
            rows = [replicas.strip_bounds(ny, r, world) for r in range(world)]
            assert rows[0][0] == 0 and rows[-1][1] == ny
            for (a, b), (c, d) in zip(rows, rows[1:]):
                assert b == c and a <= b
            assert all(a % 64 == 0 for a, _ in rows)


def test_two_rank_strips_match_single_process(tmp_path, orc):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    s = _scene()
    strips = [np.load(tmp_path / f"strip{r}.npy") for r in range(world)]
    full = replicas.assemble(strips, s.grid.ny, s.grid.nx, world)
    ref = orc.image(s, orc.echo(s, noise=False))
    assert np.array_equal(full, ref)
    assert [float(np.load(tmp_path / f"max{r}.npy")[0]) for r in range(world)] == [11.0, 11.0]
