"""Many-configuration batches (CPU): the seeded generator, the static partition,
and the rank-sharded solve with its final gather over world_size 2 (gloo on
127.0.0.1, spawned processes; a stand-in solver on the host replaces the GPU
solve -- what is tested here is the host-side sharding and gather)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mutual_polarization_slab_gb300 import batch  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_is_balanced_and_complete():
    rng = np.random.default_rng(0)
    sizes = [int(v) for v in np.exp(rng.uniform(np.log(500), np.log(20000), 256))]
    for world in (1, 2, 3, 8):
        parts = batch.partition(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)          # LPT bound
        assert all(p == sorted(p) for p in parts)


def test_fft_friendly_grid():
    assert [batch.fft_size(v) for v in (1, 31, 32, 47, 61, 89, 97, 191)] == [1, 32, 32, 48, 64, 90, 100, 192]
    box = np.array([30.0, 30.0, 30.0])
    ng0, P0 = batch.grid_for(box, 0.55, 1e-4, fft_friendly=False)
    ng, P = batch.grid_for(box, 0.55, 1e-4)
    assert np.all(ng >= ng0) and P >= P0
    assert all(batch.fft_size(int(v)) == int(v) for v in ng)


def test_make_configurations_properties():
    cfgs = batch.make_configurations(count=3, seed=4, n_range=(100, 400))
    assert [c.index for c in cfgs] == [0, 1, 2]
    for c in cfgs:
        assert 100 <= c.n <= 400
        assert np.all((c.radii >= 0.7) & (c.radii <= 1.3))
        assert set(np.unique(c.beta)) <= {0.3, 0.9} and abs(np.mean(c.beta == 0.3) - 0.5) <= 1.0 / c.n
        # no overlaps (minimum image, contact at a_i + a_j)
        d = c.x[:, None, :] - c.x[None, :, :]
        d -= c.box * np.round(d / c.box)
        dist = np.sqrt((d ** 2).sum(-1)) + np.eye(c.n) * 1e9
        assert np.all(dist >= (c.radii[:, None] + c.radii[None, :]) - 1e-9)
        phi = 4 * np.pi * np.sum(c.radii ** 3) / (3 * np.prod(c.box))
        assert abs(phi - c.meta["phi"]) < 1e-9
    again = batch.make_configurations(count=3, seed=4, n_range=(100, 400))
    assert all(np.array_equal(a.x, b.x) for a, b in zip(cfgs, again))


def _rank_main(rank, world, port, sizes, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfgs = [batch.Configuration(np.zeros((n, 3)), np.ones(n), np.full(n, 0.5), np.ones(3), index=i)
            for i, n in enumerate(sizes)]
    seen = []

    def solver(cfg):
        seen.append(cfg.index)
        return np.full((2, 3, 3), float(cfg.index)), True

    res = batch.solve_configurations(cfgs, [0.5, 1.0], solver=solver)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"),
            np.array([sorted(res.keys()), sorted(seen) + [-1] * (len(sizes) - len(seen))], dtype=np.int64))
    assert all(np.all(res[k][0] == k) for k in res)
    dist.destroy_process_group()


def test_sharded_solve_and_gather_world2(tmp_path):
    import torch.multiprocessing as mp

    sizes = [900, 300, 5000, 1200, 50, 700, 2500]
    mp.start_processes(_rank_main, args=(2, _free_port(), sizes, str(tmp_path)), nprocs=2, start_method="spawn")
    r0 = np.load(tmp_path / "rank0.npy")
    r1 = np.load(tmp_path / "rank1.npy")
    assert list(r0[0]) == list(range(len(sizes))) and list(r1[0]) == list(range(len(sizes)))
    s0 = [v for v in r0[1] if v >= 0]
    s1 = [v for v in r1[1] if v >= 0]
    assert sorted(s0 + s1) == list(range(len(sizes))) and not set(s0) & set(s1)
    assert (s0, s1) == tuple(batch.partition(sizes, 2))
