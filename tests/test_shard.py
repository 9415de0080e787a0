"""Frame sharding across ranks: the partition (host logic) and a world-size-2 run on
CPU ranks over gloo, each rank rendering its own frames, checked against one render
of the whole stack.  The CPU ranks use the oracle in place of the GPU renderer, so
this covers the partition, the per-rank views and the scalar reduction."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from cbclib_v2_gb300 import shard, workloads


def _ragged_offsets(seed, F, lo=0, hi=5000):
    rng = np.random.default_rng(seed)
    counts = np.clip(np.round(rng.lognormal(np.log(800), 1.0, F)), lo, hi).astype(np.int64)
    return np.concatenate([[0], np.cumsum(counts)])


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_frames_in_balanced_ranges(world):
    offs = _ragged_offsets(1, 256)
    b = shard.partition_frames(offs, world)
    assert b[0] == 0 and b[-1] == 256 and np.all(np.diff(b) >= 0)
    cost = np.diff(offs) + max(1.0, 0.05 * np.diff(offs).mean())
    per_rank = np.array([cost[b[r]:b[r + 1]].sum() for r in range(world)])
    # every rank within one frame's cost of the ideal share
    assert np.all(np.abs(per_rank - cost.sum() / world) <= cost.max() + 1e-9)
    shards = [shard.shard_of(offs, r, world) for r in range(world)]
    assert sum(s.n_lines for s in shards) == offs[-1]
    assert all(shards[r].l1 == shards[r + 1].l0 for r in range(world - 1))


def test_partition_edge_cases():
    assert list(shard.partition_frames([0], 3)) == [0, 0, 0, 0]          # no frames
    b = shard.partition_frames([0, 10, 10, 10], 8)                          # world > frames
    assert b[0] == 0 and b[-1] == 3 and np.all(np.diff(b) >= 0)
    b = shard.partition_frames([0, 0, 0, 0, 0], 2)                          # empty frames
    assert list(b) == [0, 2, 4]
    with pytest.raises(ValueError):
        shard.partition_frames([1, 2], 2)
    with pytest.raises(ValueError):
        shard.partition_frames([0, 3, 2], 2)
    with pytest.raises(ValueError):
        shard.shard_of([0, 1], 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, tmpdir):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        ls = workloads.ragged_stack(seed=11, F=12, H=96, W=80, median=300.0)
        offs = ls.frame_offsets()
        sh = shard.shard_of(offs, rank, world)
        # this rank's frames only: lines [l0, l1), frames rebased to 0
        local = np.zeros((sh.n_frames, ls.shape[1], ls.shape[2]), np.float64)
        idxs = np.repeat(np.arange(sh.n_frames), np.diff(sh.local_offsets(offs)))
        oracle.draw_lines(local, ls.lines[sh.l0:sh.l1], idxs, ls.max_val, ls.kernel, ls.overlap, 1)
        loss = torch.tensor([float((local ** 2).sum())], dtype=torch.float64)
        dist.all_reduce(loss)                          # the only cross-rank value
        parts = [None] * world
        dist.all_gather_object(parts, (sh.f0, sh.f1, local))
        if rank == 0:
            np.save(os.path.join(tmpdir, 'loss.npy'), loss.numpy())
            full = np.zeros((ls.shape[0], ls.shape[1], ls.shape[2]), np.float64)
            for f0, f1, img in parts:
                full[f0:f1] = img
            np.save(os.path.join(tmpdir, 'image.npy'), full)
    finally:
        dist.destroy_process_group()


def test_two_cpu_ranks_render_their_frames(tmp_path):
    oracle._load()                                     # build once, before the ranks start
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2,
                       start_method='spawn', join=True)
    ls = workloads.ragged_stack(seed=11, F=12, H=96, W=80, median=300.0)
    ref = np.zeros(ls.shape, np.float64)
    oracle.draw_lines(ref, ls.lines, ls.idxs, ls.max_val, ls.kernel, ls.overlap, 1)
    got = np.load(tmp_path / 'image.npy')
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
    assert np.isclose(np.load(tmp_path / 'loss.npy')[0], (ref ** 2).sum(), rtol=1e-12)


def _fit_rank_main(rank, world, port, tmpdir):
    """fit.shard_problem + fit.reduce_losses on CPU ranks: each rank's target frames,
    lines and rebased indices, its loss (the oracle's render in place of the GPU fit)
    and the summed loss"""
    from cbclib_v2_gb300 import fit
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        ls = workloads.fit_loop_stack(seed=21, F=5, H=64, W=72, per_frame=20)
        offs = ls.frame_offsets()
        target = torch.from_numpy(np.random.default_rng(3).random(ls.shape))
        sh, t, ln, ix = fit.shard_problem(target, torch.from_numpy(ls.lines), offs, rank, world)
        assert t.shape[0] == sh.n_frames and ln.shape[0] == sh.n_lines
        img = oracle.draw_lines(np.zeros(tuple(t.shape)), ln.numpy(), ix.numpy(), ls.max_val,
                                ls.kernel, ls.overlap, 1)
        mine = float(((img - t.numpy()) ** 2).sum())
        total = fit.reduce_losses([mine, 2 * mine])
        parts = [None] * world
        dist.all_gather_object(parts, (sh.f0, sh.f1, sh.l0, sh.l1, ix.numpy()))
        if rank == 0:
            np.save(os.path.join(tmpdir, 'total.npy'), np.array(total))
            np.save(os.path.join(tmpdir, 'parts.npy'), np.array(
                [p[:4] for p in parts], dtype=np.int64))
    finally:
        dist.destroy_process_group()


def test_two_cpu_ranks_split_a_fit(tmp_path):
    oracle._load()
    mp.start_processes(_fit_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2,
                       start_method='spawn', join=True)
    ls = workloads.fit_loop_stack(seed=21, F=5, H=64, W=72, per_frame=20)
    target = np.random.default_rng(3).random(ls.shape)
    img = oracle.draw_lines(np.zeros(ls.shape), ls.lines, ls.idxs, ls.max_val, ls.kernel,
                            ls.overlap, 1)
    want = float(((img - target) ** 2).sum())
    total = np.load(tmp_path / 'total.npy')
    assert np.isclose(total[0], want, rtol=1e-12) and np.isclose(total[1], 2 * want, rtol=1e-12)
    parts = np.load(tmp_path / 'parts.npy')
    assert parts[0][0] == 0 and parts[-1][1] == ls.shape[0] and parts[0][1] == parts[1][0]
    assert parts[0][2] == 0 and parts[-1][3] == ls.n_lines and parts[0][3] == parts[1][2]
