"""The multi-rank path of the binned sums (pg_gpu_gb300/shard.py) on the CPU:
shard planning, the per-rank anchor ranges and the sum of partials over a
gloo process group of two ranks, with the oracle as each rank's compute (the
device compute of an anchor range is checked against the oracle in
tests/test_gpu_tc.py)."""
import os
import socket

import numpy as np
import pytest

from oracle import ld_oracle as O

torch = pytest.importorskip("torch")
from pg_gpu_gb300 import shard as S  # noqa: E402


def _panel(seed, H=24, M=300):
    rng = np.random.default_rng(seed)
    hap = (rng.random((H, M)) < rng.uniform(0.1, 0.9, M)).astype(np.int8)
    hap[rng.random((H, M)) < 0.05] = -1
    pos = np.sort(rng.choice(60_000, M, replace=False)).astype(np.int64)
    return hap, pos


def _oracle_compute(hap, pos, rows, bins):
    def compute(s, e):
        sums, cnt = O.binned_sums(hap, pos, rows, bins, anchor_start=s, anchor_stop=e)
        return torch.as_tensor(np.asarray(sums, np.float64)), torch.as_tensor(np.asarray(cnt, np.int64))
    return compute


@pytest.mark.parametrize("world", [1, 2, 3, 5, 8])
def test_plan_covers_anchors_with_halos_and_balance(world):
    _, pos = _panel(world)
    md = 5_000.0
    shards = S.plan_shards(pos, md, world)
    assert len(shards) == world and shards[0].start == 0 and shards[-1].stop == len(pos)
    for a, b in zip(shards, shards[1:]):
        assert a.stop == b.start
    jend = np.searchsorted(pos, pos + md, side="right")
    per = jend - np.arange(len(pos)) - 1
    for sh in shards:
        if sh.stop > sh.start:
            # every partner of every anchor lies inside the halo
            assert sh.halo == jend[sh.stop - 1] and sh.halo >= sh.stop
    loads = [int(per[sh.start:sh.stop].sum()) for sh in shards]
    assert sum(loads) == int(per.sum())
    assert max(loads) <= per.sum() / world + per.max() + 1


def test_plan_edge_cases():
    assert [(s.start, s.stop) for s in S.plan_shards([], 10, 3)] == [(0, 0)] * 3
    sh = S.plan_shards([5.0], 10, 2)
    assert sum(s.stop - s.start for s in sh) == 1
    with pytest.raises(ValueError):
        S.plan_shards([3.0, 1.0], 10, 2)
    with pytest.raises(ValueError):
        S.plan_shards([1.0, 2.0], 10, 0)


@pytest.mark.parametrize("world", [2, 3, 4])
def test_shard_partials_sum_to_the_whole(world):
    hap, pos = _panel(10 + world)
    bins = np.array([0.0, 500.0, 2_000.0, 8_000.0])
    rows = [np.arange(0, 12), np.arange(12, 24)]
    compute = _oracle_compute(hap, pos, rows, bins)
    tot_s, tot_c = compute(0, len(pos))
    acc_s = torch.zeros_like(tot_s)
    acc_c = torch.zeros_like(tot_c)
    for sh in S.plan_shards(pos, bins[-1], world):
        part = S.shard_partial(compute, sh)
        if part is not None:
            acc_s += part[0]
            acc_c += part[1]
    assert torch.equal(acc_c, tot_c)
    torch.testing.assert_close(acc_s, tot_s, rtol=1e-12, atol=1e-12 * float(tot_s.abs().max()))


def _gloo_rank(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        hap, pos = _panel(7)
        bins = np.array([0.0, 1_000.0, 4_000.0, 8_000.0])
        rows = [np.arange(0, 12), np.arange(12, 24)]
        sh = S.plan_shards(pos, bins[-1], world)[rank]
        part = S.shard_partial(_oracle_compute(hap, pos, rows, bins), sh)
        assert part is not None
        sums, cnt = S.reduce_partials(part[0].clone(), part[1].clone())
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), sums=sums.numpy(), cnt=cnt.numpy())
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_gloo_two_ranks_reduce_to_the_oracle(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_gloo_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    hap, pos = _panel(7)
    bins = np.array([0.0, 1_000.0, 4_000.0, 8_000.0])
    ref_s, ref_c = O.binned_sums(hap, pos, [np.arange(0, 12), np.arange(12, 24)], bins)
    for r in range(2):
        z = np.load(tmp_path / f"rank{r}.npz")
        assert np.array_equal(z["cnt"], np.asarray(ref_c))
        np.testing.assert_allclose(z["sums"], ref_s, rtol=1e-12,
                                   atol=1e-12 * float(np.abs(ref_s).max()))
