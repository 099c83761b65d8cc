"""Block sharding over ranks: the reference's multi-rank step with one rank per GPU.

The reference puts contiguous leaf ranges on MPI ranks (ModAllocation_Init,
3_6/ModAllocation.f90:25-39), moves the ghost entries that cross ranks in
per-peer packed messages (3_6/ModCommunication.f90:375-634, 725-765) and takes
the MIN of dt over ranks (3_6/ModAdvance.f90:48). The library gives the
partition and the per-peer entry lists (host side, no GPU needed) and, on a
sharded context, the pack/unpack of those entries on the GPU.

On CPU ranks (gloo, world size 2) the oracle computes each rank's blocks, the
library's plan says which entries travel, and the messages go through
torch.distributed: the 2-rank FP64 step is bit-identical to the 1-rank step.
On the GPU, two sharded contexts (ranks 0 and 1 of 2) run one after the other
in one process, their pack buffers passed between them on the host: the
result is bit-identical to one unsharded context. The path has not run on
several GPUs (every run here has one).
"""
import os
import socket

import numpy as np
import pytest

import falcon_gb300 as fg
import oracle
from falcon_gb300 import config, synth

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


@pytest.fixture(scope="module", autouse=True)
def _built(built_lib):
    return built_lib


def test_partition_is_the_reference_rule():
    f = fg.Falcon(config.shell_fp64_cpu(device=-1))
    assert f.nblocks == 864
    assert list(f.shard_ranges(3)) == [0, 288, 576, 864]
    # 864 = 5 x 172 + 4: the first four ranks hold one leaf more
    first = f.shard_ranges(5)
    assert list(np.diff(first)) == [173, 173, 173, 173, 172] and first[-1] == 864


def test_plan_lists_every_ghost_entry_once_in_matching_order():
    f = fg.Falcon(config.shell_fp64_cpu(device=-1))
    gm = f.ghost_map()
    R = 3
    first = f.shard_ranges(R)
    rank_of = lambda b: int(np.searchsorted(first, b, side="right") - 1)
    seen = np.zeros(len(gm), dtype=np.int32)
    for r in range(R):
        for p in range(R):
            send = f.shard_plan(R, r, p, fg.SHARD_SEND)
            recv = f.shard_plan(R, p, r, fg.SHARD_RECV)
            assert np.array_equal(send, recv)          # the sender's order is the receiver's
            assert (np.diff(send) > 0).all()           # in map order
            seen[send] += 1
            for k in send[:: max(1, len(send) // 50)]:
                assert rank_of(gm[k]["sblock"]) == r and rank_of(gm[k]["tblock"]) == p
    assert (seen == 1).all()
    cross = sum(len(f.shard_plan(R, r, p, fg.SHARD_SEND)) for r in range(R) for p in range(R) if p != r)
    assert 0 < cross < len(gm)


def _entries(gm, idx):
    e = gm[idx]
    ent = np.stack([e["tblock"], e["ti"], e["tj"], e["tk"], e["sblock"]], 1).astype(np.int32)
    return ent, np.ascontiguousarray(e["src_x"])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cpu_rank(rank, world, port, outdir, steps):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg = config.shell_fp64_cpu(device=-1)
        plan = fg.Falcon(cfg)                       # host side only: tree, ghost map, partition, plan
        gm = plan.ghost_map()
        first = plan.shard_ranges(world)
        o = oracle.Oracle(config.shell_fp64_cpu(device=-1))
        o.set_owned(int(first[rank]), int(first[rank + 1]))
        o.set_state(synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=1001))
        peers = [p for p in range(world) if p != rank]
        send = {p: _entries(gm, plan.shard_plan(world, rank, p, fg.SHARD_SEND)) for p in peers}
        recv = {p: _entries(gm, plan.shard_plan(world, rank, p, fg.SHARD_RECV)) for p in peers}

        def remote(rk):
            reqs, bufs = [], {}
            for p in peers:
                vals = torch.from_numpy(o.interp_entries(rk, *send[p]))
                reqs.append(dist.isend(vals, p))
                bufs[p] = torch.zeros((len(recv[p][0]), oracle.NVAR), dtype=torch.float64)
                reqs.append(dist.irecv(bufs[p], p))
            for q in reqs:
                q.wait()
            for p in peers:
                o.write_ghosts(rk, recv[p][0], bufs[p].numpy())

        for _ in range(2):                          # the two exchanges after an upload
            o.exchange()
            remote(False)
        for _ in range(steps):
            o.phase(0)
            dt = torch.tensor([o.dt()], dtype=torch.float64)
            dist.all_reduce(dt, op=dist.ReduceOp.MIN)
            o.set_dt(float(dt.item()))
            for ph in range(1, 6):
                o.phase(ph)
                remote(ph < 4)                      # stages 1-3 fill the stage buffer's ghosts
        u = o.get_state()
        np.save(os.path.join(outdir, "rank%d.npy" % rank), u[first[rank]:first[rank + 1]])
        np.save(os.path.join(outdir, "dt%d.npy" % rank), np.array([o.dt()]))
    finally:
        dist.destroy_process_group()


def test_two_cpu_ranks_step_bit_identical_to_one_rank(tmp_path):
    """cfg1 (864 blocks of 8^3): two gloo ranks, each computing its half of
    the blocks with the oracle and exchanging the library's per-peer entry
    lists, give after two steps exactly the one-rank state, every cell of
    every block (ghosts included), and the same dt."""
    world, steps = 2, 2
    mp.spawn(_cpu_rank, args=(world, _free_port(), str(tmp_path), steps), nprocs=world, join=True)
    cfg = config.shell_fp64_cpu(device=-1)
    o = oracle.Oracle(cfg)
    o.set_state(synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=1001))
    o.exchange()
    o.exchange()
    for _ in range(steps):
        o.step()
    ref = o.get_state()
    first = fg.Falcon(config.shell_fp64_cpu(device=-1)).shard_ranges(world)
    for r in range(world):
        part = np.load(os.path.join(str(tmp_path), "rank%d.npy" % r))
        assert np.array_equal(part, ref[first[r]:first[r + 1]]), r
        assert np.load(os.path.join(str(tmp_path), "dt%d.npy" % r))[0] == o.dt()


@pytest.mark.gpu
def test_gpu_sharded_contexts_step_bit_identical_to_one_context():
    """Ranks 0 and 1 of 2 as two sharded FP64 contexts on one GPU, run one
    after the other (no kernel waits on the other context): owned-block
    phases, the MIN of the local CFL minima, and pack -> host buffer ->
    unpack of the per-peer entries after every phase. After three steps each
    rank's blocks equal an unsharded context's bit for bit."""
    mk = lambda: config.shell_fp64_cpu()
    ref = fg.Falcon(mk())
    ranks = [fg.Falcon(mk()) for _ in range(2)]
    u0 = synth.initial_state(mk(), ref.block_ranges(), ref.block_flags(), seed=1001)
    ref.upload_state(u0)
    ref.exchange()
    ref.exchange()
    for r, f in enumerate(ranks):
        f.upload_state(u0)
        f.set_shard(2, r)
        n_send, n_recv = f.shard_counts(1 - r)
        assert n_send > 0 and n_recv > 0

    def remote():
        bufs = [f.shard_pack(1 - r) for r, f in enumerate(ranks)]
        for r, f in enumerate(ranks):
            f.shard_unpack(1 - r, bufs[1 - r])

    for _ in range(2):
        for f in ranks:
            f.exchange()
        remote()
    dts = []
    for _ in range(3):
        dts.append(ref.advance_rk4())
        for f in ranks:
            f.step_phase(0)
        m = min(f.shard_min_ratio() for f in ranks)
        for f in ranks:
            f.shard_set_min_ratio(m)
        for ph in range(1, 6):
            for f in ranks:
                f.step_phase(ph)
            remote()
    u = ref.download_state()
    first = ranks[0].shard_ranges(2)
    for r, f in enumerate(ranks):
        ur = f.download_state()
        assert np.array_equal(ur[first[r]:first[r + 1]], u[first[r]:first[r + 1]]), r
