"""Multi-rank voxel sharding on CPU (gloo, world size 2).

Each rank fits its contiguous voxel range (shard_range, CUDIMOT's
split_parts rule) with the voxel index offset by the range start, the ranks
gather the results and reduce their step times with MAX (as bench.py
does). Because the fit of a voxel depends only on the voxel and its global
index (MCMC draws are keyed by it), the gathered result must equal the
single-process fit exactly. The per-rank fit is the CPU oracle, and, where
a GPU is present, the library itself (both ranks on the one GPU, each
fitting its own voxels: no kernel of one rank waits on the other's)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from cudimot_gb300 import capi, parts


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _fit(meas, init, cfp, fixp, offset):
    from tests.helpers import oracle
    cfg = capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=50, njumps=100, sampleevery=10)
    o = oracle("Ball_1_Stick")
    p, _, _, _ = o.levmar(cfg, meas, init, cfp, fixp, threads=1)
    p, s, _ = o.mcmc(cfg, meas, p, cfp, fixp, threads=1, voxel_offset=offset)
    return p, s


def _fit_library(meas, init, cfp, fixp, offset):
    # explicit lane counts: the automatic choice widens groups for small calls
    cfg = capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=50, njumps=100, sampleevery=10,
                         lanes_levmar=4, lanes_mcmc=2, first_voxel=offset)
    dev = torch.device("cuda:0")
    lib = capi.Cudimot("Ball_1_Stick", cfg)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    p = t(init)
    s = torch.zeros(meas.shape[0], 5, 10, dtype=torch.float64, device=dev)
    lib.fit(t(meas), p, t(cfp), t(fixp), s)
    torch.cuda.synchronize()
    return p.cpu().numpy(), s.cpu().numpy()


def _worker(rank, world, port, data, out, fit="oracle"):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    meas, init, cfp, fixp = data
    a, b = parts.shard_range(meas.shape[0], world, rank)
    p, s = (_fit if fit == "oracle" else _fit_library)(meas[a:b], init[a:b], cfp, fixp[a:b], a)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    gathered = [None] * world
    dist.all_gather_object(gathered, (a, b, p, s))
    if rank == 0:
        out.put((t.item(), gathered))
    dist.barrier()
    dist.destroy_process_group()


def _run_ranks(wl, fit):
    data = (wl.meas, wl.init, wl.cfp, wl.fixp)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, data, q, fit)) for r in range(2)]
    for p in procs:
        p.start()
    tmax, gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert tmax == 2.0
    return gathered


def test_two_rank_shards_equal_single_process(built):
    from cudimot_gb300 import synth
    wl = synth.ball_1_stick(37, seed=5)  # odd size: the last shard takes the remainder
    gathered = _run_ranks(wl, "oracle")
    assert [(a, b) for a, b, _, _ in gathered] == [(0, 18), (18, 37)]
    p_all = np.concatenate([g[2] for g in gathered])
    s_all = np.concatenate([g[3] for g in gathered])
    p_ref, s_ref = _fit(wl.meas, wl.init, wl.cfp, wl.fixp, 0)
    assert np.array_equal(p_all, p_ref)
    assert np.array_equal(s_all, s_ref)


@pytest.mark.gpu
def test_two_rank_shards_through_library(built, cuda):
    from cudimot_gb300 import synth
    wl = synth.ball_1_stick(1001, seed=6)
    gathered = _run_ranks(wl, "library")
    assert [(a, b) for a, b, _, _ in gathered] == [(0, 500), (500, 1001)]
    p_all = np.concatenate([g[2] for g in gathered])
    s_all = np.concatenate([g[3] for g in gathered])
    p_ref, s_ref = _fit_library(wl.meas, wl.init, wl.cfp, wl.fixp, 0)
    assert np.array_equal(p_all, p_ref)
    assert np.array_equal(s_all, s_ref)


def test_shard_range_and_subparts():
    assert parts.shard_range(10, 3, 0) == (0, 3)
    assert parts.shard_range(10, 3, 2) == (6, 10)
    with pytest.raises(ValueError):
        parts.shard_range(2, 3, 0)
    # dMRI_Data.cu:65-79: a small last part is spread over the others
    assert parts.subparts(12800 * 2 + 100) == [(0, 12850), (12850, 25700)]
    assert parts.subparts(12800 + 7000) == [(0, 12800), (12800, 19800)]
    assert parts.subparts(100) == [(0, 100)]
