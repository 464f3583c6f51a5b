"""Multi-rank generator sharding, checked on CPU ranks (gloo, world size 2):
each rank runs the oracle on its generator mask (rank 0 also runs pertu's
reference candidates), the per-root sums and counters are all-reduced, and
the result equals the unsharded run.  The same masks drive the GPU engine
(cipsi_opts.gen_mask / run_pertu) in bench.py --gpus N."""
import json
import os
import shutil

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from cipsi_gb300 import shard, synth
from oracle import build as ob


def _worker(rank, world, wd, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    run = wd + f"_r{rank}"
    shutil.rmtree(run, ignore_errors=True)
    shutil.copytree(wd, run)
    ncf = json.load(open(os.path.join(wd, "info.json")))["ncf"]
    mask = shard.generator_mask(ncf, rank, world)
    mpath = os.path.join(run, "mask.bin")
    mask.tofile(mpath)
    j = json.load(open(ob.run(run, genmask=mpath, no_pertu_ref=(rank != 0))))
    v = torch.from_numpy(shard.flatten(j))
    dist.all_reduce(v)
    dp = torch.tensor([j["dpivot"]], dtype=torch.float64)
    dist.all_reduce(dp, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((v.numpy().tolist(), float(dp[0])))
    dist.destroy_process_group()


def test_two_rank_generator_sharding(tmp_path, oracle_exe):
    cfg = synth.SynthConfig("sh", norb=12, nocc=4, ncholesky=12, ncf=60, metat=2, tau=0.02,
                            ranks=(1, 2, 3), coef_mode="decay09", seed=21)
    wd = str(tmp_path / "in")
    info = synth.generate(cfg, wd)
    json.dump(info, open(os.path.join(wd, "info.json"), "w"))
    full = str(tmp_path / "full")
    shutil.copytree(wd, full)
    jf = json.load(open(ob.run(full)))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, wd, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    vals, dpiv = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = shard.flatten(jf)
    np.testing.assert_allclose(np.array(vals), ref, rtol=1e-12, atol=1e-12)
    assert dpiv == jf["dpivot"]
