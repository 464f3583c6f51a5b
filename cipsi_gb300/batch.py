"""Batched form of the engine: many geometries of a potential-curve grid
(Autocip runs one cip per geometry, Autocip_13/calcul.f90:320) evaluated in
one persistent launch per class, captured as a CUDA graph.

`load_geometries` generates seeded geometries in worker processes (one temp
directory each, in the reference's file formats), reads each into an engine
context on the GPU and removes the directory, so only a few exist at a time.
`autotune` picks the launch tuning (removed-electron blocks per work unit,
CTAs per SM) by timing a sub-batch.  `run_grid` runs a whole grid in
batches with a checkpoint per geometry, and resumes a stopped run.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import shutil
import tempfile
import time
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import engine, synth


def _gen_one(args):
    cfg, base = args
    wd = os.path.join(base, cfg.name)
    synth.generate(cfg, wd)
    return wd


def load_geometries(cfgs: Sequence[synth.SynthConfig], device: int = 0, workers: Optional[int] = None,
                    base: Optional[str] = None):
    """(inputs' opts, contexts) for every configuration, inputs on the GPU."""
    base = base or tempfile.mkdtemp(prefix="cipsi_geos_")
    workers = workers or max(1, min(16, (os.cpu_count() or 2) - 1))
    ctxs, opts = [], []
    ctx_mp = mp.get_context("spawn")
    try:
        with ctx_mp.Pool(workers) as pool:
            for wd in pool.imap(_gen_one, [(c, base) for c in cfgs]):
                inp = engine.Inputs(wd)
                ctx = engine.Context(inp.dims, device=device)
                ctx.upload(inp)
                opts.append(engine.Opts.from_buffer_copy(inp.opts))
                ctxs.append(ctx)
                inp.close()
                shutil.rmtree(wd, ignore_errors=True)
    finally:
        shutil.rmtree(base, ignore_errors=True)
    return opts, ctxs


def run_serial(ctxs, opts) -> Tuple[float, list]:
    """The plain form, one geometry after another: wall seconds, results."""
    res = []
    t0 = time.perf_counter()
    for c, o in zip(ctxs, opts):
        c.run_async(o)
        res.append(_fetch_allow_overflow(c))
    return time.perf_counter() - t0, res


def _fetch_allow_overflow(c):
    import ctypes
    r = engine.Result()
    rc = c.lib.cipsi_fetch_result(c._c, ctypes.byref(r))
    if rc not in (0, -4):
        raise engine.CipsiError(c.lib.cipsi_last_error(c._c).decode())
    d = engine.result_dict(r, c.dims.metat, getattr(c, "_last_nclass", engine.NCLASS))
    d["overflow"] = rc == -4
    return d


CANDIDATES: List[Tuple[int, int]] = [(6, 2), (3, 2), (12, 2), (6, 1), (12, 1)]


def autotune(ctxs, opts, sample: int = 16, candidates: Sequence[Tuple[int, int]] = CANDIDATES,
             repeats: int = 1) -> Tuple[Tuple[int, int], dict]:
    """Time each (r_chunk, ctas_per_sm) on a sub-batch of `sample` contexts
    spread over the batch's size range; return the fastest and all times."""
    order = np.argsort([c.dims.ncf * c.dims.norb for c in ctxs])
    pick = sorted(set(int(order[int(i)]) for i in np.linspace(0, len(ctxs) - 1, min(sample, len(ctxs)))))
    sub_c = [ctxs[i] for i in pick]
    sub_o = [opts[i] for i in pick]
    times = {}
    for cand in candidates:
        with engine.Batch(sub_c, sub_o, r_chunk=cand[0], ctas_per_sm=cand[1]) as b:
            b.run()
            b.wait()  # first replay: warm-up
            ms = []
            for _ in range(repeats):
                b.run()
                ms.append(b.wait())
            b.fetch_all()
        times[cand] = min(ms)
    best = min(times, key=times.get)
    return best, times


def run_batch(cfgs: Sequence[synth.SynthConfig], device: int = 0, r_chunk: int = 6, ctas_per_sm: int = 0,
              workers: Optional[int] = None) -> list:
    """The geometries of `cfgs` in one batched launch: each one's result."""
    opts, ctxs = load_geometries(cfgs, device=device, workers=workers)
    try:
        with engine.Batch(ctxs, opts, r_chunk=r_chunk, ctas_per_sm=ctas_per_sm) as b:
            b.run()
            b.wait()
            return b.fetch_all()
    finally:
        for c in ctxs:
            c.close()


def _result_path(results_dir: str, cfg: synth.SynthConfig) -> str:
    return os.path.join(results_dir, cfg.name + ".json")


# configuration fields saved with each result and compared on resume
_KEY_FIELDS = ("norb", "ncf", "metat", "seed", "curve_R")


def _saved_result(results_dir: str, cfg: synth.SynthConfig):
    """The saved result of `cfg`, or None when there is none to reuse: no
    file, a file that does not parse (cut short by a crash), or a file
    written for a different configuration under the same name (another
    seed, grid or system size in the same results directory)."""
    path = _result_path(results_dir, cfg)
    try:
        with open(path) as fh:
            rec = json.load(fh)
    except (OSError, ValueError):
        return None
    if not isinstance(rec, dict) or "result" not in rec:
        return None
    if any(rec.get(f) != getattr(cfg, f) for f in _KEY_FIELDS):
        return None
    return rec["result"]


def run_grid(cfgs: Sequence[synth.SynthConfig], results_dir: str, batch_size: int = 32, runner=run_batch,
             **runner_kw) -> dict:
    """A grid of geometries with checkpoints: the geometries run in batches of
    `batch_size`, and each one's result goes to results_dir/<name>.json
    (written to a temporary name, flushed to disk, then renamed, so a file is
    complete or absent) as soon as its batch finishes.  Geometries that
    already have a result for the same configuration (norb, ncf, metat, seed,
    curve_R) are not run again, so a run that stopped -- killed, out of time,
    a failed batch -- continues where it stopped when called again, as the
    Autocip driver re-reads finished geometries instead of recomputing them
    (Autocip_13/autocip13.f90:162, l_calc).  A result file that does not
    parse, or that was written for another configuration of the same name,
    is run again and replaced.  Returns every geometry's result by name."""
    os.makedirs(results_dir, exist_ok=True)
    names = [c.name for c in cfgs]
    if len(set(names)) != len(names):
        raise ValueError("geometry names must be unique: they name the result files")
    out = {}
    todo = []
    for c in cfgs:
        r = _saved_result(results_dir, c)
        if r is None:
            todo.append(c)
        else:
            out[c.name] = r
    for s in range(0, len(todo), batch_size):
        chunk = todo[s:s + batch_size]
        results = runner(chunk, **runner_kw)
        if len(results) != len(chunk):
            raise RuntimeError("the batch returned %d results for %d geometries" % (len(results), len(chunk)))
        for cfg, res in zip(chunk, results):
            rec = {f: getattr(cfg, f) for f in _KEY_FIELDS}
            rec.update(name=cfg.name, result=res)
            path = _result_path(results_dir, cfg)
            tmp = path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(rec, fh)
                fh.flush()
                os.fsync(fh.fileno())
            os.replace(tmp, path)
            out[cfg.name] = json.loads(json.dumps(res))
    return {c.name: out[c.name] for c in cfgs}
