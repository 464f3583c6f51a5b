#!/usr/bin/env python3
"""Benchmark of the CIPSI perturbation / selection step on GB300.

Workload (default "large", the configuration the engine's target is quoted
on): 120 orbitals, 30 electrons (Ms = 0), S = 20,000 determinants (the
reference plus doubles, spin-flip closed), 2 roots, MP + EN partitions,
selection threshold 0.005; seeded synthetic integrals (240 Cholesky
vectors).  "--workload medium": 60 orbitals, 20 electrons, S = 2000
(singles/doubles/triples), 3 roots, threshold 0.01.

A step is one full pass of the hot path (the work of pertu + diexcit) over
the workload, with every selected perturber's unit-60 record produced.
Metric: perturber contributions per second, one contribution being one
(perturber that reaches the E2 loop, root) term.

  value   device time of a streamed run (cipsi_run_pt2_stream without a
          consumer: the records are made and gathered in device memory,
          chunk after chunk), inputs resident in HBM, L2 flushed (256 MiB
          write) before every step;
  e2e     the same through the C ABI from host buffers: every step uploads
          the inputs (cipsi_inputs_upload) and streams the run to a consumer
          that folds every record, in order, into a digest on the host cores
          (cipsi_record_digest): the unit-60 records are delivered to host
          memory inside the timed region;
  cpu_baseline  the CPU oracle (a restatement of the reference's loop nest)
          on one core, on a systematic sample of one generator's candidates.

--impl reference times that CPU restatement on all host cores: one
long-lived process per core reads the inputs once and runs one sampled
generator per step (its own clock around the perturbation loop); the
reference's Fortran cannot be built here (no Fortran compiler).

For --gpus N (torchrun), every rank runs its own instance of the workload
(seed + rank: independent geometries, as the Autocip driver runs its grid), so
per-GPU work is fixed (weak scaling); value = all contributions / max time.
"""
from __future__ import annotations

import argparse
import hashlib
import importlib.util
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "perturber contributions/s"
UNIT = "contributions/s"
WORKLOADS = {
    "large": {"workload": "large: 120 MOs, 30 e-, Ms=0, S=20000 dets (ref + doubles, spin-flip closed), "
                          "2 roots, MP+EN, tau=0.005",
              "norb": 120, "electrons": 30, "ncf": 20000, "roots": 2, "tau": 0.005},
    "medium": {"workload": "medium: 60 MOs, 20 e-, Ms=0, S=2000 dets (ref+S/D/T, spin-flip closed), "
                           "3 roots, MP+EN, tau=0.01",
               "norb": 60, "electrons": 20, "ncf": 2000, "roots": 3, "tau": 0.01},
}
# systematic CPU sample: one candidate (and one diexcit quadruple) in
# CPU_SAMPLE of the sampled generators, per process and step
CPU_SAMPLE = {"large": 200, "medium": 10}


def workload_desc(name: str) -> dict:
    d = dict(WORKLOADS[name])
    d["l2"] = "flushed before each step (256 MiB write)"
    d["records"] = "every selected perturber's unit-60 record made each step (value: in device memory; " \
                   "e2e: delivered to host memory and folded into a digest)"
    return d


def _synth():
    """The synthetic-input generator, loaded from its file (numpy only), so
    the reference arm runs without importing the engine's package."""
    mod = sys.modules.get("cipsi_synth")
    if mod is None:
        spec = importlib.util.spec_from_file_location("cipsi_synth", os.path.join(ROOT, "cipsi_gb300", "synth.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules["cipsi_synth"] = mod
        spec.loader.exec_module(mod)
    return mod


def make_workload(name: str, seed_offset: int, base: str):
    import dataclasses
    synth = _synth()
    cfg = dataclasses.replace(synth.CONFIGS[name])
    cfg.seed = cfg.seed + seed_offset
    wd = os.path.join(base, f"{name}_s{cfg.seed}")
    info = synth.generate(cfg, wd)
    return wd, info


# ------------------------------------------------------------ clocks sampler
class Clocks:
    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------ CPU baseline
def sample_plan(ncf: int, ysaut, nsteps: int, nproc: int, sample: int, seed: int = 7):
    """Per process, one line per step: (residue, generator).  Generators are
    drawn without repetition from the determinants of S that are not
    spin-flip partners (the generators); residue m keeps one candidate in
    `sample`, in enumeration order."""
    import numpy as np
    rng = np.random.default_rng(seed)
    gens = [k for k in range(ncf) if not ysaut[k]]
    pick = rng.choice(len(gens), size=min(len(gens), nsteps * nproc), replace=False)
    lines = [[] for _ in range(nproc)]
    for i, g in enumerate(pick):
        c, st = i % nproc, i // nproc
        if st < nsteps:
            lines[c].append((int(rng.integers(0, sample)), gens[int(g)] + 1))
    return lines


def oracle_plan(wd: str, lines, sample: int, tmpbase: str):
    """One oracle process on its plan (inputs read once): [(perturbers,
    loop seconds)] per line, by the oracle's own clock, and metat."""
    from oracle import build as ob
    run = tempfile.mkdtemp(dir=tmpbase)
    for f in os.listdir(wd):  # the integrals are only read: linked, not copied
        src = os.path.join(wd, f)
        if f == "ijkl":
            os.symlink(src, os.path.join(run, f))
        elif os.path.isfile(src):
            shutil.copy(src, os.path.join(run, f))
    plan = os.path.join(run, "plan.txt")
    with open(plan, "w") as fh:
        for m, k in lines:
            fh.write(f"{m} {k}\n")
    j = json.load(open(ob.run(run, sample=sample, plan=plan)))
    shutil.rmtree(run, ignore_errors=True)
    return [(int(n), float(t)) for n, t in j["plan"]], int(j["metat"])


def _ysaut(wd: str, info: dict):
    """Spin-flip partner flags of S from the generator's output (partners
    follow their representative in the file)."""
    synth = _synth()
    flags = []
    for r in synth.read_records(os.path.join(wd, "det")):
        import struct
        m, n = struct.unpack_from("<ii", r, 0)
        idet = struct.unpack_from(f"<{m}i", r, 8)
        nex = struct.unpack_from(f"<{n}i", r, 8 + 4 * m)
        pos = 0
        for ne in nex:
            flags.append((tuple(idet[pos:pos + 2 * ne:2]), tuple(idet[pos + 1:pos + 2 * ne:2])))
            pos += 2 * ne
    norb = info["norb"]
    seen, out = set(), []
    for h, p in flags:
        fl = (tuple(sorted((x - norb if x > norb else x + norb) for x in h)),
              tuple(sorted((x - norb if x > norb else x + norb) for x in p)))
        out.append(1 if fl in seen and fl != (h, p) else 0)
        seen.add((h, p))
    return out


def run_reference(args, rank: int, world: int):
    """CPU restatement on all host cores; rank 0 only.  One long-lived
    oracle process per core reads the inputs once, then runs one sampled
    generator per step (W + K lines); a step's time is the slowest
    process's loop time for that line, by the oracle's own clock."""
    if rank != 0:
        return
    from concurrent.futures import ProcessPoolExecutor
    import multiprocessing as mpm
    from oracle import build as ob
    ob.build()
    base = tempfile.mkdtemp(prefix="cipsi_ref_bench_")
    wd, info = make_workload(args.workload, 0, base)
    ncores = os.cpu_count() or 1
    sample = CPU_SAMPLE[args.workload]
    nsteps = args.warmup + args.steps
    plans = sample_plan(info["ncf"], _ysaut(wd, info), nsteps, ncores, sample)
    ctx = mpm.get_context("spawn")
    with ProcessPoolExecutor(max_workers=ncores, mp_context=ctx) as ex:
        futs = [ex.submit(oracle_plan, wd, plans[c], sample, base) for c in range(ncores)]
        res = [f.result() for f in futs]
    shutil.rmtree(base, ignore_errors=True)
    metat = res[0][1]
    contrib = tot_t = 0.0
    for st in range(args.warmup, nsteps):
        step = [r[0][st] for r in res if st < len(r[0])]
        contrib += sum(n for n, _ in step) * metat
        tot_t += max(t for _, t in step)
    val = contrib / tot_t
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded integrals and reference space)", "config": workload_desc(args.workload),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": f"each step: {ncores} processes (inputs read once per process), each on "
                                       f"one generator of S with 1 candidate in {sample} kept (systematic "
                                       "sample); rate = contributions / slowest loop time; extrapolated"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ batched form
def run_batched(args, rank: int, world: int, local_rank: int):
    """Potential-curve batch: `--geometries` seeded geometries (norb 40..100,
    |S| 500..5000, 1 root) run (a) one after another through the plain form
    and (b) as one batch (one persistent launch per class, CUDA graph, tuning
    picked by the autotuner on a sub-batch).  Metric: geometries per second."""
    import numpy as np
    import torch
    from cipsi_gb300 import batch, build, engine, synth
    torch.cuda.set_device(local_rank)
    build.build()
    cfgs = synth.curve_geometries(args.geometries, seed=100 + rank)
    t0 = time.perf_counter()
    opts, ctxs = batch.load_geometries(cfgs, device=local_rank)
    t_load = time.perf_counter() - t0
    ng = len(ctxs)
    clocks = Clocks(local_rank)
    # plain form, serially (first pass sizes the buffers, second is timed)
    batch.run_serial(ctxs, opts)
    torch.cuda.synchronize()
    clocks.start()
    t_serial, res_serial = batch.run_serial(ctxs, opts)
    serial_kernel_ms = sum(r["kernel_ms"] for r in res_serial)
    # autotuner on a sub-batch, then the batch with the chosen tuning
    best, tune_ms = batch.autotune(ctxs, opts, sample=16)
    b = engine.Batch(ctxs, opts, r_chunk=best[0], ctas_per_sm=best[1])
    for _ in range(args.batch_warmup):
        b.run()
        b.wait()
        b.fetch_all()
    dev_ms, wall = [], []
    for _ in range(args.batch_steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        b.run()
        dev_ms.append(b.wait())
        res_b = b.fetch_all()
        wall.append(time.perf_counter() - t1)
    clk = clocks.stop()
    ok = all(rb["n_processed"] == rs["n_processed"] and rb["ietat"] == rs["ietat"]
             for rb, rs in zip(res_b, res_serial))
    b.close()
    line = {"metric": "geometries/s (batched form)", "value": ng / (statistics.mean(dev_ms) / 1e3),
            "unit": "geometries/s", "n_gpus": world, "steps": args.batch_steps, "warmup": args.batch_warmup,
            "ms_per_step": statistics.mean(dev_ms), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded potential-curve geometries)",
            "config": {"workload": f"{ng} geometries, R uniform [2,12] bohr, norb uniform 40..100, "
                                   "|S| uniform 500..5000, 20 e-, 1 root, tau 0.01",
                       "geometries": ng, "perturbers": int(sum(r["n_processed"] for r in res_b))},
            "batched": {"device_ms": statistics.mean(dev_ms), "wall_ms": 1e3 * statistics.mean(wall),
                        "geometries_per_s_wall": ng / statistics.mean(wall), "tuning": list(best),
                        "autotune_ms": {f"{k[0]},{k[1]}": v for k, v in tune_ms.items()}},
            "plain_serial": {"wall_ms": 1e3 * t_serial, "kernel_ms_sum": serial_kernel_ms,
                             "geometries_per_s": ng / t_serial},
            "speedup_wall": t_serial / statistics.mean(wall),
            "same_counts_as_plain": ok, "load_s": t_load, "clocks": clk}
    for c in ctxs:
        c.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------ moy form
MOY_WORKLOAD = ("moy over S: 60 MOs, 20 e-, Ms=0, {n} determinants (ref + singles/doubles/triples, "
                "spin-flip closed), the list of the run that only writes S (Autocip's moy input)")


def _moy_workdir(base: str, ndet: int, seed: int) -> str:
    """Synthetic inputs of the moy form: the medium system's integrals and a
    list of `ndet` determinants; unit 4 and unit 60 from the run that only
    writes S (ityper = -1, host only), as Autocip feeds moy."""
    import dataclasses
    synth = _synth()
    cfg = dataclasses.replace(synth.CONFIGS["medium"], name="moy", ncf=ndet, metat=2, seed=seed,
                              energy="diagonal")
    wd = os.path.join(base, f"moy_{ndet}_{seed}")
    synth.generate(cfg, wd)
    txt = open(os.path.join(wd, "cip.in")).read().replace(f"ityper={cfg.ityper}", "ityper=-1")
    open(os.path.join(wd, "cip.in"), "w").write(txt)
    with open(os.path.join(wd, "moy.in"), "w") as fh:
        fh.write(" &moyfil\n &end\n &moyen\n  tau=0d0, title='moy'\n &end\n")
    return wd


def run_moy_form(args, rank: int, world: int, local_rank: int):
    """The moy drop-in (cipsi_moy_main): the Hamiltonian over a list of
    --moy-dets determinants.  value: pair tests per second of the two GPU
    passes (count + fill, device time of the library's events); e2e: the
    whole drop-in (read the files, build the list, the GPU passes, write
    units 1, 61, 64); cpu_baseline: the oracle's restatement of moy on a
    smaller list of the same recipe, extrapolated by the number of pair
    tests (they grow as n^2)."""
    import torch
    import cipsi_gb300 as cg
    from cipsi_gb300 import build
    torch.cuda.set_device(local_rank)
    build.build()
    base = tempfile.mkdtemp(prefix=f"cipsi_moy_r{rank}_")
    t0 = time.perf_counter()
    wd = _moy_workdir(base, args.moy_dets, 7 + rank)
    cg.run_cip(wd)  # ityper = -1: S ordered and written back, unit 4 (host only)
    t_gen = time.perf_counter() - t0
    for _ in range(args.warmup):
        j = cg.run_moy(wd)
    n = j["ncf"]
    tests = n * (n - 1) // 2
    clocks = Clocks(local_rank)
    clocks.start()
    dev_ms, wall = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        j = cg.run_moy(wd)
        wall.append(time.perf_counter() - t1)
        dev_ms.append(j["hbuild_ms"])
    clk = clocks.stop()
    line = {"metric": "moy pair tests/s", "value": tests / (statistics.mean(dev_ms) / 1e3), "unit": "pair tests/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(dev_ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded integrals and determinant list)",
            "config": {"workload": MOY_WORKLOAD.format(n=n), "determinants": n,
                       "l2": "the list (<= 3.2 MB) stays L2-resident by design; inputs re-read from files each step"},
            "e2e": {"value": tests / statistics.mean(wall), "unit": "pair tests/s", "ms_per_step":
                    1e3 * statistics.mean(wall), "h2d_bytes_per_step": int(n * 32),
                    "d2h_bytes_per_step": int(j["pairs"] * 12 + 4 * n)},
            "gpu_launches": 2 * args.steps,
            "work": {"pairs_within_two": j["pairs"], "unit1_elements": j["nhij"], "unit1_records": j["unit1_records"],
                     "generation_s": t_gen},
            "clocks": clk}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import subprocess
        from oracle import build as ob
        exe = ob.build()
        ws = _moy_workdir(base, args.moy_cpu_dets, 7)
        cg.run_cip(ws)
        with open(os.path.join(ws, "moy.in")) as fin:
            subprocess.run([exe, "--moy", "--json", "moy_ref.json"], cwd=ws, stdin=fin, stdout=subprocess.DEVNULL,
                           check=True)
        jr = json.load(open(os.path.join(ws, "moy_ref.json")))
        ns = jr["ncf"]
        line["cpu_baseline"] = {"value": ns * (ns - 1) // 2 / jr["hloop_s"], "unit": "pair tests/s", "cores": 1,
                                "kind": "port",
                                "sample": f"the oracle's moy over {ns} determinants of the same recipe, its own "
                                          f"clock around the matrix loop ({jr['hloop_s']:.1f} s, unit 1 written); "
                                          "rate extrapolated to the full list (pair tests grow as n^2)"}
    shutil.rmtree(base, ignore_errors=True)
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------ bd form
def _unit1_csr(path: str, n: int):
    """moy's unit 1 (8192-element records of row, column, value; the last
    record holds its count in jtab(8192)) as the full symmetric matrix
    L + L^T in scipy CSR form (the diagonal is stored halved)."""
    import numpy as np
    import scipy.sparse as sp
    lsize = 8192
    synth = _synth()
    rows, cols, vals = [], [], []
    recs = synth.read_records(path)
    for k, r in enumerate(recs):
        it = np.frombuffer(r, dtype="<i4", count=lsize, offset=0)
        jt = np.frombuffer(r, dtype="<i4", count=lsize, offset=4 * lsize)
        vb = np.frombuffer(r, dtype="<f8", count=lsize, offset=8 * lsize)
        m = int(jt[lsize - 1]) if k == len(recs) - 1 else lsize
        rows.append(it[:m] - 1)
        cols.append(jt[:m] - 1)
        vals.append(vb[:m])
    L = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    return (L + L.T).tocsr()


def run_bd_form(args, rank: int, world: int, local_rank: int):
    """The bd drop-in (cipsi_bd_main): the lowest roots of moy's matrix over
    --moy-dets determinants by the block Davidson iteration on the GPU.
    value: seconds of the Davidson solve (the library's clock around it);
    e2e: the whole drop-in (read unit 1 and unit 4, the solve, write units
    59 and 33).  cpu_baseline: scipy's Lanczos (ARPACK eigsh) on the host
    cores for the same roots of the same matrix to the same residual, the
    reference's own bd being Fortran that cannot be built here."""
    import numpy as np
    import torch
    import cipsi_gb300 as cg
    from cipsi_gb300 import build
    torch.cuda.set_device(local_rank)
    build.build()
    base = tempfile.mkdtemp(prefix=f"cipsi_bd_r{rank}_")
    t0 = time.perf_counter()
    wd = _moy_workdir(base, args.moy_dets, 7 + rank)
    cg.run_cip(wd)
    jm = cg.run_moy(wd)
    with open(os.path.join(wd, "bd.in"), "w") as fh:
        fh.write(" &bdfil\n &end\n &option\n  ncper=800, test=0.3d-3, qwvec=t\n &end\n")
    t_gen = time.perf_counter() - t0
    for _ in range(args.warmup):
        j = cg.run_bd(wd)
    clocks = Clocks(local_rank)
    clocks.start()
    solve, wall = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        j = cg.run_bd(wd)
        wall.append(time.perf_counter() - t1)
        solve.append(j["davidson_s"])
    clk = clocks.stop()
    n, netat = j["ncf"], len(j["eigenvalues"])
    H = _unit1_csr(os.path.join(wd, "mat"), n)
    ev = np.array(j["eigenvalues"])
    line = {"metric": "bd lowest roots: solve time", "value": statistics.mean(solve), "unit": "s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(solve), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded integrals and determinant list)",
            "config": {"workload": f"bd over moy's matrix of {n} determinants ({MOY_WORKLOAD.format(n=n)}), "
                                   f"{netat} roots, every residual norm below 1e-8 Eh",
                       "determinants": n, "roots": netat, "matrix_elements": int(H.nnz)},
            "e2e": {"value": statistics.mean(wall), "unit": "s", "ms_per_step": 1e3 * statistics.mean(wall),
                    "h2d_bytes_per_step": int(jm["nhij"] * 16), "d2h_bytes_per_step": int(8 * n * netat)},
            "gpu_launches": None,
            "work": {"iterations": j["iterations"], "eigenvalues": j["eigenvalues"], "residuals": j["residuals"],
                     "generation_s": t_gen},
            "clocks": clk}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import scipy.sparse.linalg as spl
        t1 = time.perf_counter()
        w, v = spl.eigsh(H, k=netat, which="SA", tol=1e-10)
        t_cpu = time.perf_counter() - t1
        order = np.argsort(w)
        w, v = w[order], v[:, order]
        res = [float(np.linalg.norm(H @ v[:, m] - w[m] * v[:, m])) for m in range(netat)]
        line["cpu_baseline"] = {"value": t_cpu, "unit": "s", "cores": os.cpu_count(), "kind": "library",
                                "sample": "scipy.sparse.linalg.eigsh (ARPACK Lanczos, tol 1e-10) on the same "
                                          f"matrix, the same {netat} roots; residual norms {res}",
                                "max_abs_eigenvalue_diff": float(np.max(np.abs(w - ev)))}
    shutil.rmtree(base, ignore_errors=True)
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------ adjoint form
def run_adjoint_form(args, rank: int, world: int, local_rank: int):
    """The medium system plus a seeded symmetric dipole matrix mu ~ N(0, 0.5):
    dE2/dh and dE2/d(pq|rs) from one backward pass (and E2 with dE2/dh from
    one one-electron adjoint pass), checked against central
    differences (step 1e-5) on `--fd-elements` random integrals and the
    dipole sum mu_pq dE2/dh_pq against finite-field runs at F = +-1e-4
    (integrals in FP64 on the device)."""
    import dataclasses
    import numpy as np
    import torch
    from cipsi_gb300 import adjoint, build, synth
    torch.cuda.set_device(local_rank)
    build.build()
    cfg = synth.CONFIGS["medium"]
    base = tempfile.mkdtemp(prefix="cipsi_adj_")
    wd = os.path.join(base, "sys")
    synth.generate(cfg, wd)
    h, L, _ = synth.make_integrals(cfg, np.random.default_rng(cfg.seed))
    S = adjoint.System(wd, device=local_rank)
    eri = S.pk.pack_from_cholesky(L, S.ninte)
    n, mt = cfg.norb, S.dims.metat
    ti, tj = np.tril_indices(n)
    h_tri = np.zeros(n * (n + 1) // 2)
    h_tri[adjoint._tri(ti, tj)] = h[ti, tj]
    rng = np.random.default_rng(12345)
    mu = rng.normal(0.0, 0.5, size=(n, n))
    mu = 0.5 * (mu + mu.T)
    seed = np.zeros((3, mt))
    seed[1, 0] = 1.0  # e2vp of the first root
    args_e = [x.numpy().copy() for x in S.engine_inputs(torch.as_tensor(h_tri), torch.as_tensor(eri))]
    eng = [args_e[0], args_e[1], args_e[2], eri.copy(), args_e[3], args_e[4], args_e[5], args_e[6]]
    S.run_engine(*[torch.as_tensor(x) for x in eng])  # warm-up (sizes the buffers)
    fwd_ms, adj_ms, one_ms = [], [], []
    e2_fwd = S.run_engine(*[torch.as_tensor(x) for x in eng])
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        S.run_engine(*[torch.as_tensor(x) for x in eng])
        fwd_ms.append(1e3 * (time.perf_counter() - t0))
        t0 = time.perf_counter()
        g = S.ctx.adjoint(S.opts, seed)  # at the inputs the forward above loaded
        adj_ms.append(1e3 * (time.perf_counter() - t0))
        t0 = time.perf_counter()
        e2_1e, g1 = S.ctx.adjoint_1e(S.opts, seed)
        one_ms.append(1e3 * (time.perf_counter() - t0))
    # the one-electron pass against the full adjoint and the forward sums
    one_check = {"max_rel_diff_e2": float(np.max(np.abs(e2_1e - e2_fwd)) / np.max(np.abs(e2_fwd))),
                 "max_rel_diff_gF": float(np.max(np.abs(g1["F"] - g["F"])) / np.max(np.abs(g["F"])))}
    # finite differences on random integrals the sums depend on
    nz = np.nonzero(g["eri"])[0]
    picks = rng.choice(nz, min(args.fd_elements, len(nz)), replace=False)
    step, worst = 1e-5, 0.0
    for i in picks:
        v = []
        for sgn in (1.0, -1.0):
            a = [x.copy() for x in eng]
            a[3][i] += sgn * step
            v.append(float((S.run_engine(*[torch.as_tensor(x) for x in a]) * seed).sum()))
        fd = (v[0] - v[1]) / (2 * step)
        worst = max(worst, abs(g["eri"][i] - fd) / max(1.0, abs(fd)))
    # dipole: one backward pass against two finite-field runs
    def dipole_check(system, h_t, eri_t):
        t0 = time.perf_counter()
        d_full = adjoint.dipole(system, h_t, eri_t, mu, seed, one_electron=False)
        t_full = time.perf_counter() - t0
        t0 = time.perf_counter()
        d_adj = adjoint.dipole(system, h_t, eri_t, mu, seed)  # one-electron adjoint pass
        t_dip = time.perf_counter() - t0
        mu_tri = np.zeros_like(h_t)
        mu_tri[adjoint._tri(ti, tj)] = mu[ti, tj]
        ff = {}
        t0 = time.perf_counter()
        for field in (1e-4, 1e-5):
            e = []
            for sgn in (1.0, -1.0):
                with torch.no_grad():
                    E = system.e2(torch.as_tensor(h_t + sgn * field * mu_tri), torch.as_tensor(eri_t))
                e.append(float((E.numpy() * seed).sum()))
            ff[f"{field:g}"] = (e[0] - e[1]) / (2 * field)
        t_ff = (time.perf_counter() - t0) / 2
        return {"adjoint": d_adj, "forward_plus_full_backward": d_full, "finite_field": ff,
                "abs_diff_1e-4": abs(d_adj - ff["0.0001"]), "adjoint_s": t_dip,
                "forward_plus_full_backward_s": t_full, "finite_field_s": t_ff}

    dip = dipole_check(S, h_tri, eri)
    S.close()
    # the same sizes with a near-ground-state first root (HF = 1, the other
    # coefficients N(0, 0.002)) and a 3 Eh occupied/virtual gap: the EN
    # denominators of root 1 stay away from zero, the finite-field difference
    # converges and checks the dipole
    cfg_w = dataclasses.replace(cfg, name="medium_hf_gap", virt_shift=3.0, coef_mode="gauss005",
                                coef_sigma=0.002)
    wd_w = os.path.join(base, "gap")
    synth.generate(cfg_w, wd_w)
    h_w, L_w, _ = synth.make_integrals(cfg_w, np.random.default_rng(cfg_w.seed))
    S = adjoint.System(wd_w, device=local_rank)
    eri_w = S.pk.pack_from_cholesky(L_w, S.ninte)
    h_tri_w = np.zeros(n * (n + 1) // 2)
    h_tri_w[adjoint._tri(ti, tj)] = h_w[ti, tj]
    dip_w = dipole_check(S, h_tri_w, eri_w)
    S.close()
    shutil.rmtree(base, ignore_errors=True)
    line = {"metric": "adjoint dE2/d(h, (pq|rs)): backward / forward time", "value": statistics.mean(adj_ms)
            / statistics.mean(fwd_ms), "unit": "ratio", "n_gpus": 1, "steps": args.steps, "warmup": 1,
            "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded medium system + dipole)",
            "config": {"workload": "medium (60 MOs, S = 2000, 3 roots), integrals in FP64, seed on e2vp[0]"},
            "forward_ms": statistics.mean(fwd_ms), "adjoint_ms": statistics.mean(adj_ms),
            "adjoint_1e_ms": statistics.mean(one_ms), "adjoint_1e_check": one_check,
            # cost of dE2/dh for a field direction, in forward runs: the
            # one-electron pass (E2 included), a forward plus the full
            # backward, a central finite difference, ffield.f90's 3-point fit
            "dipole_cost_in_forward_runs": {
                "one_electron_adjoint": statistics.mean(one_ms) / statistics.mean(fwd_ms),
                "forward_plus_full_backward": 1.0 + statistics.mean(adj_ms) / statistics.mean(fwd_ms),
                "finite_field_central": 2.0, "finite_field_three_point_fit": 3.0},
            "fd_check": {"elements": len(picks), "step": step, "max_rel_err": worst},
            "dipole_medium": dip, "dipole_medium_near_ground_state": dip_w,
            "note": "the medium recipe (random decay-0.9 roots) has EN denominators near zero, so its "
                    "finite-field differences do not converge with the field; the near-ground-state "
                    "variant of the same sizes is the dipole check"}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------ GPU arm
KERNEL_SOURCES = ["pt2_kernel.cuh", "pt2_common.cuh", "pt2_w1.cu", "pt2_w2.cu"]


def kernel_sha() -> str:
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "cipsi_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def kernel_profile(workload: str):
    """The ncu figures of k_pt2 on this workload (profiles/k_pt2_<workload>.json)
    when they were captured on the current kernel sources, else None."""
    path = os.path.join(ROOT, "profiles", f"k_pt2_{workload}.json")
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    return d if d.get("kernel_sha") == kernel_sha() else None


def run_gpu(args, rank: int, world: int, local_rank: int):
    import numpy as np
    import torch
    from cipsi_gb300 import build, engine
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    build.build()
    base = tempfile.mkdtemp(prefix=f"cipsi_bench_r{rank}_")
    t0 = time.perf_counter()
    wd, info = make_workload(args.workload, rank, base)
    t_gen = time.perf_counter() - t0
    inp = engine.Inputs(wd)
    mt = inp.dims.metat
    W = 1 if inp.dims.norb <= 64 else 2
    ctx = engine.Context(inp.dims, device=local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(inp)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    gmask = None
    if args.gen_every > 1:
        gmask = np.zeros(inp.dims.ncf, dtype=np.uint8)
        gmask[args.gen_offset::args.gen_every] = 1
    chunk = args.chunk_records
    for _ in range(args.warmup):
        res = ctx.run_stream(inp.opts, chunk_records=chunk, gen_mask=gmask)
    contrib_per_step = res["n_processed"] * mt
    clocks = Clocks(local_rank)
    clocks.start()
    # ---- device-resident timing: the streamed run, records kept on the device
    barrier()
    torch.cuda.synchronize()
    step_ms, pt2_ms = [], []
    launches = 0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = ctx.run_stream(inp.opts, chunk_records=chunk, gen_mask=gmask)
        e1.record(stream)
        stream.synchronize()
        assert r["n_processed"] * mt == contrib_per_step and r["n_selected"] == res["n_selected"]
        step_ms.append(e0.elapsed_time(e1))
        pt2_ms.append(r["pt2_ms"])
        launches += r["launches"]
    torch.cuda.synchronize()
    barrier()
    # ---- end to end through the C ABI: upload from host buffers, stream,
    # every record delivered to host memory and folded into a digest
    e2e_ms = []
    upload_ms = []
    digests = []
    n_e2e = max(1, min(args.steps, args.e2e_steps))
    for _ in range(n_e2e):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.upload(inp)
        upload_ms.append(1e3 * (time.perf_counter() - t0))
        d = engine.Digest()
        d.threads = max(1, (os.cpu_count() or 2) - 1)
        r2 = ctx.run_stream(inp.opts, chunk_records=chunk, consumer=d, gen_mask=gmask)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        assert d.records == r2["n_selected"] == res["n_selected"]
        digests.append(d.value())
    assert all(x == digests[0] for x in digests), "streamed records differ between runs"
    clk = clocks.stop()
    tot_ms = sum(step_ms)
    tot_e2e = sum(e2e_ms)
    if world > 1:
        t = torch.tensor([tot_ms, tot_e2e / n_e2e * args.steps, float(contrib_per_step)], dtype=torch.float64,
                         device="cuda")
        mx = t.clone()
        torch.distributed.all_reduce(mx[:2], op=torch.distributed.ReduceOp.MAX)
        sm = t.clone()
        torch.distributed.all_reduce(sm[2:], op=torch.distributed.ReduceOp.SUM)
        tot_ms, tot_e2e_k, all_contrib = float(mx[0]), float(mx[1]), float(sm[2])
    else:
        tot_e2e_k = tot_e2e / n_e2e * args.steps
        all_contrib = float(contrib_per_step)
    value = all_contrib * args.steps / (tot_ms / 1e3)
    e2e_value = all_contrib * args.steps / (tot_e2e_k / 1e3)
    # bytes copied per e2e step: the inputs up, the results and records down
    synth = _synth()
    import struct
    recs = synth.read_records(os.path.join(wd, "ijkl"))
    ninte = struct.unpack_from("<i", recs[7], 0)[0]
    n, ncf = inp.dims.norb, inp.dims.ncf
    nter = n * (n + 1) // 2
    h2d = (ninte * 4 + 3 * nter * 8 + n * n * 4 + inp.dims.nsym * 4 + n + ncf * 2 * W * 8
           + ncf * (1 + 1 + 4) + ncf * mt * 8 + 2 * n * 8)
    nsel = res["n_selected"]
    rec_bytes = 2 * W * 8 + 4 + 8 + mt * 8
    d2h = 5 * mt * 8 + 8 * (10 + 1 + 10 + 10 * 8) + 2 * 10 * 8 * 8 + nsel * rec_bytes
    peak, peak_kind = measured_peaks()
    kms = statistics.mean(pt2_ms)
    nl = max(1, (r["launches"] - 1) // 3)  # k_pt2 launches per step (one per chunk)
    achieved = r["alg_bytes"] / (kms / 1e3) / 1e9
    prof = kernel_profile(args.workload) if args.gen_every == 1 else None
    traffic = prof.get("dram_bytes_per_launch") if prof else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded integrals and reference space)",
            "config": dict(workload_desc(args.workload),
                           **({"generator_sample": f"1/{args.gen_every} (profiling run)"}
                              if args.gen_every > 1 else {})),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": tot_e2e / n_e2e, "steps": n_e2e,
                    "upload_ms_per_step": statistics.mean(upload_ms),
                    "records_delivered_per_step": int(nsel), "record_bytes": rec_bytes,
                    "digest": [format(x, "016x") for x in digests[0]]},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_pt2", "peak_source": peak_kind, "launches_per_step": nl,
                         "algorithmic_bytes_per_launch": r["alg_bytes"] / nl,
                         "kernel_ms_per_launch": kms / nl,
                         "note": "achieved = algorithmic bytes of the E2 loop (integral, coefficient and "
                                 "diagonal-term reads) / k_pt2 time (CUDA events around each chunk's launch on "
                                 "its stream), against the measured HBM copy bandwidth; traffic: DRAM bytes per "
                                 "k_pt2 launch, the mean over every launch of one step of this workload in a "
                                 "single-pass ncu capture of this kernel build (null when the kernel changed "
                                 "since); the kernel is bound by integer issue and latency, not HBM"},
            "clocks": clk,
            "work": {"perturbers": r["n_processed"], "candidates": r["n_candidates"],
                     "compares": r["n_compares"], "pairs_1": r["n_pairs_1"], "pairs_2": r["n_pairs_2"],
                     "selected": r["n_selected"], "ietat": r["ietat"], "e2vp": r["e2vp"], "e2mp": r["e2mp"],
                     "device_ms_per_step_incl_records": tot_ms / args.steps,
                     "k_pt2_ms_per_step": kms, "generation_s": t_gen}}
    if prof:
        line["roofline"]["issue_slots"] = {"frac": prof.get("issue_active_frac"),
                                           "fp64_pipe_frac": prof.get("fp64_pipe_frac"),
                                           "source": prof.get("command")}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import build as ob
        ob.build()
        sample = CPU_SAMPLE[args.workload]
        plan = sample_plan(inp.dims.ncf, inp.array("ysaut"), 1, 1, sample, seed=11)[0]
        res_c, metat = oracle_plan(wd, plan, sample, base)
        nproc, secs = res_c[0]
        line["cpu_baseline"] = {"value": nproc * metat / secs, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"generator {plan[0][1]} of S, 1 candidate in {sample} (systematic "
                                          f"sample), {secs:.1f} s loop time on one core, inputs read once; "
                                          "extrapolated linearly in contributions"}
    ctx.close()
    shutil.rmtree(base, ignore_errors=True)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description="CIPSI E2/selection benchmark")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", choices=["plain", "batched", "adjoint", "moy", "bd"], default="plain",
                    help="batched: the potential-curve batch (geometries/s, batched vs plain); "
                         "adjoint: dE2/d integrals on the medium system with checks; "
                         "moy: the Hamiltonian over a determinant list (the moy drop-in)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="large")
    ap.add_argument("--chunk-records", type=int, default=0,
                    help="records per streamed chunk (0 = sized from free device memory)")
    ap.add_argument("--e2e-steps", type=int, default=3, help="end-to-end steps (at most --steps)")
    ap.add_argument("--fd-elements", type=int, default=200)
    ap.add_argument("--geometries", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--batch-warmup", type=int, default=1)
    ap.add_argument("--moy-dets", type=int, default=100000, help="moy form: determinants in the list")
    ap.add_argument("--moy-cpu-dets", type=int, default=20000, help="moy form: list size of the CPU sample")
    ap.add_argument("--gen-every", type=int, default=1,
                    help="profiling aid: run only every n-th determinant of S as a generator")
    ap.add_argument("--gen-offset", type=int, default=0, help="profiling aid: first generator of --gen-every")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.form == "batched":
        run_batched(args, rank, world, local_rank)
        return
    if args.form == "adjoint":
        run_adjoint_form(args, rank, world, local_rank)
        return
    if args.form == "moy":
        run_moy_form(args, rank, world, local_rank)
        return
    if args.form == "bd":
        run_bd_form(args, rank, world, local_rank)
        return
    run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
