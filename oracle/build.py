"""Build recipe for the CPU oracle (test infrastructure; never linked into
the product).  Compiles oracle/cipsi_ref.c with gcc into oracle/_build/."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
EXE = os.path.join(OUT, "cipsi_ref")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "cipsi_ref.c")
    # -O3 without fused multiply-add contraction and without -march=native:
    # the same results on the x86 and Arm hosts the tests and the timed CPU
    # baseline run on (IEEE semantics kept: no fast-math)
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-std=c11", "-Wall", "-o", EXE, src, "-lm"]
    stamp = os.path.join(OUT, ".stamp")
    key = " ".join(cmd)
    if (not force and os.path.exists(EXE) and os.path.getmtime(EXE) >= os.path.getmtime(src)
            and os.path.exists(stamp) and open(stamp).read() == key):
        return EXE
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    with open(stamp, "w") as fh:
        fh.write(key)
    return EXE


def run(workdir: str, variant: str = "cipsym", json_name: str = "cipsi_ref.json",
        candlog: str | None = None, genmask: str | None = None, no_pertu_ref: bool = False,
        timeout: float | None = None, sample: int = 0, plan: str | None = None) -> str:
    """Run the oracle in `workdir` (it rewrites unit 60 and appends to unit 33,
    as cip does).  Returns the JSON path."""
    exe = build()
    args = [exe]
    if variant == "cipsym":
        args.append("--sym")
    args += ["--json", json_name]
    if candlog:
        args += ["--candlog", candlog]
    if genmask:
        args += ["--genmask", genmask]
    if no_pertu_ref:
        args.append("--no-pertu-ref")
    if plan:
        args += ["--sample", str(sample), "--plan", plan]
    with open(os.path.join(workdir, "cip.in")) as fin:
        r = subprocess.run(args, cwd=workdir, stdin=fin, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                           text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("oracle failed: " + r.stderr)
    return os.path.join(workdir, json_name)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
