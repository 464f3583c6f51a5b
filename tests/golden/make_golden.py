"""Regenerate the committed known-answer fixtures (run from the repo root):

    python tests/golden/make_golden.py

Writes tests/golden/small/ (the seeded 20-orbital configuration in the
reference's file formats: ijkl, ener, det, bdvec, f04, cip.in) and
tests/golden/small_expected.json: the CPU oracle's E2 totals, counters,
histogram and a digest of the unit-60 selection for those exact files.
"""
import hashlib
import json
import os
import shutil
import struct
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cipsi_gb300 import synth  # noqa: E402
from oracle import build as ob  # noqa: E402


def selection_digest(det_path, metat, sym):
    """Order-independent digest of the unit-60 records after S: sorted
    (holes, particles, round(v, 12)) tuples."""
    items = []
    for r in synth.read_records(det_path):
        m, n = struct.unpack_from("<ii", r, 0)
        idet = struct.unpack_from(f"<{m}i", r, 8)
        nex = struct.unpack_from(f"<{n}i", r, 8 + 4 * m)
        v = struct.unpack_from(f"<{n}d", r, 8 + 4 * m + 4 * n)
        pos = 0
        for i, nec in enumerate(nex):
            h = sorted(idet[pos + 2 * q] for q in range(nec))
            p = sorted(idet[pos + 2 * q + 1] for q in range(nec))
            pos += 2 * nec
            items.append((tuple(h), tuple(p), round(v[i], 12)))
    items.sort()
    return len(items), hashlib.sha256(repr([(h, p) for h, p, _ in items]).encode()).hexdigest()


def main():
    out = os.path.join(HERE, "small")
    shutil.rmtree(out, ignore_errors=True)
    synth.generate(synth.CONFIGS["small"], out)
    with tempfile.TemporaryDirectory() as td:
        run = os.path.join(td, "run")
        shutil.copytree(out, run)
        j = json.load(open(ob.run(run, variant="cipsym")))
        nrec, dig = selection_digest(os.path.join(run, "det"), j["metat"], True)
    j.pop("t_pertu_s", None)
    j.pop("t_diexcit_s", None)
    j["unit60_records"] = nrec
    j["unit60_sets_sha256"] = dig
    with open(os.path.join(HERE, "small_expected.json"), "w") as fh:
        json.dump(j, fh, indent=1, sort_keys=True)
    print(json.dumps({k: j[k] for k in ("ncf", "ietat", "n_processed", "e2mp", "e2vp")}))


if __name__ == "__main__":
    main()
