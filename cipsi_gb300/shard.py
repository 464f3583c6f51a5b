"""Generator sharding for several GPUs (one process per GPU).

Each perturber is processed by exactly one generator of S (its owner, the
lowest-index generator that interacts with it: cip/pert1.f:104-118), so a
partition of the generators partitions the perturbers: every rank runs the
same inputs with its own generator mask, and the only exchange is the final
reduction of a few numbers per root plus the concatenation of the selected
determinants.  The reference-only / reference-single candidates of pertu
(no owner) run on rank 0 only.
"""
from __future__ import annotations

from typing import Dict, List

import numpy as np

SUM_KEYS = ("e2mp", "e2vp", "e2b", "psimp", "psivp")
COUNT_KEYS = ("ietat", "n_processed", "n_selected", "n_candidates", "n_compares", "n_pairs_1",
              "n_pairs_2", "alg_bytes")


def generator_mask(ncf: int, rank: int, world: int) -> np.ndarray:
    """Round-robin ownership of S determinants (as generators) for `rank`."""
    if not 0 <= rank < world:
        raise ValueError("rank outside [0, world)")
    m = np.zeros(ncf, dtype=np.uint8)
    m[rank::world] = 1
    return m


def combine(parts: List[Dict]) -> Dict:
    """Reduce per-rank result dicts (engine or oracle JSON layout)."""
    out: Dict = {}
    metat = len(parts[0]["e2mp"])
    for k in SUM_KEYS:
        if k in parts[0]:
            out[k] = [float(sum(p[k][m] for p in parts)) for m in range(metat)]
    for k in COUNT_KEYS:
        if k in parts[0]:
            out[k] = int(sum(p[k] for p in parts))
    out["dpivot"] = max(p["dpivot"] for p in parts)
    for k in ("nom",):
        if k in parts[0]:
            out[k] = [int(sum(p[k][i] for p in parts)) for i in range(len(parts[0][k]))]
    for k in ("nam",):
        if k in parts[0]:
            out[k] = [[int(sum(p[k][m][i] for p in parts)) for i in range(len(parts[0][k][m]))]
                      for m in range(metat)]
    for k in ("tabmp", "tabvp"):
        if k in parts[0]:
            out[k] = [[float(sum(p[k][m][i] for p in parts)) for i in range(len(parts[0][k][m]))]
                      for m in range(metat)]
    return out


def flatten(res: Dict) -> np.ndarray:
    """Vector view of a result dict for an all-reduce (sums) of one rank."""
    vals: List[float] = []
    for k in SUM_KEYS:
        vals += list(res[k])
    vals += [float(res[k]) for k in ("ietat", "n_processed")]
    vals += [float(x) for x in res["nom"]]
    for row in res["nam"]:
        vals += [float(x) for x in row]
    return np.array(vals, dtype=np.float64)
