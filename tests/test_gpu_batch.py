"""Batched form (cipsi_batch_*): many geometries in one persistent launch per
class, replayed from a CUDA graph, against the plain run of each context.

Counts (processed perturbers, ietat, histogram counts, selection count) must
be identical; energies within 1e-10 relative (+1e-12 absolute): the per-unit
partial sums and their fixed-order reduction are the same as in the plain
run, only the histogram's class sums are added atomically."""
import dataclasses

import numpy as np
import pytest

from cipsi_gb300 import CipsiError, batch, engine, synth

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-10, 1e-12


def geometry_configs():
    out = []
    specs = [  # norb, nocc, ncf, metat, R, seed
        (14, 4, 80, 1, 2.5, 21), (16, 4, 120, 2, 4.0, 22), (70, 6, 100, 2, 7.5, 23),
        (12, 3, 60, 1, 11.0, 24), (66, 5, 90, 1, 3.3, 25), (18, 5, 150, 3, 9.1, 26),
    ]
    for i, (norb, nocc, ncf, mt, R, seed) in enumerate(specs):
        out.append(synth.SynthConfig(f"g{i}", norb=norb, nocc=nocc, ncholesky=2 * norb, ncf=ncf, metat=mt,
                                     tau=0.02, ranks=(1, 2, 3), coef_mode="decay09", seed=seed,
                                     curve_R=R, energy="diagonal"))
    return out


@pytest.fixture(scope="module")
def loaded(engine_lib):
    opts, ctxs = batch.load_geometries(geometry_configs(), workers=3)
    yield opts, ctxs
    for c in ctxs:
        c.close()


def compare(ref, got):
    for k in ("ietat", "n_processed", "n_selected", "n_candidates", "n_pairs_1", "n_pairs_2", "nom", "nam"):
        assert got[k] == ref[k], k
    for k in ("e2mp", "e2vp", "e2b", "psimp", "psivp", "tabmp", "tabvp"):
        np.testing.assert_allclose(got[k], ref[k], rtol=RTOL, atol=ATOL, err_msg=k)
    np.testing.assert_allclose(got["dpivot"], ref["dpivot"], rtol=RTOL, atol=ATOL)


def test_batch_matches_plain_runs(loaded):
    opts, ctxs = loaded
    plain = [c.run(o) for c, o in zip(ctxs, opts)]
    assert all(r["n_processed"] > 0 for r in plain)
    with engine.Batch(ctxs, opts) as b:
        for _ in range(2):  # two replays of the graph
            b.run()
            ms = b.wait()
            assert ms > 0
            got = b.fetch_all(allow_overflow=False)
            for ref, g in zip(plain, got):
                compare(ref, g)
                assert g["kernel_ms"] == -1.0
        # the records of the last replay are the plain run's, in the same
        # order (generators in plan order, then removed-electron blocks, then
        # added orbitals: independent of the work-unit size and of scheduling)
        for c, ref in zip(ctxs, plain):
            n = ref["n_selected"]
            s_b = c.selection(n)
            rows_b = list(zip(s_b["owner"].tolist(), map(tuple, s_b["holes"].tolist()),
                              map(tuple, s_b["parts"].tolist()), s_b["xam"].tolist()))
            c.run(opts[ctxs.index(c)])
            s_p = c.selection(n)
            rows_p = list(zip(s_p["owner"].tolist(), map(tuple, s_p["holes"].tolist()),
                              map(tuple, s_p["parts"].tolist()), s_p["xam"].tolist()))
            assert rows_b == rows_p


def test_batch_generator_masks_and_tuning(loaded):
    opts, ctxs = loaded
    masks = [(np.arange(c.dims.ncf) % 2 == 1).astype(np.uint8) for c in ctxs]
    ref = [c.run(o, gen_mask=m, run_pertu=False) for c, o, m in zip(ctxs, opts, masks)]
    opts_np = []
    for o in opts:
        o2 = engine.Opts.from_buffer_copy(o)
        o2.run_pertu = 0
        opts_np.append(o2)
    for r_chunk, ctas in ((1, 0), (12, 1)):
        with engine.Batch(ctxs, opts_np, r_chunk=r_chunk, ctas_per_sm=ctas, gen_masks=masks) as b:
            b.run()
            b.wait()
            for r, g in zip(ref, b.fetch_all(allow_overflow=False)):
                compare(r, g)


def test_batch_refuses_after_reallocation(loaded):
    opts, ctxs = loaded
    with engine.Batch(ctxs, opts, r_chunk=12) as b:
        b.run()
        b.wait()
        b.fetch_all()
        # a plain run with finer work units grows the unit buffer of ctxs[0]
        ctxs[0].set_tuning(1, 0)
        ctxs[0].run(opts[0])
        ctxs[0].set_tuning(6, 0)
        with pytest.raises(CipsiError, match="rebuild the batch"):
            b.run()


def test_autotune_picks_a_candidate(loaded):
    opts, ctxs = loaded
    best, times = batch.autotune(ctxs, opts, sample=4)
    assert best in batch.CANDIDATES
    assert set(times) == set(batch.CANDIDATES)
    assert all(t > 0 for t in times.values())
