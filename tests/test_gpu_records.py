"""Unit-60 records: fixed order and the streamed run (cipsi_run_pt2_stream).

The records of a run come out in one order whatever the GPU's scheduling:
generators in the run's order, then blocks of removed electrons, then added
orbitals.  So two runs with different launch shapes (work-unit size, CTAs
per SM) give identical record arrays, and a streamed run cut into many
chunks hands its consumer exactly cipsi_run_pt2's arrays, in order, with
the same sums.  The drop-in executable writes byte-identical unit-60 files
on two runs."""
import os
import shutil
import struct

import numpy as np
import pytest

import cipsi_gb300 as cg
from cipsi_gb300 import engine, synth

pytestmark = pytest.mark.gpu

CASES = [
    ("small", synth.CONFIGS["small"]),
    ("mix_sym2", synth.SynthConfig("mix_sym2", norb=12, nocc=4, ncholesky=20, ncf=60, metat=2, tau=0.02,
                                   ranks=(1, 2, 3), coef_mode="decay09", seed=4, nsym=2)),
    ("two_word", synth.SynthConfig("two_word", norb=70, nocc=6, ncholesky=16, ncf=100, metat=2, tau=0.02,
                                   ranks=(1, 2, 3), coef_mode="decay09", seed=11)),
]
SUMS = ("e2mp", "e2vp", "e2b", "psimp", "psivp")
COUNTS = ("ietat", "n_processed", "n_selected", "n_candidates", "nom", "nam")


def _load(tmp_path, cfg):
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    return engine.Inputs(wd)


def _arrays(ctx, n):
    return ctx.selection_raw(n)


def _equal(a, b):
    for k in ("bits", "owner", "xam", "evp"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name,cfg", CASES, ids=[c[0] for c in CASES])
def test_record_order_does_not_depend_on_the_launch_shape(tmp_path, engine_lib, name, cfg):
    inp = _load(tmp_path, cfg)
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts)
        a = _arrays(ctx, ref["n_selected"])
        for r_chunk, ctas in ((1, 1), (12, 2), (3, 0)):
            ctx.set_tuning(r_chunk, ctas)
            got = ctx.run(inp.opts)
            for k in COUNTS:
                assert got[k] == ref[k], (k, r_chunk, ctas)
            _equal(_arrays(ctx, got["n_selected"]), a)
    assert ref["n_selected"] > 0
    # generators appear in the run's order: pertu's candidates (owner 0)
    # first, then owners grouped, never interleaved
    own = a["owner"]
    seen, prev = set(), None
    for o in own.tolist():
        if o != prev:
            assert o not in seen, "owner segments interleaved"
            seen.add(o)
            prev = o


@pytest.mark.parametrize("chunk", [1024, 50000])
@pytest.mark.parametrize("name,cfg", CASES, ids=[c[0] for c in CASES])
def test_stream_delivers_the_records_of_run_pt2(tmp_path, engine_lib, name, cfg, chunk):
    inp = _load(tmp_path, cfg)
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts)
        n = ref["n_selected"]
        a = _arrays(ctx, n)
        pieces = []

        def take(first, bits, owner, xam, evp):
            assert first == sum(len(p[1]) for p in pieces)
            pieces.append((bits, owner, xam, evp))

        got = ctx.run_stream(inp.opts, chunk_records=chunk, consumer=take)
        for k in COUNTS:
            assert got[k] == ref[k], k
        for k in SUMS + ("tabmp", "tabvp"):
            np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=1e-13, err_msg=k)
        # the per-unit partial sums are reduced in one fixed order in both
        for k in SUMS:
            assert got[k] == ref[k], k
        cat = {"bits": np.concatenate([p[0] for p in pieces]) if pieces else np.zeros((0, a["bits"].shape[1]), np.uint64),
               "owner": np.concatenate([p[1] for p in pieces]) if pieces else np.zeros(0, np.int32),
               "xam": np.concatenate([p[2] for p in pieces]) if pieces else np.zeros(0),
               "evp": np.concatenate([p[3] for p in pieces]) if pieces else np.zeros((0, inp.dims.metat))}
        _equal(cat, a)
        # the native digest consumer over the same stream
        d = engine.Digest()
        d.threads = 4
        ctx.run_stream(inp.opts, chunk_records=chunk, consumer=d)
        assert d.records == n
        assert d.value() == engine.digest_arrays(a["bits"], a["owner"], a["xam"], a["evp"])
        # no consumer: the same results, records left on the device
        dev = ctx.run_stream(inp.opts, chunk_records=chunk)
        for k in COUNTS:
            assert dev[k] == ref[k], k


def test_stream_on_the_medium_workload_sample(tmp_path, engine_lib):
    """60 orbitals, S = 2000, 3 roots, every 23rd generator: many chunks of a
    few hundred thousand records, against one cipsi_run_pt2 call."""
    inp = _load(tmp_path, synth.CONFIGS["medium"])
    mask = np.zeros(inp.dims.ncf, np.uint8)
    mask[::23] = 1
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts, gen_mask=mask)
        a = _arrays(ctx, ref["n_selected"])
        d = engine.Digest()
        d.threads = 8
        got = ctx.run_stream(inp.opts, chunk_records=1 << 19, consumer=d, gen_mask=mask)
    assert ref["n_selected"] > 1 << 20
    for k in COUNTS:
        assert got[k] == ref[k], k
    for k in SUMS:
        assert got[k] == ref[k], k
    assert d.value() == engine.digest_arrays(a["bits"], a["owner"], a["xam"], a["evp"])


def test_drop_in_writes_the_same_unit60_twice(tmp_path, engine_lib):
    """Two runs of the cipsym drop-in on copies of one calculation directory
    write byte-identical unit 60, and its records are the engine's, in the
    engine's order, after S."""
    cfg = CASES[2][1]
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    outs = []
    for i in range(2):
        d = str(tmp_path / f"run{i}")
        shutil.copytree(wd, d)
        j = cg.run_cip(d, variant="cipsym")
        with open(os.path.join(d, "det"), "rb") as fh:
            outs.append(fh.read())
    assert len(outs[0]) > 1000
    assert outs[0] == outs[1]
    inp = engine.Inputs(wd)
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts)
        sel = ctx.selection(ref["n_selected"])
    assert j["ntot60"] == inp.dims.ncf + ref["n_selected"]
    recs = []
    for r in synth.read_records(os.path.join(str(tmp_path / "run0"), "det")):
        m, n = struct.unpack_from("<ii", r, 0)
        idet = struct.unpack_from(f"<{m}i", r, 8)
        nex = struct.unpack_from(f"<{n}i", r, 8 + 4 * m)
        v = struct.unpack_from(f"<{n}d", r, 8 + 4 * m + 4 * n)
        pos = 0
        for q, ne in enumerate(nex):
            recs.append((tuple(idet[pos:pos + 2 * ne:2]), tuple(idet[pos + 1:pos + 2 * ne:2]), v[q]))
            pos += 2 * ne
    pert = recs[inp.dims.ncf:]
    assert len(pert) == ref["n_selected"]
    for i, (h, p, v) in enumerate(pert):
        ne = sel["nec"][i]
        assert h == tuple(sel["holes"][i][:ne]) and p == tuple(sel["parts"][i][:ne]) and v == sel["xam"][i], i
