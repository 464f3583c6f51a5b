"""Unit-60 records written into caller-provided pinned host arrays
(cipsi_set_selection_sink) against the device-buffer records: the same
records in the same order."""
import ctypes

import numpy as np
import pytest
import torch

from cipsi_gb300 import engine, synth

pytestmark = pytest.mark.gpu


def pinned(cap, W, mt):
    return {"bits": torch.zeros((cap, 2 * W), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64),
            "owner": torch.zeros(cap, dtype=torch.int32, pin_memory=True).numpy(),
            "xam": torch.zeros(cap, dtype=torch.float64, pin_memory=True).numpy(),
            "evp": torch.zeros((cap, mt), dtype=torch.float64, pin_memory=True).numpy()}


def rows(sel, n):
    # in order: the records' order is fixed (work units, then candidates)
    return list(zip(map(tuple, sel["bits"][:n].tolist()), sel["owner"][:n].tolist(), sel["xam"][:n].tolist(),
                    map(tuple, sel["evp"][:n].tolist())))


@pytest.mark.parametrize("cfg", [synth.CONFIGS["small"],
                                 synth.SynthConfig("w2", norb=70, nocc=6, ncholesky=16, ncf=100, metat=2,
                                                   tau=0.02, ranks=(1, 2, 3), coef_mode="decay09", seed=11)],
                         ids=["small", "two_word"])
def test_sink_records_match_device_records(tmp_path, engine_lib, cfg):
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    inp = engine.Inputs(wd)
    W = 1 if inp.dims.norb <= 64 else 2
    mt = inp.dims.metat
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts)
        n = ref["n_selected"]
        assert n > 10
        dev = ctx.selection_raw(n)
        # a sink large enough: same results, same records in the same order,
        # nothing to copy back
        sink = pinned(n + 5, W, mt)
        ctx.set_selection_sink(sink)
        got = ctx.run(inp.opts)
        for k in ("n_selected", "n_processed", "ietat", "nom", "nam"):
            assert got[k] == ref[k], k
        assert rows(sink, n) == rows(dev, n)
        assert rows(ctx.selection_raw(n), n) == rows(dev, n)
        # a sink too small: counts are complete, the first records are kept
        small = pinned(n // 2, W, mt)
        ctx.set_selection_sink(small)
        ctx.run_async(inp.opts)
        r = engine.Result()
        assert ctx.lib.cipsi_fetch_result(ctx._c, ctypes.byref(r)) == -4  # CIPSI_ERR_OVERFLOW
        assert r.n_selected == n
        assert rows(small, n // 2) == rows(dev, n // 2)
        # back to device buffers
        ctx.set_selection_sink(None)
        again = ctx.run(inp.opts)
        assert again["n_selected"] == n
        assert rows(ctx.selection_raw(n), n) == rows(dev, n)
