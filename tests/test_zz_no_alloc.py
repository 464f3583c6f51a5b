"""cipsi_run_pt2_static (the entry point that allocates no device memory)
against cipsi_run_pt2 on the same context, through the C ABI.

Two static calls in a row must both give cipsi_run_pt2's energies (within
1e-10 relative, plus 1e-12 absolute), and identical counters, histogram
counts and selection count, and must leave the device's free memory as it
was.  This file is collected last so that it also runs
after every other GPU test in the same process."""
import ctypes
import dataclasses

import numpy as np
import pytest

from cipsi_gb300 import engine, synth

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL = 1e-12


def _static_fn():
    lib = engine._lib()
    f = lib.cipsi_run_pt2_static
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(engine.Opts), ctypes.POINTER(engine.Result)]
    f.restype = ctypes.c_int
    return lib, f


def _run_static(ctx, opts):
    lib, f = _static_fn()
    r = engine.Result()
    rc = f(ctx._c, ctypes.byref(opts), ctypes.byref(r))
    assert rc == 0, lib.cipsi_last_error(ctx._c).decode()
    return engine.result_dict(r, ctx.dims.metat, opts.nclass)


def _free_bytes():
    """Free device memory (cudaMemGetInfo through torch's runtime)."""
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def _compare(ref, got):
    for k in ("ietat", "n_processed", "n_selected", "n_candidates", "n_pairs_1", "n_pairs_2", "nom", "nam"):
        assert got[k] == ref[k], k
    for k in ("e2mp", "e2vp", "e2b", "psimp", "psivp", "tabmp", "tabvp"):
        np.testing.assert_allclose(got[k], ref[k], rtol=RTOL, atol=ATOL, err_msg=k)
    np.testing.assert_allclose(got["dpivot"], ref["dpivot"], rtol=RTOL, atol=ATOL)


CASES = [
    ("small", synth.CONFIGS["small"]),
    ("mix_sym2", synth.SynthConfig("mix_sym2", norb=12, nocc=4, ncholesky=20, ncf=60, metat=2, tau=0.02,
                                   ranks=(1, 2, 3), coef_mode="decay09", seed=4, nsym=2)),
    ("two_word", synth.SynthConfig("two_word", norb=70, nocc=6, ncholesky=16, ncf=100, metat=2, tau=0.02,
                                   ranks=(1, 2, 3), coef_mode="decay09", seed=11)),
    ("medium", synth.CONFIGS["medium"]),
]


@pytest.mark.parametrize("name,cfg", CASES, ids=[c[0] for c in CASES])
def test_static_matches_run_pt2(tmp_path, engine_lib, name, cfg):
    wd = str(tmp_path / "in")
    synth.generate(cfg, wd)
    inp = engine.Inputs(wd)
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts)
        # the context and the library's device code are set up by now, so
        # the two static calls must leave the device's free memory unchanged
        free0 = _free_bytes()
        first = _run_static(ctx, inp.opts)
        second = _run_static(ctx, inp.opts)
        assert _free_bytes() == free0, "a static call allocated device memory"
        # the records of the cipsi_run_pt2 run stay readable
        sel = ctx.selection_raw(min(ref["n_selected"], 16))
    assert ref["n_processed"] > 0
    _compare(ref, first)
    _compare(ref, second)
    assert len(sel["owner"]) == min(ref["n_selected"], 16)


def test_static_with_generator_mask(tmp_path, engine_lib):
    """A generator subset and no pertu block, as one shard of a multi-GPU run."""
    from cipsi_gb300 import shard
    wd = str(tmp_path / "in")
    synth.generate(dataclasses.replace(synth.CONFIGS["small"], seed=5), wd)
    inp = engine.Inputs(wd)
    mask = np.ascontiguousarray(shard.generator_mask(inp.dims.ncf, 1, 2), dtype=np.uint8)
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ref = ctx.run(inp.opts, gen_mask=mask, run_pertu=False)
        o = ctx._opts(inp.opts, mask, False)
        for _ in range(2):
            _compare(ref, _run_static(ctx, o))


def test_static_refuses_while_async_pending(tmp_path, engine_lib):
    wd = str(tmp_path / "in")
    synth.generate(synth.CONFIGS["small"], wd)
    inp = engine.Inputs(wd)
    lib, f = _static_fn()
    with engine.Context(inp.dims) as ctx:
        ctx.upload(inp)
        ctx.run_async(inp.opts)
        r = engine.Result()
        assert f(ctx._c, ctypes.byref(inp.opts), ctypes.byref(r)) == -3  # CIPSI_ERR_STATE
        assert b"pending" in lib.cipsi_last_error(ctx._c)
        ref = ctx.fetch()
        _compare(ref, _run_static(ctx, inp.opts))
