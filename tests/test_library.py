"""The C-ABI library: it builds, loads and exports every function that
include/cipsi_gb300.h declares; without a GPU every compute entry point fails
loudly (no CPU fallback); malformed inputs are rejected before any device
work."""
import ctypes
import os
import re
import shutil

import pytest

import cipsi_gb300 as cg
from conftest import ROOT


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "cipsi_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cipsi_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(engine_lib):
    lib = ctypes.CDLL(engine_lib)
    names = declared_functions()
    assert len(names) >= 13
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(cg.EXPORTED) == names


def test_ctx_create_validates_dims(engine_lib):
    lib = ctypes.CDLL(engine_lib)

    class Dims(ctypes.Structure):
        _fields_ = [(f, ctypes.c_int32) for f in ("norb", "noca", "nsym", "isym", "isz", "metat", "ncf")]

    lib.cipsi_ctx_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Dims), ctypes.c_int32]
    lib.cipsi_last_error.restype = ctypes.c_char_p
    lib.cipsi_last_error.argtypes = [ctypes.c_void_p]
    lib.cipsi_ctx_destroy.argtypes = [ctypes.c_void_p]
    for bad, msg in [(Dims(200, 5, 1, 1, 0, 1, 10), b"norb"), (Dims(20, 5, 1, 1, 2, 1, 10), b"isz"),
                     (Dims(20, 5, 1, 1, 0, 9, 10), b"metat"), (Dims(20, 5, 1, 2, 0, 1, 10), b"isym")]:
        ctx = ctypes.c_void_p()
        rc = lib.cipsi_ctx_create(ctypes.byref(ctx), ctypes.byref(bad), 0)
        assert rc == -1
        assert msg in lib.cipsi_last_error(ctx)
        lib.cipsi_ctx_destroy(ctx)


def _golden(tmp_path):
    src = os.path.join(ROOT, "tests", "golden", "small")
    dst = str(tmp_path / "run")
    shutil.copytree(src, dst)
    return dst


def test_unsupported_inputs_are_rejected(tmp_path, engine_lib):
    wd = _golden(tmp_path)
    txt = open(os.path.join(wd, "cip.in")).read()
    for extra, word in [("isz=2", "isz"), ("ninact=1, nonact=3", "ninact"), ("ybrd=t, metat=2", None)]:
        with open(os.path.join(wd, "cip_bad.in"), "w") as fh:
            fh.write(txt.replace("ymoyen=t", "ymoyen=t, " + extra))
        if word is None:
            continue
        with pytest.raises(cg.CipsiError, match=word):
            cg.run_cip(wd, stdin_path=os.path.join(wd, "cip_bad.in"))


def test_s_diagonalisation_needs_the_drop_in(tmp_path, engine_lib):
    """A perturbation run with lecdet != 5 diagonalises S (ic001.f:81-131)
    on the GPU inside cipsi_cip_main; the host-only input reader refuses it
    with that reason instead of running without vectors."""
    from cipsi_gb300 import engine
    wd = _golden(tmp_path)
    txt = open(os.path.join(wd, "cip.in")).read()
    with open(os.path.join(wd, "cip.in"), "w") as fh:
        fh.write(txt.replace("lecdet=5", "lecdet=2"))
    with pytest.raises(cg.CipsiError, match="lecdet != 5"):
        engine.Inputs(wd)


def test_missing_and_corrupt_files_fail_cleanly(tmp_path, engine_lib):
    wd = _golden(tmp_path)
    os.remove(os.path.join(wd, "bdvec"))
    with pytest.raises(cg.CipsiError, match="bdvec"):
        cg.run_cip(wd)
    wd2 = str(tmp_path / "run2")
    shutil.copytree(os.path.join(ROOT, "tests", "golden", "small"), wd2)
    with open(os.path.join(wd2, "ijkl"), "r+b") as fh:
        fh.truncate(1000)
    with pytest.raises(cg.CipsiError, match="unit 40|record"):
        cg.run_cip(wd2)


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="checks the no-GPU failure path")
def test_no_gpu_means_error_not_fallback(tmp_path, engine_lib):
    wd = _golden(tmp_path)
    with pytest.raises(cg.CipsiError, match="cuda|CUDA"):
        cg.run_cip(wd)


def test_record_digest_consumer_matches_its_restatement(engine_lib):
    """cipsi_record_digest (host code, the streamed run's native consumer)
    over pieces of records, with several host threads, against the numpy
    restatement; a piece out of order is refused."""
    import numpy as np
    from cipsi_gb300 import engine
    lib = engine._lib()
    f = lib.cipsi_record_digest
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(3)
    n, words, mt = 300_000, 4, 3
    bits = rng.integers(0, 2**63, size=(n, words), dtype=np.uint64)
    owner = rng.integers(-5, 20000, size=n).astype(np.int32)
    xam = rng.random(n)
    evp = rng.normal(size=(n, mt))
    d = engine.Digest()
    d.threads = 6
    for a, b in ((0, 70_001), (70_001, 70_001), (70_001, 250_000), (250_000, n)):
        rc = f(ctypes.addressof(d), a, b - a, words, mt, bits[a:].ctypes.data, owner[a:].ctypes.data,
               xam[a:].ctypes.data, evp[a:].ctypes.data)
        assert rc == 0
    assert d.records == n
    assert d.value() == engine.digest_arrays(bits, owner, xam, evp)
    # the digest depends on the order of the records
    sw = [x.copy() for x in (bits, owner, xam, evp)]
    for x in sw:
        x[[5, 6]] = x[[6, 5]]
    assert engine.digest_arrays(*sw) != d.value()
    assert f(ctypes.addressof(d), 5, 1, words, mt, bits.ctypes.data, owner.ctypes.data, xam.ctypes.data,
             evp.ctypes.data) != 0
