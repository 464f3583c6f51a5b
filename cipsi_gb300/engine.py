"""ctypes binding of the engine's C ABI (include/cipsi_gb300.h).

`Inputs` holds one run's host-side inputs (read from a calculation directory
like cip does); `Context` is one engine context on one GPU.  Typical use:

    inp = Inputs(workdir, variant="cipsym")
    with Context(inp.dims, device=0) as ctx:
        ctx.upload(inp)                  # host -> device
        res = ctx.run(inp.opts)          # pertu + diexcit on the GPU
        sel = ctx.selection(res["n_selected"])
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import CipsiError, load_library

MAX_ROOTS = 8
NCLASS = 10


class Dims(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int32) for f in ("norb", "noca", "nsym", "isym", "isz", "metat", "ncf")]


class Opts(ctypes.Structure):
    _fields_ = [("yen", ctypes.c_int32), ("ysele", ctypes.c_int32), ("ymoyen", ctypes.c_int32),
                ("ywdeg", ctypes.c_int32), ("sym_variant", ctypes.c_int32), ("nclass", ctypes.c_int32),
                ("tau", ctypes.c_double), ("teseff", ctypes.c_double),
                ("aval", ctypes.c_double * NCLASS), ("gen_mask", ctypes.c_void_p),
                ("run_pertu", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("e2mp", ctypes.c_double * MAX_ROOTS), ("e2vp", ctypes.c_double * MAX_ROOTS),
                ("e2b", ctypes.c_double * MAX_ROOTS), ("psimp", ctypes.c_double * MAX_ROOTS),
                ("psivp", ctypes.c_double * MAX_ROOTS), ("dpivot", ctypes.c_double),
                ("ietat", ctypes.c_int64), ("n_processed", ctypes.c_int64),
                ("n_selected", ctypes.c_int64), ("nom", ctypes.c_int64 * NCLASS),
                ("nam", ctypes.c_int64 * (NCLASS * MAX_ROOTS)),
                ("tabmp", ctypes.c_double * (NCLASS * MAX_ROOTS)),
                ("tabvp", ctypes.c_double * (NCLASS * MAX_ROOTS)),
                ("n_candidates", ctypes.c_int64), ("n_compares", ctypes.c_int64),
                ("n_pairs_1", ctypes.c_int64), ("n_pairs_2", ctypes.c_int64),
                ("alg_bytes", ctypes.c_int64), ("kernel_ms", ctypes.c_double)]


_bound = False


def _lib():
    global _bound
    lib = load_library()
    if _bound:
        return lib
    P = ctypes.c_void_p
    sig = {
        "cipsi_ctx_create": ([ctypes.POINTER(P), ctypes.POINTER(Dims), ctypes.c_int32], ctypes.c_int),
        "cipsi_ctx_destroy": ([P], None),
        "cipsi_last_error": ([P], ctypes.c_char_p),
        "cipsi_set_stream": ([P, P], ctypes.c_int),
        "cipsi_run_pt2": ([P, ctypes.POINTER(Opts), ctypes.POINTER(Result)], ctypes.c_int),
        "cipsi_run_pt2_async": ([P, ctypes.POINTER(Opts)], ctypes.c_int),
        "cipsi_fetch_result": ([P, ctypes.POINTER(Result)], ctypes.c_int),
        "cipsi_selection_get": ([P, ctypes.c_int64, ctypes.c_int64, P, P, P, P, P, P], ctypes.c_int),
        "cipsi_selection_raw": ([P, ctypes.c_int64, ctypes.c_int64, P, P, P, P], ctypes.c_int),
        "cipsi_inputs_read": ([ctypes.POINTER(P), ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                               ctypes.c_char_p, ctypes.c_int32], ctypes.c_int),
        "cipsi_inputs_dims": ([P, ctypes.POINTER(Dims), ctypes.POINTER(Opts)], ctypes.c_int),
        "cipsi_inputs_upload": ([P, P], ctypes.c_int),
        "cipsi_inputs_free": ([P], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _bound = True
    return lib


def result_dict(r: Result, metat: int, nclass: int = NCLASS) -> dict:
    d = {k: list(getattr(r, k))[:metat] for k in ("e2mp", "e2vp", "e2b", "psimp", "psivp")}
    for k in ("dpivot", "ietat", "n_processed", "n_selected", "n_candidates", "n_compares",
              "n_pairs_1", "n_pairs_2", "alg_bytes", "kernel_ms"):
        d[k] = getattr(r, k)
    d["nom"] = list(r.nom)[:nclass]
    d["nam"] = [[r.nam[c * MAX_ROOTS + m] for c in range(nclass)] for m in range(metat)]
    d["tabmp"] = [[r.tabmp[c * MAX_ROOTS + m] for c in range(nclass)] for m in range(metat)]
    d["tabvp"] = [[r.tabvp[c * MAX_ROOTS + m] for c in range(nclass)] for m in range(metat)]
    return d


class Inputs:
    """Host-side inputs of one run (no device work)."""

    def __init__(self, workdir: str, variant: str = "cipsym", stdin_path: Optional[str] = None):
        lib = _lib()
        self._h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(2048)
        rc = lib.cipsi_inputs_read(ctypes.byref(self._h), os.fspath(workdir).encode(),
                                   (stdin_path or os.path.join(workdir, "cip.in")).encode(),
                                   1 if variant == "cipsym" else 0, err, len(err))
        if rc != 0:
            raise CipsiError(err.value.decode(errors="replace"))
        self.dims = Dims()
        self.opts = Opts()
        lib.cipsi_inputs_dims(self._h, ctypes.byref(self.dims), ctypes.byref(self.opts))

    def close(self):
        if self._h:
            _lib().cipsi_inputs_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One engine context on one CUDA device."""

    def __init__(self, dims: Dims, device: int = 0):
        self.lib = _lib()
        self.dims = dims
        self._c = ctypes.c_void_p()
        rc = self.lib.cipsi_ctx_create(ctypes.byref(self._c), ctypes.byref(dims), device)
        if rc != 0:
            msg = self.lib.cipsi_last_error(self._c).decode()
            self.lib.cipsi_ctx_destroy(self._c)
            self._c = ctypes.c_void_p()
            raise CipsiError(msg)
        self._mask_keep = None

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise CipsiError(f"{what}: {self.lib.cipsi_last_error(self._c).decode()}")

    def set_stream(self, stream_handle: int):
        self._check(self.lib.cipsi_set_stream(self._c, ctypes.c_void_p(stream_handle)), "set_stream")

    def upload(self, inp: Inputs):
        self._check(self.lib.cipsi_inputs_upload(inp._h, self._c), "inputs_upload")

    def _opts(self, opts: Opts, gen_mask: Optional[np.ndarray], run_pertu: Optional[bool]) -> Opts:
        o = Opts.from_buffer_copy(opts)
        if gen_mask is not None:
            self._mask_keep = np.ascontiguousarray(gen_mask, dtype=np.uint8)
            o.gen_mask = self._mask_keep.ctypes.data
        if run_pertu is not None:
            o.run_pertu = 1 if run_pertu else 0
        return o

    def run(self, opts: Opts, gen_mask: Optional[np.ndarray] = None,
            run_pertu: Optional[bool] = None) -> dict:
        o = self._opts(opts, gen_mask, run_pertu)
        r = Result()
        self._check(self.lib.cipsi_run_pt2(self._c, ctypes.byref(o), ctypes.byref(r)), "run_pt2")
        return result_dict(r, self.dims.metat, o.nclass)

    def run_async(self, opts: Opts, gen_mask: Optional[np.ndarray] = None,
                  run_pertu: Optional[bool] = None):
        o = self._opts(opts, gen_mask, run_pertu)
        self._last_nclass = o.nclass
        self._check(self.lib.cipsi_run_pt2_async(self._c, ctypes.byref(o)), "run_pt2_async")

    def fetch(self) -> dict:
        r = Result()
        self._check(self.lib.cipsi_fetch_result(self._c, ctypes.byref(r)), "fetch_result")
        return result_dict(r, self.dims.metat, getattr(self, "_last_nclass", NCLASS))

    def selection(self, count: int) -> dict:
        mt = self.dims.metat
        nec = np.zeros(count, np.int32)
        h = np.zeros((count, 8), np.int32)
        p = np.zeros((count, 8), np.int32)
        xam = np.zeros(count, np.float64)
        evp = np.zeros((count, mt), np.float64)
        own = np.zeros(count, np.int32)
        if count:
            self._check(self.lib.cipsi_selection_get(
                self._c, 0, count, nec.ctypes.data, h.ctypes.data, p.ctypes.data, xam.ctypes.data,
                evp.ctypes.data, own.ctypes.data), "selection_get")
        return {"nec": nec, "holes": h, "parts": p, "xam": xam, "evp": evp, "owner": own}

    def selection_raw(self, count: int, out: Optional[dict] = None) -> dict:
        """Selected records as bitstrings (no conversion): bits[count, 2W],
        owner, xam, evp.  `out` may supply preallocated (pinned) arrays."""
        mt = self.dims.metat
        W = 1 if self.dims.norb <= 64 else 2
        if out is None:
            out = {"bits": np.zeros((count, 2 * W), np.uint64), "owner": np.zeros(count, np.int32),
                   "xam": np.zeros(count, np.float64), "evp": np.zeros((count, mt), np.float64)}
        if count:
            self._check(self.lib.cipsi_selection_raw(
                self._c, 0, count, out["bits"].ctypes.data, out["owner"].ctypes.data,
                out["xam"].ctypes.data, out["evp"].ctypes.data), "selection_raw")
        return out

    def close(self):
        if self._c:
            self.lib.cipsi_ctx_destroy(self._c)
            self._c = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
