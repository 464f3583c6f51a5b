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
                ("alg_bytes", ctypes.c_int64), ("kernel_ms", ctypes.c_double), ("pt2_ms", ctypes.c_double),
                ("launches", ctypes.c_int64)]


class Digest(ctypes.Structure):
    """cipsi_digest: order-sensitive digest of streamed records."""
    _fields_ = [("s1", ctypes.c_uint64 * 4), ("s2", ctypes.c_uint64 * 4), ("records", ctypes.c_int64),
                ("threads", ctypes.c_int32)]

    def value(self) -> tuple:
        return tuple(self.s1) + tuple(self.s2)


# cipsi_record_fn
RECORD_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)


def digest_arrays(bits, owner, xam, evp, state=None) -> tuple:
    """The cipsi_digest pair sums of record arrays (numpy restatement of
    cipsi_record_digest, for checks): per field array, s1 = sum of its 64-bit
    words and s2 = sum of the running s1, modulo 2^64, continuing `state`."""
    s1 = list(state[:4]) if state else [0] * 4
    s2 = list(state[4:]) if state else [0] * 4
    arrays = [np.ascontiguousarray(bits, np.uint64).ravel(),
              np.ascontiguousarray(owner, np.int32).ravel().view(np.uint32).astype(np.uint64),
              np.ascontiguousarray(xam, np.float64).ravel().view(np.uint64),
              np.ascontiguousarray(evp, np.float64).ravel().view(np.uint64)]
    for f, w in enumerate(arrays):
        with np.errstate(over="ignore"):
            run = np.cumsum(w, dtype=np.uint64) + np.uint64(s1[f])
            s2[f] = (s2[f] + int(run.sum(dtype=np.uint64))) % (1 << 64) if len(w) else s2[f]
            s1[f] = int(run[-1]) if len(w) else s1[f]
    return tuple(s1) + tuple(s2)


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
        "cipsi_set_tuning": ([P, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "cipsi_set_selection_sink": ([P, P, P, P, P, ctypes.c_int64], ctypes.c_int),
        "cipsi_fetch_result": ([P, ctypes.POINTER(Result)], ctypes.c_int),
        "cipsi_selection_get": ([P, ctypes.c_int64, ctypes.c_int64, P, P, P, P, P, P], ctypes.c_int),
        "cipsi_selection_raw": ([P, ctypes.c_int64, ctypes.c_int64, P, P, P, P], ctypes.c_int),
        "cipsi_inputs_read": ([ctypes.POINTER(P), ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                               ctypes.c_char_p, ctypes.c_int32], ctypes.c_int),
        "cipsi_inputs_dims": ([P, ctypes.POINTER(Dims), ctypes.POINTER(Opts)], ctypes.c_int),
        "cipsi_inputs_upload": ([P, P], ctypes.c_int),
        "cipsi_inputs_free": ([P], None),
        "cipsi_batch_create": ([ctypes.POINTER(P), ctypes.POINTER(P), ctypes.c_int32, ctypes.POINTER(Opts),
                                ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "cipsi_batch_run": ([P], ctypes.c_int),
        "cipsi_batch_wait": ([P, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "cipsi_batch_last_error": ([P], ctypes.c_char_p),
        "cipsi_batch_destroy": ([P], None),
        "cipsi_inputs_array": ([P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
        "cipsi_set_integrals_f64store": ([P, P, P, P, P, P, P, P, P, ctypes.c_int64], ctypes.c_int),
        "cipsi_set_roots": ([P, P, P, P, P, P, P, P], ctypes.c_int),
        "cipsi_run_pt2_adjoint": ([P, ctypes.POINTER(Opts), P, P, P, P, P, P, P], ctypes.c_int),
        "cipsi_run_pt2_adjoint_1e": ([P, ctypes.POINTER(Opts), P, P, P, P, P, P, P], ctypes.c_int),
        "cipsi_run_pt2_stream": ([P, ctypes.POINTER(Opts), ctypes.c_int64, P, P, ctypes.POINTER(Result)],
                                 ctypes.c_int),
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
              "n_pairs_1", "n_pairs_2", "alg_bytes", "kernel_ms", "pt2_ms", "launches"):
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

    _TYPES = {1: np.int32, 2: np.int16, 3: np.float32, 4: np.float64, 5: np.uint8}

    def count(self, name: str) -> int:
        data, count, typ = ctypes.c_void_p(), ctypes.c_int64(), ctypes.c_int32()
        if _lib().cipsi_inputs_array(self._h, name.encode(), ctypes.byref(data), ctypes.byref(count),
                                     ctypes.byref(typ)) != 0:
            raise CipsiError(f"no input array named {name!r}")
        return count.value

    def array(self, name: str) -> np.ndarray:
        """A copy of one input array (cipsi_inputs_array)."""
        data = ctypes.c_void_p()
        count = ctypes.c_int64()
        typ = ctypes.c_int32()
        rc = _lib().cipsi_inputs_array(self._h, name.encode(), ctypes.byref(data), ctypes.byref(count),
                                       ctypes.byref(typ))
        if rc != 0:
            raise CipsiError(f"no input array named {name!r}")
        dt = np.dtype(self._TYPES[typ.value])
        if count.value == 0:
            return np.zeros(0, dt)
        buf = (ctypes.c_char * (count.value * dt.itemsize)).from_address(data.value)
        return np.frombuffer(buf, dtype=dt).copy()

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

    def set_selection_sink(self, out: Optional[dict]):
        """Have the kernel write the unit-60 records into `out` (pinned host
        arrays: bits [cap, 2W] uint64, owner [cap] int32, xam [cap] float64,
        evp [cap, metat] float64, as selection_raw returns); None = device
        buffers again."""
        if out is None:
            self._sink = None
            self._check(self.lib.cipsi_set_selection_sink(self._c, None, None, None, None, 0), "set_selection_sink")
            return
        cap = len(out["owner"])
        self._sink = out
        self._check(self.lib.cipsi_set_selection_sink(
            self._c, out["bits"].ctypes.data, out["owner"].ctypes.data, out["xam"].ctypes.data,
            out["evp"].ctypes.data, cap), "set_selection_sink")

    def set_tuning(self, r_chunk: int = 6, ctas_per_sm: int = 0):
        self._check(self.lib.cipsi_set_tuning(self._c, r_chunk, ctas_per_sm), "set_tuning")

    def set_integrals_f64store(self, itsym, its, F, J, K, ij0, ntttt, eri):
        """Integrals with (pq|rs) kept in FP64 on the device."""
        a = [np.ascontiguousarray(itsym, np.int32), np.ascontiguousarray(its, np.int32),
             np.ascontiguousarray(F, np.float64), np.ascontiguousarray(J, np.float64),
             np.ascontiguousarray(K, np.float64), np.ascontiguousarray(ij0, np.int16),
             np.ascontiguousarray(ntttt, np.int32), np.ascontiguousarray(eri, np.float64)]
        self._check(self.lib.cipsi_set_integrals_f64store(self._c, *[x.ctypes.data for x in a], len(a[7])),
                    "set_integrals_f64store")
        self._ninte = len(a[7])

    def set_roots(self, c, e, eb, emp, teste, taum, fmpb):
        a = [np.ascontiguousarray(x, np.float64) for x in (c, e, eb, emp, teste, taum, fmpb)]
        self._check(self.lib.cipsi_set_roots(self._c, *[x.ctypes.data for x in a]), "set_roots")

    def adjoint(self, opts: Opts, seed) -> dict:
        """Gradients of sum(seed * [e2mp; e2vp; e2b]) (cipsi_run_pt2_adjoint)."""
        n, mt = self.dims.norb, self.dims.metat
        nt = n * (n + 1) // 2
        seed = np.ascontiguousarray(np.asarray(seed, np.float64).reshape(3 * mt))
        out = {"F": np.zeros(nt), "J": np.zeros(nt), "K": np.zeros(nt), "eri": np.zeros(self._ninte),
               "fmpb": np.zeros(2 * n), "roots": np.zeros(3 * mt)}
        o = Opts.from_buffer_copy(opts)
        self._check(self.lib.cipsi_run_pt2_adjoint(
            self._c, ctypes.byref(o), seed.ctypes.data, out["F"].ctypes.data, out["J"].ctypes.data,
            out["K"].ctypes.data, out["eri"].ctypes.data, out["fmpb"].ctypes.data, out["roots"].ctypes.data),
            "run_pt2_adjoint")
        r = out.pop("roots")
        out["e"], out["eb"], out["emp"] = r[:mt], r[mt:2 * mt], r[2 * mt:]
        return out

    def adjoint_1e(self, opts: Opts, seed) -> tuple:
        """E2 sums [3, metat] and the gradients of sum(seed * E2) except the
        (pq|rs) one, from one pass (cipsi_run_pt2_adjoint_1e)."""
        n, mt = self.dims.norb, self.dims.metat
        nt = n * (n + 1) // 2
        seed = np.ascontiguousarray(np.asarray(seed, np.float64).reshape(3 * mt))
        e2 = np.zeros(3 * mt)
        out = {"F": np.zeros(nt), "J": np.zeros(nt), "K": np.zeros(nt), "fmpb": np.zeros(2 * n),
               "roots": np.zeros(3 * mt)}
        o = Opts.from_buffer_copy(opts)
        self._check(self.lib.cipsi_run_pt2_adjoint_1e(
            self._c, ctypes.byref(o), seed.ctypes.data, e2.ctypes.data, out["F"].ctypes.data,
            out["J"].ctypes.data, out["K"].ctypes.data, out["fmpb"].ctypes.data, out["roots"].ctypes.data),
            "run_pt2_adjoint_1e")
        r = out.pop("roots")
        out["e"], out["eb"], out["emp"] = r[:mt], r[mt:2 * mt], r[2 * mt:]
        return e2.reshape(3, mt), out

    def upload(self, inp: Inputs):
        self._check(self.lib.cipsi_inputs_upload(inp._h, self._c), "inputs_upload")
        self._ninte = inp.count("eri")

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

    def run_stream(self, opts: Opts, chunk_records: int = 0, consumer=None, gen_mask: Optional[np.ndarray] = None,
                   run_pertu: Optional[bool] = None) -> dict:
        """cipsi_run_pt2_stream.  consumer: None (records stay on the device),
        a Digest (the library's native digest consumer), or a Python callable
        f(first, bits, owner, xam, evp) given numpy copies of each piece."""
        o = self._opts(opts, gen_mask, run_pertu)
        r = Result()
        mt = self.dims.metat
        keep = None
        if consumer is None:
            fn, user = None, None
        elif isinstance(consumer, Digest):
            fn = ctypes.cast(self.lib.cipsi_record_digest, ctypes.c_void_p).value
            user = ctypes.addressof(consumer)
        else:
            def _cb(user_, first, count, words, metat, bits, owner, xam, evp):
                try:
                    def arr(ptr, ctype, n):
                        return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctype)), shape=(n,)).copy()
                    consumer(first, arr(bits, ctypes.c_uint64, count * words).reshape(count, words),
                             arr(owner, ctypes.c_int32, count), arr(xam, ctypes.c_double, count),
                             arr(evp, ctypes.c_double, count * metat).reshape(count, metat))
                    return 0
                except Exception:  # noqa: BLE001 -- any failure stops the run
                    return 1
            keep = RECORD_FN(_cb)
            fn, user = ctypes.cast(keep, ctypes.c_void_p).value, None
        self._last_nclass = o.nclass
        self._check(self.lib.cipsi_run_pt2_stream(self._c, ctypes.byref(o), chunk_records, fn, user,
                                                  ctypes.byref(r)), "run_pt2_stream")
        del keep
        return result_dict(r, mt, o.nclass)

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


class Batch:
    """Runs of many contexts (geometries) in one persistent launch per class,
    captured as a CUDA graph (cipsi_batch_* in the C ABI).

        b = Batch(contexts, [inp.opts for inp in inputs])
        b.run(); ms = b.wait()
        results = [ctx.fetch() for ctx in contexts]
    """

    def __init__(self, contexts, opts_list, r_chunk: int = 6, ctas_per_sm: int = 0, gen_masks=None):
        self.lib = _lib()
        n = len(contexts)
        if n == 0 or len(opts_list) != n:
            raise CipsiError("Batch needs one Opts per context")
        self.contexts = list(contexts)
        arr = (ctypes.c_void_p * n)(*[c._c.value for c in contexts])
        opts = (Opts * n)()
        keep = []
        for i, o in enumerate(opts_list):
            opts[i] = Opts.from_buffer_copy(o)
            if gen_masks is not None and gen_masks[i] is not None:
                m = np.ascontiguousarray(gen_masks[i], dtype=np.uint8)
                keep.append(m)
                opts[i].gen_mask = m.ctypes.data
        self._h = ctypes.c_void_p()
        rc = self.lib.cipsi_batch_create(ctypes.byref(self._h), arr, n, opts, r_chunk, ctas_per_sm)
        if rc != 0:
            msg = self.lib.cipsi_batch_last_error(self._h).decode()
            self.lib.cipsi_batch_destroy(self._h)
            self._h = ctypes.c_void_p()
            raise CipsiError(f"batch_create: {msg}")
        self.nclass = [o.nclass for o in opts_list]

    def _check(self, rc, what):
        if rc != 0:
            raise CipsiError(f"{what}: {self.lib.cipsi_batch_last_error(self._h).decode()}")

    def run(self):
        self._check(self.lib.cipsi_batch_run(self._h), "batch_run")
        for c, nc in zip(self.contexts, self.nclass):
            c._last_nclass = nc

    def wait(self) -> float:
        ms = ctypes.c_double()
        self._check(self.lib.cipsi_batch_wait(self._h, ctypes.byref(ms)), "batch_wait")
        return ms.value

    def fetch_all(self, allow_overflow: bool = True) -> list:
        """Every context's result; a selection-capacity overflow (records
        counted but not all stored) is accepted when allow_overflow."""
        out = []
        for c, nc in zip(self.contexts, self.nclass):
            r = Result()
            rc = c.lib.cipsi_fetch_result(c._c, ctypes.byref(r))
            if rc != 0 and not (allow_overflow and rc == -4):
                raise CipsiError(f"fetch_result: {c.lib.cipsi_last_error(c._c).decode()}")
            d = result_dict(r, c.dims.metat, nc)
            d["overflow"] = rc == -4
            out.append(d)
        return out

    def close(self):
        if self._h:
            self.lib.cipsi_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
