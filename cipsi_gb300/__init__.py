"""GB300 engine for the CIPSI second-order perturbation / selection step.

Python mirror of the reference's process-level interface: `run_cip` does what
running cip.exe (variant="cip") or cipsym.exe (variant="cipsym") in a
calculation directory does, with the perturbation loop on the GPU; `run_moy`
does what moy.exe does (the Hamiltonian over S + the selected perturbers),
with the pair scan and matrix elements on the GPU; `run_bd` does what bd.exe
does (the lowest eigenpairs of that matrix), with a Davidson iteration on
the GPU.  The
compiled library is built in-tree by `cipsi_gb300.build.build()`; when it is
missing every entry point raises instead of falling back to a CPU path.
"""
from __future__ import annotations

import ctypes
import json
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcipsi_gb300.so")
EXE_PATH = os.path.join(_HERE, "_build", "cip_gpu")
MOY_EXE_PATH = os.path.join(_HERE, "_build", "moy_gpu")
BD_EXE_PATH = os.path.join(_HERE, "_build", "bd_gpu")

_lib = None

EXPORTED = [
    "cipsi_ctx_create", "cipsi_ctx_destroy", "cipsi_last_error", "cipsi_set_stream",
    "cipsi_set_integrals", "cipsi_set_integrals_fp64", "cipsi_set_space", "cipsi_set_roots",
    "cipsi_run_pt2", "cipsi_run_pt2_async", "cipsi_fetch_result", "cipsi_selection_get",
    "cipsi_cip_main", "cipsi_inputs_read", "cipsi_inputs_dims", "cipsi_inputs_upload",
    "cipsi_inputs_free", "cipsi_selection_raw", "cipsi_run_pt2_static",
    "cipsi_set_tuning", "cipsi_batch_create", "cipsi_batch_run", "cipsi_batch_wait",
    "cipsi_batch_last_error", "cipsi_batch_destroy", "cipsi_inputs_array", "cipsi_set_integrals_f64store",
    "cipsi_run_pt2_adjoint", "cipsi_run_pt2_adjoint_1e", "cipsi_set_selection_sink", "cipsi_run_pt2_stream", "cipsi_record_digest",
    "cipsi_hamiltonian_build", "cipsi_hamiltonian_get", "cipsi_hamiltonian_ms", "cipsi_moy_main",
    "cipsi_davidson", "cipsi_bd_main",
]


class CipsiError(RuntimeError):
    pass


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the engine; raises if it was not built (no silent fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CipsiError(f"engine library {path} is missing: run cipsi_gb300.build.build()")
    lib = ctypes.CDLL(path)
    lib.cipsi_cip_main.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_char_p,
                                   ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p, ctypes.c_int32]
    lib.cipsi_cip_main.restype = ctypes.c_int
    lib.cipsi_moy_main.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                   ctypes.c_char_p, ctypes.c_int32]
    lib.cipsi_moy_main.restype = ctypes.c_int
    lib.cipsi_bd_main.argtypes = lib.cipsi_moy_main.argtypes
    lib.cipsi_bd_main.restype = ctypes.c_int
    _lib = lib
    return lib


def run_cip(workdir: str, variant: str = "cipsym", json_path: Optional[str] = None,
            gen_mask: Optional[np.ndarray] = None, device: int = 0,
            stdin_path: Optional[str] = None) -> dict:
    """Run the GPU drop-in in `workdir` (namelists from `stdin_path`, default
    workdir/cip.in).  Returns the JSON summary (E2 totals, counters)."""
    lib = load_library()
    if json_path is None:
        json_path = os.path.join(workdir, "cip_gpu.json")
    err = ctypes.create_string_buffer(2048)
    mask_ptr = None
    if gen_mask is not None:
        gen_mask = np.ascontiguousarray(gen_mask, dtype=np.uint8)
        mask_ptr = gen_mask.ctypes.data_as(ctypes.c_void_p)
    rc = lib.cipsi_cip_main(workdir.encode(), (stdin_path or os.path.join(workdir, "cip.in")).encode(),
                            1 if variant == "cipsym" else 0, json_path.encode(), mask_ptr, device,
                            err, len(err))
    if rc != 0:
        raise CipsiError(err.value.decode(errors="replace"))
    with open(json_path) as fh:
        return json.load(fh)


def run_moy(workdir: str, json_path: Optional[str] = None, device: int = 0,
            stdin_path: Optional[str] = None) -> dict:
    """Run the moy drop-in in `workdir` (namelists &moyfil/&moyen from
    `stdin_path`, default workdir/moy.in).  Returns the JSON summary (list
    size, element counts, morue's second-order sums, device time)."""
    lib = load_library()
    if json_path is None:
        json_path = os.path.join(workdir, "moy_gpu.json")
    err = ctypes.create_string_buffer(2048)
    rc = lib.cipsi_moy_main(workdir.encode(), (stdin_path or os.path.join(workdir, "moy.in")).encode(),
                            json_path.encode(), device, err, len(err))
    if rc != 0:
        raise CipsiError(err.value.decode(errors="replace"))
    with open(json_path) as fh:
        return json.load(fh)


def run_bd(workdir: str, json_path: Optional[str] = None, device: int = 0,
           stdin_path: Optional[str] = None) -> dict:
    """Run the bd drop-in in `workdir` (namelists &bdfil/&option from
    `stdin_path`, default workdir/bd.in).  Returns the JSON summary
    (eigenvalues, residual norms, iterations)."""
    lib = load_library()
    if json_path is None:
        json_path = os.path.join(workdir, "bd_gpu.json")
    err = ctypes.create_string_buffer(2048)
    rc = lib.cipsi_bd_main(workdir.encode(), (stdin_path or os.path.join(workdir, "bd.in")).encode(),
                           json_path.encode(), device, err, len(err))
    if rc != 0:
        raise CipsiError(err.value.decode(errors="replace"))
    with open(json_path) as fh:
        return json.load(fh)
