"""ctypes wrapper of the CPU restatements (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import build as _build


class OracleCfg(C.Structure):
    _fields_ = [
        ("Nc", C.c_int), ("Np", C.c_int), ("Ntpb", C.c_int), ("Nb", C.c_int),
        ("nbits", C.c_int), ("Nant", C.c_int), ("No", C.c_int),
        ("Nts", C.c_int * 4), ("Nas", C.c_int * 4), ("Npolout", C.c_int * 4),
        ("conj", C.c_int), ("inverse", C.c_int), ("ics", C.c_int),
        ("weights", C.POINTER(C.c_float)),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(_build.build()))
        P = C.POINTER(OracleCfg)
        _lib.oracle_block_bytes.restype = C.c_long
        _lib.oracle_block_bytes.argtypes = [P]
        _lib.oracle_dump_doubles.restype = C.c_long
        _lib.oracle_dump_doubles.argtypes = [P, C.c_int]
        _lib.oracle_num_dumps.restype = C.c_long
        _lib.oracle_num_dumps.argtypes = [P, C.c_int, C.c_int]
        _lib.oracle_snorm.restype = C.c_double
        _lib.oracle_snorm.argtypes = [C.c_int, C.c_int]
        _lib.oracle_fft.restype = None
        _lib.oracle_fft.argtypes = [C.POINTER(C.c_double), C.c_long, C.c_int]
        _lib.oracle_run.restype = C.c_int
        _lib.oracle_run.argtypes = [P, C.POINTER(C.c_uint8), C.c_int, C.POINTER(C.POINTER(C.c_double)),
                                    C.POINTER(C.POINTER(C.c_double))]
        _lib.cpu_run.restype = C.c_int
        _lib.cpu_run.argtypes = [P, C.POINTER(C.c_uint8), C.c_int, C.POINTER(C.POINTER(C.c_float)),
                                 C.POINTER(C.POINTER(C.c_float)), C.c_int]
        _lib.cpu_max_threads.restype = C.c_int
    return _lib


def make_cfg(Nc: int, Np: int, Ntpb: int, Nb: int, nbits: int, products: Sequence[tuple[int, int, int]], *,
             Nant: int = 1, conj: int = 0, inverse: int = 0, weights: Sequence[float] | None = None) -> OracleCfg:
    """products: (Nt, Na, Npolout) after the library's coercions."""
    cfg = OracleCfg()
    cfg.Nc, cfg.Np, cfg.Ntpb, cfg.Nb, cfg.nbits = Nc, Np, Ntpb, Nb, nbits
    cfg.Nant = Nant
    cfg.No = len(products)
    for i, (nt, na, npo) in enumerate(products):
        cfg.Nts[i], cfg.Nas[i], cfg.Npolout[i] = nt, na, npo
    cfg.conj, cfg.inverse = conj, inverse
    if weights is not None:
        w = (C.c_float * len(weights))(*[float(x) for x in weights])
        cfg._w = w  # keep alive
        cfg.weights = C.cast(w, C.POINTER(C.c_float))
        cfg.ics = 1
    return cfg


def _run(fn, dtype, ctype, cfg: OracleCfg, blocks: np.ndarray, extra=()):
    L = lib()
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    nblocks = blocks.shape[0]
    nbuf = nblocks // cfg.Nb
    outs, icss = [], []
    out_ptrs = (C.POINTER(ctype) * 4)()
    ics_ptrs = (C.POINTER(ctype) * 4)()
    for i in range(cfg.No):
        nd = L.oracle_num_dumps(C.byref(cfg), i, nbuf)
        n = L.oracle_dump_doubles(C.byref(cfg), i)
        o = np.zeros((nd, n), dtype=dtype)
        outs.append(o)
        out_ptrs[i] = o.ctypes.data_as(C.POINTER(ctype))
        if cfg.ics:
            s = np.zeros((nd, n // max(cfg.Nant, 1)), dtype=dtype)
            icss.append(s)
            ics_ptrs[i] = s.ctypes.data_as(C.POINTER(ctype))
    rc = fn(C.byref(cfg), blocks.ctypes.data_as(C.POINTER(C.c_uint8)), nblocks, out_ptrs, ics_ptrs, *extra)
    if rc != 0:
        raise RuntimeError("oracle run failed")
    return outs, icss


def run_oracle(cfg: OracleCfg, blocks: np.ndarray):
    """FP64 dumps per product: list of [ndumps, Nd*|P|*Nc*Nt] arrays (and ICS)."""
    return _run(lib().oracle_run, np.float64, C.c_double, cfg, blocks)


def run_cpu(cfg: OracleCfg, blocks: np.ndarray, nthreads: int = 0):
    """FP32 OpenMP dumps, same layout as run_oracle."""
    return _run(lib().cpu_run, np.float32, C.c_float, cfg, blocks, (nthreads,))


def snorm(code: int, nbits: int) -> float:
    return lib().oracle_snorm(code, nbits)


def fft(z: np.ndarray, inverse: bool = False) -> np.ndarray:
    a = np.ascontiguousarray(z, dtype=np.complex128).copy()
    lib().oracle_fft(a.ctypes.data_as(C.POINTER(C.c_double)), a.size, 1 if inverse else 0)
    return a
