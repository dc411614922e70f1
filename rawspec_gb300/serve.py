"""ctypes mirror of include/rawspec_gb300_serve.h: the spectrometer job server
(jobs admitted under a device-memory budget, their buffers processed
concurrently on one GPU, block-to-dump latencies recorded)."""
from __future__ import annotations

import ctypes as C
import threading
from typing import Sequence

import numpy as np

from .api import RAWSPEC_CALLBACK_POST_DUMP, RawspecContext, load_library, make_context

JOB_PENDING, JOB_ACTIVE, JOB_DONE, JOB_FAILED = 0, 1, 2, 3

JOB_DUMP_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.POINTER(RawspecContext), C.c_int, C.c_int)


class JobStats(C.Structure):
    _fields_ = [("state", C.c_int), ("buffers", C.c_longlong), ("dumps", C.c_longlong),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("buffer_p50_ms", C.c_double), ("buffer_p99_ms", C.c_double),
                ("dump_p50_ms", C.c_double), ("dump_p99_ms", C.c_double), ("device_bytes", C.c_size_t)]


class ServerStats(C.Structure):
    _fields_ = [("pending", C.c_int), ("active", C.c_int), ("done", C.c_int), ("failed", C.c_int),
                ("budget", C.c_size_t), ("used", C.c_size_t), ("peak_used", C.c_size_t), ("peak_active", C.c_int),
                ("buffers", C.c_longlong), ("dumps", C.c_longlong),
                ("buffer_p50_ms", C.c_double), ("buffer_p99_ms", C.c_double),
                ("dump_p50_ms", C.c_double), ("dump_p99_ms", C.c_double), ("group_calls", C.c_longlong)]


_declared = False


def lib() -> C.CDLL:
    global _declared
    L = load_library()
    if not _declared:
        S = C.c_void_p
        sig = {
            "rawspec_gb300_server_create": (S, [C.c_int, C.c_size_t, C.c_int, C.c_int]),
            "rawspec_gb300_server_submit": (C.c_int, [S, C.POINTER(RawspecContext), C.c_int, JOB_DUMP_FN, C.c_void_p]),
            "rawspec_gb300_server_push": (C.c_int, [S, C.c_int, C.c_void_p, C.c_size_t]),
            "rawspec_gb300_server_close_job": (C.c_int, [S, C.c_int]),
            "rawspec_gb300_server_wait_job": (C.c_int, [S, C.c_int, C.c_double]),
            "rawspec_gb300_server_job_stats": (C.c_int, [S, C.c_int, C.POINTER(JobStats)]),
            "rawspec_gb300_server_get_stats": (C.c_int, [S, C.POINTER(ServerStats)]),
            "rawspec_gb300_server_destroy": (None, [S]),
            "rawspec_gb300_device_bytes_estimate": (C.c_int, [C.POINTER(RawspecContext), C.POINTER(C.c_size_t)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _declared = True
    return L


def device_bytes_estimate(ctx: RawspecContext) -> int:
    n = C.c_size_t()
    if lib().rawspec_gb300_device_bytes_estimate(C.byref(ctx), C.byref(n)) != 0:
        raise ValueError("invalid context")
    return n.value


class Server:
    """A job server on one GPU.  With collect=True every POST_DUMP's output
    (and incoherent sum) is copied into dumps[job][product] / ics[job][product]."""

    def __init__(self, budget_bytes: int, max_active: int = 8, max_queued: int = 2, gpu: int = 0,
                 collect: bool = True):
        self.lib = lib()
        self.h = self.lib.rawspec_gb300_server_create(gpu, budget_bytes, max_active, max_queued)
        if not self.h:
            raise RuntimeError("rawspec_gb300_server_create failed")
        self.collect = collect
        self.gpu = gpu
        self.dumps: dict[int, list[list[np.ndarray]]] = {}
        self.ics: dict[int, list[list[np.ndarray]]] = {}
        self.buffer_bytes: dict[int, int] = {}
        self._lock = threading.Lock()
        self._cb = JOB_DUMP_FN(self._on_dump)

    def _on_dump(self, user, job, pctx, product, kind):
        if kind != RAWSPEC_CALLBACK_POST_DUMP or not self.collect:
            return
        ctx = pctx.contents
        n = ctx.h_pwrbuf_size[product] // 4
        d = np.ctypeslib.as_array(ctx.h_pwrbuf[product], shape=(n,)).copy()
        s = (np.ctypeslib.as_array(ctx.h_icsbuf[product], shape=(n // ctx.Nant,)).copy()
             if ctx.incoherently_sum else None)
        with self._lock:
            self.dumps[job][product].append(d)
            if s is not None:
                self.ics[job][product].append(s)

    def submit(self, Nc: int, Np: int, Ntpb: int, nbits: int, products: Sequence[tuple[int, int, int]], *,
               Nant: int = 1, Nb: int = 0, conj: int = 0, fft_dir: int = 1,
               weights: Sequence[float] | None = None) -> int:
        ctx = make_context(Nc, Np, Ntpb, nbits, products, Nant=Nant, Nb=Nb, conj=conj, gpu_index=self.gpu,
                           weights=weights)
        job = self.lib.rawspec_gb300_server_submit(self.h, C.byref(ctx), fft_dir, self._cb, None)
        if job < 0:
            raise ValueError("job rejected (invalid, or larger than the memory budget)")
        v = make_context(Nc, Np, Ntpb, nbits, products, Nant=Nant, Nb=Nb, conj=conj, gpu_index=self.gpu,
                         weights=weights)
        load_library().rawspec_gb300_validate(C.byref(v))
        blk = Nc * Ntpb * Np if nbits == 4 else Nc * Ntpb * Np * 2 * (nbits // 8)
        self.buffer_bytes[job] = blk * v.Nb
        with self._lock:
            self.dumps[job] = [[] for _ in products]
            self.ics[job] = [[] for _ in products]
        return job

    def push(self, job: int, blocks: np.ndarray) -> None:
        """One buffer: Nb host blocks (rows of `blocks`, uint8)."""
        a = np.ascontiguousarray(blocks, dtype=np.uint8)
        if self.lib.rawspec_gb300_server_push(self.h, job, a.ctypes.data, a.nbytes) != 0:
            raise RuntimeError(f"push to job {job} failed")

    def close_job(self, job: int) -> None:
        if self.lib.rawspec_gb300_server_close_job(self.h, job) != 0:
            raise RuntimeError(f"close of job {job} failed")

    def wait_job(self, job: int, timeout: float = -1.0) -> int:
        return self.lib.rawspec_gb300_server_wait_job(self.h, job, timeout)

    def job_stats(self, job: int) -> JobStats:
        st = JobStats()
        if self.lib.rawspec_gb300_server_job_stats(self.h, job, C.byref(st)) != 0:
            raise KeyError(job)
        return st

    def stats(self) -> ServerStats:
        st = ServerStats()
        self.lib.rawspec_gb300_server_get_stats(self.h, C.byref(st))
        return st

    def close(self) -> None:
        if self.h:
            self.lib.rawspec_gb300_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
