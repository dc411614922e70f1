"""ctypes mirror of the librawspec C interface (include/rawspec.h).

`RawspecContext` has the member layout of the reference's rawspec_context
(rawspec.h:32-148); `load_library()` binds the twelve reference entry points
(rawspec.h:161-234) and the extensions of include/rawspec_gb300.h.  This is how
a Python client (or the tests and the benchmark) drives the native library;
there is no other compute path: if the shared library is missing,
`load_library()` raises.

`Spectrometer` wraps the usual client sequence of the reference CLI
(rawspec.c:758-1092): initialise, fill host blocks, copy them to the GPU,
start processing, wait, and collect every dump that the POST_DUMP callback
announces.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import Sequence

import numpy as np

MAX_OUTPUTS = 4
RAWSPEC_FORWARD_FFT = +1
RAWSPEC_INVERSE_FFT = -1
RAWSPEC_CALLBACK_PRE_DUMP = 0
RAWSPEC_CALLBACK_POST_DUMP = 1

K_SMALL, K_FINALIZE, K_LARGE_A, K_LARGE_B, K_ICS, K_EXPAND4, K_D2H, K_H2D, K_LARGE_FUSED = range(9)
KERNEL_CLASS_NAMES = ["small", "finalize", "large_a", "large_b", "ics", "expand4", "d2h", "h2d", "large_fused", "tc",
                      "merge"]

LIB_PATH = Path(__file__).resolve().parent / "lib" / "librawspec.so"


class TuneEntry(C.Structure):
    """rawspec_gb300_tune: one entry of the tuning table (-1 / 0: unset)."""
    _fields_ = [("dft", C.c_int), ("ctas", C.c_int), ("lag", C.c_int), ("ring", C.c_int)]


def tune_lookup(nfft: int, nbits: int, npolout: int) -> tuple[int, TuneEntry]:
    """rawspec_gb300_tune_lookup: (1 found / 0 not / -1 unreadable, entry)."""
    t = TuneEntry()
    r = load_library().rawspec_gb300_tune_lookup(nfft, nbits, npolout, C.byref(t))
    return int(r), t


class RawspecContext(C.Structure):
    pass


DUMP_CALLBACK = C.CFUNCTYPE(None, C.POINTER(RawspecContext), C.c_int, C.c_int)

RawspecContext._fields_ = [
    ("No", C.c_uint),
    ("Np", C.c_uint),
    ("Nant", C.c_uint),
    ("Nc", C.c_uint),
    ("Ntpb", C.c_uint),
    ("exit_soon", C.c_uint),
    ("Nbc", C.c_uint),
    ("Nbps", C.c_uint),
    ("Npolout", C.c_int * MAX_OUTPUTS),
    ("Nts", C.c_uint * MAX_OUTPUTS),
    ("Nas", C.c_uint * MAX_OUTPUTS),
    ("dump_callback", DUMP_CALLBACK),
    ("user_data", C.c_void_p),
    ("Nb", C.c_uint),
    ("Nb_host", C.c_uint),
    ("h_blkbufs", C.POINTER(C.c_void_p)),
    ("gpu_index", C.c_int),
    ("input_conjugated", C.c_int),
    ("incoherently_sum", C.c_int),
    ("Naws", C.c_int),
    ("Aws", C.POINTER(C.c_float)),
    ("h_pwrbuf", C.POINTER(C.c_float) * MAX_OUTPUTS),
    ("h_pwrbuf_size", C.c_size_t * MAX_OUTPUTS),
    ("h_icsbuf", C.POINTER(C.c_float) * MAX_OUTPUTS),
    ("Nds", C.c_uint * MAX_OUTPUTS),
    ("Ntmax", C.c_uint),
    ("gpu_ctx", C.c_void_p),
]

_lib = None
_lib_lock = threading.Lock()


def load_library(path: str | Path | None = None) -> C.CDLL:
    """Loads librawspec.so and declares every exported function."""
    global _lib
    with _lib_lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise FileNotFoundError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(str(p))
        P = C.POINTER(RawspecContext)
        sig = {
            "get_librawspec_version": (C.c_char_p, []),
            "get_cufft_version": (C.c_char_p, []),
            "rawspec_initialize": (C.c_int, [P]),
            "rawspec_cleanup": (None, [P]),
            "rawspec_copy_blocks_to_gpu": (C.c_int, [P, C.c_long, C.c_long, C.c_size_t]),
            "rawspec_copy_blocks_to_gpu_expanding_complex4": (C.c_int, [P, C.c_long, C.c_long, C.c_size_t]),
            "rawspec_zero_blocks_to_gpu": (C.c_int, [P, C.c_long, C.c_size_t]),
            "rawspec_start_processing": (C.c_int, [P, C.c_int]),
            "rawspec_copy_blocks_to_gpu_and_start_processing": (C.c_int, [P, C.c_size_t, C.c_char, C.c_int]),
            "rawspec_reset_integration": (C.c_int, [P]),
            "rawspec_check_for_completion": (C.c_uint, [P]),
            "rawspec_wait_for_completion": (C.c_int, [P]),
            "rawspec_gb300_validate": (C.c_int, [P]),
            "rawspec_gb300_product_info": (C.c_int, [P, C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                                    C.POINTER(C.c_uint)]),
            "rawspec_gb300_stream": (C.c_void_p, [P]),
            "rawspec_gb300_device_input": (C.c_void_p, [P, C.POINTER(C.c_size_t)]),
            "rawspec_gb300_set_profiling": (C.c_int, [P, C.c_int]),
            "rawspec_gb300_profile": (C.c_int, [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_ulonglong)]),
            "rawspec_gb300_reset_profile": (C.c_int, [P]),
            "rawspec_gb300_kernel_launches": (C.c_ulonglong, [P]),
            "rawspec_gb300_device_bytes": (C.c_size_t, [P]),
            "rawspec_gb300_product_kernel": (C.c_int, [P, C.c_int]),
            "rawspec_gb300_tune_lookup": (C.c_int, [C.c_uint, C.c_int, C.c_int, C.POINTER(TuneEntry)]),
            "rawspec_gb300_start_processing_group": (C.c_int, [C.POINTER(P), C.POINTER(C.c_int), C.c_int]),
            "rawspec_gb300_shared_launches": (C.c_ulonglong, [P]),
            "rawspec_gb300_shard_range": (C.c_int, [C.c_uint, C.c_uint, C.c_int, C.c_int, C.POINTER(C.c_uint),
                                                   C.POINTER(C.c_uint)]),
            "rawspec_gb300_shard_context": (C.c_int, [P, C.c_int, C.c_int, P]),
            "rawspec_gb300_shard_fill_block": (C.c_int, [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                                        C.c_size_t, C.c_void_p]),
            "rawspec_gb300_shard_place_dump": (C.c_int, [C.POINTER(C.c_float), C.c_uint, C.c_uint, C.c_uint,
                                                        C.c_uint, C.c_uint, C.c_uint, C.c_int,
                                                        C.POINTER(C.c_float)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        if path is None:
            _lib = lib
        return lib


# Names of the functions include/rawspec.h declares (the drop-in boundary).
REFERENCE_ENTRY_POINTS = [
    "get_librawspec_version", "get_cufft_version", "rawspec_initialize", "rawspec_cleanup",
    "rawspec_copy_blocks_to_gpu", "rawspec_copy_blocks_to_gpu_expanding_complex4", "rawspec_zero_blocks_to_gpu",
    "rawspec_start_processing", "rawspec_copy_blocks_to_gpu_and_start_processing", "rawspec_reset_integration",
    "rawspec_check_for_completion", "rawspec_wait_for_completion",
]


def make_context(Nc: int, Np: int, Ntpb: int, nbits: int, products: Sequence[tuple[int, int, int]], *,
                 Nant: int = 1, Nbc: int = 0, Nb: int = 0, conj: int = 0, gpu_index: int = 0,
                 weights: Sequence[float] | None = None) -> RawspecContext:
    """Fills a context like a client would (products are (Nt, Na, Npolout))."""
    ctx = RawspecContext()
    ctx.No = len(products)
    ctx.Np = Np
    ctx.Nant = Nant
    ctx.Nc = Nc
    ctx.Ntpb = Ntpb
    ctx.Nbc = Nbc
    ctx.Nbps = nbits
    for i, (nt, na, npo) in enumerate(products):
        ctx.Nts[i] = nt
        ctx.Nas[i] = na
        ctx.Npolout[i] = npo
    ctx.Nb = Nb
    ctx.gpu_index = gpu_index
    ctx.input_conjugated = conj
    if weights is not None:
        w = (C.c_float * len(weights))(*weights)
        ctx._weights_keepalive = w  # type: ignore[attr-defined]
        ctx.incoherently_sum = 1
        ctx.Naws = len(weights)
        ctx.Aws = C.cast(w, C.POINTER(C.c_float))
    return ctx


def start_group(specs: Sequence["Spectrometer"], fft_dirs: Sequence[int] | None = None) -> None:
    """rawspec_gb300_start_processing_group over the specs' contexts (each
    spec's buffer already copied to the device)."""
    n = len(specs)
    arr = (C.POINTER(RawspecContext) * n)(*[C.pointer(sp.ctx) for sp in specs])
    dirs = (C.c_int * n)(*(fft_dirs if fft_dirs is not None else [RAWSPEC_FORWARD_FFT] * n))
    if load_library().rawspec_gb300_start_processing_group(arr, dirs, n) != 0:
        raise RuntimeError("rawspec_gb300_start_processing_group failed")


def shard_range(Nc: int, Nant: int, rank: int, world: int) -> tuple[int, int]:
    """rawspec_gb300_shard_range: (k0, nk), the channels-within-antenna of a shard."""
    k0, nk = C.c_uint(), C.c_uint()
    if load_library().rawspec_gb300_shard_range(Nc, Nant, rank, world, C.byref(k0), C.byref(nk)) != 0:
        raise ValueError(f"no shard {rank} of {world} for {Nc} channels in {Nant} antennas")
    return k0.value, nk.value


def shard_fill_block(full_block: np.ndarray, Nc: int, Nant: int, k0: int, nk: int) -> np.ndarray:
    """rawspec_gb300_shard_fill_block: the shard's channels of one full host block."""
    full_block = np.ascontiguousarray(full_block, dtype=np.uint8)
    cb = full_block.size // Nc
    out = np.empty(Nant * nk * cb, dtype=np.uint8)
    if load_library().rawspec_gb300_shard_fill_block(full_block.ctypes.data, Nc, Nant, k0, nk, cb,
                                                      out.ctypes.data) != 0:
        raise ValueError("shard_fill_block: invalid arguments")
    return out


def shard_place_dump(shard_dump: np.ndarray, full_dump: np.ndarray, Nc: int, Nant: int, k0: int, nk: int, Nt: int,
                     ics: bool = False) -> None:
    """rawspec_gb300_shard_place_dump: writes one shard dump into full_dump
    (float32, the full observation's dump layout) in place."""
    sd = np.ascontiguousarray(shard_dump, dtype=np.float32)
    assert full_dump.dtype == np.float32 and full_dump.flags["C_CONTIGUOUS"]
    per_row = (1 if ics else Nant) * nk * Nt
    rows = sd.size // per_row
    Pf = C.POINTER(C.c_float)
    if load_library().rawspec_gb300_shard_place_dump(sd.ctypes.data_as(Pf), Nc, Nant, k0, nk, rows, Nt,
                                                      1 if ics else 0, full_dump.ctypes.data_as(Pf)) != 0:
        raise ValueError("shard_place_dump: invalid arguments")


class Spectrometer:
    """A librawspec context plus the host-side loop of a typical client.
    With shard=(rank, world) the context is that shard of the observation
    (rawspec_gb300_shard_context): Nant * nk of its Nc channels."""

    def __init__(self, Nc: int, Np: int, Ntpb: int, nbits: int, products: Sequence[tuple[int, int, int]], *,
                 Nant: int = 1, Nbc: int = 0, Nb: int = 0, conj: int = 0, gpu_index: int = 0,
                 weights: Sequence[float] | None = None, collect: bool = True,
                 shard: tuple[int, int] | None = None):
        self.lib = load_library()
        self.nbits_in = nbits
        self.ctx = make_context(Nc, Np, Ntpb, nbits, products, Nant=Nant, Nbc=Nbc, Nb=Nb, conj=conj,
                                gpu_index=gpu_index, weights=weights)
        self.full_Nc, self.k0, self.nk = Nc, 0, Nc // max(Nant, 1)
        if shard is not None:
            full = self.ctx
            self.ctx = RawspecContext()
            if self.lib.rawspec_gb300_shard_context(C.byref(full), shard[0], shard[1], C.byref(self.ctx)) != 0:
                raise ValueError(f"no shard {shard} of {Nc} channels in {Nant} antennas")
            self.ctx._weights_keepalive = getattr(full, "_weights_keepalive", None)  # type: ignore[attr-defined]
            self.k0, self.nk = shard_range(Nc, Nant, shard[0], shard[1])
        self.collect = collect
        self.dumps: list[list[np.ndarray]] = [[] for _ in products]
        self.ics: list[list[np.ndarray]] = [[] for _ in products]
        self.events: list[tuple[int, int]] = []
        # With collect=False no callback is installed (as a client without
        # writers would do); the library then queues no host functions.
        self._cb = DUMP_CALLBACK(self._on_dump)
        if collect:
            self.ctx.dump_callback = self._cb
        rc = self.lib.rawspec_initialize(C.byref(self.ctx))
        if rc != 0:
            raise RuntimeError(f"rawspec_initialize failed ({rc})")
        self._open = True

    # Called on a CUDA host-function thread.
    def _on_dump(self, pctx, product, kind):
        self.events.append((product, kind))
        if kind != RAWSPEC_CALLBACK_POST_DUMP or not self.collect:
            return
        ctx = pctx.contents
        n = ctx.h_pwrbuf_size[product] // 4
        self.dumps[product].append(np.ctypeslib.as_array(ctx.h_pwrbuf[product], shape=(n,)).copy())
        if ctx.incoherently_sum:
            self.ics[product].append(np.ctypeslib.as_array(ctx.h_icsbuf[product], shape=(n // ctx.Nant,)).copy())

    @property
    def Nb(self) -> int:
        return self.ctx.Nb

    @property
    def packed_block_bytes(self) -> int:
        c = self.ctx
        if self.nbits_in == 4:
            return c.Nc * c.Ntpb * c.Np
        return c.Nc * c.Ntpb * c.Np * 2 * (c.Nbps // 8)

    def host_block(self, i: int) -> np.ndarray:
        c = self.ctx
        nbytes = c.Nc * c.Ntpb * c.Np * 2 * (c.Nbps // 8)
        ptr = C.cast(c.h_blkbufs[i], C.POINTER(C.c_uint8))
        return np.ctypeslib.as_array(ptr, shape=(nbytes,))

    def load_blocks(self, blocks: np.ndarray) -> None:
        """Copies Nb host blocks (rows of `blocks`) into the library's host buffers."""
        nb = blocks.shape[0]
        for b in range(nb):
            self.host_block(b)[: blocks.shape[1]] = blocks[b]

    def copy_to_gpu(self, num_blocks: int | None = None) -> None:
        nb = self.Nb if num_blocks is None else num_blocks
        if self.nbits_in == 4:
            rc = self.lib.rawspec_copy_blocks_to_gpu_expanding_complex4(C.byref(self.ctx), 0, 0, nb)
        else:
            rc = self.lib.rawspec_copy_blocks_to_gpu(C.byref(self.ctx), 0, 0, nb)
        if rc != 0:
            raise RuntimeError("copy to GPU failed")

    def start(self, fft_dir: int = RAWSPEC_FORWARD_FFT) -> None:
        if self.lib.rawspec_start_processing(C.byref(self.ctx), fft_dir) != 0:
            raise RuntimeError("rawspec_start_processing failed")

    def wait(self) -> int:
        return self.lib.rawspec_wait_for_completion(C.byref(self.ctx))

    def copy_and_start(self, fft_dir: int = RAWSPEC_FORWARD_FFT) -> None:
        """rawspec_copy_blocks_to_gpu_and_start_processing, as the reference CLI calls it."""
        rc = self.lib.rawspec_copy_blocks_to_gpu_and_start_processing(C.byref(self.ctx), self.Nb,
                                                                        1 if self.nbits_in == 4 else 0, fft_dir)
        if rc != 0:
            raise RuntimeError("rawspec_copy_blocks_to_gpu_and_start_processing failed")

    def process(self, blocks: np.ndarray, fft_dir: int = RAWSPEC_FORWARD_FFT, combined: bool = False) -> None:
        """Feeds every complete buffer (Nb blocks) of `blocks` through the library
        (separate copy and start calls, or the combined call of the CLI)."""
        nb = self.Nb
        for b0 in range(0, blocks.shape[0] - nb + 1, nb):
            if self.wait() != 0:
                raise RuntimeError("wait_for_completion reported an error")
            self.load_blocks(blocks[b0:b0 + nb])
            if combined:
                self.copy_and_start(fft_dir)
            else:
                self.copy_to_gpu(nb)
                self.start(fft_dir)
        if self.wait() != 0:
            raise RuntimeError("wait_for_completion reported an error")

    def product_info(self, i: int) -> tuple[int, int, int]:
        a, b, c = C.c_uint(), C.c_uint(), C.c_uint()
        self.lib.rawspec_gb300_product_info(C.byref(self.ctx), i, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def set_profiling(self, on: bool) -> None:
        self.lib.rawspec_gb300_set_profiling(C.byref(self.ctx), 1 if on else 0)

    def profile(self, kclass: int) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_ulonglong()
        self.lib.rawspec_gb300_profile(C.byref(self.ctx), kclass, C.byref(ms), C.byref(n))
        return ms.value, n.value

    def reset_profile(self) -> None:
        self.lib.rawspec_gb300_reset_profile(C.byref(self.ctx))

    def product_kernel(self, i: int) -> str:
        """Name of the kernel class that computes product i ("small", "tc",
        "large_fused" or "large_a" for the two-kernel path)."""
        k = int(self.lib.rawspec_gb300_product_kernel(C.byref(self.ctx), i))
        if k < 0:
            raise ValueError(f"no product {i}")
        return KERNEL_CLASS_NAMES[k]

    def kernel_launches(self) -> int:
        return int(self.lib.rawspec_gb300_kernel_launches(C.byref(self.ctx)))

    def shared_launches(self) -> int:
        """Launches of this context that also carried other contexts' buffers."""
        return int(self.lib.rawspec_gb300_shared_launches(C.byref(self.ctx)))

    def stream(self) -> int:
        return int(self.lib.rawspec_gb300_stream(C.byref(self.ctx)) or 0)

    def close(self) -> None:
        if getattr(self, "_open", False):
            self.lib.rawspec_cleanup(C.byref(self.ctx))
            self._open = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
