"""Driver of the reference's own GPU library, oracle/_ref/libreference_rawspec.so
(rawspec_gpu.cu compiled unchanged: cuFFT plans with load/store callbacks).
TEST INFRASTRUCTURE ONLY: tests/ use it to compare the native library with
the reference's cuFFT-callback output, and bench.py to time the reference
build on the same GPU.  Nothing in the product loads it.

The reference library is run in a child process of its own
(`python -m oracle.ref_gpu REQUEST RESULT`): it exports the same twelve
entry points as librawspec.so, keeps its texture object in a global device
symbol (one context per process) and links its own copy of cuFFT and of the
CUDA runtime.  The context structure is the reference's rawspec_context
(rawspec.h:32-148), which rawspec_gb300.api mirrors field for field.

Only configurations free of the reference's known out-of-range accesses are
run (rawspec_gpu.cu): an incoherent sum is run with channel batches of one
antenna (Nbc = Nc/Nant; with Nbc = Nc the kernel at :321-340 indexes
channels past Nc), and full-pol or Stokes products whose integration spans
buffers are not run with channel batching (the cache offsets of :1580 and
:1737 overrun the cache for |Npolout| = 4).  `check_request` rejects the
others before the library is loaded.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402

ENTRY_POINTS = [
    "get_librawspec_version", "get_cufft_version", "rawspec_initialize", "rawspec_cleanup",
    "rawspec_copy_blocks_to_gpu", "rawspec_copy_blocks_to_gpu_expanding_complex4", "rawspec_zero_blocks_to_gpu",
    "rawspec_start_processing", "rawspec_copy_blocks_to_gpu_and_start_processing", "rawspec_reset_integration",
    "rawspec_check_for_completion", "rawspec_wait_for_completion",
]


def check_request(req: dict) -> None:
    """Refuses configurations that make the reference read or write out of
    range (module docstring)."""
    Nc, Nant = req["Nc"], req.get("Nant", 1)
    nbc = req.get("Nbc", 0) or Nc
    if req.get("weights") is not None and Nant > 1 and nbc != Nc // Nant:
        raise ValueError("reference incoherent sum needs Nbc = Nc / Nant")
    if nbc < Nc:
        Tbuf = req["Ntpb"] * _nb(req)
        for nt, na, npol in req["products"]:
            if abs(npol) == 4 and nt * na > Tbuf:
                raise ValueError("reference channel batching with |Npolout| 4 across buffers overruns its cache")


def _nb(req: dict) -> int:
    ntmax = max(p[0] for p in req["products"])
    return 1 if ntmax < req["Ntpb"] else ntmax // req["Ntpb"]


def load(path: str | Path | None = None) -> C.CDLL:
    """Loads the reference library and declares its twelve entry points
    (rawspec.h:161-234)."""
    from rawspec_gb300.api import RawspecContext
    p = Path(path) if path else ref_build.GPU_LIB
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
    }
    for name in ENTRY_POINTS:
        res, args = sig[name]
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


class RefSpectrometer:
    """A reference context with the client loop of the reference CLI
    (rawspec.c:906-1032): wait, fill the host blocks, copy, start."""

    def __init__(self, lib: C.CDLL, req: dict, collect: bool = True):
        from rawspec_gb300.api import DUMP_CALLBACK, make_context
        self.lib = lib
        self.nbits_in = req["nbits"]
        self.ctx = make_context(req["Nc"], req["Np"], req["Ntpb"], req["nbits"], [tuple(p) for p in req["products"]],
                                Nant=req.get("Nant", 1), Nbc=req.get("Nbc", 0), conj=req.get("conj", 0),
                                weights=req.get("weights"))
        self.dumps = [[] for _ in req["products"]]
        self.ics = [[] for _ in req["products"]]
        self._cb = DUMP_CALLBACK(self._on_dump)
        if collect:
            self.ctx.dump_callback = self._cb
        rc = lib.rawspec_initialize(C.byref(self.ctx))
        if rc != 0:
            raise RuntimeError(f"reference rawspec_initialize failed ({rc})")
        self._open = True

    def _on_dump(self, pctx, product, kind):
        if kind != 1:
            return
        ctx = pctx.contents
        n = ctx.h_pwrbuf_size[product] // 4
        self.dumps[product].append(np.ctypeslib.as_array(ctx.h_pwrbuf[product], shape=(n,)).copy())
        if ctx.incoherently_sum:
            self.ics[product].append(np.ctypeslib.as_array(ctx.h_icsbuf[product], shape=(n // ctx.Nant,)).copy())

    def host_block(self, i: int) -> np.ndarray:
        c = self.ctx
        nbytes = c.Nc * c.Ntpb * c.Np * (1 if self.nbits_in == 4 else 2 * (c.Nbps // 8))
        return np.ctypeslib.as_array(C.cast(c.h_blkbufs[i], C.POINTER(C.c_uint8)), shape=(nbytes,))

    def feed(self, buffer_blocks: np.ndarray, fft_dir: int) -> None:
        """One input buffer (Nb host blocks) through the reference."""
        if self.lib.rawspec_wait_for_completion(C.byref(self.ctx)) != 0:
            raise RuntimeError("reference wait_for_completion failed")
        for b in range(buffer_blocks.shape[0]):
            self.host_block(b)[:] = buffer_blocks[b]
        if self.nbits_in == 4:
            rc = self.lib.rawspec_copy_blocks_to_gpu_expanding_complex4(C.byref(self.ctx), 0, 0, self.ctx.Nb)
        else:
            rc = self.lib.rawspec_copy_blocks_to_gpu(C.byref(self.ctx), 0, 0, self.ctx.Nb)
        if rc != 0 or self.lib.rawspec_start_processing(C.byref(self.ctx), fft_dir) != 0:
            raise RuntimeError("reference copy/start failed")

    def finish(self) -> None:
        if self.lib.rawspec_wait_for_completion(C.byref(self.ctx)) != 0:
            raise RuntimeError("reference wait_for_completion failed")

    def close(self) -> None:
        if self._open:
            # rawspec_cleanup hands ctx->Aws to cudaFreeHost (rawspec_gpu.cu:1379-1382);
            # the weights here are ordinary host memory owned by Python
            self.ctx.Aws = None
            self.lib.rawspec_cleanup(C.byref(self.ctx))
            self._open = False


def _buffers(req: dict, blocks: np.ndarray | None):
    """Yields the input buffers (Nb host blocks each) of a request: from the
    given blocks, or generated per buffer on the GPU (synth.gaussian_buffer_cuda)."""
    nb = _nb(req)
    if blocks is not None:
        for b0 in range(0, blocks.shape[0] - nb + 1, nb):
            yield blocks[b0:b0 + nb]
        return
    from rawspec_gb300 import synth
    g = req["generate"]
    for k in range(g["nbuf"]):
        yield synth.gaussian_buffer_cuda(k, nb, req["Nc"], req["Ntpb"], req["Np"], sigma=g["sigma"], seed=g["seed"])


def run_dumps(req: dict, blocks: np.ndarray | None) -> dict:
    """Feeds every buffer of the request through a reference context and
    returns its dumps (out<i>, ics<i>: [ndumps, values]).  req["keep"] may
    name, per product index, the dump indices to keep (all by default)."""
    lib = load(req.get("lib"))
    spec = RefSpectrometer(lib, req)
    try:
        for buf in _buffers(req, blocks):
            spec.feed(buf, req.get("fft_dir", 1))
        spec.finish()
        out = {"cufft_version": np.array(lib.get_cufft_version().decode())}
        keep = {int(k): v for k, v in req.get("keep", {}).items()}
        for i in range(len(req["products"])):
            sel = keep.get(i)
            for name, lst in (("out", spec.dumps[i]), ("ics", spec.ics[i])):
                if lst:
                    arr = [lst[j] for j in sel] if sel is not None else lst
                    out[f"{name}{i}"] = np.array(arr)
            out[f"ndumps{i}"] = np.array(len(spec.dumps[i]))
        return out
    finally:
        spec.close()


def run_timing(req: dict, blocks: np.ndarray | None) -> dict:
    """Per-buffer wall-clock time of rawspec_start_processing +
    rawspec_wait_for_completion with the buffer already on the device (the
    input is copied once), after `warmup` buffers; no dump callback."""
    lib = load(req.get("lib"))
    spec = RefSpectrometer(lib, req, collect=False)
    try:
        buf = next(iter(_buffers(req, blocks)))
        spec.feed(buf, req.get("fft_dir", 1))
        spec.finish()
        P = C.byref(spec.ctx)
        times = []
        for k in range(req["warmup"] + req["steps"]):
            t0 = time.perf_counter()
            if lib.rawspec_start_processing(P, req.get("fft_dir", 1)) != 0:
                raise RuntimeError("reference start_processing failed")
            if lib.rawspec_wait_for_completion(P) != 0:
                raise RuntimeError("reference wait_for_completion failed")
            if k >= req["warmup"]:
                times.append(time.perf_counter() - t0)
        return {"seconds": np.array(times), "cufft_version": np.array(lib.get_cufft_version().decode())}
    finally:
        spec.close()


def _tmpdir() -> str | None:
    """Large results go through shared memory where the machine has it."""
    return "/dev/shm" if os.path.isdir("/dev/shm") and os.access("/dev/shm", os.W_OK) else None


def run_in_child(jobs: list[tuple[dict, np.ndarray | None]], timeout: float = 1200) -> list[dict]:
    """Runs requests (dumps or timing) one after another in one child process;
    returns one dict of result arrays per request, plus the child's output
    under "stdout" / "stderr" of the first.  Raises RuntimeError with the
    child's output if it fails."""
    for req, _ in jobs:
        check_request(req)
    with tempfile.TemporaryDirectory(prefix="rawspec_ref_", dir=_tmpdir()) as td:
        rq = Path(td) / "req.npz"
        arrays = {"n": np.array(len(jobs))}
        for k, (req, blocks) in enumerate(jobs):
            arrays[f"req{k}"] = np.array(json.dumps(req))
            if blocks is not None:
                arrays[f"blocks{k}"] = np.ascontiguousarray(blocks)
        np.savez(rq, **arrays)
        env = dict(os.environ)
        env["PYTHONPATH"] = str(ROOT) + os.pathsep + env.get("PYTHONPATH", "")
        res = subprocess.run([sys.executable, "-m", "oracle.ref_gpu", str(rq), td], cwd=str(ROOT), env=env,
                             capture_output=True, text=True, timeout=timeout)
        outs = []
        for k in range(len(jobs)):
            rs = Path(td) / f"res{k}.npz"
            if res.returncode != 0 or not rs.exists():
                raise RuntimeError(f"reference child failed (rc {res.returncode}):\n{res.stdout[-4000:]}\n"
                                   f"{res.stderr[-4000:]}")
            with np.load(rs) as z:
                outs.append({key: z[key] for key in z.files})
        outs[0]["stdout"] = res.stdout
        outs[0]["stderr"] = res.stderr
        return outs


def main(argv: list[str]) -> int:
    with np.load(argv[0]) as z:
        n = int(z["n"])
        jobs = [(json.loads(str(z[f"req{k}"])), z[f"blocks{k}"] if f"blocks{k}" in z.files else None)
                for k in range(n)]
    for k, (req, blocks) in enumerate(jobs):
        check_request(req)
        out = run_timing(req, blocks) if req.get("mode") == "time" else run_dumps(req, blocks)
        np.savez(Path(argv[1]) / f"res{k}.npz", **out)
        sys.stdout.flush()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
