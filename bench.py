"""Benchmark of the GB300 spectrometer on the production configuration.

Workload (one "step" = one GPU input buffer of Nb = 2 blocks):
  64 coarse channels, 2 polarisations, 8-bit complex Gaussian voltages
  (sigma 20, clipped), Ntpb = 524288 time samples per block (128 MiB blocks,
  256 MiB per buffer), three simultaneous products Nfft 2^20 / 8 / 1024 with
  Nint 51 / 128 / 3072, total power (the headline) and full pol (Npolout 4,
  reported alongside).

Metric: RAW-in GB/s (RAW bytes of the step / step time).
  value  device-resident throughput: the buffer is in HBM, the timed region
         is K x rawspec_start_processing (kernels + dumps to pinned host
         memory), timed with CUDA events on the library's stream;
  e2e    through the C-ABI from pinned host blocks, the reference CLI's
         per-buffer sequence: K x (rawspec_wait_for_completion +
         rawspec_copy_blocks_to_gpu_and_start_processing), then a final
         wait; wall clock; buffer_ms_p50 / buffer_ms_p99 are the
         percentiles of one loop iteration (the wait for the previous buffer
         and the copy and start of this one).

ingest  GUPPI RAW files of the same shape in /dev/shm streamed through
        rawspec_gb300_ingest_files into filterbank files (RAW file bytes over
        wall clock).

`--impl reference` times the CPU restatement of the same chain (the
reference has no CPU implementation of its spectrometer; the OpenMP FP32
port under oracle/ stands in) with all host threads, on the same metric.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NC, NP, NTPB, NBITS = 64, 2, 524288, 8
PRODUCTS = [(1 << 20, 51), (8, 128), (1024, 3072)]
SIGMA = 20.0
E2E_REPS = 7  # end-to-end runs; the median stands against two runs slowed by host jitter
BLOCK_BYTES = NC * NTPB * NP * 2
WORKLOAD = "production shape: 64 ch x 2 pol int8, Ntpb 524288 (128 MiB blocks), Nfft 2^20/8/1024, Nint 51/128/3072"
# The same config object on both arms (native and reference).
CONFIG = {"workload": WORKLOAD, "npolout": 1, "step": "one 2-block input buffer (256 MiB RAW)",
          "l2": "inputs larger than L2 (256 MiB per step)"}


def products(npol):
    return [(nt, na, npol) for nt, na in PRODUCTS]


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class RankGroup:
    """Host-side coordination of a multi-GPU run: one process per GPU, each
    with the context of its channel shard of the observation and its own data
    (the channels of different ranks are independent, so no data moves
    between ranks).  Only the barrier around the timed region and the max
    over ranks of the timings go through the process group (gloo, on the
    host)."""

    def __init__(self, world: int):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max_over_ranks(self, x: float) -> float:
        if self.dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def whole_job_gbs(world: int, step_bytes: int, steps: int, seconds_max: float) -> float:
    """Whole-job RAW-in GB/s: every rank processes steps x step_bytes; the
    job takes as long as its slowest rank."""
    return world * step_bytes * steps / seconds_max / 1e9


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(ctx, i: int, nt: int, na: int, npol: int) -> float:
    """RAW bytes of the buffer read once plus the product's integrated output
    bytes amortised per buffer: |P| * Nc * Nt * 4 * Nss / Na."""
    raw = 2 * BLOCK_BYTES
    nss = (2 * NTPB) // nt
    return raw + abs(npol) * NC * nt * 4 * nss / na


def load_traffic() -> dict:
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return {}
    return {}


_CPU_CASES: dict = {}


def cpu_sample_run(nthreads: int, nc_sample: int, reps: int = 1) -> tuple[float, float]:
    """Times the OpenMP FP32 CPU chain on nc_sample channels of one buffer of
    the workload, reps times; returns (GB/s of RAW input, seconds per rep)."""
    from oracle import oracle as O
    from rawspec_gb300 import synth
    if nc_sample not in _CPU_CASES:
        blocks = synth.gaussian_blocks(2, nc_sample, NTPB, NP, sigma=SIGMA, seed=1)
        _CPU_CASES[nc_sample] = (blocks, O.make_cfg(nc_sample, NP, NTPB, 2, NBITS, products(1)))
    blocks, cfg = _CPU_CASES[nc_sample]
    t0 = time.perf_counter()
    for _ in range(reps):
        O.run_cpu(cfg, blocks, nthreads=nthreads)
    dt = (time.perf_counter() - t0) / reps
    return blocks.nbytes / dt / 1e9, dt


def host_cpu_model() -> str:
    """The host CPU as /proc/cpuinfo names it (x86: model name; Arm: the
    implementer and part codes), else the machine type."""
    try:
        lines = Path("/proc/cpuinfo").read_text().splitlines()
    except OSError:
        return platform.machine()
    fields = {}
    for line in lines:
        if ":" in line:
            k, v = line.split(":", 1)
            fields.setdefault(k.strip(), v.strip())
    if fields.get("model name"):
        return fields["model name"]
    if fields.get("CPU implementer") and fields.get("CPU part"):
        return f"{platform.machine()}, CPU implementer {fields['CPU implementer']}, part {fields['CPU part']}"
    return platform.machine()


def pin_host_threads() -> None:
    """OpenMP threads bound close together, as the CPU baseline is specified;
    set before the oracle's OpenMP runtime is loaded (a caller's own
    setting is kept)."""
    os.environ.setdefault("OMP_PROC_BIND", "close")


def cpu_baseline_leg(min_seconds: float = 12.0, min_seconds_1: float = 3.0) -> dict:
    """The CPU chain on whole buffers of the workload (all 64 channels),
    repeated until at least min_seconds of CPU work have been timed, on all
    host threads; then on one thread over 4 channels of a buffer for at
    least min_seconds_1."""
    pin_host_threads()
    from oracle import oracle as O
    threads = O.lib().cpu_max_threads()
    cpu_sample_run(threads, NC)  # warm-up (page-in, thread pool)
    reps, secs = 0, 0.0
    while secs < min_seconds:
        _, dt = cpu_sample_run(threads, NC)
        secs += dt
        reps += 1
    v = reps * 2 * BLOCK_BYTES / secs / 1e9
    nc1 = 4
    cpu_sample_run(1, nc1)
    reps1, secs1 = 0, 0.0
    while secs1 < min_seconds_1:
        _, dt = cpu_sample_run(1, nc1)
        secs1 += dt
        reps1 += 1
    v1 = reps1 * 2 * BLOCK_BYTES * nc1 / NC / secs1 / 1e9
    return {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{reps} whole buffers (64 channels x 2 blocks, 256 MiB RAW each), all three products, "
                      f"total power, {secs:.1f} s",
            "one_thread": {"value": v1, "unit": "GB/s", "cores": 1,
                           "sample": f"{reps1} x {nc1} channels of a buffer, {secs1:.1f} s"},
            "cpu_model": host_cpu_model(), "omp_proc_bind": os.environ.get("OMP_PROC_BIND", "")}


def cufft_reference_leg(blocks, steps: int, warmup: int, ours_wall_ms: dict) -> dict:
    """The reference's own GPU library (rawspec_gpu.cu, cuFFT with its load
    and store callbacks, compiled unchanged for sm_103a) on the same GPU and
    workload, in a child process: per-buffer wall clock of
    rawspec_start_processing + rawspec_wait_for_completion with the buffer
    on the device, no dump callback.  ours_wall_ms: the native library's
    per-buffer time measured the same way in this process."""
    from oracle import ref_build, ref_gpu
    try:
        lib = ref_build.build_gpu()
    except RuntimeError as e:
        return {"unavailable": f"reference GPU build failed: {str(e).splitlines()[0]}"}
    if lib is None:
        return {"unavailable": "the reference's GPU sources are not present"}
    jobs = [(dict(Nc=NC, Np=NP, Ntpb=NTPB, nbits=8, products=[list(p) for p in products(npol)], fft_dir=1,
                  mode="time", steps=steps, warmup=warmup), blocks) for npol in (1, 4)]
    try:
        outs = ref_gpu.run_in_child(jobs)
    except RuntimeError as e:
        return {"unavailable": f"reference run failed: {str(e)[-300:]}"}
    res = {"unit": "GB/s", "timing": "wall clock per buffer of rawspec_start_processing + "
                                     "rawspec_wait_for_completion, input resident, no dump callback, median of "
                                     f"{steps} after {warmup} warm-up buffers; both libraries measured the same way",
           "cufft_version": str(outs[0]["cufft_version"]), "build": "rawspec_gpu.cu unchanged, nvcc -dc for "
           "sm_103a, static cuFFT (oracle/ref_build.py)"}
    for npol, out in zip((1, 4), outs):
        ms = 1e3 * float(statistics.median(out["seconds"]))
        key = "npolout1" if npol == 1 else "npolout4"
        res[key] = {"value": 2 * BLOCK_BYTES / (ms / 1e3) / 1e9, "ms_per_step": ms,
                    "ms_p99": 1e3 * float(sorted(out["seconds"])[max(0, int(0.99 * len(out["seconds"])) - 1)]),
                    "native_ms_per_step": ours_wall_ms[npol],
                    "native_speedup": ms / ours_wall_ms[npol]}
    res["value"] = res["npolout1"]["value"]
    return res


def c3_leg(steps: int, warmup: int, peak_gbs: float) -> dict:
    """The batched multi-antenna 4-bit configuration: 4 antennas x 16 coarse
    channels, 2 pols, 4-bit samples (uniform in [-8, 7] scaled by a gain per
    antenna), Ntpb 262144, products Nfft 4096 / Nint 64 and Nfft 64 / Nint
    1024 in full Stokes, weighted incoherent sum over the antennas.  One step
    = one block (32 MiB of packed RAW input, 64 MiB once expanded).
      value  RAW-in GB/s, expanded block resident: K x rawspec_start_processing,
             CUDA events on the library's stream;
      e2e    wall clock of K x (rawspec_wait_for_completion +
             rawspec_copy_blocks_to_gpu_and_start_processing with the 4-bit
             expansion) from pinned host blocks;
      roofline  the dominant kernel's bytes per launch (the expanded input
             it reads + its integrated output) over its CUDA-event time."""
    import torch

    from rawspec_gb300 import api, synth
    nant, nc, ntpb = 4, 64, 262144
    prods = [(4096, 64, -4), (64, 1024, -4)]
    blocks, _gains = synth.int4_blocks(1, nc, ntpb, 2, Nant=nant, seed=3)
    w = list(synth.weights(nant, seed=5))
    raw = nc * ntpb * 2  # packed bytes of one block
    with api.Spectrometer(nc, 2, ntpb, 4, prods, Nant=nant, weights=w, collect=False) as spec:
        lib, cp = spec.lib, C.byref(spec.ctx)
        stream = torch.cuda.ExternalStream(spec.stream())
        spec.load_blocks(blocks)
        spec.copy_to_gpu()
        for _ in range(warmup):
            spec.start()
        spec.wait()
        l0 = spec.kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            if lib.rawspec_start_processing(cp, 1) != 0:
                raise RuntimeError("start_processing failed")
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        launches = (spec.kernel_launches() - l0) / steps
        spec.wait()
        spec.reset_profile()
        spec.set_profiling(True)
        for _ in range(steps):
            spec.start()
        spec.wait()
        prof = {name: spec.profile(k) for k, name in enumerate(api.KERNEL_CLASS_NAMES)}
        spec.set_profiling(False)
        ts = time.perf_counter()
        for _ in range(steps):
            if lib.rawspec_wait_for_completion(cp) != 0 or \
                    lib.rawspec_copy_blocks_to_gpu_and_start_processing(cp, 1, 1, 1) != 0:
                raise RuntimeError("copy/start failed")
        if lib.rawspec_wait_for_completion(cp) != 0:
            raise RuntimeError("wait failed")
        e2e_s = (time.perf_counter() - ts) / steps
        kinds = [spec.product_kernel(i) for i in range(len(prods))]
    cls = max((k for k in prof if k not in ("d2h", "h2d")), key=lambda k: prof[k][0])
    t_ms, n = prof[cls]
    # bytes the dominant kernel must move per launch: the expanded input
    # (2 bytes per complex sample and polarisation) + the integrated output
    # of its product (4 planes x Nc x Nt floats per integration)
    expanded = nc * ntpb * 2 * 2
    out_bytes = {i: 4 * nc * nt * 4 * (ntpb // (nt * na)) for i, (nt, na, _p) in enumerate(prods)}
    prod_of = [i for i, k in enumerate(kinds) if k == cls]
    alg = expanded + (sum(out_bytes[i] for i in prod_of) / max(len(prod_of), 1))
    per_launch_ms = t_ms / n if n else None
    achieved = alg / (per_launch_ms / 1e3) / 1e9 if per_launch_ms else None
    return {"workload": "4 antennas x 16 ch, 4-bit, Ntpb 262144, Nfft 4096/64, Nint 64/1024, Stokes, weighted "
                        "incoherent sum; one block (32 MiB packed) per step",
            "value": raw / (ms / 1e3) / 1e9, "unit": "GB/s", "ms_per_step": ms, "steps": steps,
            "gpu_launches_per_step": launches,
            "e2e": {"value": raw / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": raw},
            "kernels": kinds,
            "kernel_ms_per_step": {k: v[0] / steps for k, v in prof.items() if v[1]},
            "roofline": {"bound": "hbm", "kernel": f"k_{cls}", "achieved": achieved, "peak": peak_gbs,
                         "unit": "GB/s", "frac": achieved / peak_gbs if achieved else None,
                         "bytes_per_launch": alg}}


def cpu_baseline_subprocess() -> dict:
    """cpu_baseline_leg in a child process of its own (no CUDA, no torch)."""
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--cpu-leg"], capture_output=True, text=True,
                         cwd=str(ROOT), timeout=900)
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    if res.returncode != 0 or not lines:
        raise RuntimeError(f"CPU baseline leg failed:\n{res.stdout[-2000:]}\n{res.stderr[-2000:]}")
    out = json.loads(lines[-1])
    out["process"] = "fresh child process, before any GPU work"
    return out


def ingest_leg(nbuf: int = 8) -> dict:
    """GUPPI RAW files -> librawspec -> SIGPROC filterbank files at the
    production shape: a two-file stem of 2 * nbuf blocks (128 MiB each) in
    /dev/shm (RAM-backed), streamed by rawspec_gb300_ingest_files with the
    filterbank writer as the dump callback; RAW file bytes over wall clock."""
    import ctypes as Cc
    import tempfile

    from rawspec_gb300 import api, io, synth
    base = Path("/dev/shm") if Path("/dev/shm").is_dir() else Path(tempfile.gettempdir())
    blocks = synth.gaussian_blocks(2, NC, NTPB, NP, sigma=SIGMA, seed=5)
    L = io.lib()
    with tempfile.TemporaryDirectory(dir=base) as d:
        paths = []
        per_file = nbuf  # blocks per file: 2 files of nbuf blocks = nbuf buffers
        for k in range(2):
            p = Path(d) / f"bench.{k:04d}.raw"
            io.write_raw_file(p, [blocks[i % 2] for i in range(per_file)],
                              [(k * per_file + i) * 32 for i in range(per_file)], NC, NP, NBITS, NTPB)
            paths.append(p)
        hdr = io.RawHeader()
        fd = os.open(paths[0], os.O_RDONLY)
        L.rawspec_gb300_raw_read_header(fd, Cc.byref(hdr))
        os.close(fd)
        ctx = api.RawspecContext()
        e4 = Cc.c_int(0)
        if L.rawspec_gb300_ingest_geometry(Cc.byref(hdr), 0, 0, Cc.byref(ctx), Cc.byref(e4)) != 0:
            raise RuntimeError("ingest geometry")
        ctx.No = len(PRODUCTS)
        for i, (nt, na) in enumerate(PRODUCTS):
            ctx.Nts[i], ctx.Nas[i], ctx.Npolout[i] = nt, na, 1
        if L.rawspec_initialize(Cc.byref(ctx)) != 0:
            raise RuntimeError("rawspec_initialize failed")
        writers = []
        try:
            for i in range(ctx.No):
                fh = io.FilHeader()
                L.rawspec_gb300_fil_header_for_product(Cc.byref(hdr), Cc.byref(ctx), i, 0, b"bench.0000.raw",
                                                       Cc.byref(fh))
                w = L.rawspec_gb300_fil_writer_open(Cc.byref(ctx), i, Cc.byref(fh), d.encode(), b"bench", i, 0, None)
                if not w:
                    raise RuntimeError("filterbank writer")
                writers.append(w)
            arr = (Cc.c_void_p * len(writers))(*writers)
            ctx.user_data = Cc.cast(arr, Cc.c_void_p)
            ctx.dump_callback = Cc.cast(L.rawspec_gb300_fil_dump_callback, api.DUMP_CALLBACK)
            plist = (Cc.c_char_p * 2)(*[str(p).encode() for p in paths])
            st = io.IngestStats()
            ing = L.rawspec_gb300_ingest_open(Cc.byref(ctx), 0)
            if not ing:
                raise RuntimeError("ingest open")
            L.rawspec_gb300_ingest_stem(ing, plist, 2, 0, Cc.byref(st))  # warm-up (page cache, GPU)
            t0 = time.perf_counter()
            rc = L.rawspec_gb300_ingest_stem(ing, plist, 2, 0, Cc.byref(st))
            dt = time.perf_counter() - t0
            L.rawspec_gb300_ingest_close(ing)
            if rc != 0 or st.stop != 0:
                raise RuntimeError("ingest failed")
        finally:
            for w in writers:
                L.rawspec_gb300_fil_writer_close(w)
            L.rawspec_cleanup(Cc.byref(ctx))
        file_bytes = sum(p.stat().st_size for p in paths)
    return {"value": file_bytes / dt / 1e9, "unit": "GB/s", "files": 2, "file_bytes": file_bytes,
            "blocks": int(st.blocks_read), "buffers": int(st.buffers), "storage": str(base),
            "timing": "wall clock of rawspec_gb300_ingest_stem over the stem (warm page cache), filterbank "
                      "files written by the dump callback"}


def serving_leg(njobs: int = 256, rate: float = 40.0, budget: float = 120e9) -> dict:
    """The serving mix (rawspec_gb300.mix: jobs of 2-16 blocks, Nchan 8/32/64,
    4/8-bit, 1-3 products of Nfft 8 ... 2^20) through the job server under a
    120 GB device-memory budget: once with the Poisson arrivals (mean 40 jobs
    per second) and once with every job submitted at the start (capacity);
    beside them a serial plain-path replay of the same jobs (a context per job,
    one after another).  RAW bytes over wall clock; latencies from the push of
    a buffer (its data in pinned memory) to its processing complete, and to the
    POST_DUMP of the dumps it ends."""
    import numpy as np

    from rawspec_gb300 import api, mix, serve
    jobs = mix.serving_jobs(njobs, rate)
    bufs = [mix.block_bytes(j) * j["Nb"] for j in jobs]
    pool = np.random.default_rng(9).integers(-128, 128, size=max(bufs), dtype=np.int16).astype(np.uint8)
    total = sum(mix.block_bytes(j) * j["blocks"] for j in jobs)

    def served(on_schedule: bool) -> dict:
        srv = serve.Server(int(budget), max_active=16, max_queued=2, collect=False)
        try:
            def feed(k, jid):
                for _ in range(jobs[k]["blocks"] // jobs[k]["Nb"]):
                    srv.push(jid, pool[:bufs[k]])
                srv.close_job(jid)
            threads = []
            t0 = time.perf_counter()
            for k, j in enumerate(jobs):
                if on_schedule:
                    dt = t0 + j["arrival"] - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                jid = srv.submit(j["Nc"], 2, j["ntpb"], j["nbits"], j["products"], Nb=j["Nb"])
                th = threading.Thread(target=feed, args=(k, jid))
                th.start()
                threads.append((jid, th))
            for jid, th in threads:
                th.join()
            states = [srv.wait_job(jid, 600.0) for jid, _ in threads]
            secs = time.perf_counter() - t0
            st = srv.stats()
        finally:
            srv.close()
        if any(x != serve.JOB_DONE for x in states):
            raise RuntimeError("serving mix: a job failed")
        return {"value": total / secs / 1e9, "unit": "GB/s", "seconds": secs, "jobs_per_s": njobs / secs,
                "buffers": int(st.buffers), "dumps": int(st.dumps), "peak_active_jobs": int(st.peak_active),
                "peak_device_bytes": int(st.peak_used),
                "buffer_ms_p50": st.buffer_p50_ms, "buffer_ms_p99": st.buffer_p99_ms,
                "dump_ms_p50": st.dump_p50_ms, "dump_ms_p99": st.dump_p99_ms,
                "group_calls": int(st.group_calls)}

    arrivals = served(True)
    burst = served(False)
    # serial plain path: one context per job, the CLI's per-buffer calls
    lat = []
    t0 = time.perf_counter()
    for k, j in enumerate(jobs):
        spec = api.Spectrometer(j["Nc"], 2, j["ntpb"], j["nbits"], j["products"], Nb=j["Nb"], collect=False)
        try:
            blocks = pool[:bufs[k]].reshape(j["Nb"], -1)
            for _ in range(j["blocks"] // j["Nb"]):
                spec.load_blocks(blocks)
                ts = time.perf_counter()
                spec.copy_and_start()
                if spec.wait() != 0:
                    raise RuntimeError("serial replay failed")
                lat.append(1e3 * (time.perf_counter() - ts))
        finally:
            spec.close()
    serial_s = time.perf_counter() - t0
    return {"workload": f"{njobs} jobs, Poisson arrivals at {rate:g} jobs/s, 2-16 blocks of Ntpb 262144, "
                        "Nchan 8/32/64, 4/8-bit, 1-3 products of Nfft 8/1024/65536/1048576, Nint 16-3072, "
                        f"Npolout 1/4/-4; {budget / 1e9:g} GB device-memory budget",
            "raw_bytes": total, "arrivals": arrivals, "all_at_start": burst,
            "serial_plain": {"value": total / serial_s / 1e9, "unit": "GB/s", "seconds": serial_s,
                             "buffer_ms_p50": float(np.percentile(lat, 50)),
                             "buffer_ms_p99": float(np.percentile(lat, 99))},
            "speedup_vs_serial": serial_s / burst["seconds"]}


def run_reference(args, rank, world):
    """CPU restatement of the chain (kind "port") with all host threads."""
    if rank != 0:
        return 0
    pin_host_threads()
    from oracle import oracle as O
    threads = O.lib().cpu_max_threads()
    # one step = one whole buffer (64 channels x 2 blocks, about 0.5 s on 16
    # host cores), so the default --steps/--warmup run takes well under a minute
    nc_sample = NC
    for _ in range(args.warmup):
        cpu_sample_run(threads, nc_sample)
    vals, secs = [], 0.0
    for _ in range(args.steps):
        v, dt = cpu_sample_run(threads, nc_sample)
        vals.append(v)
        secs += dt
    value = statistics.median(vals)
    sample = "one whole buffer per step (64 channels x 2 blocks, 256 MiB RAW), all three products, total power"
    line = {
        "metric": "RAW-in GB/s", "value": value, "unit": "GB/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded complex Gaussian int8)",
        "config": dict(CONFIG), "parallelism": "host threads",
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port", "sample": sample,
                         "cpu_model": host_cpu_model(), "omp_proc_bind": os.environ.get("OMP_PROC_BIND", "")},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_native(args, rank, world, local_rank):
    import numpy as np
    import torch

    from rawspec_gb300 import api, synth

    # the CPU baseline first, on an otherwise idle host, in a fresh process
    # (after the GPU legs it measured up to 40 % lower in the same process)
    cpu = cpu_baseline_subprocess() if rank == 0 and world == 1 and not args.no_cpu else None

    torch.cuda.set_device(local_rank)
    group = RankGroup(world)
    barrier, max_over_ranks = group.barrier, group.max_over_ranks

    blocks = synth.gaussian_blocks(2, NC, NTPB, NP, sigma=SIGMA, seed=1 + rank)
    results = {}
    for npol in (1, 4):
        # one observation of 64 x N channels, sharded by channel: this rank's
        # context holds its 64 (rawspec_gb300_shard_context)
        spec = api.Spectrometer(NC * world, NP, NTPB, NBITS, products(npol), gpu_index=local_rank, collect=False,
                                shard=(rank, world))
        assert spec.ctx.Nc == NC
        lib = spec.lib
        cp = C.byref(spec.ctx)
        stream = torch.cuda.ExternalStream(spec.stream(), device=local_rank)
        spec.load_blocks(blocks)
        spec.copy_to_gpu()
        # device-resident timed region
        for _ in range(args.warmup):
            spec.start()
        spec.wait()
        l0 = spec.kernel_launches()
        sampler = ClockSampler(local_rank)
        sampler.start()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            if lib.rawspec_start_processing(cp, 1) != 0:
                raise RuntimeError("start_processing failed")
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier()
        launches = spec.kernel_launches() - l0
        ms = max_over_ranks(e0.elapsed_time(e1))
        spec.wait()
        # per-kernel device times: a separate pass in which the library runs
        # the products one after another, so each kernel's events time it alone
        spec.reset_profile()
        spec.set_profiling(True)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(args.steps):
            if lib.rawspec_start_processing(cp, 1) != 0:
                raise RuntimeError("start_processing failed")
        p1.record(stream)
        p1.synchronize()
        ms_serial = p0.elapsed_time(p1)
        prof = {}
        for k, name in enumerate(api.KERNEL_CLASS_NAMES):
            t, n = spec.profile(k)
            prof[name] = (t, n)
        spec.set_profiling(False)
        # per-buffer wall clock of start_processing + wait_for_completion, the
        # way the reference build is timed (cufft_reference)
        wall = []
        for _ in range(args.steps):
            ts = time.perf_counter()
            if lib.rawspec_start_processing(cp, 1) != 0 or lib.rawspec_wait_for_completion(cp) != 0:
                raise RuntimeError("start/wait failed")
            wall.append(1e3 * (time.perf_counter() - ts))
        # end-to-end through the C-ABI from pinned host blocks: K steps of the
        # reference CLI's per-buffer sequence (rawspec.c:1012-1014), timed
        # E2E_REPS times (host jitter moves single runs); the median is reported,
        # every sample is kept
        nbuf = args.warmup + 3 * args.steps  # buffers processed so far
        for _ in range(args.warmup):
            spec.copy_and_start()
            spec.wait()
            nbuf += 1
        sizes = [spec.ctx.h_pwrbuf_size[i] for i in range(3)]
        nis = [spec.product_info(i)[1] for i in range(3)]
        reps, d2h, step_ms = [], 0, []
        for _ in range(E2E_REPS):
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                ts = time.perf_counter()
                if lib.rawspec_wait_for_completion(cp) != 0:
                    raise RuntimeError("wait failed")
                if lib.rawspec_copy_blocks_to_gpu_and_start_processing(cp, 2, 0, 1) != 0:
                    raise RuntimeError("copy/start failed")
                step_ms.append(1e3 * (time.perf_counter() - ts))
            if lib.rawspec_wait_for_completion(cp) != 0:
                raise RuntimeError("wait failed")
            reps.append(max_over_ranks(time.perf_counter() - t0))
            # device->host dump bytes of these buffers (a product dumps after
            # every Nis-th buffer)
            for b in range(nbuf + 1, nbuf + args.steps + 1):
                d2h += sum(sizes[i] for i in range(3) if b % nis[i] == 0)
            nbuf += args.steps
        e2e_s = statistics.median(reps)
        d2h /= E2E_REPS
        # clock samples from the start of the device-resident timed region to
        # the end of the end-to-end runs (the first region alone is shorter
        # than the sampling period)
        clocks = sampler.stop()
        clocks["window"] = "device-resident and end-to-end timed legs, with the profiling pass between them"
        results[npol] = dict(ms=ms, ms_serial=ms_serial, prof=prof, launches=launches, clocks=clocks, e2e_s=e2e_s,
                             e2e_samples=[whole_job_gbs(world, 2 * BLOCK_BYTES, args.steps, x) for x in reps],
                             step_p50=float(np.percentile(step_ms, 50)), step_p99=float(np.percentile(step_ms, 99)),
                             d2h=d2h / args.steps, device_bytes=int(lib.rawspec_gb300_device_bytes(cp)),
                             wall_ms=float(statistics.median(wall)))
        spec.close()

    r = results[1]
    step_bytes = 2 * BLOCK_BYTES
    value = whole_job_gbs(world, step_bytes, args.steps, r["ms"] / 1e3)
    e2e = whole_job_gbs(world, step_bytes, args.steps, r["e2e_s"])
    # dominant kernel class of the headline run
    prof = r["prof"]
    kernel_classes = ["small", "finalize", "large_a", "large_b", "ics", "expand4", "large_fused", "tc"]
    t_large = prof["large_a"][0] + prof["large_b"][0]
    dom = max(kernel_classes, key=lambda k: t_large if k in ("large_a", "large_b") else prof[k][0])
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    tr = load_traffic()
    # algorithmic bytes per launch of the dominant class: RAW bytes of the
    # buffer + the product's integrated output bytes
    if dom in ("large_a", "large_b"):
        alg = algorithmic_bytes(None, 0, PRODUCTS[0][0], PRODUCTS[0][1], 1)
        dom_name = "k_large_a + k_large_b (Nfft 2^20)"
        t_ms, n = t_large, prof["large_a"][1]
        traffic = tr.get("k_large_a+k_large_b")
    elif dom == "large_fused":
        alg = algorithmic_bytes(None, 0, PRODUCTS[0][0], PRODUCTS[0][1], 1)
        dom_name = "k_large_fused (Nfft 2^20)"
        t_ms, n = prof[dom]
        traffic = tr.get("k_large_fused")
    else:
        idx = [1, 2]
        alg = sum(algorithmic_bytes(None, i, PRODUCTS[i][0], PRODUCTS[i][1], 1) for i in idx) / len(idx)
        dom_name = f"k_{dom}"
        t_ms, n = prof[dom]
        traffic = tr.get(dom_name)
    achieved = alg / (t_ms / max(n, 1) / 1e3) / 1e9 if n else None
    # FP32 view of the same kernel: 5 N log2 N flops per complex transform
    # plus 4 per detected sample (total power), against the nominal non-tensor
    # FP32 rate of 152 SMs x 128 lanes x 2 flops x 2.07 GHz
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    if dom in ("large_a", "large_b", "large_fused"):
        nt_dom = [PRODUCTS[0][0]]
    else:
        nt_dom = [PRODUCTS[1][0], PRODUCTS[2][0]]
    samples = NC * NP * 2 * NTPB  # complex samples of one buffer, both polarisations
    flops = sum(samples * (5 * math.log2(nt) + 4) for nt in nt_dom) / len(nt_dom)
    fp32_tflops = flops / (t_ms / max(n, 1) / 1e3) / 1e12 if n else None
    line = {
        "metric": "RAW-in GB/s", "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded complex Gaussian int8, sigma 20)",
        "config": dict(CONFIG),
        "parallelism": (f"channel shards x{world}: one observation of {NC * world} channels, {NC} per GPU, "
                        "no data exchanged") if world > 1 else "single GPU",
        "e2e": {"value": e2e, "unit": "GB/s", "h2d_bytes_per_step": step_bytes,
                "d2h_bytes_per_step": int(r["d2h"]), "samples": r["e2e_samples"],
                "buffer_ms_p50": r["step_p50"], "buffer_ms_p99": r["step_p99"],
                "timing": f"wall clock of K steps, median of {E2E_REPS} runs"},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "peak_source": peak_src,
                     "fp32": {"achieved_tflops": fp32_tflops, "peak_tflops": fp32_peak, "peak_source": "nominal",
                              "frac": (fp32_tflops / fp32_peak) if fp32_tflops else None},
                     "kernel_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
                     "kernel_timing": "CUDA events around each launch in a separate pass with the products "
                                      "serialised on one stream",
                     "serialised_ms_per_step": r["ms_serial"] / args.steps},
        "npolout4": {"value": whole_job_gbs(world, step_bytes, args.steps, results[4]["ms"] / 1e3),
                     "e2e": whole_job_gbs(world, step_bytes, args.steps, results[4]["e2e_s"]),
                     "ms_per_step": results[4]["ms"] / args.steps},
        "device_bytes": r["device_bytes"],
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu
    if rank == 0 and world == 1 and not args.no_cufft:
        line["cufft_reference"] = cufft_reference_leg(blocks, args.steps, args.warmup,
                                                      {p: results[p]["wall_ms"] for p in (1, 4)})
    if rank == 0 and world == 1 and not args.no_c3:
        line["c3"] = c3_leg(args.steps, args.warmup, peak)
    if rank == 0 and world == 1 and not args.no_ingest:
        line["ingest"] = ingest_leg()
    if rank == 0 and world == 1 and not args.no_serve:
        line["serving"] = serving_leg()
    if rank == 0:
        print(json.dumps(line), flush=True)
    group.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=24)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-ingest", action="store_true", help="skip the RAW-file ingest leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-mix leg")
    ap.add_argument("--no-cufft", action="store_true", help="skip the reference cuFFT-build leg")
    ap.add_argument("--no-c3", action="store_true", help="skip the multi-antenna 4-bit leg")
    ap.add_argument("--cpu-leg", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.cpu_leg:
        print(json.dumps(cpu_baseline_leg()), flush=True)
        return 0
    rank, world, local_rank = rank_info()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    import __graft_entry__
    __graft_entry__.build()
    return run_native(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
