"""Autotuner of the kernel choices per (FFT length, sample bits, Npolout).

usage: python -m rawspec_gb300.tune --nc 64 --ntpb 524288 --nt 1048576 --na 51 --nt 8 --na 128 --nt 1024 --na 3072
       [--np 2] [--nbits 8] [--npol 1] [--steps 20] [--reps 3] [--rounds 2] [--passes 1] [--min-gain 0.02]
       [--out tuning.txt]

Times whole buffers of the given configuration -- all its products at once,
on their concurrent streams, input resident on the device -- with one
candidate setting at a time, and keeps per product the fastest (coordinate
descent over the products, the others at their current best).  Timing the
whole buffer rather than one kernel alone lets the choice see how the
products share the GPU.  The current setting is measured again beside its
candidates, in interleaved rounds, each setting keeps its fastest time, and
a candidate replaces the current setting only if it is faster by more than
--min-gain (2 %; repeated timings of one setting on a GB300 spread by about
that much).  The candidates depend on the kernel the library
picked for the product:

- N <= 4096: the CUDA-core kernel k_small with 1, 2, 4, 8 or 16 CTAs per SM
  as the target of its chunking, and the tensor-core DFT k_tc where the
  library supports it for the product;
- the persistent four-step kernel k_large_fused: lag 2 .. 6 with a ring of
  twice the lag;
- the two-kernel four-step path k_large_a/b: 1 .. 16 CTAs per SM.

The result is a tuning table (format in rawspec_gb300/csrc/tune.c) holding
the entries that beat the library's own choice; RAWSPEC_GB300_TUNE_FILE names
it for rawspec_initialize.  Entries are keyed by (Nfft, bits, Npolout), so
products that share a key share the entry.
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile
import time
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

from rawspec_gb300 import api, synth  # noqa: E402

ENV = "RAWSPEC_GB300_TUNE_FILE"
CTAS = (1, 2, 4, 8, 16)
LAGS = (2, 3, 4, 5, 6)


def entry_line(key: tuple[int, int, int], setting: dict) -> str:
    return " ".join(str(k) for k in key) + "".join(f" {k}={v}" for k, v in setting.items())


def write_table(path: str, entries: dict, comments: list[str] = ()) -> None:
    with open(path, "w") as f:
        for c in comments:
            f.write(f"# {c}\n")
        for key, setting in entries.items():
            if setting:
                f.write(entry_line(key, setting) + "\n")


class Case:
    """One configuration: its products and a seeded Gaussian input buffer."""

    def __init__(self, a):
        self.a = a
        self.prods = [(nt, na, a.npol) for nt, na in zip(a.nt, a.na)]
        spec = api.Spectrometer(a.nc, a.np, a.ntpb, a.nbits, self.prods, collect=False)
        try:
            self.nb = spec.Nb
            self.keys = [(int(spec.ctx.Nts[i]), 16 if a.nbits == 16 else 8, int(spec.ctx.Npolout[i]))
                         for i in range(len(self.prods))]
        finally:
            spec.close()
        self.blocks = synth.gaussian_blocks(self.nb, a.nc, a.ntpb, a.np, sigma=20.0, seed=1, nbits=a.nbits)

    def run(self, table: dict, path: str) -> tuple[float, list[str]]:
        """Fastest ms per buffer over the repetitions, and the kernel class of
        each product, with `table` as the tuning table."""
        write_table(path, table)
        os.environ[ENV] = path
        a = self.a
        spec = api.Spectrometer(a.nc, a.np, a.ntpb, a.nbits, self.prods, collect=False)
        try:
            kinds = [spec.product_kernel(i) for i in range(len(self.prods))]
            spec.load_blocks(self.blocks)
            spec.copy_to_gpu()
            for _ in range(3):
                spec.start()
            if spec.wait() != 0:
                raise RuntimeError("processing failed")
            reps = []
            for _ in range(a.reps):
                t0 = time.perf_counter()
                for _ in range(a.steps):
                    spec.start()
                if spec.wait() != 0:
                    raise RuntimeError("processing failed")
                reps.append(1e3 * (time.perf_counter() - t0) / a.steps)
            return min(reps), kinds
        finally:
            spec.close()


def candidates(kind: str) -> list[dict]:
    if kind in ("small", "tc"):
        return [{"dft": "cuda", "ctas": c} for c in CTAS] + [{"dft": "tc"}]
    if kind == "large_fused":
        return [{"lag": g, "ring": 2 * g} for g in LAGS]
    return [{"ctas": c} for c in CTAS]


def tune(a, log=print, case=None) -> tuple[dict, list[str]]:
    """Coordinate descent over the products of `a`; returns the table of
    settings that beat the library's choices and the timing notes.  `case`
    replaces the GPU measurement (anything with prods, keys and run())."""
    case = case if case is not None else Case(a)
    tmp = tempfile.NamedTemporaryFile("w", suffix=".tune", delete=False)
    tmp.close()
    saved = os.environ.get(ENV)
    notes = []
    try:
        table: dict = {}
        base_ms, kinds = case.run(table, tmp.name)
        notes.append(f"library defaults: {base_ms:.3f} ms per buffer, kernels {kinds}")
        log(notes[-1])
        for _ in range(a.passes):
            for i, (nt, na, npol) in enumerate(case.prods):
                key = case.keys[i]
                current = dict(table.get(key, {}))
                settings = [current] + [c for c in candidates(kinds[i]) if c != current]
                best = [float("inf")] * len(settings)
                for _ in range(a.rounds):
                    for j, cand in enumerate(settings):
                        if best[j] is None:
                            continue
                        trial = dict(table)
                        trial[key] = cand
                        ms, k2 = case.run(trial, tmp.name)
                        if cand.get("dft") == "tc" and k2[i] != "tc":
                            log(f"product {i} (Nfft {nt}): no tensor-core DFT for this product, skipped")
                            best[j] = None
                            continue
                        best[j] = min(best[j], ms)
                for j, cand in enumerate(settings):
                    if best[j] is None:
                        continue
                    line = entry_line(key, cand) + ("" if j else " (current)")
                    log(f"product {i} (Nfft {nt}, Na {na}): {line}: {best[j]:.3f} ms")
                    notes.append(f"{line}: {best[j]:.3f} ms")
                j = min((j for j in range(len(settings)) if best[j] is not None), key=lambda j: best[j])
                if best[j] < best[0] * (1 - a.min_gain):
                    current = settings[j]
                table[key] = current
        best_ms, _ = case.run(table, tmp.name)
        notes.append(f"tuned: {best_ms:.3f} ms per buffer ({base_ms / best_ms:.3f}x the defaults)")
        log(notes[-1])
        return {k: v for k, v in table.items() if v}, notes
    finally:
        os.unlink(tmp.name)
        if saved is None:
            os.environ.pop(ENV, None)
        else:
            os.environ[ENV] = saved


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--nc", type=int, default=64)
    ap.add_argument("--np", type=int, default=2)
    ap.add_argument("--ntpb", type=int, default=524288)
    ap.add_argument("--nbits", type=int, default=8, choices=[4, 8, 16])
    ap.add_argument("--nt", type=int, action="append", required=True)
    ap.add_argument("--na", type=int, action="append", required=True)
    ap.add_argument("--npol", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="buffers per timed repetition")
    ap.add_argument("--reps", type=int, default=3, help="timed repetitions per run")
    ap.add_argument("--rounds", type=int, default=2, help="interleaved runs of every setting")
    ap.add_argument("--passes", type=int, default=1, help="rounds of coordinate descent over the products")
    ap.add_argument("--min-gain", type=float, default=0.02, help="relative gain a candidate needs over the current")
    ap.add_argument("--out", default="tuning.txt")
    a = ap.parse_args(argv)
    if len(a.nt) != len(a.na):
        ap.error("one --na per --nt")
    table, notes = tune(a)
    cfg = f"Nc {a.nc}, Np {a.np}, Ntpb {a.ntpb}, {a.nbits}-bit, products {list(zip(a.nt, a.na))}, Npolout {a.npol}"
    write_table(a.out, table, [f"rawspec_gb300 tuning table for {cfg}"] + notes)
    print(f"wrote {a.out}: {len(table)} entries")
    return 0


if __name__ == "__main__":
    sys.exit(main())
