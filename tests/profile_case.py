"""Runs one spectrometer configuration through the C-ABI a few times, for
profiling a single kernel with Nsight Compute.

usage: python tests/profile_case.py --nc 64 --ntpb 524288 --nt 1048576 --na 51 [--npol 1] [--buffers 2]
       [--nbits 4|8|16] [--np 1|2] [--nant A --ics] [--copy-each] [--timing]

Input: seeded Gaussian voltages (sigma 20; 4-bit: uniform with per-antenna
gains), device resident after the first copy (or copied, and expanded, for
every buffer with --copy-each); each buffer is processed with
rawspec_start_processing.  --timing then processes 3 more buffers and times
10 with the library's per-kernel-class CUDA events, printing the average
microseconds per buffer of each class.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))  # the repository root


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--nc", type=int, default=64)
    ap.add_argument("--np", type=int, default=2)
    ap.add_argument("--ntpb", type=int, default=524288)
    ap.add_argument("--nbits", type=int, default=8, choices=[4, 8, 16])
    ap.add_argument("--nt", type=int, action="append", required=True)
    ap.add_argument("--na", type=int, action="append", required=True)
    ap.add_argument("--npol", type=int, default=1)
    ap.add_argument("--nant", type=int, default=1)
    ap.add_argument("--ics", action="store_true", help="weighted incoherent sum over the antennas")
    ap.add_argument("--nb", type=int, default=0)
    ap.add_argument("--buffers", type=int, default=2)
    ap.add_argument("--copy-each", action="store_true", help="copy (and expand 4-bit) the blocks for every buffer")
    ap.add_argument("--timing", action="store_true", help="time 10 more buffers per kernel class")
    a = ap.parse_args()
    from rawspec_gb300 import api, synth
    prods = [(nt, na, a.npol) for nt, na in zip(a.nt, a.na)]
    w = list(synth.weights(a.nant, seed=2)) if a.ics else None
    with api.Spectrometer(a.nc, a.np, a.ntpb, a.nbits, prods, Nb=a.nb, Nant=a.nant, weights=w,
                          collect=False) as spec:
        if a.nbits == 4:
            blocks, _ = synth.int4_blocks(spec.Nb, a.nc, a.ntpb, a.np, Nant=a.nant, seed=1)
        else:
            blocks = synth.gaussian_blocks(spec.Nb, a.nc, a.ntpb, a.np, sigma=20.0, seed=1, nbits=a.nbits)
        spec.load_blocks(blocks)
        spec.copy_to_gpu()
        for _ in range(a.buffers):
            if a.copy_each:
                spec.copy_to_gpu()
            spec.start()
        rc = spec.wait()
        print(f"processed {a.buffers} buffers of {spec.Nb} blocks, launches {spec.kernel_launches()}, rc {rc}")
        if a.timing and rc == 0:
            for _ in range(3):
                spec.start()
            spec.wait()
            spec.reset_profile()
            spec.set_profiling(True)
            for _ in range(10):
                if a.copy_each:
                    spec.copy_to_gpu()
                spec.start()
            rc = spec.wait()
            us = {}
            for k, name in enumerate(api.KERNEL_CLASS_NAMES):
                ms, n = spec.profile(k)[:2]
                if n:
                    us[name] = round(ms * 1e3 / 10, 1)
            print(f"microseconds per buffer by kernel class: {us}")
    return rc


if __name__ == "__main__":
    sys.exit(main())
