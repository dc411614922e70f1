"""Runs one spectrometer configuration through the C-ABI a few times, for
profiling a single kernel with Nsight Compute.

usage: python -m rawspec_gb300.profile_case --nc 64 --ntpb 524288 --nt 1048576 --na 51 [--npol 1] [--buffers 2]

Input: seeded 8-bit Gaussian voltages (sigma 20), device resident after the
first copy; each buffer is processed with rawspec_start_processing.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--nc", type=int, default=64)
    ap.add_argument("--ntpb", type=int, default=524288)
    ap.add_argument("--nt", type=int, action="append", required=True)
    ap.add_argument("--na", type=int, action="append", required=True)
    ap.add_argument("--npol", type=int, default=1)
    ap.add_argument("--nb", type=int, default=0)
    ap.add_argument("--buffers", type=int, default=2)
    a = ap.parse_args()
    from rawspec_gb300 import api, synth
    prods = [(nt, na, a.npol) for nt, na in zip(a.nt, a.na)]
    with api.Spectrometer(a.nc, 2, a.ntpb, 8, prods, Nb=a.nb, collect=False) as spec:
        blocks = synth.gaussian_blocks(spec.Nb, a.nc, a.ntpb, 2, sigma=20.0, seed=1)
        spec.load_blocks(blocks)
        spec.copy_to_gpu()
        for _ in range(a.buffers):
            spec.start()
        rc = spec.wait()
        print(f"processed {a.buffers} buffers of {spec.Nb} blocks, launches {spec.kernel_launches()}, rc {rc}")
    return rc


if __name__ == "__main__":
    sys.exit(main())
