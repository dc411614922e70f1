"""Generates the golden fixtures tests/golden/<case>.npz: the seeded input
bytes of each case in cases.py and the FP64 oracle's dumps (and incoherent
sums) for every product.

usage: python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

from cases import CASES, blocks_for, derived_nb  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    for name, c in CASES.items():
        blocks, weights = blocks_for(name)
        cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), c["nbits"], c["products"],
                         Nant=c.get("Nant", 1), conj=c["conj"], inverse=1 if c["fft_dir"] <= 0 else 0,
                         weights=weights)
        outs, icss = O.run_oracle(cfg, blocks)
        arrays = {"blocks": blocks}
        if weights is not None:
            arrays["weights"] = weights
        for i, o in enumerate(outs):
            arrays[f"out{i}"] = o
        for i, s in enumerate(icss):
            arrays[f"ics{i}"] = s
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        print(name, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
