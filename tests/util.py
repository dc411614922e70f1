"""Helpers shared by the parity tests."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

# Tolerance of the FP32 path against the FP64 oracle, relative per fine
# channel.  The denominator of a bin is its total power (I, or XX+YY, or P),
# floored at 1% of the spectrum's mean total power so that bins with almost no
# power do not turn rounding noise into large relative numbers; cross terms
# (Re/Im XY*, Q, U, V) are normalised by the same total power.
REL_TOL = 1e-5


def total_power_planes(arr: np.ndarray, npol: int, Nc: int, Nt: int) -> tuple[np.ndarray, np.ndarray]:
    """arr: [ndump, Nd*|P|*Nc*Nt] -> (values [ndump, Nd, |P|, Nc, Nt], total power [ndump, Nd, 1, Nc, Nt])."""
    a = arr.reshape(arr.shape[0], -1, abs(npol), Nc, Nt)
    if npol == 1:
        tp = a[:, :, :1]
    elif npol == 4:
        tp = a[:, :, 0:1] + a[:, :, 1:2]
    else:
        tp = a[:, :, 0:1]
    return a, tp


def normalized_error(got: np.ndarray, ref: np.ndarray, npol: int, Nc: int, Nt: int) -> float:
    g, _ = total_power_planes(np.asarray(got, np.float64), npol, Nc, Nt)
    r, tp = total_power_planes(np.asarray(ref, np.float64), npol, Nc, Nt)
    mean = tp.mean(axis=-1, keepdims=True)
    den = np.maximum(np.abs(tp), 1e-2 * np.abs(mean))
    den = np.where(den > 0, den, 1.0)
    return float(np.max(np.abs(g - r) / den))


def rms_normalized_error(got: np.ndarray, ref: np.ndarray, npol: int, Nc: int, Nt: int) -> float:
    """Root mean square of the per-bin errors of normalized_error."""
    g, _ = total_power_planes(np.asarray(got, np.float64), npol, Nc, Nt)
    r, tp = total_power_planes(np.asarray(ref, np.float64), npol, Nc, Nt)
    mean = tp.mean(axis=-1, keepdims=True)
    den = np.maximum(np.abs(tp), 1e-2 * np.abs(mean))
    den = np.where(den > 0, den, 1.0)
    return float(np.sqrt(np.mean(((g - r) / den) ** 2)))


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}
