"""Shared helpers for the tests (fixture decoding, fidelity)."""
import numpy as np

from qcs_gb300 import workloads as W


def gates_from(d) -> W.GateList:
    g = W.GateList()
    for k, t, c, a, ix in zip(d["kinds"], d["targets"], d["controls"], d["angles"],
                              d["indices"]):
        g.add(int(k), int(t), int(c), float(a), int(ix))
    return g


def infidelity(a: np.ndarray, b: np.ndarray) -> float:
    """1 - |<a|b>|^2 / (<a|a><b|b>) in FP64."""
    a = a.astype(np.complex128)
    b = b.astype(np.complex128)
    num = abs(np.vdot(a, b)) ** 2
    den = np.vdot(a, a).real * np.vdot(b, b).real
    return float(1.0 - num / den)


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    """Bit-for-bit equality of complex128 arrays (+0 and -0 compare equal)."""
    return bool(np.array_equal(a.view(np.float64), b.view(np.float64)))
