"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run here, where the reference sources are present (they are not on the GPU
machine):

    make -C oracle ref              # builds oracle/_ref/libqcs_ref_seq.so
    python tests/golden/make_golden.py

Each fixture records the reference's own sequential build (compiled from its
sources by oracle/Makefile, driven through its public API) on a seeded
workload, plus, where the reference's semantics are not the textbook ones, an
independent numpy complex128 computation of the physical result.  The
fixtures are small (n <= 12) and stored as .npz.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from qcs_gb300 import workloads as W  # noqa: E402


# ---- independent numpy model of the physical semantics ----------------------

def np_gate(kind, angle):
    h = 1 / math.sqrt(2.0)
    c, s = math.cos(angle / 2.0), math.sin(angle / 2.0)
    return {
        W.H: np.array([[h, h], [h, -h]], complex),
        W.X: np.array([[0, 1], [1, 0]], complex),
        W.CNOT: np.array([[0, 1], [1, 0]], complex),
        W.Y: np.array([[0, -1j], [1j, 0]], complex),
        W.Z: np.array([[1, 0], [0, -1]], complex),
        W.P: np.array([[1, 0], [0, np.exp(1j * angle)]], complex),
        W.CPHASE: np.array([[1, 0], [0, np.exp(1j * angle)]], complex),
        W.RX: np.array([[c, -1j * s], [-1j * s, c]], complex),
        W.RY: np.array([[c, -s], [s, c]], complex),
        W.RZ: np.array([[c - 1j * s, 0], [0, c + 1j * s]], complex),
    }[kind]


def np_apply(psi, n, kind, target, control=-1, angle=0.0):
    """Textbook (controlled-)U on a complex128 vector, via reshapes."""
    g = np_gate(kind, angle)
    t = psi.reshape([2] * n)  # axis a <-> qubit n-1-a
    ax = n - 1 - target
    if kind in (W.CNOT, W.CPHASE):
        cax = n - 1 - control
        idx = [slice(None)] * n
        idx[cax] = 1
        sub = t[tuple(idx)]
        ax2 = ax if ax < cax else ax - 1
        sub = np.moveaxis(np.tensordot(g, sub, axes=([1], [ax2])), 0, ax2)
        t = t.copy()
        t[tuple(idx)] = sub
    else:
        t = np.moveaxis(np.tensordot(g, t, axes=([1], [ax])), 0, ax)
    return np.ascontiguousarray(t).reshape(-1)


def np_run(n, gates, psi=None):
    if psi is None:
        psi = np.zeros(1 << n, complex)
        psi[0] = 1
    for k, t, c, a, ix in zip(gates.kinds, gates.targets, gates.controls, gates.angles,
                              gates.indices):
        if k == W.PHASE_FLIP:
            psi = psi.copy()
            psi[ix] = -psi[ix]
        elif k == W.DIFFUSION:
            psi = 2 * psi.mean() - psi
        else:
            psi = np_apply(psi, n, k, t, c, a)
    return psi


def gates_arrays(g):
    return dict(kinds=np.array(g.kinds, np.int32), targets=np.array(g.targets, np.int32),
                controls=np.array(g.controls, np.int32), angles=np.array(g.angles, np.float64),
                indices=np.array(g.indices, np.int64))


def ref_run(n, g):
    r = O.RefCircuit(n)
    r.run(g)
    a = r.amplitudes()
    r.close()
    return a


def main():
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libqcs_ref_seq.so missing: run `make -C oracle ref`")
    out = {}

    # 1. one-qubit-gate circuit: reference == physical == this backend, bit for bit
    g = W.one_qubit_circuit(10, 7, 300)
    out["ref_1q_n10"] = dict(n=10, **gates_arrays(g), ref=ref_run(10, g))

    # 2. mixed random circuits (basis prep, QFT, 300 random gates): the
    #    reference's own (non-unitary) controlled sweep, and the physical result
    for seed in (0, 1):
        basis, g0 = W.random_circuit(10, seed, 300)
        g = W.basis_gates(10, basis)
        g.extend(g0)
        out[f"ref_mixed_n10_s{seed}"] = dict(n=10, **gates_arrays(g), ref=ref_run(10, g),
                                             physical=np_run(10, g))

    # 3. the 20-qubit random-circuit workload's shape at 12 qubits
    basis, g0 = W.random_circuit(12, 2024, 200)
    g = W.basis_gates(12, basis)
    g.extend(g0)
    out["ref_random_n12"] = dict(n=12, **gates_arrays(g), ref=ref_run(12, g),
                                 physical=np_run(12, g))

    # 4. Grover n=6, solution 42 through qc_grover_search
    r = O.RefCircuit(6)
    r.L.qc_grover_search(r._h, 42)
    ga = W.GateList()
    for q in range(6):
        ga.add(W.H, q)
    for _ in range(O.grover_iterations(6)):
        ga.add(W.PHASE_FLIP, index=42)
        ga.add(W.DIFFUSION)
    out["ref_grover_n6"] = dict(n=6, solution=42, iterations=O.grover_iterations(6),
                                ref=r.amplitudes(),
                                ref_prob=r.L.qc_get_probability(r._h, 42),
                                physical=np_run(6, ga), **gates_arrays(ga))
    r.close()

    # 5. measurement sequence with the reference's rand() draws
    libc = C.CDLL(None)
    libc.rand.restype = C.c_int
    n = 5
    prep = W.GateList()
    rng = W.Rng(99)
    for q in range(n):
        prep.add(W.H, q)
        prep.add(W.RY, q, -1, rng.angle())
    r = O.RefCircuit(n)
    r.run(prep)
    seed = 12345
    libc.srand(seed)
    outcomes = [r.L.qc_measure(r._h, q) for q in (0, 2, 4)]
    libc.srand(seed)
    draws = [libc.rand() / float(2**31 - 1) for _ in range(3)]
    out["ref_measure_n5"] = dict(n=n, **gates_arrays(prep), seed=seed,
                                 qubits=np.array([0, 2, 4]), outcomes=np.array(outcomes),
                                 draws=np.array(draws), ref=r.amplitudes())
    r.close()

    # 6. shots: histogram of qc_run_shots with its draws
    r = O.RefCircuit(n)
    r.run(prep)
    hist = np.zeros(1 << n, np.int32)
    libc.srand(777)
    r.L.qc_run_shots(r._h, 2000, hist.ctypes.data_as(C.POINTER(C.c_int)))
    libc.srand(777)
    draws = np.array([libc.rand() / float(2**31 - 1) for _ in range(2000)])
    out["ref_shots_n5"] = dict(n=n, **gates_arrays(prep), seed=777, shots=2000, hist=hist,
                               draws=draws, ref=r.amplitudes())
    r.close()

    # 7. Bernstein-Vazirani, all 32 five-bit secrets: the reference's argmax
    bv = []
    for secret in range(32):
        r = O.RefCircuit(6)
        r.L.qc_bernstein_vazirani(r._h, secret)
        bv.append(r.L.qc_find_most_likely_state(r._h))
        r.close()
    out["ref_bv_n6"] = dict(secrets=np.arange(32), ref_argmax=np.array(bv))

    # 8. known answers of the reference's own test suite (test/test_qc_*.c),
    #    as the reference's sequential build computes them
    ka = {}
    r = O.RefCircuit(2)
    r.L.qc_x(r._h, 0)
    r.L.qc_cnot(r._h, 0, 1)
    ka["cnot_argmax"] = r.L.qc_find_most_likely_state(r._h)  # test_qc_cnot.c:10 expects 3
    r.close()
    r = O.RefCircuit(3)
    r.L.qc_quantum_fourier_transform(r._h)
    ka["qft3_probs"] = np.array([r.L.qc_get_probability(r._h, i) for i in range(8)])
    r.close()
    out["ref_known_answers"] = ka

    for name, d in out.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
