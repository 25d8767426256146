"""Seeded synthetic circuits for the QCS hot path.

One project PRNG (xoshiro256** seeded through splitmix64) generates every
workload, so the GPU path, the oracle and the reference library all run the
same gate list for a given seed.  The circuit shapes restate the benchmark
configurations of this backend:

* ``random_circuit``  -- n qubits, random basis state, the reference's QFT
  (``qc_quantum_fourier_transform``, src/qcs.c:443-457) and then ``count``
  random gates: 70 % one-qubit gates drawn uniformly from
  {H, X, Y, Z, RX, RY, RZ, P} with angles uniform in [0, 2 pi), 30 % CNOT on
  a uniform ordered pair of distinct qubits.
* ``brick_circuit``   -- per layer RZ.RY.RZ on every qubit (angles uniform
  in [0, 2 pi)), then CNOT(2i, 2i+1) on even layers and CNOT(2i+1, 2i+2) on
  odd layers.
* ``grover_workload`` -- QFT on a random basis state, then rounds of
  (Hadamard layer, phase flip on a random marked index, diffusion); and the
  structure of ``qc_grover_search`` (src/qcs.c:402-419) from |0...0>.
* ``variational_batch`` -- instances with n ~ U[10, 22] and depth
  ~ U[4, 16]; per layer RY and RZ on every qubit, then a linear CNOT ladder.
* ``mixed_circuit``   -- per layer a random rotation on every qubit, then
  CNOTs and QFT-style controlled phases (pi / 2^d) on a random pairing.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import NamedTuple

import numpy as np

# Gate kinds: identical to QCS_GATE_* in include/qcs_cuda.h.
H, X, Y, Z, P, RX, RY, RZ, CNOT, CPHASE, I = range(11)
PHASE_FLIP = 20
DIFFUSION = 21
ONE_QUBIT_SET = (H, X, Y, Z, RX, RY, RZ, P)
PARAMETRIC = (P, RX, RY, RZ, CPHASE)
NAMES = {H: "H", X: "X", Y: "Y", Z: "Z", P: "P", RX: "RX", RY: "RY", RZ: "RZ",
         CNOT: "CNOT", CPHASE: "CPHASE", I: "I", PHASE_FLIP: "FLIP", DIFFUSION: "DIFFUSION"}

# struct qcs_cuda_op (include/qcs_cuda.h): 32 bytes.
OP_DTYPE = np.dtype([("kind", "<i4"), ("target", "<i4"), ("control", "<i4"),
                     ("reserved", "<i4"), ("angle", "<f8"), ("index", "<i8")])

_MASK = (1 << 64) - 1


def _rotl(x: int, k: int) -> int:
    return ((x << k) | (x >> (64 - k))) & _MASK


class Rng:
    """xoshiro256** seeded by splitmix64 (Blackman & Vigna)."""

    def __init__(self, seed: int):
        x = seed & _MASK
        s = []
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & _MASK
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
            s.append(z ^ (z >> 31))
        self.s = s

    def next_u64(self) -> int:
        s0, s1, s2, s3 = self.s
        result = (_rotl((s1 * 5) & _MASK, 7) * 9) & _MASK
        t = (s1 << 17) & _MASK
        s2 ^= s0
        s3 ^= s1
        s1 ^= s2
        s0 ^= s3
        s2 ^= t
        s3 = _rotl(s3, 45)
        self.s = [s0, s1, s2, s3]
        return result

    def uniform(self) -> float:
        """Uniform double in [0, 1) with 53 random bits."""
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def below(self, n: int) -> int:
        """Uniform integer in [0, n) (n <= 2^53)."""
        return int(self.uniform() * n)

    def angle(self) -> float:
        return self.uniform() * (2.0 * math.pi)


@dataclass
class GateList:
    kinds: list = field(default_factory=list)
    targets: list = field(default_factory=list)
    controls: list = field(default_factory=list)
    angles: list = field(default_factory=list)
    indices: list = field(default_factory=list)

    def add(self, kind: int, target: int = -1, control: int = -1,
            angle: float = 0.0, index: int = 0) -> None:
        self.kinds.append(kind)
        self.targets.append(target)
        self.controls.append(control)
        self.angles.append(angle)
        self.indices.append(index)

    def extend(self, other: "GateList") -> None:
        self.kinds += other.kinds
        self.targets += other.targets
        self.controls += other.controls
        self.angles += other.angles
        self.indices += other.indices

    def __len__(self) -> int:
        return len(self.kinds)

    def ops(self) -> np.ndarray:
        """The list as an array of struct qcs_cuda_op records."""
        a = np.zeros(len(self), dtype=OP_DTYPE)
        a["kind"] = self.kinds
        a["target"] = self.targets
        a["control"] = self.controls
        a["angle"] = self.angles
        a["index"] = self.indices
        return a

    def gate_count(self) -> int:
        """Original gates (phase flips and diffusions count one each)."""
        return len(self)

    def only_gates(self) -> bool:
        return all(k <= CPHASE for k in self.kinds)


def qft_gates(n: int) -> GateList:
    """qc_quantum_fourier_transform (src/qcs.c:443-457)."""
    g = GateList()
    for i in range(n):
        g.add(H, i)
        for j in range(i + 1, n):
            g.add(CPHASE, i, j, math.pi / float(1 << (j - i)))
    return g


def basis_gates(n: int, index: int) -> GateList:
    """X on every set bit: prepares |index> exactly from |0...0>."""
    g = GateList()
    for q in range(n):
        if (index >> q) & 1:
            g.add(X, q)
    return g


def random_gates(n: int, count: int, rng: Rng, p_one_qubit: float = 0.7) -> GateList:
    g = GateList()
    for _ in range(count):
        if rng.uniform() < p_one_qubit:
            kind = ONE_QUBIT_SET[rng.below(len(ONE_QUBIT_SET))]
            t = rng.below(n)
            a = rng.angle() if kind in PARAMETRIC else 0.0
            g.add(kind, t, -1, a)
        else:
            c = rng.below(n)
            t = rng.below(n - 1)
            if t >= c:
                t += 1
            g.add(CNOT, t, c)
    return g


def random_circuit(n: int, seed: int, count: int = 200, with_qft: bool = True):
    """(basis index, gate list): random basis, QFT, `count` random gates."""
    rng = Rng(seed)
    basis = rng.below(1 << n)
    g = GateList()
    if with_qft:
        g.extend(qft_gates(n))
    g.extend(random_gates(n, count, rng))
    return basis, g


def one_qubit_circuit(n: int, seed: int, count: int) -> GateList:
    rng = Rng(seed)
    g = GateList()
    for _ in range(count):
        kind = ONE_QUBIT_SET[rng.below(len(ONE_QUBIT_SET))]
        g.add(kind, rng.below(n), -1, rng.angle() if kind in PARAMETRIC else 0.0)
    return g


def brick_circuit(n: int, depth: int, seed: int) -> GateList:
    rng = Rng(seed)
    g = GateList()
    for layer in range(depth):
        for q in range(n):
            g.add(RZ, q, -1, rng.angle())
            g.add(RY, q, -1, rng.angle())
            g.add(RZ, q, -1, rng.angle())
        start = 0 if layer % 2 == 0 else 1
        for a in range(start, n - 1, 2):
            g.add(CNOT, a + 1, a)
    return g


class GroverWorkload(NamedTuple):
    basis: int       # start of the QFT part
    marked: int      # the phase-flipped index
    qft: GateList    # qc_quantum_fourier_transform
    rounds: GateList  # iterations x (Hadamard layer, phase flip, diffusion)
    search: GateList  # Hadamard layer, then iterations x (phase flip, diffusion)


def grover_workload(n: int, seed: int, iterations: int = 64) -> GroverWorkload:
    """The 33/34-qubit workload: QFT on the random basis state |basis>, then
    `iterations` rounds of (Hadamard layer, phase flip on the random marked
    index, diffusion) -- `qft` followed by `rounds`.

    After those rounds no amplitude dominates: at 16 qubits the top
    probabilities agree to 4e-16 relative, so which index is the argmax is
    decided by rounding, in FP64 too.  `search` is qc_grover_search's own
    structure (src/qcs.c:402-419) with the same marked index and iteration
    count, run from |0...0>: one Hadamard layer, then `iterations` x (phase
    flip, diffusion).  There the marked index dominates (by ~1e4 at 28
    qubits), so its argmax is a well-posed basis-state answer."""
    rng = Rng(seed)
    basis = rng.below(1 << n)
    marked = rng.below(min(1 << n, 1 << 31))
    rounds = GateList()
    search = GateList()
    for q in range(n):
        search.add(H, q)
    for _ in range(iterations):
        for q in range(n):
            rounds.add(H, q)
        for g in (rounds, search):
            g.add(PHASE_FLIP, index=marked)
            g.add(DIFFUSION)
    return GroverWorkload(basis, marked, qft_gates(n), rounds, search)


def variational_instance(rng: Rng, n_range=(10, 22), depth_range=(4, 16)):
    n = n_range[0] + rng.below(n_range[1] - n_range[0] + 1)
    depth = depth_range[0] + rng.below(depth_range[1] - depth_range[0] + 1)
    g = GateList()
    for _ in range(depth):
        for q in range(n):
            g.add(RY, q, -1, rng.angle())
            g.add(RZ, q, -1, rng.angle())
        for q in range(n - 1):
            g.add(CNOT, q + 1, q)
    return n, g


def variational_batch(count: int, seed: int, n_range=(10, 22), depth_range=(4, 16)):
    rng = Rng(seed)
    return [variational_instance(rng, n_range, depth_range) for _ in range(count)]


def mixed_circuit(n: int, depth: int, seed: int) -> GateList:
    rng = Rng(seed)
    g = GateList()
    rot = (RX, RY, RZ)
    for _ in range(depth):
        for q in range(n):
            g.add(rot[rng.below(3)], q, -1, rng.angle())
        perm = list(range(n))
        for i in range(n - 1, 0, -1):
            j = rng.below(i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        for i in range(0, n - 1, 2):
            c, t = perm[i], perm[i + 1]
            if rng.uniform() < 0.5:
                g.add(CNOT, t, c)
            else:
                d = 1 + rng.below(min(8, n - 1))
                g.add(CPHASE, t, c, math.pi / float(1 << d))
    return g
