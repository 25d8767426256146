"""ctypes front end for the CPU checkers (test infrastructure only).

Loads ``liboracle.so`` (the FP64 restatement in ``qcs_oracle.c``) and, where
it was built, the reference's own sequential / OpenMP libraries under
``oracle/_ref``.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs
of ``bench.py`` import this module; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

PHYSICAL = 0
COMPAT = 1

_lib = None


def ref_sources_present() -> bool:
    """Whether the reference's sources are where the Makefile reads them
    (``make ref-present``)."""
    return subprocess.run(["make", "-s", "-C", HERE, "ref-present"],
                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 0


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference libraries when ``ref``).
    Libraries built on another machine type are rebuilt."""
    import platform
    stamp = os.path.join(HERE, ".arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        for p in (LIB_PATH, os.path.join(REF_DIR, "libqcs_ref_seq.so"),
                  os.path.join(REF_DIR, "libqcs_ref_omp.so")):
            if os.path.exists(p):
                os.remove(p)
        with open(stamp, "w") as f:
            f.write(arch + "\n")
    targets = ["oracle"]
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def set_threads(threads: int) -> int:
    """OpenMP threads of the oracle's sweeps; returns the previous count."""
    return lib().orc_set_threads(threads)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, i, l, d = C.c_void_p, C.c_int, C.c_long, C.c_double
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        lp = C.POINTER(C.c_long)
        sig = {
            "orc_create": (vp, [i, i]),
            "orc_destroy": (None, [vp]),
            "orc_num_qubits": (i, [vp]),
            "orc_size": (l, [vp]),
            "orc_set_basis": (None, [vp, l]),
            "orc_read": (None, [vp, l, l, dp]),
            "orc_write": (None, [vp, l, l, dp]),
            "orc_gate_matrix": (None, [i, d, dp]),
            "orc_apply_1q": (i, [vp, dp, i]),
            "orc_apply_controlled": (i, [vp, dp, i, i]),
            "orc_apply_gate": (i, [vp, i, i, i, d]),
            "orc_run_gates": (i, [vp, i, ip, ip, ip, dp]),
            "orc_run_ops": (i, [vp, i, ip, ip, ip, dp, lp]),
            "orc_apply_block": (i, [vp, i, ip, dp]),
            "orc_phase_flip": (i, [vp, l]),
            "orc_diffusion": (i, [vp]),
            "orc_norm_sq": (d, [vp]),
            "orc_normalize": (None, [vp]),
            "orc_prob_zero": (d, [vp, i]),
            "orc_measure": (i, [vp, i, d]),
            "orc_probability": (d, [vp, l]),
            "orc_argmax": (l, [vp]),
            "orc_sample": (None, [vp, dp, i, lp]),
            "orc_expect_z": (d, [vp, i]),
            "orc_grover_iterations": (i, [i]),
            "orc_qft": (None, [vp]),
            "orc_grover": (None, [vp, l, i]),
            "orc_set_threads": (i, [i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def gate_matrix(kind: int, angle: float = 0.0) -> np.ndarray:
    out = np.zeros(8, dtype=np.float64)
    lib().orc_gate_matrix(kind, angle, _dp(out))
    return out


class OracleState:
    """One FP64 state vector of the oracle (physical or compat mode)."""

    def __init__(self, n: int, mode: int = PHYSICAL):
        self.n = n
        self.mode = mode
        self._h = lib().orc_create(n, mode)
        if not self._h:
            raise MemoryError(f"oracle: cannot allocate {n} qubits")

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def size(self) -> int:
        return 1 << self.n

    def set_basis(self, index: int):
        lib().orc_set_basis(self._h, index)

    def amplitudes(self) -> np.ndarray:
        out = np.zeros(2 * self.size, dtype=np.float64)
        lib().orc_read(self._h, 0, self.size, _dp(out))
        return out.view(np.complex128)

    def set_amplitudes(self, amps: np.ndarray):
        a = np.ascontiguousarray(amps, dtype=np.complex128).view(np.float64)
        lib().orc_write(self._h, 0, self.size, _dp(a))

    def apply_1q(self, m: np.ndarray, target: int) -> int:
        m = np.ascontiguousarray(m, dtype=np.float64)
        return lib().orc_apply_1q(self._h, _dp(m), target)

    def apply_controlled(self, m: np.ndarray, control: int, target: int) -> int:
        m = np.ascontiguousarray(m, dtype=np.float64)
        return lib().orc_apply_controlled(self._h, _dp(m), control, target)

    def apply_gate(self, kind: int, target: int, control: int = -1, angle: float = 0.0) -> int:
        return lib().orc_apply_gate(self._h, kind, target, control, angle)

    def run(self, gates) -> None:
        k = np.ascontiguousarray(gates.kinds, dtype=np.int32)
        t = np.ascontiguousarray(gates.targets, dtype=np.int32)
        c = np.ascontiguousarray(gates.controls, dtype=np.int32)
        a = np.ascontiguousarray(gates.angles, dtype=np.float64)
        ix = np.ascontiguousarray(getattr(gates, "indices", [0] * len(k)), dtype=np.int64)
        rc = lib().orc_run_ops(self._h, len(k), _ip(k), _ip(t), _ip(c), _dp(a),
                               ix.ctypes.data_as(C.POINTER(C.c_long)))
        if rc != 0:
            raise ValueError("oracle: invalid gate in list")

    def apply_block(self, qubits, u: np.ndarray) -> None:
        q = np.ascontiguousarray(qubits, dtype=np.int32)
        uu = np.ascontiguousarray(u, dtype=np.complex128).view(np.float64)
        if lib().orc_apply_block(self._h, len(q), _ip(q), _dp(uu)) != 0:
            raise ValueError("oracle: invalid block")

    def phase_flip(self, index: int):
        lib().orc_phase_flip(self._h, index)

    def diffusion(self):
        lib().orc_diffusion(self._h)

    def norm_sq(self) -> float:
        return lib().orc_norm_sq(self._h)

    def normalize(self):
        lib().orc_normalize(self._h)

    def prob_zero(self, q: int) -> float:
        return lib().orc_prob_zero(self._h, q)

    def measure(self, q: int, r: float) -> int:
        return lib().orc_measure(self._h, q, r)

    def probability(self, index: int) -> float:
        return lib().orc_probability(self._h, index)

    def argmax(self) -> int:
        return lib().orc_argmax(self._h)

    def sample(self, r: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros(len(r), dtype=np.int64)
        lib().orc_sample(self._h, _dp(r), len(r), out.ctypes.data_as(C.POINTER(C.c_long)))
        return out

    def expect_z(self, q: int) -> float:
        return lib().orc_expect_z(self._h, q)

    def qft(self):
        lib().orc_qft(self._h)

    def grover(self, solution: int, iterations: int = -1):
        lib().orc_grover(self._h, solution, iterations)


def grover_iterations(n: int) -> int:
    return lib().orc_grover_iterations(n)


# --------------------------------------------------------------------------
# The reference's own library (compiled from its sources by `make ref`).
# --------------------------------------------------------------------------


class _TComplex(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class _TQState(C.Structure):
    # struct t_q_state (src/internal.h:43-48)
    _fields_ = [
        ("qubits_num", C.c_int),
        ("size", C.c_long),
        ("vector", C.POINTER(_TComplex)),
        ("scratch_vector", C.POINTER(_TComplex)),
    ]


class _TQCircuitHead(C.Structure):
    # leading members of struct t_q_circuit (src/qcs.c:13-16)
    _fields_ = [
        ("num_qubits", C.c_int),
        ("num_gates", C.c_int),
        ("state", C.POINTER(_TQState)),
    ]


def ref_path(kind: str = "seq") -> str:
    return os.path.join(REF_DIR, f"libqcs_ref_{kind}.so")


def ref_available(kind: str = "seq") -> bool:
    return os.path.exists(ref_path(kind))


_ref_libs: dict = {}


def ref_lib(kind: str = "seq") -> C.CDLL:
    if kind not in _ref_libs:
        L = C.CDLL(ref_path(kind))
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        ip = C.POINTER(C.c_int)
        sig = {
            "qc_create": (vp, [i]),
            "qc_destroy": (None, [vp]),
            "qc_h": (None, [vp, i]),
            "qc_x": (None, [vp, i]),
            "qc_y": (None, [vp, i]),
            "qc_z": (None, [vp, i]),
            "qc_cnot": (None, [vp, i, i]),
            "qc_cphase": (None, [vp, i, i, d]),
            "qc_phase": (None, [vp, i, d]),
            "qc_rx": (None, [vp, i, d]),
            "qc_ry": (None, [vp, i, d]),
            "qc_rz": (None, [vp, i, d]),
            "qc_measure": (i, [vp, i]),
            "qc_measure_all": (None, [vp, ip]),
            "qc_run_shots": (None, [vp, i, ip]),
            "qc_find_most_likely_state": (i, [vp]),
            "qc_get_probability": (d, [vp, i]),
            "qc_grover_search": (None, [vp, i]),
            "qc_quantum_fourier_transform": (None, [vp]),
            "qc_bernstein_vazirani": (None, [vp, i]),
            "qc_ghz_state": (None, [vp]),
            "qc_reset": (None, [vp, i]),
            "qc_get_num_gates": (i, [vp]),
            "q_apply_phase_flip": (None, [vp, i]),
            "q_apply_diffusion": (None, [vp]),
            "q_state_normalize": (None, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _ref_libs[kind] = L
    return _ref_libs[kind]


class RefCircuit:
    """A circuit of the reference library, driven through its public API."""

    def __init__(self, n: int, kind: str = "seq"):
        self.L = ref_lib(kind)
        self.n = n
        self._h = self.L.qc_create(n)
        if not self._h:
            raise MemoryError("reference qc_create failed")

    def close(self):
        if self._h:
            self.L.qc_destroy(self._h)
            self._h = None

    __del__ = close

    def _state(self) -> _TQState:
        head = C.cast(self._h, C.POINTER(_TQCircuitHead)).contents
        return head.state.contents

    def state_ptr(self):
        head = C.cast(self._h, C.POINTER(_TQCircuitHead)).contents
        return C.cast(head.state, C.c_void_p)

    def amplitudes(self) -> np.ndarray:
        st = self._state()
        buf = C.cast(st.vector, C.POINTER(C.c_double * (2 * st.size))).contents
        return np.frombuffer(buf, dtype=np.float64).copy().view(np.complex128)

    def apply_gate(self, kind: int, target: int, control: int = -1, angle: float = 0.0):
        L, h = self.L, self._h
        if kind == 0:
            L.qc_h(h, target)
        elif kind == 1:
            L.qc_x(h, target)
        elif kind == 2:
            L.qc_y(h, target)
        elif kind == 3:
            L.qc_z(h, target)
        elif kind == 4:
            L.qc_phase(h, target, angle)
        elif kind == 5:
            L.qc_rx(h, target, angle)
        elif kind == 6:
            L.qc_ry(h, target, angle)
        elif kind == 7:
            L.qc_rz(h, target, angle)
        elif kind == 8:
            L.qc_cnot(h, control, target)
        elif kind == 9:
            L.qc_cphase(h, control, target, angle)
        else:
            raise ValueError(kind)

    def run(self, gates):
        for k, t, c, a in zip(gates.kinds, gates.targets, gates.controls, gates.angles):
            self.apply_gate(int(k), int(t), int(c), float(a))
