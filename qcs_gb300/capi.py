"""ctypes bindings of libqcs_gb300.so.

Two surfaces, both plain C:

* the backend C ABI of ``include/qcs_cuda.h`` (``State`` wraps one
  ``qcs_cuda_state``), and
* the reference's public API of ``include/qcs.h`` / ``include/qcs_ext.h``
  (``api()`` returns the library with ``qc_*`` signatures set), so tests can
  read exactly like the reference's ``test/test_qc_*.c``.

There is no CPU fallback: if the library is missing this module raises, and
without a GPU ``State`` creation fails with ``QcsCudaError(ENODEV)``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import workloads as W

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libqcs_gb300.so")

OK, EINVAL, ENOMEM, ENODEV, ELAUNCH, ETIMEOUT, EUNSUP = range(7)
C64, C128 = 0, 1
PHYSICAL, REFERENCE = 0, 1
FUSE_AUTO, FUSE_SIMT, FUSE_TENSOR = 0, 1, 2
PARTITION_GREEDY, PARTITION_LEARNED = 0, 1
# QCS_KCLASS_* order (include/qcs_cuda.h)
KCLASS_NAMES = ("dense1q", "diag1q", "phase_mask", "ctrl1q", "block_simt", "block_tc",
                "reduce", "diffuse", "collapse", "sample", "other", "block_tc7")


class QcsCudaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


RUN_NO_PLAN_CACHE = 1


class RunOptions(C.Structure):
    _fields_ = [("fusion_k", C.c_int), ("fusion_engine", C.c_int),
                ("partitioner", C.c_int), ("flags", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(
                f"{LIB_PATH} is missing: run `python -m qcs_gb300.build` first")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    vp, i, d, ll = C.c_void_p, C.c_int, C.c_double, C.c_longlong
    dp, ip, llp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_longlong)
    vpp = C.POINTER(C.c_void_p)
    fp = C.POINTER(C.c_float)
    sig = {
        "qcs_cuda_strerror": (C.c_char_p, [i]),
        "qcs_cuda_last_error": (C.c_char_p, []),
        "qcs_cuda_device_count": (i, [ip]),
        "qcs_cuda_debug_inject": (i, [i, i]),
        "qcs_cuda_debug_set_wait_cycles": (i, [ll]),
        "qcs_cuda_state_create": (i, [i, i, i, vpp]),
        "qcs_cuda_state_destroy": (i, [vp]),
        "qcs_cuda_state_info": (i, [vp, ip, ip, ip]),
        "qcs_cuda_state_stream": (i, [vp, vpp]),
        "qcs_cuda_state_device_ptr": (i, [vp, vpp]),
        "qcs_cuda_synchronize": (i, [vp]),
        "qcs_cuda_set_basis": (i, [vp, ll]),
        "qcs_cuda_read_amplitudes": (i, [vp, ll, ll, dp]),
        "qcs_cuda_write_amplitudes": (i, [vp, ll, ll, dp]),
        "qcs_cuda_apply_1q": (i, [vp, dp, i]),
        "qcs_cuda_apply_controlled_1q": (i, [vp, dp, i, i]),
        "qcs_cuda_apply_gate": (i, [vp, i, i, i, d]),
        "qcs_cuda_apply_block": (i, [vp, i, ip, dp, i]),
        "qcs_cuda_phase_flip": (i, [vp, ll]),
        "qcs_cuda_diffusion": (i, [vp]),
        "qcs_cuda_run": (i, [vp, vp, i, C.POINTER(RunOptions)]),
        "qcs_cuda_transfer_bytes": (i, [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "qcs_cuda_norm_sq": (i, [vp, dp]),
        "qcs_cuda_normalize": (i, [vp]),
        "qcs_cuda_prob_zero": (i, [vp, i, dp]),
        "qcs_cuda_measure": (i, [vp, i, d, ip]),
        "qcs_cuda_probability": (i, [vp, ll, dp]),
        "qcs_cuda_argmax": (i, [vp, llp, dp]),
        "qcs_cuda_expect_z": (i, [vp, i, dp]),
        "qcs_cuda_sample": (i, [vp, dp, i, llp]),
        "qcs_cuda_plan": (i, [vp, i, i, i, ip, ip, ip]),
        "qcs_cuda_profile_enable": (i, [vp, i]),
        "qcs_cuda_profile_read": (i, [vp, i, llp, dp, dp]),
        "qcs_cuda_launch_count": (i, [vp, llp]),
        "qcs_cuda_event_record": (i, [vp, vpp]),
        "qcs_cuda_event_elapsed": (i, [vp, vp, dp]),
        "qcs_cuda_event_destroy": (i, [vp]),
        "qcs_cuda_sample_noalloc": (i, [vp, ll, i, vp, i, vp, vp]),
        "qcs_cuda_batch_create": (i, [i, ip, ip, vp, i, C.c_ulonglong, vpp]),
        "qcs_cuda_batch_destroy": (i, [vp]),
        "qcs_cuda_batch_set_angles": (i, [vp, dp]),
        "qcs_cuda_batch_run": (i, [vp, dp, llp, dp]),
        "qcs_cuda_batch_autotune": (i, [vp, i, ip]),
        "qcs_cuda_batch_config": (i, [vp, i, i, i, i]),
        "qcs_cuda_batch_schedule": (i, [vp, ip]),
        "qcs_cuda_batch_split": (i, [vp, i]),
        "qcs_cuda_batch_traffic": (i, [vp, dp]),
        "qcs_cuda_costmodel_create": (i, [i, C.c_ulonglong, vpp]),
        "qcs_cuda_costmodel_destroy": (i, [vp]),
        "qcs_cuda_costmodel_num_params": (i, [vp, ip]),
        "qcs_cuda_costmodel_get_params": (i, [vp, fp]),
        "qcs_cuda_costmodel_set_params": (i, [vp, fp, i]),
        "qcs_cuda_costmodel_loss_grad": (i, [vp, fp, fp, i, dp, fp]),
        "qcs_cuda_costmodel_train": (i, [vp, fp, fp, i, i, i, C.c_float, dp]),
        "qcs_cuda_costmodel_predict": (i, [vp, fp, i, fp]),
        "qcs_cuda_costmodel_predict_host": (i, [vp, fp, i, fp]),
        "qcs_cuda_item_features": (i, [i, i, i, ip, i, fp]),
        "qcs_cuda_collect_timings": (i, [vp, vp, i, i, i, fp, fp, i, ip]),
        "qcs_cuda_state_set_costmodel": (i, [vp, vp]),
        "qcs_cuda_plan_learned": (i, [vp, i, i, i, vp, ip, ip, ip, dp, dp, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


# Every symbol include/qcs_cuda.h, include/qcs.h and include/qcs_ext.h declare.
def declared_symbols() -> list:
    import re
    names = []
    inc = os.path.join(os.path.dirname(PKG), "include")
    for h in ("qcs_cuda.h", "qcs.h", "qcs_ext.h"):
        src = open(os.path.join(inc, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(q[a-z_0-9]+)\s*\(", src)
    return sorted(set(n for n in names if n.startswith(("qc_", "qcs_"))))


def _check(rc: int):
    if rc != OK:
        msg = lib().qcs_cuda_last_error().decode(errors="replace")
        raise QcsCudaError(rc, msg)


def device_count() -> int:
    c = C.c_int(0)
    lib().qcs_cuda_device_count(C.byref(c))
    return c.value


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class State:
    """One device state vector (include/qcs_cuda.h)."""

    def __init__(self, n: int, precision: int = C64, semantics: int = PHYSICAL):
        self.n = n
        self.precision = precision
        self.semantics = semantics
        h = C.c_void_p()
        _check(lib().qcs_cuda_state_create(n, precision, semantics, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().qcs_cuda_state_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def size(self) -> int:
        return 1 << self.n

    def stream(self) -> int:
        p = C.c_void_p()
        _check(lib().qcs_cuda_state_stream(self._h, C.byref(p)))
        return p.value or 0

    def device_ptr(self) -> int:
        p = C.c_void_p()
        _check(lib().qcs_cuda_state_device_ptr(self._h, C.byref(p)))
        return p.value or 0

    def synchronize(self):
        _check(lib().qcs_cuda_synchronize(self._h))

    def set_basis(self, index: int):
        _check(lib().qcs_cuda_set_basis(self._h, index))

    def amplitudes(self, first: int = 0, count: int | None = None) -> np.ndarray:
        if count is None:
            count = self.size - first
        out = np.zeros(2 * count, dtype=np.float64)
        _check(lib().qcs_cuda_read_amplitudes(self._h, first, count, _dp(out)))
        return out.view(np.complex128)

    def set_amplitudes(self, amps: np.ndarray, first: int = 0):
        a = np.ascontiguousarray(amps, dtype=np.complex128).view(np.float64)
        _check(lib().qcs_cuda_write_amplitudes(self._h, first, len(a) // 2, _dp(a)))

    def apply_1q(self, m, target: int):
        m = np.ascontiguousarray(m, dtype=np.float64)
        _check(lib().qcs_cuda_apply_1q(self._h, _dp(m), target))

    def apply_controlled(self, m, control: int, target: int):
        m = np.ascontiguousarray(m, dtype=np.float64)
        _check(lib().qcs_cuda_apply_controlled_1q(self._h, _dp(m), control, target))

    def apply_gate(self, kind: int, target: int, control: int = -1, angle: float = 0.0):
        _check(lib().qcs_cuda_apply_gate(self._h, kind, target, control, angle))

    def apply_block(self, qubits, u: np.ndarray, engine: int = FUSE_AUTO):
        q = np.ascontiguousarray(qubits, dtype=np.int32)
        uu = np.ascontiguousarray(u, dtype=np.complex128).view(np.float64)
        _check(lib().qcs_cuda_apply_block(self._h, len(q), q.ctypes.data_as(C.POINTER(C.c_int)),
                                          _dp(uu), engine))

    def phase_flip(self, index: int):
        _check(lib().qcs_cuda_phase_flip(self._h, index))

    def diffusion(self):
        _check(lib().qcs_cuda_diffusion(self._h))

    def run(self, gates, fusion_k: int = 0, engine: int = FUSE_AUTO,
            partitioner: int = PARTITION_GREEDY, plan_cache: bool = True):
        ops = gates.ops() if isinstance(gates, W.GateList) else np.ascontiguousarray(gates)
        assert ops.dtype == W.OP_DTYPE
        opt = RunOptions(fusion_k, engine, partitioner, 0 if plan_cache else RUN_NO_PLAN_CACHE)
        _check(lib().qcs_cuda_run(self._h, ops.ctypes.data_as(C.c_void_p), len(ops),
                                  C.byref(opt)))

    def transfer_bytes(self):
        """(host->device, device->host) bytes moved for this state so far."""
        a, b = C.c_longlong(), C.c_longlong()
        _check(lib().qcs_cuda_transfer_bytes(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def norm_sq(self) -> float:
        x = C.c_double()
        _check(lib().qcs_cuda_norm_sq(self._h, C.byref(x)))
        return x.value

    def normalize(self):
        _check(lib().qcs_cuda_normalize(self._h))

    def prob_zero(self, q: int) -> float:
        x = C.c_double()
        _check(lib().qcs_cuda_prob_zero(self._h, q, C.byref(x)))
        return x.value

    def measure(self, q: int, r: float) -> int:
        o = C.c_int()
        _check(lib().qcs_cuda_measure(self._h, q, r, C.byref(o)))
        return o.value

    def probability(self, index: int) -> float:
        x = C.c_double()
        _check(lib().qcs_cuda_probability(self._h, index, C.byref(x)))
        return x.value

    def argmax(self) -> int:
        i = C.c_longlong()
        _check(lib().qcs_cuda_argmax(self._h, C.byref(i), None))
        return i.value

    def expect_z(self, q: int) -> float:
        x = C.c_double()
        _check(lib().qcs_cuda_expect_z(self._h, q, C.byref(x)))
        return x.value

    def profile(self, enable: bool = True):
        _check(lib().qcs_cuda_profile_enable(self._h, 1 if enable else 0))

    def profile_read(self) -> dict:
        """{class: (launches, device ms, algorithmic bytes)} since profile()."""
        out = {}
        for cls, name in enumerate(KCLASS_NAMES):
            n, ms, b = C.c_longlong(), C.c_double(), C.c_double()
            _check(lib().qcs_cuda_profile_read(self._h, cls, C.byref(n), C.byref(ms),
                                               C.byref(b)))
            if n.value:
                out[name] = (n.value, ms.value, b.value)
        return out

    def event(self):
        """Record a CUDA event on this state's stream (an opaque handle)."""
        e = C.c_void_p()
        _check(lib().qcs_cuda_event_record(self._h, C.byref(e)))
        return e

    @staticmethod
    def elapsed_ms(start, stop) -> float:
        ms = C.c_double()
        _check(lib().qcs_cuda_event_elapsed(start, stop, C.byref(ms)))
        lib().qcs_cuda_event_destroy(start)
        lib().qcs_cuda_event_destroy(stop)
        return ms.value

    def set_costmodel(self, model):
        _check(lib().qcs_cuda_state_set_costmodel(self._h, model.handle if model else None))

    def launch_count(self) -> int:
        n = C.c_longlong()
        _check(lib().qcs_cuda_launch_count(self._h, C.byref(n)))
        return n.value

    def sample(self, draws: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(draws, dtype=np.float64)
        out = np.zeros(len(r), dtype=np.int64)
        _check(lib().qcs_cuda_sample(self._h, _dp(r), len(r),
                                     out.ctypes.data_as(C.POINTER(C.c_longlong))))
        return out


def plan(gates, n: int, kmax: int):
    """(order, item, num_items) of the fused execution plan (host only)."""
    ops = gates.ops() if isinstance(gates, W.GateList) else np.ascontiguousarray(gates)
    order = np.zeros(len(ops), dtype=np.int32)
    item = np.zeros(len(ops), dtype=np.int32)
    cnt = C.c_int(0)
    ipp = C.POINTER(C.c_int)
    _check(lib().qcs_cuda_plan(ops.ctypes.data_as(C.c_void_p), len(ops), n, kmax,
                               order.ctypes.data_as(ipp), item.ctypes.data_as(ipp),
                               C.byref(cnt)))
    return order, item, cnt.value


class Batch:
    """Many circuits in one persistent kernel (qcs_cuda_batch_*)."""

    def __init__(self, instances, shots: int = 1024, seed: int = 1):
        """instances: list of (num_qubits, GateList)."""
        self.count = len(instances)
        self.shots = shots
        nq = np.array([n for n, _ in instances], dtype=np.int32)
        offs = np.zeros(self.count + 1, dtype=np.int32)
        chunks = []
        for i, (_, g) in enumerate(instances):
            ops = g.ops()
            chunks.append(ops)
            offs[i + 1] = offs[i] + len(ops)
        self.ops = np.concatenate(chunks) if chunks else np.zeros(0, dtype=W.OP_DTYPE)
        h = C.c_void_p()
        ipp = C.POINTER(C.c_int)
        _check(lib().qcs_cuda_batch_create(self.count, nq.ctypes.data_as(ipp),
                                           offs.ctypes.data_as(ipp),
                                           self.ops.ctypes.data_as(C.c_void_p), shots,
                                           C.c_ulonglong(seed), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().qcs_cuda_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, want_samples: bool = True):
        """(<Z_0> per instance, samples [count, shots] or None, device ms)."""
        z = np.zeros(self.count, dtype=np.float64)
        samples = np.zeros((self.count, self.shots), dtype=np.int64) if want_samples else None
        ms = C.c_double()
        _check(lib().qcs_cuda_batch_run(
            self._h, _dp(z),
            samples.ctypes.data_as(C.POINTER(C.c_longlong)) if samples is not None else None,
            C.byref(ms)))
        return z, samples, ms.value

    def set_angles(self, angles: np.ndarray):
        a = np.ascontiguousarray(angles, dtype=np.float64)
        assert len(a) == len(self.ops)
        _check(lib().qcs_cuda_batch_set_angles(self._h, _dp(a)))

    def autotune(self, repeats: int = 2):
        out = (C.c_int * 4)()
        _check(lib().qcs_cuda_batch_autotune(self._h, repeats, out))
        return self.schedule()

    def schedule(self):
        out = (C.c_int * 5)()
        _check(lib().qcs_cuda_batch_schedule(self._h, out))
        return {"threads": out[0], "tile_q": out[1], "ctas_per_sm": out[2],
                "order": "largest-first" if out[3] == 0 else "given",
                "split_q": out[4]}

    def config(self, threads: int, tile_q: int, ctas_per_sm: int, order: int = 0):
        _check(lib().qcs_cuda_batch_config(self._h, threads, tile_q, ctas_per_sm, order))

    def traffic(self) -> float:
        """Algorithmic HBM bytes of one run (qcs_cuda_batch_traffic)."""
        out = C.c_double()
        _check(lib().qcs_cuda_batch_traffic(self._h, C.byref(out)))
        return out.value

    def split(self, split_q: int):
        _check(lib().qcs_cuda_batch_split(self._h, split_q))


COSTMODEL_FEATURES = 20


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class CostModel:
    """The learned fusion cost model (qcs_cuda_costmodel_*)."""

    def __init__(self, seed: int = 1, features: int = COSTMODEL_FEATURES):
        self.F = features
        h = C.c_void_p()
        _check(lib().qcs_cuda_costmodel_create(features, C.c_ulonglong(seed), C.byref(h)))
        self._h = h
        n = C.c_int()
        _check(lib().qcs_cuda_costmodel_num_params(h, C.byref(n)))
        self.num_params = n.value

    def close(self):
        if getattr(self, "_h", None):
            lib().qcs_cuda_costmodel_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, dtype=np.float32)
        _check(lib().qcs_cuda_costmodel_get_params(self._h, _fp(out)))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().qcs_cuda_costmodel_set_params(self._h, _fp(p), len(p)))

    def loss_grad(self, x: np.ndarray, y: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_double()
        _check(lib().qcs_cuda_costmodel_loss_grad(self._h, _fp(x), _fp(y), len(y), C.byref(loss),
                                                  _fp(g)))
        return loss.value, g

    def train(self, x, y, epochs=30, batch=256, lr=1e-3) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_double()
        _check(lib().qcs_cuda_costmodel_train(self._h, _fp(x), _fp(y), len(y), epochs, batch,
                                              C.c_float(lr), C.byref(loss)))
        return loss.value

    def predict(self, x, host: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros(len(x), dtype=np.float32)
        f = lib().qcs_cuda_costmodel_predict_host if host else lib().qcs_cuda_costmodel_predict
        _check(f(self._h, _fp(x), len(x), _fp(out)))
        return out


def collect_timings(state: "State", gates, kmax: int, engine: int = FUSE_AUTO, max_items=100000):
    """(features [m, F], device ms [m]) of every plan item of `gates`."""
    ops = gates.ops() if isinstance(gates, W.GateList) else np.ascontiguousarray(gates)
    feats = np.zeros((max_items, COSTMODEL_FEATURES), dtype=np.float32)
    ms = np.zeros(max_items, dtype=np.float32)
    n = C.c_int()
    _check(lib().qcs_cuda_collect_timings(state.handle, ops.ctypes.data_as(C.c_void_p), len(ops),
                                          kmax, engine, _fp(feats), _fp(ms), max_items,
                                          C.byref(n)))
    return feats[:n.value], ms[:n.value]


def plan_learned(gates, n: int, kmax: int, model: CostModel):
    ops = gates.ops() if isinstance(gates, W.GateList) else np.ascontiguousarray(gates)
    order = np.zeros(len(ops), dtype=np.int32)
    item = np.zeros(len(ops), dtype=np.int32)
    cnt = C.c_int()
    pred, greedy = C.c_double(), C.c_double()
    choice = C.c_int()
    ipp = C.POINTER(C.c_int)
    _check(lib().qcs_cuda_plan_learned(ops.ctypes.data_as(C.c_void_p), len(ops), n, kmax,
                                       model.handle, order.ctypes.data_as(ipp),
                                       item.ctypes.data_as(ipp), C.byref(cnt), C.byref(pred),
                                       C.byref(greedy), C.byref(choice)))
    return {"order": order, "item": item, "items": cnt.value, "pred_ms": pred.value,
            "greedy_pred_ms": greedy.value, "choice": choice.value}


_api = None


def api() -> C.CDLL:
    """The library with the qc_* (include/qcs.h, include/qcs_ext.h) signatures."""
    global _api
    if _api is None:
        L = lib()
        vp, i, d, ll = C.c_void_p, C.c_int, C.c_double, C.c_longlong
        ip, llp = C.POINTER(C.c_int), C.POINTER(C.c_longlong)
        sig = {
            "qc_create": (vp, [i]),
            "qc_create_ex": (vp, [i, i, i, i]),
            "qc_destroy": (None, [vp]),
            "qc_h": (None, [vp, i]), "qc_x": (None, [vp, i]),
            "qc_y": (None, [vp, i]), "qc_z": (None, [vp, i]),
            "qc_cnot": (None, [vp, i, i]),
            "qc_cphase": (None, [vp, i, i, d]),
            "qc_phase": (None, [vp, i, d]), "qc_rx": (None, [vp, i, d]),
            "qc_ry": (None, [vp, i, d]), "qc_rz": (None, [vp, i, d]),
            "qc_barrier": (None, [vp]), "qc_reset": (None, [vp, i]),
            "qc_measure": (i, [vp, i]), "qc_measure_all": (None, [vp, ip]),
            "qc_run": (None, [vp]), "qc_run_shots": (None, [vp, i, ip]),
            "qc_find_most_likely_state": (i, [vp]),
            "qc_get_probability": (d, [vp, i]),
            "qc_print_state": (None, [vp, i]), "qc_print_circuit": (None, [vp]),
            "qc_grover_search": (None, [vp, i]),
            "qc_quantum_fourier_transform": (None, [vp]),
            "qc_bernstein_vazirani": (None, [vp, i]),
            "qc_ghz_state": (None, [vp]),
            "qc_get_num_qubits": (i, [vp]), "qc_get_num_gates": (i, [vp]),
            "qc_optimize": (None, [vp]),
            "qc_get_probability64": (d, [vp, ll]),
            "qc_find_most_likely_state64": (ll, [vp]),
            "qc_set_basis": (None, [vp, ll]),
            "qc_sample_shots": (i, [vp, i, llp]),
            "qc_expect_z": (d, [vp, i]),
            "qc_flush": (None, [vp]),
            "qc_cuda_state": (vp, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _api = L
    return _api


def libc() -> C.CDLL:
    """The C library whose rand()/srand() qc_measure and qc_run_shots draw from."""
    L = C.CDLL(None)
    L.rand.restype = C.c_int
    L.srand.argtypes = [C.c_uint]
    L.fflush.argtypes = [C.c_void_p]
    return L
