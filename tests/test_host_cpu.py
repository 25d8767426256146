"""Host-side tests of libqcs_gb300.so that need no GPU.

* the library loads and exports every function include/*.h declares;
* without a device every state-creating call fails loudly (no CPU fallback);
* the fusion planner (qcs_cuda_plan) yields a valid reordering: replaying
  the ops in plan order on the oracle gives the original state, and every
  block respects the width limit;
* the workload generators are deterministic.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from qcs_gb300 import capi
from qcs_gb300 import workloads as W


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    syms = capi.declared_symbols()
    assert len(syms) > 50
    missing = [s for s in syms if not hasattr(L, s)]
    assert missing == []


def test_gate_kind_numbering_matches_oracle():
    assert (W.H, W.X, W.Y, W.Z, W.P, W.RX, W.RY, W.RZ, W.CNOT, W.CPHASE) == tuple(range(10))
    assert W.OP_DTYPE.itemsize == 32


@pytest.mark.skipif(capi.device_count() > 0, reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly():
    with pytest.raises(capi.QcsCudaError) as e:
        capi.State(4)
    assert e.value.status == capi.ENODEV
    assert capi.api().qc_create(3) is None


def test_invalid_arguments_rejected_before_any_device_work():
    L = capi.lib()
    h = C.c_void_p()
    assert L.qcs_cuda_state_create(0, 0, 0, C.byref(h)) == capi.EINVAL
    assert L.qcs_cuda_state_create(40, 0, 0, C.byref(h)) == capi.EINVAL
    assert L.qcs_cuda_state_create(4, 7, 0, C.byref(h)) == capi.EINVAL
    assert L.qcs_cuda_state_create(4, 0, 9, C.byref(h)) == capi.EINVAL
    assert L.qcs_cuda_apply_gate(None, 0, 0, -1, 0.0) == capi.EINVAL
    assert L.qcs_cuda_strerror(capi.ENODEV) == b"no usable CUDA device"


def test_debug_inject_arguments():
    L = capi.lib()
    assert L.qcs_cuda_debug_inject(1, 2) == capi.OK
    assert L.qcs_cuda_debug_inject(5, 1) == capi.EINVAL
    assert L.qcs_cuda_debug_inject(0, 0) == capi.OK


def test_debug_wait_limit_arguments():
    L = capi.lib()
    assert L.qcs_cuda_debug_set_wait_cycles(-1) == capi.EINVAL
    assert L.qcs_cuda_debug_set_wait_cycles(1000) == capi.OK
    assert L.qcs_cuda_debug_set_wait_cycles(0) == capi.OK  # back to the default


def _replay(n, gates, order):
    ops = gates.ops()[order]
    g = W.GateList()
    for o in ops:
        g.add(int(o["kind"]), int(o["target"]), int(o["control"]), float(o["angle"]),
              int(o["index"]))
    with O.OracleState(n) as s:
        s.run(g)
        return s.amplitudes()


@pytest.mark.parametrize("kmax", [2, 3, 4, 5, 6, 7])
def test_plan_is_a_valid_reordering(kmax):
    n = 9
    basis, g = W.random_circuit(n, 31 + kmax, 150)
    order, item, nitems = capi.plan(g, n, kmax)
    assert sorted(order) == list(range(len(g)))
    with O.OracleState(n) as s:
        s.run(g)
        ref = s.amplitudes()
    np.testing.assert_allclose(_replay(n, g, order), ref, atol=1e-12)
    ops = g.ops()
    for it in range(nitems):
        sel = order[item == it]
        qs = set()
        for o in ops[sel]:
            qs.add(int(o["target"]))
            if o["kind"] in (W.CNOT, W.CPHASE):
                qs.add(int(o["control"]))
        assert len(qs) <= kmax
    # items are contiguous in the order
    assert np.all(np.diff(item) >= 0)


def test_plan_keeps_non_gate_ops_as_barriers():
    n = 6
    w = W.grover_workload(n, 3, iterations=3)
    g = w.qft
    g.extend(w.rounds)
    order, item, nitems = capi.plan(g, n, 4)
    kinds = g.ops()["kind"][order]
    flips = np.nonzero(kinds == W.PHASE_FLIP)[0]
    for f in flips:
        assert np.sum(item == item[f]) == 1  # alone in its item
    # non-gate ops keep their relative order
    ng = [i for i in order if g.kinds[i] >= W.PHASE_FLIP]
    assert ng == sorted(ng)


def test_plan_block_counts_brick30():
    """Wider blocks mean fewer passes over the state; width 7 (the widest the
    tensor cores take) plans the headline circuit in 51 blocks against 63 at
    width 6, and the planner caps wider requests at 7."""
    g = W.brick_circuit(30, 40, 1)
    counts = [capi.plan(g, 30, k)[2] for k in (2, 4, 6, 7, 8)]
    assert counts[0] > counts[1] > counts[2] > counts[3] == counts[4]
    assert counts[1] * 10 < len(g)
    assert counts[2:4] == [63, 51]


def test_workloads_are_deterministic():
    a = W.brick_circuit(10, 4, 5).ops()
    b = W.brick_circuit(10, 4, 5).ops()
    assert np.array_equal(a, b)
    b1, g1 = W.random_circuit(20, 1)
    b2, g2 = W.random_circuit(20, 1)
    assert b1 == b2 and np.array_equal(g1.ops(), g2.ops())
    assert len(W.qft_gates(20)) == 20 * 21 // 2
    # the configured mix: ~70 % one-qubit gates
    _, g = W.random_circuit(12, 9, 2000, with_qft=False)
    frac = np.mean(np.array(g.kinds) != W.CNOT)
    assert 0.66 < frac < 0.74
