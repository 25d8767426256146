"""Bounded device-side waits made to run out (qcs_cuda_debug_set_wait_cycles).

A wait limit of a few hundred clock cycles makes the handoff waits of the
tensor-core pipelines, and the CTA-group counters of the batched kernel,
give up almost at once.  Each test checks that
* the call that launched the kernel returns and the next synchronize (or
  batch run) reports QCS_CUDA_ETIMEOUT from the device error flag;
* the aborted kernel left cleanly: with the default limit restored, the same
  kernel runs again on the same GPU -- a tensor-core launch could not
  allocate its tensor memory had the aborted one kept its columns -- and its
  result equals the oracle's (or, for batches, the earlier run's bits);
* reporting the timeout cleared the flag.
Nothing here faults, traps or waits without a limit: every wait in these
kernels is bounded, and the final drain of issued MMAs keeps the default
limit whatever the override.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qcs_gb300 import capi
from qcs_gb300 import workloads as W
from tests.helpers import infidelity

pytestmark = pytest.mark.gpu

SHORT = 200  # clock cycles: ~0.1 us


def _set_wait(cycles):
    assert capi.lib().qcs_cuda_debug_set_wait_cycles(cycles) == capi.OK


@pytest.mark.parametrize("k", [6, 7])
@pytest.mark.parametrize("placement", ["col", "low"])
def test_tensor_core_waits_run_out_and_the_kernel_recovers(k, placement):
    n = 20
    rng = np.random.default_rng(10 * k + len(placement))
    qubits = (list(range(k)) if placement == "low"
              else [int(q) for q in rng.choice(range(1, n), size=k, replace=False)])
    K = 1 << k
    u, _ = np.linalg.qr(rng.normal(size=(K, K)) + 1j * rng.normal(size=(K, K)))
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    with capi.State(n, capi.C64) as s:
        s.set_amplitudes(init)
        s.synchronize()
        try:
            _set_wait(SHORT)
            s.apply_block(qubits, u, capi.FUSE_TENSOR)  # the launch itself succeeds
            with pytest.raises(capi.QcsCudaError) as e:
                s.synchronize()
            assert e.value.status == capi.ETIMEOUT
        finally:
            _set_wait(0)
        s.synchronize()  # the report cleared the flag
        s.set_amplitudes(init)
        s.apply_block(qubits, u, capi.FUSE_TENSOR)
        s.synchronize()
        a = s.amplitudes()
    with O.OracleState(n) as o:
        o.set_amplitudes(init)
        o.apply_block(qubits, u)
        b = o.amplitudes()
    assert np.max(np.abs(a - b)) < 5e-5
    assert infidelity(a, b) < 1e-8


def test_batch_group_counter_wait_runs_out_and_the_batch_recovers():
    inst = W.variational_batch(8, seed=12, n_range=(15, 16), depth_range=(3, 4))
    with capi.Batch(inst, shots=64, seed=4) as b:
        b.config(512, 12, 2, 0)
        b.split(12)  # instances of 15-16 qubits on groups of 8-16 CTAs
        z_ref, s_ref, _ = b.run()
        try:
            _set_wait(SHORT)
            with pytest.raises(capi.QcsCudaError) as e:
                b.run()
            assert e.value.status == capi.ETIMEOUT
        finally:
            _set_wait(0)
        z2, s2, _ = b.run()
    assert np.array_equal(z_ref, z2) and np.array_equal(s_ref, s2)
    for i, (n, g) in enumerate(inst[:3]):
        with O.OracleState(n) as o:
            o.run(g)
            assert abs(o.expect_z(0) - z2[i]) < 1e-5
