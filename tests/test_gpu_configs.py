"""Parity at the sizes of the benchmark configurations, against the oracle.

* 20 qubits, complex128: a seeded random basis state, the reference's QFT
  (src/qcs.c:443-457), then 200 seeded random gates (70 % one-qubit gates
  from {H, X, Y, Z, RX, RY, RZ, P}, 30 % CNOT), one kernel per gate
  (src/q_gates.c:25-298).  REFERENCE semantics must equal the oracle's COMPAT
  mode (the reference's own sequential rule) bit for bit over the whole
  vector, and PHYSICAL semantics the oracle's physical mode.
* 28 qubits, complex64: qc_grover_search's structure (src/qcs.c:402-419) --
  one Hadamard layer, then 64 x (phase flip on a seeded marked index,
  diffusion) -- fused into 7-qubit tensor-core blocks.  The argmax must be
  the FP64 oracle's, and the marked probability within 1e-5 relative.
* Batched variational instances with the configured ranges, n ~ U[10, 22]
  and depth ~ U[4, 16] layers: <Z_0> of every instance within 1e-5 of the
  per-instance FP64 oracle, and every shot histogram through a chi-square
  test at p > 0.01.  Instances above the shared-memory tile run from global
  slots in cache-blocked stages; the batch holds several of 20-22 qubits.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qcs_gb300 import capi
from qcs_gb300 import workloads as W
from tests.helpers import bits_equal
from tests.test_gpu_batch import chi2_pvalue

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [2026, 7])
def test_c1_random20_c128_bitexact(seed):
    n = 20
    basis, g = W.random_circuit(n, seed, 200)
    full = W.basis_gates(n, basis)
    full.extend(g)
    assert len(full) >= 200 + n * (n + 1) // 2
    for sem, mode in ((capi.REFERENCE, O.COMPAT), (capi.PHYSICAL, O.PHYSICAL)):
        with capi.State(n, capi.C128, sem) as s, O.OracleState(n, mode) as o:
            s.run(full)
            o.run(full)
            a, b = s.amplitudes(), o.amplitudes()
            assert bits_equal(a, b), (sem, int(np.sum(a != b)))
            assert s.argmax() == o.argmax()


def test_c3_search_argmax_28q():
    n = 28
    w = W.grover_workload(n, 2026, iterations=64)
    with O.OracleState(n) as o:
        o.run(w.search)
        o_arg, o_p = o.argmax(), o.probability(w.marked)
    assert o_arg == w.marked  # the marked index dominates this form
    for k in (7, 0):  # fused into 7-qubit tensor-core blocks, and plain
        with capi.State(n, capi.C64) as s:
            s.run(w.search.ops(), fusion_k=k)
            g_arg, g_p = s.argmax(), s.probability(w.marked)
        assert g_arg == o_arg, (k, g_arg, o_arg)
        assert abs(g_p - o_p) <= 1e-5 * o_p, (k, g_p, o_p)


def test_batch_config_ranges():
    inst = W.variational_batch(256, seed=2026)  # n ~ U[10, 22], depth ~ U[4, 16]
    ns = np.array([n for n, _ in inst])
    assert ns.min() >= 10 and ns.max() <= 22
    assert np.sum(ns >= 20) >= 20  # instances on the global-slot path
    with capi.Batch(inst, shots=1024, seed=11) as b:
        z, samples, _ = b.run()
        tile_q = b.schedule()["tile_q"]
    assert np.sum(ns > tile_q) >= 100
    pvals = []
    for i, (n, g) in enumerate(inst):
        with O.OracleState(n) as o:
            o.run(g)
            zo = o.expect_z(0)
            probs = np.abs(o.amplitudes()) ** 2
        assert abs(z[i] - zo) < 1e-5, (i, n, z[i], zo)
        assert samples[i].min() >= 0 and samples[i].max() < (1 << n)
        pvals.append(chi2_pvalue(np.bincount(samples[i], minlength=1 << n), probs))
    # p > 0.01 per instance; ~1 % of 256 fail by chance, so allow up to 8
    assert sum(p <= 0.01 for p in pvals) <= 8, sorted(pvals)[:10]
