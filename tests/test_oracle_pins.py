"""Pins of the CPU oracle (oracle/qcs_oracle.c) -- CPU only.

The oracle is the checker of every GPU parity test, so it is pinned first:
  * against golden vectors produced by the reference's own sequential build
    (tests/golden/make_golden.py), bit for bit in compat mode and on
    one-qubit-gate circuits in physical mode;
  * against an independent numpy model of the physical semantics;
  * against the reference library itself where oracle/_ref was built here;
  * against the known answers of the reference's test suite (test/*.c).
"""
import numpy as np
import pytest

from oracle import oracle as O
from qcs_gb300 import workloads as W
from tests.helpers import bits_equal, gates_from


def run_oracle(n, gates, mode):
    with O.OracleState(n, mode) as s:
        s.run(gates)
        return s.amplitudes()


def test_one_qubit_circuit_bitexact_both_modes(golden):
    d = golden("ref_1q_n10")
    g = gates_from(d)
    for mode in (O.PHYSICAL, O.COMPAT):
        assert bits_equal(run_oracle(10, g, mode), d["ref"])


@pytest.mark.parametrize("name", ["ref_mixed_n10_s0", "ref_mixed_n10_s1", "ref_random_n12"])
def test_compat_bitexact_vs_reference(golden, name):
    d = golden(name)
    n = int(d["n"])
    g = gates_from(d)
    assert bits_equal(run_oracle(n, g, O.COMPAT), d["ref"])


@pytest.mark.parametrize("name", ["ref_mixed_n10_s0", "ref_mixed_n10_s1", "ref_random_n12"])
def test_physical_matches_numpy(golden, name):
    d = golden(name)
    n = int(d["n"])
    a = run_oracle(n, gates_from(d), O.PHYSICAL)
    np.testing.assert_allclose(a, d["physical"], rtol=0, atol=1e-12)
    assert abs(np.vdot(a, a).real - 1.0) < 1e-12


def test_grover_compat_reproduces_reference_quirk(golden):
    d = golden("ref_grover_n6")
    with O.OracleState(6, O.COMPAT) as s:
        s.grover(42)
        assert bits_equal(s.amplitudes(), d["ref"])
        assert s.probability(42) == float(d["ref_prob"]) == 17.015625
    with O.OracleState(6, O.PHYSICAL) as s:
        s.grover(42)
        np.testing.assert_allclose(s.amplitudes(), d["physical"], atol=1e-12)
        assert s.probability(42) > 0.99


def test_measure_sequence(golden):
    d = golden("ref_measure_n5")
    with O.OracleState(5, O.COMPAT) as s:
        s.run(gates_from(d))
        outs = [s.measure(int(q), float(r)) for q, r in zip(d["qubits"], d["draws"])]
        assert outs == list(d["outcomes"])
        assert bits_equal(s.amplitudes(), d["ref"])


def test_shots_histogram(golden):
    d = golden("ref_shots_n5")
    with O.OracleState(5, O.PHYSICAL) as s:
        s.run(gates_from(d))
        idx = s.sample(d["draws"])
    hist = np.bincount(idx[idx >= 0], minlength=32)
    assert np.array_equal(hist, d["hist"])


def test_bernstein_vazirani(golden):
    d = golden("ref_bv_n6")
    ref_hits = 0
    for secret, ref_arg in zip(d["secrets"], d["ref_argmax"]):
        g = W.GateList()
        n = 5
        g.add(W.X, n)
        g.add(W.H, n)
        for i in range(n):
            g.add(W.H, i)
        for i in range(n):
            if (secret >> i) & 1:
                g.add(W.CNOT, n, i)
        for i in range(n):
            g.add(W.H, i)
        with O.OracleState(6, O.COMPAT) as s:
            s.run(g)
            assert s.argmax() == ref_arg
        with O.OracleState(6, O.PHYSICAL) as s:
            s.run(g)
            assert s.argmax() & 31 == secret  # ancilla in |->: secret in bits 0..4
        ref_hits += int(ref_arg == secret)
    assert ref_hits == 6  # the reference recovers 6 of 32 secrets


def test_reference_test_suite_known_answers(golden):
    """test/test_qc_*.c assertions, evaluated on the oracle."""
    ka = golden("ref_known_answers")
    # test_qc_cnot.c:10 expects 3; the reference's own sweep gives 0
    with O.OracleState(2, O.COMPAT) as s:
        s.apply_gate(W.X, 0)
        s.apply_gate(W.CNOT, 1, 0)
        assert s.argmax() == int(ka["cnot_argmax"]) == 0
    with O.OracleState(2, O.PHYSICAL) as s:
        s.apply_gate(W.X, 0)
        s.apply_gate(W.CNOT, 1, 0)
        assert s.argmax() == 3
    # test_qc_qft.c:12-14 (uniform 1/8)
    for mode in (O.PHYSICAL, O.COMPAT):
        with O.OracleState(3, mode) as s:
            s.qft()
            p = [s.probability(i) for i in range(8)]
            np.testing.assert_allclose(p, ka["qft3_probs"], atol=1e-6)
    # test_qc_h.c:12-13, test_qc_x/y/z/phase/rotations
    with O.OracleState(1, O.PHYSICAL) as s:
        s.apply_gate(W.H, 0)
        assert abs(s.probability(0) - 0.5) < 1e-6 and abs(s.probability(1) - 0.5) < 1e-6
    with O.OracleState(1, O.PHYSICAL) as s:
        s.apply_gate(W.X, 0)
        s.apply_gate(W.P, 0, -1, np.pi)
        assert s.argmax() == 1
    with O.OracleState(1, O.PHYSICAL) as s:
        s.apply_gate(W.RX, 0, -1, np.pi)
        assert s.argmax() == 1
        s.apply_gate(W.RY, 0, -1, np.pi)
        assert s.argmax() == 0
        s.apply_gate(W.H, 0)
        s.apply_gate(W.RZ, 0, -1, np.pi)
        s.apply_gate(W.H, 0)
        assert s.argmax() == 1


def test_block_apply_matches_gates():
    rng = np.random.default_rng(5)
    n = 8
    g = W.brick_circuit(n, 2, 11)
    with O.OracleState(n) as a, O.OracleState(n) as b:
        a.run(g)
        # the same circuit as one dense block on all qubits (numpy-built)
        from tests.golden.make_golden import np_run
        u = np.stack([np_run(n, g, psi=np.eye(1 << n, dtype=complex)[:, j]) for j in range(1 << n)],
                     axis=1)
        b.apply_block(list(range(n)), u)
        np.testing.assert_allclose(a.amplitudes(), b.amplitudes(), atol=1e-12)
    del rng


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_compat_bitexact_vs_reference_library_live():
    for seed in range(3):
        basis, g0 = W.random_circuit(9, 100 + seed, 250)
        g = W.basis_gates(9, basis)
        g.extend(g0)
        r = O.RefCircuit(9)
        r.run(g)
        a = r.amplitudes()
        r.close()
        assert bits_equal(run_oracle(9, g, O.COMPAT), a)


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_grover_bitexact_vs_reference_library_live():
    for n, sol in ((4, 5), (5, 17), (7, 100)):
        r = O.RefCircuit(n)
        r.L.qc_grover_search(r._h, sol)
        a = r.amplitudes()
        r.close()
        with O.OracleState(n, O.COMPAT) as s:
            s.grover(sol)
            assert bits_equal(s.amplitudes(), a)
