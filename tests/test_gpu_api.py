"""The reference's test suite (test/test_qc_*.c), restated against the
drop-in public API (include/qcs.h) served by libqcs_gb300.so.

Each test follows the reference test of the same name.  Where the reference's
own sequential build contradicts its test (CNOT, Bernstein-Vazirani, Grover;
its controlled sweep is not unitary), the PHYSICAL backend satisfies the
test's intent and the REFERENCE-semantics backend reproduces what the
reference actually returns.
"""
import ctypes as C
import math

import numpy as np
import pytest

from qcs_gb300 import capi

pytestmark = pytest.mark.gpu

PI = math.pi


@pytest.fixture(scope="module")
def A():
    return capi.api()


@pytest.fixture(scope="module")
def libc():
    return capi.libc()


def close(a, b, tol=1e-6):
    return abs(a - b) < tol


def test_qc_create_destroy(A):
    c = A.qc_create(2)
    assert c
    A.qc_destroy(c)
    assert A.qc_create(0) is None


def test_qc_getters(A):
    c = A.qc_create(4)
    assert A.qc_get_num_qubits(c) == 4
    assert A.qc_get_num_gates(c) == 0
    A.qc_h(c, 0)
    assert A.qc_get_num_gates(c) == 1
    A.qc_destroy(c)


def test_qc_h(A):
    c = A.qc_create(1)
    A.qc_h(c, 0)
    assert close(A.qc_get_probability(c, 0), 0.5)
    assert close(A.qc_get_probability(c, 1), 0.5)
    A.qc_destroy(c)


@pytest.mark.parametrize("prep,expect", [("x", 1), ("y", 0), ("z", 1)])
def test_qc_x_y_z(A, prep, expect):
    c = A.qc_create(1)
    if prep == "x":
        A.qc_x(c, 0)
    elif prep == "y":
        A.qc_x(c, 0)
        A.qc_y(c, 0)
    else:
        A.qc_h(c, 0)
        A.qc_z(c, 0)
        A.qc_h(c, 0)
    assert A.qc_find_most_likely_state(c) == expect
    A.qc_destroy(c)


def test_qc_cnot(A):
    c = A.qc_create(2)
    A.qc_x(c, 0)
    A.qc_cnot(c, 0, 1)
    assert A.qc_find_most_likely_state(c) == 3
    A.qc_destroy(c)


def test_qc_cnot_reference_semantics(A):
    """The reference's sequential build maps this |01> to the zero vector."""
    c = A.qc_create_ex(2, capi.C128, capi.REFERENCE, 0)
    A.qc_x(c, 0)
    A.qc_cnot(c, 0, 1)
    assert A.qc_find_most_likely_state(c) == 0
    assert sum(A.qc_get_probability(c, i) for i in range(4)) == 0.0
    A.qc_destroy(c)


def test_qc_phase(A):
    c = A.qc_create(1)
    A.qc_x(c, 0)
    A.qc_phase(c, 0, PI)
    assert A.qc_find_most_likely_state(c) == 1
    A.qc_destroy(c)


def test_qc_rotations(A):
    c = A.qc_create(1)
    A.qc_rx(c, 0, PI)
    assert A.qc_find_most_likely_state(c) == 1
    A.qc_ry(c, 0, PI)
    assert A.qc_find_most_likely_state(c) == 0
    A.qc_h(c, 0)
    A.qc_rz(c, 0, PI)
    A.qc_h(c, 0)
    assert A.qc_find_most_likely_state(c) == 1
    A.qc_destroy(c)


def test_qc_barrier(A):
    c = A.qc_create(1)
    A.qc_barrier(c)
    assert A.qc_get_num_gates(c) == 1
    A.qc_destroy(c)


def test_qc_reset(A):
    c = A.qc_create(1)
    A.qc_h(c, 0)
    A.qc_reset(c, 0)
    assert A.qc_find_most_likely_state(c) == 0
    assert abs(A.qc_get_probability(c, 0) - 1.0) < 1e-9
    A.qc_destroy(c)


def test_qc_measure(A):
    c = A.qc_create(2)
    res = (C.c_int * 2)()
    A.qc_x(c, 1)
    assert A.qc_measure(c, 0) == 0 and A.qc_measure(c, 1) == 1
    A.qc_measure_all(c, res)
    assert res[0] == 0 and res[1] == 1
    A.qc_destroy(c)


def test_qc_run(A):
    c = A.qc_create(1)
    A.qc_x(c, 0)
    A.qc_run(c)
    assert A.qc_find_most_likely_state(c) == 1
    assert abs(A.qc_get_probability(c, 1) - 1.0) < 1e-9
    A.qc_destroy(c)


def test_qc_run_shots(A, libc):
    libc.srand(2024)
    c = A.qc_create(1)
    res = (C.c_int * 2)()
    A.qc_h(c, 0)
    A.qc_run_shots(c, 1000, res)
    assert res[0] + res[1] == 1000
    assert 400 < res[0] < 600
    A.qc_destroy(c)


def test_qc_run_shots_same_draws_as_reference(A, libc, golden):
    """Same srand seed and state as the golden run of the reference: the
    histogram is identical."""
    d = golden("ref_shots_n5")
    c = A.qc_create_ex(5, capi.C128, capi.PHYSICAL, 0)
    for k, t, a in zip(d["kinds"], d["targets"], d["angles"]):
        if k == 0:
            A.qc_h(c, int(t))
        else:
            A.qc_ry(c, int(t), float(a))
    hist = (C.c_int * 32)()
    libc.srand(int(d["seed"]))
    A.qc_run_shots(c, int(d["shots"]), hist)
    assert list(hist) == list(d["hist"])
    A.qc_destroy(c)


def test_qc_state_access(A):
    c = A.qc_create(2)
    A.qc_h(c, 0)
    assert close(A.qc_get_probability(c, 0), 0.5)
    assert A.qc_find_most_likely_state(c) in (0, 2)
    A.qc_destroy(c)


def test_qc_print(A, capfd):
    c = A.qc_create(1)
    A.qc_h(c, 0)
    A.qc_print_state(c, -1)
    A.qc_print_circuit(c)
    A.qc_destroy(c)
    capi.libc().fflush(None)  # C stdio buffers stdout when it is not a terminal
    out = capfd.readouterr().out
    assert "--- Quantum State (1 Qubits) ---" in out
    assert "|0>: 0.707107 + i0.000000" in out
    assert "QUANTUM CIRCUIT" in out and "GATE SEQUENCE: H(0)" in out


def test_qc_grover_search(A):
    c = A.qc_create(6)
    A.qc_grover_search(c, 42)
    assert A.qc_get_probability(c, 42) > 0.9
    A.qc_destroy(c)


def test_qc_grover_search_reference_semantics(A):
    c = A.qc_create_ex(6, capi.C128, capi.REFERENCE, 0)
    A.qc_grover_search(c, 42)
    assert abs(A.qc_get_probability(c, 42) - 17.015625) < 1e-9
    A.qc_destroy(c)


def test_qc_qft(A):
    c = A.qc_create(3)
    A.qc_quantum_fourier_transform(c)
    for i in range(8):
        assert close(A.qc_get_probability(c, i), 1 / 8)
    A.qc_destroy(c)


@pytest.mark.parametrize("secret", [0, 1, 13, 22, 31])
def test_qc_bv(A, secret):
    c = A.qc_create(6)
    A.qc_bernstein_vazirani(c, secret)
    # the ancilla (qubit 5) ends in |->, so the most likely index carries the
    # secret in bits 0..4 (the reference's test compares the full index)
    assert A.qc_find_most_likely_state(c) & 31 == secret
    A.qc_destroy(c)


def test_qc_bv_reference_semantics_matches_reference(A, golden):
    d = golden("ref_bv_n6")
    for secret, ref_arg in zip(d["secrets"], d["ref_argmax"]):
        c = A.qc_create_ex(6, capi.C128, capi.REFERENCE, 0)
        A.qc_bernstein_vazirani(c, int(secret))
        assert A.qc_find_most_likely_state(c) == ref_arg
        A.qc_destroy(c)


def test_qc_ghz_state(A):
    c = A.qc_create(5)
    A.qc_ghz_state(c)
    assert close(A.qc_get_probability(c, 0), 0.5)
    assert close(A.qc_get_probability(c, 31), 0.5)
    A.qc_destroy(c)


def test_qc_optimize(A):
    c = A.qc_create(2)
    A.qc_h(c, 0)
    A.qc_h(c, 0)
    before = A.qc_get_num_gates(c)
    A.qc_optimize(c)
    assert A.qc_get_num_gates(c) == before - 2
    A.qc_destroy(c)


def test_invalid_gate_arguments_are_reported_and_recorded(A, capfd):
    c = A.qc_create(2)
    A.qc_h(c, 5)
    A.qc_cnot(c, 1, 1)
    err = capfd.readouterr().err
    assert "Invalid arguments for 1-qubit gate application" in err
    assert "Invalid arguments for 2-qubit gate application" in err
    assert A.qc_get_num_gates(c) == 2  # the reference records them anyway
    assert A.qc_find_most_likely_state(c) == 0
    A.qc_destroy(c)


@pytest.mark.parametrize("n,widths", [(8, (0, 4)), (15, (0, 5, 6, 7))])
def test_fusion_mode_same_answers(A, n, widths):
    """The drop-in API gives the same probabilities fused (CUDA cores at 8
    qubits; the tensor cores at 15, up to 7-qubit blocks) as per gate."""
    for k in widths:
        c = A.qc_create_ex(n, capi.C64, capi.PHYSICAL, k)
        A.qc_quantum_fourier_transform(c)
        for q in range(n):
            A.qc_rx(c, q, 0.1 * q)
        A.qc_ghz_state(c)
        for q in range(0, n - 1, 2):
            A.qc_cnot(c, q, q + 1)
            A.qc_ry(c, q + 1, 0.3)
        p = np.array([A.qc_get_probability(c, i) for i in range(1 << n)])
        if k == 0:
            ref = p
        else:
            np.testing.assert_allclose(p, ref, atol=1e-6)
        A.qc_destroy(c)


def test_64bit_extensions(A):
    c = A.qc_create(31)
    A.qc_set_basis(c, (1 << 31) - 5)
    assert A.qc_find_most_likely_state64(c) == (1 << 31) - 5
    assert A.qc_get_probability64(c, (1 << 31) - 5) == 1.0
    samples = (C.c_longlong * 4)()
    assert A.qc_sample_shots(c, 4, samples) == 0
    assert list(samples) == [(1 << 31) - 5] * 4
    A.qc_destroy(c)


def test_transfer_counters():
    """qcs_cuda_transfer_bytes counts what crosses the host/device boundary:
    amplitude writes and reads, shot draws and samples, the 2x2 matrices in
    kernel parameters and the tensor-core block images."""
    from qcs_gb300 import capi
    n = 14
    with capi.State(n, capi.C64) as s:
        h0, d0 = s.transfer_bytes()
        s.set_amplitudes(np.ones(1 << n) / np.sqrt(1 << n))
        h1, d1 = s.transfer_bytes()
        assert h1 - h0 == 8 << n and d1 == d0
        s.amplitudes()
        h2, d2 = s.transfer_bytes()
        assert d2 - d1 == 8 << n and h2 == h1
        s.apply_gate(capi.W.H, 3)
        h3, _ = s.transfer_bytes()
        assert h3 - h2 == 32
        u, _ = np.linalg.qr(np.random.default_rng(1).normal(size=(64, 64)) + 0j)
        s.apply_block(list(range(6)), u, capi.FUSE_TENSOR)
        h4, _ = s.transfer_bytes()
        # bf16 hi + lo image of the 128 x 128 real form, then the 64 complex
        # row sums (float2) a fused diffusion reads
        assert h4 - h3 == 2 * 128 * 128 * 2 + 64 * 8
        draws = np.linspace(0.01, 0.99, 100)
        s.sample(draws)
        h5, d5 = s.transfer_bytes()
        assert h5 - h4 == 800 and d5 - d2 == 800
