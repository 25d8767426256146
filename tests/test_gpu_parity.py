"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Bars:
  * complex128 gate sweeps: bit-exact -- against the reference's own
    sequential build (golden fixtures, REFERENCE semantics) and against the
    oracle (PHYSICAL semantics);
  * complex64: max |delta| <= 2e-5 and infidelity <= 1e-9 against the FP64
    oracle on the same inputs (FP32 rounding only);
  * integer answers (argmax, sample indices, measurement outcomes):
    identical.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qcs_gb300 import capi
from qcs_gb300 import workloads as W
from tests.helpers import bits_equal, gates_from, infidelity

pytestmark = pytest.mark.gpu

C64_ATOL = 2e-5
C64_INFID = 1e-9


def oracle_state(n, gates, mode=O.PHYSICAL):
    s = O.OracleState(n, mode)
    s.run(gates)
    return s


# ---- complex128: bit-exact ---------------------------------------------------

@pytest.mark.parametrize("name", ["ref_1q_n10", "ref_mixed_n10_s0", "ref_mixed_n10_s1",
                                  "ref_random_n12"])
def test_c128_reference_semantics_bitexact_vs_reference_build(golden, name):
    d = golden(name)
    n = int(d["n"])
    with capi.State(n, capi.C128, capi.REFERENCE) as s:
        s.run(gates_from(d))
        assert bits_equal(s.amplitudes(), d["ref"])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_c128_physical_bitexact_vs_oracle(seed):
    n = 13
    basis, g = W.random_circuit(n, seed, 200)
    full = W.basis_gates(n, basis)
    full.extend(g)
    with capi.State(n, capi.C128) as s, oracle_state(n, full) as o:
        s.run(full)
        assert bits_equal(s.amplitudes(), o.amplitudes())


def test_c128_physical_matches_numpy_golden(golden):
    d = golden("ref_random_n12")
    with capi.State(12, capi.C128) as s:
        s.run(gates_from(d))
        np.testing.assert_allclose(s.amplitudes(), d["physical"], atol=1e-12)


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_every_gate_every_qubit(prec):
    n = 6
    rng = np.random.default_rng(1)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    for kind in (W.H, W.X, W.Y, W.Z, W.P, W.RX, W.RY, W.RZ, W.CNOT, W.CPHASE):
        for t in range(n):
            ctrls = [c for c in range(n) if c != t] if kind in (W.CNOT, W.CPHASE) else [-1]
            for c in ctrls:
                ang = 0.3 + 0.7 * t + 0.11 * c
                with capi.State(n, prec) as s, O.OracleState(n) as o:
                    s.set_amplitudes(init)
                    o.set_amplitudes(init)
                    s.apply_gate(kind, t, c, ang)
                    o.apply_gate(kind, t, c, ang)
                    if prec == capi.C128:
                        assert bits_equal(s.amplitudes(), o.amplitudes()), (kind, t, c)
                    else:
                        np.testing.assert_allclose(s.amplitudes(), o.amplitudes(), atol=1e-6)


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_reference_semantics_controlled_rule(prec):
    """REFERENCE semantics reproduce [[U00,U01],[0,1]] on control=1 pairs."""
    n = 7
    rng = np.random.default_rng(3)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    for kind, c, t in ((W.CNOT, 0, 3), (W.CNOT, 5, 1), (W.CPHASE, 2, 6)):
        with capi.State(n, prec, capi.REFERENCE) as s, O.OracleState(n, O.COMPAT) as o:
            s.set_amplitudes(init)
            o.set_amplitudes(init)
            s.apply_gate(kind, t, c, 0.7)
            o.apply_gate(kind, t, c, 0.7)
            if prec == capi.C128:
                assert bits_equal(s.amplitudes(), o.amplitudes())
            else:
                np.testing.assert_allclose(s.amplitudes(), o.amplitudes(), atol=1e-5)


@pytest.mark.parametrize("sem,mode", [(capi.PHYSICAL, O.PHYSICAL), (capi.REFERENCE, O.COMPAT)])
def test_plain_runs_replay_from_a_graph(sem, mode):
    """The same plain op list run again and again: from its second run in a
    row it is captured into a CUDA graph and replayed.  complex128: every run
    equals the oracle bit for bit and counts its kernels; a changed angle
    runs kernel by kernel again, and again matches the oracle.  In REFERENCE
    semantics every sweep swaps the state's two buffers; the list has an odd
    number of sweeps, so successive runs start from alternate buffers and
    each starting buffer gets a recording of its own."""
    n = 14
    basis, g = W.random_circuit(n, 5, 120)
    full = W.basis_gates(n, basis)
    full.extend(g)
    if len(full) % 2 == 0:
        full.add(W.I, 3)
    with O.OracleState(n, mode) as o:
        o.run(full)
        want = o.amplitudes()
    with capi.State(n, capi.C128, sem) as s:
        counts = []
        for rep in range(5):
            s.set_basis(0)
            l0 = s.launch_count()
            s.run(full)
            counts.append(s.launch_count() - l0)
            assert bits_equal(s.amplitudes(), want), rep
        assert len(set(counts)) == 1 and counts[0] > 0, counts
        g2 = W.GateList()
        g2.extend(full)
        i = next(j for j, k in enumerate(g2.kinds) if k in W.PARAMETRIC)
        g2.angles[i] += 0.25
        with O.OracleState(n, mode) as o:
            o.run(g2)
            want2 = o.amplitudes()
        for rep in range(4):
            s.set_basis(0)
            s.run(g2)
            assert bits_equal(s.amplitudes(), want2), rep


def test_plain_graph_with_grover_barriers_is_deterministic():
    """Phase flips and diffusions (whose sums the graph recomputes) inside a
    replayed plain run: every replay equals the first, kernel-by-kernel run
    bit for bit, and the FP64 oracle to complex64 rounding."""
    n = 12
    w = W.grover_workload(n, 9, iterations=6)
    full = W.basis_gates(n, w.basis)
    full.extend(w.qft)
    full.extend(w.rounds)
    with O.OracleState(n) as o:
        o.run(full)
        want = o.amplitudes()
    with capi.State(n, capi.C64) as s:
        first = None
        for rep in range(4):
            s.set_basis(0)
            s.run(full)
            a = s.amplitudes()
            if first is None:
                first = a
            assert np.array_equal(a, first), rep
        assert infidelity(first, want) < C64_INFID


# ---- complex64 against the FP64 oracle ----------------------------------------

@pytest.mark.parametrize("n,seed", [(12, 0), (16, 1), (18, 2)])
def test_c64_random_circuit(n, seed):
    basis, g = W.random_circuit(n, seed, 200)
    full = W.basis_gates(n, basis)
    full.extend(g)
    with capi.State(n, capi.C64) as s, oracle_state(n, full) as o:
        s.run(full)
        a, b = s.amplitudes(), o.amplitudes()
        assert np.max(np.abs(a - b)) < C64_ATOL
        assert infidelity(a, b) < C64_INFID


def test_c64_brick_circuit_24q():
    """The brick workload at 24 qubits (the size its oracle runs at)."""
    n = 24
    g = W.brick_circuit(n, 6, 7)
    with capi.State(n, capi.C64) as s, oracle_state(n, g) as o:
        s.run(g)
        a, b = s.amplitudes(), o.amplitudes()
        assert np.max(np.abs(a - b)) < C64_ATOL
        assert infidelity(a, b) < C64_INFID


# ---- reductions and read-out ------------------------------------------------------

@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_reductions(prec):
    n = 15
    _, g = W.random_circuit(n, 5, 120)
    with capi.State(n, prec) as s, oracle_state(n, g) as o:
        s.run(g)
        tol = 1e-6 if prec == capi.C64 else 1e-12
        assert abs(s.norm_sq() - o.norm_sq()) < tol
        for q in (0, 3, n - 1):
            assert abs(s.prob_zero(q) - o.prob_zero(q)) < tol
            assert abs(s.expect_z(q) - o.expect_z(q)) < 2 * tol
        for i in (0, 1, 12345, (1 << n) - 1):
            assert abs(s.probability(i) - o.probability(i)) < tol
        assert s.probability(1 << n) == 0.0
        assert s.probability(-1) == 0.0


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_argmax_exact(prec):
    for n, idx in ((3, 5), (12, 3000), (20, 777777), (22, (1 << 22) - 1)):
        with capi.State(n, prec) as s:
            s.set_basis(idx)
            assert s.argmax() == idx
    with capi.State(10, prec) as s:
        s.set_amplitudes(np.zeros(1 << 10))
        assert s.argmax() == 0  # all-zero state: index 0 like the reference
        v = np.zeros(1 << 10, complex)
        v[[17, 300, 900]] = 0.5  # ties: first index wins
        s.set_amplitudes(v)
        assert s.argmax() == 17


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_measure_with_reference_draws(golden, prec):
    d = golden("ref_measure_n5")
    with capi.State(5, prec, capi.REFERENCE) as s:
        s.run(gates_from(d))
        outs = [s.measure(int(q), float(r)) for q, r in zip(d["qubits"], d["draws"])]
        assert outs == list(d["outcomes"])
        tol = 1e-14 if prec == capi.C128 else 1e-6
        np.testing.assert_allclose(s.amplitudes(), d["ref"], atol=tol)


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_measure_collapse_and_normalize(prec):
    n = 14
    _, g = W.random_circuit(n, 8, 100, with_qft=False)
    rng = np.random.default_rng(0)
    with capi.State(n, prec) as s, oracle_state(n, g) as o:
        s.run(g)
        for q in (0, 7, 13, 2):
            r = float(rng.random())
            assert s.measure(q, r) == o.measure(q, r)
        tol = 1e-6 if prec == capi.C64 else 1e-13
        np.testing.assert_allclose(s.amplitudes(), o.amplitudes(), atol=tol)
        assert abs(s.norm_sq() - 1.0) < tol


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_shots_histogram_vs_reference(golden, prec):
    d = golden("ref_shots_n5")
    with capi.State(5, prec) as s:
        s.run(gates_from(d))
        idx = s.sample(d["draws"])
    hist = np.bincount(idx[idx >= 0], minlength=32)
    assert np.array_equal(hist, d["hist"])


@pytest.mark.parametrize("n", [10, 13, 17])
def test_sample_indices_vs_oracle(n):
    _, g = W.random_circuit(n, 21, 80, with_qft=False)
    draws = np.random.default_rng(n).random(3000)
    draws[:3] = [0.0, 1.0, 0.999999999]
    with capi.State(n, capi.C128) as s, oracle_state(n, g) as o:
        s.run(g)
        a = s.sample(draws)
        b = o.sample(draws)
        # identical except on a knife edge of FP64 rounding: the draw r = 1.0
        # sits on the total, which the reference's sequential sum and the
        # device's tree sum round differently (-1 or the last index)
        assert np.array_equal(a[2:], b[2:])
        assert a[0] == b[0]
        assert a[1] in (-1, b[1])


def sample_rule(amps: np.ndarray, draws: np.ndarray) -> np.ndarray:
    """qc_run_shots' rule (src/qcs.c:589-605) on FP64 amplitudes: the first
    index whose sequential running sum of |a|^2 exceeds the draw, else -1
    (np.cumsum adds in order, as the reference's loop does)."""
    cum = np.cumsum(np.abs(amps.astype(np.complex128)) ** 2)
    idx = np.searchsorted(cum, draws, side="right")
    return np.where(idx < len(cum), idx, -1)


@pytest.mark.parametrize("n", [23])
def test_sample_indices_vs_oracle_several_tiles_per_range(n):
    """2048 tiles of 4096 amplitudes: the tile-sum pass gives each block a
    range of two tiles, so the prefix is a range offset plus a prefix within
    the range, and each shot searches the ranges, then the tiles."""
    _, g = W.random_circuit(n, 31, 60, with_qft=False)
    draws = np.random.default_rng(n).random(3000)
    draws[0] = 0.0  # (a draw on an exact cumulative sum would be a knife edge)
    with capi.State(n, capi.C128) as s, oracle_state(n, g) as o:
        s.run(g)
        a = s.sample(draws)
        b = sample_rule(o.amplitudes(), draws)
        # a draw within FP64 rounding of a tile edge may land on either side
        assert np.mean(a == b) > 0.999, int(np.sum(a != b))
        assert a[0] == b[0]


def test_sample_c64_large_state_vs_rule():
    """complex64 at 24 qubits (4096 tiles, ranges of four), against the rule
    applied in FP64 to the same amplitudes.  The sampler sums a complex64
    tile's |a|^2 in FP32 (per thread, then a warp tree) and in FP64 beyond:
    a tile mass is off by ~5e-8 of itself, and over 4096 tiles the prefix
    where a tile's scan starts by ~1e-9, a few percent of one amplitude's
    probability (~6e-8) here.  So a draw occasionally lands one index over,
    as it would with the state's own FP32 rounding; 99 % of the indices must
    be the rule's.  (Against the FP64 oracle's own state the indices would
    also move with the complex64 circuit's ~1e-6 norm error.)"""
    n = 24
    g = W.brick_circuit(n, 2, 5)
    draws = np.random.default_rng(7).random(4000)
    with capi.State(n, capi.C64) as s:
        s.run(g)
        a = s.sample(draws)
        b = sample_rule(s.amplitudes(), draws)
    assert np.mean(a == b) > 0.99, int(np.sum(a != b))
    assert np.all(np.abs(a - b) <= 64)  # never another region of the state
    assert np.all(a >= 0)


def test_normalize_rule():
    with capi.State(6, capi.C128) as s:
        v = np.zeros(64, complex)
        v[3] = 2.0
        v[5] = 1j
        s.set_amplitudes(v)
        s.normalize()
        np.testing.assert_allclose(s.amplitudes(), v / np.sqrt(5.0), atol=1e-15)
        s.set_amplitudes(np.zeros(64))
        s.normalize()  # below 1e-12: left alone
        assert np.all(s.amplitudes() == 0)


# ---- Grover -------------------------------------------------------------------------

def test_grover_reference_semantics(golden):
    d = golden("ref_grover_n6")
    with capi.State(6, capi.C128, capi.REFERENCE) as s:
        s.run(gates_from(d))
        np.testing.assert_allclose(s.amplitudes(), d["ref"], rtol=1e-13, atol=1e-13)
        assert abs(s.probability(42) - 17.015625) < 1e-9


@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_grover_physical(prec, golden):
    d = golden("ref_grover_n6")
    with capi.State(6, prec) as s:
        s.run(gates_from(d))
        np.testing.assert_allclose(s.amplitudes(), d["physical"], atol=1e-6)
        assert s.argmax() == 42
    n = 12
    w = W.grover_workload(n, 4, iterations=20)
    with capi.State(n, prec) as s, oracle_state(n, w.search) as o:
        s.run(w.search)
        assert s.argmax() == o.argmax() == w.marked
        assert abs(s.probability(w.marked) - o.probability(w.marked)) < 1e-5
    full = W.basis_gates(n, w.basis)
    full.extend(w.qft)
    full.extend(w.rounds)
    with capi.State(n, prec) as s, oracle_state(n, full) as o:
        s.run(full)
        assert infidelity(s.amplitudes(), o.amplitudes()) < 1e-8
        pm = o.probability(w.marked)
        assert abs(s.probability(w.marked) - pm) < 1e-4 * pm


# ---- fused blocks ---------------------------------------------------------------------

@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("prec", [capi.C64, capi.C128])
def test_apply_block_random_unitary(k, prec):
    n = 11
    rng = np.random.default_rng(k)
    for trial in range(3):
        qubits = list(rng.choice(n, size=k, replace=False))
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        u, _ = np.linalg.qr(m)
        init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        init /= np.linalg.norm(init)
        with capi.State(n, prec) as s, O.OracleState(n) as o:
            s.set_amplitudes(init)
            o.set_amplitudes(init)
            s.apply_block(qubits, u, capi.FUSE_SIMT)
            o.apply_block(qubits, u)
            tol = 1e-5 if prec == capi.C64 else 1e-13
            np.testing.assert_allclose(s.amplitudes(), o.amplitudes(), atol=tol)


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_fused_circuit_simt(k):
    n = 16
    g = W.brick_circuit(n, 8, 3)
    _, r = W.random_circuit(n, 9, 150)
    g.extend(r)
    with capi.State(n, capi.C64) as s, oracle_state(n, g) as o:
        s.run(g, fusion_k=k, engine=capi.FUSE_SIMT)
        a, b = s.amplitudes(), o.amplitudes()
        assert np.max(np.abs(a - b)) < C64_ATOL
        assert infidelity(a, b) < C64_INFID
    with capi.State(n, capi.C128) as s, oracle_state(n, g) as o:
        s.run(g, fusion_k=k, engine=capi.FUSE_SIMT)
        np.testing.assert_allclose(s.amplitudes(), o.amplitudes(), atol=1e-12)


# Tensor-core engine (split BF16 x 3, FP32 accumulation): per-block relative
# error ~2^-16, so the bars are infidelity <= 1e-8 per block and <= 1e-6 over a
# circuit, and max |delta| <= 5e-5.
TC_ATOL = 5e-5


@pytest.mark.parametrize("k", [5, 6, 7])
@pytest.mark.parametrize("placement", ["col", "pair", "low"])
def test_apply_block_tensor_cores(k, placement):
    """The kernel's three access modes: qubit 0 a column qubit, qubit 0 in the
    block, the block exactly qubits 0..k-1; qubits in random order.  At k = 7
    (the complex-form kernel) a block on qubits 0..6 runs in the paired mode."""
    n = 15
    rng = np.random.default_rng(10 * k + len(placement))
    for trial in range(3):
        rest = [q for q in range(1, n)]
        if placement == "low":
            qubits = [int(q) for q in rng.permutation(k)]
        else:
            qubits = list(rng.choice(rest, size=k - 1 if placement == "pair" else k,
                                     replace=False))
        if placement == "pair":
            qubits.insert(int(rng.integers(0, k)), 0)
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        u, _ = np.linalg.qr(m)
        init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        init /= np.linalg.norm(init)
        with capi.State(n, capi.C64) as s, O.OracleState(n) as o:
            s.set_amplitudes(init)
            o.set_amplitudes(init)
            s.apply_block(qubits, u, capi.FUSE_TENSOR)
            o.apply_block(qubits, u)
            s.synchronize()
            a, b = s.amplitudes(), o.amplitudes()
            assert np.max(np.abs(a - b)) < TC_ATOL
            assert infidelity(a, b) < 1e-8


@pytest.mark.parametrize("k,n", [(6, 13), (5, 12), (6, 14), (7, 14), (7, 15)])
def test_tensor_cores_smallest_states(k, n):
    """The smallest states the tensor engine takes (n = k + 7: one tile, one
    CTA) and a few tiles: every pipeline stage runs with fewer tiles than
    stages in flight."""
    rng = np.random.default_rng(100 + n)
    for placement in ("col", "pair", "low"):
        if placement == "low":
            qubits = list(range(k))
        elif placement == "pair":
            qubits = [0] + [int(q) for q in rng.choice(range(1, n), size=k - 1, replace=False)]
        else:
            qubits = [int(q) for q in rng.choice(range(1, n), size=k, replace=False)]
        u, _ = np.linalg.qr(rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k)))
        init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        init /= np.linalg.norm(init)
        with capi.State(n, capi.C64) as s, O.OracleState(n) as o:
            s.set_amplitudes(init)
            o.set_amplitudes(init)
            s.apply_block(qubits, u, capi.FUSE_TENSOR)
            o.apply_block(qubits, u)
            a, b = s.amplitudes(), o.amplitudes()
            assert np.max(np.abs(a - b)) < TC_ATOL, placement
            assert infidelity(a, b) < 1e-8, placement


def test_auto_engine_widens_four_qubit_blocks():
    """AUTO runs a 4-qubit block on the tensor cores, widened to 5 qubits with
    the identity on the added qubit; fused circuits at width 4 likewise."""
    n = 15
    rng = np.random.default_rng(44)
    for trial in range(3):
        qubits = [int(q) for q in rng.choice(n, size=4, replace=False)]
        m = rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))
        u, _ = np.linalg.qr(m)
        init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        init /= np.linalg.norm(init)
        with capi.State(n, capi.C64) as s, O.OracleState(n) as o:
            s.set_amplitudes(init)
            o.set_amplitudes(init)
            s.profile(True)
            s.apply_block(qubits, u, capi.FUSE_AUTO)
            prof = s.profile_read()
            s.profile(False)
            o.apply_block(qubits, u)
            a, b = s.amplitudes(), o.amplitudes()
            assert "block_tc" in prof and "block_simt" not in prof
            assert np.max(np.abs(a - b)) < TC_ATOL
            assert infidelity(a, b) < 1e-8
    g = W.brick_circuit(n, 6, 8)
    with capi.State(n, capi.C64) as s, oracle_state(n, g) as o:
        s.run(g, fusion_k=4)
        assert infidelity(s.amplitudes(), o.amplitudes()) < 1e-6


def test_tensor_cores_apply_non_unitary_matrices_as_given():
    """A matrix that is not unitary (scaled, or a projector) passed to
    qcs_cuda_apply_block is applied as the plain linear map: the per-column
    norm restore is only for unitary blocks."""
    n = 15
    rng = np.random.default_rng(55)
    for qubits in ([1, 4, 6, 8, 11, 13], [0, 2, 3, 7, 9, 12, 14]):
        K = 1 << len(qubits)
        u, _ = np.linalg.qr(rng.normal(size=(K, K)) + 1j * rng.normal(size=(K, K)))
        proj = np.diag([1.0 if i % 3 else 0.0 for i in range(K)]).astype(complex)
        for m in (0.5 * u, proj, u @ proj):
            init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
            init /= np.linalg.norm(init)
            with capi.State(n, capi.C64) as s, O.OracleState(n) as o:
                s.set_amplitudes(init)
                o.set_amplitudes(init)
                s.apply_block(qubits, m, capi.FUSE_TENSOR)
                o.apply_block(qubits, m)
                a, b = s.amplitudes(), o.amplitudes()
                assert np.max(np.abs(a - b)) < TC_ATOL


def test_tensor_cores_preserve_the_norm_over_many_blocks():
    """100 random 6-qubit unitaries: FP32 accumulation in the tensor cores
    rounds toward zero; the per-column norm restore must keep the state's
    norm to FP32 rounding."""
    n = 16
    rng = np.random.default_rng(77)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    with capi.State(n, capi.C64) as s:
        s.set_amplitudes(init)
        for i in range(100):
            m = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
            u, _ = np.linalg.qr(m)
            qubits = (list(range(6)) if i % 5 == 0 else
                      list(rng.choice(n, size=6, replace=False)))
            s.apply_block(qubits, u, capi.FUSE_TENSOR)
        s.synchronize()
        assert abs(s.norm_sq() - 1.0) < 1e-5


def test_tensor_engine_rejects_unsupported():
    with capi.State(12, capi.C128) as s:
        with pytest.raises(capi.QcsCudaError) as e:
            s.apply_block(list(range(6)), np.eye(64), capi.FUSE_TENSOR)
        assert e.value.status == capi.EUNSUP


@pytest.mark.parametrize("k", [5, 6, 7])
def test_fused_circuit_tensor_cores(k):
    n = 18
    g = W.brick_circuit(n, 10, 4)
    _, r = W.random_circuit(n, 12, 200)
    g.extend(r)
    with capi.State(n, capi.C64) as s, oracle_state(n, g) as o:
        s.run(g, fusion_k=k, engine=capi.FUSE_TENSOR)
        s.synchronize()
        a, b = s.amplitudes(), o.amplitudes()
        assert np.max(np.abs(a - b)) < TC_ATOL
        assert infidelity(a, b) < 1e-6


def test_fused_with_grover_barriers():
    n = 11
    w = W.grover_workload(n, 6, iterations=8)
    full = W.basis_gates(n, w.basis)
    full.extend(w.qft)
    full.extend(w.rounds)
    with capi.State(n, capi.C64) as s, oracle_state(n, full) as o:
        s.run(full, fusion_k=4)
        assert infidelity(s.amplitudes(), o.amplitudes()) < C64_INFID
    with capi.State(n, capi.C64) as s, oracle_state(n, w.search) as o:
        s.run(w.search, fusion_k=4)
        assert s.argmax() == o.argmax() == w.marked


@pytest.mark.parametrize("engine,k", [(capi.FUSE_SIMT, 5), (capi.FUSE_TENSOR, 6),
                                      (capi.FUSE_AUTO, 4), (capi.FUSE_AUTO, 7)])
def test_kept_plan_replays_identically(engine, k):
    """A second run of the same op list reuses the kept plan and block
    matrices and gives the same amplitudes, bit for bit, as planning afresh;
    a list with one angle changed is planned afresh.  Tensor-core blocks of a
    kept plan stay on the device, so a replay uploads no block images."""
    n = 16
    g = W.mixed_circuit(n, 12, 5)
    with capi.State(n, capi.C64) as s:
        h0, _ = s.transfer_bytes()
        s.run(g, fusion_k=k, engine=engine, plan_cache=False)
        h1, _ = s.transfer_bytes()
        a = s.amplitudes()
        for _ in range(2):
            s.set_basis(0)
            h2, _ = s.transfer_bytes()
            s.run(g, fusion_k=k, engine=engine)
            h3, _ = s.transfer_bytes()
            assert np.array_equal(s.amplitudes(), a)
        if engine != capi.FUSE_SIMT:  # the last replay moved no block image
            assert h3 - h2 < min(h1 - h0, 2 * 64 * 64 * 2)  # one 5-qubit image
        ops = g.ops().copy()
        i = int(np.nonzero(np.isin(ops["kind"], (W.RX, W.RY, W.RZ, W.P)))[0][0])
        ops["angle"][i] += 0.5
        s.set_basis(0)
        s.run(ops, fusion_k=k, engine=engine)
        c = s.amplitudes()
        s.set_basis(0)
        s.run(ops, fusion_k=k, engine=engine, plan_cache=False)
        assert np.array_equal(s.amplitudes(), c)
        assert not np.array_equal(a, c)


@pytest.mark.parametrize("k", [6, 7])
def test_grover_rounds_fuse_diffusion_into_tensor_core_blocks(k):
    """QFT + rounds of (Hadamard layer, phase flip, diffusion), fused at width
    6 or 7 on a state the tensor cores take: every diffusion but the last
    runs inside the following block, and the block before each flip leaves
    the sum the diffusion needs, so no separate reduction or diffusion sweep
    runs; the state still matches the FP64 oracle."""
    n = 16
    w = W.grover_workload(n, 8, iterations=8)
    full = W.basis_gates(n, w.basis)
    full.extend(w.qft)
    full.extend(w.rounds)
    with capi.State(n, capi.C64) as s, oracle_state(n, full) as o:
        s.profile(True)
        s.run(full, fusion_k=k)
        prof = s.profile_read()
        s.profile(False)
        a, b = s.amplitudes(), o.amplitudes()
        assert infidelity(a, b) < 1e-6
        pm = o.probability(w.marked)
        assert abs(s.probability(w.marked) - pm) < 1e-3 * pm
    assert prof["diffuse"][0] == 1        # the last round's, with no block after it
    assert "reduce" not in prof           # sums come from the blocks' epilogues
    with capi.State(n, capi.C64) as s, oracle_state(n, w.search) as o:
        s.run(w.search, fusion_k=k)
        assert s.argmax() == o.argmax() == w.marked
        assert infidelity(s.amplitudes(), o.amplitudes()) < 1e-6


# ---- full size: size-independent properties ------------------------------------------

def _inverse(g: W.GateList) -> W.GateList:
    inv = W.GateList()
    for k, t, c, a in reversed(list(zip(g.kinds, g.targets, g.controls, g.angles))):
        if k in (W.RX, W.RY, W.RZ, W.P, W.CPHASE):
            a = -a
        elif k not in (W.H, W.X, W.Y, W.Z, W.CNOT):
            raise ValueError(k)
        inv.add(k, t, c, a)
    return inv


@pytest.mark.parametrize("fusion_k,engine", [(0, capi.FUSE_AUTO), (4, capi.FUSE_SIMT),
                                             (6, capi.FUSE_TENSOR), (7, capi.FUSE_TENSOR)])
def test_30q_brick_then_inverse_returns_to_zero(fusion_k, engine):
    n = 30
    g = W.brick_circuit(n, 3, 5)
    with capi.State(n, capi.C64) as s:
        s.run(g, fusion_k=fusion_k, engine=engine)
        assert abs(s.norm_sq() - 1.0) < 1e-5
        s.run(_inverse(g), fusion_k=fusion_k, engine=engine)
        s.synchronize()
        assert s.argmax() == 0
        assert s.probability(0) > 1 - 1e-5


def test_30q_basis_state_argmax_and_collapse():
    n = 30
    idx = (1 << 29) + 123456789
    with capi.State(n, capi.C64) as s:
        s.run(W.basis_gates(n, idx))
        assert s.argmax() == idx
        s.apply_gate(W.H, 29)
        assert abs(s.prob_zero(29) - 0.5) < 1e-6
        assert s.measure(29, 0.25) == 0
        assert s.argmax() == idx - (1 << 29)
        assert abs(s.norm_sq() - 1.0) < 1e-6


def test_30q_grover_matches_closed_form():
    """From the uniform state, k iterations give sin^2((2k+1) asin(2^-n/2))."""
    n = 30
    marked = 987654321
    g = W.GateList()
    for q in range(n):
        g.add(W.H, q)
    for _ in range(5):
        g.add(W.PHASE_FLIP, index=marked)
        g.add(W.DIFFUSION)
    with capi.State(n, capi.C64) as s:
        s.run(g)
        theta = np.arcsin(2.0 ** (-n / 2))
        want = np.sin(11 * theta) ** 2
        assert abs(s.probability(marked) - want) / want < 1e-4
        assert s.argmax() == marked


# ---- error handling -----------------------------------------------------------------------

def test_invalid_arguments():
    with capi.State(4) as s:
        for bad in (lambda: s.apply_gate(W.H, 4), lambda: s.apply_gate(W.CNOT, 1, 1),
                    lambda: s.apply_gate(99, 0), lambda: s.phase_flip(16),
                    lambda: s.set_basis(-1), lambda: s.apply_block([0, 0], np.eye(4))):
            with pytest.raises(capi.QcsCudaError) as e:
                bad()
            assert e.value.status == capi.EINVAL
        s.apply_gate(W.X, 0)  # still usable
        assert s.argmax() == 1


def test_injected_failures_leave_library_usable():
    L = capi.lib()
    L.qcs_cuda_debug_inject(1, 1)
    with pytest.raises(capi.QcsCudaError) as e:
        capi.State(5)
    assert e.value.status == capi.ENOMEM
    with capi.State(5) as s:
        L.qcs_cuda_debug_inject(2, 1)
        with pytest.raises(capi.QcsCudaError) as e:
            s.apply_gate(W.H, 0)
        assert e.value.status == capi.ELAUNCH
        s.apply_gate(W.X, 2)
        assert s.argmax() in (4, 5)
    L.qcs_cuda_debug_inject(0, 0)
