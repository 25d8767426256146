"""Cost-model host logic without a GPU: the FP64 checker itself (against
finite differences) and the item features the planner feeds the network."""
import ctypes as C

import numpy as np

from oracle import mlp
from qcs_gb300 import capi


def test_checker_gradient_matches_finite_differences():
    F = 6
    rng = np.random.default_rng(0)
    _, P = mlp.layout(F)
    p = rng.normal(scale=0.3, size=P)
    x = rng.normal(size=(17, F))
    y = rng.normal(size=17)
    _, g = mlp.loss_grad(p, x, y, F)
    for idx in rng.choice(P, size=40, replace=False):
        e = np.zeros(P)
        e[idx] = 1e-6
        num = (mlp.loss_grad(p + e, x, y, F)[0] - mlp.loss_grad(p - e, x, y, F)[0]) / 2e-6
        assert abs(num - g[idx]) <= 1e-6 + 1e-5 * abs(num)


def test_item_features():
    L = capi.lib()
    L.qcs_cuda_item_features.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                         C.POINTER(C.c_float)]
    q = (C.c_int * 6)(0, 2, 9, 10, 11, 29)
    out = (C.c_float * 20)()
    assert L.qcs_cuda_item_features(6, 30, 6, q, 17, out) == 0
    f = np.array(out[:])
    assert f[6] == 1 and f[:6].sum() == 0          # tensor-core block
    assert abs(f[7] - 30 / 32) < 1e-7 and abs(f[8] - 6 / 8) < 1e-7
    assert abs(f[9] - 17 / 64) < 1e-7
    assert f[10] == 1 and f[12] == 1 and f[11] == 0  # qubits 0 and 2 of 0..7
    assert abs(f[18] - 2 / 7) < 1e-7 and abs(f[19] - 29 / 32) < 1e-7
    assert L.qcs_cuda_item_features(9, 30, 6, q, 17, out) == capi.EINVAL


def _replay(n, gates, order):
    from oracle import oracle as O
    from qcs_gb300 import workloads as W
    ops = gates.ops()[order]
    g = W.GateList()
    for o in ops:
        g.add(int(o["kind"]), int(o["target"]), int(o["control"]), float(o["angle"]),
              int(o["index"]))
    with O.OracleState(n) as s:
        s.run(g)
        return s.amplitudes()


def test_learned_plan_is_a_valid_reordering_for_any_model():
    """The learned partitioner (through qcs_cuda_plan_learned, with a model
    that lives on the host only) must return every op exactly once in an
    order that leaves the state unchanged, whatever the network predicts:
    models with random weights at random scales drive it through every
    candidate, split and widening path, and through none of them."""
    from oracle import oracle as O
    from qcs_gb300 import workloads as W
    choices = set()
    for trial in range(60):
        rng = np.random.default_rng(trial)
        m = capi.CostModel(seed=trial)
        p = m.params()
        p = (p * rng.uniform(0.1, 5.0) + rng.normal(size=p.shape) * rng.uniform(0, 1))
        m.set_params(p.astype(np.float32))
        n = int(rng.integers(12, 26))
        kind = trial % 3
        g = (W.mixed_circuit(n, int(rng.integers(2, 6)), trial) if kind == 0 else
             W.brick_circuit(n, int(rng.integers(2, 6)), trial) if kind == 1 else
             W.random_circuit(n, trial, 150, with_qft=False)[1])
        plan = capi.plan_learned(g, n, 6, m)
        m.close()
        choices.add(plan["choice"] // 1000 > 0)
        assert sorted(plan["order"]) == list(range(len(g)))
        assert np.all(np.diff(plan["item"]) >= 0)
        assert plan["pred_ms"] <= plan["greedy_pred_ms"] * (1 + 1e-12)
        if trial % 10 == 0 and n <= 16:
            with O.OracleState(n) as s:
                s.run(g)
                ref = s.amplitudes()
            np.testing.assert_allclose(_replay(n, g, plan["order"]), ref, atol=1e-12)
    assert choices == {False, True}  # both with and without refinement
