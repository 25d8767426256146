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
