"""Batched variational circuits (qcs_cuda_batch_*) against per-instance
complex128 runs of the oracle.

Bars: <Z_0> within 1e-5 of the FP64 oracle for every instance; each
instance's shot histogram passes a chi-square test against the oracle's
probabilities at p > 0.01 (bins with expected count < 5 merged); results are
identical on replay and independent of the schedule.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qcs_gb300 import capi
from qcs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def chi2_pvalue(counts: np.ndarray, probs: np.ndarray) -> float:
    from scipy.stats import chi2
    shots = counts.sum()
    exp = probs * shots
    order = np.argsort(exp)
    c, e = counts[order].astype(float), exp[order]
    # merge the smallest bins until every merged bin expects >= 5
    bins_c, bins_e, acc_c, acc_e = [], [], 0.0, 0.0
    for ci, ei in zip(c, e):
        acc_c += ci
        acc_e += ei
        if acc_e >= 5:
            bins_c.append(acc_c)
            bins_e.append(acc_e)
            acc_c = acc_e = 0.0
    if acc_e > 0 and bins_e:
        bins_c[-1] += acc_c
        bins_e[-1] += acc_e
    bins_c, bins_e = np.array(bins_c), np.array(bins_e)
    if len(bins_e) < 2:
        return 1.0
    stat = np.sum((bins_c - bins_e) ** 2 / bins_e)
    return float(chi2.sf(stat, len(bins_e) - 1))


def oracle_instance(n, g):
    with O.OracleState(n) as o:
        o.run(g)
        return o.expect_z(0), np.abs(o.amplitudes()) ** 2


@pytest.mark.parametrize("schedule", [None, (256, 12, 2, 1), (1024, 14, 1, 0), (256, 12, 4, 0)])
def test_batch_matches_oracle(schedule):
    inst = W.variational_batch(48, seed=5, n_range=(6, 17), depth_range=(2, 8))
    with capi.Batch(inst, shots=2048, seed=9) as b:
        if schedule:
            b.config(*schedule)
        z, samples, ms = b.run()
        z2, samples2, _ = b.run()
    assert np.array_equal(z, z2) and np.array_equal(samples, samples2)
    pvals = []
    for i, (n, g) in enumerate(inst):
        zo, probs = oracle_instance(n, g)
        assert abs(z[i] - zo) < 1e-5, (i, n, z[i], zo)
        assert samples[i].min() >= 0 and samples[i].max() < (1 << n)
        pvals.append(chi2_pvalue(np.bincount(samples[i], minlength=1 << n), probs))
    # p > 0.01 for each instance; allow the expected ~1 % of chance failures
    assert sum(p <= 0.01 for p in pvals) <= 2, sorted(pvals)[:5]


@pytest.mark.parametrize("split_q", [12, 13])
def test_batch_instances_shared_by_groups_of_ctas(split_q):
    """Instances above the tile run on groups of 2^(n - split_q) CTAs that
    split every stage's tiles and meet at a counter between stages; the
    results equal the oracle's and, bit for bit, the one-CTA results."""
    inst = W.variational_batch(24, seed=12, n_range=(13, 16), depth_range=(3, 6))
    with capi.Batch(inst, shots=1024, seed=4) as b:
        b.config(512, 12, 2, 0)
        b.split(27)
        z1, s1, _ = b.run()
        b.split(split_q)
        sched = b.schedule()
        z2, s2, _ = b.run()
        z3, s3, _ = b.run()
    assert sched["split_q"] == split_q
    assert np.array_equal(z2, z3) and np.array_equal(s2, s3)
    assert np.array_equal(z1, z2) and np.array_equal(s1, s2)
    for i, (n, g) in enumerate(inst[:8]):
        zo, _ = oracle_instance(n, g)
        assert abs(z2[i] - zo) < 1e-5


def test_batch_set_angles_and_autotune():
    inst = W.variational_batch(24, seed=8, n_range=(8, 16), depth_range=(2, 5))
    with capi.Batch(inst, shots=256, seed=3) as b:
        z0, _, _ = b.run(want_samples=False)
        rng = np.random.default_rng(0)
        angles = b.ops["angle"] + rng.normal(scale=0.3, size=len(b.ops))
        b.set_angles(angles)
        z1, _, _ = b.run(want_samples=False)
        chosen = b.autotune(repeats=1)
        z2, _, _ = b.run(want_samples=False)
    assert chosen["threads"] in (256, 512, 1024) and chosen["tile_q"] in (12, 13, 14)
    off = 0
    for i, (n, g) in enumerate(inst):
        gg = W.GateList()
        for k, t, c, a in zip(g.kinds, g.targets, g.controls, angles[off:off + len(g)]):
            gg.add(int(k), int(t), int(c), float(a))
        off += len(g)
        zo, _ = oracle_instance(n, gg)
        assert abs(z1[i] - zo) < 1e-5
        assert abs(z2[i] - zo) < 1e-5
    assert not np.allclose(z0, z1)


def test_batch_rejects_bad_gates():
    g = W.GateList()
    g.add(W.H, 5)
    with pytest.raises(capi.QcsCudaError) as e:
        capi.Batch([(4, g)])
    assert e.value.status == capi.EINVAL
