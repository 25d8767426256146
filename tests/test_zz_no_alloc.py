"""The allocation-free sampler, qcs_cuda_sample_noalloc, through the C ABI.

Some callers cannot let a library call cudaMalloc where they sample: a host
application that hands out all device memory from its own pool, or a
latency-critical loop that must not take cudaMalloc's implicit device
synchronisation.  For
them the sampler keeps its scratch in a fixed array inside the library, and
the caller passes the amplitudes, the draws and the output as device
pointers.  It must give the same indices as qcs_cuda_sample, which keeps its
scratch in buffers it allocates itself.

This file is named so that pytest collects it last; it needs nothing from
the other tests and passes on its own as well.
"""
import ctypes as C

import numpy as np
import pytest

from qcs_gb300 import capi
from qcs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(state: capi.State, draws: np.ndarray, torch):
    d_draws = torch.from_numpy(draws).to("cuda")
    d_out = torch.full((len(draws),), -7, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = capi.lib().qcs_cuda_sample_noalloc(
        C.c_void_p(state.device_ptr()), state.size, state.precision,
        C.c_void_p(d_draws.data_ptr()), len(draws), C.c_void_p(d_out.data_ptr()),
        C.c_void_p(state.stream()))
    assert rc == capi.OK, capi.lib().qcs_cuda_last_error()
    state.synchronize()
    return d_out.cpu().numpy()


def test_sample_noalloc_matches_sample_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    cases = [(12, capi.C64, 1), (20, capi.C128, 2)]  # second call reuses the scratch
    for n, prec, seed in cases:
        _, g = W.random_circuit(n, seed, 60, with_qft=False)
        draws = np.random.default_rng(seed).random(4096)
        with capi.State(n, prec) as s:
            s.run(g)
            want = s.sample(draws)
            got = _noalloc(s, draws, torch)
        # identical rule and arithmetic: the indices must agree exactly
        assert np.array_equal(got, want), (n, int(np.sum(got != want)))
        assert np.all(got >= 0)


def test_sample_noalloc_matches_sample_on_states_below_one_warp():
    """States of 2, 8 and 32 amplitudes (one tile narrower than a warp), and
    a call with no shots, which only refreshes the scratch."""
    torch = pytest.importorskip("torch")
    for n, prec in ((1, capi.C64), (3, capi.C128), (5, capi.C64)):
        g = W.one_qubit_circuit(n, n, 12)
        draws = np.random.default_rng(n).random(257)
        with capi.State(n, prec) as s:
            s.run(g)
            want = s.sample(draws)
            got = _noalloc(s, draws, torch)
            assert np.array_equal(got, want), (n, got[got != want][:5])
            rc = capi.lib().qcs_cuda_sample_noalloc(
                C.c_void_p(s.device_ptr()), s.size, s.precision, None, 0, None,
                C.c_void_p(s.stream()))
            assert rc == capi.OK, capi.lib().qcs_cuda_last_error()
            s.synchronize()
            assert np.array_equal(_noalloc(s, draws, torch), want)


def test_sample_noalloc_rejects_sizes_beyond_its_scratch():
    L = capi.lib()
    dummy = C.c_void_p(16)  # never dereferenced: the call fails its checks first
    rc = L.qcs_cuda_sample_noalloc(dummy, 1 << 29, capi.C64, dummy, 1, dummy, None)
    assert rc == capi.EINVAL
    assert b"2^28" in L.qcs_cuda_last_error()
    rc = L.qcs_cuda_sample_noalloc(dummy, 3000, capi.C64, dummy, 1, dummy, None)
    assert rc == capi.EINVAL
