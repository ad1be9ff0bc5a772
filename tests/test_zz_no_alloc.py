"""nbh_direct_f64_static: the FP64 direct sum for callers that cannot allocate device
memory while they run (their device memory is handed out up front by their own pool or
budget, or a cudaMalloc/cudaFree would synchronise the device in a time-critical loop).  It
keeps its scratch in a fixed array inside the library, so it must give the same sums as
nbh_direct_f64 (which allocates per call), call after call, and refuse lists larger than the
array.  This file is collected last; it passes alone in a fresh process too."""
import numpy as np
import pytest

from helpers import gpu_sim, plummer

pytestmark = pytest.mark.gpu


def _static(sim, idx):
    from nbh import _lib as L
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    out = [np.empty(idx.size, np.float64) for _ in range(3)]
    code = sim._L.nbh_direct_f64_static(sim._h, idx.size, idx.ctypes.data, *[o.ctypes.data for o in out])
    return code, out


def test_static_scratch_matches_allocating_direct_sum_twice():
    from nbh import _lib as L
    n = 60000
    sim = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    sim.load(*plummer(n, seed=21))
    rng = np.random.default_rng(4)
    for call in range(2):                    # two calls in a row share the scratch
        idx = rng.choice(n, 5000 if call == 0 else 3000, replace=False).astype(np.int32)
        code, got = _static(sim, idx)
        assert code == L.NBH_OK, sim._L.nbh_last_error_message(sim._h)
        want = sim.direct_f64(idx)
        for g, w in zip(got, want):
            np.testing.assert_allclose(g, w, rtol=1e-10, atol=1e-13)


def test_static_scratch_rejects_oversized_lists_and_recovers():
    from nbh import _lib as L
    n = 70000
    sim = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    sim.load(*plummer(n, seed=22))
    code, _ = _static(sim, np.arange(L.NBH_DIRECT_STATIC_MAX + 1, dtype=np.int32))
    assert code == L.NBH_ERR_INVALID
    assert b"65536" in sim._L.nbh_last_error_message(sim._h)
    idx = np.arange(0, n, 7, dtype=np.int32)
    code, got = _static(sim, idx)
    assert code == L.NBH_OK
    want = sim.direct_f64(idx)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g, w, rtol=1e-10, atol=1e-13)


def test_static_scratch_full_array_and_batched_universes():
    """A list of exactly NBH_DIRECT_STATIC_MAX targets fills the whole array; a batch of
    uneven universes (one of them a single body) makes each target find its own universe's
    body range on the device, which must agree with the allocating entry point's ranges."""
    from nbh import _lib as L
    rng = np.random.default_rng(8)
    counts = np.array([1, 700, 40000, 5, 31000, 1], np.int32)
    parts = [plummer(int(c), seed=30 + u) for u, c in enumerate(counts)]
    arrs = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    n = int(counts.sum())
    sim = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    sim.load_batch(counts, *arrs)
    sim.step(1)
    for idx in (np.sort(rng.choice(n, L.NBH_DIRECT_STATIC_MAX, replace=False)).astype(np.int32),
                np.array([0, 1, n - 1, 701, 40701, 40705, 71705, 71704], np.int32)):
        code, got = _static(sim, idx)
        assert code == L.NBH_OK, sim._L.nbh_last_error_message(sim._h)
        want = sim.direct_f64(idx)
        for g, w in zip(got, want):
            np.testing.assert_allclose(g, w, rtol=1e-10, atol=1e-13)
    # a single-body universe feels no force at all
    code, got = _static(sim, np.array([0, n - 1], np.int32))
    assert code == L.NBH_OK
    assert all(np.all(g == 0.0) for g in got)
