"""Failure detection without a GPU fault: the kernels' bounded waits.

Every kernel that stages its inputs with asynchronous bulk copies waits on an
mbarrier with a bounded number of tries; on giving up it sets the device
error word, lets its own copies and MMAs land, frees its tensor memory and
returns, and the host call reports error code 1.  The test hook
gpuisac_test_stall_ccf makes those kernels issue no copies -- a wait on a
barrier that nothing completes -- with a short limit (64 tries of at most
20 us), so the wait runs out with no copy outstanding.  The call must come
back with the error, quickly, and the next normal call on the same context
must give correct results.  Allocation failures are injected on the host
(gpuisac_test_fail_alloc): the call reports them and the next call is right.
"""
import os
import time

import numpy as np
import pytest

from gpuisac import GpuIsacError, synth

from test_gpu_align import oracle_run, compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stack():
    return synth.make_stack(24, 64, 6, 2, 0.1, 28.0, 4711)


@pytest.mark.parametrize("kernel,mode", [("ws", "fp32"), ("tmem", "fp32"), ("ws", "bf16x3")])
def test_stalled_wait_returns_error_and_context_survives(gpulib, cuda, oracle_mod, stack, monkeypatch, kernel, mode):
    from gpuisac import multi_ref_align
    monkeypatch.setenv("GPUISAC_CCF_KERNEL", kernel)
    gpulib.gpuisac_clear_error()
    gpulib.gpuisac_test_stall_ccf(64)
    try:
        t0 = time.perf_counter()
        with pytest.raises(GpuIsacError, match="timed out"):
            multi_ref_align(stack.particles, stack.refs, 29, 2.0, 2.0, contraction_mode=mode)
        assert time.perf_counter() - t0 < 30.0
    finally:
        gpulib.gpuisac_test_stall_ccf(0)
        gpulib.gpuisac_clear_error()
    # the same context, a normal call: correct results
    pl, d = multi_ref_align(stack.particles, stack.refs, 29, 2.0, 2.0, contraction_mode=mode)
    peak_o, d_o = oracle_run(oracle_mod, stack.particles, stack.refs, 29, 2.0, tex=gpulib.get_texture_limit(64))
    compare(pl.reshape(6, 24, 4), d, peak_o, d_o)


def test_stalled_averaging_wait_returns_error_and_context_survives(gpulib, cuda, oracle_mod):
    """The averaging step's sum kernel stages each member image with a bulk
    copy: stalled, the call reports the timeout and the next call is right."""
    from gpuisac.averages import class_averages
    rng = np.random.default_rng(5)
    P, R, D = 400, 5, 64
    imgs = rng.standard_normal((P, D, D)).astype(np.float32)
    peaks = np.concatenate([rng.uniform(0, 360, (R, P, 1)), rng.uniform(-3, 3, (R, P, 2)),
                            rng.integers(0, 2, (R, P, 1))], 2).astype(np.float32)
    bel = (np.arange(P) % R).astype(np.int32)
    gpulib.gpuisac_clear_error()
    gpulib.gpuisac_test_stall_ccf(64)
    try:
        t0 = time.perf_counter()
        with pytest.raises(GpuIsacError, match="timed out"):
            class_averages(imgs, peaks, bel, 0.2, 0.2, True)
        assert time.perf_counter() - t0 < 30.0
    finally:
        gpulib.gpuisac_test_stall_ccf(0)
        gpulib.gpuisac_clear_error()
    avg, prm, mem, sh = class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    a_o, p_o, m_o, s_o = oracle_mod.class_averages(imgs, peaks, bel, 0.2, 0.2, True)
    assert np.abs(avg - a_o).max() < 2e-5 * np.abs(a_o).max()
    assert np.abs(prm - p_o).max() < 2e-6


@pytest.mark.parametrize("n", [1, 4])
def test_injected_allocation_failure_returns_error_and_next_call_works(gpulib, cuda, oracle_mod, stack, n):
    """The alignment's work-space allocations fail as if the device were out
    of memory (gpuisac_test_fail_alloc, on the host): the call reports it,
    and the next call, with nothing injected, allocates and is right."""
    from gpuisac import multi_ref_align
    gpulib.gpu_clear()  # an empty work space: the next call allocates
    gpulib.gpuisac_clear_error()
    gpulib.gpuisac_test_fail_alloc(n)
    try:
        with pytest.raises(GpuIsacError, match="injected"):
            multi_ref_align(stack.particles, stack.refs, 29, 2.0, 2.0)
    finally:
        gpulib.gpuisac_test_fail_alloc(0)
        gpulib.gpuisac_clear_error()
    pl, d = multi_ref_align(stack.particles, stack.refs, 29, 2.0, 2.0)
    peak_o, d_o = oracle_run(oracle_mod, stack.particles, stack.refs, 29, 2.0, tex=gpulib.get_texture_limit(64))
    compare(pl.reshape(6, 24, 4), d, peak_o, d_o)
