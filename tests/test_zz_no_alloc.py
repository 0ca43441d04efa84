"""The allocation-free smoothing entry point, through the C ABI.

gb_filter_apply_noalloc serves callers that cannot allocate device memory
when they smooth a gradient (a host application whose own pool allocator
owns the device memory, or one that cannot take the device-wide
synchronisation of cudaMalloc/cudaFree): its scratch is a fixed array inside
the library. It must give the same field as the allocating entry point
(gb_filter_create + gb_filter_apply), call after call, although every call
reuses the same scratch. This file is collected last on purpose, and its
tests pass alone in a fresh process as well as after the other tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def smooth_both(pkg, nx, nz, sigma, data):
    lib = pkg.lib()
    d = pkg.DeviceArray(data)
    pkg.check(lib.gb_filter_apply_noalloc(nx, nz, sigma, d.ptr), "gb_filter_apply_noalloc")
    got = d.numpy()
    ref = pkg.GaussianFilter(nx, nz, sigma).apply_host(data)
    return got, ref


def test_noalloc_matches_allocating_filter_two_calls_in_a_row(gpu):
    rng = np.random.default_rng(31)
    for nx, nz, sigma in ((181, 97, 5), (300, 40, 10)):
        data = rng.standard_normal(nx * nz).astype(np.float32)
        got, ref = smooth_both(gpu, nx, nz, sigma, data)
        # the same kernels and the same operation order: the results agree to
        # the tolerance of the other filter tests (they are in fact equal)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6
        np.testing.assert_array_equal(got, ref)


def test_noalloc_sums_the_same_terms_on_non_finite_input(gpu):
    """Both entry points stop at the same last nonzero weight, so a value
    that is not finite spreads to exactly the same cells in both."""
    nx, nz, sigma = 160, 90, 4
    data = np.random.default_rng(32).standard_normal(nx * nz).astype(np.float32)
    data[37 * nz + 11] = np.inf
    data[101 * nz + 60] = np.nan
    for _ in range(2):
        got, ref = smooth_both(gpu, nx, nz, sigma, data)
        np.testing.assert_array_equal(np.isfinite(got), np.isfinite(ref))
        np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_grids_beyond_its_scratch(gpu):
    lib = gpu.lib()
    d = gpu.DeviceArray(np.zeros(16, np.float32))
    rc = lib.gb_filter_apply_noalloc(4096, 1025, 5, d.ptr)
    assert rc == gpu.GB_ERR_ARG
    assert "exceeds the fixed scratch" in gpu.last_error()
    rc = lib.gb_filter_apply_noalloc(8193, 2, 5, d.ptr)
    assert rc == gpu.GB_ERR_ARG
