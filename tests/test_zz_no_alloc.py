"""whir_compress_hi_noalloc against whir_compress_hi, through the C ABI.

The no-allocation entry point serves callers that may not allocate device
memory (their GPU memory belongs to their own pool, or they cannot risk the
device-wide synchronisation of cudaMalloc/cudaFree mid-proof).  It keeps its
scratch in one fixed device array shared by every call, so these tests check
that two calls in a row each return exactly what the allocating entry point
returns (the shared accumulators are cleared between calls), and that sizes
beyond the fixed scratch are refused.  This file is collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def _noalloc():
    f = W.lib().whir_compress_hi_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, W.u32p, ctypes.c_int, W.u32p]
    return f


def _call(ctx, dev_poly, k, point, kz):
    out = np.full(4 << (k - kz), 0xFFFFFFFF, np.uint32)
    pt = np.ascontiguousarray(point, np.uint32)
    rc = _noalloc()(ctx.stream(), dev_poly.ptr, k, pt.ctypes.data_as(W.u32p), kz,
                    out.ctypes.data_as(W.u32p))
    assert rc == 0, W.lib().whir_last_error()
    return out


def test_noalloc_matches_allocating_entry_point_twice(ctx, oracle):
    # two consecutive calls of the same shape (leftover accumulators would
    # show up in the second), the largest shape the scratch holds, and the
    # shapes whose split eq tables are smaller than the 2^10-entry halves
    # (kz < 10: a one-entry high table at kz = 0); each result also equals
    # the oracle's (exact: field arithmetic, zero tolerance)
    for k, kz, seed in ((20, 16, 3), (20, 16, 4), (8, 0, 8), (12, 5, 9), (18, 10, 10),
                        (28, 20, 5)):
        poly = W.random_field(seed, 1 << k)
        point = W.random_field(seed + 100, 4 * kz)
        dev = ctx.to_device(poly)
        want = W.compress_hi(ctx, dev, k, point, kz)
        got = _call(ctx, dev, k, point, kz)
        assert np.array_equal(got, want), (k, kz)
        assert np.array_equal(got, oracle.compress_hi(poly, k, point, kz)), (k, kz)
        dev.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(ctx):
    poly = ctx.to_device(W.random_field(6, 1 << 12))
    point = W.random_field(7, 4 * 12)
    out = np.zeros(4 << 9, np.uint32)
    f = _noalloc()
    for k, kz in ((12, 3), (30, 21)):  # 9 kept variables; 21 fixed variables
        rc = f(ctx.stream(), poly.ptr, k, point.ctypes.data_as(W.u32p), kz,
               out.ctypes.data_as(W.u32p))
        assert rc == -1
        assert b"40 KiB" in W.lib().whir_last_error()
