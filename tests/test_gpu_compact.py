"""Stable queue compaction (mt_compact_isects) against a serial run of
CompactAtomic (src/cl/kernel/Compact.cl:21-40): bit-exact records, pixel ids
and count, including the empty, all-kept, ragged-tail and nonzero-start cases."""
import ctypes as C

import numpy as np
import pytest

from mambatracer_gb300 import _lib, layout

pytestmark = pytest.mark.gpu


def dev(ctx, arr):
    b = C.c_void_p()
    _lib.check(_lib.lib().mt_buf_create_from(ctx.h, arr.ctypes.data_as(C.c_void_p), max(arr.nbytes, 4), C.byref(b)))
    return b


def read(b, like):
    out = np.zeros_like(like)
    _lib.check(_lib.lib().mt_buf_read(b, 0, out.ctypes.data_as(C.c_void_p), out.nbytes))
    return out


def make_isects(n, frac, seed):
    rng = np.random.default_rng(seed)
    isects = np.zeros(max(n, 1), layout.INTERSECTION)
    raw = isects.view(np.uint8).reshape(len(isects), 96)
    raw[:] = rng.integers(0, 256, size=raw.shape, dtype=np.uint8)  # every byte, padding included
    isects["hit"] = (rng.random(len(isects)) < frac).astype(np.int32)
    pixels = rng.permutation(max(n, 1)).astype(np.int32)
    return isects, pixels


def serial_compact(isects, pixels, n, start):
    keep = np.nonzero(isects["hit"][:n] != 0)[0]
    return keep, start + len(keep)


def run(ctx, isects, pixels, n, start):
    L = _lib.lib()
    b_in, b_pix = dev(ctx, isects), dev(ctx, pixels)
    out_init = np.zeros(len(isects) + start, layout.INTERSECTION)
    pix_init = np.full(len(isects) + start, -7, np.int32)
    b_out, b_pout = dev(ctx, out_init), dev(ctx, pix_init)
    cnt = np.array([start], np.int32)
    b_cnt = dev(ctx, cnt)
    p = L.mt_buf_device_ptr
    _lib.check(L.mt_compact_isects(ctx.h, p(b_in), p(b_pix), n, p(b_out), p(b_pout), p(b_cnt)))
    res = read(b_out, out_init), read(b_pout, pix_init), int(read(b_cnt, cnt)[0])
    for b in (b_in, b_pix, b_out, b_pout, b_cnt):
        L.mt_buf_free(b)
    return res


@pytest.mark.parametrize("n,frac,start", [(0, 0.5, 0), (1, 1.0, 0), (255, 0.5, 0), (256, 1.0, 0), (257, 0.0, 0),
                                          (100003, 0.37, 0), (2_073_600, 0.53, 0), (50000, 0.5, 1234)])
def test_matches_serial_compact_atomic(ctx, n, frac, start):
    isects, pixels = make_isects(n, frac, seed=n + 7)
    out, pout, count = run(ctx, isects, pixels, n, start)
    keep, expect_count = serial_compact(isects, pixels, n, start)
    assert count == expect_count
    k = len(keep)
    got = out.view(np.uint8).reshape(-1, 96)[start:start + k]
    want = isects.view(np.uint8).reshape(-1, 96)[keep]
    assert np.array_equal(got, want)  # the whole 96-byte record moves
    assert np.array_equal(pout[start:start + k], pixels[keep])
    assert (pout[:start] == -7).all() and (pout[start + k:] == -7).all()
