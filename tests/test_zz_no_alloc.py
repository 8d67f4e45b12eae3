"""The compaction entry point for callers that cannot allocate device memory.

mt_compact_isects_noalloc keeps its scratch in a fixed array inside the
library instead of allocating it, so hosts whose device memory belongs to
another allocator can still compact a hit queue. Its output must equal the
regular entry point's (mt_compact_isects) bit for bit, on consecutive calls
that reuse the same scratch. Collected last so that a run stopping at the
first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from mambatracer_gb300 import _lib, layout

pytestmark = pytest.mark.gpu


def _dev(ctx, nbytes, host=None):
    b = C.c_void_p()
    if host is None or host.nbytes == 0:
        _lib.check(_lib.lib().mt_buf_alloc(ctx.h, max(nbytes, 4), C.byref(b)))
    else:
        _lib.check(_lib.lib().mt_buf_create_from(ctx.h, host.ctypes.data_as(C.c_void_p), max(host.nbytes, 4),
                                                 C.byref(b)))
    return b


def _read(b, like):
    out = np.zeros_like(like)
    _lib.check(_lib.lib().mt_buf_read(b, 0, out.ctypes.data_as(C.c_void_p), out.nbytes))
    return out


def _case(n, frac, seed):
    rng = np.random.default_rng(seed)
    isects = np.zeros(n, layout.INTERSECTION)
    isects.view(np.uint8).reshape(n, 96)[:] = rng.integers(0, 256, size=(n, 96), dtype=np.uint8)
    isects["hit"] = (rng.random(n) < frac).astype(np.int32)
    pixels = rng.permutation(n).astype(np.int32)
    return isects, pixels


def _compact(ctx, fn, isects, pixels, start, use_stream_arg):
    L = _lib.lib()
    n = len(isects)
    b_in, b_pix = _dev(ctx, 0, isects), _dev(ctx, 0, pixels)
    b_out, b_pout = _dev(ctx, 96 * (n + start)), _dev(ctx, 4 * (n + start))
    cnt = np.array([start], np.int32)
    b_cnt = _dev(ctx, 0, cnt)
    p = L.mt_buf_device_ptr
    if use_stream_arg:
        _lib.check(fn(None, p(b_in), p(b_pix), n, p(b_out), p(b_pout), p(b_cnt)))
    else:
        _lib.check(fn(ctx.h, p(b_in), p(b_pix), n, p(b_out), p(b_pout), p(b_cnt)))
    out = _read(b_out, np.zeros(96 * (n + start), np.uint8))
    pout = _read(b_pout, np.zeros(n + start, np.int32))
    count = int(_read(b_cnt, cnt)[0])
    for b in (b_in, b_pix, b_out, b_pout, b_cnt):
        L.mt_buf_free(b)
    return out, pout, count


def test_no_alloc_matches_regular_entry_point(ctx):
    L = _lib.lib()
    L.mt_compact_isects_noalloc.restype = C.c_int
    L.mt_compact_isects_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
    # two calls in a row on the shared scratch: a large queue, then a smaller one
    for n, frac, start, seed in ((2_073_600, 0.53, 0, 1), (300_001, 0.2, 17, 2)):
        isects, pixels = _case(n, frac, seed)
        ref = _compact(ctx, L.mt_compact_isects, isects, pixels, start, False)
        got = _compact(ctx, L.mt_compact_isects_noalloc, isects, pixels, start, True)
        assert got[2] == ref[2] == start + int((isects["hit"] != 0).sum())
        k = got[2]
        assert np.array_equal(got[0][96 * start:96 * k], ref[0][96 * start:96 * k])
        assert np.array_equal(got[1][start:k], ref[1][start:k])


def test_no_alloc_empty_and_full_scratch(ctx):
    L = _lib.lib()
    L.mt_compact_isects_noalloc.restype = C.c_int
    L.mt_compact_isects_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
    # n = 0: nothing is launched and the count keeps its entry value; then
    # exactly the largest queue the fixed scratch holds (every tile slot in use)
    for n, frac, start, seed in ((0, 0.5, 5, 3), (1 << 22, 0.61, 3, 4)):
        isects, pixels = _case(n, frac, seed)
        ref = _compact(ctx, L.mt_compact_isects, isects, pixels, start, False)
        got = _compact(ctx, L.mt_compact_isects_noalloc, isects, pixels, start, True)
        assert got[2] == ref[2] == start + int((isects["hit"] != 0).sum())
        k = got[2]
        assert np.array_equal(got[0][96 * start:96 * k], ref[0][96 * start:96 * k])
        assert np.array_equal(got[1][start:k], ref[1][start:k])


def test_no_alloc_refuses_oversized_queue(ctx):
    L = _lib.lib()
    L.mt_compact_isects_noalloc.restype = C.c_int
    L.mt_compact_isects_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_void_p]
    one = C.c_void_p(8)  # never dereferenced: the size check comes first
    rc = L.mt_compact_isects_noalloc(None, one, one, (1 << 22) + 1, one, one, one)
    assert rc == -1
    assert b"4194304" in L.mt_last_error()
