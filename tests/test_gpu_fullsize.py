"""Parity at the benchmark's full sizes, through properties that hold at any size.

The 1M-triangle soup and the 3.3M-triangle stadium of the benchmark:
  * the GPU BVH build equals the host build of CNormalBVH.build (nodes element
    for element, bounds as values), and its traversal layout equals the one
    imported from the host build;
  * a sample of rays hits the same triangles at the same distances as the oracle;
  * closest hits and any-hit queries agree on every ray: nothing is hit before
    the closest hit, and the closest hit is found by an any-hit query that
    reaches just past it (both traversals enter a node exactly when its box
    passes the slab test for the ray's interval);
  * the traversal work of the FP32 records (mt_trace_counts): the oracle's
    triangle tests exactly, and no more interior visits than the oracle (deferred
    nodes beyond the closest hit are dropped);
  * FP16 records, the wide BVH with 8-bit boxes and the 4-wide FP16 nodes give
    the same distances as FP32 records, and the wide formats visit fewer nodes.
"""
import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes
from tests.helpers import oracle_trace

pytestmark = pytest.mark.gpu


def _check_scene(ctx, orc, sc, nrays, nsample):
    hn, hb, hd = api.bvh_build_host(sc)
    S = api.Scene(ctx, sc)
    dn, db = S.build_bvh_device()
    assert S.depth == hd <= 64
    assert np.array_equal(dn, hn) and np.array_equal(db, hb)
    dev = S.layout()
    S.import_bvh(hn, hb)
    host = S.layout()
    assert dev[2] == host[2] and dev[0].shape == host[0].shape
    assert np.array_equal(dev[0][:, :12], host[0][:, :12]) and dev[0][:, 12:].tobytes() == host[0][:, 12:].tobytes()
    assert dev[1].tobytes() == host[1].tobytes()

    o, d = scenes.random_rays(sc, nrays, seed=71, inside=True)
    rays = layout.make_rays(o, d)
    t, p = S.trace_closest(rays)
    hit = p >= 0
    assert hit.sum() > nrays // 10

    # a sample against the oracle, bit for bit
    idx = np.random.default_rng(72).choice(nrays, nsample, replace=False)
    sub = np.ascontiguousarray(layout.make_rays(o[idx], d[idx]))
    to, po, oc = oracle_trace(orc, sc, hn, hb, sub, counts=True)
    assert np.array_equal(p[idx], po)
    assert t[idx].tobytes() == to.tobytes()
    _, _, gc = S.trace_counts(sub)
    assert np.array_equal(gc[:, 1], oc[:, 1])
    assert np.all(gc[:, 0] <= oc[:, 0])

    # any-hit before the closest hit: never occluded; just past it: occluded
    before = layout.make_rays(o, d)
    before["tMax"] = np.where(hit, t, np.float32(np.inf))
    assert not S.trace_any(before).any()
    past = layout.make_rays(o[hit], d[hit])
    past["tMax"] = t[hit] * np.float32(1.001) + np.float32(1e-6)
    assert S.trace_any(past).all()

    # FP16 records, the wide BVH, 4-wide FP16 nodes: the same distances
    wc = {}
    for prec in (1, 2, 3):
        S.set_precision(prec)
        tq, pq = S.trace_closest(rays)
        assert tq.tobytes() == t.tobytes()
        assert (pq != p).sum() <= max(2, nrays // 10000)
        wc[prec] = S.trace_counts(sub)[2]
    print(f"interior visits per ray: oracle {oc[:, 0].mean():.1f}, FP32 records {gc[:, 0].mean():.1f}, "
          f"wide BVH {wc[2][:, 0].mean():.1f}, 4-wide {wc[3][:, 0].mean():.1f}; triangle tests "
          f"{oc[:, 1].mean():.2f} / {wc[2][:, 1].mean():.2f} / {wc[3][:, 1].mean():.2f}")
    assert wc[2][:, 0].mean() < 0.6 * gc[:, 0].mean()
    assert wc[3][:, 0].mean() < 0.6 * gc[:, 0].mean()
    S.close()


def test_soup_1m(ctx, orc):
    _check_scene(ctx, orc, scenes.soup(1_000_000, seed=1), 1_000_000, 20000)


def test_stadium_3m(ctx, orc):
    _check_scene(ctx, orc, scenes.stadium(), 500_000, 10000)
