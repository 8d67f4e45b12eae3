"""Environment-map SAT built on the GPU in FP64, and light-grid per-cell SATs.

The reference builds the full-map SAT in FP32 (host, serial) and the grid
SATs in FP32 with Kogge-Stone passes (LightGrid.cl:347-400). The FP32 grid
build must match the reference order bit for bit; the FP64 builds must match an
FP64 host sum, and the sampling decisions they lead to are counted against the
FP32 reference SAT (differences reported, not required to be zero)."""
import numpy as np
import pytest

from mambatracer_gb300 import _lib, api, scenes
from tests.helpers import bvh_build, env_tables, ptr

pytestmark = pytest.mark.gpu


def test_env_fp64_sat(ctx, orc):
    w, h = 2048, 1024
    env = scenes.sky_env(w, h)
    sc = scenes.box_room(8, 8)
    S = api.Scene(ctx, sc)
    S.set_env(env, w, h)
    lum, sat64, sat32 = S.env_arrays(w, h)
    lum_ref, sat_ref32 = env_tables(orc, env, w, h)
    assert lum.tobytes() == lum_ref.tobytes()
    expect = np.cumsum(np.cumsum(lum.astype(np.float64).reshape(h, w), axis=1), axis=0).ravel()
    assert np.max(np.abs(sat64 - expect) / np.maximum(expect, 1e-30)) < 1e-12
    assert sat32.tobytes() == sat64.astype(np.float32).tobytes()
    # the FP32 serial SAT drifts; count how many sampled texels change
    rng = np.random.default_rng(4)
    u = rng.random((4000, 2)).astype(np.float32)
    reg = np.array([w, h, 0, 0, w, h], np.int32)
    diff = 0
    for k in range(u.shape[0]):
        offs = []
        for s in (sat_ref32, sat32):
            off, pdf = np.zeros(2, np.int32), np.zeros(1, np.float32)
            orc.lib.or_sat_sample_discrete(ptr(s), ptr(lum), ptr(reg), float(u[k, 0]), float(u[k, 1]), ptr(off),
                                           ptr(pdf))
            offs.append(tuple(off))
        diff += offs[0] != offs[1]
    # Reported, not required to be zero: the reference's serial FP32 SAT accumulates
    # rounding over 2M texels, so some boundary decisions move (2.6 % measured on GB300).
    print(f"texel choices changed by the FP64 SAT: {diff} of {u.shape[0]}")
    assert diff < 0.10 * u.shape[0]
    S.close()


@pytest.mark.parametrize("nu,nv,rx,ry", [(16, 16, 16, 16), (64, 64, 16, 32), (1600, 1600, 16, 32)])
def test_grid_sat_fp32_reference_order(ctx, orc, nu, nv, rx, ry):
    rng = np.random.default_rng(nu)
    func = rng.random(nu * nv).astype(np.float32)
    gpu = np.zeros_like(func)
    _lib.check(_lib.lib().mt_env_grid_sat(ctx.h, ptr(func), ptr(gpu), nu, nv, rx, ry, 0))
    cpu = np.zeros_like(func)
    orc.lib.or_lightgrid_sat(ptr(func), ptr(cpu), nu, nv, rx, ry)
    assert gpu.tobytes() == cpu.tobytes()


def test_grid_sat_spike_and_fp64(ctx, golden):
    spike = np.zeros(256, np.float32)
    spike[11 * 16 + 10] = 0.01
    out = np.zeros(256, np.float32)
    _lib.check(_lib.lib().mt_env_grid_sat(ctx.h, ptr(spike), ptr(out), 16, 16, 16, 16, 0))
    assert out.tobytes() == golden["spike_sat"].tobytes()
    nu = nv = 1600
    rng = np.random.default_rng(9)
    func = rng.random(nu * nv).astype(np.float32)
    out = np.zeros_like(func)
    _lib.check(_lib.lib().mt_env_grid_sat(ctx.h, ptr(func), ptr(out), nu, nv, 16, 32, 1))
    cells = func.astype(np.float64).reshape(nv // 32, 32, nu // 16, 16)
    expect = np.cumsum(np.cumsum(cells, axis=3), axis=1).reshape(nu * nv)
    assert np.array_equal(out, expect.astype(np.float32))


def test_api_errors(ctx, orc):
    sc = scenes.box_room(8, 8)
    bad = sc.faces.copy()
    bad["mat"][0] = 99
    with pytest.raises(_lib.MTError) as e:
        api.Scene(ctx, scenes.Scene(points=sc.points, faces=bad, materials=sc.materials))
    assert e.value.code == -1
    S = api.Scene(ctx, sc)
    with pytest.raises(_lib.MTError):
        api.Job(ctx, S, 8, 8)  # no BVH yet
    S.build_bvh()
    J = api.Job(ctx, S, 8, 8, max_depth=2, mode=0)
    with pytest.raises(_lib.MTError):
        J.render(np.zeros(10, np.int32), 1.0)  # camera not set
    J.set_camera(sc.camera)
    with pytest.raises(_lib.MTError):
        J.render(None, 1.0)  # mode 0 needs seeds
    nodes, bounds, _, _ = bvh_build(orc, sc)
    nodes[0, 2] = 10 ** 6
    with pytest.raises(_lib.MTError):
        S.import_bvh(nodes, bounds)
    J.close()
    S.close()
