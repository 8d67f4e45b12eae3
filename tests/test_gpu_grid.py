"""Grid-guided environment sampling on the GPU against the oracle.

The adaptive light grid (LightGrid.cl, CAdaptiveEnvironment.java) picks a tile of
the environment map per shading-point cell from an accumulated luminance function
before the texel. With the grid frozen, a GPU frame equals the oracle's frame with
the same tolerances as other benchmark-semantics frames (ray counts within 0.5 %,
film relative RMSE 1e-4); the grid itself (initial function, per-cell SATs) is
bit-exact. Accumulation uses float atomics on the GPU, so its sums are compared
within FP32 summation-order tolerance, and the update (func = accum, SATs rebuilt)
exactly. Grid-guided and full-map sampling estimate the same image.
"""
import numpy as np
import pytest

from mambatracer_gb300 import api, scenes
from mambatracer_gb300._lib import MTError
from tests.helpers import bvh_build, env_tables, oracle_frames, oracle_grid, ptr, rel_rmse

pytestmark = pytest.mark.gpu

NU, NV, RX, RY = 320, 320, 16, 32
W, H, DEPTH = 96, 64, 6


def setup(ctx, orc, enable=1, env_size=(512, 256), ntri=20000):
    sc = scenes.soup(ntri, seed=6, extent=0.8, edge_sigma=0.015)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    ew, eh = env_size
    envmap = scenes.sky_env(ew, eh)
    lum, sat = env_tables(orc, envmap, ew, eh)
    S.set_env_with_sat(envmap, lum, sat, ew, eh)
    S.grid_config(NU, NV, RX, RY, enable)
    return sc, S, nodes, bounds, (envmap, ew, eh)


def test_frozen_grid_frames(ctx, orc):
    sc, S, nodes, bounds, env = setup(ctx, orc)
    J = api.Job(ctx, S, W, H, max_depth=DEPTH, mode=1, rr_depth=3, film_kahan=0, grid_updates=0)
    J.set_camera(sc.camera)
    func, gsat = oracle_grid(orc, env, NU, NV, RX, RY)
    gf, gs, ga = J.grid()
    assert gf.tobytes() == func.tobytes()
    assert gs.tobytes() == gsat.tobytes()
    assert not ga.any()
    grid = dict(func=func, sat=gsat, nu=NU, nv=NV, rx=RX, ry=RY)
    acc = None
    for f in range(2):
        J.render(None, float(f + 1))
        rays, _ = J.stats()
        acc, _, orays = oracle_frames(orc, sc, nodes, bounds, W, H, DEPTH, 1, 3, [None], env=env, acc=acc,
                                      first_frame=f + 1, grid=grid)
        assert np.abs(rays - orays).max() <= 0.005 * orays.max()
    assert rel_rmse(J.film(), acc) < 1e-4
    assert not J.grid()[2].any()  # nothing accumulates once the updates are done
    J.close()
    S.close()


def test_accumulation_and_update(ctx, orc):
    sc, S, nodes, bounds, env = setup(ctx, orc)
    J = api.Job(ctx, S, W, H, max_depth=DEPTH, mode=1, rr_depth=3, film_kahan=0, grid_updates=2)
    J.set_camera(sc.camera)
    func0, gsat0 = oracle_grid(orc, env, NU, NV, RX, RY)
    oacc = np.zeros(NU * NV, np.float32)
    J.render(None, 1.0)
    film1 = J.film()
    o1, _, _ = oracle_frames(orc, sc, nodes, bounds, W, H, DEPTH, 1, 3, [None], env=env, first_frame=1,
                             grid=dict(func=func0, sat=gsat0, nu=NU, nv=NV, rx=RX, ry=RY, accum=oacc))
    assert rel_rmse(film1, o1) < 1e-4
    gf, gs, ga = J.grid()
    assert oacc.sum() > 0 and np.count_nonzero(oacc) > 50
    assert abs(float(ga.sum(dtype=np.float64)) - float(oacc.sum(dtype=np.float64))) <= 1e-3 * float(oacc.sum())
    assert np.count_nonzero(ga) == np.count_nonzero(oacc)
    # the update after an accumulating frame: func = accum, per-cell SATs in the reference's order
    assert gf.tobytes() == ga.tobytes()
    sat1 = np.zeros_like(gf)
    orc.lib.or_lightgrid_sat(ptr(gf), ptr(sat1), NU, NV, RX, RY)
    assert gs.tobytes() == sat1.tobytes()
    # the next frame samples the updated grid (and accumulates on top)
    J.render(None, 2.0)
    film2 = J.film()
    o2, _, _ = oracle_frames(orc, sc, nodes, bounds, W, H, DEPTH, 1, 3, [None], env=env, first_frame=2,
                             grid=dict(func=gf, sat=gs, nu=NU, nv=NV, rx=RX, ry=RY))
    assert rel_rmse(film2 - film1, o2) < 1e-4
    J.render(None, 3.0)  # past grid_updates: the grid stays as the second update left it
    gf3, _, ga3 = J.grid()
    assert gf3.tobytes() == ga3.tobytes()
    J.close()
    S.close()


@pytest.mark.parametrize("enable", [1, 2])
def test_cdf_tables_give_the_same_samples(ctx, orc, monkeypatch, enable):
    """The grid-guided sampler reads its searches' CDF values from tables built
    once per cell and per tile; sampling straight from the SATs (MT_CDF_TABLES=0)
    gives byte-identical films, so the tables hold exactly the values they
    replace (frozen grid: no float-atomic accumulation between the two runs)."""
    sc, S, nodes, bounds, env = setup(ctx, orc, enable=enable)
    films = {}
    for tables in ("0", "1"):
        monkeypatch.setenv("MT_CDF_TABLES", tables)
        J = api.Job(ctx, S, W, H, max_depth=DEPTH, mode=1, rr_depth=3, film_kahan=1, grid_updates=0)
        J.set_camera(sc.camera)
        for f in range(3):
            J.render(None, float(f + 1))
        films[tables] = (J.film(), J.stats()[0])
        J.close()
    assert films["0"][0].tobytes() == films["1"][0].tobytes()
    assert np.array_equal(films["0"][1], films["1"][1])
    S.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_map_cdf_tables_give_the_same_samples(ctx, orc, monkeypatch, mode):
    """Full-map environment sampling (grid off; reference semantics always sample
    the full map) searches tables of the map's CDFs built when the environment
    is set; without them (MT_CDF_TABLES=0 when the map is set) the films are
    byte-identical."""
    depth = 4
    seeds = np.random.default_rng(11).integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * depth)).astype(np.int32)
    films = {}
    for tables in ("0", "1"):
        monkeypatch.setenv("MT_CDF_TABLES", tables)
        sc, S, nodes, bounds, env = setup(ctx, orc, enable=0)
        J = api.Job(ctx, S, W, H, max_depth=depth, mode=mode, rr_depth=3, film_kahan=1)
        J.set_camera(sc.camera)
        for f in range(2):
            J.render(seeds if mode == 0 else None, float(f + 1))
        films[tables] = (J.film(), J.stats()[0])
        J.close()
        S.close()
    assert films["0"][0].tobytes() == films["1"][0].tobytes()
    assert np.array_equal(films["0"][1], films["1"][1])


def test_grid_and_full_map_estimate_the_same_image(ctx, orc):
    sc, S, nodes, bounds, env = setup(ctx, orc, ntri=5000)
    means = {}
    for enable in (0, 1, 2):
        S.grid_config(NU, NV, RX, RY, enable)
        J = api.Job(ctx, S, 64, 64, max_depth=4, mode=1, rr_depth=3, film_kahan=1, spp=16, use_graph=1,
                    grid_updates=5)
        J.set_camera(sc.camera)
        for f in range(16):
            J.render(None, float(1 + 16 * f))
        img = J.film(resolve=True)
        assert np.isfinite(img).all()
        means[enable] = float(img[:, :3].mean())
        J.close()
    assert abs(means[1] - means[0]) <= 0.02 * means[0], means
    assert abs(means[2] - means[0]) <= 0.02 * means[0], means
    S.close()


def test_grid_needs_tiles_that_divide_the_map(ctx, orc):
    sc, S, nodes, bounds, env = setup(ctx, orc, env_size=(500, 250), ntri=2000)
    with pytest.raises(MTError, match="divide"):
        api.Job(ctx, S, 32, 32, max_depth=2, mode=1)
    J = api.Job(ctx, S, 32, 32, max_depth=2, mode=0)  # reference semantics never use the grid
    J.close()
    S.close()
