"""The workload generators build the named configurations' shapes (host only): particle counts,
grids, pad meshes, materials, horizons and checkpointing of configurations 1-5."""
import numpy as np

from difftactile_gb300 import configs
from difftactile_gb300 import scene as S


def test_configuration_1_elastic_cube():
    c = configs.elastic_cube()
    e = c.envs[0]
    assert c.n_particles == 32_768 and e.n_grid == (64, 64, 64) and np.isclose(e.dx, 1 / 64)
    assert e.materials[0].model == S.MODEL_NEOHOOKEAN and e.bc == S.BC_STICKY_FLOOR
    assert c.substeps == 200 and not e.sensors


def test_configuration_2_sensor_press():
    c = configs.sensor_press()
    e = c.envs[0]
    sp = e.sensors[0]
    assert c.n_particles == 64_000 and e.n_grid == (96, 96, 96)
    assert (len(sp.verts), len(sp.tets), len(sp.tris)) == (2_646, 12_000, 800)  # 20x20x5 hexes, 6 tets each
    m = e.materials[0]
    assert m.model == S.MODEL_VON_MISES and m.yield_stress == 50.0 and e.kn == 1e4
    assert (c.n_steps, c.substeps, c.ckpt_every) == (100, 20, 0)
    assert np.asarray(c.actions).shape == (100, 1, 6)


def test_configuration_3_grasp_sphere():
    c, kin = configs.grasp_sphere()
    e = c.envs[0]
    assert 195_000 < c.n_particles < 205_000 and e.n_grid == (128, 128, 128)
    assert len(e.sensors) == 2 and all(len(sp.tets) == 12_000 for sp in e.sensors)
    assert len(e.materials) == 2  # rigid core + elastic shell
    assert (c.n_steps, c.substeps, c.ckpt_every) == (1000, 25, 50)
    assert np.asarray(c.actions).shape == (1000, 7)


def test_configuration_4_batched_population():
    c = configs.batched_population()
    n = [e.n_particles for e in c.envs]
    g = [e.n_grid[0] for e in c.envs]
    assert len(c.envs) == 64 and 8_000 <= min(n) and max(n) <= 128_000
    assert 48 <= min(g) and max(g) <= 128
    assert all(len(e.sensors) == 1 and len(e.sensors[0].tets) == 12_000 for e in c.envs)
    assert (c.n_steps, c.substeps) == (200, 20)
    assert len({round(e.materials[0].E) for e in c.envs}) > 32  # materials sampled per environment


def test_configuration_5_rope_pads():
    c = configs.rope_pads()
    e = c.envs[0]
    assert len(c.envs) == 16 and abs(c.n_particles - 16 * 512_000) < 0.001 * 16 * 512_000 and e.n_grid == (160,) * 3
    assert e.materials[0].model == 1 and e.materials[0].yield_stress > 0  # elastoplastic slab
    assert [r.n for r in e.ropes] == [2_000] and e.ropes[0].iters == 50 and e.ropes[0].compliance == (1e-6, 1e-6)
    assert c.ckpt_every == 10 and len(c.rope_terms) == 16
    assert (len(e.sensors[0].verts), len(e.sensors[0].tets)) == (10_086, 48_000)  # 40x40x5 hexes
    assert (c.n_steps, c.substeps) == (500, 20)
