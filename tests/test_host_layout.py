"""Host-side layout logic (no GPU): particle Morton order and the contact-search triangle order."""
import numpy as np

from difftactile_gb300 import configs
from difftactile_gb300 import scene as S
from difftactile_gb300.world import _kd_groups, _morton_key


def test_kd_groups_is_a_permutation():
    for n in (0, 1, 31, 32, 33, 800, 1543, 5000):
        p = np.random.default_rng(n).random((n, 3))
        o = _kd_groups(p)
        assert sorted(o.tolist()) == list(range(n))


def test_kd_groups_are_compact_patches():
    """Groups of 32 consecutive triangles of the press pad's surface cover about 1/25 of it each."""
    sp = configs.sensor_press(n_steps=1).envs[0].sensors[0]
    cen = sp.verts[sp.tris].mean(1)
    c = cen[_kd_groups(cen)]
    ext = np.array([np.ptp(c[g:g + 32], 0) for g in range(0, len(c), 32)])
    full = np.ptp(cen, 0)
    area = (ext[:, 0] * ext[:, 2]).mean()
    assert area < 1.5 * full[0] * full[2] / 25


def test_kd_groups_on_the_dome():
    nodes, tets, tris, layer = S.dome_mesh()
    cen = nodes[tris].mean(1)
    o = _kd_groups(cen)
    c = cen[o]
    ext = np.array([np.linalg.norm(np.ptp(c[g:g + 32], 0)) for g in range(0, len(c), 32)])
    assert ext.mean() < 0.35 * np.linalg.norm(np.ptp(cen, 0))


def test_morton_key_is_block_major():
    cells = np.array([[i, j, k] for i in range(8) for j in range(8) for k in range(8)])
    key = _morton_key(cells)
    order = cells[np.argsort(key)]
    blocks = order >> 2
    # the 64 cells of each 4x4x4 block are consecutive
    for b in range(8):
        assert len(np.unique(blocks[64 * b:64 * b + 64], axis=0)) == 1
