"""Probe classification and the adaptive schedule on the CPU: the oracle's
probesInit restatement and the selectProbesToUpdate restatement against
hand-worked cases."""
import numpy as np

from oracle.oracle import Oracle, select_probes
from vulkanexp_gb300 import abi, scenes


def test_select_all_without_cap():
    states = np.array([1, 2, 0, 8, 2, 1, 4, 3], np.uint32)
    # loop 0: idx % s == 0 -> 0 (s1), 1? 1%2 no, 2 OFF, 3%8 no, 4%2 yes, 5%1 yes, 6%4 no, 7%3 no
    picked, off, loop = select_probes(states, 0, 0)
    assert picked.tolist() == [0, 4, 5] and off == 0 and loop == 1
    # loop 1: (idx + 1) % s == 0 -> 0 (s1), 1 (2%2), 3? 4%8 no, 4? 5%2 no, 5, 6? 7%4 no, 7 (8%3 no)
    picked, off, loop = select_probes(states, off, loop)
    assert picked.tolist() == [0, 1, 5] and off == 0 and loop == 2


def test_select_with_cap_wraps_and_counts_loops():
    states = np.ones(10, np.uint32)
    picked, off, loop = select_probes(states, 7, 5, max_probes=4)
    assert picked.tolist() == [7, 8, 9, 0] and off == 1 and loop == 6
    picked, off, loop = select_probes(states, off, loop, max_probes=4)
    assert picked.tolist() == [1, 2, 3, 4] and off == 5 and loop == 6
    # all OFF: a full visit, nothing picked, one wrap
    picked, off, loop = select_probes(np.zeros(10, np.uint32), 3, 0, max_probes=4)
    assert picked.size == 0 and off == 3 and loop == 1


def test_select_loop_index_spreads_slow_probes():
    states = np.full(16, 8, np.uint32)
    seen = np.zeros(16, int)
    off, loop = 0, 0
    for _ in range(8):
        picked, off, loop = select_probes(states, off, loop)
        seen[picked] += 1
    assert (seen == 1).all()  # every state-8 probe once in 8 updates


def box_scene():
    """One outward-facing unit box at the origin."""
    from vulkanexp_gb300.abi import INSTANCE_DTYPE, MESH_DTYPE, OFFSET_DTYPE

    p, n, t = scenes.box_geometry((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    mats = scenes.make_materials(np.random.default_rng(0), 1, 0.5, 0.5)
    meshes = np.zeros(1, MESH_DTYPE)
    meshes[0] = (0, len(p), 0, t.size)
    inst = np.zeros(1, INSTANCE_DTYPE)
    inst[0]["transform"] = scenes.affine_3x4(np.eye(3), np.zeros(3))
    inst[0]["mask"] = 1
    offs = np.zeros(1, OFFSET_DTYPE)
    return scenes.Scene(scenes.make_vertices(p, n), t.reshape(-1).astype(np.uint32), meshes, inst, offs, mats)


def box_grid(rays=128):
    return abi.make_grid((-4, -4, -4), (4, 4, 4), (5, 5, 5), rays)


def test_init_probes_known_answers():
    sc = box_scene()
    o = Oracle(sc)
    g = box_grid()
    st = o.init_probes(g, scenes.random_orientation(3, 0))
    idx = lambda x, y, z: x + 5 * (y + 5 * z)
    assert st[idx(2, 2, 2)] == 0  # inside the box: every ray sees a back face
    assert st[idx(3, 2, 2)] == 1  # 1.5 m from a face: hits within one cell (2 m)
    assert st[idx(4, 4, 4)] == 8  # nothing within |cell| = 3.46 m
    assert st[idx(0, 0, 0)] == 8
    assert set(np.unique(st)) <= {0, 1, 8}


def test_init_probes_ignores_masked_instances():
    sc = box_scene()
    sc.instances["mask"] = 2  # not INSTANCE_STATIC: the init rays do not see it
    st = Oracle(sc).init_probes(box_grid(), scenes.random_orientation(3, 0))
    assert (st == 8).all()
