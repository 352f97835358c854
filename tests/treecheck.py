"""Structural checks of a preorder Barnes-Hut record array (the reference's counts /
radiuses / nodePos / nodeMass layout, TreeMoveShader.comp:74-77, ParticleSortShader.comp:104-107)."""
import numpy as np


def edge_case_inputs():
    """Inputs the reference's fixed box treats specially (InitShader.comp:83, 110-117)."""
    rng = np.random.default_rng(123)
    cases = {}
    # all particles in one finest cell
    p = (10.3 + 0.4 * rng.random((100, 2))).astype(np.float32)
    cases["one_cell"] = (p, np.zeros_like(p), (1 + 9 * rng.random(100)).astype(np.float32))
    # duplicates of one position
    p = np.tile(np.array([[3.0, -7.0]], np.float32), (70, 1))
    cases["duplicates"] = (p, np.zeros_like(p), np.ones(70, np.float32))
    # particles on cell edges and on the box edges (+-500), some outside (removed)
    w = np.float32(1000.0 / 1024.0)
    k = np.arange(-520, 525, 7, dtype=np.float32)
    xs = np.concatenate([-500.0 + k * w, [-500.0, 500.0, 499.99997, -500.00003, 1e30, -1e30]]).astype(np.float32)
    ys = np.roll(xs, 5)
    p = np.stack([xs, ys], 1).astype(np.float32)
    cases["edges"] = (p, (0.01 * rng.standard_normal(p.shape)).astype(np.float32),
                      (1 + rng.random(len(xs))).astype(np.float32))
    # NaN position: outside the box by the shader's comparisons
    p = (50 * rng.standard_normal((90, 2))).astype(np.float32)
    p[17] = np.nan
    cases["nan"] = (p, np.zeros_like(p), np.ones(90, np.float32))
    for n in (1, 2, 63, 64, 65):
        p = (100 * rng.standard_normal((n, 2))).astype(np.float32)
        cases[f"n{n}"] = (p, np.zeros_like(p), (1 + 9 * rng.random(n)).astype(np.float32))
    return cases


def check_tree(tree, r0, valid_count):
    skip = tree["skip"].astype(np.int64)
    radius = tree["radius"]
    mass = tree["mass"].astype(np.float64)
    pos = tree["pos"].astype(np.float64)
    T = len(skip)
    assert T == tree["tree_size"]
    if valid_count == 0:
        assert T == 0
        return
    assert skip[0] == T
    leaves = skip == 1
    assert leaves.sum() == valid_count
    assert np.all(radius[leaves] == 0)
    # walk: every internal node's children tile its range exactly; radius follows depth
    stack = [(0, 0)]
    seen = 0
    while stack:
        i, d = stack.pop()
        seen += 1
        if skip[i] == 1 and radius[i] == 0:
            continue
        assert radius[i] == np.float32(r0) / np.float32(4.0 ** d), (i, d, radius[i])
        j, kids, m = i + 1, 0, 0.0
        mx = my = 0.0
        while j < i + skip[i]:
            stack.append((j, d + 1))
            m += mass[j]
            mx += mass[j] * pos[j, 0]
            my += mass[j] * pos[j, 1]
            j += skip[j]
            kids += 1
        assert j == i + skip[i]
        assert kids >= 1
        assert abs(m - mass[i]) <= 1e-5 * max(1.0, abs(mass[i]))
        if mass[i] > 0:
            assert abs(mx / m - pos[i, 0]) <= 1e-4 * (1 + abs(pos[i, 0]))
            assert abs(my / m - pos[i, 1]) <= 1e-4 * (1 + abs(pos[i, 1]))
    assert seen == T
