"""The CPU restatement of the Barnes-Hut shaders (no GPU): the literal 1024x1024 grid of
ClearShader..ForceShader and the sorted-key construction must agree bit for bit; the
tree must be structurally sound; theta = 0 must reduce to the direct sum."""
import numpy as np
import pytest

from treecheck import check_tree, edge_case_inputs

FIELDS = ("keys", "sorted_src", "skip", "radius", "pos", "mass")


def _same(a, b):
    return all(np.array_equal(a[k], b[k], equal_nan=True) for k in FIELDS)


@pytest.mark.parametrize("kind,n,size", [(17, 3000, 100.0), (16, 4096, 100.0), (2, 2500, 700.0), (0, 1000, 100.0),
                                         (3, 1024, 300.0)])
def test_grid_equals_sorted(gs, orc, kind, n, size):
    pos, vel, mass = gs.generate(kind, n, size=size, seed=21)
    a, b = orc.State(pos, vel, mass), orc.State(pos, vel, mass)
    for _ in range(3):
        ra = orc.bh_step(a, method="grid")
        rb = orc.bh_step(b, method="sorted")
        assert _same(ra, rb)
        assert ra["interactions"] == rb["interactions"]
        for x, y in zip(a.current(), b.current()):
            np.testing.assert_array_equal(x, y)
        check_tree(rb, 500000.0, rb["valid_count"])


@pytest.mark.parametrize("name", list(edge_case_inputs().keys()))
def test_grid_equals_sorted_edge_cases(orc, name):
    pos, vel, mass = edge_case_inputs()[name]
    a, b = orc.State(pos, vel, mass), orc.State(pos, vel, mass)
    for _ in range(2):
        ra = orc.bh_step(a, method="grid")
        rb = orc.bh_step(b, method="sorted")
        assert _same(ra, rb)
        for x, y in zip(a.current(), b.current()):
            np.testing.assert_array_equal(x, y)


def test_removal_semantics(orc):
    # InitShader.comp:110-117: outside particles move to (-1000, -1000) with mass 0 in both sets
    pos = np.array([[0.0, 0.0], [600.0, 0.0], [10.0, 10.0], [0.0, -501.0]], np.float32)
    vel = np.ones_like(pos)
    mass = np.ones(4, np.float32)
    st = orc.State(pos, vel, mass)
    r = orc.bh_step(st, method="grid")
    p, v, m = st.current()
    assert r["keys"][1] == orc.KEY_REMOVED and r["keys"][3] == orc.KEY_REMOVED
    np.testing.assert_array_equal(p[[1, 3]], -1000.0)
    np.testing.assert_array_equal(m, [1, 0, 1, 0])
    np.testing.assert_array_equal(v[[1, 3]], 1.0)  # never written: the output set's old value


def test_theta_zero_is_direct_sum(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 700, seed=4)
    a, b = orc.State(pos, vel, mass), orc.State(pos, vel, mass)
    orc.bh_step(a, theta=0.0)
    orc.direct_step(b)
    pa, va, _ = a.current()
    pb, vb, _ = b.current()
    np.testing.assert_allclose(va, vb, rtol=2e-4, atol=1e-4 * np.abs(vb).max())
    np.testing.assert_allclose(pa, pb, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("kind,n", [(17, 5000), (2, 3000), (16, 64)])
def test_bounding_box_tree(gs, orc, kind, n):
    pos, vel, mass = gs.generate(kind, n, size=100.0, seed=8)
    st = orc.State(pos, vel, mass)
    r = orc.bh_step(st, box_mode=orc.BOX_BOUNDING)
    assert r["valid_count"] == st.n_al  # nothing is removed
    check_tree(r, r["box"][3], r["valid_count"])
    keys = r["keys"][r["sorted_src"][: r["valid_count"]]]
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    assert np.all(keys < (1 << 24))


def test_bounding_box_force_accuracy(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 4000, seed=2)
    st = orc.State(pos, vel, mass)
    k = np.float32(1e-3)
    orc.bh_step(st, box_mode=orc.BOX_BOUNDING, theta=0.5)
    _, v1, _ = st.current()
    acc_bh = (v1.astype(np.float64) - vel) / float(k)
    a64 = orc.direct_accel_f64(*orc.pad_state(pos, vel, mass)[::2])[:4000]
    err = np.linalg.norm(acc_bh - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert np.median(err) < 2e-2


def test_accurate_mode_moments_and_radius(gs, orc):
    """Mass, centre of mass, second central moments and safe opening radius of every node
    against numpy in FP64: the accurate mode takes them from exact integer sums (positions
    on a grid of 2^-30 of the box half-size, masses of 2^-31 of the largest) rounded once,
    so they agree to about FP32 rounding."""
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 3000, seed=13)
    st = orc.State(pos, vel, mass)
    r = orc.bh_step(st, box_mode=orc.BOX_BOUNDING, theta=0.35, flags=orc.ACCURATE)
    skip, npos, nmass, quad, rad = r["skip"], r["pos"], r["mass"], r["quad"], r["radius"]
    P, _, M = orc.pad_state(pos, vel, mass)
    half = float(np.abs(P[:3000]).max()) * 2
    leaf_src = {}
    # leaves in preorder map to sorted slots in order
    leaves = np.nonzero(skip == 1)[0]
    src = r["sorted_src"][: len(leaves)]
    for li, i in zip(leaves, src):
        leaf_src[li] = i
    checked = 0
    for n in np.nonzero(skip > 1)[0]:
        members = [leaf_src[q] for q in range(n + 1, n + skip[n]) if skip[q] == 1]
        m = M[members].astype(np.float64)
        x = P[members].astype(np.float64)
        if m.sum() == 0:  # padding particles only: centre (0, 0), no moments
            assert nmass[n] == 0 and np.all(npos[n] == 0) and np.all(quad[n] == 0)
            continue
        c = (m[:, None] * x).sum(0) / m.sum()
        assert abs(nmass[n] - m.sum()) <= 1e-6 * m.sum()
        assert np.all(np.abs(npos[n] - c) <= 1e-6 * half)
        d = x - c
        sxx, sxy, syy = (m * d[:, 0] ** 2).sum(), (m * d[:, 0] * d[:, 1]).sum(), (m * d[:, 1] ** 2).sum()
        scale = sxx + syy + m.sum() * (1e-6 * half) ** 2
        assert abs(quad[n, 0] - sxx) < 1e-5 * scale and abs(quad[n, 1] - sxy) < 1e-5 * scale
        assert abs(quad[n, 2] - syy) < 1e-5 * scale
        # every member lies within the opening radius of the centre of mass
        assert np.max(((x - npos[n].astype(np.float64)) ** 2).sum(1)) <= rad[n] * (1 + 1e-5) + 1e-9
        checked += 1
    assert checked > 1000


@pytest.mark.parametrize("box_mode", [0, 1])
def test_accurate_mode_moments_independent_of_input_order(gs, orc, box_mode):
    """Exact sums: reversing the particles' input order changes no bit of any node's
    centre, mass or second moments (the reference's FP32 child sums would)."""
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 4000, size=300.0, seed=17)
    rev = slice(None, None, -1)
    out = []
    for p, v, m in ((pos, vel, mass), (pos[rev].copy(), vel[rev].copy(), mass[rev].copy())):
        st = orc.State(p, v, m)
        r = orc.bh_step(st, box_mode=box_mode, theta=0.35, flags=orc.ACCURATE)
        internal = r["skip"] > 1
        out.append((r["pos"][internal], r["mass"][internal], r["quad"][internal]))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_accurate_mode_theta_zero_is_direct_sum(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, 900, seed=14)
    a, b = orc.State(pos, vel, mass), orc.State(pos, vel, mass)
    orc.bh_step(a, box_mode=orc.BOX_BOUNDING, theta=0.0, flags=orc.ACCURATE)
    orc.direct_step(b)
    np.testing.assert_allclose(a.current()[1], b.current()[1], rtol=2e-4, atol=1e-4 * np.abs(b.current()[1]).max())


def test_accurate_mode_error_small(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 30000, seed=15)
    st = orc.State(pos, vel, mass)
    orc.bh_step(st, box_mode=orc.BOX_BOUNDING, theta=0.35, flags=orc.ACCURATE)
    _, v1, _ = st.current()
    sub = np.random.default_rng(1).choice(30000, 1024, replace=False).astype(np.uint32)
    P, _, M = orc.pad_state(pos, vel, mass)
    a64 = orc.direct_accel_f64(P, M, targets=sub)
    acc = (v1[sub].astype(np.float64) - vel[sub]) / 1e-3
    e = np.linalg.norm(acc - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert np.sqrt(np.mean(e ** 2)) < 1.5e-3


# ---- relative opening criterion (not in the reference) ----
def _acc_err(orc, pos, vel, mass, v1, sub, dt=1e-3):
    P, _, M = orc.pad_state(pos, vel, mass)
    a64 = orc.direct_accel_f64(P, M, targets=sub)
    acc = (v1[sub].astype(np.float64) - vel[sub]) / dt
    e = np.linalg.norm(acc - a64, axis=1) / np.linalg.norm(a64, axis=1)
    return np.sqrt(np.mean(e ** 2))


def test_relative_criterion_first_step_estimates(gs, orc):
    """With no previous |a| (NaN) a group first estimates its particles' |a| by a walk with
    the theta test, then opens nodes by the relative criterion with those estimates.  So
    the first step is, bit for bit, a relative step fed the |a| of a theta walk, and its
    interactions are the two walks' together; it leaves every particle's |a| behind."""
    n = 5120  # a multiple of 64: no zero-mass padding, whose empty-mass cells the alpha-0
    # relative test below would accept where the theta test opens them
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, n, seed=16)
    flags = orc.ACCURATE | orc.RELATIVE_MAC
    a = orc.State(pos, vel, mass)
    ra = orc.bh_step(a, box_mode=orc.BOX_BOUNDING, theta=0.4, flags=flags, rel_alpha=0.01, rel_floor=0.2)
    # the theta walk alone: a known |a| everywhere with alpha 0 leaves only the floor test
    c = orc.State(pos, vel, mass)
    rc = orc.bh_step(c, box_mode=orc.BOX_BOUNDING, theta=0.4, flags=flags, rel_alpha=0.0, rel_floor=0.4,
                     amag_in=np.ones(c.n_al, np.float32))
    est = c.amag.copy()
    d = orc.State(pos, vel, mass)
    rd = orc.bh_step(d, box_mode=orc.BOX_BOUNDING, theta=0.4, flags=flags, rel_alpha=0.01, rel_floor=0.2,
                     amag_in=est)
    assert ra["interactions"] == rc["interactions"] + rd["interactions"]
    assert ra["warp_visits"] == rc["warp_visits"] + rd["warp_visits"]
    for x, y in zip(a.current(), d.current()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.amag, d.amag)
    assert np.all(np.isfinite(a.amag)) and np.all(a.amag > 0)
    acc = (a.current()[1].astype(np.float64) - vel) / 1e-3
    dev = np.abs(a.amag / np.linalg.norm(acc, axis=1) - 1.0)  # velocity rounding blurs acc
    assert np.median(dev) < 1e-4 and dev.max() < 5e-2


def test_relative_criterion_beats_theta(gs, orc):
    """Second step of a 100k spiral: alpha = 0.006 with a theta floor of 0.2 is more
    accurate than theta = 0.3 alone while testing fewer records and summing fewer
    interactions; against theta = 0.35 it costs about the same and errs far less."""
    n = 100000
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, n, seed=2002)
    st = orc.State(pos, vel, mass)
    flags = orc.ACCURATE | orc.RELATIVE_MAC
    orc.bh_step(st, box_mode=orc.BOX_BOUNDING, theta=1.0, flags=flags, rel_alpha=0.006, rel_floor=0.2)
    p1, v1, m1 = [x[:n].copy() for x in st.current()]
    rel = orc.bh_step(st, box_mode=orc.BOX_BOUNDING, theta=1.0, flags=flags, rel_alpha=0.006, rel_floor=0.2,
                      keep_tree=False)
    sub = np.random.default_rng(3).choice(n, 4096, replace=False).astype(np.uint32)
    e_rel = _acc_err(orc, p1, v1, m1, st.current()[1], sub)
    geo, e_geo = {}, {}
    for th in (0.3, 0.35):
        g = orc.State(p1, v1, m1)
        geo[th] = orc.bh_step(g, box_mode=orc.BOX_BOUNDING, theta=th, flags=orc.ACCURATE, keep_tree=False)
        e_geo[th] = _acc_err(orc, p1, v1, m1, g.current()[1], sub)
    print(f"relative {e_rel:.3e} {rel['interactions'] / n:.0f}/particle; theta 0.3 {e_geo[0.3]:.3e} "
          f"{geo[0.3]['interactions'] / n:.0f}; theta 0.35 {e_geo[0.35]:.3e} {geo[0.35]['interactions'] / n:.0f}")
    assert e_rel < e_geo[0.3] < e_geo[0.35]
    assert rel["interactions"] < 0.9 * geo[0.3]["interactions"] and rel["warp_visits"] < geo[0.3]["warp_visits"]
    assert rel["interactions"] < 1.05 * geo[0.35]["interactions"] and e_rel < 0.7 * e_geo[0.35]


def test_relative_criterion_alpha_zero_is_direct_sum(gs, orc):
    """alpha = 0 with theta = 0 accepts no node of nonzero mass and size: every particle
    sums every particle leaf, as the direct sum does (to rounding)."""
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, 900, seed=17)
    a, b = orc.State(pos, vel, mass), orc.State(pos, vel, mass)
    flags = orc.ACCURATE | orc.RELATIVE_MAC
    orc.bh_step(a, box_mode=orc.BOX_BOUNDING, theta=0.0, flags=flags, rel_alpha=0.0)
    orc.direct_step(b)
    a.pos[a.inp][:900], a.vel[a.inp][:900] = b.current()[:2]  # continue both from the same state
    orc.bh_step(a, box_mode=orc.BOX_BOUNDING, theta=0.0, flags=flags, rel_alpha=0.0)
    orc.direct_step(b)
    np.testing.assert_allclose(a.current()[1], b.current()[1], rtol=2e-4, atol=1e-4 * np.abs(b.current()[1]).max())


@pytest.mark.parametrize("kind,n", [(17, 5000), (2, 3000), (16, 64)])
def test_key_bits_refine(gs, orc, kind, n):
    """Bounding-box keys of 15 bits per axis (30-bit Morton codes) refine the 12-bit cells
    of the same box: the scale is 8x the 12-bit one exactly, so key15 >> 6 == key12 for
    every particle, and the deeper tree keeps every structural invariant."""
    pos, vel, mass = gs.generate(kind, n, size=100.0, seed=9)
    r12 = orc.bh_step(orc.State(pos, vel, mass), box_mode=orc.BOX_BOUNDING, key_bits=12)
    r15 = orc.bh_step(orc.State(pos, vel, mass), box_mode=orc.BOX_BOUNDING, key_bits=15)
    assert r15["box"][:2] == r12["box"][:2]
    assert np.array_equal(r15["keys"] >> 6, r12["keys"])
    assert np.all(r15["keys"] < (1 << 30))
    keys = r15["keys"][r15["sorted_src"][: r15["valid_count"]]]
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    check_tree(r15, r15["box"][3], r15["valid_count"])
    assert r15["tree_size"] >= r12["tree_size"]


def test_key_bits_out_of_range(orc):
    pos = np.zeros((64, 2), np.float32)
    for bits in (16, 40):
        with pytest.raises(ValueError):
            orc.bh_step(orc.State(pos, pos, np.ones(64, np.float32)), box_mode=orc.BOX_BOUNDING, key_bits=bits)


def test_pair_walk_changes_only_the_order_of_sums(gs, orc):
    """In a system of 2^18 particles the costly groups (every previous |a| known, the
    smallest below a tenth of the largest) walk as warp pairs: 64-record pops and two-part
    sums.  Against the same steps with every group walked alone: the same interactions and
    visits at each step, and the same state up to the rounding of the reordered sums."""
    n = 1 << 18
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, n, size=100.0, seed=67)
    kw = dict(box_mode=orc.BOX_BOUNDING, theta=1.0, flags=orc.ACCURATE | orc.RELATIVE_MAC, rel_alpha=0.006,
              rel_floor=0.2, keep_tree=False)
    runs = []
    try:
        for pairs in (True, False):
            orc.set_heavy_pairs(pairs)
            st = orc.State(pos, vel, mass)
            stats = []
            for _ in range(2):  # the first step estimates |a|: pairs start at the second
                r = orc.bh_step(st, **kw)
                stats.append((r["interactions"], r["warp_visits"]))
            runs.append((stats, [a.copy() for a in st.current()]))
    finally:
        orc.set_heavy_pairs(True)
    (sp, (pp, vp, mp)), (sa, (pa, va, ma)) = runs
    assert sp == sa
    assert np.array_equal(mp, ma)
    assert not np.array_equal(vp, va)  # some groups were paired
    np.testing.assert_allclose(vp, va, rtol=0, atol=1e-5 * np.abs(va).max())
    np.testing.assert_allclose(pp, pa, rtol=0, atol=1e-6 * np.abs(pa).max())
