"""Batched systems (gs_batch_*): one launch per stage over many systems of uneven N.

Every member of a batch must end bit-identical to the same system stepped alone with
gs_run: the batched kernels run the plain path's per-system bodies, only the mapping of
blocks to systems changes.  Compared through the C ABI on the full state (positions,
velocities, masses) and, for Barnes-Hut, on the last tree and interaction counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ACCURATE_BH = dict(algorithm=1, box_mode=1, flags=0x70 | 0x8, accuracy_parameter=0.7)
REFRULE_BH = dict(algorithm=1, box_mode=0, flags=0x8, accuracy_parameter=1.0)
DIRECT = dict(algorithm=0)

# (generator, N, size, params): uneven sizes, both algorithms, padding (N not a multiple
# of 64), a one-block system and a system larger than the sort tile
MIXED = [
    (17, 40000, 100.0, ACCURATE_BH),
    (16, 700, 100.0, ACCURATE_BH),
    (17, 9000, 100.0, ACCURATE_BH),
    (16, 64, 100.0, ACCURATE_BH),
    (16, 3000, 100.0, DIRECT),
    (17, 1000, 100.0, DIRECT),
    (16, 70, 100.0, DIRECT),
    (16, 20000, 100.0, DIRECT),
]


def _make(gs, specs, seed0, math=0):
    sims = []
    for j, (kind, n, size, prm) in enumerate(specs):
        pos, vel, mass = gs.generate(kind, n, size=size, seed=seed0 + j)
        p = gs.default_params(math_mode=math, **prm)
        sims.append(gs.Simulation(pos, vel, mass, params=p))
    return sims


def _state(sim):
    p, v, m = sim.get_particles()
    return np.concatenate([p.ravel(), v.ravel(), m.ravel()]).view(np.uint32)


def _assert_same(alone, batched, specs):
    for j, (a, b) in enumerate(zip(alone, batched)):
        sa, sb = _state(a), _state(b)
        bad = np.nonzero(sa != sb)[0]
        assert bad.size == 0, f"system {j} {specs[j][:2]}: {bad.size} words differ, first {bad[:5]}"
        if specs[j][3]["algorithm"] == 1:
            ta, tb = a.bh_tree(), b.bh_tree()
            assert ta["tree_size"] == tb["tree_size"]
            for k in ("keys", "sorted_src", "skip", "radius", "pos", "mass", "quad"):
                assert np.array_equal(ta[k].view(np.uint32), tb[k].view(np.uint32)), (j, k)
            assert a.stats().interactions == b.stats().interactions, j


def _run_alone(sims, steps):
    for s in sims:
        s.run(steps)
    for s in sims:
        s.sync()


@pytest.mark.parametrize("flags", [0, 1])
def test_mixed_batch_bit_identical(gs, flags):
    alone = _make(gs, MIXED, 500)
    batched = _make(gs, MIXED, 500)
    for s in alone + batched:
        s.reset_stats()
    _run_alone(alone, 3)
    with gs.Batch(batched, flags=flags) as b:
        # clear bbox keys 3x sort scan records, moment tiles and prefix, nodes, node moments, force; direct
        assert b.kernels_per_step == 1 + 1 + 1 + 3 + 1 + 1 + 2 + 1 + 1 + 1 + 1
        b.run(3)
        b.sync()
        _assert_same(alone, batched, MIXED)


# bounding-box systems whose next box comes from the extent their last step gathered
# (accurate walk with and without the relative criterion; the reference's walk in the
# bounding box), each batch with a direct-sum member
AFTER_BATCH = {
    "accurate": [
        (17, 9000, 100.0, ACCURATE_BH),
        (16, 3000, 100.0, dict(ACCURATE_BH, flags=0x70 | 0x8 | 0x100, accuracy_parameter=0.35)),
        (16, 2000, 100.0, DIRECT),
    ],
    "reference-walk": [
        (17, 5000, 100.0, dict(algorithm=1, box_mode=1, flags=0x8, accuracy_parameter=0.7)),
        (16, 1500, 100.0, dict(algorithm=1, box_mode=1, flags=0x8, accuracy_parameter=0.7)),
        (16, 2000, 100.0, DIRECT),
    ],
}


@pytest.mark.parametrize("kind", sorted(AFTER_BATCH))
def test_plain_steps_after_batch_bit_identical(gs, kind):
    """Steps alone, then in a batch, then alone again end bit-identical to the same steps
    alone throughout: a batched step leaves each system's parity and the extent of its new
    positions (the next plain step's box) as a plain step would."""
    specs = AFTER_BATCH[kind]
    alone = _make(gs, specs, 700)
    mixed = _make(gs, specs, 700)
    for s in alone + mixed:
        s.reset_stats()
    _run_alone(alone, 7)
    _run_alone(mixed, 2)
    with gs.Batch(mixed) as b:
        b.run(3)
        b.sync()
    _run_alone(mixed, 2)
    _assert_same(alone, mixed, specs)


def test_reference_rule_batch_bit_identical(gs):
    """The reference's algorithm (fixed box with removal, theta 1, REFERENCE math) in a
    batch: removal touches both particle sets, so a member must match alone exactly."""
    specs = [(0, 5000, 700.0, REFRULE_BH), (2, 2500, 300.0, REFRULE_BH), (1, 777, 100.0, REFRULE_BH),
             (16, 1500, 100.0, DIRECT)]
    alone = _make(gs, specs, 900, math=1)
    batched = _make(gs, specs, 900, math=1)
    for s in alone + batched:
        s.reset_stats()
    _run_alone(alone, 2)
    with gs.Batch(batched) as b:
        # clear keys 3x sort scan records nodes, moments (levels 10..5 + top), force; direct
        assert b.kernels_per_step == 1 + 1 + 3 + 1 + 1 + 1 + 7 + 1 + 1
        b.run(2)
        b.sync()
        _assert_same(alone, batched, specs)


def test_member_runs_alone_between_batches(gs):
    """A member stepped with gs_run between two batch runs changes ping-pong parity; the
    batch re-plans and every system still matches its plain twin."""
    specs = MIXED[:2] + MIXED[4:6]
    alone = _make(gs, specs, 700)
    batched = _make(gs, specs, 700)
    with gs.Batch(batched) as b:
        b.run(2)
        b.sync()
        batched[1].run(1)
        batched[2].run(1)
        b.run(3)
        b.sync()
        for j, s in enumerate(alone):
            s.run(6 if j in (1, 2) else 5)
            s.sync()
        _assert_same(alone, batched, specs)


def test_batch_many_small_systems(gs):
    """Hundreds of members (more than one table search level per block)."""
    rng = np.random.default_rng(5)
    specs = [(int(rng.choice([16, 17])), int(rng.integers(64, 3000)), 100.0,
              ACCURATE_BH if rng.random() < 0.5 else DIRECT) for _ in range(300)]
    alone = _make(gs, specs, 1300)
    batched = _make(gs, specs, 1300)
    _run_alone(alone, 2)
    with gs.Batch(batched) as b:
        b.run(2)
        b.sync()
    for j, (a, c) in enumerate(zip(alone, batched)):
        assert np.array_equal(_state(a), _state(c)), j


def test_batch_rejects_bad_members(gs):
    a = _make(gs, [MIXED[0]], 1)[0]
    c = _make(gs, [(16, 500, 100.0, REFRULE_BH)], 2)[0]
    with pytest.raises(gs.GsimError):
        gs.Batch([a, c])  # Barnes-Hut members with different box mode and flags
    with pytest.raises(gs.GsimError):
        gs.Batch([a, a])
    with pytest.raises(gs.GsimError):
        gs.Batch([])


def test_tuner_smoke(gs):
    d = gs.default_params(algorithm=0)
    h = gs.default_params(accuracy_parameter=0.7, **{k: v for k, v in ACCURATE_BH.items() if k != "accuracy_parameter"})
    h.flags = 0x70
    t = gs.tune_crossover(d, h, min_n=1024, max_n=8192, particles_per_probe=1 << 16)
    assert 1 <= len(t["n"]) <= 4
    assert all(x > 0 for x in t["direct_ms"] + t["bh_ms"])
    assert 1024 <= t["crossover"] <= 8192


def test_relative_criterion_batch_bit_identical(gs):
    """Members with the relative opening criterion and different alphas and floors: each
    keeps its own |a| buffer, alpha and floor in the batch and matches its twin alone,
    through a first step (|a| estimated by the theta walk, then the relative walk), later
    ones (relative walk), and a step after one member alone was reset (only its groups
    estimate)."""
    rel = dict(algorithm=1, box_mode=1, flags=0x170 | 0x8, accuracy_parameter=0.5)
    specs = [(17, 30000, 100.0, dict(rel, relative_accuracy=0.007, relative_theta_floor=0.3)),
             (16, 5000, 100.0, dict(rel, relative_accuracy=0.02)),
             (17, 700, 100.0, dict(rel, relative_accuracy=0.001, relative_theta_floor=0.4)),
             (16, 2000, 100.0, DIRECT)]
    alone = _make(gs, specs, 1500)
    batched = _make(gs, specs, 1500)
    for s in alone + batched:
        s.reset_stats()
    _run_alone(alone, 3)
    with gs.Batch(batched) as b:
        b.run(3)
        b.sync()
        _assert_same(alone, batched, specs)
        pos, vel, mass = gs.generate(16, 5000, size=100.0, seed=99)
        for s in (alone[1], batched[1]):
            s.set_particles(pos, vel, mass)
        _run_alone(alone, 2)
        b.run(2)
        b.sync()
        _assert_same(alone, batched, specs)


def test_batched_uniform_disk_at_rest_error_gate(gs):
    """The batched line's parameters (accurate mode, relative criterion alpha 0.006 with
    floor 0.2, theta 1 for the |a| estimate) on a uniform disk that starts at rest (the
    case where neighbours cancel the field of many particles), N = 68,893, batched beside
    a spiral and a direct-sum system: after 110 steps, each of three more steps has RMS
    relative force error <= 1e-3 against the FP64 direct sum on 16384 particles."""
    rel = dict(algorithm=1, box_mode=1, flags=0x170 | 0x1, accuracy_parameter=1.0, relative_accuracy=0.006,
               relative_theta_floor=0.2)
    specs = [(16, 68893, 100.0, rel), (17, 40000, 100.0, rel), (16, 2000, 100.0, DIRECT)]
    sims = _make(gs, specs, 1004258)
    disk = sims[0]
    sub = np.random.default_rng(2).choice(68893, 16384, replace=False).astype(np.uint32)
    rms = []
    with gs.Batch(sims) as b:
        b.run(110)
        b.sync()
        for _ in range(3):
            start = disk.get_particles()
            b.run(1)
            b.sync()
            acc = disk.get_accel()[sub].astype(np.float64)
            with gs.Simulation(*start, algorithm=gs.DIRECT_SUM) as ref:
                a64 = ref.accel_f64(sub)
            e = np.linalg.norm(acc - a64, axis=1) / np.linalg.norm(a64, axis=1)
            rms.append(float(np.sqrt(np.mean(e ** 2))))
    for s in sims:
        s.close()
    print("uniform disk at rest, batched, RMS per step:", ", ".join(f"{r:.3e}" for r in rms))
    assert max(rms) <= 1e-3


def test_costly_groups_batch_bit_identical(gs):
    """Members of at least 2^18 particles walk their costly groups on warp pairs, taken
    from one list over the whole batch before any other walk; each member still matches its
    twin stepped alone (smaller members walk every group on one warp, as alone)."""
    rel = dict(algorithm=1, box_mode=1, flags=0x170 | 0x8, accuracy_parameter=1.0, relative_accuracy=0.006,
               relative_theta_floor=0.2)
    specs = [(17, 270000, 100.0, rel), (16, 262144, 100.0, dict(rel, relative_accuracy=0.01)),
             (17, 20000, 100.0, rel), (16, 2000, 100.0, DIRECT)]
    alone = _make(gs, specs, 1700)
    batched = _make(gs, specs, 1700)
    for s in alone + batched:
        s.reset_stats()
    _run_alone(alone, 3)
    with gs.Batch(batched) as b:
        b.run(3)
        b.sync()
        _assert_same(alone, batched, specs)
        b.set_shape(force_warps=1)  # runs as two warps per block: pairs need both
        b.run(2)
        b.sync()
        _run_alone(alone, 2)
        _assert_same(alone, batched, specs)
