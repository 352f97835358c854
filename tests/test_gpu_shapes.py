"""Launch shapes (gs_shape) and the autotuner that picks them.

Every shape the tuner can choose runs the same arithmetic: in REFERENCE math each one is
bit-identical to the oracle (the whole Barnes-Hut state over several steps, for every
combination of sort tile, sort and scan look-back widths, group-walk warps and list caps,
and moments grid).  The direct sum's targets per thread change no bit either; its
j-split (direct_blocks_per_sm) changes the FAST-math summation grouping only."""
import itertools
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BH_SPACE = dict(sort_keys_per_thread=(8, 16), sort_lookback=(8, 16, 32), scan_lookback=(32, 64, 128),
                force=((1, 0), (2, 0), (2, 1), (4, 0)), moment_blocks_per_sm=(1, 2))


def _bh_shapes(gs):
    for kpt, lb, scan, (warps, short), mom in itertools.product(*BH_SPACE.values()):
        sh = gs.shape_defaults()
        sh.sort_keys_per_thread, sh.sort_lookback, sh.scan_lookback = kpt, lb, scan
        sh.force_warps, sh.force_short_lists, sh.moment_blocks_per_sm = warps, short, mom
        yield sh


def _words(sim):
    return np.concatenate([a.ravel() for a in sim.padded_state()[:3]]).view(np.uint32)


@pytest.mark.parametrize("mode", ["accurate_relative_bbox", "reference_rule_fixed"])
def test_every_barnes_hut_shape_bit_exact_reference_math(gs, orc, mode):
    n, steps = 3000, 3
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, n, size=100.0, seed=61)
    if mode == "accurate_relative_bbox":
        prm = dict(algorithm=1, box_mode=1, math_mode=1, accuracy_parameter=1.0, relative_accuracy=0.006,
                   relative_theta_floor=0.2, flags=0x170)
        okw = dict(box_mode=1, theta=1.0, flags=orc.ACCURATE | orc.RELATIVE_MAC, rel_alpha=0.006, rel_floor=0.2)
    else:
        prm = dict(algorithm=1, box_mode=0, math_mode=1, accuracy_parameter=1.0, flags=0)
        okw = dict(box_mode=0, theta=1.0)
    st = orc.State(pos, vel, mass)
    want = []
    for _ in range(steps):
        orc.bh_step(st, keep_tree=False, **okw)
        want.append(np.concatenate([a.ravel() for a in (st.pos[st.inp], st.vel[st.inp], st.mass[st.inp])])
                    .view(np.uint32).copy())
    count = 0
    for sh in _bh_shapes(gs):
        with gs.Simulation(pos, vel, mass, params=gs.default_params(**prm)) as sim:
            sim.set_shape(sh)
            for k in range(steps):
                sim.run(1)
                got = _words(sim)
                assert np.array_equal(got, want[k]), (sh.as_dict(), k)
        count += 1
    assert count == 144


def test_direct_shapes(gs, orc):
    """Targets per thread change no bit; every j-split stays within FP32 tolerance of the
    oracle's sequential sum; REFERENCE math ignores both."""
    n = 5000
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, n, size=100.0, seed=62)
    st = orc.State(pos, vel, mass)
    orc.direct_step(st)
    _, ov, _ = st.current()
    for bps in (4, 8, 12, 16, 24):
        got = []
        for ipt in (2, 4):
            sh = gs.shape_defaults()
            sh.direct_targets, sh.direct_blocks_per_sm = ipt, bps
            with gs.Simulation(pos, vel, mass, algorithm=gs.DIRECT_SUM) as sim:
                try:
                    sim.set_shape(sh)
                except gs.GsimError as e:  # more j-chunks than the default split's scratch holds
                    assert e.status == 7 and bps > 12
                    continue
                sim.run(1)
                got.append(sim.get_particles()[1])
        if len(got) == 2:
            assert np.array_equal(got[0].view(np.uint32), got[1].view(np.uint32))
        for g in got:
            assert np.max(np.abs(g - ov)) <= 1e-4 * np.abs(ov).max() + 1e-7
    ref = []
    for ipt in (2, 4):
        with gs.Simulation(pos, vel, mass, algorithm=gs.DIRECT_SUM, math_mode=gs.MATH_REFERENCE) as sim:
            sim.set_shape(direct_targets=ipt, direct_blocks_per_sm=4)
            sim.run(1)
            ref.append(sim.get_particles()[1])
    _, ov_exact, _ = st.current()
    for r in ref:
        np.testing.assert_array_equal(r, ov_exact)


def test_batch_shapes_bit_identical_to_alone(gs):
    """The batched kernels under every value of every knob (one at a time from the
    defaults): each member ends bit-identical to the same system stepped alone."""
    specs = [(17, 20000, dict(algorithm=1, box_mode=1, accuracy_parameter=1.0, relative_accuracy=0.006,
                              relative_theta_floor=0.2, flags=0x170)),
             (16, 6000, dict(algorithm=1, box_mode=1, accuracy_parameter=1.0, relative_accuracy=0.006,
                             relative_theta_floor=0.2, flags=0x170)),
             (16, 2000, dict(algorithm=0))]
    inputs = [gs.generate(k, n, size=100.0, seed=70 + j) for j, (k, n, _) in enumerate(specs)]
    alone = []
    for (k, n, prm), (p, v, m) in zip(specs, inputs):
        with gs.Simulation(p, v, m, params=gs.default_params(**prm)) as s:
            s.run(2)
            alone.append(_words(s))
    variants = [dict(sort_keys_per_thread=8), dict(sort_lookback=8), dict(sort_lookback=16), dict(scan_lookback=64),
                dict(scan_lookback=128), dict(force_warps=1), dict(force_warps=4), dict(force_short_lists=1),
                dict(moment_blocks_per_sm=1), dict(direct_targets=4)]
    for var in variants:
        sims = [gs.Simulation(p, v, m, params=gs.default_params(**prm)) for (_, _, prm), (p, v, m) in zip(specs, inputs)]
        with gs.Batch(sims) as b:
            b.set_shape(**var)
            b.run(2)
            b.sync()
        for j, s in enumerate(sims):
            assert np.array_equal(_words(s), alone[j]), (var, j)
            s.close()


def test_tuner_picks_caches_and_reloads(gs, tmp_path):
    """gs_tune_shape measures candidates and keeps the fastest; the JSON cache it writes
    loads back into a cleared table, and gs_create then gives the tuned shape to a system
    of the same key (device, parameters, log2 N)."""
    cache = str(tmp_path / "shapes.json")
    bh = gs.default_params(algorithm=1, box_mode=1, accuracy_parameter=1.0, relative_accuracy=0.006,
                           relative_theta_floor=0.2, flags=0x170)
    r = gs.tune_shape(bh, 40000, generator=gs.GEN_SPIRAL, seed=5, steps=3, cache_path=cache)
    assert r.candidates >= 9 and 0 < r.best_ms <= r.default_ms
    d = gs.default_params(algorithm=0)
    rd = gs.tune_shape(d, 8192, generator=gs.GEN_UNIFORM_DISK, seed=5, steps=3, cache_path=cache)
    assert rd.candidates >= 3 and 0 < rd.best_ms <= rd.default_ms
    doc = json.load(open(cache))
    assert doc["format"] == "gsim-shapes-1" and len(doc["entries"]) == 2
    gs.clear_shape_table()
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 40000, seed=6)
    with gs.Simulation(pos, vel, mass, params=bh) as s:
        assert s.shape().as_dict() == gs.shape_defaults().as_dict()
    assert gs.load_shape_cache(cache) == 2
    with gs.Simulation(pos, vel, mass, params=bh) as s:
        assert s.shape().as_dict() == r.best.as_dict()
    p2, v2, m2 = gs.generate(gs.GEN_UNIFORM_DISK, 9000, seed=6)  # same log2 bucket as 8192
    with gs.Simulation(p2, v2, m2, params=d) as s:
        assert s.shape().as_dict() == rd.best.as_dict()
    gs.clear_shape_table()
    os.remove(cache)


def test_batch_tuner(gs):
    prm = dict(algorithm=1, box_mode=1, accuracy_parameter=1.0, relative_accuracy=0.006, relative_theta_floor=0.2,
               flags=0x170)
    sims = [gs.Simulation(*gs.generate(17, n, size=100.0, seed=80 + n), params=gs.default_params(**prm))
            for n in (30000, 9000, 3000)]
    with gs.Batch(sims) as b:
        r = b.tune(steps=2)
        assert r.candidates >= 10 and 0 < r.best_ms <= r.default_ms
        assert b.shape().as_dict() == r.best.as_dict()
        b.run(1)
        b.sync()
    for s in sims:
        s.close()
    gs.clear_shape_table()
