"""Host transfers through the C ABI: pinned host arrays are read and written in place by a
kernel, any other host memory goes through the copy engine.  Both routes must leave the
same bits on the device and in the caller's arrays (ParticleSystem::SetParticles /
GetParticles, src/Particles/ParticleSystem.cpp:206-217)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(torch, a, offset=0):
    """A float32 copy of `a` in pinned host memory, starting `offset` floats into the
    allocation (offset 1 gives an address that is 4- but not 8-byte aligned, offset 2 one
    that is 8- but not 16-byte aligned)."""
    flat = np.ascontiguousarray(a, np.float32).ravel()
    buf = torch.empty(flat.size + offset, dtype=torch.float32).pin_memory().numpy()
    out = buf[offset:offset + flat.size]
    out[:] = flat
    return out.reshape(a.shape)


def _params(gs):
    return gs.default_params(algorithm=gs.BARNES_HUT, box_mode=gs.BOX_BOUNDING, accuracy_parameter=1.0,
                             relative_accuracy=0.006, relative_theta_floor=0.2,
                             flags=gs.FLAGS_ACCURATE | gs.FLAG_RELATIVE_MAC | gs.FLAG_COUNT_INTERACTIONS)


def _words(sim):
    p, v, m = sim.get_particles()
    return np.concatenate([p.ravel(), v.ravel(), m.ravel()]).view(np.uint32)


def _get_into(gs, sim, pos, vel, mass):
    gs._check(gs.lib().gs_get_particles(sim.handle, gs._fp(pos), gs._fp(vel), gs._fp(mass)))


@pytest.mark.parametrize("offset", [0, 1, 2])
def test_pinned_upload_matches_pageable(gs, offset):
    torch = pytest.importorskip("torch")
    n = 5000  # not a multiple of 64: the padding slots are written too
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, n, size=100.0, seed=11)
    a = gs.Simulation(pos, vel, mass, params=_params(gs))
    b = gs.Simulation(_pinned(torch, pos, offset), _pinned(torch, vel, offset), _pinned(torch, mass, offset),
                      params=_params(gs))
    for s in (a, b):
        s.reset_stats()
        s.run(3)
    assert np.array_equal(_words(a), _words(b))
    assert a.stats().interactions == b.stats().interactions
    # a new state without velocities: both routes zero them and forget the previous |a|
    p2, _, m2 = gs.generate(gs.GEN_UNIFORM_DISK, n, size=100.0, seed=12)
    gs._check(gs.lib().gs_set_particles(a.handle, gs._fp(p2), None, gs._fp(m2)))
    gs._check(gs.lib().gs_set_particles(b.handle, gs._fp(_pinned(torch, p2, offset)), None,
                                        gs._fp(_pinned(torch, m2, offset))))
    for s in (a, b):
        s.reset_stats()
        s.run(1)
    assert np.array_equal(_words(a), _words(b))
    assert a.stats().interactions == b.stats().interactions
    a.close()
    b.close()


@pytest.mark.parametrize("offset", [0, 1, 2])
def test_pinned_readback_matches_pageable(gs, offset):
    torch = pytest.importorskip("torch")
    n = 3001
    pos, vel, mass = gs.generate(gs.GEN_GALAXY, n, size=100.0, seed=13)
    with gs.Simulation(pos, vel, mass, params=_params(gs)) as sim:
        sim.run(2)
        p, v, m = sim.get_particles()  # pageable: copy engine
        hp = _pinned(torch, np.full((n, 2), np.nan, np.float32), offset)
        hv = _pinned(torch, np.full((n, 2), np.nan, np.float32), offset)
        hm = _pinned(torch, np.full(n, np.nan, np.float32), offset)
        _get_into(gs, sim, hp, hv, hm)
        assert np.array_equal(hp.view(np.uint32), p.view(np.uint32))
        assert np.array_equal(hv.view(np.uint32), v.view(np.uint32))
        assert np.array_equal(hm.view(np.uint32), m.view(np.uint32))
        # only some arrays asked for: the others stay untouched
        hp[:] = np.nan
        hm[:] = np.nan
        _get_into(gs, sim, hp, None, None)
        assert np.array_equal(hp.view(np.uint32), p.view(np.uint32))
        assert np.all(np.isnan(hm))


def test_timeout_leaves_pinned_arrays_in_use(gs):
    """A transfer whose bounded wait runs out returns GS_ERR_TIMEOUT with its kernel still
    queued behind the submitted steps; the pinned arrays stay in use until gs_sync
    succeeds, and then hold what the call promised (include/gsim.h)."""
    torch = pytest.importorskip("torch")
    n = 131072  # direct sum: about 7 ms per step, so 20 steps outlast a 1 ms bound
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, n, size=100.0, seed=21)
    with gs.Simulation(pos, vel, mass, algorithm=gs.DIRECT_SUM) as sim, \
            gs.Simulation(pos, vel, mass, algorithm=gs.DIRECT_SUM) as ref:
        ref.run(20)
        want = _words(ref)
        hp = _pinned(torch, np.full((n, 2), np.nan, np.float32))
        hv = _pinned(torch, np.full((n, 2), np.nan, np.float32))
        hm = _pinned(torch, np.full(n, np.nan, np.float32))
        sim.run(20)
        sim.set_timeout(1000000)  # 1 ms
        st = gs.lib().gs_get_particles(sim.handle, gs._fp(hp), gs._fp(hv), gs._fp(hm))
        assert st == 4  # GS_ERR_TIMEOUT: the steps are still running
        sim.set_timeout(0)
        sim.sync()
        got = np.concatenate([hp.ravel(), hv.ravel(), hm.ravel()]).view(np.uint32)
        assert np.array_equal(got, want)  # the queued readback wrote them after the steps

        # an upload behind running steps: after the timeout and a successful sync, the
        # state is the uploaded one
        p2, v2, m2 = gs.generate(gs.GEN_SPIRAL, n, size=100.0, seed=22)
        sim.run(20)
        up = [_pinned(torch, a) for a in (p2, v2, m2)]  # in use until the sync below
        sim.set_timeout(1000000)
        st = gs.lib().gs_set_particles(sim.handle, *[gs._fp(a) for a in up])
        assert st == 4
        sim.set_timeout(0)
        sim.sync()
        del up
        p, v, m = sim.get_particles()
        assert np.array_equal(p, p2) and np.array_equal(v, v2) and np.array_equal(m, m2)
