"""Continuous batching of simulation requests (gs_server_*).

The mix test is the serving contract: every request's final state, computed while other
requests join and leave the batch around it, is bit-identical to the same system run
alone with gs_run.  The other tests hold the admission rules (memory budget, particle
cap, order) and the edge cases (no steps, caller-given particles, rejected requests)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEN = (16, 17, 18)  # uniform disk, spiral galaxy, two-disk collision


def _params(gs):
    d = gs.default_params(algorithm=gs.DIRECT_SUM)
    b = gs.default_params(algorithm=gs.BARNES_HUT, box_mode=gs.BOX_BOUNDING, accuracy_parameter=0.5,
                          flags=gs.FLAGS_ACCURATE)
    return d, b


def _alone(gs, req, d, b, crossover):
    pos, vel, mass = gs.generate(req.generator, req.particle_count, size=req.generate_size, seed=req.seed)
    p = d if req.particle_count < crossover else b
    with gs.Simulation(pos, vel, mass, params=p) as sim:
        if req.steps:
            sim.run(req.steps)
        return sim.get_particles()


def _same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))


def test_results_same_alone_and_in_mix(gs):
    d, b = _params(gs)
    crossover = 3000
    rng = np.random.default_rng(11)
    reqs, arrivals = [], []
    for j in range(14):
        n = int(np.exp(rng.uniform(np.log(500), np.log(60000))))
        reqs.append(gs.make_request(n, int(rng.integers(3, 25)), int(rng.choice(GEN)), seed=100 + j))
        arrivals.append(0.002 * j)  # they arrive while earlier ones run
    with gs.Server(64 << 30, crossover, d, b, keep_results=True) as srv:
        ids = srv.run_trace(reqs, arrivals, timeout_s=120)
        st = srv.stats()
        assert st["finished"] == len(reqs) and st["failed"] == 0
        assert st["plan_changes"] >= 2  # members joined and left between steps
        for r, i in zip(reqs, ids):
            info = srv.request(i)
            assert info.state == gs.REQUEST_DONE and info.steps_enqueued == r.steps
            assert info.arrival_s <= info.admit_s <= info.finish_s
            assert info.algorithm == (gs.DIRECT_SUM if r.particle_count < crossover else gs.BARNES_HUT)
            _same(srv.result(i), _alone(gs, r, d, b, crossover))


def test_memory_budget_holds(gs):
    d, b = _params(gs)
    reqs = [gs.make_request(20000, 6, 17, seed=200 + j) for j in range(6)]
    fp = gs.footprint(b, 20000)
    budget = 2 * fp + fp // 2  # two at a time
    with gs.Server(budget, 1000, d, b) as srv:
        ids = srv.run_trace(reqs, [0.0] * len(reqs), timeout_s=120)
        st = srv.stats()
        assert st["finished"] == 6
        assert st["peak_memory_in_use"] <= budget
        assert st["peak_memory_in_use"] == 2 * fp
        assert st["memory_in_use"] == 0 and st["resident"] == 0
        admits = sorted(srv.request(i).admit_s for i in ids)
        finishes = sorted(srv.request(i).finish_s for i in ids)
        assert admits[2] >= finishes[0]  # the third waited for a slot


def _given(gs, n, steps, seed):
    """A request carrying its particles (ready at submit, unlike generator requests)."""
    pos, vel, mass = gs.generate(16, n, seed=seed)
    r = gs.Request()
    r.particle_count, r.steps = n, steps
    r.pos_xy, r.vel_xy, r.mass = gs._fp(pos), gs._fp(vel), gs._fp(mass)
    return r, (pos, vel, mass)


def _drain(srv, count, limit=100000):
    for _ in range(limit):
        if srv.stats()["finished"] + srv.stats()["failed"] >= count:
            return
        srv.poll()
    raise AssertionError("requests did not finish")


def test_particle_cap_and_shortest_first(gs):
    d, b = _params(gs)
    work = [(4000, 40), (4000, 5), (4000, 20), (4000, 10)]
    given = [_given(gs, n, k, 300 + j) for j, (n, k) in enumerate(work)]
    with gs.Server(64 << 30, 100, d, b, max_resident_particles=4000, policy=gs.SERVE_SHORTEST_FIRST) as srv:
        ids = [srv.submit(r, 0.0) for r, _ in given]
        for _ in range(100000):
            if srv.stats()["finished"] >= len(given):
                break
            srv.poll()
            assert srv.stats()["resident_particles"] <= 4000
        assert srv.stats()["finished"] == len(given)
        order = sorted(range(len(given)), key=lambda j: srv.request(ids[j]).admit_s)
        assert order == [1, 3, 2, 0]  # least N x steps first


def test_zero_steps_and_given_particles(gs):
    d, b = _params(gs)
    pos, vel, mass = gs.generate(17, 3000, seed=5)
    r = gs.Request()
    r.particle_count, r.steps = 3000, 0
    r.pos_xy, r.vel_xy, r.mass = gs._fp(pos), gs._fp(vel), gs._fp(mass)
    r2 = gs.make_request(3000, 7, 17, seed=5)
    with gs.Server(1 << 34, 1000, d, b, keep_results=True) as srv:
        a = srv.submit(r)
        c = srv.submit(r2)
        _drain(srv, 2)
        _same(srv.result(a), (pos, vel, mass))  # no steps: the input comes back
        _same(srv.result(c), _alone(gs, r2, d, b, 1000))


def test_rejects(gs):
    d, b = _params(gs)
    with gs.Server(1 << 20, 1000, d, b) as srv:
        with pytest.raises(gs.GsimError):
            srv.submit(gs.make_request(100000, 5, 17))  # footprint above the whole budget
        with pytest.raises(gs.GsimError):
            srv.submit(gs.make_request(100, 5, 99))  # no such generator
        with pytest.raises(gs.GsimError):
            srv.submit(gs.make_request(0, 5, 17))
    with pytest.raises(gs.GsimError):
        gs.Server(1 << 30, 1000, b, d)  # parameter sets swapped
