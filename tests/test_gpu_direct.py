"""Direct-sum CUDA path (through the C ABI) against the CPU restatement of SimShader.comp.

REFERENCE math: bit-identical to the oracle.  FAST math (hardware rsqrt, Kahan tile
sums): accelerations within 2e-6 relative (RMS) of the FP64 direct sum and within
2e-5 (max per particle, relative to |a|) of the FP32 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(gs, pos, vel, mass, **kw):
    p = gs.default_params(algorithm=gs.DIRECT_SUM, **kw)
    return gs.Simulation(pos, vel, mass, params=p)


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 1000, 4096])
def test_reference_math_bit_exact(gs, orc, n):
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, n, seed=100 + n)
    vel = (0.1 * np.random.default_rng(n).standard_normal(pos.shape)).astype(np.float32)
    st = orc.State(pos, vel, mass)
    with _sim(gs, pos, vel, mass, math_mode=gs.MATH_REFERENCE) as sim:
        for step in range(3):
            sim.run(1)
            orc.direct_step(st)
            gp, gv, gm = sim.get_particles()
            op, ov, om = st.current()
            np.testing.assert_array_equal(gp, op)
            np.testing.assert_array_equal(gv, ov)
            np.testing.assert_array_equal(gm, om)


def test_config1_reference_math_10_steps(gs, orc):
    # N=4096 uniform disk r=100, v=0, m in [1,10], G=1, dt=1e-3, softening 0.2, 10 steps
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, 4096, size=100.0, seed=1001)
    st = orc.State(pos, vel, mass)
    with _sim(gs, pos, vel, mass, math_mode=gs.MATH_REFERENCE) as sim:
        sim.run(10)
        for _ in range(10):
            orc.direct_step(st)
        gp, gv, _ = sim.get_particles()
    op, ov, _ = st.current()
    np.testing.assert_array_equal(gp, op)
    np.testing.assert_array_equal(gv, ov)


@pytest.mark.parametrize("n,kind", [(4096, 16), (1000, 0), (20000, 18), (50000, 18)])
def test_fast_math_accuracy(gs, orc, n, kind):
    size = 100.0
    pos, vel, mass = gs.generate(kind, n, size=size, seed=7)
    with _sim(gs, pos, vel, mass, flags=gs.FLAG_RECORD_ACCEL) as sim:
        sim.run(1)
        acc = sim.get_accel().astype(np.float64)
        targets = np.arange(0, n, max(1, n // 4096), dtype=np.uint32)
        # the step changed positions; recompute FP64 on the initial state with a fresh sim
    P, V, M = orc.pad_state(pos, vel, mass)
    a64 = orc.direct_accel_f64(P, M, targets=targets)
    a32 = orc.direct_accel(P, M)[targets].astype(np.float64)
    g = acc[targets]
    den = np.linalg.norm(a64, axis=1)
    err_gpu = np.linalg.norm(g - a64, axis=1) / den
    err_orc = np.linalg.norm(a32 - a64, axis=1) / den
    assert np.sqrt(np.mean(err_gpu ** 2)) < 2e-6, np.sqrt(np.mean(err_gpu ** 2))
    assert np.sqrt(np.mean(err_gpu ** 2)) <= np.sqrt(np.mean(err_orc ** 2)) * 1.5
    assert np.max(np.linalg.norm(g - a32, axis=1) / den) < 2e-4


def test_fast_math_config1_trajectory(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, 4096, size=100.0, seed=1001)
    st = orc.State(pos, vel, mass)
    with _sim(gs, pos, vel, mass) as sim:
        sim.run(10)
        for _ in range(10):
            orc.direct_step(st)
        gp, gv, _ = sim.get_particles()
    op, ov, _ = st.current()
    np.testing.assert_allclose(gp, op, rtol=0, atol=1e-5)
    scale = np.abs(ov).max()
    assert np.max(np.abs(gv - ov)) < 1e-4 * scale


def test_fast_math_momentum(gs):
    pos, vel, mass = gs.generate(gs.GEN_GALAXY, 10000, size=100.0, seed=5)
    with _sim(gs, pos, vel, mass) as sim:
        sim.run(20)
        p, v, m = sim.get_particles()
    p0 = (mass[:, None].astype(np.float64) * vel).sum(0)
    p1 = (m[:, None].astype(np.float64) * v).sum(0)
    scale = np.abs(mass[:, None] * vel).sum()
    assert np.all(np.abs(p1 - p0) < 1e-5 * scale)


def test_accel_f64_matches_oracle(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 3000, seed=3)
    with _sim(gs, pos, vel, mass) as sim:
        t = np.arange(0, 3000, 7, dtype=np.uint32)
        g = sim.accel_f64(t)
    P, V, M = orc.pad_state(pos, vel, mass)
    o = orc.direct_accel_f64(P, M, targets=t)
    np.testing.assert_allclose(g, o, rtol=1e-11, atol=1e-14)


def test_run_zero_and_async_batches(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_RANDOM, 500, seed=2)
    st = orc.State(pos, vel, mass)
    with _sim(gs, pos, vel, mass, math_mode=gs.MATH_REFERENCE) as sim:
        sim.run(0)  # the reference's first call asks for 0 steps (src/Main.cpp:270-283)
        for k in (3, 0, 2, 5):
            sim.run(k)
            for _ in range(k):
                orc.direct_step(st)
        gp, gv, _ = sim.get_particles()
    np.testing.assert_array_equal(gp, st.current()[0])
    np.testing.assert_array_equal(gv, st.current()[1])


def test_energy_f64_matches_oracle(gs, orc):
    """gs_energy_f64 (GPU, FP64) against the CPU FP64 energy of the oracle."""
    pos, vel, mass = gs.generate(gs.GEN_EXP_DISK_COLLISION, 3000, seed=77)
    with _sim(gs, pos, vel, mass) as sim:
        ke, pe = sim.energy_f64()
    e_orc = orc.energy_f64(pos, vel, mass, G=1.0, softening=0.2)
    ke_ref = 0.5 * np.sum(mass.astype(np.float64) * np.sum(vel.astype(np.float64) ** 2, axis=1))
    assert abs(ke - ke_ref) <= 1e-12 * abs(ke_ref)
    assert abs((ke + pe) - e_orc) <= 1e-10 * abs(e_orc)
    assert pe < 0.0


def test_plain_sum_variant(gs):
    """GS_FLAG_PLAIN_SUM: the uncompensated tile sums stay close to FP64 but no closer
    than the compensated ones on average; it is rejected for Barnes-Hut and in a batch
    with compensated direct-sum members."""
    n = 20000
    pos, vel, mass = gs.generate(gs.GEN_EXP_DISK_COLLISION, n, seed=3)
    sub = np.arange(0, n, 10, dtype=np.uint32)
    err = {}
    for flag in (0, gs.FLAG_PLAIN_SUM):
        with _sim(gs, pos, vel, mass, flags=flag | gs.FLAG_RECORD_ACCEL) as sim:
            sim.run(1)
            acc = sim.get_accel()[sub].astype(np.float64)
            sim.set_particles(pos, vel, mass)
            a64 = sim.accel_f64(sub)
        e = np.linalg.norm(acc - a64, axis=1) / np.linalg.norm(a64, axis=1)
        err[flag] = np.sqrt(np.mean(e ** 2))
    assert err[gs.FLAG_PLAIN_SUM] < 1e-4
    assert err[0] <= err[gs.FLAG_PLAIN_SUM]
    with pytest.raises(gs.GsimError):
        gs.Simulation(pos, vel, mass, params=gs.default_params(algorithm=gs.BARNES_HUT, flags=gs.FLAG_PLAIN_SUM))
    a = _sim(gs, pos[:500], vel[:500], mass[:500])
    b = _sim(gs, pos[:700], vel[:700], mass[:700], flags=gs.FLAG_PLAIN_SUM)
    with pytest.raises(gs.GsimError):
        gs.Batch([a, b])
