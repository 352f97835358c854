"""The CPU restatement of SimShader.comp (oracle) against FP64 and the physical
invariants the reference's direct sum implies (no GPU)."""
import numpy as np
import pytest


def _rel_err(a, ref):
    num = np.linalg.norm(a - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    return num / np.maximum(den, 1e-30)


def test_fp32_accel_close_to_fp64(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, 2048, seed=11)
    a32 = orc.direct_accel(pos, mass)
    a64 = orc.direct_accel_f64(pos, mass)
    err = _rel_err(a32.astype(np.float64), a64)
    assert np.sqrt(np.mean(err ** 2)) < 1e-4
    assert np.median(err) < 2e-5


def test_momentum_conserved(gs, orc):
    # Newton's third law: pair forces cancel, so total momentum changes only by rounding.
    pos, vel, mass = gs.generate(gs.GEN_GALAXY, 1000, size=100.0, seed=5)
    st = orc.State(pos, vel, mass)
    p0 = (mass[:, None] * vel).sum(0)
    scale = np.abs(mass[:, None] * vel).sum()
    for _ in range(5):
        orc.direct_step(st)
    p, v, m = st.current()
    p1 = (m[:, None].astype(np.float64) * v).sum(0)
    assert np.all(np.abs(p1 - p0) < 1e-5 * scale)


def test_permutation_invariant(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_RANDOM, 777, seed=3)
    perm = np.random.default_rng(0).permutation(777)
    a = orc.direct_accel(pos, mass)
    b = orc.direct_accel(pos[perm], mass[perm])
    np.testing.assert_allclose(b, a[perm], rtol=1e-4, atol=1e-3 * np.abs(a).max() * 1e-3)


def test_mirror_symmetry(gs, orc):
    # symmetrical-galaxy-collision pairs (i, i+1) are x-mirror images (ParticleSystem.cpp:127-148)
    pos, vel, mass = gs.generate(gs.GEN_SYMMETRICAL_GALAXY_COLLISION, 1024, size=300.0, seed=9)
    np.testing.assert_array_equal(pos[1::2, 0], -pos[0::2, 0])
    a = orc.direct_accel_f64(pos, mass)
    np.testing.assert_allclose(a[1::2, 0], -a[0::2, 0], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(a[1::2, 1], a[0::2, 1], rtol=1e-9, atol=1e-12)


def test_two_body_circular_orbit(orc):
    # two unit masses at distance 2r circle their centre of mass: m v^2 / r = G m^2 / (2r)^2.
    # Softening must be > 0: the self term of the shader is 0 * inf otherwise.
    r = 1.0
    v = np.sqrt(r / 4.0) / r
    pos = np.array([[-r, 0.0], [r, 0.0]], np.float32)
    vel = np.array([[0.0, -v], [0.0, v]], np.float32)
    mass = np.ones(2, np.float32)
    st = orc.State(pos, vel, mass)
    for _ in range(2000):
        orc.direct_step(st, dt=1e-3, softening=1e-3)
    p, _, _ = st.current()
    d = np.linalg.norm(p[0] - p[1])
    assert abs(d - 2 * r) < 1e-3
    ang = np.arctan2(p[1, 1] - p[0, 1], p[1, 0] - p[0, 0])
    assert abs(ang - (v / r) * 2.0) < 5e-3  # angular speed v / r over 2 time units


def test_reference_padding_and_step_shape(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_RANDOM, 63, seed=1)
    st = orc.State(pos, vel, mass)
    assert st.n_al == 64
    orc.direct_step(st)
    p, v, m = st.current()
    assert p.shape == (63, 2) and np.all(np.isfinite(p)) and np.array_equal(m, mass)


def test_render_points_pixel_mapping(orc):
    """The oracle's point splat: screen = (p - c) / size, y flipped, pixel = floor((s + 1) * n / 2)."""
    cam = (0.0, 0.0, 2.0, 2.0)
    pos = np.array([[0.0, 0.0], [-1.0, 1.0], [0.99, -0.99], [1.0, 0.0], [-1.01, 0.0]], np.float32)
    img = orc.render_points(pos, cam, 4, 4)
    # (0, 0) -> screen (0, 0) -> pixel (2, 2); (-1, 1) -> screen (-0.5, -0.5) -> (1, 1)
    # (0.99, -0.99) -> screen (0.495, 0.495) -> (2, 2) again; x = 1 lands at 3.0 -> pixel 3;
    # x = -1.01 -> screen -0.505 -> 0.99 -> pixel 0
    expect = np.zeros((4, 4), np.uint8)
    expect[2, 2] = expect[1, 1] = expect[2, 3] = expect[2, 0] = 255
    assert np.array_equal(img, expect)
    assert not orc.render_points(np.array([[5.0, 5.0]], np.float32), cam, 4, 4).any()


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 16, 17, 18])
def test_generators_restated_bit_exact(gs, orc, kind):
    """The oracle's generators (used where the library must not be loaded) give the
    library's particles bit for bit."""
    for n, seed in ((1000, 1), (4096, 1001), (20001 if kind != 3 else 20000, 77)):
        a = gs.generate(kind, n, size=100.0, seed=seed)
        b = orc.generate(kind, n, size=100.0, seed=seed)
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
