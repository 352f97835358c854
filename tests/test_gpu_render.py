"""Headless point splat (gs_render_points) and the snapshot ring, through the C ABI.

The image must equal the CPU restatement of VertShader.vert / FragShader.frag byte for
byte; snapshots must hold the state of the moment they were taken while later steps
run, and a ticket whose slot was reused must be refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _direct(gs, pos, vel, mass):
    return gs.Simulation(pos, vel, mass, params=gs.default_params(algorithm=gs.DIRECT_SUM))


CAMERAS = [
    (0.0, 0.0, 200.0, 200.0),        # the whole disk
    (10.0, -5.0, 50.0, 30.0),        # zoomed, off centre, non-square
    (0.0, 0.0, 200.0 * 16 / 9, 200.0),  # the reference's size * aspect / zoom form
    (-100.0, 100.0, 1.0, 1.0),       # almost nothing in view
]


@pytest.mark.parametrize("width,height", [(64, 48), (640, 360), (1, 1), (1920, 1080)])
def test_render_matches_oracle(gs, orc, width, height):
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 20000, seed=11)
    # points on the view edges and non-finite positions
    extra = np.array([[-100.0, 0.0], [100.0, 0.0], [0.0, 100.0], [0.0, -100.0], [np.nan, 0.0], [np.inf, 1.0],
                      [-np.inf, -np.inf], [99.999, 99.999]], np.float32)
    pos = np.concatenate([pos, extra]).astype(np.float32)
    vel = np.concatenate([vel, np.zeros_like(extra)]).astype(np.float32)
    mass = np.concatenate([mass, np.ones(len(extra), np.float32)])
    with _direct(gs, pos, vel, mass) as sim:
        for cam in CAMERAS:
            img = sim.render(width, height, cam)
            ref = orc.render_points(pos, cam, width, height)
            assert np.array_equal(img, ref), cam
            assert set(np.unique(img)) <= {0, 255}


def test_camera_start_is_the_reference_extent(gs):
    pos, vel, mass = gs.generate(gs.GEN_EXP_DISK_COLLISION, 5000, seed=2)
    with _direct(gs, pos, vel, mass) as sim:
        cam = sim.camera_start()
    mn, mx = pos.min(axis=0), pos.max(axis=0)
    w, h = np.float32(mx[0] - mn[0]), np.float32(mx[1] - mn[1])
    assert cam[0] == np.float32((mn[0] + mx[0]) * np.float32(0.5))
    assert cam[1] == np.float32((mn[1] + mx[1]) * np.float32(0.5))
    assert cam[2] == cam[3] == max(w, h)


def test_snapshot_holds_its_moment_while_steps_run(gs, orc):
    pos, vel, mass = gs.generate(gs.GEN_SPIRAL, 30000, seed=4)
    with _direct(gs, pos, vel, mass) as sim:
        sim.run(2)
        at_take, _, _ = sim.get_particles()
        t1 = sim.snapshot(2)
        sim.run(5)  # enqueued after the copy; the snapshot must not see these steps
        snap = sim.snapshot_positions(t1)
        assert np.array_equal(snap, at_take)
        cam = (0.0, 0.0, 220.0, 220.0)
        assert np.array_equal(sim.snapshot_render(t1, 320, 200, cam), orc.render_points(at_take, cam, 320, 200))
        now, _, _ = sim.get_particles()
        assert not np.array_equal(now, at_take)
        t2 = sim.snapshot(2)
        assert np.array_equal(sim.snapshot_positions(t2), now)
        t3 = sim.snapshot(2)  # reuses the slot of t1
        with pytest.raises(gs.GsimError):
            sim.snapshot_positions(t1)
        assert np.array_equal(sim.snapshot_positions(t3), now)
        with pytest.raises(gs.GsimError):
            sim.snapshot(3)  # the ring of this system has 2 slots


def test_write_ppm(gs, tmp_path):
    pos = np.array([[0.0, 0.0], [0.9, 0.9]], np.float32)
    vel = np.zeros_like(pos)
    mass = np.ones(2, np.float32)
    with _direct(gs, pos, vel, mass) as sim:
        img = sim.render(4, 3, (0.0, 0.0, 2.0, 2.0))
    f = str(tmp_path / "frame.ppm")
    gs.write_ppm(f, img)
    data = open(f, "rb").read()
    header = b"P6\n4 3\n255\n"
    assert data[:len(header)] == header
    body = np.frombuffer(data[len(header):], np.uint8).reshape(3, 4, 3)
    assert np.array_equal(body[:, :, 0], img) and np.array_equal(body[:, :, 1], img)
