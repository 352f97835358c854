"""gsim-cli: the headless command line with the reference's flags (src/Main.cpp:20-48),
built on the C++ mirror include/gsim.hpp."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "gravity-sim_gb300", "lib", "gsim-cli")


def _run(args, **kw):
    return subprocess.run([CLI] + args, capture_output=True, text=True, timeout=600, **kw)


def test_help_exits(gs):
    r = _run(["--help"])
    assert r.returncode == 0 and "--simulation-algorithm" in r.stdout and "--particles-out" in r.stdout


def test_argument_checks(gs):
    r = _run(["--simulation-algorithm=barnes-hut", "--simulation-count=5"])
    assert r.returncode == 1 and "generation args" in r.stdout
    r = _run(["--particle-count=10", "--generate-type=random", "--generate-size=10", "--min-mass=1",
              "--max-mass=2", "--simulation-count=5"])
    assert r.returncode == 1 and "simulation algorithm" in r.stdout
    r = _run(["--particle-count=10", "--generate-type=random", "--generate-size=10", "--min-mass=1",
              "--max-mass=2", "--simulation-algorithm=direct-sum"])
    assert r.returncode == 1 and "simulation count" in r.stdout
    r = _run(["--particle-count=10", "--generate-type=random", "--generate-size=10", "--min-mass=1",
              "--max-mass=2", "--simulation-algorithm=barnes-hut", "--simulation-count=5",
              "--relative-accuracy=0.006"])
    assert r.returncode == 1 and "needs --accurate" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("algo,extra", [("barnes-hut", ["--math=reference"]), ("direct-sum", []),
                                        ("barnes-hut", ["--box=bbox", "--accurate", "--accuracy-parameter=0.35"]),
                                        ("barnes-hut", ["--box=bbox", "--accurate", "--accuracy-parameter=1",
                                                        "--relative-accuracy=0.006", "--relative-floor=0.2"]),
                                        ("barnes-hut", ["--box=bbox", "--key-bits=15", "--accurate",
                                                        "--accuracy-parameter=0.5"])])
def test_file_roundtrip_matches_binding(gs, tmp_path, algo, extra):
    pos, vel, mass = gs.generate(gs.GEN_GALAXY, 3000, size=100.0, seed=17)
    fin, fout = str(tmp_path / "in.txt"), str(tmp_path / "out.txt")
    gs.write_particles(fin, pos, vel, mass)
    r = _run([f"--particles-in={fin}", f"--particles-out={fout}", f"--simulation-algorithm={algo}",
              "--simulation-count=7", "--no-graphics", "--benchmark"] + extra)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Average runtime/simulation" in r.stdout
    p2, v2, m2 = gs.read_particles(fin)  # the values the CLI started from
    kw = dict(algorithm=gs.BARNES_HUT if algo == "barnes-hut" else gs.DIRECT_SUM)
    if "--math=reference" in extra:
        kw["math_mode"] = gs.MATH_REFERENCE
    if "--box=bbox" in extra:
        kw.update(box_mode=gs.BOX_BOUNDING, flags=gs.FLAGS_ACCURATE,
                  accuracy_parameter=float([a for a in extra if a.startswith("--accuracy-parameter=")][0][21:]))
    if "--key-bits=15" in extra:
        kw["key_bits"] = 15
    if "--relative-accuracy=0.006" in extra:
        kw.update(flags=gs.FLAGS_ACCURATE | gs.FLAG_RELATIVE_MAC, relative_accuracy=0.006, relative_theta_floor=0.2)
    with gs.Simulation(p2, v2, m2, **kw) as sim:
        sim.run(7)
        p, v, m = sim.get_particles()
    fref = str(tmp_path / "ref.txt")
    gs.write_particles(fref, p, v, m)
    assert open(fout).read() == open(fref).read()


@pytest.mark.gpu
def test_image_out_matches_binding(gs, orc, tmp_path):
    """--image-out draws the final state with the start camera of the initial state,
    widened to the image's aspect ratio."""
    pos, vel, mass = gs.generate(gs.GEN_GALAXY, 2000, size=100.0, seed=5)
    fin, img = str(tmp_path / "in.txt"), str(tmp_path / "frame.ppm")
    gs.write_particles(fin, pos, vel, mass)
    r = _run([f"--particles-in={fin}", f"--image-out={img}", "--image-size=160x90", "--simulation-algorithm=direct-sum",
              "--simulation-count=3"])
    assert r.returncode == 0, r.stdout + r.stderr
    p2, v2, m2 = gs.read_particles(fin)
    with gs.Simulation(p2, v2, m2, algorithm=gs.DIRECT_SUM) as sim:
        cam = sim.camera_start()
        cam[2] = cam[3] * (np.float32(160.0) / np.float32(90.0))
        sim.run(3)
        expect = sim.render(160, 90, cam)
    data = open(img, "rb").read()
    header = b"P6\n160 90\n255\n"
    assert data.startswith(header)
    got = np.frombuffer(data[len(header):], np.uint8).reshape(90, 160, 3)[:, :, 0]
    assert np.array_equal(got, expect) and got.any()
