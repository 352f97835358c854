"""The C ABI library without a GPU: it loads, exports every entry point include/gsim.h
declares, and its host-only helpers (generators, particle files) behave."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^GS_API\s+[\w\s\*]+?\b(gs_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(gs):
    names = _declared("gsim.h")
    assert len(names) >= 20
    lib = ctypes.CDLL(gs.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing
    out = subprocess.run(["nm", "-D", "--defined-only", gs.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gs_\w+)", out))
    assert set(names) <= exported
    assert set(gs.EXPORTS) <= exported


def test_alignment_and_capacity(gs):
    assert gs.required_alignment(gs.DIRECT_SUM) == 64
    assert gs.required_alignment(gs.BARNES_HUT) == 64
    # leaves + at most min(4^d, n/2 + 1) internal nodes per level d (levels 0..10 / 0..15) + 64
    for box, depth in ((gs.BOX_FIXED_500, 10), (gs.BOX_BOUNDING, 15)):
        for n in (64, 640, 1 << 20):
            levels = sum(min(4 ** d, n // 2 + 1) for d in range(depth + 1))
            assert gs.node_capacity(box, n) == n + levels + 64


def test_generators_deterministic(gs):
    for kind in (gs.GEN_RANDOM, gs.GEN_GALAXY, gs.GEN_GALAXY_COLLISION, gs.GEN_SYMMETRICAL_GALAXY_COLLISION,
                 gs.GEN_UNIFORM_DISK, gs.GEN_SPIRAL, gs.GEN_EXP_DISK_COLLISION):
        a = gs.generate(kind, 1000, seed=42)
        b = gs.generate(kind, 1000, seed=42)
        c = gs.generate(kind, 1000, seed=43)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
        assert not np.array_equal(a[0], c[0])
        assert np.all(np.isfinite(a[0])) and np.all(np.isfinite(a[1]))


def test_workload_shapes(gs):
    p, v, m = gs.generate(gs.GEN_UNIFORM_DISK, 20000, size=100.0, seed=1)
    r = np.linalg.norm(p, axis=1)
    assert r.max() <= 100.0 and np.all(v == 0) and m.min() >= 1 and m.max() <= 10
    p, v, m = gs.generate(gs.GEN_SPIRAL, 20000, size=100.0, seed=1)
    r = np.linalg.norm(p, axis=1)
    assert r.max() <= 100.0 + 1e-3 and 40 < r.mean() < 70  # Gamma(2, 30) truncated at 100
    vt = (p[:, 0] * v[:, 1] - p[:, 1] * v[:, 0]) / np.maximum(r, 1e-6)
    assert np.mean(vt > 0) > 0.95  # rotating disk
    p, v, m = gs.generate(gs.GEN_EXP_DISK_COLLISION, 20000, seed=1)
    left = p[:, 0] < 0
    assert abs(left.mean() - 0.5) < 0.01
    assert abs(v[left, 1].mean() + 3.0) < 0.5 and abs(v[~left, 1].mean() - 3.0) < 0.5


def test_particle_file_roundtrip(gs, tmp_path):
    p, v, m = gs.generate(gs.GEN_GALAXY, 257, seed=3)
    f = str(tmp_path / "out.txt")
    gs.write_particles(f, p, v, m)
    lines = open(f).read().splitlines()
    assert len(lines) == 257
    expect = "%.7f %.7f %.7f %.7f %.7f" % tuple(float(x) for x in (p[0, 0], p[0, 1], v[0, 0], v[0, 1], m[0]))
    assert lines[0] == expect  # SaveParticles format, ParticleSystem.cpp:743
    p2, v2, m2 = gs.read_particles(f)
    np.testing.assert_allclose(p2, p, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(m2, m, rtol=1e-6)
    gs.write_particles(f + "2", p2, v2, m2)
    assert open(f + "2").read() == open(f).read()  # second pass is a fixed point


def test_particle_file_errors(gs, tmp_path):
    with pytest.raises(gs.GsimError):
        gs.read_particles(str(tmp_path / "missing.txt"))
    bad = tmp_path / "bad.txt"
    bad.write_text("1 2 3 4\n")
    with pytest.raises(gs.GsimError, match="at least one valid particle"):
        gs.read_particles(str(bad))
    partial = tmp_path / "partial.txt"
    partial.write_text("1 2 3 4 5\n6 7 8 9 10\n11 12 x\n")
    p, v, m = gs.read_particles(str(partial))
    assert len(m) == 2 and m[1] == 10


def test_create_rejects_bad_arguments(gs):
    p, v, m = gs.generate(gs.GEN_RANDOM, 10, seed=1)
    with pytest.raises(gs.GsimError):
        gs.Simulation(p, v, m, algorithm=7)
    with pytest.raises(gs.GsimError):
        gs.Simulation(p[:0], v[:0], m[:0])


def test_fails_loudly_without_gpu(gs):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p, v, m = gs.generate(gs.GEN_RANDOM, 10, seed=1)
    with pytest.raises(gs.GsimError) as e:
        gs.Simulation(p, v, m)
    assert e.value.status == 8  # GS_ERR_NO_DEVICE: no CPU fallback


def test_create_rejects_bad_key_bits_before_any_device_call(gs):
    """Parameter validation comes first: an out-of-range key width is refused with
    GS_ERR_INVALID_ARGUMENT whether or not a GPU is present."""
    pos = np.zeros((64, 2), np.float32)
    mass = np.ones(64, np.float32)
    for bits in (-1, 16):
        p = gs.default_params(algorithm=gs.BARNES_HUT, box_mode=gs.BOX_BOUNDING, key_bits=bits)
        h = ctypes.c_void_p()
        st = gs.lib().gs_create(ctypes.byref(p), 64, gs._fp(pos), gs._fp(pos), gs._fp(mass), ctypes.byref(h))
        assert st == 1 and not h.value
        assert b"key_bits" in gs.lib().gs_last_error()
