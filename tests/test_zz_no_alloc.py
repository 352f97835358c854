"""gs_direct_step_noalloc: the direct-sum step for callers that cannot let the library
allocate device memory (the host owns every allocation, or a fixed memory budget must
not be disturbed by cudaMalloc / cudaFree mid-run).  Its scratch lives in fixed arrays
inside the library, so the caller only supplies the particle buffers.

Checked through the C ABI against the allocating entry point (gs_create + gs_run, FAST
math) on two calls in a row, within the tolerance of the other direct-sum tests:
positions within 1e-5 absolute, velocities within 1e-4 * max|v|.  This file is
collected last so a failure here stops a run only after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(gs):
    L = gs.lib()
    f = L.gs_direct_step_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_float, C.c_float,
                  C.c_float, C.c_void_p]
    f.restype = C.c_int
    return f


def _padded(pos, vel, mass):
    n = len(mass)
    n_al = (n + 63) // 64 * 64
    P = np.zeros((n_al, 2), np.float32)
    V = np.zeros((n_al, 2), np.float32)
    M = np.zeros(n_al, np.float32)
    P[:n], V[:n], M[:n] = pos, vel, mass
    return P, V, M


@pytest.mark.parametrize("n", [4096, 1000, 65536])
def test_noalloc_matches_allocating_path(gs, n):
    import torch

    step = _bind(gs)
    pos, vel, mass = gs.generate(gs.GEN_UNIFORM_DISK, n, size=100.0, seed=4242 + n)
    vel = (0.5 * np.random.default_rng(n).standard_normal(pos.shape)).astype(np.float32)
    P, V, M = _padded(pos, vel, mass)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    p_in, v_in = torch.from_numpy(P).to(dev), torch.from_numpy(V).to(dev)
    m = torch.from_numpy(M).to(dev)
    p_out, v_out = torch.empty_like(p_in), torch.empty_like(v_in)
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):  # two calls in a row; the second reads the first one's output
        st = step(p_in.data_ptr(), v_in.data_ptr(), m.data_ptr(), p_out.data_ptr(), v_out.data_ptr(), len(M),
                  1.0, 1e-3, 0.2, stream.cuda_stream)
        assert st == 0, gs.lib().gs_last_error().decode()
        p_in, p_out = p_out, p_in
        v_in, v_out = v_out, v_in
    torch.cuda.synchronize()
    got_p = p_in.cpu().numpy()[:n]
    got_v = v_in.cpu().numpy()[:n]

    with gs.Simulation(pos, vel, mass, algorithm=gs.DIRECT_SUM) as sim:
        sim.run(2)
        ref_p, ref_v, _ = sim.get_particles()
    np.testing.assert_allclose(got_p, ref_p, rtol=0, atol=1e-5)
    assert np.max(np.abs(got_v - ref_v)) <= 1e-4 * np.abs(ref_v).max()


def test_noalloc_rejects_sizes_beyond_its_scratch(gs):
    import torch

    step = _bind(gs)
    n = 65536 + 64
    buf = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    m = torch.zeros(n, dtype=torch.float32, device="cuda")
    out_p, out_v = torch.empty_like(buf), torch.empty_like(buf)
    st = step(buf.data_ptr(), buf.data_ptr(), m.data_ptr(), out_p.data_ptr(), out_v.data_ptr(), n, 1.0, 1e-3, 0.2,
              None)
    assert st == 7  # GS_ERR_CAPACITY
    assert "GS_NOALLOC_MAX_PARTICLES" in gs.lib().gs_last_error().decode()
    st = step(buf.data_ptr(), buf.data_ptr(), m.data_ptr(), out_p.data_ptr(), out_v.data_ptr(), 100, 1.0, 1e-3, 0.2,
              None)
    assert st == 1  # not a multiple of 64
    # positions are read as 16-byte float4 pairs: a misaligned array is refused before any launch
    st = step(buf.data_ptr() + 8, buf.data_ptr(), m.data_ptr(), out_p.data_ptr(), out_v.data_ptr(), 64, 1.0, 1e-3,
              0.2, None)
    assert st == 1 and "aligned" in gs.lib().gs_last_error().decode()
