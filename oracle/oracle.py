"""ctypes wrapper of the CPU oracle (oracle/gsim_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py -- never by the product path.

Parity unpinned against reference outputs: the reference computes forces only in
Vulkan compute shaders and has no tests, fixtures or golden vectors.  See the header of
gsim_oracle.h for what the restatement is pinned against instead.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

BOX_FIXED_500, BOX_BOUNDING = 0, 1
QUADRUPOLE, SAFE_RADIUS, GROUP_WALK, RELATIVE_MAC = 1, 2, 4, 8
ACCURATE = QUADRUPOLE | SAFE_RADIUS | GROUP_WALK
KEY_REMOVED = 0xFFFFFFFF
_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint32)
_DP = C.POINTER(C.c_double)


class BHOut(C.Structure):
    _fields_ = [("keys", _UP), ("sorted_src", _UP), ("node_skip", _UP), ("node_radius", _FP),
                ("node_pos", _FP), ("node_mass", _FP), ("node_quad", _FP), ("node_capacity", C.c_uint64),
                ("walk_stride", C.c_uint32),
                ("tree_size", C.c_uint64), ("valid_count", C.c_uint64), ("internal_count", C.c_uint64),
                ("interactions", C.c_uint64), ("warp_visits", C.c_uint64),
                ("box_center_x", C.c_float), ("box_center_y", C.c_float), ("box_scale", C.c_float),
                ("box_radius0", C.c_float), ("build_seconds", C.c_double), ("walk_seconds", C.c_double),
                ("max_stack", C.c_uint32), ("max_warp_interactions", C.c_uint64),
                ("rel_alpha", C.c_float), ("rel_floor2", C.c_float), ("amag_in", _FP), ("amag_out", _FP),
                ("key_bits", C.c_uint32), ("group_visits", _UP), ("group_interactions", C.POINTER(C.c_uint64))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_direct_step.argtypes = [C.c_uint32, _FP, _FP, _FP, _FP, _FP, C.c_float, C.c_float, C.c_float, C.c_int]
        L.orc_direct_step.restype = None
        L.orc_direct_accel.argtypes = [C.c_uint32, _FP, _FP, C.c_float, _FP, C.c_int]
        L.orc_direct_accel.restype = None
        L.orc_direct_accel_f64.argtypes = [C.c_uint32, _FP, _FP, C.c_double, C.c_uint32, _UP, _DP, C.c_int]
        L.orc_direct_accel_f64.restype = None
        for f in (L.orc_bh_grid_step,):
            f.argtypes = [C.c_uint32, _FP, _FP, _FP, _FP, _FP, _FP, C.c_float, C.c_float, C.c_float, C.c_float,
                          C.POINTER(BHOut), C.c_int]
            f.restype = C.c_int
        L.orc_bh_sorted_step.argtypes = [C.c_int, C.c_uint32, _FP, _FP, _FP, _FP, _FP, _FP, C.c_float, C.c_float,
                                         C.c_float, C.c_float, C.POINTER(BHOut), C.c_int]
        L.orc_bh_sorted_step.restype = C.c_int
        L.orc_bh_sorted_step_ex.argtypes = [C.c_int, C.c_int, C.c_uint32, _FP, _FP, _FP, _FP, _FP, _FP, C.c_float,
                                            C.c_float, C.c_float, C.c_float, C.POINTER(BHOut), C.c_int]
        L.orc_bh_sorted_step_ex.restype = C.c_int
        L.orc_set_heavy_pairs.argtypes = [C.c_int]
        L.orc_set_heavy_pairs.restype = None
        L.orc_bh_node_capacity.argtypes = [C.c_int, C.c_uint32]
        L.orc_bh_node_capacity.restype = C.c_uint64
        L.orc_energy_f64.argtypes = [C.c_uint32, _FP, _FP, _FP, C.c_double, C.c_double]
        L.orc_energy_f64.restype = C.c_double
        L.orc_render_points.argtypes = [C.c_uint32, _FP, _FP, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint8)]
        L.orc_render_points.restype = None
        L.orc_generate.argtypes = [C.c_int, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint64,
                                   _FP, _FP, _FP]
        L.orc_generate.restype = C.c_int
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(_FP)


def generate(kind, n, size=100.0, min_mass=1.0, max_mass=10.0, G=1.0, seed=1):
    """The library's seeded generators restated on the CPU: pos (n, 2), vel (n, 2), mass (n,)."""
    pos = np.empty((n, 2), np.float32)
    vel = np.empty((n, 2), np.float32)
    mass = np.empty(n, np.float32)
    if lib().orc_generate(kind, n, size, min_mass, max_mass, G, seed, _fp(pos), _fp(vel), _fp(mass)) != 0:
        raise ValueError("orc_generate: unknown generator type or bad count")
    return pos, vel, mass


def pad_state(pos, vel, mass, align=64):
    """Pad to the alignment with zero particles (ParticleSystem.cpp:487-491)."""
    n = len(mass)
    n_al = (n + align - 1) // align * align
    P = np.zeros((n_al, 2), np.float32)
    V = np.zeros((n_al, 2), np.float32)
    M = np.zeros(n_al, np.float32)
    P[:n], V[:n], M[:n] = pos, vel, mass
    return P, V, M


class State:
    """Two buffer sets with the reference's ping-pong (ParticleSystem.hpp:169-174)."""

    def __init__(self, pos, vel, mass, align=64):
        self.n = len(mass)
        P, V, M = pad_state(pos, vel, mass, align)
        self.pos = [P.copy(), P.copy()]
        self.vel = [V.copy(), V.copy()]
        self.mass = [M.copy(), M.copy()]
        self.inp = 0
        self.amag = np.full(len(M), np.nan, np.float32)  # |a| of the last Barnes-Hut step (relative criterion)

    @property
    def n_al(self):
        return len(self.mass[0])

    def current(self):
        i = self.inp
        return self.pos[i][: self.n].copy(), self.vel[i][: self.n].copy(), self.mass[i][: self.n].copy()

    def sets(self):
        i, o = self.inp, self.inp ^ 1
        return (self.pos[i], self.vel[i], self.mass[i]), (self.pos[o], self.vel[o], self.mass[o])

    def flip(self):
        self.inp ^= 1


def direct_step(state, dt=1e-3, G=1.0, softening=0.2, threads=os.cpu_count()):
    (pi, vi, mi), (po, vo, _) = state.sets()
    eps2 = np.float32(softening) * np.float32(softening)
    lib().orc_direct_step(state.n_al, _fp(pi), _fp(vi), _fp(mi), _fp(po), _fp(vo), dt, G, float(eps2), threads)
    state.flip()


def direct_accel(pos, mass, softening=0.2, threads=os.cpu_count()):
    pos = np.ascontiguousarray(pos, np.float32)
    mass = np.ascontiguousarray(mass, np.float32)
    acc = np.empty_like(pos)
    eps2 = np.float32(softening) * np.float32(softening)
    lib().orc_direct_accel(len(mass), _fp(pos), _fp(mass), float(eps2), _fp(acc), threads)
    return acc


def direct_accel_f64(pos, mass, softening=0.2, targets=None, threads=os.cpu_count()):
    pos = np.ascontiguousarray(pos, np.float32)
    mass = np.ascontiguousarray(mass, np.float32)
    if targets is None:
        targets = np.arange(len(mass), dtype=np.uint32)
    t = np.ascontiguousarray(targets, np.uint32)
    out = np.empty((len(t), 2), np.float64)
    eps2 = float(np.float32(softening) * np.float32(softening))
    lib().orc_direct_accel_f64(len(mass), _fp(pos), _fp(mass), eps2, len(t), t.ctypes.data_as(_UP),
                               out.ctypes.data_as(_DP), threads)
    return out


def set_heavy_pairs(on):
    """Whether costly groups of large systems walk as warp pairs (the default, as the
    library does) or alone: a test switch, pairing changes only the order of the sums."""
    lib().orc_set_heavy_pairs(1 if on else 0)


def bh_step(state, method="sorted", box_mode=BOX_FIXED_500, dt=1e-3, speed=1.0, G=1.0, softening=0.2, theta=1.0,
            keep_tree=True, threads=os.cpu_count(), walk_stride=1, flags=0, rel_alpha=0.0, rel_floor=None,
            key_bits=0, amag_in=None, group_stats=False):
    """One Barnes-Hut step; returns a dict with keys, sorted_src and the preorder records.
    key_bits: bounding-box cells per axis as a power of two (0: 12).  amag_in: the previous
    |a| per particle to use instead of the state's own (relative criterion)."""
    (pi, vi, mi), (po, vo, mo) = state.sets()
    n_al = state.n_al
    L = lib()
    cap = int(L.orc_bh_node_capacity(box_mode, n_al))
    out = BHOut()
    out.walk_stride = walk_stride
    out.key_bits = key_bits
    gv = gi = None
    if group_stats:  # records tested and interactions of each group of 64 (group walk)
        gv = np.zeros(n_al // 64, np.uint32)
        gi = np.zeros(n_al // 64, np.uint64)
        out.group_visits = gv.ctypes.data_as(_UP)
        out.group_interactions = gi.ctypes.data_as(C.POINTER(C.c_uint64))
    amag_out = None
    if amag_in is not None:
        state.amag = np.ascontiguousarray(amag_in, np.float32).copy()
    if flags & RELATIVE_MAC:  # |a| of this step; particles the walk skips keep their value
        amag_out = state.amag.copy()
        out.rel_alpha = rel_alpha
        f = np.float32(theta if not rel_floor else rel_floor)
        out.rel_floor2 = float(f * f)
        out.amag_in = _fp(state.amag)
        out.amag_out = _fp(amag_out)
    res = {}
    if keep_tree:
        res = dict(keys=np.empty(n_al, np.uint32), sorted_src=np.empty(n_al, np.uint32),
                   skip=np.empty(cap, np.uint32), radius=np.empty(cap, np.float32),
                   pos=np.empty((cap, 2), np.float32), mass=np.empty(cap, np.float32),
                   quad=np.zeros((cap, 3), np.float32))
        out.keys = res["keys"].ctypes.data_as(_UP)
        out.sorted_src = res["sorted_src"].ctypes.data_as(_UP)
        out.node_skip = res["skip"].ctypes.data_as(_UP)
        out.node_radius = _fp(res["radius"])
        out.node_pos = _fp(res["pos"])
        out.node_mass = _fp(res["mass"])
        out.node_quad = _fp(res["quad"])
        out.node_capacity = cap
    dt_eff = float(np.float32(dt) * np.float32(speed))
    eps2 = float(np.float32(softening) * np.float32(softening))
    th2 = float(np.float32(theta) * np.float32(theta))
    if method == "grid":
        assert box_mode == BOX_FIXED_500
        L.orc_bh_grid_step(n_al, _fp(pi), _fp(vi), _fp(mi), _fp(po), _fp(vo), _fp(mo), dt_eff, G, eps2, th2,
                           C.byref(out), threads)
    else:
        if L.orc_bh_sorted_step_ex(box_mode, flags, n_al, _fp(pi), _fp(vi), _fp(mi), _fp(po), _fp(vo), _fp(mo),
                                   dt_eff, G, eps2, th2, C.byref(out), threads) != 0:
            raise ValueError("orc_bh_sorted_step_ex rejected its arguments")
    state.flip()
    if amag_out is not None:
        state.amag = amag_out
    t = out.tree_size
    if keep_tree:
        for k in ("skip", "radius", "pos", "mass", "quad"):
            res[k] = res[k][:t]
    res.update(tree_size=t, valid_count=out.valid_count, internal_count=out.internal_count,
               interactions=out.interactions, warp_visits=out.warp_visits,
               build_seconds=out.build_seconds, walk_seconds=out.walk_seconds, max_stack=out.max_stack,
               max_warp_interactions=out.max_warp_interactions,
               box=(out.box_center_x, out.box_center_y, out.box_scale, out.box_radius0))
    if group_stats:
        res.update(group_visits=gv, group_interactions=gi)
    return res


def energy_f64(pos, vel, mass, G=1.0, softening=0.2):
    pos = np.ascontiguousarray(pos, np.float32)
    vel = np.ascontiguousarray(vel, np.float32)
    mass = np.ascontiguousarray(mass, np.float32)
    eps2 = float(np.float32(softening) * np.float32(softening))
    return lib().orc_energy_f64(len(mass), _fp(pos), _fp(vel), _fp(mass), G, eps2)


def render_points(pos, camera, width, height):
    """Point splat of the reference's vertex/fragment shaders: (height, width) uint8."""
    pos = np.ascontiguousarray(pos, np.float32)
    cam = np.ascontiguousarray(camera, np.float32)
    img = np.empty((height, width), np.uint8)
    lib().orc_render_points(len(pos), _fp(pos), _fp(cam), width, height, img.ctypes.data_as(C.POINTER(C.c_uint8)))
    return img
