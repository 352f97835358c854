"""ctypes binding of libgsim.so (include/gsim.h) -- the binding a Python caller of the
C ABI would add.  Arrays are numpy float32 (x, y interleaved as shape (N, 2)).

There is no fallback: if libgsim.so is missing or fails to load, every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgsim.so")

OK = 0
DIRECT_SUM, BARNES_HUT = 0, 1
BOX_FIXED_500, BOX_BOUNDING = 0, 1
MATH_FAST, MATH_REFERENCE = 0, 1
FLAG_RECORD_ACCEL, FLAG_PROFILE, FLAG_NO_GRAPH, FLAG_COUNT_INTERACTIONS = 0x1, 0x2, 0x4, 0x8
FLAG_QUADRUPOLE, FLAG_SAFE_RADIUS, FLAG_GROUP_WALK = 0x10, 0x20, 0x40
FLAGS_ACCURATE = 0x70
GEN_RANDOM, GEN_GALAXY, GEN_GALAXY_COLLISION, GEN_SYMMETRICAL_GALAXY_COLLISION = 0, 1, 2, 3
GEN_UNIFORM_DISK, GEN_SPIRAL, GEN_EXP_DISK_COLLISION = 16, 17, 18
STAGES = ("bbox", "keys", "sort", "scan", "records", "sums", "force", "direct")

EXPORTS = (
    "gs_params_init", "gs_status_string", "gs_last_error", "gs_required_alignment", "gs_create", "gs_run",
    "gs_sync", "gs_get_particles", "gs_set_particles", "gs_get_accel", "gs_get_stats", "gs_reset_stats",
    "gs_particle_count", "gs_aligned_particle_count", "gs_stream", "gs_destroy", "gs_accel_f64",
    "gs_debug_bh_tree", "gs_bh_node_capacity", "gs_generate", "gs_read_particles", "gs_write_particles",
    "gs_direct_step_noalloc", "gs_batch_create", "gs_batch_run", "gs_batch_sync", "gs_batch_kernels_per_step",
    "gs_batch_stream", "gs_batch_destroy", "gs_tune_crossover", "gs_footprint", "gs_server_create",
    "gs_server_submit", "gs_server_poll", "gs_server_request", "gs_server_result", "gs_server_get_stats",
    "gs_server_clock", "gs_server_run_trace", "gs_server_destroy", "gs_energy_f64", "gs_camera_start",
    "gs_render_points", "gs_snapshot_take", "gs_snapshot_positions", "gs_snapshot_render", "gs_write_ppm",
    "gs_set_timeout", "gs_debug_state", "gs_get_shape", "gs_set_shape", "gs_shape_defaults", "gs_tune_shape",
    "gs_tune_batch_shape", "gs_load_shape_cache", "gs_clear_shape_table", "gs_batch_get_shape",
    "gs_batch_set_shape",
)
SHAPE_FIELDS = ("sort_keys_per_thread", "sort_lookback", "scan_lookback", "force_warps", "force_short_lists",
                "direct_targets", "direct_blocks_per_sm", "moment_blocks_per_sm")
FLAG_PLAIN_SUM = 0x80
FLAG_RELATIVE_MAC = 0x100
SERVE_FIFO, SERVE_SHORTEST_FIRST = 0, 1
REQUEST_QUEUED, REQUEST_RESIDENT, REQUEST_DONE, REQUEST_FAILED = 0, 1, 2, 3
BATCH_NO_GRAPH = 0x1
TUNE_MAX_SIZES = 16


class Params(C.Structure):
    _fields_ = [("gravitational_const", C.c_float), ("simulation_time", C.c_float),
                ("simulation_speed", C.c_float), ("softening_len", C.c_float),
                ("accuracy_parameter", C.c_float), ("algorithm", C.c_int32), ("box_mode", C.c_int32),
                ("math_mode", C.c_int32), ("device", C.c_int32), ("flags", C.c_uint32),
                ("relative_accuracy", C.c_float), ("relative_theta_floor", C.c_float), ("key_bits", C.c_int32)]


class Shape(C.Structure):
    _fields_ = [(k, C.c_uint32) for k in SHAPE_FIELDS]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k in SHAPE_FIELDS}


class TuneResult(C.Structure):
    _fields_ = [("best", Shape), ("best_ms", C.c_double), ("default_ms", C.c_double), ("candidates", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("steps_done", C.c_uint64), ("tree_records", C.c_uint64), ("internal_nodes", C.c_uint64),
                ("placed_particles", C.c_uint64), ("interactions", C.c_uint64), ("warp_visits", C.c_uint64),
                ("kernel_launches", C.c_uint64),
                ("stage_ms", C.c_float * 8), ("stage_launches", C.c_uint32 * 8), ("node_interactions", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("crossover", C.c_uint64), ("sizes", C.c_uint32), ("n", C.c_uint64 * 16),
                ("direct_ms", C.c_double * 16), ("bh_ms", C.c_double * 16)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget", C.c_uint64), ("max_resident_particles", C.c_uint64), ("crossover", C.c_uint64),
                ("direct_params", Params), ("bh_params", Params), ("steps_in_flight", C.c_uint32),
                ("policy", C.c_uint32), ("keep_results", C.c_uint32), ("worker_threads", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("particle_count", C.c_uint64), ("steps", C.c_uint32), ("generator", C.c_int32), ("seed", C.c_uint64),
                ("generate_size", C.c_float), ("min_mass", C.c_float), ("max_mass", C.c_float),
                ("pos_xy", C.POINTER(C.c_float)), ("vel_xy", C.POINTER(C.c_float)), ("mass", C.POINTER(C.c_float))]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("algorithm", C.c_int32), ("steps_enqueued", C.c_uint32), ("steps", C.c_uint32),
                ("particle_count", C.c_uint64), ("footprint", C.c_uint64), ("arrival_s", C.c_double),
                ("admit_s", C.c_double), ("finish_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "finished", "failed", "queued", "resident", "memory_in_use",
                                          "peak_memory_in_use", "resident_particles", "peak_resident_particles",
                                          "batched_steps", "plan_changes", "particle_steps")] + \
               [("gpu_busy_seconds", C.c_double)]


class GsimError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None
_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint32)
_DP = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GsimError(-1, f"libgsim.so not built at {LIB_PATH}; run the package build first")
    L = C.CDLL(LIB_PATH)
    st = C.c_int
    sim = C.c_void_p
    L.gs_params_init.argtypes = [C.POINTER(Params)]
    L.gs_params_init.restype = None
    L.gs_status_string.argtypes = [st]
    L.gs_status_string.restype = C.c_char_p
    L.gs_last_error.argtypes = []
    L.gs_last_error.restype = C.c_char_p
    L.gs_required_alignment.argtypes = [C.c_int32]
    L.gs_required_alignment.restype = C.c_uint64
    L.gs_create.argtypes = [C.POINTER(Params), C.c_uint64, _FP, _FP, _FP, C.POINTER(sim)]
    L.gs_create.restype = st
    L.gs_run.argtypes = [sim, C.c_uint32]
    L.gs_run.restype = st
    L.gs_sync.argtypes = [sim, C.c_uint64]
    L.gs_sync.restype = st
    L.gs_get_particles.argtypes = [sim, _FP, _FP, _FP]
    L.gs_get_particles.restype = st
    L.gs_set_particles.argtypes = [sim, _FP, _FP, _FP]
    L.gs_set_particles.restype = st
    L.gs_get_accel.argtypes = [sim, _FP]
    L.gs_get_accel.restype = st
    L.gs_get_stats.argtypes = [sim, C.POINTER(Stats)]
    L.gs_get_stats.restype = st
    L.gs_reset_stats.argtypes = [sim]
    L.gs_reset_stats.restype = st
    L.gs_particle_count.argtypes = [sim]
    L.gs_particle_count.restype = C.c_uint64
    L.gs_aligned_particle_count.argtypes = [sim]
    L.gs_aligned_particle_count.restype = C.c_uint64
    L.gs_stream.argtypes = [sim]
    L.gs_stream.restype = C.c_void_p
    L.gs_destroy.argtypes = [sim]
    L.gs_destroy.restype = None
    L.gs_set_timeout.argtypes = [sim, C.c_uint64]
    L.gs_set_timeout.restype = st
    L.gs_debug_state.argtypes = [sim, _FP, _FP, _FP, _FP]
    L.gs_debug_state.restype = st
    L.gs_get_shape.argtypes = [sim, C.POINTER(Shape)]
    L.gs_get_shape.restype = st
    L.gs_set_shape.argtypes = [sim, C.POINTER(Shape)]
    L.gs_set_shape.restype = st
    L.gs_shape_defaults.argtypes = [C.POINTER(Shape)]
    L.gs_shape_defaults.restype = None
    L.gs_tune_shape.argtypes = [C.POINTER(Params), C.c_uint64, C.c_int32, C.c_uint64, C.c_uint32, C.c_char_p,
                                C.POINTER(TuneResult)]
    L.gs_tune_shape.restype = st
    L.gs_tune_batch_shape.argtypes = [C.c_void_p, C.c_uint32, C.c_char_p, C.POINTER(TuneResult)]
    L.gs_tune_batch_shape.restype = st
    L.gs_load_shape_cache.argtypes = [C.c_char_p, C.POINTER(C.c_uint32)]
    L.gs_load_shape_cache.restype = st
    L.gs_clear_shape_table.argtypes = []
    L.gs_clear_shape_table.restype = None
    L.gs_batch_get_shape.argtypes = [C.c_void_p, C.POINTER(Shape)]
    L.gs_batch_get_shape.restype = st
    L.gs_batch_set_shape.argtypes = [C.c_void_p, C.POINTER(Shape)]
    L.gs_batch_set_shape.restype = st
    L.gs_accel_f64.argtypes = [sim, C.c_uint32, _UP, _DP]
    L.gs_accel_f64.restype = st
    L.gs_debug_bh_tree.argtypes = [sim, _UP, _UP, _UP, _FP, _FP, _FP, _FP, C.c_uint64, C.POINTER(C.c_uint64)]
    L.gs_debug_bh_tree.restype = st
    L.gs_bh_node_capacity.argtypes = [C.c_int32, C.c_uint64]
    L.gs_bh_node_capacity.restype = C.c_uint64
    L.gs_generate.argtypes = [C.c_int32, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint64,
                              _FP, _FP, _FP]
    L.gs_generate.restype = st
    L.gs_read_particles.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(C.c_uint64), _FP, _FP, _FP]
    L.gs_read_particles.restype = st
    L.gs_write_particles.argtypes = [C.c_char_p, C.c_uint64, _FP, _FP, _FP]
    L.gs_write_particles.restype = st
    batch = C.c_void_p
    L.gs_batch_create.argtypes = [C.POINTER(sim), C.c_uint32, C.c_uint32, C.POINTER(batch)]
    L.gs_batch_create.restype = st
    L.gs_batch_run.argtypes = [batch, C.c_uint32]
    L.gs_batch_run.restype = st
    L.gs_batch_sync.argtypes = [batch, C.c_uint64]
    L.gs_batch_sync.restype = st
    L.gs_batch_kernels_per_step.argtypes = [batch]
    L.gs_batch_kernels_per_step.restype = C.c_uint32
    L.gs_batch_stream.argtypes = [batch]
    L.gs_batch_stream.restype = C.c_void_p
    L.gs_batch_destroy.argtypes = [batch]
    L.gs_batch_destroy.restype = None
    L.gs_tune_crossover.argtypes = [C.POINTER(Params), C.POINTER(Params), C.c_uint64, C.c_uint64, C.c_uint64,
                                    C.c_uint64, C.POINTER(Tuning)]
    L.gs_tune_crossover.restype = st
    srv = C.c_void_p
    _BP = C.POINTER(C.c_uint8)
    L.gs_camera_start.argtypes = [sim, _FP]
    L.gs_camera_start.restype = st
    L.gs_render_points.argtypes = [sim, C.c_uint32, C.c_uint32, _FP, _BP]
    L.gs_render_points.restype = st
    L.gs_snapshot_take.argtypes = [sim, C.c_uint32, C.POINTER(C.c_uint64)]
    L.gs_snapshot_take.restype = st
    L.gs_snapshot_positions.argtypes = [sim, C.c_uint64, _FP]
    L.gs_snapshot_positions.restype = st
    L.gs_snapshot_render.argtypes = [sim, C.c_uint64, C.c_uint32, C.c_uint32, _FP, _BP]
    L.gs_snapshot_render.restype = st
    L.gs_write_ppm.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, _BP]
    L.gs_write_ppm.restype = st
    L.gs_energy_f64.argtypes = [sim, _DP, _DP]
    L.gs_energy_f64.restype = st
    L.gs_footprint.argtypes = [C.POINTER(Params), C.c_uint64]
    L.gs_footprint.restype = C.c_uint64
    L.gs_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(srv)]
    L.gs_server_create.restype = st
    L.gs_server_submit.argtypes = [srv, C.POINTER(Request), C.c_double, C.POINTER(C.c_uint64)]
    L.gs_server_submit.restype = st
    L.gs_server_poll.argtypes = [srv, C.POINTER(C.c_uint32)]
    L.gs_server_poll.restype = st
    L.gs_server_request.argtypes = [srv, C.c_uint64, C.POINTER(RequestStatus)]
    L.gs_server_request.restype = st
    L.gs_server_result.argtypes = [srv, C.c_uint64, _FP, _FP, _FP]
    L.gs_server_result.restype = st
    L.gs_server_get_stats.argtypes = [srv, C.POINTER(ServerStats)]
    L.gs_server_get_stats.restype = st
    L.gs_server_clock.argtypes = [srv]
    L.gs_server_clock.restype = C.c_double
    L.gs_server_run_trace.argtypes = [srv, C.POINTER(Request), C.POINTER(C.c_double), C.c_uint32, C.c_double,
                                      C.POINTER(C.c_uint64)]
    L.gs_server_run_trace.restype = st
    L.gs_server_destroy.argtypes = [srv]
    L.gs_server_destroy.restype = None
    _lib = L
    return L


def _check(status):
    if status != OK:
        L = lib()
        raise GsimError(status, L.gs_last_error().decode() or L.gs_status_string(status).decode())


def _fp(a):
    return None if a is None else a.ctypes.data_as(_FP)


def _f32(a, shape):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape)


def default_params(**kw):
    p = Params()
    lib().gs_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def generate(kind, n, size=100.0, min_mass=1.0, max_mass=10.0, G=1.0, seed=1):
    pos = np.empty((n, 2), np.float32)
    vel = np.empty((n, 2), np.float32)
    mass = np.empty(n, np.float32)
    _check(lib().gs_generate(kind, n, size, min_mass, max_mass, G, seed, _fp(pos), _fp(vel), _fp(mass)))
    return pos, vel, mass


def read_particles(path):
    cnt = C.c_uint64(0)
    L = lib()
    _check(L.gs_read_particles(path.encode(), 0, C.byref(cnt), None, None, None))
    n = cnt.value
    pos = np.empty((n, 2), np.float32)
    vel = np.empty((n, 2), np.float32)
    mass = np.empty(n, np.float32)
    _check(L.gs_read_particles(path.encode(), n, C.byref(cnt), _fp(pos), _fp(vel), _fp(mass)))
    return pos, vel, mass


def write_particles(path, pos, vel, mass):
    n = len(mass)
    pos, vel, mass = _f32(pos, (n, 2)), _f32(vel, (n, 2)), _f32(mass, (n,))
    _check(lib().gs_write_particles(path.encode(), n, _fp(pos), _fp(vel), _fp(mass)))


def required_alignment(algorithm=DIRECT_SUM):
    return int(lib().gs_required_alignment(algorithm))


def node_capacity(box_mode, n_al):
    return int(lib().gs_bh_node_capacity(box_mode, n_al))


class Simulation:
    """One simulated system resident on the GPU (gs_sim)."""

    def __init__(self, pos, vel, mass, params=None, **kw):
        self._h = C.c_void_p()
        self.params = params if params is not None else default_params(**kw)
        n = len(mass)
        self.n = n
        pos, vel, mass = _f32(pos, (n, 2)), _f32(vel, (n, 2)), _f32(mass, (n,))
        _check(lib().gs_create(C.byref(self.params), n, _fp(pos), _fp(vel), _fp(mass), C.byref(self._h)))
        self.n_al = int(lib().gs_aligned_particle_count(self._h))

    def close(self):
        if self._h:
            lib().gs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def run(self, count=1):
        _check(lib().gs_run(self._h, count))

    def sync(self, timeout_ns=0):
        _check(lib().gs_sync(self._h, timeout_ns))

    def shape(self):
        sh = Shape()
        _check(lib().gs_get_shape(self._h, C.byref(sh)))
        return sh

    def set_shape(self, shape=None, **kw):
        sh = Shape.from_buffer_copy(shape) if shape is not None else self.shape()
        for k, v in kw.items():
            setattr(sh, k, v)
        _check(lib().gs_set_shape(self._h, C.byref(sh)))

    def set_timeout(self, timeout_ns):
        """Bound of every host wait of this system (0: 600 s)."""
        _check(lib().gs_set_timeout(self._h, timeout_ns))

    def get_particles(self):
        pos = np.empty((self.n, 2), np.float32)
        vel = np.empty((self.n, 2), np.float32)
        mass = np.empty(self.n, np.float32)
        _check(lib().gs_get_particles(self._h, _fp(pos), _fp(vel), _fp(mass)))
        return pos, vel, mass

    def set_particles(self, pos, vel, mass):
        n = self.n
        pos, vel, mass = _f32(pos, (n, 2)), _f32(vel, (n, 2)), _f32(mass, (n,))
        _check(lib().gs_set_particles(self._h, _fp(pos), _fp(vel), _fp(mass)))

    def get_accel(self):
        acc = np.empty((self.n, 2), np.float32)
        _check(lib().gs_get_accel(self._h, _fp(acc)))
        return acc

    def stats(self):
        s = Stats()
        _check(lib().gs_get_stats(self._h, C.byref(s)))
        return s

    def reset_stats(self):
        _check(lib().gs_reset_stats(self._h))

    def stream(self):
        return lib().gs_stream(self._h)

    def camera_start(self):
        """The reference's start camera {x, y, size, size} of the current state."""
        cam = np.empty(4, np.float32)
        _check(lib().gs_camera_start(self._h, _fp(cam)))
        return cam

    def render(self, width, height, camera):
        """Point splat of the current state: (height, width) uint8 image, 255 = particle."""
        cam = np.ascontiguousarray(camera, np.float32)
        img = np.empty((height, width), np.uint8)
        _check(lib().gs_render_points(self._h, width, height, _fp(cam), img.ctypes.data_as(C.POINTER(C.c_uint8))))
        return img

    def snapshot(self, slots=3):
        t = C.c_uint64()
        _check(lib().gs_snapshot_take(self._h, slots, C.byref(t)))
        return t.value

    def snapshot_positions(self, ticket):
        pos = np.empty((self.n, 2), np.float32)
        _check(lib().gs_snapshot_positions(self._h, ticket, _fp(pos)))
        return pos

    def snapshot_render(self, ticket, width, height, camera):
        cam = np.ascontiguousarray(camera, np.float32)
        img = np.empty((height, width), np.uint8)
        _check(lib().gs_snapshot_render(self._h, ticket, width, height, _fp(cam),
                                        img.ctypes.data_as(C.POINTER(C.c_uint8))))
        return img

    def energy_f64(self):
        """(kinetic, potential) of the current state in FP64."""
        k, p = C.c_double(), C.c_double()
        _check(lib().gs_energy_f64(self._h, C.byref(k), C.byref(p)))
        return k.value, p.value

    def accel_f64(self, targets):
        t = np.ascontiguousarray(targets, dtype=np.uint32)
        out = np.empty((len(t), 2), np.float64)
        _check(lib().gs_accel_f64(self._h, len(t), t.ctypes.data_as(_UP), out.ctypes.data_as(_DP)))
        return out

    def padded_state(self):
        """All N_al particles of the current state (padding included) and the |a| the next
        relative-criterion step reads (NaN: unknown)."""
        n_al = self.n_al
        pos = np.empty((n_al, 2), np.float32)
        vel = np.empty((n_al, 2), np.float32)
        mass = np.empty(n_al, np.float32)
        amag = np.empty(n_al, np.float32)
        _check(lib().gs_debug_state(self._h, _fp(pos), _fp(vel), _fp(mass), _fp(amag)))
        return pos, vel, mass, amag

    def bh_tree(self):
        n_al = self.n_al
        cap = node_capacity(self.params.box_mode, n_al)
        keys = np.empty(n_al, np.uint32)
        src = np.empty(n_al, np.uint32)
        skip = np.empty(cap, np.uint32)
        radius = np.empty(cap, np.float32)
        npos = np.empty((cap, 2), np.float32)
        nmass = np.empty(cap, np.float32)
        quad = np.empty((cap, 3), np.float32)
        T = C.c_uint64(0)
        _check(lib().gs_debug_bh_tree(self._h, keys.ctypes.data_as(_UP), src.ctypes.data_as(_UP),
                                      skip.ctypes.data_as(_UP), _fp(radius), _fp(npos), _fp(nmass), _fp(quad), cap,
                                      C.byref(T)))
        t = T.value
        return dict(keys=keys, sorted_src=src, skip=skip[:t], radius=radius[:t], pos=npos[:t], mass=nmass[:t],
                    quad=quad[:t], tree_size=t)


class Batch:
    """Independent systems advanced together, one launch per stage (gs_batch).  Holds
    references to its members so that they outlive it."""

    def __init__(self, sims, flags=0):
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s.handle.value for s in self.sims])
        self._h = C.c_void_p()
        _check(lib().gs_batch_create(arr, len(self.sims), flags, C.byref(self._h)))

    def close(self):
        if self._h:
            lib().gs_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, steps=1):
        _check(lib().gs_batch_run(self._h, steps))

    def sync(self, timeout_ns=0):
        _check(lib().gs_batch_sync(self._h, timeout_ns))

    def shape(self):
        sh = Shape()
        _check(lib().gs_batch_get_shape(self._h, C.byref(sh)))
        return sh

    def set_shape(self, shape=None, **kw):
        sh = Shape.from_buffer_copy(shape) if shape is not None else self.shape()
        for k, v in kw.items():
            setattr(sh, k, v)
        _check(lib().gs_batch_set_shape(self._h, C.byref(sh)))

    def tune(self, steps=5, cache_path=None):
        r = TuneResult()
        _check(lib().gs_tune_batch_shape(self._h, steps, cache_path.encode() if cache_path else None, C.byref(r)))
        return r

    @property
    def kernels_per_step(self):
        return int(lib().gs_batch_kernels_per_step(self._h))

    @property
    def stream(self):
        return lib().gs_batch_stream(self._h)


def tune_crossover(direct_params, bh_params, min_n=1024, max_n=262144, particles_per_probe=1 << 21, seed=4000):
    """gs_tune_crossover: measured direct-sum / Barnes-Hut crossover N and the timings."""
    t = Tuning()
    _check(lib().gs_tune_crossover(C.byref(direct_params), C.byref(bh_params), min_n, max_n, particles_per_probe,
                                   seed, C.byref(t)))
    k = t.sizes
    return dict(crossover=int(t.crossover), n=[int(x) for x in t.n[:k]], direct_ms=list(t.direct_ms[:k]),
                bh_ms=list(t.bh_ms[:k]))


def shape_defaults():
    sh = Shape()
    lib().gs_shape_defaults(C.byref(sh))
    return sh


def tune_shape(params, n, generator=GEN_UNIFORM_DISK, seed=1, steps=10, cache_path=None):
    """Launch-shape autotuner (gs_tune_shape): the fastest shape for this workload, entered in
    the process's tuned table (and the cache file, if given)."""
    r = TuneResult()
    _check(lib().gs_tune_shape(C.byref(params), n, generator, seed, steps,
                               cache_path.encode() if cache_path else None, C.byref(r)))
    return r


def load_shape_cache(path):
    count = C.c_uint32(0)
    _check(lib().gs_load_shape_cache(path.encode() if path else None, C.byref(count)))
    return count.value


def clear_shape_table():
    lib().gs_clear_shape_table()


def footprint(params, n):
    """gs_footprint: device bytes gs_create allocates for N particles with these parameters."""
    return int(lib().gs_footprint(C.byref(params), n))


def make_request(n, steps, generator=GEN_UNIFORM_DISK, seed=1, size=100.0, min_mass=1.0, max_mass=10.0):
    r = Request()
    r.particle_count, r.steps, r.generator, r.seed = n, steps, generator, seed
    r.generate_size, r.min_mass, r.max_mass = size, min_mass, max_mass
    return r


class Server:
    """Continuous batching of simulation requests (gs_server)."""

    def __init__(self, memory_budget, crossover, direct_params, bh_params, max_resident_particles=0,
                 steps_in_flight=0, policy=SERVE_FIFO, keep_results=False, worker_threads=0):
        c = ServerConfig()
        c.memory_budget, c.max_resident_particles, c.crossover = memory_budget, max_resident_particles, crossover
        c.direct_params, c.bh_params = direct_params, bh_params
        c.steps_in_flight, c.policy, c.keep_results, c.worker_threads = steps_in_flight, policy, int(keep_results), \
            worker_threads
        self.config = c
        self._h = C.c_void_p()
        _check(lib().gs_server_create(C.byref(c), C.byref(self._h)))
        self._n = {}

    def close(self):
        if self._h:
            lib().gs_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, request, arrival_s=-1.0):
        rid = C.c_uint64()
        _check(lib().gs_server_submit(self._h, C.byref(request), arrival_s, C.byref(rid)))
        self._n[rid.value] = request.particle_count
        return rid.value

    def poll(self):
        f = C.c_uint32()
        _check(lib().gs_server_poll(self._h, C.byref(f)))
        return f.value

    def request(self, rid):
        st = RequestStatus()
        _check(lib().gs_server_request(self._h, rid, C.byref(st)))
        return st

    def result(self, rid):
        n = self._n[rid]
        pos, vel, mass = np.empty((n, 2), np.float32), np.empty((n, 2), np.float32), np.empty(n, np.float32)
        _check(lib().gs_server_result(self._h, rid, _fp(pos), _fp(vel), _fp(mass)))
        return pos, vel, mass

    def stats(self):
        st = ServerStats()
        _check(lib().gs_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def clock(self):
        return float(lib().gs_server_clock(self._h))

    def run_trace(self, requests, arrival_s, timeout_s=0.0):
        n = len(requests)
        arr = (Request * n)(*requests)
        t = (C.c_double * n)(*[float(x) for x in arrival_s])
        ids = (C.c_uint64 * n)()
        _check(lib().gs_server_run_trace(self._h, arr, t, n, timeout_s, ids))
        out = list(ids)
        for r, i in zip(requests, out):
            self._n[i] = r.particle_count
        return out


def write_ppm(path, image):
    """Binary PPM of a (height, width) uint8 image from Simulation.render."""
    img = np.ascontiguousarray(image, np.uint8)
    _check(lib().gs_write_ppm(path.encode(), img.shape[1], img.shape[0], img.ctypes.data_as(C.POINTER(C.c_uint8))))
