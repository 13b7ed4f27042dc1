"""ctypes binding of the C ABI in include/frg.h (libfrg.so, built in-tree).

There is no CPU fallback: if libfrg.so is missing or no CUDA device is present
every entry point raises FrgError.

The Python names mirror the reference's entry points for this path:
``forward_dynamics_gradient`` is forwardDynamicsGradient[Threaded]
(helpers_CPU/dynamicsGradient.h:916-934) over a batch, with q̈ and Minv
produced on the device (forwardDynamics, :936-939, fused in), and
``Context.gradient`` is the dynamicsGradientKernel launch of time_GPU.cu:314.
"""
import ctypes
import os

from .build import LIB_PATH

# per-knot sizes of the default (iiwa_14) build; dims() gives the loaded library's
NUM_JOINTS = 7
DQDD_FLOATS = 98
MINV_FLOATS = 49

FRG_OK = 0
STATUS_NAMES = {
    0: "FRG_OK", 1: "FRG_ERR_INVALID_ARGUMENT", 2: "FRG_ERR_CUDA", 3: "FRG_ERR_OUT_OF_MEMORY",
    4: "FRG_ERR_NOT_READY", 5: "FRG_ERR_ADMISSION", 6: "FRG_ERR_TIMEOUT", 7: "FRG_ERR_SHUTDOWN",
    8: "FRG_ERR_NOT_FOUND", 9: "FRG_ERR_INTERNAL", 10: "FRG_ERR_CANCELLED",
}

# every symbol include/frg.h declares (checked by tests/test_abi.py)
EXPORTED = (
    "frg_options_default", "frg_status_string", "frg_create", "frg_destroy", "frg_last_error",
    "frg_set_launch_shape", "frg_get_launch_shape", "frg_set_lanes_per_knot", "frg_get_lanes_per_knot", "frg_gradient", "frg_gradient_host",
    "frg_gradient_per_trajectory", "frg_gradient_batched", "frg_gradient_ragged", "frg_plan_create",
    "frg_plan_create_ragged", "frg_plan_launch", "frg_plan_launch_many", "frg_plan_knots", "frg_plan_destroy",
    "frg_autotune",
    "frg_host_alloc", "frg_host_free", "frg_gradient_ragged_noalloc", "frg_server_options_default",
    "frg_server_create", "frg_server_destroy", "frg_server_submit", "frg_server_poll", "frg_server_wait",
    "frg_server_wait_any", "frg_server_release", "frg_server_get_stats", "frg_gradient_fext",
    "frg_forward_dynamics", "frg_discrete_jacobians", "frg_gradient_f64", "frg_verify_f64", "frg_get_tuning",
    "frg_set_tuning", "frg_knot_status", "frg_model_name", "frg_gradient_knots", "frg_server_cancel",
    "frg_single_knot_latency", "frg_server_submit_device", "frg_server_submit_resident", "frg_server_slot",
    "frg_model_dofs", "frg_gradient_host_batches",
)
SERVE_HOST_RESULTS = 1

KNOT_NONFINITE_INPUT = 1
KNOT_NONFINITE_OUTPUT = 2


class FrgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("vel_damping", ctypes.c_int), ("mpc_mode", ctypes.c_int),
                ("warps_per_cta", ctypes.c_int), ("ctas_per_sm", ctypes.c_int), ("lanes_per_knot", ctypes.c_int)]


class Traj(ctypes.Structure):
    _fields_ = [("n_knots", ctypes.c_int64), ("q", ctypes.c_void_p), ("qd", ctypes.c_void_p),
                ("u", ctypes.c_void_p), ("dqdd", ctypes.c_void_p), ("qdd", ctypes.c_void_p),
                ("minv", ctypes.c_void_p)]


class HostBatch(ctypes.Structure):
    _fields_ = [("n_knots", ctypes.c_int), ("q", ctypes.c_void_p), ("qd", ctypes.c_void_p), ("u", ctypes.c_void_p),
                ("dqdd", ctypes.c_void_p), ("qdd", ctypes.c_void_p), ("minv", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    _fields_ = [("warps_per_cta", ctypes.c_int), ("lanes_per_knot", ctypes.c_int),
                ("ragged_warps_per_cta", ctypes.c_int), ("ragged_ctas_per_sm", ctypes.c_int),
                ("ragged_lanes_per_knot", ctypes.c_int)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("pool_bytes", ctypes.c_size_t), ("max_batch_knots", ctypes.c_int), ("max_inflight", ctypes.c_int),
                ("warps_per_cta", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("latency_mapping_max_knots", ctypes.c_int)]


_fp = ctypes.POINTER(ctypes.c_float)


class RequestInfo(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("traj_id", ctypes.c_uint64), ("horizon", ctypes.c_int64),
                ("status", ctypes.c_int), ("dqdd", _fp), ("qdd", _fp), ("minv", _fp), ("dev_q", ctypes.c_void_p),
                ("dev_qd", ctypes.c_void_p), ("dev_u", ctypes.c_void_p), ("dev_dqdd", ctypes.c_void_p),
                ("dev_qdd", ctypes.c_void_p), ("dev_minv", ctypes.c_void_p), ("latency_us", ctypes.c_double),
                ("queue_us", ctypes.c_double), ("batch_id", ctypes.c_uint64), ("batch_requests", ctypes.c_int)]


class SlotInfo(ctypes.Structure):
    _fields_ = [("horizon", ctypes.c_int64), ("q", ctypes.c_void_p), ("qd", ctypes.c_void_p), ("u", ctypes.c_void_p),
                ("dqdd", ctypes.c_void_p), ("qdd", ctypes.c_void_p), ("minv", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("knots", ctypes.c_uint64), ("admission_stalls", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("pool_bytes_cap", ctypes.c_size_t), ("pool_bytes_used", ctypes.c_size_t),
                ("pool_bytes_peak", ctypes.c_size_t), ("queued_admission", ctypes.c_size_t),
                ("queued_ready", ctypes.c_size_t), ("cancelled", ctypes.c_uint64)]


_lib = None


def _declare(L):
    vp, i32, i64, st = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int
    sig = {
        "frg_options_default": (None, [ctypes.POINTER(Options)]),
        "frg_status_string": (ctypes.c_char_p, [st]),
        "frg_create": (st, [ctypes.POINTER(vp), ctypes.POINTER(Options)]),
        "frg_destroy": (None, [vp]),
        "frg_last_error": (ctypes.c_char_p, [vp]),
        "frg_set_launch_shape": (st, [vp, i32, i32]),
        "frg_get_launch_shape": (st, [vp, ctypes.POINTER(i32), ctypes.POINTER(i32)]),
        "frg_set_lanes_per_knot": (st, [vp, i32]),
        "frg_get_lanes_per_knot": (i32, [vp]),
        "frg_gradient": (st, [vp, i32, vp, vp, vp, vp, vp, vp, vp]),
        "frg_gradient_host": (st, [vp, i32, vp, vp, vp, vp, vp, vp]),
        "frg_gradient_per_trajectory": (st, [vp, i32, ctypes.POINTER(Traj), vp]),
        "frg_gradient_batched": (st, [vp, i32, ctypes.POINTER(Traj), vp]),
        "frg_gradient_ragged": (st, [vp, i32, ctypes.POINTER(i64), vp, vp, vp, vp, vp, vp, vp]),
        "frg_plan_create": (st, [vp, i32, ctypes.POINTER(Traj), ctypes.POINTER(vp)]),
        "frg_plan_create_ragged": (st, [vp, i32, ctypes.POINTER(i64), vp, vp, vp, vp, vp, vp, ctypes.POINTER(vp)]),
        "frg_plan_launch": (st, [vp, vp]),
        "frg_plan_launch_many": (st, [vp, i32, ctypes.POINTER(vp), i32, vp]),
        "frg_plan_knots": (i64, [vp]),
        "frg_plan_destroy": (None, [vp]),
        "frg_autotune": (st, [vp, i64, ctypes.POINTER(ctypes.c_double)]),
        "frg_host_alloc": (vp, [ctypes.c_size_t]),
        "frg_host_free": (None, [vp]),
        "frg_gradient_ragged_noalloc": (st, [vp, i32, ctypes.POINTER(i64), vp, vp, vp, vp, vp, vp, vp]),
        "frg_server_options_default": (None, [ctypes.POINTER(ServerOptions)]),
        "frg_server_create": (st, [vp, ctypes.POINTER(ServerOptions), ctypes.POINTER(vp)]),
        "frg_server_destroy": (None, [vp]),
        "frg_server_submit": (st, [vp, ctypes.c_uint64, i64, vp, vp, vp, ctypes.POINTER(ctypes.c_uint64)]),
        "frg_server_poll": (st, [vp, ctypes.c_uint64, ctypes.POINTER(RequestInfo)]),
        "frg_server_wait": (st, [vp, ctypes.c_uint64, i64, ctypes.POINTER(RequestInfo)]),
        "frg_server_wait_any": (st, [vp, i64, ctypes.POINTER(RequestInfo)]),
        "frg_server_release": (st, [vp, ctypes.c_uint64]),
        "frg_server_cancel": (st, [vp, ctypes.c_uint64]),
        "frg_server_get_stats": (st, [vp, ctypes.POINTER(ServerStats)]),
        "frg_gradient_fext": (st, [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
        "frg_forward_dynamics": (st, [vp, i32, vp, vp, vp, vp, vp, vp, vp]),
        "frg_discrete_jacobians": (st, [vp, i32, vp, vp, ctypes.c_float, vp, vp, vp]),
        "frg_gradient_f64": (st, [vp, i32, vp, vp, vp, vp, vp, vp, vp]),
        "frg_verify_f64": (st, [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
        "frg_get_tuning": (st, [vp, ctypes.POINTER(Tuning)]),
        "frg_set_tuning": (st, [vp, ctypes.POINTER(Tuning)]),
        "frg_knot_status": (st, [vp, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
        "frg_model_name": (ctypes.c_char_p, []),
        "frg_gradient_knots": (st, [vp, i32, vp, vp, vp]),
        "frg_single_knot_latency": (st, [vp, i32, i32, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_double)]),
        "frg_server_submit_device": (st, [vp, ctypes.c_uint64, i64, vp, vp, vp, ctypes.c_uint,
                                          ctypes.POINTER(ctypes.c_uint64)]),
        "frg_server_submit_resident": (st, [vp, ctypes.c_uint64, ctypes.c_uint, ctypes.POINTER(ctypes.c_uint64)]),
        "frg_server_slot": (st, [vp, ctypes.c_uint64, ctypes.POINTER(SlotInfo)]),
        "frg_model_dofs": (i32, []),
        "frg_gradient_host_batches": (st, [vp, i32, ctypes.POINTER(HostBatch)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """The loaded libfrg.so (raises FrgError if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FrgError(9, f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                              "(the engine is CUDA-only and has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def dims():
    """(N, 2 N^2, N^2): joints, gradient floats and Minv floats per knot of the
    loaded library (the robot it was built for)."""
    n = lib().frg_model_dofs()
    return n, 2 * n * n, n * n


def model_name():
    """Name of the robot compiled into the loaded library."""
    return lib().frg_model_name().decode()


def _ptr(x):
    """Device/host address of an int, a torch tensor, a numpy array or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def make_trajs(trajs):
    """(ctypes array, count) from dicts/tuples (n, q, qd, u, dqdd, qdd, minv)."""
    arr = (Traj * max(1, len(trajs)))()
    for i, t in enumerate(trajs):
        n, q, qd, u, dqdd, qdd, minv = t
        arr[i] = Traj(int(n), _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd), _ptr(minv))
    return arr, len(trajs)


class Plan:
    def __init__(self, ctx, handle):
        self._ctx, self._h = ctx, handle

    @property
    def knots(self):
        return lib().frg_plan_knots(self._h)

    def launch(self, stream=None):
        self._ctx._check(lib().frg_plan_launch(self._h, _stream_ptr(stream)), "frg_plan_launch")

    def close(self):
        if self._h:
            lib().frg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """An engine context on one CUDA device (frg_create / frg_destroy)."""

    def __init__(self, device=0, vel_damping=False, mpc_mode=False, warps_per_cta=0, ctas_per_sm=0, lanes_per_knot=0):
        L = lib()
        opt = Options()
        L.frg_options_default(ctypes.byref(opt))
        opt.device, opt.vel_damping, opt.mpc_mode = int(device), int(bool(vel_damping)), int(bool(mpc_mode))
        opt.warps_per_cta, opt.ctas_per_sm = int(warps_per_cta), int(ctas_per_sm)
        opt.lanes_per_knot = int(lanes_per_knot)
        h = ctypes.c_void_p()
        st = L.frg_create(ctypes.byref(h), ctypes.byref(opt))
        if st != FRG_OK:
            raise FrgError(st, "frg_create: " + L.frg_last_error(None).decode())
        self._h = h
        self.device = device
        self.vel_damping, self.mpc_mode = bool(vel_damping), bool(mpc_mode)

    def close(self):
        if getattr(self, "_h", None):
            lib().frg_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, st, what):
        if st != FRG_OK:
            msg = lib().frg_last_error(self._h).decode()
            raise FrgError(st, msg if msg.startswith(what) else f"{what}: {msg}")

    def last_error(self):
        return lib().frg_last_error(self._h).decode()

    # ---------------------------------------------------------- shapes
    def launch_shape(self):
        w, c = ctypes.c_int(), ctypes.c_int()
        self._check(lib().frg_get_launch_shape(self._h, ctypes.byref(w), ctypes.byref(c)), "frg_get_launch_shape")
        return w.value, c.value

    def set_launch_shape(self, warps_per_cta, ctas_per_sm):
        self._check(lib().frg_set_launch_shape(self._h, int(warps_per_cta), int(ctas_per_sm)), "frg_set_launch_shape")

    def lanes_per_knot(self):
        return lib().frg_get_lanes_per_knot(self._h)

    def set_lanes_per_knot(self, lanes):
        self._check(lib().frg_set_lanes_per_knot(self._h, int(lanes)), "frg_set_lanes_per_knot")

    def autotune(self, n_knots):
        best = ctypes.c_double()
        self._check(lib().frg_autotune(self._h, int(n_knots), ctypes.byref(best)), "frg_autotune")
        return best.value

    def tuning(self):
        """The tuned launch shapes as a dict (to cache and restore with set_tuning)."""
        t = Tuning()
        self._check(lib().frg_get_tuning(self._h, ctypes.byref(t)), "frg_get_tuning")
        return {f: getattr(t, f) for f, _ in Tuning._fields_}

    def set_tuning(self, tuning):
        t = Tuning(**{f: int(tuning[f]) for f, _ in Tuning._fields_})
        self._check(lib().frg_set_tuning(self._h, ctypes.byref(t)), "frg_set_tuning")

    # ---------------------------------------------------------- calls
    def gradient(self, n_knots, q, qd, u, dqdd, qdd, minv, stream=None):
        """Plain path on device buffers (addresses, torch tensors)."""
        self._check(lib().frg_gradient(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd),
                                       _ptr(minv), _stream_ptr(stream)), "frg_gradient")

    def single_knot_latency(self, lanes_per_knot, iters, q, qd, u, dqdd, qdd, minv, stream=None, timed=False):
        """One knot (device arrays) through the whole path `iters` times in one
        launch; with timed=True waits and returns µs per repetition (CUDA events,
        launch included)."""
        us = ctypes.c_double(0.0)
        self._check(lib().frg_single_knot_latency(self._h, int(lanes_per_knot), int(iters), _ptr(q), _ptr(qd), _ptr(u),
                                                  _ptr(dqdd), _ptr(qdd), _ptr(minv), _stream_ptr(stream),
                                                  ctypes.byref(us) if timed else None), "frg_single_knot_latency")
        return us.value if timed else None

    def gradient_fext(self, n_knots, q, qd, u, fext, dqdd, qdd, minv, stream=None):
        """Gradient with external link forces fext [n][7][6] (device buffers)."""
        self._check(lib().frg_gradient_fext(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(fext), _ptr(dqdd),
                                            _ptr(qdd), _ptr(minv), _stream_ptr(stream)), "frg_gradient_fext")

    def forward_dynamics(self, n_knots, q, qd, u, qdd, minv=None, fext=None, stream=None):
        """q̈ (and Minv if given) only (device buffers)."""
        self._check(lib().frg_forward_dynamics(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(fext), _ptr(qdd),
                                               _ptr(minv), _stream_ptr(stream)), "frg_forward_dynamics")

    def discrete_jacobians(self, n_knots, dqdd, minv, dt, A, B, stream=None):
        """Explicit-Euler A [n][14x14], B [n][14x7] from dqdd and minv (device buffers)."""
        self._check(lib().frg_discrete_jacobians(self._h, int(n_knots), _ptr(dqdd), _ptr(minv), float(dt), _ptr(A),
                                                 _ptr(B), _stream_ptr(stream)), "frg_discrete_jacobians")

    def gradient_knots(self, n_knots, knots, dqdd, stream=None):
        """The reference's packed knot records [n, 77] (device): q, qd, u in;
        q̈ and Minv written into the records; the gradient to dqdd [n, 98]."""
        self._check(lib().frg_gradient_knots(self._h, int(n_knots), _ptr(knots), _ptr(dqdd), _stream_ptr(stream)),
                    "frg_gradient_knots")

    def knot_status(self, n_knots, q, qd, u, dqdd, qdd, minv, status, stream=None):
        """status [n] (uint32/int32 device buffer): KNOT_NONFINITE_INPUT / _OUTPUT flags per knot."""
        self._check(lib().frg_knot_status(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd),
                                          _ptr(minv), _ptr(status), _stream_ptr(stream)), "frg_knot_status")

    def gradient_f64(self, n_knots, q, qd, u, dqdd, qdd, minv, stream=None):
        """FP64 verification build of the plain path (device double buffers)."""
        self._check(lib().frg_gradient_f64(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd),
                                           _ptr(minv), _stream_ptr(stream)), "frg_gradient_f64")

    def verify_f64(self, n_knots, q, qd, u, dqdd, qdd, minv, err, stream=None):
        """Per-knot Frobenius-relative errors err [n,3] (device doubles) of the
        FP32 results dqdd, qdd, minv against the FP64 build on the same inputs."""
        self._check(lib().frg_verify_f64(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd),
                                         _ptr(minv), _ptr(err), _stream_ptr(stream)), "frg_verify_f64")

    def gradient_host_into(self, n_knots, q, qd, u, dqdd, qdd, minv):
        """Host-buffer path: inputs in, outputs written to the given host arrays."""
        self._check(lib().frg_gradient_host(self._h, int(n_knots), _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd),
                                            _ptr(qdd), _ptr(minv)), "frg_gradient_host")

    def gradient_host_batches(self, batches):
        """Host-buffer batches in one call: each (n, q, qd, u, dqdd, qdd, minv)
        with host arrays or addresses; two launches kept in flight."""
        arr = (HostBatch * max(1, len(batches)))()
        for i, (n, *ptrs) in enumerate(batches):
            arr[i] = HostBatch(int(n), *[_ptr(p) for p in ptrs])
        self._check(lib().frg_gradient_host_batches(self._h, len(batches), arr), "frg_gradient_host_batches")

    def gradient_host(self, q, qd, u, want_qdd=True, want_minv=True):
        """numpy float32 [n,N] x3 -> (dqdd [n,2N^2], qdd [n,N], minv [n,N^2]);
        a result not wanted is None and is not copied back."""
        import numpy as np
        q, qd, u = (np.ascontiguousarray(x, dtype=np.float32) for x in (q, qd, u))
        n = q.shape[0]
        nj, nd, nm = dims()
        dqdd = np.empty((n, nd), np.float32)
        qdd = np.empty((n, nj), np.float32) if want_qdd else None
        minv = np.empty((n, nm), np.float32) if want_minv else None
        self.gradient_host_into(n, q, qd, u, dqdd, qdd, minv)
        return dqdd, qdd, minv

    def per_trajectory(self, trajs, stream=None):
        arr, n = make_trajs(trajs)
        self._check(lib().frg_gradient_per_trajectory(self._h, n, arr, _stream_ptr(stream)),
                    "frg_gradient_per_trajectory")

    def batched(self, trajs, stream=None):
        arr, n = make_trajs(trajs)
        self._check(lib().frg_gradient_batched(self._h, n, arr, _stream_ptr(stream)), "frg_gradient_batched")

    def ragged(self, offsets, q, qd, u, dqdd, qdd, minv, stream=None):
        import numpy as np
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        self._check(lib().frg_gradient_ragged(self._h, len(off) - 1, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                              _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd), _ptr(minv),
                                              _stream_ptr(stream)), "frg_gradient_ragged")

    def plan(self, trajs):
        arr, n = make_trajs(trajs)
        h = ctypes.c_void_p()
        self._check(lib().frg_plan_create(self._h, n, arr, ctypes.byref(h)), "frg_plan_create")
        return Plan(self, h)

    def plan_launch_many(self, plans, stream=None, in_flight=2):
        """Independent plans, several in flight (frg_plan_launch_many): plan
        i runs on stream i mod in_flight; plans at positions of different
        residues must not share memory that either one writes."""
        arr = (ctypes.c_void_p * max(1, len(plans)))(*[p._h for p in plans])
        self._check(lib().frg_plan_launch_many(self._h, len(plans), arr, int(in_flight), _stream_ptr(stream)),
                    "frg_plan_launch_many")

    def plan_ragged(self, offsets, q, qd, u, dqdd, qdd, minv):
        import numpy as np
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        h = ctypes.c_void_p()
        self._check(lib().frg_plan_create_ragged(self._h, len(off) - 1, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                                 _ptr(q), _ptr(qd), _ptr(u), _ptr(dqdd), _ptr(qdd), _ptr(minv),
                                                 ctypes.byref(h)), "frg_plan_create_ragged")
        return Plan(self, h)


class Server:
    """Continuous-batching server on a context (frg_server_*)."""

    def __init__(self, ctx, pool_bytes=1 << 30, max_batch_knots=1 << 16, max_inflight=3, warps_per_cta=0,
                 ctas_per_sm=0, latency_mapping_max_knots=None):
        L = lib()
        opt = ServerOptions()
        L.frg_server_options_default(ctypes.byref(opt))
        opt.pool_bytes, opt.max_batch_knots, opt.max_inflight = int(pool_bytes), int(max_batch_knots), int(max_inflight)
        opt.warps_per_cta, opt.ctas_per_sm = int(warps_per_cta), int(ctas_per_sm)
        if latency_mapping_max_knots is not None:
            opt.latency_mapping_max_knots = int(latency_mapping_max_knots)
        h = ctypes.c_void_p()
        ctx._check(L.frg_server_create(ctx.handle, ctypes.byref(opt), ctypes.byref(h)), "frg_server_create")
        self._ctx, self._h = ctx, h

    def close(self):
        if getattr(self, "_h", None):
            lib().frg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, traj_id, q, qd, u):
        """Queue one call; returns (status, request_id).  q, qd, u: float32 [h, 7]."""
        rid = ctypes.c_uint64()
        st = lib().frg_server_submit(self._h, int(traj_id), int(q.shape[0]), q.ctypes.data, qd.ctypes.data,
                                     u.ctypes.data, ctypes.byref(rid))
        return st, rid.value

    def submit_device(self, traj_id, q, qd, u, host_results=False):
        """Queue one call on inputs already on the GPU (torch CUDA tensors
        [h, 7], float32, unchanged until the call completes); returns
        (status, request_id)."""
        rid = ctypes.c_uint64()
        st = lib().frg_server_submit_device(self._h, int(traj_id), int(q.shape[0]), _ptr(q), _ptr(qd), _ptr(u),
                                            SERVE_HOST_RESULTS if host_results else 0, ctypes.byref(rid))
        return st, rid.value

    def submit_resident(self, traj_id, host_results=False):
        """Queue one call on the trajectory's resident device inputs."""
        rid = ctypes.c_uint64()
        st = lib().frg_server_submit_resident(self._h, int(traj_id), SERVE_HOST_RESULTS if host_results else 0,
                                              ctypes.byref(rid))
        return st, rid.value

    def slot(self, traj_id):
        """(status, SlotInfo) of the trajectory's device slot."""
        info = SlotInfo()
        st = lib().frg_server_slot(self._h, int(traj_id), ctypes.byref(info))
        return st, info

    def wait(self, request_id, timeout_us=-1):
        info = RequestInfo()
        st = lib().frg_server_wait(self._h, int(request_id), int(timeout_us), ctypes.byref(info))
        return st, info

    def poll(self, request_id):
        info = RequestInfo()
        st = lib().frg_server_poll(self._h, int(request_id), ctypes.byref(info))
        return st, info

    def wait_any(self, timeout_us=-1):
        info = RequestInfo()
        st = lib().frg_server_wait_any(self._h, int(timeout_us), ctypes.byref(info))
        return st, info

    def release(self, traj_id):
        return lib().frg_server_release(self._h, int(traj_id))

    def cancel(self, request_id):
        """Withdraw a call not yet on the GPU; returns the status code."""
        return lib().frg_server_cancel(self._h, int(request_id))

    def stats(self):
        s = ServerStats()
        lib().frg_server_get_stats(self._h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    @staticmethod
    def results(info):
        """Copies of (dqdd [h,2N^2], qdd [h,N], minv [h,N^2]) from a completed call's info."""
        import numpy as np
        h = info.horizon
        nj, nd, nm = dims()
        return tuple(np.ctypeslib.as_array(p, shape=(h, w)).copy()
                     for p, w in ((info.dqdd, nd), (info.qdd, nj), (info.minv, nm)))


def forward_dynamics_gradient(q, qd, u, vel_damping=False, mpc_mode=False, ctx=None, stream=None):
    """Batch gradient on torch CUDA tensors [n,N] (float32): returns
    (dqdd [n,2N^2], qdd [n,N], minv [n,N^2]) on the same device,
    asynchronously on `stream` (default: torch's current stream)."""
    import torch
    nj, nd, nm = dims()
    for t in (q, qd, u):
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.shape[-1] == nj):
            raise ValueError(f"q, qd, u must be contiguous float32 CUDA tensors of shape [n, {nj}]")
    n = q.shape[0]
    dev = q.device
    own = ctx is None
    if own:
        ctx = Context(device=dev.index or 0, vel_damping=vel_damping, mpc_mode=mpc_mode)
    try:
        dqdd = torch.empty((n, nd), device=dev, dtype=torch.float32)
        qdd = torch.empty((n, nj), device=dev, dtype=torch.float32)
        minv = torch.empty((n, nm), device=dev, dtype=torch.float32)
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        ctx.gradient(n, q, qd, u, dqdd, qdd, minv, stream=st)
        if own:
            st.synchronize()
    finally:
        if own:
            ctx.close()
    return dqdd, qdd, minv
