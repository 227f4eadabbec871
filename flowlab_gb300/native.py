"""ctypes binding of the engine's C ABI (include/flowlab_gb300.h).

The shared library is built in-tree by flowlab_gb300.build into
flowlab_gb300/_lib/libflowlab_gb300.so. There is no fallback: if the library
is missing, or no CUDA device is usable, the calls below raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libflowlab_gb300.so")

FL_OK, FL_EINVAL, FL_EBUSY, FL_EDEVICE, FL_ETIMEOUT, FL_ENONFINITE, FL_ENOMEM, FL_ESTATE = range(8)
FL_F32, FL_F64 = 0, 1
FL_SEMI_LAGRANGIAN, FL_MACCORMACK = 0, 1
FL_SOLVER_RBSOR, FL_SOLVER_MG = 0, 1

STATUS_NAMES = {
    FL_OK: "ok", FL_EINVAL: "invalid argument", FL_EBUSY: "not re-entrant", FL_EDEVICE: "device error",
    FL_ETIMEOUT: "device wait timed out", FL_ENONFINITE: "non-finite result", FL_ENOMEM: "out of device memory",
    FL_ESTATE: "call out of order",
}


class FlowlabError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(status, "error"), status, message))
        self.status = status


class Params(ctypes.Structure):
    """fl_params (field order is the ABI)."""

    _fields_ = [
        ("cfl_target", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("scheme", ctypes.c_int),
        ("solver", ctypes.c_int),
        ("pressure_iters", ctypes.c_int),
        ("mg_max_cycles", ctypes.c_int),
        ("omega", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("dye_decay", ctypes.c_double * 3),
        ("beta", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("confinement", ctypes.c_double),
        ("mg_pre", ctypes.c_int),
        ("mg_post", ctypes.c_int),
        ("mg_coarse_sweeps", ctypes.c_int),
        ("mg_coarsest", ctypes.c_int),
        ("mg_omega", ctypes.c_double),
        ("mixed", ctypes.c_int),
        ("rb_pairs", ctypes.c_int),
        ("warm_extrapolate", ctypes.c_int),
        ("mg_tail_side", ctypes.c_int),
        ("residual_every", ctypes.c_int),
        ("reserved", ctypes.c_int * 3),
    ]


class Stats(ctypes.Structure):
    """fl_stats."""

    _fields_ = [
        ("dt", ctypes.c_double),
        ("scale", ctypes.c_double),
        ("grad_scale", ctypes.c_double),
        ("time", ctypes.c_double),
        ("cycles", ctypes.c_int),
        ("steps", ctypes.c_int),
        ("rel_residual", ctypes.c_double),
        ("div_rms", ctypes.c_double),
        ("max_face_speed", ctypes.c_double),
        ("post_div_rms", ctypes.c_double),
        ("post_div_max", ctypes.c_double),
        ("post_div_step", ctypes.c_longlong),
        ("initial_rel_residual", ctypes.c_double),
    ]


ABI_VERSION = 3  # FL_ABI_VERSION

PHASES = ["advect_velocity", "body_forces", "divergence", "mg_pre_fine", "mg_pre", "mg_coarse", "mg_post",
          "mg_post_fine", "defect64", "rb_sweeps", "project", "advect_dye", "cfl", "control", "warm_start"]


class Profile(ctypes.Structure):
    """fl_profile."""

    _fields_ = [
        ("ms", ctypes.c_double * len(PHASES)),
        ("launches", ctypes.c_longlong * len(PHASES)),
        ("bytes", ctypes.c_double * len(PHASES)),
    ]


# (name, restype, argtypes) for every entry point of include/flowlab_gb300.h
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double
SIGNATURES = [
    ("fl_default_params", None, [_P]),
    ("fl_abi_version", _I, []),
    ("fl_last_error", ctypes.c_char_p, [_P]),
    ("fl_create", _I, [_I, _I, _D, _I, _P, _I, ctypes.POINTER(_P)]),
    ("fl_destroy", _I, [_P]),
    ("fl_set_params", _I, [_P, _P]),
    ("fl_stream", _P, [_P]),
    ("fl_synchronize", _I, [_P]),
    ("fl_upload_fields", _I, [_P, _I, _P, _P, _P, _P, _P]),
    ("fl_set_labels", _I, [_P, _P]),
    ("fl_set_dye_patch", _I, [_P, _I, _I, _I, _I, _P]),
    ("fl_set_buoyancy", _I, [_P, _D, _D]),
    ("fl_set_confinement", _I, [_P, _D]),
    ("fl_set_stir", _I, [_P, _P]),
    ("fl_step", _I, [_P, _I, _D, _D, _D, _P, _P]),
    ("fl_step_auto", _I, [_P, _I, _P]),
    ("fl_step_host", _I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("fl_get_stats", _I, [_P, _P]),
    ("fl_read_velocity", _I, [_P, _I, _P, _P]),
    ("fl_read_dye", _I, [_P, _I, _P]),
    ("fl_read_pressure", _I, [_P, _I, _P]),
    ("fl_read_divergence", _I, [_P, _I, _P]),
    ("fl_profile_enable", _I, [_P, _I]),
    ("fl_profile_read", _I, [_P, _P]),
    ("fl_advect_velocity", _I, [_P, _I, _P, _P, _P, _P, _P, _F]),
    ("fl_advect_dye", _I, [_P, _I, _P, _P, _P, _P, _P, _F]),
    ("fl_rb_solve", _I, [_P, _P, _P, _P, _F, _I, _F, _D, _P]),
    ("fl_mg_solve", _I, [_P, _P, _P, _P, _F, _I, _D, _P, _P]),
    ("fl_mg_solve_mixed", _I, [_P, _P, _P, _P, _F, _I, _D, _P, _P]),
    ("fl_divergence", _I, [_P, _P, _P, _P]),
    ("fl_rb_sweep", _I, [_P, _P, _P, _P, _F, _F, _I]),
    ("fl_subtract_gradient", _I, [_P, _P, _P, _P, _P, _F]),
    ("fl_outflow", _I, [_P, _P, _P, _P]),
    ("fl_commit_labels", _I, [_P, _P, _P, _P, _P, _P]),
    ("fl_body_forces", _I, [_P, _P, _P, _P, _P, _F, _F, _F, _F]),
    ("fl_stir", _I, [_P, _P, _P, _P, _F, _F, _F, _F, _F]),
    ("fl_dye_patch", _I, [_P, _P, _I, _I, _I, _I, _P]),
    ("fl_advect_velocity_noalloc", _I, [_I, _I, _I, _F, _F, _P, _P, _P, _P, _P, _P]),
    ("fl_unet_create", _I, [ctypes.c_longlong, _I, ctypes.POINTER(_P)]),
    ("fl_unet_destroy", _I, [_P]),
    ("fl_unet_last_error", ctypes.c_char_p, [_P]),
    ("fl_unet_num_params", ctypes.c_longlong, []),
    ("fl_unet_set_params", _I, [_P, _P]),
    ("fl_unet_get_params", _I, [_P, _P]),
    ("fl_unet_forward", _I, [_P, _I, _I, _I, _P, _P]),
    ("fl_unet_train_step", _I, [_P, _I, _I, _I, _P, _P, _P, _D, _I, _P, _P]),
    ("fl_unet_use_tensor_cores", _I, [_I]),
    ("fl_unet_set_wait_limit", _I, [ctypes.c_longlong]),
    ("fl_set_warm_start", _I, [_P, _P]),
    ("fl_read_rhs", _I, [_P, _I, _P]),
    ("fl_batch_create", _I, [_P, _I, ctypes.POINTER(_P)]),
    ("fl_batch_destroy", _I, [_P]),
    ("fl_batch_last_error", ctypes.c_char_p, [_P]),
    ("fl_batch_stream", _P, [_P]),
    ("fl_batch_worklist", _I, [_P]),
    ("fl_batch_set_worklist", _I, [_P, _I]),
    ("fl_batch_step", _I, [_P, _I]),
]

_lib = None


def load():
    """Load the engine library (built in-tree). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "flowlab_gb300 CUDA library not built: %s is missing (run flowlab_gb300.build.build())" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.fl_abi_version() != ABI_VERSION:
        raise RuntimeError("flowlab_gb300 ABI version mismatch")
    _lib = lib
    return lib


# fl_default_params' values (simulation.ts:223-234, pressureMultigrid.ts:47-67),
# held here so that building parameters needs neither the library nor a GPU;
# a CPU test checks them against the library's own.
DEFAULTS = dict(cfl_target=2.0, dt_max=1.0 / 30.0, rho=1.0, scheme=FL_SEMI_LAGRANGIAN, solver=FL_SOLVER_MG,
                pressure_iters=100, mg_max_cycles=3, omega=1.9, tol=5e-3, dye_decay=(0.0, 0.0, 0.0), beta=0.0,
                alpha=0.0, confinement=0.0, mg_pre=2, mg_post=2, mg_coarse_sweeps=8, mg_coarsest=4, mg_omega=1.0,
                mixed=0, rb_pairs=0, warm_extrapolate=0, mg_tail_side=0, residual_every=1)


def default_params(**overrides):
    """fl_params with the reference defaults and the given fields replaced."""
    p = Params()
    for k, v in DEFAULTS.items():
        if k == "dye_decay":
            p.dye_decay[:] = list(v)
        else:
            setattr(p, k, v)
    for k, v in overrides.items():
        if k == "dye_decay":
            p.dye_decay[:] = list(v)
        else:
            setattr(p, k, v)
    return p


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Engine:
    """Owns one fl_engine*: the device side for an nx*ny grid."""

    def __init__(self, nx, ny, h=None, dye_scale=1, params=None, device=0):
        self.lib = load()
        self.nx, self.ny, self.dye_scale = nx, ny, dye_scale
        self.dnx, self.dny = nx * dye_scale, ny * dye_scale
        self.h = 1.0 / ny if h is None else h
        self.params = params if params is not None else default_params()
        handle = ctypes.c_void_p()
        st = self.lib.fl_create(nx, ny, self.h, dye_scale, ctypes.byref(self.params), device, ctypes.byref(handle))
        if st != FL_OK:
            raise FlowlabError(st, self.lib.fl_last_error(None).decode())
        self.handle = handle

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fl_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        if st != FL_OK:
            raise FlowlabError(st, self.lib.fl_last_error(self.handle).decode())

    def call(self, name, *args):
        self.check(getattr(self.lib, name)(self.handle, *args))

    # sizes
    @property
    def cells(self):
        return self.nx * self.ny

    @property
    def ufaces(self):
        return (self.nx + 1) * self.ny

    @property
    def vfaces(self):
        return self.nx * (self.ny + 1)

    @property
    def dye_len(self):
        return 3 * self.dnx * self.dny

    def stream(self):
        return self.lib.fl_stream(self.handle)

    def set_params(self, params):
        self.params = params
        self.call("fl_set_params", ctypes.byref(params))

    def profile(self, enable=None):
        """Per-phase {name: (ms, launches, bytes)} since profiling was enabled."""
        if enable is not None:
            self.call("fl_profile_enable", int(enable))
            return None
        p = Profile()
        self.call("fl_profile_read", ctypes.byref(p))
        return {n: (p.ms[k], p.launches[k], p.bytes[k]) for k, n in enumerate(PHASES)}

    def stats(self):
        s = Stats()
        self.call("fl_get_stats", ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in Stats._fields_}


class Unet:
    """The pressure warm-start network (fl_unet_*): a handle plus helpers
    taking numpy arrays."""

    def __init__(self, max_pixels, device=0):
        lib = load()
        h = ctypes.c_void_p()
        st = lib.fl_unet_create(int(max_pixels), device, ctypes.byref(h))
        if st != FL_OK:
            raise FlowlabError(st, lib.fl_last_error(None).decode())
        self.lib, self.h = lib, h
        self.n = int(lib.fl_unet_num_params())

    def close(self):
        if self.h:
            self.lib.fl_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name, *args):
        st = getattr(self.lib, name)(self.h, *args)
        if st != FL_OK:
            raise FlowlabError(st, self.lib.fl_unet_last_error(self.h).decode())

    def set_params(self, theta):
        self.call("fl_unet_set_params", ptr(f32(theta)))

    def get_params(self):
        out = np.empty(self.n, np.float32)
        self.call("fl_unet_get_params", ptr(out))
        return out

    def forward(self, x):
        x = f32(x)
        B, H, W, _ = x.shape
        out = np.empty((B, H, W), np.float32)
        self.call("fl_unet_forward", B, H, W, ptr(x), ptr(out))
        return out

    def train_step(self, x, target, mask, lr=1e-3, update=True, want_grad=False):
        x, target, mask = f32(x), f32(target), f32(mask)
        B, H, W, _ = x.shape
        loss = ctypes.c_double()
        grad = np.empty(self.n, np.float32) if want_grad else None
        self.call("fl_unet_train_step", B, H, W, ptr(x), ptr(target), ptr(mask), float(lr), int(update),
                  ctypes.byref(loss), ptr(grad) if grad is not None else None)
        return (loss.value, grad) if want_grad else loss.value


class Batch:
    """Several engines stepped by one graph launch per step (fl_batch_*)."""

    def __init__(self, engines):
        lib = load()
        self.lib = lib
        self.engines = list(engines)
        arr = (ctypes.c_void_p * len(self.engines))(*[e.handle for e in self.engines])
        h = ctypes.c_void_p()
        st = lib.fl_batch_create(arr, len(self.engines), ctypes.byref(h))
        if st != FL_OK:
            raise FlowlabError(st, lib.fl_last_error(None).decode())
        self.h = h

    def step(self, n=1):
        st = self.lib.fl_batch_step(self.h, int(n))
        if st != FL_OK:
            raise FlowlabError(st, self.lib.fl_batch_last_error(self.h).decode())

    def stream(self):
        return self.lib.fl_batch_stream(self.h)

    @property
    def worklist(self):
        """True when the scenes' solves run as one launch per V-cycle phase."""
        return bool(self.lib.fl_batch_worklist(self.h))

    def set_worklist(self, on):
        st = self.lib.fl_batch_set_worklist(self.h, int(bool(on)))
        if st != FL_OK:
            raise FlowlabError(st, self.lib.fl_batch_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.fl_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
