"""ctypes front end of the oracle: the CPU restatement of flowlab's src/core.

TEST INFRASTRUCTURE ONLY — the checker the tests, the smoke check and the
bench's CPU-baseline leg compare the CUDA engine against. The product
(flowlab_gb300) never imports this package.

`Oracle("f64")` restates the reference's float64 path; `Oracle("f32")` runs the
identical operations in float32 (the ordering oracle the CUDA kernels must
match bit for bit). All arrays are numpy arrays in the reference's MAC layout
(grid.ts:1-36); dye is one array of 3 planes laid end to end.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None

FLUID, AIR, SOLID = 0, 1, 2


class Params(ctypes.Structure):
    """Mirror of orc_params in oracle_capi.cpp (field order is the ABI)."""

    _fields_ = [
        ("cflTarget", ctypes.c_double),
        ("dtMax", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("macCormack", ctypes.c_int),
        ("solver", ctypes.c_int),
        ("pressureIters", ctypes.c_int),
        ("mgMaxCycles", ctypes.c_int),
        ("omega", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("dyeDecay", ctypes.c_double * 3),
        ("beta", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("confinement", ctypes.c_double),
        ("mgPre", ctypes.c_int),
        ("mgPost", ctypes.c_int),
        ("mgCoarseSweeps", ctypes.c_int),
        ("mgCoarsest", ctypes.c_int),
        ("mgOmega", ctypes.c_double),
        ("mixed", ctypes.c_int),
        ("warmExtrapolate", ctypes.c_int),
        ("residualEvery", ctypes.c_int),
    ]


SOLVER_RBSOR, SOLVER_MG, SOLVER_SOR = 0, 1, 2


def make_params(**kw):
    """StepParams with the reference defaults (simulation.ts:223-234) and the
    reference multigrid constants (pressureMultigrid.ts:47-67)."""
    p = Params()
    p.cflTarget = 2.0
    p.dtMax = 1.0 / 30.0
    p.rho = 1.0
    p.macCormack = 0
    p.solver = SOLVER_RBSOR
    p.pressureIters = 100
    p.mgMaxCycles = 3
    p.omega = 1.9
    p.tol = 5e-3
    p.dyeDecay[:] = [0.0, 0.0, 0.0]
    p.beta = 0.0
    p.alpha = 0.0
    p.confinement = 0.0
    p.mgPre, p.mgPost, p.mgCoarseSweeps, p.mgCoarsest = 2, 2, 8, 4
    p.mgOmega = 1.0
    p.mixed = 0
    p.residualEvery = 1
    for k, v in kw.items():
        if k == "dyeDecay":
            p.dyeDecay[:] = list(v)
        else:
            setattr(p, k, v)
    return p


def params_from_engine(p):
    """The oracle's StepParams for an engine fl_params (flowlab_gb300.native.Params)."""
    return dict(cflTarget=p.cfl_target, dtMax=p.dt_max, rho=p.rho, macCormack=int(p.scheme == 1),
                solver=SOLVER_MG if p.solver == 1 else SOLVER_RBSOR, pressureIters=p.pressure_iters,
                mgMaxCycles=p.mg_max_cycles, omega=p.omega, tol=p.tol, dyeDecay=tuple(p.dye_decay), beta=p.beta,
                alpha=p.alpha, confinement=p.confinement, mgPre=p.mg_pre, mgPost=p.mg_post,
                mgCoarseSweeps=p.mg_coarse_sweeps, mgCoarsest=p.mg_coarsest, mgOmega=p.mg_omega, mixed=p.mixed,
                warmExtrapolate=p.warm_extrapolate, residualEvery=p.residual_every)


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        _LIB = ctypes.CDLL(path)
        _LIB.orc_abi_version.restype = ctypes.c_int
        for suf in ("f64", "f32"):
            for name in ("orc_rms_remaining_", "orc_fluid_div_rms_", "orc_relres_b_"):
                getattr(_LIB, name + suf).restype = ctypes.c_double
            getattr(_LIB, "orc_sim_create_" + suf).restype = ctypes.c_void_p
        _LIB.orc_mg_solve_df_f32.restype = ctypes.c_int
        _LIB.orc_residual_df_f32.restype = ctypes.c_double
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Oracle:
    def __init__(self, precision="f64"):
        assert precision in ("f64", "f32")
        self.suf = precision
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.ct = ctypes.c_double if precision == "f64" else ctypes.c_float
        self.L = lib()

    def _f(self, name):
        return getattr(self.L, "orc_%s_%s" % (name, self.suf))

    def _arr(self, a):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        return a

    def _lab(self, label):
        return np.ascontiguousarray(label, dtype=np.uint8)

    # -------------------------------------------------------------- kernels
    def advect_velocity(self, nx, ny, h, mac, u, v, label, dt):
        u, v, label = self._arr(u), self._arr(v), self._lab(label)
        uo, vo = np.full_like(u, np.nan), np.full_like(v, np.nan)
        self._f("advect_velocity")(nx, ny, self.ct(h), int(mac), _p(u), _p(v), _p(uo), _p(vo), _p(label), self.ct(dt))
        return uo, vo

    def advect_dye(self, nx, ny, h, dnx, dny, dh, mac, u, v, q, label, dt):
        u, v, q, label = self._arr(u), self._arr(v), self._arr(q), self._lab(label)
        qo = np.full_like(q, np.nan)
        self._f("advect_dye")(nx, ny, self.ct(h), dnx, dny, self.ct(dh), int(mac), _p(u), _p(v), _p(q), _p(qo), _p(label), self.ct(dt))
        return qo

    def divergence(self, nx, ny, h, u, v):
        u, v = self._arr(u), self._arr(v)
        out = np.zeros(nx * ny, self.dtype)
        self._f("divergence")(nx, ny, self.ct(h), _p(u), _p(v), _p(out))
        return out

    def rb_sweep(self, nx, ny, p, div, label, scale, omega, color):
        p, div, label = self._arr(p).copy(), self._arr(div), self._lab(label)
        self._f("rb_sweep")(nx, ny, _p(p), _p(div), _p(label), self.ct(scale), self.ct(omega), int(color))
        return p

    def rb_solve(self, nx, ny, p, div, label, scale, iters, omega, tol):
        p, div, label = self._arr(p).copy(), self._arr(div), self._lab(label)
        used = self._f("rb_solve")(nx, ny, _p(p), _p(div), _p(label), self.ct(scale), int(iters), self.ct(omega), ctypes.c_double(tol))
        return p, used

    def gs_sweep(self, nx, ny, p, div, label, scale, omega, rx=False, ry=False):
        p, div, label = self._arr(p).copy(), self._arr(div), self._lab(label)
        self._f("gs_sweep")(nx, ny, _p(p), _p(div), _p(label), self.ct(scale), self.ct(omega), int(rx), int(ry))
        return p

    def sor_solve(self, nx, ny, p, div, label, scale, iters, omega, tol):
        p, div, label = self._arr(p).copy(), self._arr(div), self._lab(label)
        used = self._f("sor_solve")(nx, ny, _p(p), _p(div), _p(label), self.ct(scale), int(iters), self.ct(omega), ctypes.c_double(tol))
        return p, used

    def rms_remaining(self, nx, ny, p, div, label, scale):
        p, div, label = self._arr(p), self._arr(div), self._lab(label)
        return self._f("rms_remaining")(nx, ny, _p(p), _p(div), _p(label), self.ct(scale))

    def fluid_div_rms(self, div, label):
        div, label = self._arr(div), self._lab(label)
        return self._f("fluid_div_rms")(ctypes.c_long(div.size), _p(div), _p(label))

    def relres_b(self, nx, ny, x, b, label):
        x, b, label = self._arr(x), self._arr(b), self._lab(label)
        return self._f("relres_b")(nx, ny, _p(x), _p(b), _p(label))

    def mg_solve(self, nx, ny, p, div, label, scale, cycles, tol, pre=2, post=2, coarse=8, coarsest=4, omega=1.0):
        p, div, label = self._arr(p).copy(), self._arr(div), self._lab(label)
        rr = ctypes.c_double(-1)
        used = self._f("mg_solve")(nx, ny, _p(p), _p(div), _p(label), self.ct(scale), int(cycles), ctypes.c_double(tol),
                                   int(pre), int(post), int(coarse), int(coarsest), ctypes.c_double(omega), ctypes.byref(rr))
        return p, used, rr.value

    def mg_solve_mixed(self, nx, ny, p64, div, label, scale, cycles, tol, pre=2, post=2, coarse=8, coarsest=4,
                       omega=1.0):
        """solveMixed: float64 pressure, defect correction around the multigrid."""
        p64 = np.ascontiguousarray(p64, dtype=np.float64).copy()
        div, label = self._arr(div), self._lab(label)
        rr = ctypes.c_double(-1)
        used = self._f("mg_solve_mixed")(nx, ny, _p(p64), _p(div), _p(label), self.ct(scale), int(cycles),
                                         ctypes.c_double(tol), int(pre), int(post), int(coarse), int(coarsest),
                                         ctypes.c_double(omega), ctypes.byref(rr))
        return p64, used, rr.value

    def mg_solve_df(self, nx, ny, p64, div, label, scale, cycles, tol, pre=2, post=2, coarse=8, coarsest=4,
                    omega=1.0):
        """solveMixedDF (float32 only): the defect correction with a double-float
        pressure. p64 in (float64, split into pairs as the engine does) and out
        (hi + lo in float64)."""
        assert self.suf == "f32"
        p64 = np.ascontiguousarray(p64, dtype=np.float64)
        hi = p64.astype(np.float32)
        pairs = np.empty(2 * p64.size, np.float32)
        pairs[0::2] = hi
        pairs[1::2] = (p64 - hi.astype(np.float64)).astype(np.float32)
        div, label = self._arr(div), self._lab(label)
        rr = ctypes.c_double(-1)
        used = self.L.orc_mg_solve_df_f32(nx, ny, _p(pairs), _p(div), _p(label), ctypes.c_float(scale), int(cycles),
                                          ctypes.c_double(tol), int(pre), int(post), int(coarse), int(coarsest),
                                          ctypes.c_double(omega), ctypes.byref(rr))
        return pairs[0::2].astype(np.float64) + pairs[1::2].astype(np.float64), used, rr.value

    def residual(self, nx, ny, x, b, label):
        x, b, label = self._arr(x), self._arr(b), self._lab(label)
        r = np.zeros(nx * ny, self.dtype)
        self._f("residual")(nx, ny, _p(x), _p(b), _p(label), _p(r))
        return r

    def restrict(self, fnx, fny, r, cnx, cny):
        r = self._arr(r)
        bc = np.full(cnx * cny, np.nan, self.dtype)
        ec = np.full(cnx * cny, np.nan, self.dtype)
        self._f("restrict")(fnx, fny, _p(r), cnx, cny, _p(bc), _p(ec))
        return bc, ec

    def prolong(self, fnx, fny, x, label, cnx, cny, e):
        x, label, e = self._arr(x).copy(), self._lab(label), self._arr(e)
        self._f("prolong")(fnx, fny, _p(x), _p(label), cnx, cny, _p(e))
        return x

    def coarsen_labels(self, fnx, fny, fine, cnx, cny):
        fine = self._lab(fine)
        c = np.zeros(cnx * cny, np.uint8)
        self._f("coarsen_labels")(fnx, fny, _p(fine), cnx, cny, _p(c))
        return c

    def subtract_gradient(self, nx, ny, p, u, v, label, grad_scale):
        p, u, v, label = self._arr(p), self._arr(u).copy(), self._arr(v).copy(), self._lab(label)
        self._f("subtract_gradient")(nx, ny, _p(p), _p(u), _p(v), _p(label), self.ct(grad_scale))
        return u, v

    def commit_labels(self, nx, ny, p, u, v, label, dye=None, dye_cells=0):
        p, u, v, label = self._arr(p).copy(), self._arr(u).copy(), self._arr(v).copy(), self._lab(label)
        d = self._arr(dye).copy() if dye is not None else None
        self._f("commit_labels")(nx, ny, _p(p), _p(u), _p(v), _p(label), _p(d), ctypes.c_long(dye_cells))
        return p, u, v, d

    def outflow(self, nx, ny, u, v, label):
        u, v, label = self._arr(u).copy(), self._arr(v).copy(), self._lab(label)
        self._f("outflow")(nx, ny, _p(u), _p(v), _p(label))
        return u, v

    def buoyancy(self, nx, ny, h, dnx, dny, dh, v, heat, smoke, label, beta, alpha, dt):
        v, heat, smoke, label = self._arr(v).copy(), self._arr(heat), self._arr(smoke), self._lab(label)
        self._f("buoyancy")(nx, ny, self.ct(h), dnx, dny, self.ct(dh), _p(v), _p(heat), _p(smoke), _p(label),
                            self.ct(beta), self.ct(alpha), self.ct(dt))
        return v

    def vorticity(self, nx, ny, h, u, v):
        u, v = self._arr(u), self._arr(v)
        out = np.zeros(nx * ny, self.dtype)
        self._f("vorticity")(nx, ny, self.ct(h), _p(u), _p(v), _p(out))
        return out

    def confine(self, nx, ny, h, u, v, label, eps, dt):
        u, v, label = self._arr(u).copy(), self._arr(v).copy(), self._lab(label)
        self._f("confine")(nx, ny, self.ct(h), _p(u), _p(v), _p(label), self.ct(eps), self.ct(dt))
        return u, v

    def body_forces(self, nx, ny, h, dnx, dny, dh, u, v, heat, smoke, label, beta, alpha, eps, dt):
        u, v = self._arr(u).copy(), self._arr(v).copy()
        heat, smoke, label = self._arr(heat), self._arr(smoke), self._lab(label)
        self._f("body_forces")(nx, ny, self.ct(h), dnx, dny, self.ct(dh), _p(u), _p(v), _p(heat), _p(smoke), _p(label),
                               self.ct(beta), self.ct(alpha), self.ct(eps), self.ct(dt))
        return u, v

    def stir(self, nx, ny, h, u, v, label, x, y, r, dx, dy):
        u, v, label = self._arr(u).copy(), self._arr(v).copy(), self._lab(label)
        self._f("stir")(nx, ny, self.ct(h), _p(u), _p(v), _p(label), self.ct(x), self.ct(y), self.ct(r), self.ct(dx), self.ct(dy))
        return u, v

    def dye_patch(self, dnx, dny, dye, pi0, pj0, pnx, pny, data):
        dye = self._arr(dye).copy()
        data = np.ascontiguousarray(data, dtype=np.float32)
        self._f("dye_patch")(dnx, dny, _p(dye), pi0, pj0, pnx, pny, _p(data))
        return dye

    # -------------------------------------------------------- whole steps
    def simulation(self, nx, ny, dye_scale=1, **params):
        return OracleSimulation(self, nx, ny, dye_scale, make_params(**params))


class OracleSimulation:
    """simulation.ts's Simulation on the oracle (CPU phase-wise path)."""

    def __init__(self, orc, nx, ny, dye_scale, params):
        self.o = orc
        self.nx, self.ny = nx, ny
        s = max(1, int(dye_scale))
        self.dnx, self.dny = nx * s, ny * s
        self.params = params
        self.h = self.o.ct(1.0 / ny).value
        self.handle = ctypes.c_void_p(orc._f("sim_create")(nx, ny, s, ctypes.byref(params)))

    def __del__(self):
        try:
            if self.handle:
                self.o._f("sim_destroy")(self.handle)
                self.handle = None
        except Exception:
            pass

    def set_fields(self, u, v, p, label, dye):
        a = [self.o._arr(x) for x in (u, v, p)]
        d = self.o._arr(dye)
        lab = self.o._lab(label)
        self.o._f("sim_set_fields")(self.handle, _p(a[0]), _p(a[1]), _p(a[2]), _p(lab), _p(d))

    def get_fields(self):
        nx, ny = self.nx, self.ny
        u = np.zeros((nx + 1) * ny, self.o.dtype)
        v = np.zeros(nx * (ny + 1), self.o.dtype)
        p = np.zeros(nx * ny, self.o.dtype)
        dye = np.zeros(3 * self.dnx * self.dny, self.o.dtype)
        self.o._f("sim_get_fields")(self.handle, _p(u), _p(v), _p(p), _p(dye))
        return u, v, p, dye

    def get_p64(self):
        p = np.zeros(self.nx * self.ny, np.float64)
        self.o._f("sim_get_p64")(self.handle, _p(p))
        return p

    def set_stir(self, st):
        """A one-shot stir (x, y, r, dx, dy) taken by the next step."""
        if st is None:
            self.o._f("sim_set_stir")(self.handle, None)
        else:
            a = np.asarray(st, np.float64)
            self.o._f("sim_set_stir")(self.handle, _p(a))

    def set_patch(self, i0, j0, pnx, pny, data):
        if data is None:
            self.o._f("sim_set_patch")(self.handle, 0, 0, 0, 0, None)
            return
        self._patch = np.ascontiguousarray(data, dtype=np.float32)
        self.o._f("sim_set_patch")(self.handle, i0, j0, pnx, pny, _p(self._patch))

    def step(self):
        return self.o._f("sim_step")(self.handle)

    def get_div(self):
        """The last step's divergence (the pressure solve's input)."""
        d = np.zeros(self.nx * self.ny, self.o.dtype)
        self.o._f("sim_get_div")(self.handle, _p(d))
        return d

    def get_div_post(self):
        """(post-step divergence, index of the step that computed it or -1)."""
        d = np.zeros(self.nx * self.ny, self.o.dtype)
        f = self.o._f("sim_get_div_post")
        f.restype = ctypes.c_longlong
        step = f(self.handle, _p(d))
        return d, int(step)

    def scale(self):
        """The last step's scale rho*h^2/dt."""
        f = self.o._f("sim_scale")
        f.restype = ctypes.c_double
        return f(self.handle)

    def info(self):
        dt, t, rr = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.o._f("sim_info")(self.handle, ctypes.byref(dt), ctypes.byref(t), ctypes.byref(rr))
        return {"dt": dt.value, "time": t.value, "rel_res": rr.value}
