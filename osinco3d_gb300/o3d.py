"""ctypes binding of libo3d.so (include/o3d.h).

The class :class:`Context` mirrors the Fortran interface of the osinco3d hot
path: ``predict_velocity`` (src/integration.f90:14), ``correct_pression``
(:199), ``correct_velocity`` (:257), ``transeq`` (:332), the ``der_type``
derivative operators (src/initialization.f90:86-91), ``poi_type`` Poisson
solvers (:93-102) and ``statistics_calc`` (src/utils.f90:243).  Fields are
numpy float64 arrays in Fortran order with shape (nx, ny, nz).

There is no CPU fallback: every call runs the CUDA kernels of libo3d.so, and
loading fails with an error if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import re

import numpy as np

from . import build as _build

OK = 0
WARN_POISSON_MAXIT = 1
WARN_STAGNATION = 2
ERR_BADARG = -1
ERR_CUDA = -2
ERR_NONFINITE = -3
ERR_NOMEM = -4
ERR_NOT_BUILT = -5

PREC_FP64, PREC_MIXED = 0, 1
SOLVER_SOR, SOLVER_MG = 0, 1
GUESS_PREVIOUS, GUESS_ZERO, GUESS_LEARNED, GUESS_EXTRAPOLATED, GUESS_EXTRAPOLATED2 = 0, 1, 2, 3, 4

FIELD = {"ux": 0, "uy": 1, "uz": 2, "pp": 3, "ux_pred": 4, "uy_pred": 5, "uz_pred": 6,
         "phi": 7, "src": 8, "nu_t": 9, "rhs": 10}
FIELD_FU0, FIELD_FPHI0 = 16, 24

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "o3d.h")


class O3DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libo3d error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("xlx", C.c_double), ("yly", C.c_double), ("zlz", C.c_double),
        ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
        ("nbcx1", C.c_int), ("nbcxn", C.c_int), ("nbcy1", C.c_int), ("nbcyn", C.c_int),
        ("nbcz1", C.c_int), ("nbczn", C.c_int), ("sim2d", C.c_int),
        ("itscheme", C.c_int), ("dt", C.c_double),
        ("re", C.c_double),
        ("omega", C.c_double), ("eps", C.c_double), ("kmax", C.c_int), ("idyn", C.c_int),
        ("nscr", C.c_int), ("sc", C.c_double),
        ("iles", C.c_int), ("cs", C.c_double),
        ("precision", C.c_int), ("solver", C.c_int), ("mg_levels", C.c_int),
        ("mg_pre", C.c_int), ("mg_post", C.c_int), ("guess", C.c_int), ("diagnostics", C.c_int),
        ("mg_cycles", C.c_int), ("mg_omega", C.c_double), ("mg_kernels", C.c_int),
    ]


class StepInfo(C.Structure):
    _fields_ = [
        ("poisson_status", C.c_int), ("poisson_iters", C.c_int), ("poisson_cycles", C.c_int),
        ("poisson_dmax", C.c_double), ("poisson_res_inf", C.c_double), ("omega", C.c_double),
        ("diverged", C.c_int),
        ("divu_pred_stats", C.c_double * 6), ("divu_stats", C.c_double * 6),
        ("cfl", C.c_double * 3), ("umin", C.c_double * 3), ("umax", C.c_double * 3),
        ("poisson_ms", C.c_double), ("step_ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


_dp = C.POINTER(C.c_double)
_LIB = None


def library_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Loads libo3d.so, building it first if it is missing or stale."""
    global _LIB
    if _LIB is None:
        if build_if_missing:
            _build.build()
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"libo3d.so is not built ({path}); run osinco3d_gb300.build.build()")
        L = C.CDLL(path)
        vp = C.c_void_p
        sig = {
            "o3d_default_params": (None, [C.POINTER(Params)]),
            "o3d_create": (C.c_int, [C.POINTER(Params), C.POINTER(vp)]),
            "o3d_destroy": (C.c_int, [vp]),
            "o3d_last_error": (C.c_char_p, []),
            "o3d_launch_count": (C.c_longlong, [vp]),
            "o3d_stream": (vp, [vp]),
            "o3d_upload": (C.c_int, [vp, C.c_int, _dp]),
            "o3d_download": (C.c_int, [vp, C.c_int, _dp]),
            "o3d_der": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, _dp, _dp]),
            "o3d_der_dev": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp, vp]),
            "o3d_divergence": (C.c_int, [vp, _dp, _dp, _dp, C.c_int, _dp]),
            "o3d_calculate_nu_t": (C.c_int, [vp]),
            "o3d_predict_velocity": (C.c_int, [vp, C.c_int]),
            "o3d_correct_pression": (C.c_int, [vp, _dp, C.POINTER(StepInfo)]),
            "o3d_correct_velocity": (C.c_int, [vp]),
            "o3d_transeq": (C.c_int, [vp, C.c_int]),
            "o3d_poisson_solve": (C.c_int, [vp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                            C.POINTER(C.c_int), _dp]),
            "o3d_step": (C.c_int, [vp, C.c_int, C.POINTER(StepInfo)]),
            "o3d_step_host": (C.c_int, [vp, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(StepInfo)]),
            "o3d_statistics_calc": (C.c_int, [vp, C.c_double, _dp]),
            "o3d_vorticity": (C.c_int, [vp, _dp, _dp, _dp, _dp]),
            "o3d_write_output": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_double]),
            "o3d_output_wait": (C.c_int, [vp]),
            "o3d_save_fields": (C.c_int, [vp, C.c_char_p, C.c_double]),
            "o3d_load_fields": (C.c_int, [vp, C.c_char_p, _dp]),
            "o3d_save_history": (C.c_int, [vp, C.c_char_p]),
            "o3d_load_history": (C.c_int, [vp, C.c_char_p]),
            "o3d_save_old_velocity": (C.c_int, [vp]),
            "o3d_velocity_residuals": (C.c_int, [vp, C.c_double, C.c_double, _dp]),
            "o3d_rbsor_sweeps_dev": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, _dp]),
            "o3d_time_kernel": (C.c_int, [vp, C.c_int, C.c_int, _dp]),
            "o3d_check_conversions": (C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]),
            "o3d_unet_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_int,
                                          C.c_int, C.c_ulonglong, C.POINTER(vp)]),
            "o3d_unet_destroy": (C.c_int, [vp]),
            "o3d_unet_num_params": (C.c_longlong, [vp]),
            "o3d_unet_get_params": (C.c_int, [vp, C.POINTER(C.c_float)]),
            "o3d_unet_set_params": (C.c_int, [vp, C.POINTER(C.c_float)]),
            "o3d_unet_forward_dev": (C.c_int, [vp, vp, vp, vp]),
            "o3d_unet_gradients": (C.c_int, [vp, vp, vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "o3d_unet_train_step": (C.c_int, [vp, vp, vp, C.c_float, C.POINTER(C.c_float)]),
            "o3d_guess_grid": (C.c_int, [vp, C.POINTER(C.c_int)]),
            "o3d_attach_unet": (C.c_int, [vp, vp]),
            "o3d_set_sample_buffers": (C.c_int, [vp, vp, vp]),
            "o3d_sample_ready": (C.c_int, [vp]),
            "o3d_divergence_stats_noalloc": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                                       C.c_double, C.c_double, C.c_double, C.c_int,
                                                       C.c_int, C.c_int, C.c_int, vp, _dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def declared_symbols() -> list[str]:
    """Every o3d_* function declared in include/o3d.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"O3D_API\s+[\w\s\*]+?\b(o3d_\w+)\s*\(", txt)))


def default_params(**kw) -> Params:
    p = Params()
    lib().o3d_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def tgv_params(n: int, **kw) -> Params:
    """Periodic Taylor-Green box [0, 2 pi)^3 on n^3 nodes: xlx = 2 pi (n-1)/n so
    that the node-inclusive spacing xlx/(n-1) equals the period 2 pi / n."""
    L = 2.0 * math.pi * (n - 1) / n
    base = dict(nx=n, ny=n, nz=n, xlx=L, yly=L, zlz=L, dt=0.2 * 2.0 * math.pi / n,
                omega=2.0 / (1.0 + math.sin(math.pi * 2.0 * math.pi / n)))
    base.update(kw)
    return default_params(**base)


def mixing_layer_params(nx: int = 512, ny: int = 256, nz: int = 256, lx: float = 60.0, ly: float = 30.0,
                        lz: float = 30.0, cfl: float = 0.2, ratio: float = 0.5, **kw) -> Params:
    """Temporal mixing layer: x and z periodic (xlx = lx (nx-1)/nx, zlz likewise),
    y free-slip on [-ly/2, ly/2] node-inclusive, Re 3000, Smagorinsky c_s 0.17,
    passive scalar Sc 1, AB3; dt from the CFL number on the faster stream
    u2 = u0 / (1 - ratio)."""
    u2 = 1.0 / (1.0 - ratio) if abs(ratio) > 1e-12 else 1.0
    xl, zl = lx * (nx - 1) / nx, lz * (nz - 1) / nz
    base = dict(nx=nx, ny=ny, nz=nz, xlx=xl, yly=ly, zlz=zl, x0=0.0, y0=-0.5 * ly, z0=0.0,
                nbcx1=0, nbcxn=0, nbcy1=1, nbcyn=1, nbcz1=0, nbczn=0, re=3000.0, iles=1, cs=0.17,
                nscr=1, sc=1.0, itscheme=3, dt=cfl * (xl / (nx - 1)) / u2)
    base.update(kw)
    return default_params(**base)


def mixing_layer_fields(params: Params, ratio: float = 0.5, u0: float = 1.0, l0: float = 1.0,
                        noise: float = 0.05, seed: int = 1234):
    """Initial state of the mixing layer of src/initial_conditions.f90:329-394:
    u = (u2 + u1)/2 - (u1 - u2)/2 tanh(y ln2 / (2 theta)), u2 = u0/(1 - ratio),
    u1 = ratio u2, theta = 1/(13 l0); v = w = 0; p = 1; phi = 1/2 - 1/2 tanh(.).
    The reference's clock-seeded noise is replaced by seeded uniform noise
    U(-1, 1) * noise * u0 on the three velocity components."""
    nx, ny, nz = params.nx, params.ny, params.nz
    dy = params.yly / (ny - 1)
    u2 = u0 / (1.0 - ratio) if abs(ratio) > 1e-12 else u0
    u1 = u2 * ratio if abs(ratio) > 1e-12 else 0.0
    theta = 1.0 / (13.0 * l0)
    y = params.y0 + np.arange(ny) * dy
    t3 = y * math.log(2.0) / (2.0 * theta)
    prof = 0.5 * (u2 + u1) - 0.5 * (u1 - u2) * np.tanh(t3)
    shape = (nx, ny, nz)
    ux = np.asfortranarray(np.broadcast_to(prof[None, :, None], shape).copy())
    uy = np.zeros(shape, order="F")
    uz = np.zeros(shape, order="F")
    rng = np.random.default_rng(seed)
    for f in (ux, uy, uz):
        f += noise * u0 * rng.uniform(-1.0, 1.0, shape)
    pp = np.ones(shape, order="F")
    phi = np.asfortranarray(np.broadcast_to((0.5 - 0.5 * np.tanh(t3))[None, :, None], shape).copy())
    return ux, uy, uz, pp, phi


def coplanar_jet_params(nx: int = 768, ny: int = 384, nz: int = 384, lx: float = 20.0, ly: float = 10.0,
                        lz: float = 10.0, cfl: float = 0.25, ratio: float = 0.5, **kw) -> Params:
    """Co-planar jet: x open (inflow at x = 0, outflow at x = lx), y and z
    free-slip on [-ly/2, ly/2] and [-lz/2, lz/2] node-inclusive, Re 2200,
    Smagorinsky c_s 0.17, passive scalar Sc 0.7, AB3; dt from the CFL number
    on the inner jet's velocity u0 / ratio.  The domain lengths are this
    library's choice (the reference gives none for this case)."""
    u1 = 1.0 / ratio
    base = dict(nx=nx, ny=ny, nz=nz, xlx=lx, yly=ly, zlz=lz, x0=0.0, y0=-0.5 * ly, z0=-0.5 * lz,
                nbcx1=2, nbcxn=2, nbcy1=1, nbcyn=1, nbcz1=1, nbczn=1, re=2200.0, iles=1, cs=0.17,
                nscr=1, sc=0.7, itscheme=3, dt=cfl * (lx / (nx - 1)) / u1)
    base.update(kw)
    return default_params(**base)


def coplanar_jet_fields(params: Params, ratio: float = 0.5, u0: float = 1.0, l0: float = 1.0,
                        noise: float = 0.05, seed: int = 1234):
    """Initial state of the co-planar jet of src/initial_conditions.f90:244-327:
    an inner jet u1 = u0 / ratio for |y| < (h1 + h2) / 2 and a co-flow u0
    beyond, tanh layers at h1 = l0/2 (thickness h1/10) and h2 = l0 (h2/25),
    v = w = p = 0, phi 0 in the inner jet, 1 in the co-flow, 0 beyond.  Seeded
    uniform noise U(-1, 1) * noise * u0, scaled by the inner layer's shear
    profile, is added to the three velocity components (the reference's
    noise is clock-seeded); the inflow plane x = 0 keeps the noisy values it
    starts with."""
    nx, ny, nz = params.nx, params.ny, params.nz
    dy = params.yly / (ny - 1)
    u2 = u0
    u1 = u2 / ratio
    u3 = 0.0 * u2
    d1 = l0
    d2 = 2.0 * d1
    h1, h2 = 0.5 * d1, 0.5 * d2
    th1, th2 = h1 / 10.0, h2 / 25.0
    hm = 0.5 * (h1 + h2)
    ay = np.abs(params.y0 + np.arange(ny) * dy)
    inner = ay < hm
    prof = np.where(inner, 0.5 * (u1 + u2) + 0.5 * (u2 - u1) * np.tanh((ay - h1) / (2.0 * th1)),
                    0.5 * (u2 + u3) + 0.5 * (u3 - u2) * np.tanh((ay - h2) / (2.0 * th2)))
    ph = np.where(inner, 0.5 + 0.5 * np.tanh((ay - h1) / (2.0 * th1)),
                  0.5 - 0.5 * np.tanh((ay - h2) / (2.0 * th2)))
    shape = (nx, ny, nz)
    ux = np.asfortranarray(np.broadcast_to(prof[None, :, None], shape).copy())
    uy = np.zeros(shape, order="F")
    uz = np.zeros(shape, order="F")
    env = (1.0 / np.cosh((ay - h1) / (2.0 * th1)) ** 2)[None, :, None]
    rng = np.random.default_rng(seed)
    for f in (ux, uy, uz):
        f += noise * u0 * env * rng.uniform(-1.0, 1.0, shape)
    pp = np.zeros(shape, order="F")
    phi = np.asfortranarray(np.broadcast_to(ph[None, :, None], shape).copy())
    return ux, uy, uz, pp, phi


def _ptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.f_contiguous:
        raise TypeError("fields must be float64 Fortran-ordered arrays")
    return a.ctypes.data_as(_dp)


class Context:
    """One solver context (grid, device fields, stream)."""

    def __init__(self, params: Params):
        self.L = lib()
        self.params = params
        self.shape = (params.nx, params.ny, params.nz)
        h = C.c_void_p()
        self._check(self.L.o3d_create(C.byref(params), C.byref(h)))
        self.h = h
        self.omega = params.omega

    def _check(self, code: int) -> int:
        if code < 0:
            raise O3DError(code, self.L.o3d_last_error().decode())
        return code

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.o3d_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- fields -------------------------------------------------------------
    def field(self) -> np.ndarray:
        return np.zeros(self.shape, dtype=np.float64, order="F")

    def upload(self, name, arr: np.ndarray) -> None:
        fid = FIELD[name] if isinstance(name, str) else name
        self._check(self.L.o3d_upload(self.h, fid, _ptr(np.asfortranarray(arr, dtype=np.float64))))

    def download(self, name) -> np.ndarray:
        fid = FIELD[name] if isinstance(name, str) else name
        out = self.field()
        self._check(self.L.o3d_download(self.h, fid, _ptr(out)))
        return out

    def flux(self, comp: int, age: int) -> np.ndarray:
        return self.download(FIELD_FU0 + 2 * comp + age)

    @property
    def launches(self) -> int:
        return int(self.L.o3d_launch_count(self.h))

    # -- operators ----------------------------------------------------------
    def der(self, f: np.ndarray, axis: int, order: int, odd: bool) -> np.ndarray:
        f = np.asfortranarray(f, dtype=np.float64)
        out = self.field()
        self._check(self.L.o3d_der(self.h, axis, order, int(odd), _ptr(f), _ptr(out)))
        return out

    def divergence(self, fx, fy, fz, odd: int = 1) -> np.ndarray:
        out = self.field()
        fx, fy, fz = (np.asfortranarray(a, dtype=np.float64) for a in (fx, fy, fz))
        self._check(self.L.o3d_divergence(self.h, _ptr(fx), _ptr(fy), _ptr(fz), odd, _ptr(out)))
        return out

    def calculate_nu_t(self) -> np.ndarray:
        self._check(self.L.o3d_calculate_nu_t(self.h))
        return self.download("nu_t")

    def predict_velocity(self, itime: int) -> None:
        self._check(self.L.o3d_predict_velocity(self.h, itime))

    def correct_pression(self) -> StepInfo:
        info = StepInfo()
        om = C.c_double(self.omega)
        self._check(self.L.o3d_correct_pression(self.h, C.byref(om), C.byref(info)))
        self.omega = om.value
        return info

    def correct_velocity(self) -> int:
        return self._check(self.L.o3d_correct_velocity(self.h))

    def transeq(self, itime: int) -> None:
        self._check(self.L.o3d_transeq(self.h, itime))

    def poisson_solve(self, pp: np.ndarray, rhs: np.ndarray, omega: float, eps: float, kmax: int,
                      idyn: int = 0):
        """poi_type(pp, rhs, ..., omega, eps, kmax, idyn): pp is updated in place."""
        om = C.c_double(omega)
        it = C.c_int(0)
        dm = C.c_double(0.0)
        rhs = np.asfortranarray(rhs, dtype=np.float64)
        st = self._check(self.L.o3d_poisson_solve(self.h, _ptr(pp), _ptr(rhs), C.byref(om), eps, kmax,
                                                  idyn, C.byref(it), C.byref(dm)))
        return st, it.value, dm.value, om.value

    def step(self, itime: int) -> StepInfo:
        info = StepInfo()
        self.last_status = self._check(self.L.o3d_step(self.h, itime, C.byref(info)))
        return info

    def step_host(self, itime: int, ux, uy, uz, pp) -> StepInfo:
        info = StepInfo()
        self.last_status = self._check(
            self.L.o3d_step_host(self.h, itime, _ptr(ux), _ptr(uy), _ptr(uz), _ptr(pp), C.byref(info)))
        return info

    def statistics_calc(self, t: float) -> np.ndarray:
        out = (C.c_double * 17)()
        self._check(self.L.o3d_statistics_calc(self.h, t, out))
        return np.array(out[:])

    def write_output(self, directory: str, num: int, time: float) -> None:
        """write_all_data + write_xdmf: the raw FP64 fields and the XDMF file
        of output `num`, written asynchronously (see output_wait)."""
        self._check(self.L.o3d_write_output(self.h, os.fsencode(directory), num, time))

    def output_wait(self) -> None:
        self._check(self.L.o3d_output_wait(self.h))

    # -- checkpoint and restart ------------------------------------------------
    def save_fields(self, path: str, time: float) -> None:
        """The reference's fields_%06d.bin flow-state file (save_fields)."""
        self._check(self.L.o3d_save_fields(self.h, os.fsencode(path), time))

    def load_fields(self, path: str) -> float:
        t = C.c_double(0.0)
        self._check(self.L.o3d_load_fields(self.h, os.fsencode(path), C.byref(t)))
        return t.value

    def save_history(self, path: str) -> None:
        self._check(self.L.o3d_save_history(self.h, os.fsencode(path)))

    def load_history(self, path: str) -> None:
        self._check(self.L.o3d_load_history(self.h, os.fsencode(path)))

    # -- output-cadence diagnostics ----------------------------------------------
    def vorticity(self):
        """(rotx, roty, rotz, Q-criterion) of the current velocity."""
        out = [self.field() for _ in range(4)]
        self._check(self.L.o3d_vorticity(self.h, *[a.ctypes.data_as(_dp) for a in out]))
        return out

    def save_old_velocity(self) -> None:
        self._check(self.L.o3d_save_old_velocity(self.h))

    def velocity_residuals(self, t_ref: float = 1.0, u_ref: float = 1.0) -> np.ndarray:
        """res_u, res_v, res_w, linf_u, linf_v, linf_w and the 1-based (i, j, k)
        of each max (calculate_residuals, src/utils.f90:93-163)."""
        out = (C.c_double * 15)()
        self._check(self.L.o3d_velocity_residuals(self.h, t_ref, u_ref, out))
        return np.array(out[:])

    # -- learned warm start ----------------------------------------------------
    def guess_grid(self):
        dims = (C.c_int * 3)()
        self._check(self.L.o3d_guess_grid(self.h, dims))
        return tuple(dims)

    def attach_unet(self, net: "UNet | None") -> None:
        self._check(self.L.o3d_attach_unet(self.h, net.h if net else None))
        self._net = net  # keep the network alive while attached

    def set_sample_buffers(self, d_feat: int | None, d_tgt: int | None) -> None:
        self._check(self.L.o3d_set_sample_buffers(self.h, C.c_void_p(d_feat or 0), C.c_void_p(d_tgt or 0)))

    def sample_ready(self) -> bool:
        return bool(self.L.o3d_sample_ready(self.h))

    KERNELS = {"predict": 0, "rhs": 1, "correct": 2, "mg_smooth": 3, "resid64": 4, "mg_down": 5, "mg_up": 6,
               "mg_pre": 7, "mg_resid": 8, "mg_prolong": 9, "mg_red": 10, "mg_post": 11}

    def time_kernel(self, name: str, reps: int = 20) -> float:
        """Milliseconds per launch of one hot kernel on the live state."""
        ms = C.c_double(0.0)
        self._check(self.L.o3d_time_kernel(self.h, self.KERNELS[name], reps, C.byref(ms)))
        return ms.value

    def rbsor_sweeps_dev(self, d_pp: int, d_rhs: int, omega: float, nsweeps: int) -> float:
        dm = C.c_double(0.0)
        self._check(self.L.o3d_rbsor_sweeps_dev(self.h, C.c_void_p(d_pp), C.c_void_p(d_rhs), omega,
                                                nsweeps, C.byref(dm)))
        return dm.value


class UNet:
    """The 3D U-Net of the learned warm start (o3d_unet_*): BF16 tensor-core
    convolutions, trained by the library's own forward/backward kernels."""

    def __init__(self, dims, periodic=(1, 1, 1), base=16, levels=4, in_channels=2, seed=1234):
        self.L = lib()
        h = C.c_void_p()
        per = (C.c_int * 3)(*periodic)
        st = self.L.o3d_unet_create(dims[0], dims[1], dims[2], per, base, levels, in_channels, seed, C.byref(h))
        if st < 0:
            raise O3DError(st, self.L.o3d_last_error().decode())
        self.h = h
        self.dims, self.base, self.levels, self.in_channels = tuple(dims), base, levels, in_channels
        self.periodic = tuple(periodic)

    def _check(self, code: int) -> int:
        if code < 0:
            raise O3DError(code, self.L.o3d_last_error().decode())
        return code

    @property
    def nparams(self) -> int:
        return int(self.L.o3d_unet_num_params(self.h))

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.nparams, dtype=np.float32)
        self._check(self.L.o3d_unet_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.L.o3d_unet_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def forward(self, d_in: int, d_out: int, stream: int | None = None) -> None:
        self._check(self.L.o3d_unet_forward_dev(self.h, C.c_void_p(d_in), C.c_void_p(d_out), C.c_void_p(stream or 0)))

    def gradients(self, d_in: int, d_tgt: int):
        loss = C.c_float(0)
        g = np.zeros(self.nparams, dtype=np.float32)
        self._check(self.L.o3d_unet_gradients(self.h, C.c_void_p(d_in), C.c_void_p(d_tgt), C.byref(loss),
                                              g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    def train_step(self, d_in: int, d_tgt: int, lr: float) -> float:
        loss = C.c_float(0)
        self._check(self.L.o3d_unet_train_step(self.h, C.c_void_p(d_in), C.c_void_p(d_tgt), lr, C.byref(loss)))
        return loss.value

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.o3d_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def check_conversions(n: int = 1 << 24, seed: int = 1) -> int:
    """Mismatches of the integer-pipe FP64 <-> FP32 conversions against the
    conversion instructions over n seeded bit patterns (0 expected)."""
    L = lib()
    bad = C.c_longlong(-1)
    st = L.o3d_check_conversions(n, seed, C.byref(bad))
    if st < 0:
        raise O3DError(st, L.o3d_last_error().decode())
    return bad.value


# block records held by the scratch of o3d_divergence_stats_noalloc
# (O3D_NOALLOC_MAX_RECORDS in include/o3d.h); a grid needs
# noalloc_records(shape) of them
NOALLOC_MAX_RECORDS = 24576


def noalloc_records(shape) -> int:
    """Block records o3d_divergence_stats_noalloc needs for a grid: one per
    32 x 8 column of 28 planes."""
    nx, ny, nz = shape
    return -(-nx // 32) * -(-ny // 8) * -(-nz // 28)


def divergence_stats_noalloc(d_fx: int, d_fy: int, d_fz: int, d_div: int | None, shape, spacing, bcs,
                             odd: int = 1, stream: int | None = None):
    """o3d_divergence_stats_noalloc on the caller's device buffers (raw device
    addresses); returns (status, stats[6]).  It allocates nothing."""
    L = lib()
    out = (C.c_double * 6)()
    st = L.o3d_divergence_stats_noalloc(
        C.c_void_p(d_fx), C.c_void_p(d_fy), C.c_void_p(d_fz), C.c_void_p(d_div or 0),
        shape[0], shape[1], shape[2], spacing[0], spacing[1], spacing[2], bcs[0], bcs[1], bcs[2], odd,
        C.c_void_p(stream or 0), out)
    if st < 0:
        raise O3DError(st, L.o3d_last_error().decode())
    return st, np.array(out[:])


def tgv_fields(params: Params):
    """Taylor-Green initial state of initialize_taylor_green_vortex
    (src/initial_conditions.f90:139-151) on the context grid, u0 = l0 = ratio = 1."""
    nx, ny, nz = params.nx, params.ny, params.nz
    dx, dy, dz = params.xlx / (nx - 1), params.yly / (ny - 1), params.zlz / (nz - 1)
    x = params.x0 + np.arange(nx) * dx
    y = params.y0 + np.arange(ny) * dy
    z = params.z0 + np.arange(nz) * dz
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    ux = np.asfortranarray(np.sin(X) * np.cos(Y) * np.cos(Z))
    uy = np.asfortranarray(-np.cos(X) * np.sin(Y) * np.cos(Z))
    uz = np.zeros_like(ux, order="F")
    pp = np.asfortranarray(0.0625 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0))
    return ux, uy, uz, pp
