"""ctypes binding of the FP64 CPU oracle (oracle/o3d_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline leg
of the benchmark load this module to check or time against the oracle; the
product library never imports it.

Arrays are numpy float64 in Fortran order with shape (nx, ny, nz), matching
the reference's column-major ``real(8)`` fields.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "o3d_oracle.c")

PERIODIC, EVEN, ODD, ZERO, OPEN = 0, 1, 2, 3, 4
SOR_CONVERGED, SOR_STAGNATED, SOR_MAXIT = 0, 1, 2

_dp = C.POINTER(C.c_double)


def build(force: bool = False) -> None:
    """Compile the oracle twice: serial, and with OpenMP on the stencil passes."""
    import subprocess

    os.makedirs(BUILD, exist_ok=True)
    common = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]
    for name, extra in (("libo3d_oracle.so", []), ("libo3d_oracle_omp.so", ["-fopenmp"])):
        out = os.path.join(BUILD, name)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
                os.path.getmtime(SRC), os.path.getmtime(SRC.replace(".c", ".h"))):
            continue
        subprocess.check_call(common + extra + ["-o", out, SRC, "-lm"])


class orc_model(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("bcx", C.c_int), ("bcy", C.c_int), ("bcz", C.c_int),
        ("sim2d", C.c_int), ("itscheme", C.c_int),
        ("dt", C.c_double), ("re", C.c_double), ("sc", C.c_double),
        ("adt", C.c_double * 3), ("bdt", C.c_double * 3), ("cdt", C.c_double * 3),
        ("iles", C.c_int), ("cs", C.c_double), ("delta", C.c_double),
        ("nscr", C.c_int),
    ]


class orc_step_info(C.Structure):
    _fields_ = [
        ("sor_status", C.c_int), ("sor_iters", C.c_int),
        ("sor_dmax", C.c_double), ("omega", C.c_double),
        ("diverged", C.c_int),
        ("divu_pred_stats", C.c_double * 6), ("divu_stats", C.c_double * 6),
        ("cfl", C.c_double * 3),
    ]


class orc_state(C.Structure):
    _fields_ = [
        ("u", _dp * 3), ("upred", _dp * 3), ("pp", _dp), ("fu", _dp * 9),
        ("nu_t", _dp), ("phi", _dp), ("src", _dp), ("fphi", _dp * 3),
        ("omega", C.c_double), ("eps", C.c_double),
        ("kmax", C.c_int), ("idyn", C.c_int),
    ]


_LIBS: dict = {}


def lib(omp: bool = False):
    name = "libo3d_oracle_omp.so" if omp else "libo3d_oracle.so"
    if name not in _LIBS:
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_rbsor_sweep.restype = C.c_double
        for fn in ("orc_poisson_sor", "orc_poisson_rbsor", "orc_correct_pressure", "orc_correct_velocity"):
            getattr(L, fn).restype = C.c_int
        _LIBS[name] = L
    return _LIBS[name]


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.f_contiguous
    return a.ctypes.data_as(_dp)


def field3(shape) -> np.ndarray:
    return np.zeros(shape, dtype=np.float64, order="F")


def der1(f: np.ndarray, axis: int, closure: int, d: float, omp: bool = False) -> np.ndarray:
    f = np.asfortranarray(f, dtype=np.float64)
    df = field3(f.shape)
    lib(omp).orc_der1(ptr(df), ptr(f), *map(C.c_int, f.shape), C.c_int(axis),
                      C.c_int(closure), C.c_double(d))
    return df


def der2(f: np.ndarray, axis: int, closure: int, d: float, omp: bool = False) -> np.ndarray:
    f = np.asfortranarray(f, dtype=np.float64)
    df = field3(f.shape)
    lib(omp).orc_der2(ptr(df), ptr(f), *map(C.c_int, f.shape), C.c_int(axis),
                      C.c_int(closure), C.c_double(d))
    return df


@dataclass
class Case:
    """One configuration of the reference's namelists (the subset the hot path uses)."""
    nx: int
    ny: int
    nz: int
    xlx: float
    yly: float
    zlz: float
    bcx: int = 0
    bcy: int = 0
    bcz: int = 0
    sim2d: int = 0
    itscheme: int = 3
    dt: float = 1e-3
    re: float = 1600.0
    sc: float = 1.0
    iles: int = 0
    cs: float = 0.17
    nscr: int = 0
    x0: float = 0.0
    y0: float = 0.0
    z0: float = 0.0
    u0: float = 1.0
    l0: float = 1.0
    ratio: float = 1.0
    omega: float = 1.5
    eps: float = 1e-8
    kmax: int = 2000
    idyn: int = 0

    def model(self, omp: bool = False) -> orc_model:
        m = orc_model()
        lib(omp).orc_model_init(
            C.byref(m), C.c_int(self.nx), C.c_int(self.ny), C.c_int(self.nz),
            C.c_double(self.xlx), C.c_double(self.yly), C.c_double(self.zlz),
            C.c_int(self.bcx), C.c_int(self.bcy), C.c_int(self.bcz), C.c_int(self.sim2d),
            C.c_int(self.itscheme), C.c_double(self.dt), C.c_double(self.re),
            C.c_double(self.sc), C.c_int(self.iles), C.c_double(self.cs), C.c_int(self.nscr))
        return m

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz)


@dataclass
class State:
    """Persistent fields of the time loop (module globals in the reference)."""
    case: Case
    u: list = field(default_factory=list)
    upred: list = field(default_factory=list)
    pp: np.ndarray | None = None
    fu: list = field(default_factory=list)
    nu_t: np.ndarray | None = None
    phi: np.ndarray | None = None
    src: np.ndarray | None = None
    fphi: list = field(default_factory=list)

    @classmethod
    def zeros(cls, case: Case) -> "State":
        s = case.shape
        return cls(case=case, u=[field3(s) for _ in range(3)],
                   upred=[field3(s) for _ in range(3)], pp=field3(s),
                   fu=[field3(s) for _ in range(9)], nu_t=field3(s), phi=field3(s),
                   src=field3(s), fphi=[field3(s) for _ in range(3)])

    def c_state(self) -> orc_state:
        st = orc_state()
        for a in range(3):
            st.u[a] = ptr(self.u[a])
            st.upred[a] = ptr(self.upred[a])
            st.fphi[a] = ptr(self.fphi[a])
        for q in range(9):
            st.fu[q] = ptr(self.fu[q])
        st.pp = ptr(self.pp)
        st.nu_t = ptr(self.nu_t)
        st.phi = ptr(self.phi)
        st.src = ptr(self.src)
        st.omega = self.case.omega
        st.eps = self.case.eps
        st.kmax = self.case.kmax
        st.idyn = self.case.idyn
        return st


def init_tgv(case: Case, state: State, omp: bool = False) -> None:
    m = case.model(omp)
    lib(omp).orc_init_tgv(C.byref(m), C.c_double(case.x0), C.c_double(case.y0),
                          C.c_double(case.z0), C.c_double(case.u0), C.c_double(case.l0),
                          C.c_double(case.ratio), C.c_int(case.nscr), ptr(state.u[0]),
                          ptr(state.u[1]), ptr(state.u[2]), ptr(state.pp), ptr(state.phi))


def init_mixing_layer(case: Case, state: State, omp: bool = False) -> None:
    m = case.model(omp)
    lib(omp).orc_init_mixing_layer(
        C.byref(m), C.c_double(case.x0), C.c_double(case.y0), C.c_double(case.z0),
        C.c_double(case.u0), C.c_double(case.l0), C.c_double(case.ratio),
        C.c_int(case.nscr), ptr(state.u[0]), ptr(state.u[1]), ptr(state.u[2]),
        ptr(state.pp), ptr(state.phi))


def init_coplanar_jet(case: Case, state: State, omp: bool = False) -> None:
    """initialize_coplanar_jet (src/initial_conditions.f90:244-327), no noise."""
    m = case.model(omp)
    lib(omp).orc_init_coplanar_jet(
        C.byref(m), C.c_double(case.y0), C.c_double(case.u0), C.c_double(case.l0),
        C.c_double(case.ratio), C.c_int(case.nscr), ptr(state.u[0]), ptr(state.u[1]),
        ptr(state.u[2]), ptr(state.pp), ptr(state.phi))


def statistics(case: Case, state: State, t: float, omp: bool = False) -> np.ndarray:
    m = case.model(omp)
    out = (C.c_double * 17)()
    up = (_dp * 3)(*[ptr(a) for a in state.u])
    lib(omp).orc_statistics(C.byref(m), up, C.c_double(t), out)
    return np.array(out[:])


def rotational(case: Case, u) -> list:
    """curl of u (src/differential_operators.f90:40-77)."""
    m = case.model()
    rot = [field3(case.shape) for _ in range(3)]
    lib().orc_rotational(C.byref(m), (_dp * 3)(*[ptr(a) for a in u]), (_dp * 3)(*[ptr(a) for a in rot]))
    return rot


def q_criterion(case: Case, u) -> np.ndarray:
    """Q-criterion of u (src/differential_operators.f90:79-108)."""
    m = case.model()
    q = field3(case.shape)
    lib().orc_q_criterion(C.byref(m), ptr(q), (_dp * 3)(*[ptr(a) for a in u]))
    return q


def residuals(case: Case, u, old, dt: float, t_ref: float, u_ref: float) -> np.ndarray:
    """calculate_residuals (src/utils.f90:93-163): res_u, res_v, res_w,
    linf_u, linf_v, linf_w, then the 1-based (i, j, k) of each max."""
    m = case.model()
    out = (C.c_double * 15)()
    lib().orc_residuals(C.byref(m), (_dp * 3)(*[ptr(a) for a in u]), (_dp * 3)(*[ptr(a) for a in old]),
                        C.c_double(dt), C.c_double(t_ref), C.c_double(u_ref), out)
    return np.array(out[:])


class Runner:
    """Drives orc_step like the reference's time loop, keeping omega across steps."""

    def __init__(self, case: Case, state: State, omp: bool = False):
        self.case, self.state, self.omp = case, state, omp
        self.m = case.model(omp)
        self.cs = state.c_state()

    def step(self, itime: int) -> orc_step_info:
        info = orc_step_info()
        lib(self.omp).orc_step(C.byref(self.m), C.byref(self.cs), C.c_int(itime), C.byref(info))
        return info

    @property
    def omega(self) -> float:
        return self.cs.omega


def poisson_sor(case: Case, pp: np.ndarray, rhs: np.ndarray, omega: float, eps: float,
                kmax: int, idyn: int = 0):
    m = case.model()
    om = C.c_double(omega)
    it = C.c_int(0)
    dm = C.c_double(0)
    st = lib().orc_poisson_sor(C.byref(m), ptr(pp), ptr(rhs), C.byref(om), C.c_double(eps),
                               C.c_int(kmax), C.c_int(idyn), C.byref(it), C.byref(dm))
    return st, it.value, dm.value, om.value


def poisson_rbsor(case: Case, pp: np.ndarray, rhs: np.ndarray, omega: float, eps: float, kmax: int,
                  idyn: int = 0):
    """The reference's SOR control loop around red-black sweeps; returns
    (status, iters, dmax, omega, omega after each sweep, dmax of each sweep)."""
    m = case.model()
    om = C.c_double(omega)
    it = C.c_int(0)
    dm = C.c_double(0)
    otr = np.zeros(kmax)
    dtr = np.zeros(kmax)
    st = lib().orc_poisson_rbsor(C.byref(m), ptr(pp), ptr(rhs), C.byref(om), C.c_double(eps), C.c_int(kmax),
                                 C.c_int(idyn), C.byref(it), C.byref(dm), otr.ctypes.data_as(_dp),
                                 dtr.ctypes.data_as(_dp))
    return st, it.value, dm.value, om.value, otr[:it.value], dtr[:it.value]


def rbsor_sweep(case: Case, pp: np.ndarray, rhs: np.ndarray, omega: float) -> float:
    m = case.model()
    return lib().orc_rbsor_sweep(C.byref(m), ptr(pp), ptr(rhs), C.c_double(omega))


def divergence(case: Case, fx, fy, fz, odd: int = 1) -> np.ndarray:
    m = case.model()
    out = field3(case.shape)
    lib().orc_divergence(C.byref(m), ptr(out), ptr(fx), ptr(fy), ptr(fz), C.c_int(odd))
    return out


def nu_t(case: Case, ux, uy, uz) -> np.ndarray:
    m = case.model()
    out = field3(case.shape)
    lib().orc_nu_t(C.byref(m), ptr(out), ptr(ux), ptr(uy), ptr(uz))
    return out


def predict_velocity(case: Case, state: State, itime: int) -> None:
    """orc_predict_velocity on the state's fields (u -> upred, fu shifted)."""
    m = case.model()
    up = (_dp * 3)(*[ptr(a) for a in state.upred])
    u = (_dp * 3)(*[ptr(a) for a in state.u])
    fu = (_dp * 9)(*[ptr(a) for a in state.fu])
    lib().orc_predict_velocity(C.byref(m), up, u, fu, ptr(state.nu_t), C.c_int(itime))


def statistics_of(case: Case, u, t: float = 0.0) -> np.ndarray:
    m = case.model()
    out = (C.c_double * 17)()
    up = (_dp * 3)(*[ptr(np.asfortranarray(a)) for a in u])
    lib().orc_statistics(C.byref(m), up, C.c_double(t), out)
    return np.array(out[:])
