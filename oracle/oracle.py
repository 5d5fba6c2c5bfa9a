"""ctypes front end of the CPU FP64 oracle (``libflutas_oracle.so``).

TEST INFRASTRUCTURE ONLY.  The CUDA product path never imports this module;
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, to check the CUDA path against.

Parity status: "parity unpinned" against a run of the reference itself.  The
reference's ``solver_cpu`` (src/solver_cpu.f90) needs gfortran and FFTW 3.3.10,
neither of which exists on these machines, and the reference's tests hold no
golden vectors for this path.  The restatement is pinned instead by closed-form
discrete-eigenfunction known answers (tests/golden/) and by an independent
scipy.fft restatement (oracle/restate_scipy.py).

Array convention: every 3-D field is a C-contiguous numpy array of shape
``(nz+2h, ny+2h, nx+2h)``, i.e. the Fortran array ``(1-h:nx+h, 1-h:ny+h,
1-h:nz+h)`` in its own memory order (x fastest).  Pressure-like fields have
h = 1; velocities h = nh_u.  1-D z arrays are ``(1-nh_d:nz+nh_d)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libflutas_oracle.so")
_lib = None

R2HC, HC2R, REDFT00, REDFT01, REDFT10, REDFT11, RODFT00, RODFT01, RODFT10, RODFT11 = (
    0, 1, 3, 4, 5, 6, 7, 8, 9, 10)

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class OrPlan(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("kind_fwd", C.c_int * 2), ("kind_bwd", C.c_int * 2),
                ("ix", C.c_int), ("iy", C.c_int)]


def build():
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.or_r2r.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.or_eigenvalues.argtypes = [C.c_int, C.c_char, C.c_char, C.c_char, _dp]
        L.or_tridmatrix.argtypes = [C.c_char, C.c_char, C.c_int, C.c_int, _dp, _dp, C.c_char,
                                    _dp, _dp, _dp]
        L.or_initsolver.argtypes = [C.c_int * 3, C.c_double * 3, C.c_int, _dp, _dp, C.c_char_p,
                                    C.c_double * 6, C.c_char_p, _dp, _dp, _dp, _dp,
                                    C.POINTER(OrPlan), C.POINTER(C.c_double), _dp, _dp, _dp]
        L.or_solver.argtypes = [C.POINTER(OrPlan), C.c_double, _dp, _dp, _dp, _dp, C.c_char_p,
                                C.c_char_p, _dp]
        L.or_fillps.argtypes = [C.c_int] * 5 + [C.c_double] * 3 + [_dp, C.c_double, C.c_double,
                                                                      _dp, _dp, _dp, _dp]
        L.or_correc.argtypes = [C.c_int] * 5 + [C.c_double] * 3 + [_dp, C.c_double, C.c_double,
                                                                      _dp, _dp, _dp, _dp]
        L.or_boundp.argtypes = [C.c_char_p, C.c_int * 3, C.c_double * 6, C.c_int, C.c_double * 3,
                                _dp, _dp, _dp]
        L.or_bounduvw.argtypes = [C.c_char_p, C.c_int * 3, C.c_double * 18, C.c_int, C.c_int,
                                  C.c_double * 3, _dp, _dp, _dp, _dp, _dp, C.c_void_p]
        L.or_updt_rhs_b.argtypes = [C.c_int] * 3 + [C.c_char_p, C.c_char_p, _dp, _dp, _dp, _dp]
        L.or_chkdiv.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int] * 2 + [
            _dp, _dp, _dp, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_pres_tw_src.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int] * 2 + [
            _dp, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp]
        L.or_initgrid.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                  _dp, _dp]
        L.or_update_property.argtypes = [C.c_int] * 3 + [C.c_double] * 2 + [_dp, _dp]
        L.or_residual.argtypes = [C.c_int * 3, C.c_char_p, C.c_double, C.c_double, C.c_int, _dp,
                                  _dp, _dp, _dp, _dp]
        L.or_momad.argtypes = [C.c_int] * 4 + [C.c_double] * 3 + [C.c_int] * 2 + [_dp] * 7 + [C.c_double] + [_dp] * 3
        L.or_rk.argtypes = [C.c_int, C.c_double, C.c_double] + [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int] * 2 + \
            [_dp] * 7 + [C.c_double] + [_dp] * 3
        L.or_cmpt_time_factors.argtypes = [C.c_char_p, C.c_int, C.c_int, _dp, C.c_double, C.c_double, _dp]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        _lib = L
    return _lib


def set_threads(n: int):
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return lib().or_get_threads()


def _b(s):
    return s.encode() if isinstance(s, str) else s


def r2r(kind: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    if lib().or_r2r(kind, x.size, x, y) != 0:
        raise ValueError("bad r2r kind/size")
    return y


def eigenvalues(n, bc, c_or_f="c"):
    lam = np.empty(n)
    if lib().or_eigenvalues(n, _b(bc[0]), _b(bc[1]), _b(c_or_f), lam) != 0:
        raise ValueError(f"bad bc {bc}")
    return lam


def tridmatrix(bc, n, nh_d, dzci, dzfi, c_or_f="c"):
    a, b, c = np.empty(n), np.empty(n), np.empty(n)
    lib().or_tridmatrix(_b(bc[0]), _b(bc[1]), n, nh_d, np.ascontiguousarray(dzci),
                        np.ascontiguousarray(dzfi), _b(c_or_f), a, b, c)
    return a, b, c


class SolverSetup:
    """Everything initsolver (src/initsolver.f90:21-120) returns."""

    def __init__(self, n, dli, nh_d, dzci, dzfi, cbc, bc, c_or_f="ccc"):
        n = [int(x) for x in n]
        self.n = n
        self.lambdaxy = np.empty((n[1], n[0]))
        self.a, self.b, self.c = np.empty(n[2]), np.empty(n[2]), np.empty(n[2])
        self.rhsbx = np.empty((2, n[2], n[1]))
        self.rhsby = np.empty((2, n[2], n[0]))
        self.rhsbz = np.empty((2, n[1], n[0]))
        self.plan = OrPlan()
        nf = C.c_double()
        cbc = "".join(cbc) if not isinstance(cbc, str) else cbc
        self.cbc = cbc
        self.c_or_f = c_or_f
        rc = lib().or_initsolver((C.c_int * 3)(*n), (C.c_double * 3)(*dli), nh_d,
                                 np.ascontiguousarray(dzci, dtype=np.float64),
                                 np.ascontiguousarray(dzfi, dtype=np.float64), _b(cbc),
                                 (C.c_double * 6)(*bc), _b(c_or_f), self.lambdaxy, self.a, self.b,
                                 self.c, C.byref(self.plan), C.byref(nf), self.rhsbx, self.rhsby,
                                 self.rhsbz)
        if rc != 0:
            raise ValueError("initsolver: bad arguments")
        self.normfft = nf.value

    def solve(self, p: np.ndarray) -> np.ndarray:
        """solver_cpu on a halo-1 array, in place (interior overwritten)."""
        assert p.flags.c_contiguous and p.dtype == np.float64
        rc = lib().or_solver(C.byref(self.plan), self.normfft, self.lambdaxy, self.a, self.b, self.c,
                             _b(self.cbc[4:6]), _b(self.c_or_f), p)
        if rc != 0:
            raise RuntimeError("or_solver failed")
        return p


def fillps(n, nh_d, nh_u, dxi, dyi, dzi, dzfi, dti, rho0, u, v, w, p):
    lib().or_fillps(n[0], n[1], n[2], nh_d, nh_u, dxi, dyi, dzi, dzfi, dti, rho0, u, v, w, p)


def correc(n, nh_d, nh_u, dxi, dyi, dzi, dzci, dt, rho0, p, u, v, w):
    lib().or_correc(n[0], n[1], n[2], nh_d, nh_u, dxi, dyi, dzi, dzci, dt, rho0, p, u, v, w)


def boundp(cbc, n, bc, nh_d, dl, dzc, dzf, p):
    lib().or_boundp(_b(cbc), (C.c_int * 3)(*n), (C.c_double * 6)(*bc), nh_d,
                    (C.c_double * 3)(*dl), dzc, dzf, p)


def bounduvw(cbcvel, n, bcvel, nh_d, nh_u, dl, dzc, dzf, u, v, w, isoutflow=None):
    """cbcvel: 18 characters in Fortran (0:1,1:3,1:3) memory order; isoutflow: 6 flags (0:1,1:3)."""
    outf = (C.c_int * 6)(*[int(bool(x)) for x in isoutflow]) if isoutflow is not None else None
    lib().or_bounduvw(_b(cbcvel), (C.c_int * 3)(*n), (C.c_double * 18)(*bcvel), nh_d, nh_u,
                      (C.c_double * 3)(*dl), dzc, dzf, u, v, w, outf)


def updt_rhs_b(n, c_or_f, cbc, rhsbx, rhsby, rhsbz, p):
    lib().or_updt_rhs_b(n[0], n[1], n[2], _b(c_or_f), _b(cbc), rhsbx, rhsby, rhsbz, p)


def chkdiv(n, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w):
    tot, mx = C.c_double(), C.c_double()
    lib().or_chkdiv(n[0], n[1], n[2], dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w, C.byref(tot),
                    C.byref(mx))
    return tot.value, mx.value


def pres_tw_src(n, dxi, dyi, dzi, nh_d, nh_u, dzci, rho0i, f_t12, f_t12_o, p, pold, rho, u, v, w):
    lib().or_pres_tw_src(n[0], n[1], n[2], dxi, dyi, dzi, nh_d, nh_u, dzci, rho0i, f_t12, f_t12_o,
                         p, pold, rho, u, v, w)


def initgrid(n, gr, lz, nh_d=1, two_end=True):
    arrs = [np.empty(n + 2 * nh_d) for _ in range(4)]
    lib().or_initgrid(1 if two_end else 0, n, gr, lz, nh_d, *arrs)
    return tuple(arrs)  # dzc, dzf, zc, zf


def update_property(n, rho1, rho2, psi, rho=None):
    """Interior of rho from psi (src/vof.f90:240-271); the halo is the caller's (boundp)."""
    rho = np.zeros_like(psi) if rho is None else rho
    lib().or_update_property(n[0], n[1], n[2], rho1, rho2, psi, rho)
    return rho


def residual(n, cbc, dxi, dyi, nh_d, dzci, dzfi, f, p):
    r = np.zeros_like(f)
    lib().or_residual((C.c_int * 3)(*n), _b(cbc), dxi, dyi, nh_d, dzci, dzfi, f, p, r)
    return r


MOM_VARIANTS = {"cen": 0, "fll": 1, "sp": 2}


def momad(variant, n, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w, mu=None, rho=None, visc_sp=0.0):
    """momad_xyz_tw_cen / _tw_fll / _sp (src/mom.f90): returns dudt, dvdt, dwdt, shape (nz, ny, nx)."""
    nx, ny, nz = [int(x) for x in n]
    out = [np.empty((nz, ny, nx)) for _ in range(3)]
    dummy = np.zeros((nz + 2, ny + 2, nx + 2))
    lib().or_momad(MOM_VARIANTS[variant], nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w,
                   dummy if mu is None else mu, dummy if rho is None else rho, float(visc_sp), *out)
    return out


def rk(variant, f_t1, f_t2, n, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w, mu, rho, dudtrko, dvdtrko,
       dwdtrko, visc_sp=0.0):
    """rk (src/rk.f90:26-102), in place on u, v, w and the previous right-hand sides."""
    nx, ny, nz = [int(x) for x in n]
    dummy = np.zeros((nz + 2, ny + 2, nx + 2))
    lib().or_rk(MOM_VARIANTS[variant], f_t1, f_t2, nx, ny, nz, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w,
                dummy if mu is None else mu, dummy if rho is None else rho, float(visc_sp), dudtrko, dvdtrko,
                dwdtrko)


def cmpt_time_factors(time_scheme, istep, irk_ss, rkcoeff, dt, dto):
    """cmpt_time_factors (src/rk.f90:104-135): f_t1, f_t2, f_t12."""
    f = np.zeros(3)
    rc = lib().or_cmpt_time_factors(_b(time_scheme), int(istep), int(irk_ss),
                                    np.ascontiguousarray(rkcoeff, dtype=np.float64).ravel(order="F"),
                                    float(dt), float(dto), f)
    if rc != 0:
        raise ValueError("cmpt_time_factors: bad time scheme")
    return tuple(f)
