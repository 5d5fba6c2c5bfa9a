"""flutas_gb300: GB300-native pressure-projection path of FluTAS.

Python front end over the C ABI in ``include/flutas_gb300.h``
(``libflutas_gb300.so``, built in-tree by ``flutas_gb300.build``).  The
functions keep the names and argument meaning of the Fortran routines they
replace (src/initsolver.f90, src/solver_cpu.f90, src/fillps.f90,
src/correc.f90, src/bound.f90, src/chkdiv.f90, src/source.f90) and raise
``FlutasError`` where the C call returns a negative status.

Array arguments are either numpy arrays (host memory: the library copies them
to the device and back inside the call) or CUDA tensors / any object with a
``data_ptr()`` method (device memory: used in place).  3-D fields use the
Fortran memory order, i.e. a C-contiguous array of shape (nz+2h, ny+2h, nx+2h).

There is no CPU fallback: if the CUDA library is missing, importing the
compute functions raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libflutas_gb300.so")

FLUTAS_OK = 0
FLUTAS_EINVAL = -1
FLUTAS_EUNSUPPORTED = -2
FLUTAS_ECUDA = -3
FLUTAS_ENOMEM = -4
FLUTAS_EITER = -5
FLUTAS_ENONFINITE = -6
FLUTAS_EBUSY = -7

EXPORTED = [
    "flutas_gb300_initsolver", "flutas_gb300_solver", "flutas_gb300_fillps", "flutas_gb300_correc",
    "flutas_gb300_boundp", "flutas_gb300_updt_rhs_b", "flutas_gb300_chkdiv",
    "flutas_gb300_pres_tw_src", "flutas_gb300_fftend", "flutas_gb300_last_error",
    "flutas_gb300_plan_set_stream", "flutas_gb300_solve_mixed", "flutas_gb300_projection",
    "flutas_gb300_plan_info", "flutas_gb300_launch_count", "flutas_gb300_profile",
    "flutas_gb300_profile_report", "flutas_gb300_projection_df", "flutas_gb300_last_solve",
    "flutas_gb300_bounduvw", "flutas_gb300_chkdiv_noalloc", "flutas_gb300_batch_create",
    "flutas_gb300_batch_field", "flutas_gb300_batch_solve", "flutas_gb300_batch_report",
    "flutas_gb300_batch_destroy", "flutas_gb300_batch_set", "flutas_gb300_batch_get",
    "flutas_gb300_server_create", "flutas_gb300_server_submit", "flutas_gb300_server_wait",
    "flutas_gb300_server_stats", "flutas_gb300_server_reset_stats", "flutas_gb300_server_destroy",
    "flutas_gb300_load", "flutas_gb300_load_scalar", "flutas_gb300_load_ns", "flutas_gb300_update_property",
    "flutas_gb300_initgrid", "flutas_gb300_rk", "flutas_gb300_rk_sp", "flutas_gb300_cmpt_time_factors",
]


class Request(C.Structure):
    """flutas_request of include/flutas_gb300.h."""
    _fields_ = [("kind", C.c_int), ("n", C.c_int * 3), ("dli", C.c_double * 3), ("nh_d", C.c_int),
                ("dzci", C.c_void_p), ("dzfi", C.c_void_p), ("cbc", C.c_char * 6), ("bcpre", C.c_void_p),
                ("tol", C.c_double), ("max_iter", C.c_int), ("rhs", C.c_void_p), ("p", C.c_void_p),
                ("u", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p), ("rho", C.c_void_p),
                ("pold", C.c_void_p), ("nh_u", C.c_int), ("dt", C.c_double), ("dt_old", C.c_double),
                ("rho0", C.c_double), ("cbcvel", C.c_void_p), ("bcvel", C.c_void_p)]


class FlutasError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FlutasError(FLUTAS_ECUDA, f"CUDA extension missing: {p} (run flutas_gb300.build.build())")
    L = C.CDLL(p)
    vp, dp, ip = C.c_void_p, C.c_double, C.c_int
    L.flutas_gb300_initsolver.argtypes = [vp, vp, ip, vp, vp, C.c_char_p, vp, C.c_char_p, vp, vp, vp,
                                          vp, vp, vp, vp, vp, vp]
    L.flutas_gb300_solver.argtypes = [vp, vp, dp, vp, vp, vp, vp, C.c_char_p, C.c_char_p, vp]
    L.flutas_gb300_fillps.argtypes = [ip] * 5 + [dp] * 3 + [vp, dp, dp, vp, vp, vp, vp]
    L.flutas_gb300_correc.argtypes = [ip] * 5 + [dp] * 3 + [vp, dp, dp, vp, vp, vp, vp, vp]
    L.flutas_gb300_boundp.argtypes = [C.c_char_p, vp, vp, ip, ip, vp, vp, vp, vp, vp]
    L.flutas_gb300_updt_rhs_b.argtypes = [ip] * 3 + [C.c_char_p, C.c_char_p, ip, vp, vp, vp, vp]
    L.flutas_gb300_chkdiv.argtypes = [ip] * 3 + [dp] * 3 + [ip] * 2 + [vp, vp, vp, vp, vp, vp]
    L.flutas_gb300_pres_tw_src.argtypes = [ip] * 3 + [dp] * 3 + [ip] * 2 + [vp, dp, dp, dp, vp, vp,
                                                                             vp, vp, vp, vp]
    L.flutas_gb300_fftend.argtypes = [vp]
    L.flutas_gb300_last_error.argtypes = [C.c_char_p, ip]
    L.flutas_gb300_plan_set_stream.argtypes = [vp, vp, ip]
    L.flutas_gb300_solve_mixed.argtypes = [vp, vp, dp, ip, vp, vp]
    L.flutas_gb300_projection.argtypes = [vp, ip, dp, dp, vp, vp, vp, C.c_char_p, vp, dp, dp, vp, vp, vp,
                                          vp, ip, dp, ip]
    L.flutas_gb300_chkdiv_noalloc.argtypes = [ip] * 3 + [dp] * 3 + [ip] * 2 + [vp, vp, vp, vp, vp, vp]
    L.flutas_gb300_batch_create.argtypes = [ip, vp, vp, ip, vp, vp, C.c_char_p, ip, vp]
    L.flutas_gb300_batch_field.argtypes = [vp, ip, vp]
    L.flutas_gb300_batch_solve.argtypes = [vp, dp, ip, vp, vp]
    L.flutas_gb300_batch_report.argtypes = [vp, C.c_char_p, ip]
    L.flutas_gb300_batch_set.argtypes = [vp, ip, vp]
    L.flutas_gb300_server_create.argtypes = [C.c_size_t, ip, vp]
    L.flutas_gb300_server_submit.argtypes = [vp, C.POINTER(Request), vp]
    L.flutas_gb300_server_wait.argtypes = [vp, C.c_longlong, vp, vp, vp]
    L.flutas_gb300_server_stats.argtypes = [vp, C.c_char_p, ip]
    L.flutas_gb300_server_reset_stats.argtypes = [vp]
    L.flutas_gb300_server_destroy.argtypes = [vp]
    L.flutas_gb300_batch_get.argtypes = [vp, ip, vp]
    L.flutas_gb300_batch_destroy.argtypes = [vp]
    L.flutas_gb300_bounduvw.argtypes = [C.c_char_p, vp, vp, ip, ip, vp, vp, vp, vp, vp, vp, vp, vp]
    L.flutas_gb300_plan_info.argtypes = [vp, vp, vp, vp]
    L.flutas_gb300_launch_count.argtypes = [vp]
    L.flutas_gb300_projection_df.argtypes = [vp, ip, dp, dp, vp, vp, vp, C.c_char_p, vp, dp, dp, dp, vp,
                                             vp, vp, vp, vp, vp, ip, dp, ip]
    L.flutas_gb300_last_solve.argtypes = [vp, vp, vp]
    L.flutas_gb300_profile.argtypes = [ip]
    L.flutas_gb300_profile_report.argtypes = [C.c_char_p, ip, ip]
    L.flutas_gb300_load.argtypes = [C.c_char, C.c_char_p, vp, ip, vp]
    L.flutas_gb300_update_property.argtypes = [vp, vp, vp, vp]
    L.flutas_gb300_load_scalar.argtypes = [C.c_char, C.c_char_p, vp, vp, vp]
    L.flutas_gb300_load_ns.argtypes = [C.c_char, C.c_char_p, vp, ip, vp, vp, vp, vp, vp, vp]
    L.flutas_gb300_initgrid.argtypes = [C.c_char_p, ip, dp, dp, ip, vp, vp, vp, vp]
    L.flutas_gb300_rk.argtypes = [C.c_char_p, dp, dp] + [ip] * 3 + [dp] * 3 + [ip] * 2 + [vp] * 10
    L.flutas_gb300_rk_sp.argtypes = [dp, dp] + [ip] * 3 + [dp] * 3 + [ip] * 2 + [vp, vp, dp] + [vp] * 6
    L.flutas_gb300_cmpt_time_factors.argtypes = [C.c_char_p, ip, ip, ip, vp, dp, dp, vp, vp, vp]
    for name in EXPORTED:
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(512)
    load().flutas_gb300_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def _check(rc: int, allow=()):
    if rc != FLUTAS_OK and rc not in allow:
        raise FlutasError(rc, last_error())
    return rc


def _ptr(a):
    """Address of an array argument (numpy host array or device tensor)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError("device tensor must be contiguous")
        return a.data_ptr()
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous or a.dtype != np.float64:
            raise ValueError("numpy arrays must be C-contiguous float64")
        return a.ctypes.data
    raise TypeError(f"unsupported array type {type(a)}")


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


def _d6(v):
    return (C.c_double * 6)(*[float(x) for x in v])


def _i3(v):
    return (C.c_int * 3)(*[int(x) for x in v])


def _chars(s, n):
    s = "".join(s) if not isinstance(s, (str, bytes)) else s
    s = s.encode() if isinstance(s, str) else s
    if len(s) != n:
        raise ValueError(f"expected {n} BC characters, got {s!r}")
    return s


def _vel_bcs(cbcvel, bcvel):
    if cbcvel is None:
        return None, None
    cv = _chars(cbcvel, 18)
    bv = (C.c_double * 18)(*[float(x) for x in (bcvel if bcvel is not None else [0.0] * 18)])
    return cv, C.cast(bv, C.c_void_p)


class Plan:
    """The plan held in arrplan(1,1), plus every host output of initsolver.

    Mirrors ``initsolver(n,dims,dims_z,dli,nh_d,dzci,dzfi,cbc,bc,c_or_f,
    lambdaxy,a,b,c,arrplan,normfft,rhsbx,rhsby,rhsbz)`` (src/initsolver.f90:21).
    """

    def __init__(self, n, dli, nh_d, dzci, dzfi, cbc, bc, c_or_f="ccc"):
        L = load()
        self.n = [int(x) for x in n]
        nx, ny, nz = self.n
        self.nh_d = int(nh_d)
        self.dli = [float(x) for x in dli]
        self.cbc = _chars(cbc, 6).decode()
        self.bc = [float(x) for x in bc]
        self.c_or_f = _chars(c_or_f, 3).decode()
        self.dzci = np.ascontiguousarray(dzci, dtype=np.float64)
        self.dzfi = np.ascontiguousarray(dzfi, dtype=np.float64)
        if self.dzci.size != nz + 2 * self.nh_d or self.dzfi.size != nz + 2 * self.nh_d:
            raise ValueError("dzci/dzfi must have nz+2*nh_d entries")
        self.lambdaxy = np.empty((ny, nx))
        self.a, self.b, self.c = np.empty(nz), np.empty(nz), np.empty(nz)
        self.rhsbx = np.empty((2, nz, ny))
        self.rhsby = np.empty((2, nz, nx))
        self.rhsbz = np.empty((2, ny, nx))
        self.arrplan = (C.c_void_p * 4)()
        nf = C.c_double()
        _check(L.flutas_gb300_initsolver(
            C.cast(_i3(self.n), C.c_void_p), C.cast(_d3(self.dli), C.c_void_p), self.nh_d,
            self.dzci.ctypes.data, self.dzfi.ctypes.data, self.cbc.encode(),
            C.cast(_d6(self.bc), C.c_void_p), self.c_or_f.encode(), self.lambdaxy.ctypes.data,
            self.a.ctypes.data, self.b.ctypes.data, self.c.ctypes.data,
            C.cast(self.arrplan, C.c_void_p), C.addressof(nf), self.rhsbx.ctypes.data,
            self.rhsby.ctypes.data, self.rhsbz.ctypes.data))
        self.normfft = nf.value
        self.handle = self.arrplan[0]

    # -- the reference-facing calls -------------------------------------------------
    def solver(self, p):
        """solver(n,arrplan,normfft,lambdaxy,a,b,c,bcz,c_or_f,p), in place (FP64)."""
        L = load()
        _check(L.flutas_gb300_solver(
            C.cast(_i3(self.n), C.c_void_p), C.cast(self.arrplan, C.c_void_p), self.normfft,
            self.lambdaxy.ctypes.data, self.a.ctypes.data, self.b.ctypes.data, self.c.ctypes.data,
            self.cbc[4:6].encode(), self.c_or_f.encode(), _ptr(p)))
        return p

    def solve_mixed(self, p, tol=1e-10, max_iter=8, allow_unconverged=False):
        """FP32-bulk solve with FP64 residual refinement; returns (relres, nsolves)."""
        L = load()
        rr, it = C.c_double(), C.c_int()
        _check(L.flutas_gb300_solve_mixed(self.handle, _ptr(p), float(tol), int(max_iter),
                                          C.addressof(rr), C.addressof(it)),
               allow=(FLUTAS_EITER,) if allow_unconverged else ())
        return rr.value, it.value

    def projection(self, nh_u, dxi, dyi, dzci, dzfi, bcpre, dt, rho0, u, v, w, p, precision=0,
                   tol=1e-10, max_iter=8, cbcvel=None, bcvel=None):
        """fillps -> updt_rhs_b -> solve -> boundp -> correc [-> bounduvw] -> p += phi -> boundp."""
        L = load()
        cv, bv = _vel_bcs(cbcvel, bcvel)
        _check(L.flutas_gb300_projection(self.handle, int(nh_u), float(dxi), float(dyi), _ptr(dzci),
                                         _ptr(dzfi), C.cast(_d6(bcpre), C.c_void_p), cv, bv, float(dt),
                                         float(rho0), _ptr(u), _ptr(v), _ptr(w), _ptr(p),
                                         int(precision), float(tol), int(max_iter)))

    def projection_df(self, nh_u, dxi, dyi, dzci, dzfi, bcpre, f_t12, f_t12_o, rho0, rho, pold, u, v, w,
                      p, precision=0, tol=1e-10, max_iter=8, cbcvel=None, bcvel=None):
        """pres_tw_src (Dodd-Ferrante split) [-> bounduvw] + projection, one call."""
        L = load()
        cv, bv = _vel_bcs(cbcvel, bcvel)
        _check(L.flutas_gb300_projection_df(self.handle, int(nh_u), float(dxi), float(dyi), _ptr(dzci),
                                            _ptr(dzfi), C.cast(_d6(bcpre), C.c_void_p), cv, bv, float(f_t12),
                                            float(f_t12_o), float(rho0), _ptr(rho), _ptr(pold), _ptr(u),
                                            _ptr(v), _ptr(w), _ptr(p), int(precision), float(tol),
                                            int(max_iter)))

    def last_solve(self):
        rr, it = C.c_double(), C.c_int()
        _check(load().flutas_gb300_last_solve(self.handle, C.addressof(rr), C.addressof(it)))
        return rr.value, it.value

    def set_stream(self, stream_handle: int | None, synchronous: bool = True):
        _check(load().flutas_gb300_plan_set_stream(self.handle, stream_handle or None,
                                                   1 if synchronous else 0))

    def info(self):
        b, p64, p32 = C.c_size_t(), C.c_int(), C.c_int()
        _check(load().flutas_gb300_plan_info(self.handle, C.addressof(b), C.addressof(p64),
                                             C.addressof(p32)))
        return {"device_bytes": b.value, "xy_path_fp64": p64.value, "xy_path_fp32": p32.value}

    def fftend(self):
        if self.arrplan[0]:
            _check(load().flutas_gb300_fftend(C.cast(self.arrplan, C.c_void_p)))
            self.handle = None

    def __del__(self):
        try:
            if _lib is not None and self.arrplan[0]:
                _lib.flutas_gb300_fftend(C.cast(self.arrplan, C.c_void_p))
        except Exception:
            pass


def rk(space_scheme_mom, f_t1, f_t2, n, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, u, v, w, mu, rho,
       dudtrko, dvdtrko, dwdtrko):
    """rk(space_scheme_mom,f_t1,f_t2,nx,ny,nz,dxi,dyi,dzi,nh_d,nh_u,dzci,dzfi,u,v,w,mu,rho,
    dudtrko,dvdtrko,dwdtrko) (src/rk.f90:26), two-phase right-hand sides; in place."""
    _check(load().flutas_gb300_rk(_chars(space_scheme_mom, 3), float(f_t1), float(f_t2), int(n[0]), int(n[1]),
                                  int(n[2]), float(dxi), float(dyi), float(dzi), int(nh_d), int(nh_u), _ptr(dzci),
                                  _ptr(dzfi), _ptr(u), _ptr(v), _ptr(w), _ptr(mu), _ptr(rho), _ptr(dudtrko),
                                  _ptr(dvdtrko), _ptr(dwdtrko)))


def rk_sp(f_t1, f_t2, n, dxi, dyi, dzi, nh_d, nh_u, dzci, dzfi, visc_sp, u, v, w, dudtrko, dvdtrko, dwdtrko):
    """rk of the single-phase build (momad_xyz_sp, visc_sp = mu_sp/rho_sp); in place."""
    _check(load().flutas_gb300_rk_sp(float(f_t1), float(f_t2), int(n[0]), int(n[1]), int(n[2]), float(dxi),
                                     float(dyi), float(dzi), int(nh_d), int(nh_u), _ptr(dzci), _ptr(dzfi),
                                     float(visc_sp), _ptr(u), _ptr(v), _ptr(w), _ptr(dudtrko), _ptr(dvdtrko),
                                     _ptr(dwdtrko)))


def cmpt_time_factors(time_scheme, restart, istep, irk_ss, rkcoeff, dt, dto):
    """cmpt_time_factors (src/rk.f90:104): returns f_t1, f_t2, f_t12."""
    rc = np.ascontiguousarray(np.asarray(rkcoeff, dtype=np.float64).ravel(order="F"))
    f = [C.c_double() for _ in range(3)]
    _check(load().flutas_gb300_cmpt_time_factors(_chars(time_scheme, 3), int(bool(restart)), int(istep), int(irk_ss),
                                                 rc.ctypes.data, float(dt), float(dto),
                                                 *[C.addressof(x) for x in f]))
    return tuple(x.value for x in f)


def initgrid(inivel, n, gr, lz, nh_d=1):
    """initgrid(inivel,n,gr,lz,nh_d,dzc,dzf,zc,zf) (src/initgrid.f90:17): returns
    dzc, dzf, zc, zf, each with n + 2*nh_d entries (index k-1+nh_d is cell k)."""
    out = [np.empty(int(n) + 2 * int(nh_d)) for _ in range(4)]
    _check(load().flutas_gb300_initgrid(_chars(inivel, 3), int(n), float(gr), float(lz), int(nh_d),
                                        *[a.ctypes.data for a in out]))
    return tuple(out)


def initsolver(n, dli, nh_d, dzci, dzfi, cbc, bc, c_or_f="ccc") -> Plan:
    return Plan(n, dli, nh_d, dzci, dzfi, cbc, bc, c_or_f)


def fillps(n, nh_d, nh_u, dxi, dyi, dzi, dzfi, dti, rho0, u, v, w, p):
    _check(load().flutas_gb300_fillps(int(n[0]), int(n[1]), int(n[2]), int(nh_d), int(nh_u), float(dxi),
                                      float(dyi), float(dzi), _ptr(dzfi), float(dti), float(rho0),
                                      _ptr(u), _ptr(v), _ptr(w), _ptr(p)))


def correc(n, nh_d, nh_u, dxi, dyi, dzi, dzci, dt, rho0, p, u, v, w, rho=None):
    _check(load().flutas_gb300_correc(int(n[0]), int(n[1]), int(n[2]), int(nh_d), int(nh_u), float(dxi),
                                      float(dyi), float(dzi), _ptr(dzci), float(dt), float(rho0),
                                      _ptr(p), _ptr(u), _ptr(v), _ptr(w), _ptr(rho)))


def boundp(cbc, n, bc, nh_d, dl, dzc, dzf, p, nh_p=1):
    halo = (C.c_int * 3)(1, 1, 1)
    _check(load().flutas_gb300_boundp(_chars(cbc, 6), C.cast(_i3(n), C.c_void_p),
                                      C.cast(_d6(bc), C.c_void_p), int(nh_d), int(nh_p),
                                      C.cast(halo, C.c_void_p), C.cast(_d3(dl), C.c_void_p),
                                      _ptr(dzc), _ptr(dzf), _ptr(p)))


def bounduvw(cbcvel, n, bcvel, nh_d, nh_u, dl, dzc, dzf, u, v, w, isoutflow=None):
    """bounduvw(cbc,n,bc,nh_d,nh_u,halo,isoutflow,dl,dzc,dzf,u,v,w); isoutflow: 6 flags (0:1,1:3)."""
    halo = (C.c_int * 3)(1, 1, 1)
    outf = (C.c_int * 6)(*[int(bool(x)) for x in (isoutflow or [0] * 6)])
    _check(load().flutas_gb300_bounduvw(_chars(cbcvel, 18), C.cast(_i3(n), C.c_void_p),
                                        C.cast((C.c_double * 18)(*[float(x) for x in bcvel]), C.c_void_p),
                                        int(nh_d), int(nh_u), C.cast(halo, C.c_void_p), C.cast(outf, C.c_void_p),
                                        C.cast(_d3(dl), C.c_void_p), _ptr(dzc), _ptr(dzf), _ptr(u), _ptr(v),
                                        _ptr(w)))


def updt_rhs_b(n, c_or_f, cbc, rhsbx, rhsby, rhsbz, p, nh_p=1):
    _check(load().flutas_gb300_updt_rhs_b(int(n[0]), int(n[1]), int(n[2]), _chars(c_or_f, 3),
                                          _chars(cbc, 6), int(nh_p), _ptr(rhsbx), _ptr(rhsby),
                                          _ptr(rhsbz), _ptr(p)))


def chkdiv(n, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w):
    tot, mx = C.c_double(), C.c_double()
    _check(load().flutas_gb300_chkdiv(int(n[0]), int(n[1]), int(n[2]), float(dxi), float(dyi), float(dzi),
                                      int(nh_d), int(nh_u), _ptr(dzfi), _ptr(u), _ptr(v), _ptr(w),
                                      C.addressof(tot), C.addressof(mx)))
    return tot.value, mx.value


def chkdiv_noalloc(n, dxi, dyi, dzi, nh_d, nh_u, dzfi, u, v, w):
    """chkdiv without any device allocation (device arrays only; ny*nz <= 65536)."""
    tot, mx = C.c_double(), C.c_double()
    _check(load().flutas_gb300_chkdiv_noalloc(int(n[0]), int(n[1]), int(n[2]), float(dxi), float(dyi),
                                              float(dzi), int(nh_d), int(nh_u), _ptr(dzfi), _ptr(u), _ptr(v),
                                              _ptr(w), C.addressof(tot), C.addressof(mx)))
    return tot.value, mx.value


def update_property(n, prop12, vof, prop):
    """update_property (src/vof.f90:240-271): interior of prop from vof."""
    _check(load().flutas_gb300_update_property(C.cast(_i3(n), C.c_void_p),
                                               C.cast((C.c_double * 2)(*[float(x) for x in prop12]), C.c_void_p),
                                               _ptr(vof), _ptr(prop)))


def load_field(io, filename, n, fld, nh=1):
    """load (src/load.f90:21-89): io 'r' reads the raw FP64 interior of `filename`
    into fld (halo nh; host array or CUDA tensor), io 'w' writes it."""
    _check(load().flutas_gb300_load(io.encode()[:1], str(filename).encode(), C.cast(_i3(n), C.c_void_p), int(nh),
                                    _ptr(fld)))


def load_scalar(io, filename, time=0.0, istep=0, dto=0.0):
    """load_scalar (src/load.f90:91-128); returns (time, istep, dto)."""
    t, it, d = C.c_double(time), C.c_int(istep), C.c_double(dto)
    _check(load().flutas_gb300_load_scalar(io.encode()[:1], str(filename).encode(), C.addressof(t), C.addressof(it),
                                           C.addressof(d)))
    return t.value, it.value, d.value


def load_ns(io, filename, n, u, v, w, p, time=0.0, istep=0.0, nh=1):
    """load_ns (src/load.f90:130-214); returns (time, istep)."""
    t, it = C.c_double(time), C.c_double(istep)
    _check(load().flutas_gb300_load_ns(io.encode()[:1], str(filename).encode(), C.cast(_i3(n), C.c_void_p),
                                       int(nh), _ptr(u), _ptr(v), _ptr(w), _ptr(p), C.addressof(t),
                                       C.addressof(it)))
    return t.value, it.value


def pres_tw_src(n, dxi, dyi, dzi, nh_d, nh_u, dzci, rho0i, f_t12, f_t12_o, p, pold, rho, u, v, w):
    _check(load().flutas_gb300_pres_tw_src(int(n[0]), int(n[1]), int(n[2]), float(dxi), float(dyi),
                                           float(dzi), int(nh_d), int(nh_u), _ptr(dzci), float(rho0i),
                                           float(f_t12), float(f_t12_o), _ptr(p), _ptr(pold), _ptr(rho),
                                           _ptr(u), _ptr(v), _ptr(w)))


def launch_count() -> int:
    c = C.c_ulonglong()
    _check(load().flutas_gb300_launch_count(C.addressof(c)))
    return c.value


def profile(enable: bool):
    _check(load().flutas_gb300_profile(1 if enable else 0))


def profile_report(reset: bool = True) -> dict:
    """{kernel: (launches, total_ms)} of the launches recorded since the last reset."""
    buf = C.create_string_buffer(1 << 16)
    _check(load().flutas_gb300_profile_report(buf, 1 << 16, 1 if reset else 0))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.rsplit(" ", 2)
        out[name] = (int(cnt), float(ms))
    return out


class Batch:
    """Many independent grids solved together (mixed precision, one CUDA graph per solve).

    grids: list of dicts with keys n (3 ints), dli (3), dzci, dzfi (numpy, nz+2*nh_d), cbc (6 chars).
    """

    def __init__(self, grids, nh_d=1, autotune=True):
        L = load()
        self.ng = len(grids)
        n = (C.c_int * (3 * self.ng))(*[int(v) for g in grids for v in g["n"]])
        dli = (C.c_double * (3 * self.ng))(*[float(v) for g in grids for v in g["dli"]])
        self._z = [(np.ascontiguousarray(g["dzci"], dtype=np.float64),
                    np.ascontiguousarray(g["dzfi"], dtype=np.float64)) for g in grids]
        zci = (C.c_void_p * self.ng)(*[z[0].ctypes.data for z in self._z])
        zfi = (C.c_void_p * self.ng)(*[z[1].ctypes.data for z in self._z])
        cbc = "".join(g["cbc"] for g in grids).encode()
        self.n = [list(g["n"]) for g in grids]
        self.handle = C.c_void_p()
        _check(L.flutas_gb300_batch_create(self.ng, C.cast(n, C.c_void_p), C.cast(dli, C.c_void_p), int(nh_d),
                                           C.cast(zci, C.c_void_p), C.cast(zfi, C.c_void_p), cbc,
                                           1 if autotune else 0, C.addressof(self.handle)))

    def field_ptr(self, g: int) -> int:
        p = C.c_void_p()
        _check(load().flutas_gb300_batch_field(self.handle, int(g), C.addressof(p)))
        return p.value

    def set(self, g: int, arr):
        _check(load().flutas_gb300_batch_set(self.handle, int(g), _ptr(arr)))

    def get(self, g: int, out=None):
        nx, ny, nz = self.n[g]
        out = np.empty((nz + 2, ny + 2, nx + 2)) if out is None else out
        _check(load().flutas_gb300_batch_get(self.handle, int(g), _ptr(out)))
        return out

    def solve(self, tol=1e-10, max_iter=8, allow_unconverged=False):
        rr = np.zeros(self.ng)
        it = np.zeros(self.ng, dtype=np.int32)
        _check(load().flutas_gb300_batch_solve(self.handle, float(tol), int(max_iter), rr.ctypes.data, it.ctypes.data),
               allow=(FLUTAS_EITER,) if allow_unconverged else ())
        return rr, it

    def report(self) -> str:
        buf = C.create_string_buffer(1 << 20)
        _check(load().flutas_gb300_batch_report(self.handle, buf, 1 << 20))
        return buf.value.decode()

    def destroy(self):
        if self.handle:
            _check(load().flutas_gb300_batch_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            if _lib is not None and self.handle:
                _lib.flutas_gb300_batch_destroy(self.handle)
        except Exception:
            pass


class Server:
    """Continuous-batching request loop (flutas_gb300_server_*).

    submit_solve / submit_projection return a ticket; wait(ticket) blocks until
    that request is done and returns (status, relres, fp32_solves, latency_ms).
    Arrays passed to submit_* must stay alive until wait() returns.
    """

    def __init__(self, hbm_budget_bytes: int, slots: int = 4):
        self.handle = C.c_void_p()
        _check(load().flutas_gb300_server_create(int(hbm_budget_bytes), int(slots), C.addressof(self.handle)))
        self._keep = {}

    def _submit(self, req, keep):
        t = C.c_longlong()
        _check(load().flutas_gb300_server_submit(self.handle, C.byref(req), C.addressof(t)))
        self._keep[t.value] = (req, keep)
        return t.value

    @staticmethod
    def _grid(req, n, dli, nh_d, dzci, dzfi, cbc, tol, max_iter):
        req.n = (C.c_int * 3)(*[int(x) for x in n])
        req.dli = (C.c_double * 3)(*[float(x) for x in dli])
        req.nh_d = int(nh_d)
        req.dzci, req.dzfi = _ptr(dzci), _ptr(dzfi)
        req.cbc = _chars(cbc, 6)
        req.tol, req.max_iter = float(tol), int(max_iter)

    def submit_solve(self, n, dli, dzci, dzfi, cbc, rhs, out, tol=1e-10, max_iter=8, nh_d=1):
        dzci, dzfi = np.ascontiguousarray(dzci, dtype=np.float64), np.ascontiguousarray(dzfi, dtype=np.float64)
        req = Request()
        req.kind = 0
        self._grid(req, n, dli, nh_d, dzci, dzfi, cbc, tol, max_iter)
        req.rhs, req.p = _ptr(rhs), _ptr(out)
        return self._submit(req, (dzci, dzfi, rhs, out))

    def submit_projection(self, n, dli, dzci, dzfi, cbc, u, v, w, p, dt, rho0=1.0, nh_u=1, rho=None, pold=None,
                          dt_old=None, tol=1e-10, max_iter=8, cbcvel=None, bcvel=None, nh_d=1):
        dzci, dzfi = np.ascontiguousarray(dzci, dtype=np.float64), np.ascontiguousarray(dzfi, dtype=np.float64)
        req = Request()
        req.kind = 1
        self._grid(req, n, dli, nh_d, dzci, dzfi, cbc, tol, max_iter)
        req.u, req.v, req.w, req.p = _ptr(u), _ptr(v), _ptr(w), _ptr(p)
        req.rho, req.pold = _ptr(rho), _ptr(pold)
        req.nh_u, req.dt, req.dt_old, req.rho0 = int(nh_u), float(dt), float(dt_old or dt), float(rho0)
        keep = [dzci, dzfi, u, v, w, p, rho, pold]
        if cbcvel is not None:
            cv = C.create_string_buffer(_chars(cbcvel, 18), 18)
            bv = (C.c_double * 18)(*[float(x) for x in (bcvel if bcvel is not None else [0.0] * 18)])
            req.cbcvel, req.bcvel = C.cast(cv, C.c_void_p), C.cast(bv, C.c_void_p)
            keep += [cv, bv]
        return self._submit(req, keep)

    def wait(self, ticket):
        rr, it, lat = C.c_double(), C.c_int(), C.c_double()
        rc = load().flutas_gb300_server_wait(self.handle, C.c_longlong(ticket), C.addressof(rr), C.addressof(it),
                                             C.addressof(lat))
        self._keep.pop(ticket, None)
        return rc, rr.value, it.value, lat.value

    def stats(self) -> dict:
        import json
        buf = C.create_string_buffer(4096)
        _check(load().flutas_gb300_server_stats(self.handle, buf, 4096))
        return json.loads(buf.value.decode())

    def reset_stats(self):
        _check(load().flutas_gb300_server_reset_stats(self.handle))

    def close(self):
        if self.handle:
            _check(load().flutas_gb300_server_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            if _lib is not None and self.handle:
                _lib.flutas_gb300_server_destroy(self.handle)
        except Exception:
            pass
