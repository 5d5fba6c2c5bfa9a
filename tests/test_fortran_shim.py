"""CPU checks of the Fortran module fortran/mod_solver_gb300.f90.

No Fortran compiler exists on these machines, so the module is checked as
text: every bind(C) interface names a symbol that include/flutas_gb300.h
declares, with the same number of arguments, and every wrapper keeps the
dummy-argument list of the FluTAS routine it replaces, so that
`use mod_solver_gb300, only: solver_cpu => gb300_solver_cpu, ...` is a
one-line swap in the apps.
"""
import os
import re

from conftest import ROOT

F90 = os.path.join(ROOT, "fortran", "mod_solver_gb300.f90")
HDR = os.path.join(ROOT, "include", "flutas_gb300.h")

# Dummy-argument lists of the FluTAS routines (the interface the apps call):
# src/initsolver.f90:21, src/solver_cpu.f90:20, src/solver_gpu.f90:31, src/fillps.f90:16,
# src/correc.f90:16, src/bound.f90:146, src/bound.f90:17, src/bound.f90:829,
# src/chkdiv.f90:18, src/source.f90:247, src/fft.f90:159, src/vof.f90:240, src/load.f90:21,
# src/initgrid.f90:17, src/rk.f90:26, src/rk.f90:104
REFERENCE_ARGS = {
    "initsolver": "n,dims,dims_z,dli,nh_d,dzci,dzfi,cbc,bc,c_or_f,lambdaxy,a,b,c,arrplan,normfft,rhsbx,rhsby,rhsbz",
    "solver_cpu": "n,arrplan,normfft,lambdaxy,a,b,c,bcz,c_or_f,p",
    "solver_gpu": "n,dims,arrplan,normfft,lambdaxy,a,b,c,bc,c_or_f,p",
    "fillps": "nx,ny,nz,nh_d,nh_u,dxi,dyi,dzi,dzfi,dti,rho0,u,v,w,p",
    "correc": "nx,ny,nz,nh_d,nh_u,dxi,dyi,dzi,dzci,dt,rho0,p,u,v,w,rho",
    "boundp": "cbc,n,bc,nh_d,nh_p,halo,dl,dzc,dzf,p",
    "bounduvw": "cbc,n,bc,nh_d,nh_u,halo,isoutflow,dl,dzc,dzf,u,v,w",
    "updt_rhs_b": "nx,ny,nz,c_or_f,cbc,nh_p,rhsbx,rhsby,rhsbz,p",
    "chkdiv": "nx,ny,nz,dxi,dyi,dzi,nh_d,nh_u,dzfi,u,v,w,divtot,divmax",
    "pres_tw_src": "nx,ny,nz,dxi,dyi,dzi,nh_d,nh_u,dzci,rho0i,f_t12,f_t12_o,p,pold,rho,u,v,w",
    "fftend": "arrplan",
    "update_property": "n,prop12,vof,prop",
    "load": "io,filename,n,fld",
    "initgrid": "inivel,n,gr,lz,nh_d,dzc,dzf,zc,zf",
    "rk": "space_scheme_mom,f_t1,f_t2,nx,ny,nz,dxi,dyi,dzi,nh_d,nh_u,dzci,dzfi,u,v,w,mu,rho,dudtrko,dvdtrko,dwdtrko",
    "cmpt_time_factors": "time_scheme,restart,istep,irk_ss,rkcoeff,dt,dto,f_t1,f_t2,f_t12",
}


def _strip_comments(src):
    # comments and preprocessor lines (the module is preprocessed like the reference's sources)
    return "\n".join(line.split("!")[0] for line in src.splitlines() if not line.lstrip().startswith("#"))


def _join_continuations(src):
    return re.sub(r"&\s*\n\s*&?", " ", src)


def header_arity():
    hdr = open(HDR).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    out = {}
    for name, params in re.findall(r"FLUTAS_API\s+int\s+(flutas_gb300_\w+)\s*\((.*?)\)\s*;", hdr, flags=re.S):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else len(params.split(","))
    return out


def shim():
    return _join_continuations(_strip_comments(open(F90).read()))


def test_every_binding_matches_the_header():
    ar = header_arity()
    src = shim()
    binds = re.findall(r"function\s+(c_\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name='(\w+)'\)", src, flags=re.I)
    assert len(binds) >= 14
    for fname, args, cname in binds:
        assert cname in ar, cname
        n = len([a for a in args.split(",") if a.strip()])
        assert n == ar[cname], (cname, n, ar[cname])


def test_wrappers_keep_the_reference_argument_lists():
    src = shim()
    subs = dict((name.lower(), re.sub(r"\s+", "", args))
                for name, args in re.findall(r"subroutine\s+gb300_(\w+)\s*\(([^)]*)\)", src, flags=re.I))
    for routine, args in REFERENCE_ARGS.items():
        assert routine in subs, routine
        assert subs[routine] == args, (routine, subs[routine])


def test_every_wrapper_is_public_and_checks_its_status():
    src = shim()
    pub = re.search(r"public\s*::([^\n]*)", src).group(1)
    public = {s.strip() for s in pub.split(",")}
    for routine in REFERENCE_ARGS:
        assert f"gb300_{routine}" in public, routine
    # each wrapper body calls check(c_...) with the status of the C call
    bodies = re.findall(r"subroutine\s+(gb300_\w+)(.*?)end\s+subroutine", src, flags=re.S | re.I)
    assert bodies
    for name, body in bodies:
        assert re.search(r"call\s+check\s*\(\s*c_\w+\s*\(", body), name
