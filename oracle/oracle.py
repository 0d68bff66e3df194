"""CPU oracle for the SFD_EXCMG forward-solve path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only to check results.  The shipped
library (``sfd_excmg_gb300``) never imports, loads or calls anything here.

It restates the reference's FP64 algorithms: the heavy loops live in
``sfd_oracle.c`` (index-for-index restatement of fdfe_main.f90, solvers.f90,
div_correc.f90, excmg.f90, model_selec.f90), the per-frequency orchestration
(``doublemode_nor`` fdfe_main.f90:892-1063, ``u1u2`` :1228-1256,
``doublemode_acc`` :1258-1563, ``fwd_solver`` :1565-1594) is restated here.

MKL PARDISO (solvers.f90:765-875, used on the two coarsest EXCMG levels) is
closed; it is replaced by SciPy's SuperLU (``scipy.sparse.linalg.splu``),
which, like PARDISO with iterative refinement, returns the direct solution
to rounding level.

Parity status: UNPINNED against reference outputs -- the reference needs
ifort + MKL, does not compile as committed, and ships no golden vectors.
The oracle is pinned by known-answer tests instead (tests/test_oracle_*.py):
the analytic 1-D layered response, the homogeneous half-space impedance,
polynomial exactness of the prolongation, and the published DTM1 iteration
counts where they are reproducible.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import splu

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_SO = os.path.join(_BUILD, "libsfd_oracle.so")
_LIB = None
_LOCK = threading.Lock()

MU = 4 * np.pi * 1e-7
SIGMA_AIR = 1e-9  # global_para.f90:12

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


def build(force: bool = False) -> str:
    """Compile sfd_oracle.c into oracle/_build/libsfd_oracle.so (gcc, -O2)."""
    src = os.path.join(HERE, "sfd_oracle.c")
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(src):
        return _SO
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _SO + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            _LIB = ctypes.CDLL(build())
            L = _LIB
            L.orc_assemble.restype = ctypes.c_int64
            L.orc_solve.restype = ctypes.c_int
            L.orc_solve.argtypes = [
                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                c_double_p, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                ctypes.c_int64, ctypes.c_void_p, c_int64_p, c_int32_p, ctypes.c_void_p, ctypes.c_void_p,
                ctypes.c_double, ctypes.c_int, c_double_p, ctypes.c_int64]
            L.orc_bicgstab_fixed.restype = ctypes.c_int
            L.orc_extint_v.restype = ctypes.c_int
            L.orc_post_process.restype = ctypes.c_int
            L.orc_post_process_topo.restype = ctypes.c_int
            L.orc_div_correc.restype = ctypes.c_int
            L.orc_ssor_apply.restype = ctypes.c_int
            L.orc_ilu_apply.restype = ctypes.c_int
            L.orc_sgs.restype = None
    return _LIB


def _d(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def _z(x):
    return np.ascontiguousarray(x, dtype=np.complex128)


def _p(x, t=c_double_p):
    return x.ctypes.data_as(t)


def nedges(nx, ny, nz):
    return nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz


# --------------------------------------------------------------------------
# Model container (restates read_input's outputs, file_opt.f90:8-95)
# --------------------------------------------------------------------------
@dataclass
class OracleModel:
    nx: int
    ny: int
    nz: int  # total z cells, air included (z index 1 = top of air)
    nair: int
    a: np.ndarray
    b: np.ndarray
    c: np.ndarray  # length nz, air first
    sigma: np.ndarray  # shape (6, ncell): Fortran sigma(ncell,6)
    freq: np.ndarray
    recv: np.ndarray  # shape (nrec, 3)
    level: int = 3
    eps: float = 1e-8
    solver: int = 1
    out_type: int = 1


@dataclass
class OracleOpts:
    excmg: bool = False          # fwd_acc (global_para.f90:19), default 0
    pre: str = "S"               # pre_type (global_para.f90:18): 'S', 'J', 'I' (ILU(0)) or 'M'
    div_cor: bool = True         # global_para.f90:8
    corr_intv: int = 200         # global_para.f90:9
    corr_tol: float = 1e-3       # global_para.f90:10
    omega: float = 1.0           # ssor_omg (solvers.f90:14)
    maxit_plain: int = 5000      # fdfe_main.f90:993
    maxit_level: int = 1000      # fdfe_main.f90:1414
    coarsen_quirk: bool = True   # mesh_coarsen index shift (fdfe_main.f90:64)
    midpoint_quirk: bool = True  # cal_coef along-edge nodes (excmg.f90:685)
    rd: int = 2                  # arho_interp2 stencil (fdfe_main.f90:640,685)
    # exact solve of EXCMG levels 1-2 (PARDISO in the reference): "splu" (SciPy SuperLU) or
    # "converged" (converged_solve, the same answer to a 1e-15 residual, for large coarse meshes)
    coarse_solver: str = "splu"


# --------------------------------------------------------------------------
# Thin wrappers over the C restatement
# --------------------------------------------------------------------------
def mt1d_anl(ff, conv, c):
    """mt1d_anl (model_selec.f90:266-401). conv: (nz,6) array; returns ex, hx, imp."""
    conv = np.asarray(conv, dtype=np.float64)
    nz = conv.shape[0]
    cf = np.asfortranarray(conv).ravel(order="F").copy()
    ex = np.zeros(2 * nz + 2, np.complex128)
    hx = np.zeros(2 * nz + 2, np.complex128)
    imp = np.zeros(4, np.complex128)
    lib().orc_mt1d_anl(ctypes.c_double(ff), ctypes.c_int(nz), _p(cf), _p(_d(c)), _p(ex), _p(hx), _p(imp))
    return ex, hx, imp


def column_conv(sigma, nx, ny, nz):
    """cont1(k,1:3) = conv((k-1)*nx*ny+1, 1:3), off-diagonals zero (fdfe_main.f90:938-942)."""
    conv = np.zeros((nz, 6))
    idx = np.arange(nz) * nx * ny
    conv[:, 0:3] = sigma[0:3, idx].T
    return conv


def assemble(nx, ny, nz, a, b, c, sigma, ff, edc):
    """fd_assemb + dcfast: returns (csr K, p1, p2) with the reference's entry order."""
    nl = nedges(nx, ny, nz)
    ia = np.zeros(nl + 1, np.int64)
    ja = np.zeros(13 * nl, np.int32)
    km = np.zeros(13 * nl, np.complex128)
    p1 = np.zeros(nl, np.complex128)
    p2 = np.zeros(nl, np.complex128)
    sg = _d(sigma)
    nnz = lib().orc_assemble(nx, ny, nz, _p(_d(a)), _p(_d(b)), _p(_d(c)), _p(sg), ctypes.c_double(ff), _p(_z(edc)),
                             _p(ia, c_int64_p), _p(ja, c_int32_p), _p(km), _p(p1), _p(p2))
    K = sp.csr_matrix((km[:nnz].copy(), ja[:nnz].copy(), ia), shape=(nl, nl))
    return K, p1, p2


def boundary_flags(nx, ny, nz):
    nl = nedges(nx, ny, nz)
    f = np.zeros(nl, np.uint8)
    lib().orc_boundary_flags(nx, ny, nz, f.ctypes.data_as(ctypes.c_void_p))
    return f.astype(bool)


def mesh_coarsen(a, b, c, sigma, k, quirk=True):
    nx, ny, nz = len(a), len(b), len(c)
    asf = 2 ** k
    if nx % asf or ny % asf or nz % asf:
        raise ValueError("mesh_coarsen: sizes not divisible by 2**k")
    cx, cy, cz = nx // asf, ny // asf, nz // asf
    a1, b1, c1 = np.zeros(cx), np.zeros(cy), np.zeros(cz)
    nc = np.zeros((6, cx * cy * cz))
    lib().orc_mesh_coarsen(nx, ny, nz, _p(_d(a)), _p(_d(b)), _p(_d(c)), _p(_d(sigma)), k, int(quirk), _p(a1), _p(b1),
                           _p(c1), _p(nc))
    return a1, b1, c1, nc


def solve_krylov(solver, mesh, K, rhs, x0, eps, itmax, opts: OracleOpts, ilu_band=0):
    """Bicg_stab_p (solver 1) or pgpbicg (solver 3) on the CSR system.  ilu_band is
    idd(2) of the caller, used by the ILU(0) preconditioner (opts.pre = 'I') only."""
    nx, ny, nz, a, b, c, sigma = mesh
    x = _z(x0).copy()
    err = np.zeros(itmax + 1)
    ia = np.ascontiguousarray(K.indptr, dtype=np.int64)
    ja = np.ascontiguousarray(K.indices, dtype=np.int32)
    km = _z(K.data)
    it = lib().orc_solve(solver, nx, ny, nz, _p(_d(a)), _p(_d(b)), _p(_d(c)), _p(_d(sigma)), opts.pre.encode(),
                         int(opts.div_cor), opts.corr_intv, opts.corr_tol, opts.omega, K.shape[0],
                         km.ctypes.data, _p(ia, c_int64_p), _p(ja, c_int32_p), _z(rhs).ctypes.data, x.ctypes.data,
                         eps, itmax, _p(err), ctypes.c_int64(ilu_band))
    return x, int(it), err[:itmax]


def ilu_apply(K, y, band=0):
    """zilu0 + lusol (pre_type = 'I'): x = (LU)^-1 y with the band filter of zilu0
    (band = idd(2); 0 keeps every entry)."""
    ia = np.ascontiguousarray(K.indptr, dtype=np.int64)
    ja = np.ascontiguousarray(K.indices, dtype=np.int32)
    km = _z(K.data)
    x = np.zeros(K.shape[0], np.complex128)
    ierr = lib().orc_ilu_apply(ctypes.c_int64(K.shape[0]), km.ctypes.data_as(ctypes.c_void_p), _p(ia, c_int64_p),
                               _p(ja, c_int32_p), ctypes.c_int64(band), _z(y).ctypes.data_as(ctypes.c_void_p),
                               x.ctypes.data_as(ctypes.c_void_p))
    if ierr:
        raise ZeroDivisionError(f"zilu0: zero pivot in row {ierr}")
    return x


def ssor_apply(K, y, omega=1.0):
    ia = np.ascontiguousarray(K.indptr, dtype=np.int64)
    ja = np.ascontiguousarray(K.indices, dtype=np.int32)
    km = _z(K.data)
    x = np.zeros(K.shape[0], np.complex128)
    lib().orc_ssor_apply(ctypes.c_int64(K.shape[0]), km.ctypes.data_as(ctypes.c_void_p), _p(ia, c_int64_p),
                         _p(ja, c_int32_p), ctypes.c_double(omega), _z(y).ctypes.data_as(ctypes.c_void_p),
                         x.ctypes.data_as(ctypes.c_void_p))
    return x


def div_correc(nx, ny, nz, a, b, c, sigma, x, tol=1e-3):
    x = _z(x).copy()
    it = lib().orc_div_correc(nx, ny, nz, _p(_d(a)), _p(_d(b)), _p(_d(c)), _p(_d(sigma)),
                              x.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(tol))
    return x, it


def divergence(nx, ny, nz, a, b, c, sigma, x):
    np_ = (nx + 1) * (ny + 1) * (nz + 1)
    t = np.zeros(np_, np.complex128)
    lib().orc_divergence(nx, ny, nz, _p(_d(a)), _p(_d(b)), _p(_d(c)), _p(_d(sigma)),
                         _z(x).ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p))
    return t


def extint_v(nx, ny, nz, a1, b1, c1, nair, u0, u1, midpoint_quirk=True):
    nl = nedges(nx, ny, nz)
    u = np.zeros(nl, np.complex128)
    nnan = lib().orc_extint_v(nx, ny, nz, _p(_d(a1)), _p(_d(b1)), _p(_d(c1)), nair, _z(u0).ctypes.data_as(
        ctypes.c_void_p), _z(u1).ctypes.data_as(ctypes.c_void_p), u.ctypes.data_as(ctypes.c_void_p),
        int(midpoint_quirk))
    return u, nnan


def interp(m, nx, ny, nz, a, b, c, nair, u, midpoint_quirk=True):
    """quad_interp_e (m=2) or cubic_interp (m=4) alone; nx.. = output sizes."""
    out = np.zeros(nedges(nx, ny, nz), np.complex128)
    f = lib().orc_quad_interp if m == 2 else lib().orc_cubic_interp
    f(nx, ny, nz, _p(_d(a)), _p(_d(b)), _p(_d(c)), nair, _z(u).ctypes.data_as(ctypes.c_void_p),
      out.ctypes.data_as(ctypes.c_void_p), int(midpoint_quirk))
    return out


def post_process(model: OracleModel, x1, x2, ff, out_type=1, rd=2):
    """post_process + arho_interp2 for one frequency. Returns (out[nrec,4], tip[nrec,4], fields[nrec,10])."""
    nrec = model.recv.shape[0]
    recv = np.asfortranarray(model.recv, dtype=np.float64).ravel(order="F").copy()
    out = np.zeros((nrec, 4))
    tip = np.zeros((nrec, 4))
    fld = np.zeros((nrec, 10), np.complex128)
    rc = lib().orc_post_process(model.nx, model.ny, model.nz, model.nair, _p(_d(model.a)), _p(_d(model.b)),
                                _p(_d(model.c)), ctypes.c_double(ff), _z(x1).ctypes.data_as(ctypes.c_void_p),
                                _z(x2).ctypes.data_as(ctypes.c_void_p), nrec, _p(recv), out_type, rd, _p(out),
                                _p(tip), fld.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise ValueError(f"receiver {-rc} lies outside the interpolation stencil")
    return out, tip, fld


def receiver_planes(model: OracleModel, abr, topo, corrected=False):
    """The receiver plane of every surface column with topography (post_process,
    fdfe_main.f90:604-616): inside the window abr = (i1, i2, j1, j2, k1, k2) (1-based) a
    column's plane is the first cell k in k1..k2 whose centre ccz(k) lies at or below the
    surface -topo (topo = elevation, positive up; ccz of the reference, :593-595), outside it
    nair.  The reference takes that cell's lower node plane (m = k) and the vertical step
    c(nair+1) for every column; corrected = True takes its upper plane (m = k - 1, the top of
    the first earth cell, which is nair on flat ground) and the cell below that plane
    (c(m+1)).  A column with no such cell keeps nair.  Returns (mcol[ny*nx], czcol[ny*nx])."""
    nx, ny, nair = model.nx, model.ny, model.nair
    c = _d(model.c)
    ccz = -c[:nair].sum() + np.cumsum(c) - c / 2
    i1, i2, j1, j2, k1, k2 = (int(v) for v in abr)
    mcol = np.full(nx * ny, nair, np.int32)
    czcol = np.full(nx * ny, c[nair])
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            if not (i1 <= i <= i2 and j1 <= j <= j2):
                continue
            t = topo[(j - j1) * (i2 - i1 + 1) + i - i1]
            for k in range(k1, k2 + 1):
                if ccz[k - 1] >= -t:
                    m = k - 1 if corrected else k
                    mcol[(j - 1) * nx + i - 1] = m
                    if corrected:
                        czcol[(j - 1) * nx + i - 1] = c[m]
                    break
    return mcol, czcol


def post_process_topo(model: OracleModel, x1, x2, ff, mcol, czcol, out_type=1, rd=2):
    """post_process with a receiver plane per column (receiver_planes)."""
    nrec = model.recv.shape[0]
    recv = np.asfortranarray(model.recv, dtype=np.float64).ravel(order="F").copy()
    out = np.zeros((nrec, 4))
    tip = np.zeros((nrec, 4))
    fld = np.zeros((nrec, 10), np.complex128)
    mc = np.ascontiguousarray(mcol, np.int32)
    cz = _d(czcol)
    rc = lib().orc_post_process_topo(model.nx, model.ny, model.nz, model.nair, _p(_d(model.a)), _p(_d(model.b)),
                                     _p(_d(model.c)), ctypes.c_double(ff), _z(x1).ctypes.data_as(ctypes.c_void_p),
                                     _z(x2).ctypes.data_as(ctypes.c_void_p), nrec, _p(recv), out_type, rd, _p(out),
                                     _p(tip), fld.ctypes.data_as(ctypes.c_void_p),
                                     mc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _p(cz))
    if rc != 0:
        raise ValueError(f"receiver {-rc} lies outside the interpolation stencil")
    return out, tip, fld


# --------------------------------------------------------------------------
# Orchestration (fdfe_main.f90)
# --------------------------------------------------------------------------
@dataclass
class LevelInfo:
    level: int
    nx: int
    ny: int
    nz: int
    iters: list = field(default_factory=list)  # [xy, yx]
    direct: bool = False


def doublemode_nor(nx, ny, nz, a, b, c, sigma, ff, mid, slv, tol, opts: OracleOpts, x0=None):
    """doublemode_nor (fdfe_main.f90:892-1063): one mesh, both polarisations."""
    conv = column_conv(sigma, nx, ny, nz)
    edc, _, _ = mt1d_anl(ff, conv, c)
    K, p1, p2 = assemble(nx, ny, nz, a, b, c, sigma, ff, edc)
    mesh = (nx, ny, nz, a, b, c, sigma)
    info = LevelInfo(0, nx, ny, nz, direct=mid in (1, 2))
    if mid in (1, 2):
        if opts.coarse_solver == "converged":
            om = OracleModel(nx, ny, nz, 0, a, b, c, sigma, np.array([ff]), np.zeros((1, 3)))
            u1, u2, _, _, _ = converged_solve(om, ff)
            return u1, u2, info
        lu = splu(K.tocsc())
        u1 = lu.solve(p1)
        u2 = lu.solve(p2)
        return u1, u2, info
    maxit = opts.maxit_plain
    nl = K.shape[0]
    # idd(2) = nl (fdfe_main.f90:994): the ILU(0) keeps every entry
    u1, it1, _ = solve_krylov(slv if slv in (1, 3) else 1, mesh, K, p1, np.zeros(nl) if x0 is None else x0[0],
                              tol, maxit, opts, nl)
    u2, it2, _ = solve_krylov(slv if slv in (1, 3) else 1, mesh, K, p2, np.zeros(nl) if x0 is None else x0[1],
                              tol, maxit, opts, nl)
    info.iters = [it1, it2]
    return u1, u2, info


def doublemode_acc(model: OracleModel, ff, opts: OracleOpts, n_grid=None, eps=None, pols=(0, 1)):
    """doublemode_acc (fdfe_main.f90:1258-1563) with u1u2 (:1228-1256).  `pols` selects the
    polarisations whose finer levels are solved (both by default, as the reference does; the
    other's solution is returned as zeros), so that the two can run in separate processes."""
    N = model.level if n_grid is None else n_grid
    tol = (model.eps if eps is None else eps) * 10.0 ** (-N + 1)
    a, b, c, sigma = model.a, model.b, model.c, model.sigma
    infos = []
    # u1u2: levels 1 and 2 solved directly
    a1, b1, c1, s1 = mesh_coarsen(a, b, c, sigma, N - 1, opts.coarsen_quirk)
    u01, u02, inf = doublemode_nor(len(a1), len(b1), len(c1), a1, b1, c1, s1, ff, 1, model.solver, tol, opts)
    inf.level = 1
    infos.append(inf)
    a1, b1, c1, s1 = mesh_coarsen(a, b, c, sigma, N - 2, opts.coarsen_quirk)
    u11, u12, inf = doublemode_nor(len(a1), len(b1), len(c1), a1, b1, c1, s1, ff, 2, model.solver, tol, opts)
    inf.level = 2
    infos.append(inf)
    tol = tol * 10
    for i in range(3, N + 1):
        tol = tol * 10
        if i != N:
            a1, b1, c1, sf = mesh_coarsen(a, b, c, sigma, N - i, opts.coarsen_quirk)
        else:
            a1, b1, c1, sf = a, b, c, sigma
        nx, ny, nz = len(a1), len(b1), len(c1)
        nair_l = model.nair // 2 ** (N - i)
        u21, _ = extint_v(nx, ny, nz, a1, b1, c1, nair_l, u01, u11, opts.midpoint_quirk)
        u22, _ = extint_v(nx, ny, nz, a1, b1, c1, nair_l, u02, u12, opts.midpoint_quirk)
        conv = column_conv(sf, nx, ny, nz)
        edc, _, _ = mt1d_anl(ff, conv, c1)
        K, p1, p2 = assemble(nx, ny, nz, a1, b1, c1, sf, ff, edc)
        if np.isnan(np.abs(p1)).any():
            raise FloatingPointError("NaN value found in the RHS(p1)")
        mesh = (nx, ny, nz, a1, b1, c1, sf)
        slv = model.solver if model.solver in (1, 3) else 1
        band = (nx + 1) * (ny + 1) * (nz + 1)  # idd(2) = np (fdfe_main.f90:1413)
        x1, it1 = (solve_krylov(slv, mesh, K, p1, u21, tol, opts.maxit_level, opts, band)[:2] if 0 in pols
                   else (np.zeros_like(p1), 0))
        x2, it2 = (solve_krylov(slv, mesh, K, p2, u22, tol, opts.maxit_level, opts, band)[:2] if 1 in pols
                   else (np.zeros_like(p2), 0))
        infos.append(LevelInfo(i, nx, ny, nz, [it1, it2]))
        u01, u02, u11, u12 = u11, u12, x1, x2
    return u11, u12, infos


def fwd_solver(model: OracleModel, opts: OracleOpts | None = None, freqs=None):
    """fwd_solver (fdfe_main.f90:1565-1594): returns ex[nf, 2, nl] and per-frequency infos."""
    opts = opts or OracleOpts()
    freqs = model.freq if freqs is None else freqs
    nl = nedges(model.nx, model.ny, model.nz)
    ex = np.zeros((len(freqs), 2, nl), np.complex128)
    infos = []
    for k, ff in enumerate(freqs):
        if not opts.excmg:
            u1, u2, inf = doublemode_nor(model.nx, model.ny, model.nz, model.a, model.b, model.c, model.sigma, ff, 0,
                                         model.solver, model.eps, opts)
            infos.append([inf])
        else:
            u1, u2, inf = doublemode_acc(model, ff, opts)
            infos.append(inf)
        ex[k, 0] = u1
        ex[k, 1] = u2
    return ex, infos


def impedances(model: OracleModel, ex, out_type=1, rd=2, freqs=None):
    """post_process over all frequencies: results[nf, nrec, 4]."""
    freqs = model.freq if freqs is None else freqs
    res = np.zeros((len(freqs), model.recv.shape[0], 4))
    for k, ff in enumerate(freqs):
        res[k], _, _ = post_process(model, ex[k, 0], ex[k, 1], ff, out_type, rd)
    return res


def direct_solve(model: OracleModel, ff):
    """Exact (SuperLU) solution of the fine-mesh system for both polarisations."""
    conv = column_conv(model.sigma, model.nx, model.ny, model.nz)
    edc, _, _ = mt1d_anl(ff, conv, model.c)
    K, p1, p2 = assemble(model.nx, model.ny, model.nz, model.a, model.b, model.c, model.sigma, ff, edc)
    lu = splu(K.tocsc())
    return lu.solve(p1), lu.solve(p2), K, p1, p2


# --------------------------------------------------------------------------- gradient-space correction
def node_gradient(nx, ny, nz, a, b, c):
    """Nodal gradient G (edges x interior nodes): edge value (phi_end - phi_start)/length,
    boundary nodes held at zero.  Edge order as fd_assemb (fdfe_main.f90:261,310,358)."""
    a, b, c = _d(a), _d(b), _d(c)
    nid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i  # noqa: E731
    rows, cols, vals = [], [], []
    off = 0
    for o, (di, dj, dk, h) in enumerate(((1, 0, 0, a), (0, 1, 0, b), (0, 0, 1, c))):
        k, j, i = np.meshgrid(np.arange(nz + 1 - dk), np.arange(ny + 1 - dj), np.arange(nx + 1 - di), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        e = off + np.arange(i.size)
        ln = h[(i, j, k)[o]]
        rows += [e, e]
        cols += [nid(i, j, k), nid(i + di, j + dj, k + dk)]
        vals += [-1.0 / ln, 1.0 / ln]
        off += i.size
    npn = (nx + 1) * (ny + 1) * (nz + 1)
    G = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(off, npn))
    n = np.arange(npn)
    i, j, k = n % (nx + 1), (n // (nx + 1)) % (ny + 1), n // ((nx + 1) * (ny + 1))
    interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
    return G[:, interior].tocsr()


def edge_dual_volumes(nx, ny, nz, a, b, c):
    """Dual volume of every edge: length x the two transverse half-spacing sums (zero on the
    outer faces, whose rows are identity rows after dcfast)."""
    def half(h):
        d = np.zeros(len(h) + 1)
        d[1:-1] = (h[:-1] + h[1:]) / 2
        return d
    a, b, c = _d(a), _d(b), _d(c)
    ha, hb, hc = half(a), half(b), half(c)
    vx = a[None, None, :] * hb[None, :, None] * hc[:, None, None]
    vy = ha[None, None, :] * b[None, :, None] * hc[:, None, None]
    vz = ha[None, None, :] * hb[None, :, None] * c[:, None, None]
    return np.concatenate([vx.ravel(), vy.ravel(), vz.ravel()])


def grad_correct(nx, ny, nz, a, b, c, sigma, ff, rhs, x):
    """x + G phi with (G^T V Ms G) phi = G^T V (rhs - K x) / (-i w mu), solved exactly.

    No counterpart in the reference (its div_correc removes the divergence of x alone);
    this is the restatement of the library's consistent correction that its tests compare with.
    Ms, the conductivity part of the assembled rows, is recovered from two assemblies
    (K(w) = C - i w mu Ms)."""
    conv = column_conv(sigma, nx, ny, nz)
    edc, _, _ = mt1d_anl(ff, conv, c)
    K1, _, _ = assemble(nx, ny, nz, a, b, c, sigma, ff, edc)
    K2, _, _ = assemble(nx, ny, nz, a, b, c, sigma, 2 * ff, edc)
    mu = 4e-7 * np.pi
    w1, w2 = 2 * np.pi * ff * mu, 4 * np.pi * ff * mu
    Ms = ((K1 - K2) / (-1j * (w1 - w2))).real.tocsr()
    G = node_gradient(nx, ny, nz, a, b, c)
    V = sp.diags(edge_dual_volumes(nx, ny, nz, a, b, c))
    N = (G.T @ V @ Ms @ G).tocsc()
    r = _z(rhs) - K1 @ _z(x)
    t = G.T @ (V @ r) / (-1j * w1)
    lu = splu(N)
    phi = lu.solve(t.real) + 1j * lu.solve(t.imag)
    return _z(x) + G @ phi


# --------------------------------------------------------------------------- adjoint gradient
# No counterpart in the reference (it has no inversion path).  The oracle's value of the
# library's misfit gradient, computed independently of the library's route: the
# transposed system is solved directly (no use of the dual-volume symmetry), the
# operator derivative comes from re-assembling fd_assemb + dcfast with one cell
# perturbed (the rows are linear in sigma), and the derivative of the impedances
# with respect to the edge values from probing post_process (linear in the
# fields) and a fourth-order difference of Z(E, H) (holomorphic).
def _zfun(f):
    """(Zxy, Zyx) from the receiver fields f[10] = (Ex, Ey, Hx, Hy, Hz) x 2 polarisations."""
    ex1, ey1, hx1, hy1 = f[0], f[1], f[2], f[3]
    ex2, ey2, hx2, hy2 = f[5], f[6], f[7], f[8]
    det = hx1 * hy2 - hx2 * hy1
    return np.array([(ex2 * hx1 - ex1 * hx2) / det, (ey1 * hy2 - ey2 * hy1) / det])


def _dz_dfields(f):
    """d(Zxy, Zyx)/d f (2 x 10, holomorphic derivative) by a fourth-order central difference."""
    out = np.zeros((2, 10), np.complex128)
    for q in range(10):
        h = 1e-4 * max(abs(f[q]), np.abs(f).max() * 1e-3)
        e = np.zeros(10, np.complex128)
        e[q] = h
        out[:, q] = (-_zfun(f + 2 * e) + 8 * _zfun(f + e) - 8 * _zfun(f - e) + _zfun(f - 2 * e)) / (12 * h)
    return out


def _surface_edges(nx, ny, nz, nair):
    """Edge indices post_process reads: Ex and Ey on node planes nair, nair+1, Ez of layer nair."""
    xnl = nx * (ny + 1) * (nz + 1)
    ynl = (nx + 1) * ny * (nz + 1)
    pex, pey, pez = nx * (ny + 1), (nx + 1) * ny, (nx + 1) * (ny + 1)
    return np.concatenate([nair * pex + np.arange(2 * pex), xnl + nair * pey + np.arange(2 * pey),
                           xnl + ynl + nair * pez + np.arange(pez)])


def receiver_jacobian(model: OracleModel, ff, rd=2):
    """J[nrec, 5, n_surface] with fields(pol) = J x_pol on the surface edges, and those edge indices."""
    idx = _surface_edges(model.nx, model.ny, model.nz, model.nair)
    nl = nedges(model.nx, model.ny, model.nz)
    nrec = model.recv.shape[0]
    J = np.zeros((nrec, 5, idx.size), np.complex128)
    x = np.zeros(nl, np.complex128)
    zero = np.zeros(nl, np.complex128)
    for t, e in enumerate(idx):
        x[e] = 1.0
        _, _, fld = post_process(model, x, zero, ff, 1, rd)
        J[:, :, t] = fld[:, 0:5]
        x[e] = 0.0
    return J, idx


def misfit(model: OracleModel, zobs, wts=None, rd=2):
    """sum_f,r wxy |Zxy - dxy|^2 + wyx |Zyx - dyx|^2 of the exact discrete solution."""
    ex = np.zeros((model.freq.size, 2, nedges(model.nx, model.ny, model.nz)), np.complex128)
    for k, ff in enumerate(model.freq):
        u1, u2, _, _, _ = direct_solve(model, ff)
        ex[k, 0], ex[k, 1] = u1, u2
    z = impedances(model, ex, out_type=1, rd=rd)
    zc = z[..., 0::2] + 1j * z[..., 1::2]
    dc = zobs[..., 0::2] + 1j * zobs[..., 1::2]
    w = np.ones(zc.shape) if wts is None else wts
    return float((w * np.abs(zc - dc) ** 2).sum())


def misfit_grad_cells(model: OracleModel, zobs, cells, comps, wts=None, rd=2):
    """(misfit, d misfit / d sigma[comp, cell] for the listed (cell, comp) pairs, and per
    frequency the exact forward fields x[2, nl] and adjoint fields mu[2, nl] with
    K_II mu = V^-1 g_I, mu = 0 on the Dirichlet edges -- the quantities the library's
    per-cell contraction uses)."""
    nx, ny, nz = model.nx, model.ny, model.nz
    nrec = model.recv.shape[0]
    V = edge_dual_volumes(nx, ny, nz, model.a, model.b, model.c)
    grad = np.zeros(len(cells))
    phi = 0.0
    xs, mus = [], []
    conv = column_conv(model.sigma, nx, ny, nz)
    for k, ff in enumerate(model.freq):
        edc, _, _ = mt1d_anl(ff, conv, model.c)
        K, p1, p2 = assemble(nx, ny, nz, model.a, model.b, model.c, model.sigma, ff, edc)
        lu = splu(K.tocsc())
        x = np.stack([lu.solve(p1), lu.solve(p2)])
        _, _, fld = post_process(model, x[0], x[1], ff, 1, rd)
        J, idx = receiver_jacobian(model, ff, rd)
        g = np.zeros((2, x.shape[1]), np.complex128)
        for r in range(nrec):
            z = _zfun(fld[r])
            d = zobs[k, r, 0::2] + 1j * zobs[k, r, 1::2]
            w = np.ones(2) if wts is None else wts[k, r]
            phi += float((w * np.abs(z - d) ** 2).sum())
            cf = (w * np.conj(z - d)) @ _dz_dfields(fld[r])  # d phi / d fields[10]
            for p in range(2):
                g[p, idx] += cf[5 * p:5 * p + 5] @ J[r]
        luT = splu(K.T.tocsc())
        lam = np.stack([luT.solve(g[0]), luT.solve(g[1])])
        interior = V > 0
        mu = np.zeros_like(lam)
        mu[:, interior] = lam[:, interior] / V[interior]
        xs.append(x)
        mus.append(mu)
        for t, (cell, q) in enumerate(zip(cells, comps)):
            sg = model.sigma.copy()
            dl = max(abs(sg[q, cell]), 1e-3)
            sg[q, cell] += dl
            K2, q1, q2 = assemble(nx, ny, nz, model.a, model.b, model.c, sg, ff, edc)
            dK = (K2 - K) / dl
            dp = (np.stack([q1, q2]) - np.stack([p1, p2])) / dl
            for p in range(2):
                grad[t] += -2.0 * np.real(lam[p] @ (dK @ x[p] - dp[p]))
    return phi, grad, xs, mus


def sigma_grad_local(nx, ny, nz, a, b, c, wm, xs, mus):
    """Per-cell contraction restated in numpy: d misfit / d sigma[6, ncell] from forward
    fields xs[s] and adjoint fields mus[s] (zero on the Dirichlet edges) of systems with
    w mu0 = wm[s]: -2 sum_s wm_s Im(sum_ee' (V dM/dsigma)_ee' mu_e x_e'), where V dM/dsigma
    is vol/4 between an edge and itself for the diagonal components and vol/8 between the
    differently oriented edges of one face level for the off-diagonal ones."""
    a, b, c = _d(a), _d(b), _d(c)
    xnl = nx * (ny + 1) * (nz + 1)
    ynl = (nx + 1) * ny * (nz + 1)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    vol = a[i] * b[j] * c[k]
    EX = lambda dj, dk: ((k + dk) * (ny + 1) + j + dj) * nx + i  # noqa: E731
    EY = lambda di, dk: xnl + ((k + dk) * ny + j) * (nx + 1) + i + di  # noqa: E731
    EZ = lambda di, dj: xnl + ynl + (k * (ny + 1) + j + dj) * (nx + 1) + i + di  # noqa: E731
    out = np.zeros((6, nx * ny * nz))
    for s in range(len(wm)):
        x, mu = xs[s], mus[s]
        S = np.zeros((6, i.size), np.complex128)
        for u in (0, 1):
            for v in (0, 1):
                S[0] += mu[EX(u, v)] * x[EX(u, v)]
                S[1] += mu[EY(u, v)] * x[EY(u, v)]
                S[2] += mu[EZ(u, v)] * x[EZ(u, v)]
        for v in (0, 1):
            S[3] += (mu[EX(0, v)] + mu[EX(1, v)]) * (x[EY(0, v)] + x[EY(1, v)]) + \
                    (mu[EY(0, v)] + mu[EY(1, v)]) * (x[EX(0, v)] + x[EX(1, v)])
        for u in (0, 1):
            S[4] += (mu[EX(u, 0)] + mu[EX(u, 1)]) * (x[EZ(0, u)] + x[EZ(1, u)]) + \
                    (mu[EZ(0, u)] + mu[EZ(1, u)]) * (x[EX(u, 0)] + x[EX(u, 1)])
            S[5] += (mu[EY(u, 0)] + mu[EY(u, 1)]) * (x[EZ(u, 0)] + x[EZ(u, 1)]) + \
                    (mu[EZ(u, 0)] + mu[EZ(u, 1)]) * (x[EY(u, 0)] + x[EY(u, 1)])
        out += -2.0 * wm[s] * S.imag
    out[:3] *= vol / 4
    out[3:] *= vol / 8
    return out


# --------------------------------------------------------------------------- converged solutions of large meshes
# The exact discrete answer (the solution of the assembled fd_assemb + dcfast
# system) on meshes too large for SuperLU.  No counterpart in the reference:
# this is the oracle's own solver, written independently of the library
# (SciPy sparse matrices, a Gauss-Seidel smoother in C, a direct solve on the
# coarsest mesh), and it only has to deliver the discrete solution to a
# relative residual of ~1e-15, which it checks with the assembled matrix.
# Method: BiCGStab preconditioned by a geometric multigrid V-cycle on the
# 2x-coarsened meshes (rediscretised with the volume-averaged conductivity
# of mesh_coarsen without its index shift), lowest-order edge interpolation
# and its dual-volume transpose, symmetric Gauss-Seidel plus a nodal
# (gradient-space) Gauss-Seidel step as smoother (Hiptmair 1998).
def _sgs(K, b, x):
    x = _z(x).copy()
    ia = np.ascontiguousarray(K.indptr, dtype=np.int64)
    ja = np.ascontiguousarray(K.indices, dtype=np.int32)
    km = _z(K.data)
    lib().orc_sgs(ctypes.c_int64(K.shape[0]), km.ctypes.data_as(ctypes.c_void_p), _p(ia, c_int64_p), _p(ja, c_int32_p),
                  _z(b).ctypes.data_as(ctypes.c_void_p), x.ctypes.data_as(ctypes.c_void_p))
    return x


def _node_terms(h):
    """Fine node m -> (lower coarse node, its weight, upper coarse node, its weight); fine node
    2I is coarse node I, an odd node lies between two at fraction t = h(m-1)/(h(m-1)+h(m))."""
    n = len(h) + 1
    m = np.arange(n)
    lo = m // 2
    t = np.zeros(n)
    odd = m % 2 == 1
    t[odd] = h[m[odd] - 1] / (h[m[odd] - 1] + h[m[odd]])
    return lo, 1 - t, np.minimum(lo + 1, (n - 1) // 2), t


def edge_prolongation(a, b, c):
    """Lowest-order edge interpolation from the 2x-coarsened mesh to mesh (a, b, c): a fine
    edge takes the parallel coarse edges with weight 1 along it and the linear interpolation
    weights of its transverse node positions."""
    a, b, c = _d(a), _d(b), _d(c)
    nx, ny, nz = len(a), len(b), len(c)
    cx, cy, cz = nx // 2, ny // 2, nz // 2
    terms = (_node_terms(a), _node_terms(b), _node_terms(c))
    cxnl, cynl = cx * (cy + 1) * (cz + 1), (cx + 1) * cy * (cz + 1)
    rows, cols, vals = [], [], []
    off = 0
    for o in range(3):
        sx, sy, sz = nx + (o != 0), ny + (o != 1), nz + (o != 2)
        k, j, i = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
        ijk = (i.ravel(), j.ravel(), k.ravel())
        e = off + np.arange(ijk[0].size)
        off += ijk[0].size
        ax = [q for q in range(3) if q != o]
        for pa in (0, 1):
            for pb in (0, 1):
                ida = terms[ax[0]][2 * pa][ijk[ax[0]]]
                wa = terms[ax[0]][2 * pa + 1][ijk[ax[0]]]
                idb = terms[ax[1]][2 * pb][ijk[ax[1]]]
                wb = terms[ax[1]][2 * pb + 1][ijk[ax[1]]]
                w = wa * wb
                keep = w != 0
                idx = [None, None, None]
                idx[o] = ijk[o][keep] // 2
                idx[ax[0]] = ida[keep]
                idx[ax[1]] = idb[keep]
                I, J, Kk = idx
                if o == 0:
                    col = (Kk * (cy + 1) + J) * cx + I
                elif o == 1:
                    col = cxnl + (Kk * cy + J) * (cx + 1) + I
                else:
                    col = cxnl + cynl + (Kk * (cy + 1) + J) * (cx + 1) + I
                rows.append(e[keep])
                cols.append(col)
                vals.append(w[keep])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(nedges(nx, ny, nz), nedges(cx, cy, cz)))


def _boundary_edges(nx, ny, nz):
    f = np.zeros(nedges(nx, ny, nz), np.uint8)
    lib().orc_boundary_flags(nx, ny, nz, f.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    return f.astype(bool)


class _MGLevel:
    pass


def _mg_hierarchy(model: OracleModel, ff, nlev):
    levs = []
    for l in range(nlev):
        L = _MGLevel()
        if l == 0:
            a, b, c, s = _d(model.a), _d(model.b), _d(model.c), _d(model.sigma)
        else:
            a, b, c, s = mesh_coarsen(model.a, model.b, model.c, model.sigma, l, quirk=False)
        nx, ny, nz = len(a), len(b), len(c)
        L.a, L.b, L.c = a, b, c
        edc, _, _ = mt1d_anl(ff, column_conv(s, nx, ny, nz), c)
        L.K, L.p1, L.p2 = assemble(nx, ny, nz, a, b, c, s, ff, edc)
        L.V = edge_dual_volumes(nx, ny, nz, a, b, c)
        L.bnd = _boundary_edges(nx, ny, nz)
        L.G = node_gradient(nx, ny, nz, a, b, c).tocsr()
        L.GT = L.G.T.tocsr()
        L.Kn = (L.GT @ sp.diags(L.V) @ L.K @ L.G).tocsr()
        if l > 0:
            levs[-1].P = edge_prolongation(levs[-1].a, levs[-1].b, levs[-1].c)
            levs[-1].PT = levs[-1].P.T.tocsr()
        levs.append(L)
    levs[-1].lu = splu(levs[-1].K.tocsc())
    return levs


def _mg_smooth(L, b, x):
    x = _sgs(L.K, b, x)
    r = b - L.K @ x
    phi = _sgs(L.Kn, L.GT @ (L.V * r), np.zeros(L.Kn.shape[0], np.complex128))
    return x + L.G @ phi


def _vcycle(levs, l, b):
    L = levs[l]
    if l == len(levs) - 1:
        return L.lu.solve(b)
    x = _mg_smooth(L, b, np.zeros_like(b))
    C = levs[l + 1]
    rc = L.PT @ (L.V * (b - L.K @ x))
    rc = np.where(C.bnd, 0, rc / np.where(C.V > 0, C.V, 1))
    x = x + L.P @ _vcycle(levs, l + 1, rc)
    return _mg_smooth(L, b, x)


def converged_solve(model: OracleModel, ff, tol=1e-15, nlev=None, maxit=200):
    """Solutions of both polarisations of frequency ff to relative residual `tol`
    (||p - K x|| / ||p|| with the assembled K); returns (x1, x2, relres1, relres2, iters)."""
    from scipy.sparse.linalg import LinearOperator, bicgstab
    if nlev is None:
        nlev = 1
        while all(n % 2 ** nlev == 0 and n // 2 ** nlev >= 4 for n in (model.nx, model.ny, model.nz)):
            nlev += 1
    levs = _mg_hierarchy(model, ff, nlev)
    F = levs[0]
    M = LinearOperator(F.K.shape, lambda v: _vcycle(levs, 0, _z(v)), dtype=np.complex128)
    out, rr, its = [], [], []
    for p in (F.p1, F.p2):
        cnt = [0]
        x, _ = bicgstab(F.K, p, rtol=tol, atol=0.0, maxiter=maxit, M=M,
                        callback=lambda xk: cnt.__setitem__(0, cnt[0] + 1))
        rel = float(np.linalg.norm(p - F.K @ x) / np.linalg.norm(p))
        # the recurrence residual may claim convergence early: restart from x until the true one passes
        rounds = 0
        while rel > tol and rounds < 5:
            d, _ = bicgstab(F.K, p - F.K @ x, rtol=tol / max(rel, tol), atol=0.0, maxiter=maxit, M=M)
            x = x + d
            rel = float(np.linalg.norm(p - F.K @ x) / np.linalg.norm(p))
            rounds += 1
        out.append(x)
        rr.append(rel)
        its.append(cnt[0])
    return out[0], out[1], rr[0], rr[1], its


# --------------------------------------------------------------------------- the GPU's edge multigrid V-cycle
# Restatement of the V-cycle of precond = 'G' (sfdx_mgkern.cuh, emg_* in
# sfdx_krylov.cuh) on the assembled matrices, the oracle of sfdx_vcycle_apply.
# No reference counterpart (pre_type offers SSOR, Jacobi and ILU(0) only).
# Per level: x = S^-1 b with the multi-colour symmetric Gauss-Seidel of the
# Krylov preconditioner ('M', colours Ex (j+k)&1, Ey (i+k)&1, Ez (i+j)&1,
# orientation-major), a nodal step (q = b + i w mu Ms x on interior edges,
# phi = omega (G^T V q) / diag(G^T V K G), x += G phi), then the residual
# restricted by V_c^-1 P^T V_f, the coarser V-cycle from zero, x += P x_c,
# and one smoothing step (r = b - K x, x += S^-1 r, nodal step); the coarsest
# level takes `coarse_sweeps` smoothing steps.  Coarse meshes: mesh_coarsen
# without its index shift.
def _mc_colour_rows(nx, ny, nz):
    col = np.zeros(nedges(nx, ny, nz), np.int8)
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx), indexing="ij")
    xnl = i.size
    col[:xnl] = ((j + k) & 1).ravel()
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny), np.arange(nx + 1), indexing="ij")
    ynl = i.size
    col[xnl:xnl + ynl] = 2 + ((i + k) & 1).ravel()
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    col[xnl + ynl:] = 4 + ((i + j) & 1).ravel()
    return [np.flatnonzero(col == c) for c in range(6)], col


def _mc_sgs(L, b):
    """x = (D+U)^-1 D (D+L)^-1 b (the multi-colour SSOR with omega = 1), vectorised per colour."""
    x = np.zeros_like(b)
    for c in range(6):
        R = L.rows[c]
        x[R] = (b[R] - L.K[R] @ x) / L.D[R]  # later colours and the own colour are still zero
    for c in range(4, -1, -1):
        R = L.rows[c]
        later = np.where(L.col > c, x, 0)
        x[R] = x[R] - (L.K[R] @ later) / L.D[R]
    return x


def _gpu_nodal(L, b, x, omega):
    # phi = omega D^-1 G^T V q with D = diag(G^T V K G) = -i w mu N_nn; the GPU keeps 1/N_nn in
    # float (nodal_setup), and so does this restatement
    q = b + 1j * L.wm * (L.Ms @ x)
    q[L.bnd] = 0
    return x + L.G @ (omega * 1j * (L.dinv32 / L.wm) * (L.GT @ (L.V * q)))


def _gpu_smooth(L, b, x, omega):
    r = b - L.K @ x
    return _gpu_nodal(L, b, x + _mc_sgs(L, r), omega)


def _gpu_vcycle(levs, l, b, omega, coarse_sweeps):
    L = levs[l]
    x = _gpu_nodal(L, b, _mc_sgs(L, b), omega)
    if l == len(levs) - 1:
        for _ in range(coarse_sweeps - 1):
            x = _gpu_smooth(L, b, x, omega)
        return x
    C = levs[l + 1]
    rc = L.PT @ (L.V * (b - L.K @ x))
    rc = np.where(C.bnd, 0, rc / np.where(C.V > 0, C.V, 1))
    x = x + L.P @ _gpu_vcycle(levs, l + 1, rc, omega, coarse_sweeps)
    return _gpu_smooth(L, b, x, omega)


def gpu_vcycle(model: OracleModel, ff, y, nlev=3, omega=0.7, coarse_sweeps=4):
    """x = M^-1 y for one system of frequency ff with the V-cycle above (levels: the model's
    mesh and nlev - 1 coarser ones)."""
    levs = _mg_hierarchy(model, ff, nlev)
    wm = 2 * np.pi * ff * 4e-7 * np.pi
    for l, L in enumerate(levs):
        nx, ny, nz = len(L.a), len(L.b), len(L.c)
        s = _d(model.sigma) if l == 0 else mesh_coarsen(model.a, model.b, model.c, model.sigma, l, quirk=False)[3]
        # the mass part from a second assembly at twice the frequency: K(f) = C - i w mu Ms
        edc2, _, _ = mt1d_anl(2 * ff, column_conv(s, nx, ny, nz), L.c)
        K2, _, _ = assemble(nx, ny, nz, L.a, L.b, L.c, s, 2 * ff, edc2)
        L.K = L.K.tocsr()
        L.Ms = ((K2 - L.K) / (-1j * wm)).tocsr()
        L.wm = wm
        L.D = L.K.diagonal()
        L.rows, L.col = _mc_colour_rows(nx, ny, nz)
        # N = G^T V Ms G directly (G^T V K G / (-i w mu) carries the rounding of C G = 0 divided by
        # w mu); N_nn rounded to float, then 1.f / N, as the GPU does
        nd = (L.GT @ (sp.diags(L.V) @ (L.Ms.real @ L.G))).diagonal()
        n32 = nd.astype(np.float32)
        L.dinv32 = (np.float32(1.0) / n32).astype(np.float64)
    return _gpu_vcycle(levs, 0, _z(y), omega, coarse_sweeps)


# --------------------------------------------------------------------------- complex64 Krylov on a split V-cycle
# Numerical premise of a complex64 Krylov iteration under the edge multigrid
# (not built on the GPU yet): storage of every vector in complex64 is emulated
# by rounding after each step.  The V-cycle above, run with that storage, either
# adds its nodal corrections G phi into x (split=False) or carries them as a nodal
# potential psi beside x (split=True): residuals then take A(x + G psi) =
# K x - i w mu Ms G psi (C G = 0), and the prolongation moves psi by the
# trilinear nodal interpolation, which commutes with G.  BiCGStab runs on complex64
# vectors with an FP64 iterate and an FP64 residual every 8 iterations.
def _c64(v):
    return v.astype(np.complex64).astype(np.complex128)


def _node_interp_1d(h):
    lo, wlo, hi, whi = _node_terms(_d(h))
    n = len(h) + 1
    return sp.csr_matrix((np.concatenate([wlo, whi]), (np.tile(np.arange(n), 2), np.concatenate([lo, hi]))),
                         shape=(n, len(h) // 2 + 1))


def _interior_nodes(nx, ny, nz):
    n = np.arange((nx + 1) * (ny + 1) * (nz + 1))
    i, j, k = n % (nx + 1), (n // (nx + 1)) % (ny + 1), n // ((nx + 1) * (ny + 1))
    return (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)


def _split_levels(model, ff, nlev):
    levs = _mg_hierarchy(model, ff, nlev)
    wm = 2 * np.pi * ff * 4e-7 * np.pi
    for l, L in enumerate(levs):
        nx, ny, nz = len(L.a), len(L.b), len(L.c)
        s = _d(model.sigma) if l == 0 else mesh_coarsen(model.a, model.b, model.c, model.sigma, l, quirk=False)[3]
        edc2, _, _ = mt1d_anl(2 * ff, column_conv(s, nx, ny, nz), L.c)
        K2, _, _ = assemble(nx, ny, nz, L.a, L.b, L.c, s, 2 * ff, edc2)
        L.K = L.K.tocsr()
        L.Ms = ((K2 - L.K) / (-1j * wm)).tocsr()
        L.wm = wm
        L.inner = _interior_nodes(nx, ny, nz)
        if l > 0:
            F = levs[l - 1]
            Pn = sp.kron(_node_interp_1d(F.c), sp.kron(_node_interp_1d(F.b), _node_interp_1d(F.a))).tocsr()
            F.Pn = Pn[F.inner][:, L.inner].tocsr()
    return levs


def _split_smooth(L, b, x, psi, split):
    r = b - L.K @ x + 1j * L.wm * (L.Ms @ (L.G @ psi))
    x = _c64(x + _sgs(L.K, r, np.zeros_like(r)))
    r = b - L.K @ x + 1j * L.wm * (L.Ms @ (L.G @ psi))
    phi = _sgs(L.Kn, L.GT @ (L.V * r), np.zeros(L.Kn.shape[0], np.complex128))
    return (x, _c64(psi + phi)) if split else (_c64(x + L.G @ phi), psi)


def _split_vcycle(levs, l, b, split):
    L = levs[l]
    x, psi = np.zeros_like(b), np.zeros(L.G.shape[1], np.complex128)
    if l == len(levs) - 1:
        for _ in range(4):
            x, psi = _split_smooth(L, b, x, psi, split)
        return x, psi
    x, psi = _split_smooth(L, b, x, psi, split)
    C = levs[l + 1]
    rc = L.PT @ (L.V * (b - L.K @ x + 1j * L.wm * (L.Ms @ (L.G @ psi))))
    rc = np.where(C.bnd, 0, rc / np.where(C.V > 0, C.V, 1))
    xc, psic = _split_vcycle(levs, l + 1, rc, split)
    x, psi = _c64(x + L.P @ xc), _c64(psi + L.Pn @ psic)
    return _split_smooth(L, b, x, psi, split)


def complex64_vcycle_bicgstab(model: OracleModel, ff, split=True, nlev=3, tol=1e-12, maxit=200, every=8):
    """BiCGStab with complex64 storage under the V-cycle above for the xy system of frequency ff;
    returns (iterations, final FP64 relative residual, FP64 residuals every `every` iterations)."""
    levs = _split_levels(model, ff, nlev)
    F = levs[0]
    K, K32 = F.K, F.K.astype(np.complex64)
    b = F.p1
    nb = np.linalg.norm(b)

    def op(yc, psi):  # A (y_c + G psi) in complex64 arithmetic on y_c, the mass part on G psi
        return _c64((K32 @ yc.astype(np.complex64)).astype(np.complex128) - 1j * F.wm * (F.Ms @ (F.G @ psi)))

    x = np.zeros_like(b)
    r = b.copy()
    rhat = r.copy()
    p = np.zeros_like(b)
    v = np.zeros_like(b)
    rho = alpha = omega = 1.0
    its, hist = 0, []
    while its < maxit:
        rho1 = np.vdot(rhat, r)
        p = _c64(r + rho1 / rho * alpha / omega * (p - omega * v))
        yc, ypsi = _split_vcycle(levs, 0, p, split)
        v = op(yc, ypsi)
        alpha = rho1 / np.vdot(rhat, v)
        s = _c64(r - alpha * v)
        zc, zpsi = _split_vcycle(levs, 0, s, split)
        t = op(zc, zpsi)
        omega = np.vdot(t, s) / np.vdot(t, t)
        x = x + alpha * (yc + F.G @ ypsi) + omega * (zc + F.G @ zpsi)
        r = _c64(s - omega * t)
        rho = rho1
        its += 1
        if its % every == 0:
            rr = b - K @ x
            hist.append(float(np.linalg.norm(rr) / nb))
            r = _c64(rr)
            if hist[-1] < tol or not np.isfinite(hist[-1]):
                break
    return its, float(np.linalg.norm(b - K @ x) / nb), hist


# --------------------------------------------------------------------------- the reference algorithm, timed
def reference_frequency(model: OracleModel, k, eps, pols=(0, 1)):
    """One frequency (both polarisations) of the reference algorithm as the driver runs it:
    doublemode_acc (fdfe_main.f90:1258-1563) with the reference's compiled-in options -- levels
    1-2 solved exactly (PARDISO in u1u2; SuperLU here, or converged_solve where level 2 has more
    than 20,000 edges and SuperLU takes minutes to hours), levels 3.. by BiCGStab with lexicographic SSOR from
    the extint_v guess, div_correc every 200 iterations, 1000 iterations per level, tolerance
    eps 10^(l-N).  Returns (seconds of the solve, (u1, u2) finest-level solutions, relres[2] of
    the finest level against the assembled matrix (None for a polarisation not solved),
    [(level, iterations)])."""
    ff = float(model.freq[k])
    m = OracleModel(model.nx, model.ny, model.nz, model.nair, model.a, model.b, model.c, model.sigma, model.freq,
                    model.recv, model.level, eps, 1, 1)
    # SuperLU's fill on 3-D edge meshes makes it impractical beyond ~10^4 unknowns
    big = nedges(m.nx // 2 ** (m.level - 2), m.ny // 2 ** (m.level - 2), m.nz // 2 ** (m.level - 2)) > 20000
    opts = OracleOpts(excmg=True, coarse_solver="converged" if big else "splu")
    t = time.perf_counter()
    u1, u2, infos = doublemode_acc(m, ff, opts, pols=pols)
    secs = time.perf_counter() - t
    edc, _, _ = mt1d_anl(ff, column_conv(m.sigma, m.nx, m.ny, m.nz), m.c)
    K, p1, p2 = assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, edc)
    rr = [float(np.linalg.norm(p - K @ u) / np.linalg.norm(p)) if q in pols else None
          for q, (p, u) in enumerate(((p1, u1), (p2, u2)))]
    return secs, (u1, u2), rr, [(i.level, list(i.iters)) for i in infos]
