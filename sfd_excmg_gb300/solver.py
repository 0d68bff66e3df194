"""Python face of the C ABI: forward solve, impedances and the component entry points.

Every function here calls libsfdx.so; none computes anything itself.  Arrays
are numpy (host); ``Plan.solve`` additionally accepts device pointers (for
example ``torch.Tensor.data_ptr()`` of a CUDA tensor) so that conductivities
and fields can stay resident in HBM between solves.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .model import Model


def _opts(**kw) -> capi.Opts:
    return capi.Opts.defaults(**kw)


def _d(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def _sigma(model: Model, sigma=None) -> np.ndarray:
    """The conductivity handed to the C ABI: [6][ncell] float64, size checked."""
    sg = _d(model.sigma if sigma is None else sigma)
    if sg.size != 6 * model.ncell:
        raise ValueError(f"sigma has {sg.size} values, expected 6 x {model.ncell}")
    return sg


def _nl(nx, ny, nz) -> int:
    return nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz


def _mesh(nx, ny, nz, a, b, c, sigma=None):
    """Spacings (and [6][ncell] conductivity) of an nx x ny x nz mesh for the C ABI, sizes checked."""
    a, b, c = _d(a), _d(b), _d(c)
    if (a.size, b.size, c.size) != (nx, ny, nz):
        raise ValueError(f"spacings of sizes ({a.size}, {b.size}, {c.size}) for a {nx} x {ny} x {nz} mesh")
    if sigma is None:
        return a, b, c
    sg = _d(sigma)
    if sg.size != 6 * nx * ny * nz:
        raise ValueError(f"sigma has {sg.size} values, expected 6 x {nx * ny * nz}")
    return a, b, c, sg


def _vec(v, n, ns, name) -> np.ndarray:
    """n x ns interleaved complex values (system fastest), size checked."""
    z = _z(v)
    if z.size != n * ns:
        raise ValueError(f"{name} has {z.size} values, expected {n} x {ns}")
    return z.reshape(n, ns)


def _z(x):
    return np.ascontiguousarray(x, dtype=np.complex128)


class Plan:
    """Device workspace for one mesh + frequency list (``sfdx_plan_*``)."""

    def __init__(self, model: Model, **opts):
        model.validate()
        self.model = model
        self.opts = _opts(**opts)
        self.nlev = self.opts.level if self.opts.excmg else 1
        self._h = ctypes.c_void_p()
        L = capi.lib()
        self._a, self._b, self._c, self._f = _d(model.a), _d(model.b), _d(model.c), _d(model.freq)
        capi.check(L.sfdx_plan_create(ctypes.byref(self._h), ctypes.byref(self.opts), model.nx, model.ny, model.nz,
                                      model.nair, capi.dptr(self._a), capi.dptr(self._b), capi.dptr(self._c),
                                      model.nf, capi.dptr(self._f)), "sfdx_plan_create")
        self.iters = np.zeros((model.nf, 2, self.nlev), np.int32)
        self.relres = np.zeros((model.nf, 2))
        self.status = 0

    def close(self):
        if self._h:
            capi.lib().sfdx_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def solve(self, sigma=None, out=None, sigma_device_ptr: int | None = None, out_device_ptr: int | None = None,
              allow_noconv: bool = False, fetch: bool = True):
        """Solve all frequencies x polarisations.  Returns ex[nf, 2, nl] (host) unless a device output is
        given or ``fetch`` is False (fields left in the plan's device memory only)."""
        L = capi.lib()
        m = self.model
        if sigma_device_ptr is not None:
            sp, son = ctypes.c_void_p(sigma_device_ptr), 1
        else:
            sg = _sigma(m, sigma)
            sp, son = ctypes.c_void_p(sg.ctypes.data), 0
            self._sg = sg
        ex = None
        if out_device_ptr is not None:
            op, oon = ctypes.c_void_p(out_device_ptr), 1
        elif not fetch:
            op, oon = ctypes.c_void_p(0), 0
        else:
            ex = out if out is not None else np.zeros((m.nf, 2, m.nl), np.complex128)
            if ex.dtype != np.complex128 or not ex.flags.c_contiguous or ex.size != m.nf * 2 * m.nl:
                raise ValueError(f"out must be a C-contiguous complex128 array of {m.nf * 2 * m.nl} values "
                                 f"([nf, 2, nl]), got {ex.dtype} of {ex.size}")
            op, oon = ctypes.c_void_p(ex.ctypes.data), 0
        it = np.zeros(self.iters.size, np.int32)
        rr = np.zeros(self.relres.size)
        rc = L.sfdx_plan_solve(self._h, sp, son, op, oon, capi.iptr(it), capi.dptr(rr))
        self.status = rc
        if rc != 0 and not (allow_noconv and rc == 4):
            raise capi.SfdxError(rc, "sfdx_plan_solve")
        self.iters = it.reshape(self.iters.shape)
        self.relres = rr.reshape(self.relres.shape)
        return ex

    def resolve(self, sigma=None, sigma_device_ptr: int | None = None, tol: float = 0.0,
                allow_noconv: bool = False) -> None:
        """Finest-level re-solve for a changed conductivity from the last full solve's fields x0
        (sfdx_plan_resolve).  tol > 0: relative residual; tol <= 0: correction equation
        A d = b - A x0 reduced by |tol| (0: the plan's eps), x = x0 + d."""
        if sigma_device_ptr is not None:
            sp, son = ctypes.c_void_p(sigma_device_ptr), 1
        else:
            self._sg = _sigma(self.model, sigma)
            sp, son = ctypes.c_void_p(self._sg.ctypes.data), 0
        it = np.zeros(self.iters.size, np.int32)
        rr = np.zeros(self.relres.size)
        rc = capi.lib().sfdx_plan_resolve(self._h, sp, son, tol, capi.iptr(it), capi.dptr(rr))
        self.status = rc
        if rc != 0 and not (allow_noconv and rc == 4):
            raise capi.SfdxError(rc, "sfdx_plan_resolve")
        self.iters = it.reshape(self.iters.shape)
        self.relres = rr.reshape(self.relres.shape)

    def load(self, sigma=None, sigma_device_ptr: int | None = None) -> None:
        """Upload (and coarsen) the conductivity without solving."""
        if sigma_device_ptr is not None:
            sp, son = ctypes.c_void_p(sigma_device_ptr), 1
        else:
            self._sg = _sigma(self.model, sigma)
            sp, son = ctypes.c_void_p(self._sg.ctypes.data), 0
        capi.check(capi.lib().sfdx_plan_load(self._h, sp, son), "sfdx_plan_load")

    def impedance(self, recv=None, out_type: int = 1, tipper: bool = False):
        """out[nf, nrec, 4] (out_type 0/1: Re/Im Zxy, Zyx; 2: apparent resistivities and phases) or
        out[nf, nrec, 8] (out_type 3: Re/Im of Zxx, Zxy, Zyx, Zyy)."""
        m = self.model
        rv = _d(np.asarray(m.recv if recv is None else recv).T)  # [3][nrec]
        nrec = rv.shape[1]
        out = np.zeros((m.nf, nrec, 8 if out_type == 3 else 4))
        tip = np.zeros((m.nf, nrec, 4)) if tipper else None
        capi.check(capi.lib().sfdx_plan_impedance(self._h, nrec, capi.dptr(rv), out_type, capi.dptr(out),
                                                   capi.dptr(tip) if tip is not None else None),
                   "sfdx_plan_impedance")
        return (out, tip) if tipper else out

    def misfit_grad(self, zobs, wts=None, recv=None, tol: float = 0.0, grad_device_ptr: int | None = None,
                    allow_noconv: bool = False, with_grad: bool = True):
        """Impedance misfit of the last solution and d misfit / d sigma (sfdx_plan_misfit_grad).

        zobs[nf, nrec, 4] = (Re Zxy, Im Zxy, Re Zyx, Im Zyx); wts[nf, nrec, 2] (None: 1).
        Returns (misfit, grad[6, ncell] or None when written to ``grad_device_ptr`` or not
        asked for (``with_grad=False``: no adjoint solve), zpred[nf, nrec, 4], adjoint
        iterations[nf, 2], adjoint relative residuals[nf, 2])."""
        m = self.model
        rv = _d(np.asarray(m.recv if recv is None else recv).T)
        nrec = rv.shape[1]
        zo = _d(zobs).reshape(m.nf, nrec, 4)
        wt = None if wts is None else _d(wts).reshape(m.nf, nrec, 2)
        zp = np.zeros((m.nf, nrec, 4))
        mis = ctypes.c_double()
        it = np.zeros(2 * m.nf, np.int32)
        rr = np.zeros(2 * m.nf)
        if not with_grad:
            g, gp, gon = None, None, 0
        elif grad_device_ptr is not None:
            g, gp, gon = None, ctypes.cast(ctypes.c_void_p(grad_device_ptr), capi.c_double_p), 1
        else:
            g = np.zeros((6, m.ncell))
            gp, gon = capi.dptr(g), 0
        rc = capi.lib().sfdx_plan_misfit_grad(self._h, nrec, capi.dptr(rv), capi.dptr(zo),
                                               capi.dptr(wt) if wt is not None else None, tol, ctypes.byref(mis),
                                               capi.dptr(zp), gp, gon, capi.iptr(it), capi.dptr(rr))
        if rc != 0 and not (allow_noconv and rc == 4):
            raise capi.SfdxError(rc, "sfdx_plan_misfit_grad")
        return mis.value, g, zp, it.reshape(m.nf, 2), rr.reshape(m.nf, 2)

    def fields_device_ptr(self) -> int:
        return capi.lib().sfdx_plan_fields(self._h) or 0

    def level_fields(self, level: int) -> np.ndarray:
        """Solution ex[nf, 2, nl_level] of level `level` (1-based; one of the two below the finest) from the
        last EXCMG solve (sfdx_plan_level_fields)."""
        m = self.model
        f = 2 ** (self.nlev - level)
        nx, ny, nz = m.nx // f, m.ny // f, m.nz // f
        ex = np.zeros((m.nf, 2, _nl(nx, ny, nz)), np.complex128)
        capi.check(capi.lib().sfdx_plan_level_fields(self._h, level, capi.dptr(ex.view(np.float64))),
                   "sfdx_plan_level_fields")
        return ex

    def history(self, maxit: int | None = None) -> np.ndarray:
        """Finest-level residual history of the last solve, [nf, 2, maxit] (sfdx_plan_history; values at the
        host's check points, 0 elsewhere)."""
        m = self.model
        n = maxit or (self.opts.maxit_level if self.opts.excmg else self.opts.maxit_plain)
        h = np.zeros((m.nf, 2, n))
        capi.check(capi.lib().sfdx_plan_history(self._h, capi.dptr(h), n), "sfdx_plan_history")
        return h

    def level_times(self) -> np.ndarray:
        ms = np.zeros(self.nlev)
        capi.check(capi.lib().sfdx_plan_level_times(self._h, capi.dptr(ms), self.nlev), "sfdx_plan_level_times")
        return ms

    def set_stream(self, stream_handle: int | None) -> None:
        """Issue the plan's kernels on a caller's CUDA stream (e.g. torch.cuda.current_stream().cuda_stream)."""
        capi.check(capi.lib().sfdx_plan_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)), "sfdx_plan_set_stream")

    def kernel_time(self, kernel: int, reps: int = 20):
        """(ms per launch, algorithmic bytes per launch) of one kernel family on the finest level."""
        ms, b = ctypes.c_double(), ctypes.c_double()
        capi.check(capi.lib().sfdx_plan_kernel_time(self._h, kernel, reps, ctypes.byref(ms), ctypes.byref(b)),
                   "sfdx_plan_kernel_time")
        return ms.value, b.value

    def autotune(self, reps: int = 3):
        """Measure and set the systems-per-thread grouping of the hot kernels
        (sfdx_plan_autotune); returns (complex64, complex128) choices."""
        a, b = ctypes.c_int(), ctypes.c_int()
        capi.check(capi.lib().sfdx_plan_autotune(self._h, reps, ctypes.byref(a), ctypes.byref(b)),
                   "sfdx_plan_autotune")
        return a.value, b.value

    def device_bytes(self) -> int:
        return int(capi.lib().sfdx_plan_device_bytes(self._h))


def solve_batch(plans, sigmas=None, sigma_device_ptrs=None, allow_noconv: bool = False):
    """Solve several plans at once (sfdx_plan_solve_batch): one host thread and one stream per
    plan.  Fields stay in each plan's device memory (``Plan.impedance``, ``Plan.fields_device_ptr``);
    each plan's ``iters``/``relres``/``status`` are updated.  Returns the per-plan status codes."""
    n = len(plans)
    arr = lambda vals: (ctypes.c_void_p * n)(*vals)  # noqa: E731
    keep = []
    if sigma_device_ptrs is not None:
        sp, son = arr(sigma_device_ptrs), 1
    else:
        for q, p in enumerate(plans):
            keep.append(_sigma(p.model, None if sigmas is None else sigmas[q]))
        sp, son = arr([k.ctypes.data for k in keep]), 0
    its = [np.zeros(p.iters.size, np.int32) for p in plans]
    rrs = [np.zeros(p.relres.size) for p in plans]
    st = np.zeros(n, np.int32)
    rc = capi.lib().sfdx_plan_solve_batch(n, arr([p._h.value for p in plans]), sp, son, None, 0,
                                          arr([a.ctypes.data for a in its]), arr([a.ctypes.data for a in rrs]),
                                          capi.iptr(st))
    for q, p in enumerate(plans):
        p.status = int(st[q])
        p.iters = its[q].reshape(p.iters.shape)
        p.relres = rrs[q].reshape(p.relres.shape)
    if rc != 0 and not (allow_noconv and rc == 4):
        raise capi.SfdxError(rc, "sfdx_plan_solve_batch")
    return st


def fwd_solve(model: Model, **opts):
    """sfdx_fwd_solve: returns (ex[nf,2,nl], iters[nf,2,levels], relres[nf,2])."""
    o = _opts(**opts)
    nlev = o.level if o.excmg else 1
    ex = np.zeros((model.nf, 2, model.nl), np.complex128)
    it = np.zeros(model.nf * 2 * nlev, np.int32)
    rr = np.zeros(model.nf * 2)
    rc = capi.lib().sfdx_fwd_solve(ctypes.byref(o), model.nx, model.ny, model.nz, model.nair, capi.dptr(_d(model.a)),
                                   capi.dptr(_d(model.b)), capi.dptr(_d(model.c)), capi.dptr(_d(model.sigma)),
                                   model.nf, capi.dptr(_d(model.freq)), capi.zptr(ex), capi.iptr(it), capi.dptr(rr))
    capi.check(rc, "sfdx_fwd_solve")
    return ex, it.reshape(model.nf, 2, nlev), rr.reshape(model.nf, 2)


def impedance(model: Model, ex, out_type: int = 1, quirks: int = capi.QUIRKS_REFERENCE, tipper: bool = False,
              recv=None):
    rv = _d(np.asarray(model.recv if recv is None else recv).T)
    nrec = rv.shape[1]
    out = np.zeros((model.nf, nrec, 8 if out_type == 3 else 4))
    tip = np.zeros((model.nf, nrec, 4)) if tipper else None
    x = _vec(ex, model.nf * 2, model.nl, "ex")
    capi.check(capi.lib().sfdx_impedance(model.nx, model.ny, model.nz, model.nair, capi.dptr(_d(model.a)),
                                         capi.dptr(_d(model.b)), capi.dptr(_d(model.c)), model.nf,
                                         capi.dptr(_d(model.freq)), capi.zptr(x), nrec, capi.dptr(rv), out_type,
                                         quirks, capi.dptr(out), capi.dptr(tip) if tip is not None else None),
               "sfdx_impedance")
    return (out, tip) if tipper else out


def impedance_topo(model: Model, ex, abr, topo, out_type: int = 1, quirks: int = capi.QUIRKS_REFERENCE,
                   tipper: bool = False, recv=None):
    """Impedances with the receivers of each surface column on its own earth surface
    (sfdx_impedance_topo): abr = (i1, i2, j1, j2, k1, k2) 1-based window, topo the elevation
    (m) of every window column, x fastest."""
    rv = _d(np.asarray(model.recv if recv is None else recv).T)
    nrec = rv.shape[1]
    ab = np.ascontiguousarray(abr, dtype=np.int32)
    tp = _d(topo)
    if ab.size != 6 or tp.size != (ab[1] - ab[0] + 1) * (ab[3] - ab[2] + 1):
        raise ValueError("abr must hold 6 indices and topo one elevation per window column")
    out = np.zeros((model.nf, nrec, 8 if out_type == 3 else 4))
    tip = np.zeros((model.nf, nrec, 4)) if tipper else None
    x = _vec(ex, model.nf * 2, model.nl, "ex")
    capi.check(capi.lib().sfdx_impedance_topo(model.nx, model.ny, model.nz, model.nair, capi.dptr(_d(model.a)),
                                              capi.dptr(_d(model.b)), capi.dptr(_d(model.c)), model.nf,
                                              capi.dptr(_d(model.freq)), capi.zptr(x), nrec, capi.dptr(rv), out_type,
                                              quirks, capi.iptr(ab), capi.dptr(tp), capi.dptr(out),
                                              capi.dptr(tip) if tip is not None else None), "sfdx_impedance_topo")
    return (out, tip) if tipper else out


def receiver_fields(model: Model, ex, quirks: int = capi.QUIRKS_REFERENCE, recv=None) -> np.ndarray:
    """Surface E and H at the receivers, [nf, nrec, 2, 5] complex: (Ex, Ey, Hx, Hy, Hz)
    of the xy and yx polarisations, the fields post_process forms Z and the tippers from."""
    rv = _d(np.asarray(model.recv if recv is None else recv).T)
    nrec = rv.shape[1]
    out = np.zeros((model.nf, nrec, 2, 5), np.complex128)
    x = _vec(ex, model.nf * 2, model.nl, "ex")
    capi.check(capi.lib().sfdx_receiver_fields(model.nx, model.ny, model.nz, model.nair, capi.dptr(_d(model.a)),
                                               capi.dptr(_d(model.b)), capi.dptr(_d(model.c)), model.nf,
                                               capi.dptr(_d(model.freq)), capi.zptr(x), nrec, capi.dptr(rv),
                                               quirks, capi.zptr(out)), "sfdx_receiver_fields")
    return out


# ---------------------------------------------------------------- components
def mt1d(freq: float, conv: np.ndarray, c: np.ndarray):
    conv = np.asarray(conv, np.float64)
    if conv.ndim != 2 or conv.shape[1] != 6 or np.size(c) != conv.shape[0]:
        raise ValueError(f"conv must be (nz, 6) with nz = len(c), got {conv.shape} and {np.size(c)}")
    nz = conv.shape[0]
    cf = _d(conv.T.ravel())  # Fortran conv(nz,6)
    edc = np.zeros(2 * nz + 2, np.complex128)
    hx = np.zeros(2 * nz + 2, np.complex128)
    imp = np.zeros(4, np.complex128)
    capi.check(capi.lib().sfdx_mt1d(freq, nz, capi.dptr(cf), capi.dptr(_d(c)), capi.zptr(edc), capi.zptr(hx),
                                    capi.zptr(imp)), "sfdx_mt1d")
    return edc, hx, imp


def apply_operator(nx, ny, nz, a, b, c, sigma, freqs, x, precision=capi.FP64):
    """y = K x for ns interleaved systems; x: [nl, ns] complex (or [nl] for one system)."""
    freqs = _d(np.atleast_1d(freqs))
    ns = len(freqs)
    a, b, c, sigma = _mesh(nx, ny, nz, a, b, c, sigma)
    xx = _vec(x, _nl(nx, ny, nz), ns, "x")
    y = np.zeros_like(xx)
    capi.check(capi.lib().sfdx_apply_operator(nx, ny, nz, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                              capi.dptr(sigma), ns, capi.dptr(freqs), precision, capi.zptr(xx),
                                              capi.zptr(y)), "sfdx_apply_operator")
    return y.reshape(np.shape(x))


def build_rhs(nx, ny, nz, a, b, c, sigma, freq, edc):
    nl = _nl(nx, ny, nz)
    a, b, c, sigma = _mesh(nx, ny, nz, a, b, c, sigma)
    e = _vec(edc, 2 * nz + 2, 1, "edc")
    p1 = np.zeros(nl, np.complex128)
    p2 = np.zeros(nl, np.complex128)
    capi.check(capi.lib().sfdx_build_rhs(nx, ny, nz, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                         capi.dptr(sigma), freq, capi.zptr(e), capi.zptr(p1),
                                         capi.zptr(p2)), "sfdx_build_rhs")
    return p1, p2


def precond_apply(nx, ny, nz, a, b, c, sigma, freqs, y, precond="S", precision=capi.FP64):
    freqs = _d(np.atleast_1d(freqs))
    ns = len(freqs)
    a, b, c, sigma = _mesh(nx, ny, nz, a, b, c, sigma)
    yy = _vec(y, _nl(nx, ny, nz), ns, "y")
    x = np.zeros_like(yy)
    capi.check(capi.lib().sfdx_precond_apply(nx, ny, nz, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                             capi.dptr(sigma), ns, capi.dptr(freqs), ord(precond), precision,
                                             capi.zptr(yy), capi.zptr(x)), "sfdx_precond_apply")
    return x.reshape(np.shape(y))


def vcycle_apply(model: Model, freqs, y, levels: int = 3, precision=capi.FP64):
    """One edge-multigrid V-cycle x = M^{-1} y (sfdx_vcycle_apply) on the model's mesh and the
    `levels` - 1 coarser ones; y[nl, ns] complex with one frequency per system."""
    freqs = _d(np.atleast_1d(freqs))
    ns = len(freqs)
    nx, ny, nz = model.nx, model.ny, model.nz
    a, b, c, sigma = _mesh(nx, ny, nz, model.a, model.b, model.c, model.sigma)
    yy = _vec(y, _nl(nx, ny, nz), ns, "y")
    x = np.zeros_like(yy)
    capi.check(capi.lib().sfdx_vcycle_apply(nx, ny, nz, model.nair, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                            capi.dptr(sigma), ns, capi.dptr(freqs), levels, precision,
                                            capi.zptr(yy), capi.zptr(x)), "sfdx_vcycle_apply")
    return x.reshape(np.shape(y))


def mesh_coarsen(a, b, c, sigma, k, quirks=capi.QUIRKS_REFERENCE):
    nx, ny, nz = len(a), len(b), len(c)
    a, b, c, sigma = _mesh(nx, ny, nz, a, b, c, sigma)
    f = 2 ** k
    a1, b1, c1 = np.zeros(nx // f), np.zeros(ny // f), np.zeros(nz // f)
    s1 = np.zeros((6, (nx // f) * (ny // f) * (nz // f)))
    capi.check(capi.lib().sfdx_mesh_coarsen(nx, ny, nz, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                            capi.dptr(sigma), k, quirks, capi.dptr(a1), capi.dptr(b1),
                                            capi.dptr(c1), capi.dptr(s1)), "sfdx_mesh_coarsen")
    return a1, b1, c1, s1


def prolongate(nx, ny, nz, a1, b1, c1, nair, u0, u1, quirks=capi.QUIRKS_REFERENCE):
    """extint_v on the fine mesh (nx,ny,nz); u0 on the 4h mesh, u1 on the 2h mesh ([n] or [n, ns])."""
    u0 = _z(u0)
    ns = 1 if u0.ndim == 1 else u0.shape[1]
    if nx % 4 or ny % 4 or nz % 4:
        raise ValueError(f"a {nx} x {ny} x {nz} mesh has no 4h level")
    a1, b1, c1 = _mesh(nx, ny, nz, a1, b1, c1)
    v0 = _vec(u0, _nl(nx // 4, ny // 4, nz // 4), ns, "u0")
    v1 = _vec(u1, _nl(nx // 2, ny // 2, nz // 2), ns, "u1")
    u = np.zeros((_nl(nx, ny, nz), ns), np.complex128)
    rc = capi.lib().sfdx_prolongate(nx, ny, nz, capi.dptr(a1), capi.dptr(b1), capi.dptr(c1), nair, ns,
                                    capi.zptr(v0), capi.zptr(v1), capi.zptr(u), quirks)
    capi.check(rc, "sfdx_prolongate")
    return u[:, 0] if u0.ndim == 1 else u


def krylov_solve(nx, ny, nz, a, b, c, sigma, freqs, rhs, x0=None, tol=1e-8, itmax=5000, history=False, **opts):
    """One Krylov solve of ns interleaved systems.  Returns (x, iters, relres, rc[, history[ns, itmax]])."""
    freqs = _d(np.atleast_1d(freqs))
    ns = len(freqs)
    a, b, c, sigma = _mesh(nx, ny, nz, a, b, c, sigma)
    r = _vec(rhs, _nl(nx, ny, nz), ns, "rhs")
    x = np.zeros_like(r) if x0 is None else _vec(x0, _nl(nx, ny, nz), ns, "x0").copy()
    it = np.zeros(ns, np.int32)
    rr = np.zeros(ns)
    hist = np.zeros((ns, itmax)) if history else None
    o = _opts(**opts)
    rc = capi.lib().sfdx_krylov_solve(ctypes.byref(o), nx, ny, nz, capi.dptr(a), capi.dptr(b),
                                      capi.dptr(c), capi.dptr(sigma), ns, capi.dptr(freqs), capi.zptr(r),
                                      capi.zptr(x), tol, itmax, capi.iptr(it), capi.dptr(rr),
                                      capi.dptr(hist) if hist is not None else None)
    if rc not in (0, 4):
        capi.check(rc, "sfdx_krylov_solve")
    out = (x.reshape(np.shape(rhs)), it, rr, rc)
    return out + (hist,) if history else out


def impedance_misfit(model: Model, ex, zobs, wts=None, quirks: int = capi.QUIRKS_REFERENCE, grad: bool = True):
    """sfdx_impedance_misfit: (misfit, d misfit / d ex [nf, 2, nl] or None) of host fields ex[nf, 2, nl]."""
    m = model
    x = _vec(ex, m.nf * 2, m.nl, "ex")
    f = _d(m.freq)
    rv = _d(np.asarray(m.recv).T)
    nrec = rv.shape[1]
    zo = _d(zobs).reshape(m.nf, nrec, 4)
    wt = None if wts is None else _d(wts).reshape(m.nf, nrec, 2)
    g = np.zeros_like(x) if grad else None
    mis = ctypes.c_double()
    capi.check(capi.lib().sfdx_impedance_misfit(m.nx, m.ny, m.nz, m.nair, capi.dptr(_d(m.a)), capi.dptr(_d(m.b)),
                                                 capi.dptr(_d(m.c)), m.nf, capi.dptr(f), capi.zptr(x), rv.shape[1],
                                                 capi.dptr(rv), quirks, capi.dptr(zo),
                                                 capi.dptr(wt) if wt is not None else None, ctypes.byref(mis),
                                                 capi.zptr(g) if g is not None else None),
               "sfdx_impedance_misfit")
    return mis.value, (g.reshape(np.shape(ex)) if g is not None else None)


def write_res(name: str, freqs, recv, res, tipper=None) -> None:
    """output_data (file_opt.f90:131-158): <name>.res from results[nf, nrec, 4]; with
    tipper[nf, nrec, 4] the tipper block follows, as with output_tipper."""
    f = _d(np.atleast_1d(freqs))
    rv = _d(np.asarray(recv).T)
    r = _d(res)
    t = None if tipper is None else _d(tipper)
    if t is not None and t.shape != r.shape:
        raise ValueError(f"tipper shape {t.shape} differs from the results' {r.shape}")
    capi.check(capi.lib().sfdx_write_res_tipper(name.encode(), len(f), capi.dptr(f), rv.shape[1], capi.dptr(rv),
                                                capi.dptr(r), capi.dptr(t) if t is not None else None),
               "sfdx_write_res_tipper")


def write_ccv(name: str, freq: float, polar: str, tag: str, iters: int, history) -> None:
    """Convergence-history file of one solve (solvers.f90:687-704), history from krylov_solve."""
    h = _d(np.ravel(history))
    capi.check(capi.lib().sfdx_write_ccv(name.encode(), float(freq), polar.encode(), tag.encode(), int(iters),
                                         capi.dptr(h), h.size), "sfdx_write_ccv")


def grad_correct(nx, ny, nz, a, b, c, sigma, freqs, rhs, x, tol=1e-8, maxit=2000):
    """Consistent gradient-space correction of x (sfdx_grad_correct): returns
    (x + G phi, nodal PCG iterations)."""
    freqs = _d(np.atleast_1d(freqs))
    ns = len(freqs)
    a, b, c, sigma = _mesh(nx, ny, nz, a, b, c, sigma)
    r = _vec(rhs, _nl(nx, ny, nz), ns, "rhs")
    xx = _vec(x, _nl(nx, ny, nz), ns, "x").copy()
    it = np.zeros(1, np.int32)
    capi.check(capi.lib().sfdx_grad_correct(nx, ny, nz, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                            capi.dptr(sigma), ns, capi.dptr(freqs), capi.zptr(r), capi.zptr(xx),
                                            tol, maxit, capi.iptr(it)), "sfdx_grad_correct")
    return xx.reshape(np.shape(x)), int(it[0])
