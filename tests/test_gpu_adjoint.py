"""Misfit gradient on the GPU (adjoint solves + per-cell contraction) against the
oracle's exact adjoint, central finite differences of GPU forward solves, and
the torch.autograd path."""
import numpy as np
import pytest

import sfd_excmg_gb300 as S
from oracle import oracle as O
from sfd_excmg_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

MU = 4e-7 * np.pi
SOLVE = dict(eps=1e-10, excmg=1, level=3, div_cor=2, corr_intv=25, corr_tol=1e-2, solver=3)


def _case(freqs=(0.1, 3.0)):
    m = syn.small_aniso(n=16, seed=1, freqs=freqs)
    m2 = syn.small_aniso(n=16, seed=4, freqs=freqs)
    om2 = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m2.sigma, m.freq, m.recv)
    ex = np.zeros((m.nf, 2, m.nl), np.complex128)
    for k, ff in enumerate(m.freq):
        u1, u2, _, _, _ = O.direct_solve(om2, ff)
        ex[k, 0], ex[k, 1] = u1, u2
    zobs = O.impedances(om2, ex)
    return m, zobs


@pytest.mark.parametrize("precision", [S.FP64, S.MIXED])
def test_misfit_grad_matches_oracle(precision):
    m, zobs = _case()
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    phi, _, xs, mus = O.misfit_grad_cells(om, zobs, [], [])
    wm = [2 * np.pi * f * MU for f in m.freq for _ in (0, 1)]
    gref = O.sigma_grad_local(m.nx, m.ny, m.nz, m.a, m.b, m.c, wm, [x for xx in xs for x in xx],
                              [u for uu in mus for u in uu])
    with S.Plan(m, precision=precision, **SOLVE) as p:
        p.solve()
        mis, g, zp, it, rr = p.misfit_grad(zobs)
    assert np.all(rr < 1.5e-10), rr
    assert abs(mis - phi) <= 1e-4 * phi, (mis, phi)
    # the gradient of every cell and component (Frobenius norm over the model)
    err = np.linalg.norm(g - gref) / np.linalg.norm(gref)
    assert err < 1e-4, err
    # cells with a large gradient individually: forward and adjoint fields solved to
    # 1e-10 carry low-frequency errors of ~1e-4 relative (the impedance tolerances
    # of test_gpu_forward.py), which reach single cells at the 1e-3 level
    big = np.abs(gref) > 1e-2 * np.abs(gref).max()
    np.testing.assert_allclose(g[big], gref[big], rtol=3e-3)


def test_misfit_grad_matches_gpu_finite_differences():
    """Central differences (h = 1e-4 in log sigma) of the misfit from GPU forward solves.
    The perturbed solves start from the base fields and solve the correction equation
    (sfdx_plan_resolve), so the base solve's iteration error cancels in the difference."""
    m, zobs = _case(freqs=(0.3,))
    nx, ny = m.nx, m.ny
    cid = lambda i, j, k: (k * ny + j) * nx + i  # noqa: E731
    cells = [cid(8, 8, m.nair), cid(7, 9, m.nair + 1), cid(9, 7, m.nair + 2), cid(8, 8, m.nair + 4)]
    h = 1e-4
    with S.Plan(m, precision=S.FP64, **SOLVE) as p:
        p.solve()
        _, g, _, _, _ = p.misfit_grad(zobs)
        for cell in cells:
            for q in (0, 2):
                f = []
                for sgn in (1, -1):
                    sg = m.sigma.copy()
                    sg[q, cell] *= np.exp(sgn * h)
                    p.resolve(sigma=sg, tol=-1e-9)
                    f.append(p.misfit_grad(zobs, with_grad=False)[0])
                fd = (f[0] - f[1]) / (2 * h)
                ad = g[q, cell] * m.sigma[q, cell]
                assert abs(ad - fd) <= 1e-3 * abs(fd) + 1e-6 * np.abs(g[q] * m.sigma[q]).max(), (cell, q, ad, fd)


def test_autograd_log_sigma_on_device():
    torch = pytest.importorskip("torch")
    m, zobs = _case(freqs=(1.0,))
    iso = np.exp(np.log(m.sigma[0:3]).mean(axis=0))  # an isotropic model
    m.sigma[:] = 0
    m.sigma[0:3] = iso
    ls = torch.tensor(np.log(iso), dtype=torch.float64, device="cuda", requires_grad=True)
    with S.Plan(m, precision=S.MIXED, **SOLVE) as p:
        mis = S.log_sigma_misfit(ls, p, zobs)
        mis.backward()
        # the plan still holds the forward fields of the autograd forward pass: the
        # same misfit, and the same gradient from a repeated (deterministic) adjoint
        mis2, g, _, _, _ = p.misfit_grad(zobs)
    assert mis.item() == mis2
    sig = torch.exp(ls.detach()).cpu().numpy()
    ref = sig * (g[0] + g[1] + g[2])
    got = ls.grad.cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    assert abs(mis.item() - O.misfit(om, zobs)) <= 1e-4 * mis.item()


def test_fields_of_an_earlier_conductivity_are_refused():
    """After a conductivity load without a solve the plan's fields belong to the previous
    conductivity: the misfit (gradient) and the impedances are refused (SFDX_ERR_ARG), the
    field pointer is withheld, and the next solve makes them available again."""
    from sfd_excmg_gb300 import capi
    m, zobs = _case(freqs=(1.0,))
    with S.Plan(m, precision=S.FP64, **SOLVE) as p:
        p.solve(fetch=False)
        p.misfit_grad(zobs, with_grad=False)
        assert p.fields_device_ptr() != 0
        p.load(sigma=m.sigma * 1.1)
        for call in (lambda: p.misfit_grad(zobs), lambda: p.misfit_grad(zobs, with_grad=False), p.impedance):
            with pytest.raises(capi.SfdxError) as e:
                call()
            assert e.value.code == 1
        assert p.fields_device_ptr() == 0
        p.solve(sigma=m.sigma * 1.1, fetch=False)
        p.impedance()
        p.misfit_grad(zobs, with_grad=False)


def test_mixed_multigrid_adjoint_at_low_frequency_matches_fp64():
    """The complex64 multigrid V-cycle under 1e-3 Hz adjoint solves on resistive ground (the
    grf-inversion model: isotropic GRF, 1e-3..1e3 Hz), where its gradient corrections are
    largest.  The default mixed path (complex64 BiCGStab on split vectors, the nodal part kept
    as a potential) converges there; under the complex128-Krylov path (SFDX_MG_SPLIT=0) such
    systems stall, are stopped and restart with the FP64 V-cycle.  Either way every adjoint
    system meets the tolerance and the gradient agrees with the FP64 adjoint."""
    m, mt = syn.grf_inversion(0), syn.grf_inversion_true(0)
    opts = dict(eps=1e-10, excmg=1, level=m.level, div_cor=2, corr_intv=40, corr_tol=1e-2, solver=1, precond="G")
    with S.Plan(mt, precision=S.FP64, **opts) as pt:
        pt.solve(fetch=False)
        zobs = pt.impedance()
    out = {}
    for prec in (S.FP64, S.MIXED):
        with S.Plan(m, precision=prec, **opts) as p:
            p.solve(fetch=False)
            mis, g, _, its, rr = p.misfit_grad(zobs, tol=1e-9)
            out[prec] = (mis, g)
        assert rr.max() <= 1.5e-9, (prec, rr, its)
    (m64, g64), (m32, g32) = out[S.FP64], out[S.MIXED]
    # forward solves at 1e-10 leave impedance differences of ~1e-4 at 1e-3 Hz
    assert abs(m32 - m64) <= 3e-3 * m64, (m32, m64)
    err = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    print(f"grf-inversion adjoint at 1e-9: gradient mixed vs FP64 {err:.2e}")
    assert err < 1e-2, err
