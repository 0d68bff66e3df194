"""Parity of the GPU forward solve with the oracle on the benchmark workloads.

The oracle's answer is the exact discrete solution of the reference's system
(fd_assemb + dcfast with the mt1d_anl boundary values), committed as fixtures
by tests/golden/make_oracle_fixtures.py (relative residual 1e-15).  The GPU
solves the same systems with its own iteration (multi-colour smoothers,
complex64 inner iterations, multigrid), so parity is on the converged
answer: impedances Zxy, Zyx at every receiver and frequency, and the field
on a sample of earth edges, within the tolerances stated per test.  The
coarse levels of the EXCMG cascade (the reference's PARDISO solves) are
compared with the exact solution of the same coarse systems (SciPy's SuperLU, or
the oracle's converged solve to a 1e-15 residual where SuperLU is impractical).
"""
import os

import numpy as np
import pytest

import sfd_excmg_gb300 as S
from oracle import oracle as O
from sfd_excmg_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture(name):
    path = os.path.join(GOLDEN, name + "_oracle.npz")
    if not os.path.exists(path):
        pytest.skip(f"no oracle fixture {path}")
    return np.load(path)


def _earth(nx, ny, nz, nair):
    """Edges below the air layers (their values are well determined; in air the discrete
    gradients leave the field ill-conditioned at low frequency)."""
    xnl, ynl = nx * (ny + 1) * (nz + 1), (nx + 1) * ny * (nz + 1)
    e = np.arange(xnl + ynl + (nx + 1) * (ny + 1) * nz)
    k = np.where(e < xnl, e // (nx * (ny + 1)),
                 np.where(e < xnl + ynl, (e - xnl) // ((nx + 1) * ny), (e - xnl - ynl) // ((nx + 1) * (ny + 1))))
    return k > nair


def _zc(res):
    return res[..., 0::2] + 1j * res[..., 1::2]


def _errors(plan, ex, fx):
    """(max Z relative error, max earth-field error relative to each system's largest sampled value)."""
    z = _zc(plan.impedance())
    ez = np.abs(z - fx["z"]) / np.abs(fx["z"])
    got = ex[:, :, fx["edges"]]
    ref = fx["fields"]
    ef = np.abs(got - ref).max(axis=2) / np.abs(ref).max(axis=2)
    return float(ez.max()), float(ef.max())


# Impedance and field agreement of a solve converged to relative residual
# 1e-13 on the finest level: the exact answer to ~1e-6 in Z at the lowest
# frequencies (where H = curl E / (i w mu) amplifies field errors most; 3e-6
# allowed) and better elsewhere.  The earth fields keep a discrete-gradient error that the
# residual barely sees (the final gradient correction reduces it to its nodal
# tolerance, corr_tol = 1e-2): 1e-3 of the largest field of the system.
Z_TOL_CONVERGED = 3e-6
F_TOL_CONVERGED = 1e-3


@pytest.mark.parametrize("precision,precond,solver", [(S.FP64, "G", 3), (S.MIXED, "G", 1), (S.FP64, "S", 3)])
def test_halfspace_cube_converged_matches_oracle(precision, precond, solver):
    """Config 1 (32^3 core cells + padding and air, 48^3, 3 EXCMG levels) solved tightly."""
    fx = _fixture("halfspace_cube")
    m = syn.halfspace_cube()
    with S.Plan(m, eps=1e-13, excmg=1, level=3, solver=solver, precision=precision, precond=precond, div_cor=2,
                corr_intv=40, corr_tol=1e-2, maxit_level=3000) as p:
        ex = p.solve()
        ez, ef = _errors(p, ex, fx)
    print(f"halfspace-cube precision {precision} precond {precond} solver {solver}: Z {ez:.2e}, fields {ef:.2e}")
    assert ez < Z_TOL_CONVERGED and ef < F_TOL_CONVERGED, (ez, ef)


def test_halfspace_cube_reference_config_matches_oracle():
    """Config 1 as configured: EXCMG with 3 levels, FP64, BiCGStab with SSOR, tolerance 1e-8,
    with the consistent gradient correction.  A 1e-8 residual leaves impedance errors of
    ~9e-2 at the lowest frequency (0.01 Hz), falling to ~3e-3 at 100 Hz: the configuration's
    tolerance is far from the 1e-5 accuracy of the benchmark metric."""
    fx = _fixture("halfspace_cube")
    m = syn.halfspace_cube()
    with S.Plan(m, eps=1e-8, excmg=1, level=3, solver=1, precision=S.FP64, div_cor=2, corr_intv=40,
                corr_tol=1e-2) as p:
        p.solve(fetch=False)
        z = _zc(p.impedance())
    ez = (np.abs(z - fx["z"]) / np.abs(fx["z"])).max(axis=(1, 2))
    print("halfspace-cube tol 1e-8, Z error per frequency:", ez)
    assert np.all(ez < [0.2, 0.05, 0.02, 0.01]), ez


@pytest.mark.parametrize("precision,solver", [(S.FP64, 3), (S.MIXED, 1)])
def test_aniso_hills_converged_matches_oracle(precision, solver):
    """Config 2 (anisotropic blocks, Gaussian hills, 80^3 with padding and air, 8 frequencies
    over 0.001-1000 Hz, 32x32 receivers) solved tightly with the multigrid preconditioner."""
    fx = _fixture("aniso_hills")
    m = syn.aniso_hills(seed=0)
    with S.Plan(m, eps=1e-13, excmg=1, level=3, solver=solver, precision=precision, precond="G", div_cor=2,
                corr_intv=40, corr_tol=1e-2, maxit_level=3000) as p:
        ex = p.solve()
        ez, ef = _errors(p, ex, fx)
    print(f"aniso-hills precision {precision} solver {solver}: Z {ez:.2e}, fields {ef:.2e}")
    assert ez < Z_TOL_CONVERGED and ef < F_TOL_CONVERGED, (ez, ef)


def test_large_inclusions_converged_matches_oracle():
    """Config 4, the benchmark workload (128x128x96 core cells, 160x160x144 with padding and
    air, 11.2 M edges, 6 frequencies, 4 EXCMG levels), as the benchmark solves it: mixed
    precision (complex64 V-cycle under complex128 BiCGStab), tolerance 1e-12."""
    fx = _fixture("large_inclusions")
    m = syn.large_inclusions(seed=0)
    with S.Plan(m, eps=1e-12, excmg=1, level=m.level, solver=1, precision=S.MIXED, precond="G", div_cor=2,
                corr_intv=20, corr_tol=1e-2, maxit_level=3000) as p:
        ex = p.solve()
        ez, ef = _errors(p, ex, fx)
    print(f"large-inclusions mixed: Z {ez:.2e}, fields {ef:.2e}")
    assert ez < 1e-5 and ef < F_TOL_CONVERGED, (ez, ef)


def test_coarse_levels_and_guess_match_exact_solves():
    """Levels 1 and 2 of a 3-level cascade (the reference solves them with PARDISO,
    u1u2 fdfe_main.f90:1228-1256) against the exact solution of the same coarse systems, and the
    extrapolated finest-level guess (extint_v) built from each, on the earth edges."""
    m = syn.halfspace_cube()
    with S.Plan(m, eps=1e-8, excmg=1, level=3, solver=3, precision=S.FP64, div_cor=2, corr_intv=40,
                corr_tol=1e-2) as p:
        p.solve(fetch=False)
        u = [p.level_fields(1), p.level_fields(2)]
        coarse_tol = p.opts.coarse_tol
    ref = []
    for lev, k in ((1, 2), (2, 1)):
        a1, b1, c1, s1 = O.mesh_coarsen(m.a, m.b, m.c, m.sigma, k, quirk=True)
        nx, ny, nz = len(a1), len(b1), len(c1)
        rl = np.zeros((m.nf, 2, O.nedges(nx, ny, nz)), np.complex128)
        for f, ff in enumerate(m.freq):
            om = O.OracleModel(nx, ny, nz, m.nair // 2 ** k, a1, b1, c1, s1, m.freq, m.recv)
            if rl.shape[2] <= 20000:
                x1, x2, _, _, _ = O.direct_solve(om, ff)
            else:  # SuperLU takes hours on 3-D edge meshes of this size: the 1e-15 converged solve
                x1, x2, _, _, _ = O.converged_solve(om, ff)
            rl[f, 0], rl[f, 1] = x1, x2
        ref.append(rl)
        ea = _earth(nx, ny, nz, m.nair // 2 ** k)
        err = np.abs(u[lev - 1][:, :, ea] - rl[:, :, ea]).max(axis=2) / np.abs(rl[:, :, ea]).max(axis=2)
        print(f"level {lev}: max earth-field error {err.max():.2e} (coarse_tol {coarse_tol:g})")
        assert err.max() < 1e-5, err
    ea = _earth(m.nx, m.ny, m.nz, m.nair)
    for f in range(m.nf):
        for pol in range(2):
            g_gpu = S.prolongate(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.nair, u[0][f, pol], u[1][f, pol])
            g_ref, _ = O.extint_v(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.nair, ref[0][f, pol], ref[1][f, pol])
            d = np.abs(g_gpu[ea] - g_ref[ea]).max() / np.abs(g_ref[ea]).max()
            assert d < 1e-4, (f, pol, d)
