"""End-to-end forward solves on the GPU against the oracle.

The multi-colour SSOR changes the Krylov iterates, so parity is on the
converged answer: impedances and surface fields of the GPU solve are
compared with the oracle's solution of the same mesh (SuperLU direct solve,
the exact discrete answer), within tolerances stated per test.
"""
import numpy as np
import pytest

import sfd_excmg_gb300 as S
from oracle import oracle as O
from sfd_excmg_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _omodel(m):
    return O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv, m.level, m.eps, m.solver,
                         m.out_type)


def _direct_Z(m):
    om = _omodel(m)
    ex = np.zeros((m.nf, 2, m.nl), np.complex128)
    for k, ff in enumerate(m.freq):
        u1, u2, _, _, _ = O.direct_solve(om, ff)
        ex[k, 0], ex[k, 1] = u1, u2
    return ex, O.impedances(om, ex, out_type=1, rd=2)


def _zc(res):
    return res[..., 0::2] + 1j * res[..., 1::2]


def test_halfspace_known_answer():
    m = syn.halfspace(n=16, freqs=(1.0, 10.0))
    ex, it, rr = S.fwd_solve(m, eps=1e-10, div_cor=0)
    res = S.impedance(m, ex, out_type=2)
    # discretisation error of a 16^3 mesh: within 5 % and 2 degrees
    assert np.all(np.abs(res[..., 0:2] / 100.0 - 1) < 0.05), res
    assert np.all(np.abs(res[..., 2:4] - 45.0) < 2.0), res


# Impedance agreement with the exact (direct) discrete solution.  An iterative
# solve to relative residual eps leaves errors of order eps * kappa in the
# near-null space of the operator (discrete gradients in air and at low
# frequency), and the impedance evaluation is sensitive to them; the consistent
# gradient-space correction (div_cor = 2) removes that component, so what is
# left is the residual-bound error of the remaining (static air) modes.
def z_tol_corrected(freq):
    """Remaining error after the correction: eps times the conditioning of the
    non-gradient modes, which grows as the skin depth outgrows the domain."""
    return np.where(np.asarray(freq) < 0.1, 5e-4, 1e-4)[:, None, None]


@pytest.mark.parametrize("excmg", [0, 1])
def test_forward_fp64_matches_direct(excmg):
    m = syn.small_aniso(n=16, seed=1, freqs=(0.05, 20.0))
    ex, it, rr = S.fwd_solve(m, eps=1e-10, excmg=excmg, level=3, div_cor=2, corr_intv=25, corr_tol=1e-2, solver=3)
    assert np.all(rr < 1.5e-10), rr
    _, zref = _direct_Z(m)
    z = S.impedance(m, ex)
    err = np.abs(_zc(z) - _zc(zref)) / np.abs(_zc(zref))
    assert np.all(err < z_tol_corrected(m.freq)), err


def test_forward_mixed_matches_fp64():
    m = syn.small_aniso(n=16, seed=2, freqs=(0.01, 1.0, 100.0))
    opts = dict(eps=1e-10, excmg=1, level=3, div_cor=2, corr_intv=25, corr_tol=1e-2, solver=3)
    ex64, _, rr64 = S.fwd_solve(m, **opts)
    exm, _, rrm = S.fwd_solve(m, precision=S.MIXED, **opts)
    assert np.all(rrm < 1.5e-10), rrm
    z64 = _zc(S.impedance(m, ex64))
    zm = _zc(S.impedance(m, exm))
    _, zref = _direct_Z(m)
    zr = _zc(zref)
    e64 = np.abs(z64 - zr) / np.abs(zr)
    em = np.abs(zm - zr) / np.abs(zr)
    assert np.all(em < z_tol_corrected(m.freq)), (em, e64)
    assert np.all(e64 < z_tol_corrected(m.freq)), (em, e64)


def test_uncorrected_error_lies_in_gradient_space():
    """Without the correction the field error of a converged iterative solve is (almost)
    entirely a discrete gradient: one correction step brings the impedances to the
    corrected accuracy."""
    m = syn.small_aniso(n=16, seed=1, freqs=(0.05,))
    # (without the correction FP64 GPBiCG can stall near 1e-10 on this model)
    ex, it, rr = S.fwd_solve(m, eps=1e-9, excmg=1, level=3, div_cor=0, solver=3)
    _, zref = _direct_Z(m)
    zr = _zc(zref)
    e0 = np.abs(_zc(S.impedance(m, ex)) - zr) / np.abs(zr)
    ff = m.freq[0]
    conv = O.column_conv(m.sigma, m.nx, m.ny, m.nz)
    edc, _, _ = O.mt1d_anl(ff, conv, m.c)
    _, p1, p2 = O.assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, edc)
    rhs = np.stack([p1, p2], axis=1)
    xc, _ = S.grad_correct(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, [ff, ff], rhs, ex[0].T.copy(), tol=1e-6)
    exc = ex.copy()
    exc[0] = xc.T
    e1 = np.abs(_zc(S.impedance(m, exc)) - zr) / np.abs(zr)
    assert e1.max() < 0.05 * e0.max(), (e0.max(), e1.max())


def test_plan_reuse_and_device_impedance():
    m = syn.small_aniso(n=16, seed=3, freqs=(0.3, 3.0))
    with S.Plan(m, eps=1e-9, excmg=1, level=3, div_cor=0) as p:
        ex1 = p.solve()
        z1 = p.impedance()
        ex2 = p.solve()
        z2 = p.impedance()
    assert np.array_equal(ex1, ex2)
    np.testing.assert_array_equal(z1, z2)
    zh = S.impedance(m, ex1)
    # device evaluation against the host one: the same formulas, different rounding
    np.testing.assert_allclose(z1, zh, rtol=1e-11, atol=1e-14 * np.abs(zh).max())


@pytest.mark.parametrize("transpose", [True, False])
def test_device_impedance_matches_host_evaluation(transpose):
    """sfdx_plan_impedance evaluates Z on the device (post_process + arho_interp2, fdfe_main.f90:549-790,
    one thread per receiver and frequency); sfdx_impedance evaluates it on the host from fetched
    fields.  Every output type (Zxy/Zyx, apparent resistivity and phase, the full tensor) and the
    tippers agree to rounding, with the reference's transposed receiver stencil and without."""
    from sfd_excmg_gb300 import capi
    quirks = capi.QUIRKS_REFERENCE if transpose else capi.QUIRKS_REFERENCE & ~capi.QUIRK_RX_TRANSPOSE
    m = syn.small_aniso(n=16, seed=2, freqs=(0.05, 1.0, 20.0))
    with S.Plan(m, eps=1e-9, excmg=1, level=3, solver=3, precision=S.FP64, div_cor=2, corr_intv=25, corr_tol=1e-2,
                quirks=quirks) as p:
        ex = p.solve()
        for ot in (1, 2, 3):
            zd, td = p.impedance(out_type=ot, tipper=True)
            zh, th = S.impedance(m, ex, out_type=ot, quirks=quirks, tipper=True)
            np.testing.assert_allclose(zd, zh, rtol=1e-11, atol=1e-14 * np.abs(zh).max())
            np.testing.assert_allclose(td, th, rtol=1e-10, atol=1e-13 * np.abs(th).max())


def test_solve_batch_matches_single_solves():
    """Models of different meshes solved together (one host thread and stream per plan)
    give exactly the fields of the same plans solved one at a time."""
    models = [syn.small_aniso(n=16, seed=5, freqs=(0.2, 5.0)), syn.small_aniso(n=24, seed=6, freqs=(1.0,)),
              syn.halfspace(n=16, freqs=(3.0, 30.0, 300.0))]
    opts = dict(eps=1e-9, excmg=1, level=3, div_cor=2, corr_intv=25, corr_tol=1e-2, solver=3, precision=S.MIXED)
    plans = [S.Plan(m, **opts) for m in models]
    try:
        st = S.solve_batch(plans)
        assert np.all(st == 0), st
        zb = [p.impedance() for p in plans]
        its = [p.iters.copy() for p in plans]
        for p, z, it in zip(plans, zb, its):
            p.solve(fetch=False)
            np.testing.assert_array_equal(p.impedance(), z)
            np.testing.assert_array_equal(p.iters, it)
    finally:
        for p in plans:
            p.close()


def test_sfd3d_end_to_end_matches_oracle(tmp_path):
    """The drop-in host `sfd3d <model> [level eps]` (sfd_excmg.f90:20-58) on a written
    .fwd/.dat pair: reads the files, solves on the GPU (EXCMG, 3 levels, GPBiCG, the
    consistent correction and the multigrid preconditioner from the environment) and
    writes <model>.res (output_data, file_opt.f90:131-158), whose impedances match the
    oracle's exact solution of the same model."""
    import os
    import subprocess
    from sfd_excmg_gb300 import capi
    m = syn.small_aniso(n=16, seed=1, freqs=(0.05, 20.0))
    m.solver = 3
    name = str(tmp_path / "mod")
    m.write(name)
    exe = os.path.join(os.path.dirname(capi.library_path()), "sfd3d")
    env = dict(os.environ, SFDX_EXCMG="1", SFDX_DIV_COR="2", SFDX_PRECOND="G", SFDX_CCV="1")
    r = subprocess.run([exe, name, "3", "1e-10"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = np.array([[float(v) for v in ln.split()] for ln in open(name + ".res").read().splitlines()])
    nrec = m.recv.shape[0]
    assert rows.shape == (m.nf * nrec, 9)
    np.testing.assert_allclose(rows[:, 0:3], np.tile(m.recv, (m.nf, 1)), rtol=1e-4)
    np.testing.assert_allclose(rows[:, 3], np.repeat(m.freq, nrec), rtol=1e-4)
    z = rows[:, 5:9].reshape(m.nf, nrec, 4)
    _, zref = _direct_Z(m)
    err = np.abs(_zc(z) - _zc(zref)) / np.abs(_zc(zref))
    # the file holds 5 significant digits (Ew.d with d = 5)
    assert np.all(err < z_tol_corrected(m.freq) + 2e-5), err
    # output_ccv (solvers.f90:687-704): one history per frequency and polarisation, the
    # finest level's iteration count, then the residuals at the check points, falling to
    # the tolerance
    import glob
    for pol in ("xy", "yx"):
        files = sorted(glob.glob(name + "_*_" + pol + "_excmg.ccv"))
        assert len(files) == m.nf, files
        for fn in files:
            lines = open(fn).read().split()
            n_it, vals = int(lines[0]), [float(v) for v in lines[1:]]
            assert n_it > 0 and len(vals) >= 1
            assert vals[-1] < 1e-10 and min(vals) > 0, vals
