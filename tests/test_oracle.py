"""Known-answer tests that pin the oracle (CPU, no GPU needed).

The reference ships no golden vectors and cannot be compiled here (ifort +
MKL), so the oracle's restatement is pinned by answers known independently:
the analytic homogeneous and layered 1-D responses, the half-space apparent
resistivity and phase of the 3-D discretisation, a 3-D solve of a 1-D model,
exact reproduction of constant fields by the EXCMG prolongation, the
algebraic identities the gradient-space correction relies on, and the
identities of the ILU(0) factor (zilu0).
"""
import numpy as np
import pytest

from oracle import oracle as O
from sfd_excmg_gb300 import synthetic as syn

MU = 4e-7 * np.pi


def _layered_column(thick, sig, nz_per, h):
    """conv (nz,6) and c (nz) for layers of given conductivity; the last layer is the basement."""
    c, conv = [], []
    for t, s in zip(thick, sig):
        n = int(round(t / h)) if t is not None else nz_per
        c += [h] * n
        conv += [[s, s, s, 0, 0, 0]] * n
    return np.array(conv, float), np.array(c, float)


@pytest.mark.parametrize("f", [0.01, 1.0, 100.0])
def test_mt1d_homogeneous_halfspace_is_analytic(f):
    nz, h, sig = 40, 50.0, 0.01
    conv = np.zeros((nz, 6))
    conv[:, :3] = sig
    e, _, imp = O.mt1d_anl(f, conv, np.full(nz, h))
    z = np.arange(nz + 1) * h
    delta = np.sqrt(2 / (2 * np.pi * f * MU * sig))
    np.testing.assert_allclose(e[:nz + 1], np.exp(-(1 - 1j) * z / delta), rtol=0, atol=1e-13)
    w = 2 * np.pi * f
    np.testing.assert_allclose(np.abs(imp[1]) ** 2 / (w * MU), 1 / sig, rtol=1e-12)
    np.testing.assert_allclose(abs(np.degrees(np.angle(imp[1]))), 45.0, atol=1e-9)


def _wait_impedance(f, thick, sig):
    """Layered-earth impedance by Wait's recursion (isotropic layers, last = half-space)."""
    w = 2 * np.pi * f
    k = np.sqrt(-1j * w * MU * np.asarray(sig, complex))
    zeta = w * MU / k
    Z = zeta[-1]
    for n in range(len(sig) - 2, -1, -1):
        t = np.tanh(1j * k[n] * thick[n])
        Z = zeta[n] * (Z + zeta[n] * t) / (zeta[n] + Z * t)
    return Z


@pytest.mark.parametrize("f", [0.1, 3.0])
def test_mt1d_layered_impedance_matches_recursion(f):
    h = 25.0
    thick = [500.0, 750.0, None]
    sig = [0.01, 0.5, 0.002]
    conv, c = _layered_column(thick, sig, 60, h)
    e, hfield, imp = O.mt1d_anl(f, conv, c)
    Z = _wait_impedance(f, [500.0, 750.0], sig)
    # the surface impedance E/H of the propagated xy-mode fields (magnitude and
    # phase of Zxy, the sign convention of the time factor aside)
    zs = e[0] / hfield[0]
    np.testing.assert_allclose(abs(zs), abs(Z), rtol=1e-10)
    np.testing.assert_allclose(abs(np.angle(zs)), abs(np.angle(Z)), rtol=1e-9)
    # mt1d_anl's own impedance output is taken at the bottom node (model_selec.f90,
    # i = nz+1), i.e. the basement half-space
    zb = _wait_impedance(f, [], sig[-1:])
    np.testing.assert_allclose(abs(imp[1]), abs(zb), rtol=1e-10)


def _direct_res(m, out_type=2):
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    ex = np.zeros((m.nf, 2, m.nl), np.complex128)
    for k, ff in enumerate(m.freq):
        u1, u2, _, _, _ = O.direct_solve(om, ff)
        ex[k, 0], ex[k, 1] = u1, u2
    return ex, O.impedances(om, ex, out_type=out_type, rd=2)


def test_direct_halfspace_apparent_resistivity_and_phase():
    m = syn.halfspace(n=16, freqs=(1.0, 10.0))
    _, res = _direct_res(m)
    # 16^3 cells: discretisation error within 5 % and 2 degrees
    assert np.all(np.abs(res[..., 0:2] / 100.0 - 1) < 0.05), res
    assert np.all(np.abs(np.abs(res[..., 2:4]) - 45.0) < 2.0), res


def test_direct_solve_of_1d_model_is_laterally_uniform_and_matches_1d():
    """A laterally uniform model: the 3-D solution equals the 1-D background on every
    column (the Dirichlet data is the 1-D solution, and the 3-D rows of a 1-D model
    reduce to the same second difference)."""
    m = syn.halfspace(n=16, freqs=(2.0,))
    ex, _ = _direct_res(m)
    nx, ny, nz = m.nx, m.ny, m.nz
    conv = O.column_conv(m.sigma, nx, ny, nz)
    edc, _, _ = O.mt1d_anl(2.0, conv, m.c)
    exs = ex[0, 0, :nx * (ny + 1) * (nz + 1)].reshape(nz + 1, ny + 1, nx)
    col = exs[:, ny // 2, nx // 2]
    np.testing.assert_allclose(col, edc[:nz + 1], rtol=0, atol=2e-3 * np.abs(edc[:nz + 1]).max())
    # laterally uniform
    assert np.abs(exs[:, 1:-1, :] - col[:, None, None]).max() < 2e-3 * np.abs(col).max()


@pytest.mark.parametrize("quirk", [False, True])
def test_prolongation_reproduces_constant_fields(quirk):
    m = syn.small_aniso(n=16, seed=4)
    nx, ny, nz = m.nx, m.ny, m.nz
    sizes = [(nx // 4, ny // 4, nz // 4), (nx // 2, ny // 2, nz // 2)]
    vals = (1.5 - 0.5j, -0.25 + 2j, 0.75 + 0.1j)
    def field(x, y, z):
        nxl = x * (y + 1) * (z + 1)
        nyl = (x + 1) * y * (z + 1)
        nzl = (x + 1) * (y + 1) * z
        return np.concatenate([np.full(nxl, vals[0]), np.full(nyl, vals[1]), np.full(nzl, vals[2])])
    u0 = field(*sizes[0])
    u1 = field(*sizes[1])
    u, _ = O.extint_v(nx, ny, nz, m.a, m.b, m.c, m.nair, u0, u1, midpoint_quirk=quirk)
    np.testing.assert_allclose(u, field(nx, ny, nz), rtol=0, atol=1e-12)


def _ms(m, ff):
    conv = O.column_conv(m.sigma, m.nx, m.ny, m.nz)
    edc, _, _ = O.mt1d_anl(ff, conv, m.c)
    K1, p1, _ = O.assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, edc)
    K2, _, _ = O.assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, 2 * ff, edc)
    w1, w2 = 2 * np.pi * ff * MU, 4 * np.pi * ff * MU
    Ms = ((K1 - K2) / (-1j * (w1 - w2))).real
    return K1, p1, Ms, w1


def test_gradient_space_identities():
    """C G = 0 (curl-curl part of the assembled rows annihilates discrete gradients), the
    dual-volume-weighted curl-curl is symmetric, and G^T V Ms G is symmetric positive
    definite -- the facts behind the consistent gradient-space correction."""
    m = syn.small_aniso(n=12, seed=2)
    K, _, Ms, w = _ms(m, 0.5)
    C = (K + 1j * w * Ms).real
    G = O.node_gradient(m.nx, m.ny, m.nz, m.a, m.b, m.c)
    V = O.edge_dual_volumes(m.nx, m.ny, m.nz, m.a, m.b, m.c)
    interior = V > 0
    CG = (C @ G).tocsr()[interior]
    assert abs(CG).max() <= 1e-12 * abs(C).max() * abs(G).max()
    VC = (C.multiply(V[:, None])).tocsr()[interior][:, interior]
    assert abs(VC - VC.T).max() <= 1e-12 * abs(VC).max()
    N = (G.T @ (Ms.multiply(V[:, None])) @ G).toarray()
    assert np.abs(N - N.T).max() <= 1e-12 * np.abs(N).max()
    assert np.linalg.eigvalsh((N + N.T) / 2).min() > 0


def test_oracle_grad_correct_is_a_projection():
    m = syn.small_aniso(n=12, seed=5)
    ff = 0.2
    K, p1, _, _ = _ms(m, ff)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(m.nl) + 1j * rng.standard_normal(m.nl)
    x1 = O.grad_correct(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, p1, x)
    x2 = O.grad_correct(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, p1, x1)
    # idempotent up to the conditioning of N (air conductivity 1e-9 against
    # earth 1e-2..1 makes the nodal system span ~8 orders of magnitude)
    assert np.linalg.norm(x2 - x1) <= 1e-4 * np.linalg.norm(x1 - x)
    G = O.node_gradient(m.nx, m.ny, m.nz, m.a, m.b, m.c)
    V = O.edge_dual_volumes(m.nx, m.ny, m.nz, m.a, m.b, m.c)
    n0 = np.linalg.norm(G.T @ (V * (p1 - K @ x)))
    n1 = np.linalg.norm(G.T @ (V * (p1 - K @ x1)))
    assert n1 <= 1e-10 * n0
    # the exact discrete solution is a fixed point (both sides carry rounding
    # amplified by the near-singular gradient modes of K)
    from scipy.sparse.linalg import splu
    xs = splu(K.tocsc()).solve(p1)
    xs1 = O.grad_correct(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, p1, xs)
    assert np.linalg.norm(xs1 - xs) <= 1e-4 * np.linalg.norm(xs)


def _adjoint_case():
    m = syn.small_aniso(n=12, seed=2, freqs=(0.5,))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    m2 = syn.small_aniso(n=12, seed=3, freqs=(0.5,))
    om2 = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m2.sigma, m.freq, m.recv)
    u1, u2, _, _, _ = O.direct_solve(om2, 0.5)
    zobs = O.impedances(om2, np.stack([u1, u2])[None])
    return m, om, zobs


def test_oracle_adjoint_gradient_matches_finite_differences():
    """The oracle's misfit gradient (transposed direct solve, operator derivative by
    re-assembly) against central differences of the misfit, one cell per component kind."""
    m, om, zobs = _adjoint_case()
    nx, ny = m.nx, m.ny
    cid = lambda i, j, k: (k * ny + j) * nx + i  # noqa: E731
    cells = [cid(5, 6, m.nair + 1), cid(7, 7, m.nair), cid(6, 6, m.nair + 2)]
    comps = [0, 3, 5]
    _, g, _, _ = O.misfit_grad_cells(om, zobs, cells, comps)
    for t, (cell, q) in enumerate(zip(cells, comps)):
        h = 1e-4 * max(abs(m.sigma[q, cell]), 1e-3)
        f = []
        for sgn in (1, -1):
            sg = m.sigma.copy()
            sg[q, cell] += sgn * h
            f.append(O.misfit(O.OracleModel(nx, ny, m.nz, m.nair, m.a, m.b, m.c, sg, m.freq, m.recv), zobs))
        fd = (f[0] - f[1]) / (2 * h)
        assert abs(g[t] - fd) <= 1e-3 * abs(fd), (t, g[t], fd)


def test_local_contraction_matches_reassembly():
    """The closed-form per-cell contraction (vol/4, vol/8 couplings, adjoint fields
    mu = lambda / V through the dual-volume symmetry) equals the re-assembly gradient."""
    m, om, zobs = _adjoint_case()
    rng = np.random.default_rng(7)
    cells = list(rng.integers(m.nair * m.nx * m.ny, m.ncell, 6))
    comps = [0, 1, 2, 3, 4, 5]
    _, g, xs, mus = O.misfit_grad_cells(om, zobs, cells, comps)
    wm = [2 * np.pi * m.freq[0] * MU] * 2
    gl = O.sigma_grad_local(m.nx, m.ny, m.nz, m.a, m.b, m.c, wm, list(xs[0]), list(mus[0]))
    loc = np.array([gl[q, c] for c, q in zip(cells, comps)])
    np.testing.assert_allclose(loc, g, rtol=1e-7, atol=1e-9 * np.abs(g).max())


@pytest.mark.parametrize("ff", [0.01, 3.0])
def test_volume_weighted_operator_is_complex_symmetric(ff):
    """V K = K^T V for the full assembled complex rows (curl-curl and the anisotropic
    mass terms), with V the edge dual volumes on the interior and 1 on the Dirichlet
    rows: the identity behind COCR's bilinear form, BiCG's A^H products and the
    adjoint solve with the forward operator."""
    m = syn.small_aniso(n=12, seed=6)
    conv = O.column_conv(m.sigma, m.nx, m.ny, m.nz)
    edc, _, _ = O.mt1d_anl(ff, conv, m.c)
    K, _, _ = O.assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, edc)
    V = O.edge_dual_volumes(m.nx, m.ny, m.nz, m.a, m.b, m.c)
    V = np.where(V > 0, V, 1.0)
    VK = (K.multiply(V[:, None])).tocsr()
    assert abs(VK - VK.T).max() <= 1e-12 * abs(VK).max()


def _tiny_aniso_system(ff=1.0, seed=3):
    """Assembled curl-curl system of a 4x4x6-cell anisotropic model with two air layers
    (430 edges): small enough for dense checks of a preconditioner."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = 4, 4, 6
    a, b = np.full(nx, 100.0), np.full(ny, 120.0)
    c = np.array([200.0, 100, 50, 50, 80, 120])
    ncell = nx * ny * nz
    sig = np.zeros((6, ncell))
    sig[0:3] = 10 ** rng.uniform(-3, -1, (3, ncell))
    sig[3:6] = 0.2 * sig[0] * rng.uniform(-1, 1, (3, ncell))
    sig[:, : nx * ny * 2] = 0
    sig[0:3, : nx * ny * 2] = 1e-8
    edc, _, _ = O.mt1d_anl(ff, O.column_conv(sig, nx, ny, nz), c)
    K, p1, _ = O.assemble(nx, ny, nz, a, b, c, sig, ff, edc)
    return (nx, ny, nz, a, b, c, sig), K, p1


def test_ilu0_is_the_exact_lu_of_a_tridiagonal_matrix():
    """zilu0 + lusol (pre_type 'I'): without fill-in ILU(0) is the LU factorisation."""
    rng = np.random.default_rng(0)
    n = 50
    import scipy.sparse as sp
    d = 4 + rng.standard_normal(n) + 1j * rng.standard_normal(n)
    T = sp.diags([rng.standard_normal(n - 1) + 0j, d, rng.standard_normal(n - 1) + 0j], [-1, 0, 1], format="csr")
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(O.ilu_apply(T, y), np.linalg.solve(T.toarray(), y), rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("band_kind", ["all", "np"])
def test_ilu0_reproduces_the_matrix_on_its_band_pattern(band_kind):
    """The defining property of ILU(0): M = LU equals A on every entry the factor keeps.
    zilu0 keeps the columns with |jcol - ii - 1| <= idd(2): every entry for
    doublemode_nor (idd(2) = nl), only those within np for doublemode_acc (idd(2) = np),
    which leaves out the Ex-Ez couplings."""
    mesh, K, _ = _tiny_aniso_system()
    nx, ny, nz = mesh[:3]
    n = K.shape[0]
    band = 0 if band_kind == "all" else (nx + 1) * (ny + 1) * (nz + 1)
    eye = np.eye(n)
    M = np.linalg.inv(np.stack([O.ilu_apply(K, eye[:, j], band) for j in range(n)], axis=1))
    A = K.toarray()
    i, j = np.nonzero(A)
    keep = np.abs(j - i - 1) <= (band if band else n)
    scale = np.abs(A).max()
    assert np.abs(M[i[keep], j[keep]] - A[i[keep], j[keep]]).max() <= 1e-12 * scale
    if band_kind == "np":
        # the entries left out are exactly the Ex-Ez and Ez-Ex couplings
        xnl, ynl = nx * (ny + 1) * (nz + 1), (nx + 1) * ny * (nz + 1)
        orient = lambda e: np.where(e < xnl, 0, np.where(e < xnl + ynl, 1, 2))  # noqa: E731
        xz = orient(i) + orient(j) == 2
        xz &= orient(i) != 1
        np.testing.assert_array_equal(~keep, xz)
        assert np.abs(M[i[~keep], j[~keep]] - A[i[~keep], j[~keep]]).max() > 1e-6 * scale


def test_bicgstab_with_ilu0_solves_a_small_system():
    """pre = 'I' is wired through Bicg_stab_p: on the 430-edge system the recurrence
    residual reaches 1e-7 within a few iterations and the true residual agrees.  (Both
    ILU(0) and SSOR stagnate near 1e-9 on this tiny model with air layers; the
    tolerance stays above that.)"""
    mesh, K, p1 = _tiny_aniso_system()
    x, it, _ = O.solve_krylov(1, mesh, K, p1, np.zeros(K.shape[0]), 1e-7, 100,
                              O.OracleOpts(pre="I", div_cor=False), ilu_band=0)
    assert it < 30
    assert np.linalg.norm(K @ x - p1) <= 2e-7 * np.linalg.norm(p1)


def test_converged_solve_matches_superlu():
    """The oracle's converged-solution solver (multigrid-preconditioned BiCGStab, used for the
    fixtures of meshes too large for SuperLU) reaches a 1e-15 residual and the impedances of
    the direct solution."""
    m = syn.small_aniso(n=16, seed=1, freqs=(0.05, 20.0))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    exd = np.zeros((m.nf, 2, m.nl), np.complex128)
    exm = np.zeros_like(exd)
    for k, ff in enumerate(m.freq):
        u1, u2, _, _, _ = O.direct_solve(om, ff)
        exd[k, 0], exd[k, 1] = u1, u2
        x1, x2, r1, r2, _ = O.converged_solve(om, ff, tol=1e-15)
        assert r1 < 1e-14 and r2 < 1e-14, (r1, r2)
        exm[k, 0], exm[k, 1] = x1, x2
    zd = O.impedances(om, exd)
    zm = O.impedances(om, exm)
    zd, zm = zd[..., 0::2] + 1j * zd[..., 1::2], zm[..., 0::2] + 1j * zm[..., 1::2]
    assert (np.abs(zm - zd) / np.abs(zd)).max() < 1e-7


def test_edge_prolongation_reproduces_constant_fields():
    """The lowest-order edge interpolation maps a constant coarse field to the same constant
    on every fine edge whose transverse nodes have both coarse neighbours."""
    m = syn.small_aniso(n=16, seed=0)
    P = O.edge_prolongation(m.a, m.b, m.c)
    cx, cy, cz = m.nx // 2, m.ny // 2, m.nz // 2
    u = np.concatenate([np.full(cx * (cy + 1) * (cz + 1), 1.0), np.full((cx + 1) * cy * (cz + 1), 2.0),
                        np.full((cx + 1) * (cy + 1) * cz, 3.0)])
    v = P @ u
    xnl, ynl = m.nx * (m.ny + 1) * (m.nz + 1), (m.nx + 1) * m.ny * (m.nz + 1)
    np.testing.assert_allclose(v[:xnl], 1.0, rtol=1e-14)
    np.testing.assert_allclose(v[xnl:xnl + ynl], 2.0, rtol=1e-14)
    np.testing.assert_allclose(v[xnl + ynl:], 3.0, rtol=1e-14)


def test_edge_prolongation_commutes_with_the_gradient():
    """The edge interpolation of the multigrid preconditioner maps discrete gradients to discrete
    gradients: P G_c phi = G_f (Pn phi) with Pn the trilinear nodal interpolation on the same nested
    non-uniform meshes -- the property that lets the coarse levels correct the gradient part of the
    error (and the nodal step's corrections survive the transfer)."""
    import scipy.sparse as sp
    m = syn.small_aniso(n=16, seed=0)
    nx, ny, nz = m.nx, m.ny, m.nz
    a1, b1, c1, _ = O.mesh_coarsen(m.a, m.b, m.c, m.sigma, 1, quirk=False)
    cx, cy, cz = len(a1), len(b1), len(c1)

    def interp_1d(h):
        lo, wlo, hi, whi = O._node_terms(np.asarray(h, float))
        n = len(h) + 1
        return sp.csr_matrix((np.concatenate([wlo, whi]), (np.tile(np.arange(n), 2), np.concatenate([lo, hi]))),
                             shape=(n, len(h) // 2 + 1))

    Pn = sp.kron(interp_1d(m.c), sp.kron(interp_1d(m.b), interp_1d(m.a))).tocsr()

    def interior(nx_, ny_, nz_):
        n = np.arange((nx_ + 1) * (ny_ + 1) * (nz_ + 1))
        i, j, k = n % (nx_ + 1), (n // (nx_ + 1)) % (ny_ + 1), n // ((nx_ + 1) * (ny_ + 1))
        return (i > 0) & (i < nx_) & (j > 0) & (j < ny_) & (k > 0) & (k < nz_)

    ic, ifn = interior(cx, cy, cz), interior(nx, ny, nz)
    Gc = O.node_gradient(cx, cy, cz, a1, b1, c1)
    Gf = O.node_gradient(nx, ny, nz, m.a, m.b, m.c)
    P = O.edge_prolongation(m.a, m.b, m.c)
    rng = np.random.default_rng(3)
    phi = rng.standard_normal(int(ic.sum())) + 1j * rng.standard_normal(int(ic.sum()))
    full = np.zeros(ic.size, complex)
    full[ic] = phi
    phif = (Pn @ full)
    assert np.abs(phif[~ifn]).max() == 0.0  # zero coarse boundary -> zero fine boundary
    lhs = P @ (Gc @ phi)
    rhs = Gf @ phif[ifn]
    np.testing.assert_allclose(lhs, rhs, rtol=0, atol=1e-12 * np.abs(rhs).max())


def test_gpu_vcycle_restatement_preconditions_bicgstab():
    """The oracle's restatement of the GPU's edge multigrid V-cycle is a working preconditioner:
    BiCGStab with it reaches a 1e-10 residual on the 16^3 anisotropic model with air at 0.01 and
    10 Hz in a few tens of iterations (the oracle of sfdx_vcycle_apply)."""
    from scipy.sparse.linalg import LinearOperator, bicgstab
    m = syn.small_aniso(n=16, nair=8, nz_earth=24, seed=0, freqs=(0.01, 10.0))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    for ff in m.freq:
        edc, _, _ = O.mt1d_anl(ff, O.column_conv(m.sigma, m.nx, m.ny, m.nz), m.c)
        K, p1, _ = O.assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, edc)
        Mv = LinearOperator(K.shape, lambda v, ff=ff: O.gpu_vcycle(om, ff, v), dtype=np.complex128)
        its = [0]
        x, info = bicgstab(K, p1, rtol=1e-10, atol=0.0, maxiter=80, M=Mv, callback=lambda _: its.__setitem__(0, its[0] + 1))
        rel = np.linalg.norm(p1 - K @ x) / np.linalg.norm(p1)
        assert rel < 1e-9 and its[0] < 60, (ff, rel, its[0])


def test_complex64_krylov_needs_the_split_vcycle():
    """Numerical premise of a complex64 Krylov iteration under the edge multigrid: with every
    vector stored in complex64, the V-cycle that carries its nodal corrections as a potential
    psi beside x (A(x + G psi) = K x - i w mu Ms G psi) lets BiCGStab reach 1e-12 as in FP64,
    while the same V-cycle adding G phi into x stalls (its gradient parts, ~1/(w mu sigma) in
    air, swamp the curl parts in complex64)."""
    m = syn.small_aniso(n=16, nair=8, nz_earth=24, seed=0, freqs=(0.01, 1.0))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    for ff in m.freq:
        its, rel, hist = O.complex64_vcycle_bicgstab(om, ff, split=True)
        assert rel < 1e-12 and its <= 32, (ff, its, rel, hist)
    its, rel, hist = O.complex64_vcycle_bicgstab(om, 0.01, split=False, maxit=40)
    assert rel > 1e-8, (its, rel, hist)
