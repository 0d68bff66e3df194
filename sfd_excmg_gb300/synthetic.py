"""Seeded synthetic models with the shapes of the benchmark configurations.

No public model data ships with the reference beyond the DTM1 generator, so
the benchmark and tests build their models here: seeded
``numpy.random.default_rng`` draws with the sizes, conductivity ranges and
frequency bands of the benchmark workloads.  Meshes follow the reference's
conventions: a core of uniform cells, geometric padding, and air layers that
mirror the deepest earth layers (read_input, file_opt.f90:52).
"""
from __future__ import annotations

import numpy as np

from .model import Model

SIGMA_AIR = 1e-9


def padded_axis(ncore: int, h: float, npad: int, growth: float, lo: bool = True, hi: bool = True) -> np.ndarray:
    pad = h * growth ** np.arange(1, npad + 1)
    parts = []
    if lo:
        parts.append(pad[::-1])
    parts.append(np.full(ncore, h))
    if hi:
        parts.append(pad)
    return np.concatenate(parts)


def euler_tensor(rho3, strike, dip, slant) -> np.ndarray:
    """Conductivity tensor from principal resistivities and Euler angles
    (rotation order of conduc_cal, sfd_excmg/input.py:123-141).  Returns
    (xx, yy, zz, xy, xz, yz)."""
    main = np.diag(1.0 / np.asarray(rho3, dtype=np.float64))
    cs, ss = np.cos(strike), np.sin(strike)
    cd, sd = np.cos(dip), np.sin(dip)
    cl, sl = np.cos(slant), np.sin(slant)
    Rs = np.array([[cs, -ss, 0], [ss, cs, 0], [0, 0, 1]])
    Rd = np.array([[1, 0, 0], [0, cd, -sd], [0, sd, cd]])
    Rl = np.array([[cl, -sl, 0], [sl, cl, 0], [0, 0, 1]])
    D = Rs @ Rd @ Rl
    S = D @ main @ D.T
    return np.array([S[0, 0], S[1, 1], S[2, 2], S[0, 1], S[0, 2], S[1, 2]])


def _mesh(ncx, ncy, ncz, h, npad_xy, growth_xy, npad_bot, growth_z, nair):
    a = padded_axis(ncx, h, npad_xy, growth_xy)
    b = padded_axis(ncy, h, npad_xy, growth_xy)
    ce = padded_axis(ncz, h, npad_bot, growth_z, lo=False, hi=True)
    c = np.concatenate([ce[::-1][:nair], ce])  # air mirrors the deepest earth layers
    return a, b, c


def _centres(h):
    x = np.concatenate([[0], np.cumsum(h)])
    x = x - x[-1] / 2
    return (x[:-1] + x[1:]) / 2


def _core_receivers(a, b, npad, ncx, ncy, nrx, nry):
    xc, yc = _centres(a), _centres(b)
    ix = npad + np.linspace(0, ncx - 1, nrx).round().astype(int)
    iy = npad + np.linspace(0, ncy - 1, nry).round().astype(int)
    X, Y = np.meshgrid(xc[ix], yc[iy], indexing="xy")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)


def halfspace(n: int = 16, nair: int = 4, nz_earth: int = 12, h: float = 100.0, rho: float = 100.0,
              freqs=(10.0,), growth: float = 1.2, sigma_air: float = SIGMA_AIR) -> Model:
    """Small homogeneous half-space (known answer: rho_a = rho, phase = 45 deg)."""
    a = np.full(n, h)
    b = np.full(n, h)
    ce = np.full(nz_earth, h / 2) * growth ** np.arange(nz_earth)
    c = np.concatenate([ce[::-1][:nair], ce])
    nz = nz_earth + nair
    sig = np.zeros((6, n * n * nz))
    sig[0:3] = 1.0 / rho
    sig[0:3, : nair * n * n] = sigma_air
    xc = _centres(a)
    recv = np.array([[xc[n // 2 - 1], xc[n // 2 - 1], 0.0], [xc[n // 2], xc[n // 2 + 1], 0.0]])
    return Model(n, n, nz, nair, a, b, c, sig, np.asarray(freqs, float), recv)


def halfspace_cube() -> Model:
    """Plain EXCMG case: 32^3 core cells of 100 m, 8 padding cells (x1.3) per side,
    8 air layers; 100 ohm-m half-space with a 1 ohm-m cube of 8^3 cells whose
    top is at 400 m depth; 4 frequencies over 0.01-100 Hz; 3 levels, tol 1e-8."""
    npad, nc = 8, 32
    a, b, c = _mesh(nc, nc, nc, 100.0, npad, 1.3, npad, 1.3, 8)
    nx, ny, nz, nair = len(a), len(b), len(c), 8
    sig = np.zeros((6, nx * ny * nz))
    sig[0:3] = 1e-2
    sig[0:3, : nair * nx * ny] = 1e-8
    s3 = sig.reshape(6, nz, ny, nx)
    i0 = npad + nc // 2 - 4
    k0 = nair + 4  # 4 cells of 100 m below the surface
    s3[0:3, k0:k0 + 8, i0:i0 + 8, i0:i0 + 8] = 1.0
    freq = np.logspace(-2, 2, 4)
    recv = _core_receivers(a, b, npad, nc, nc, 16, 16)
    return Model(nx, ny, nz, nair, a, b, c, sig, freq, recv, level=3, eps=1e-8, solver=1, out_type=1)


def aniso_hills(seed: int = 0, hills: bool = True, nblocks: int = 20) -> Model:
    """Anisotropic model with topography: 64x64x48 core cells of 50 m, 8 lateral
    padding cells, 8 bottom padding cells, 24 air layers (80x80x80); 20 blocks
    with principal resistivities log-uniform in 1-1000 ohm-m and Euler angles
    U[0, pi); Gaussian hills (amplitude <= 500 m, widths 300-800 m) filled with
    earth conductivity; 8 frequencies over 0.001-1000 Hz; 32x32 receivers."""
    rng = np.random.default_rng(seed)
    npad, ncx, ncz, nair = 8, 64, 48, 24
    a, b, c = _mesh(ncx, ncx, ncz, 50.0, npad, 1.3, npad, 1.3, nair)
    nx, ny, nz = len(a), len(b), len(c)
    sig = np.zeros((6, nx * ny * nz))
    sig[0:3] = 1e-2  # 100 ohm-m background
    s3 = sig.reshape(6, nz, ny, nx)
    for _ in range(nblocks):
        rho3 = 10 ** rng.uniform(0, 3, 3)
        ang = rng.uniform(0, np.pi, 3)
        t = euler_tensor(rho3, *ang)
        sx, sy, sz = rng.integers(4, 20, 3)
        x0 = rng.integers(npad, npad + ncx - sx)
        y0 = rng.integers(npad, npad + ncx - sy)
        z0 = rng.integers(nair, nair + ncz - sz)
        s3[:, z0:z0 + sz, y0:y0 + sy, x0:x0 + sx] = t[:, None, None, None]
    s3[:, :nair] = 0
    s3[0:3, :nair] = SIGMA_AIR
    if hills:
        xc, yc = _centres(a), _centres(b)
        X, Y = np.meshgrid(xc, yc, indexing="xy")
        topo = np.zeros_like(X)
        for _ in range(4):
            amp = rng.uniform(100, 500)
            w = rng.uniform(300, 800)
            cx0, cy0 = rng.uniform(-1200, 1200, 2)
            topo += amp * np.exp(-((X - cx0) ** 2 + (Y - cy0) ** 2) / (2 * w * w))
        topo = np.minimum(topo, 500.0)
        zc = np.concatenate([[0], np.cumsum(c)]) - c[:nair].sum()
        zmid = (zc[:-1] + zc[1:]) / 2  # negative above the surface
        for k in range(nair):
            under = topo >= -zmid[k]
            if under.any():
                for q in range(6):
                    s3[q, k][under] = s3[q, nair][under]
    freq = np.logspace(-3, 3, 8)
    recv = _core_receivers(a, b, npad, ncx, ncx, 32, 32)
    return Model(nx, ny, nz, nair, a, b, c, sig, freq, recv, level=3, eps=1e-8, solver=1, out_type=1)


def grf(shape, corr_len, rng) -> np.ndarray:
    """Gaussian random field with unit variance and Gaussian correlation of length corr_len (cells)."""
    k = [np.fft.fftfreq(n) for n in shape]
    K2 = sum(np.meshgrid(*[kk ** 2 for kk in k], indexing="ij"))
    spec = np.exp(-2 * (np.pi * corr_len) ** 2 * K2 / 2)
    f = np.fft.ifftn(np.fft.fftn(rng.standard_normal(shape)) * np.sqrt(spec)).real
    return (f - f.mean()) / (f.std() + 1e-30)


def multi_model_batch(seed: int = 0, nmodels: int = 8, nf: int = 16) -> list:
    """Batched multi-model case: `nmodels` models whose cell counts per axis
    (padding and air included) are drawn uniformly from {48, 56, ..., 96}
    (multiples of 8, 3 levels): 50 m core cells, 4 lateral padding cells per
    side (x1.3), 4 bottom padding cells, 8 air layers; isotropic log10(rho)
    Gaussian random field (mean 2, std 0.5, correlation 5 cells); nf
    frequencies over 0.001-1000 Hz; 8x8 receivers over the core."""
    rng = np.random.default_rng(seed)
    sizes = np.arange(48, 97, 8)
    models = []
    for _ in range(nmodels):
        nx, ny, nz = (int(v) for v in rng.choice(sizes, 3))
        npad, nair, nbot = 4, 8, 4
        ncx, ncy, ncz = nx - 2 * npad, ny - 2 * npad, nz - nair - nbot
        a, b, c = _mesh(ncx, ncy, ncz, 50.0, npad, 1.3, nbot, 1.3, nair)
        sig = np.zeros((6, nx * ny * nz))
        s3 = sig.reshape(6, nz, ny, nx)
        f = 2.0 + 0.5 * grf((nz - nair, ny, nx), 5.0, rng)
        s3[0:3, nair:] = (10.0 ** -f)[None]
        s3[0:3, :nair] = SIGMA_AIR
        freq = np.logspace(-3, 3, nf)
        recv = _core_receivers(a, b, npad, ncx, ncy, 8, 8)
        models.append(Model(nx, ny, nz, nair, a, b, c, sig, freq, recv, level=3, eps=1e-8, solver=1, out_type=1))
    return models


def large_inclusions(seed: int = 0) -> Model:
    """Large single model: 128x128x96 core cells of 25 m, 16 lateral padding
    cells per side, 12 bottom padding, 36 air layers (160x160x144, 11.2 M edges);
    layers 100/10/1000 ohm-m plus 10 random anisotropic boxes (0.5-5000 ohm-m);
    6 frequencies over 0.01-100 Hz; 4 levels, tol 1e-7."""
    rng = np.random.default_rng(seed)
    npad, nc, ncz, nbot, nair = 16, 128, 96, 12, 36
    a, b, c = _mesh(nc, nc, ncz, 25.0, npad, 1.2, nbot, 1.3, nair)
    nx, ny, nz = len(a), len(b), len(c)
    sig = np.zeros((6, nx * ny * nz))
    s3 = sig.reshape(6, nz, ny, nx)
    nze = nz - nair
    layer = np.where(np.arange(nze) < 24, 1e-2, np.where(np.arange(nze) < 60, 1e-1, 1e-3))
    s3[0:3, nair:] = layer[None, :, None, None]
    for _ in range(10):
        rho3 = 10 ** rng.uniform(np.log10(0.5), np.log10(5000), 3)
        t = euler_tensor(rho3, *rng.uniform(0, np.pi, 3))
        sx, sy, sz = rng.integers(8, 32, 3)
        x0 = rng.integers(npad, npad + nc - sx)
        y0 = rng.integers(npad, npad + nc - sy)
        z0 = rng.integers(nair, nair + ncz - sz)
        s3[:, z0:z0 + sz, y0:y0 + sy, x0:x0 + sx] = t[:, None, None, None]
    s3[:, :nair] = 0
    s3[0:3, :nair] = SIGMA_AIR
    freq = np.logspace(-2, 2, 6)
    recv = _core_receivers(a, b, npad, nc, nc, 32, 32)
    return Model(nx, ny, nz, nair, a, b, c, sig, freq, recv, level=4, eps=1e-7, solver=1, out_type=1)


def grf_inversion(seed: int = 0) -> Model:
    """Adjoint case: the aniso_hills mesh without hills, isotropic log10(rho) Gaussian
    random field (mean 2, std 0.5, correlation 5 cells), 6 frequencies."""
    rng = np.random.default_rng(seed)
    m = aniso_hills(seed, hills=False, nblocks=0)
    nze = m.nz - m.nair
    f = 2.0 + 0.5 * grf((nze, m.ny, m.nx), 5.0, rng)
    s3 = m.sigma.reshape(6, m.nz, m.ny, m.nx)
    s3[:] = 0
    s3[0:3, m.nair:] = (10.0 ** -f)[None]
    s3[0:3, : m.nair] = SIGMA_AIR
    m.freq = np.logspace(-3, 3, 6)
    return m


def grf_inversion_true(seed: int = 0) -> Model:
    """The model that generates the data of the adjoint case: grf_inversion(seed) with log10(rho)
    of the earth perturbed by 0.25 x a second Gaussian random field
    (correlation 5 cells)."""
    m = grf_inversion(seed)
    rng = np.random.default_rng(seed + 1000)
    nze = m.nz - m.nair
    s3 = m.sigma.reshape(6, m.nz, m.ny, m.nx)
    s3[0:3, m.nair:] *= (10.0 ** (-0.25 * grf((nze, m.ny, m.nx), 5.0, rng)))[None]
    return m


def small_aniso(n: int = 16, nair: int = 8, nz_earth: int = 24, seed: int = 0, freqs=(0.1, 10.0)) -> Model:
    """Small anisotropic model with random tensor blocks and graded spacings (tests)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(60, 140, n)
    b = rng.uniform(60, 140, n)
    ce = 40.0 * 1.15 ** np.arange(nz_earth)
    c = np.concatenate([ce[::-1][:nair], ce])
    nz = nz_earth + nair
    sig = np.zeros((6, n * n * nz))
    sig[0:3] = 1e-2
    s3 = sig.reshape(6, nz, n, n)
    for _ in range(4):
        t = euler_tensor(10 ** rng.uniform(0, 3, 3), *rng.uniform(0, np.pi, 3))
        x0, y0 = rng.integers(2, n - 6, 2)
        z0 = rng.integers(nair, nz - 6)
        s3[:, z0:z0 + 5, y0:y0 + 5, x0:x0 + 5] = t[:, None, None, None]
    s3[:, :nair] = 0
    s3[0:3, :nair] = SIGMA_AIR
    xc = _centres(a)
    yc = _centres(b)
    recv = np.array([[xc[n // 2], yc[n // 2], 0.0], [xc[n // 2 - 2], yc[n // 2 + 1], 0.0]])
    return Model(n, n, nz, nair, a, b, c, sig, np.asarray(freqs, float), recv)


def dtm1(sigma_air: float = SIGMA_AIR) -> Model:
    """The reference's own example model DTM1.0 (generator sfd_excmg/input.py:6-95,
    receivers :97-117), restated: 128x128 cells laterally, 128 earth layers under 64
    air layers (nz = 192, ~9.6 M edges); 16 blocks of 8 equal cells per axis with
    block widths 29.2, 16.2, 9, 5 km towards the 8 central 5 km blocks, vertical
    blocks 10 x 5 km then 5 km * 1.8^n; 100 ohm-m half-space with three isotropic
    bodies (10, 1 and 10^4 ohm-m); air layers mirror the deepest earth layers;
    frequencies 0.001-1 Hz; 4 receiver lines of 17 sites; 4 levels, tol 1e-10,
    BiCGStab."""
    edge = [2.92e4, 1.62e4, 9e3, 5e3]
    a0 = np.array(edge + [5e3] * 8 + edge[::-1])
    c0 = np.array([5e3] * 10 + [5e3 * 1.8 ** (i + 1) for i in range(6)])
    a = np.repeat(a0 / 8, 8)
    b = a.copy()
    ce = np.repeat(c0 / 8, 8)
    nair = 64
    c = np.concatenate([ce[::-1][:nair], ce])
    nx, ny, nze = 128, 128, 128
    nz = nze + nair
    s3 = np.zeros((6, nz, ny, nx))
    s3[0:3, nair:] = 1e-2
    bodies = (((32, 96), (60, 68), (8, 32), 0.1), ((40, 64), (60, 100), (32, 40), 1.0),
              ((64, 88), (28, 68), (32, 80), 1e-4))
    for (x0, x1), (y0, y1), (z0, z1), s in bodies:
        s3[0:3, nair + z0:nair + z1, y0:y1, x0:x1] = s
    s3[0:3, :nair] = sigma_air
    sites = np.array([-37.5, -32.5, -27.5, -22.5, -17.5, -12.5, -7.5, -2.5, 0.0, 2.5, 7.5, 12.5, 17.5, 22.5, 27.5,
                      32.5, 37.5]) * 1e3
    z = np.zeros_like(sites)
    recv = np.concatenate([np.stack([sites, z, z], 1), np.stack([z - 15e3, sites, z], 1),
                           np.stack([z, sites, z], 1), np.stack([z + 15e3, sites, z], 1)])
    freq = np.array([0.001, 0.01, 0.1, 1.0])
    return Model(nx, ny, nz, nair, a, b, c, s3.reshape(6, -1), freq, recv, level=4, eps=1e-10, solver=1, out_type=1)
