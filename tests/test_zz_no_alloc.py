"""The allocation-free residual entry point (sfdx_residual_noalloc).

It exists for callers that cannot call cudaMalloc (their device memory is
owned by their own pool or by another runtime, or they must not allocate in
a hot loop): they pass device buffers they already own, and the library uses
only a fixed device array reserved when it is loaded.  The test calls it
through the C ABI twice in a row (the shared array keeps the first call's
data, which must not leak into the second) and checks both results against
the regular, allocating operator entry point.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_residual_noalloc_matches_allocating_entry_point():
    import torch

    import sfd_excmg_gb300 as S
    from sfd_excmg_gb300 import capi
    from sfd_excmg_gb300 import synthetic as syn

    m = syn.small_aniso(n=16, seed=11)
    freqs = np.array([0.01, 1.0, 30.0])
    ns = len(freqs)
    rng = np.random.default_rng(42)
    L = capi.lib()
    d = lambda v: np.ascontiguousarray(v, dtype=np.float64)
    a, b, c = d(m.a), d(m.b), d(m.c)
    sig = torch.from_numpy(d(m.sigma)).cuda()
    for call in range(2):
        x = np.ascontiguousarray(rng.standard_normal((m.nl, ns)) + 1j * rng.standard_normal((m.nl, ns)))
        rhs = np.ascontiguousarray(rng.standard_normal((m.nl, ns)) + 1j * rng.standard_normal((m.nl, ns)))
        dx = torch.from_numpy(x.view(np.float64).ravel().copy()).cuda()
        db = torch.from_numpy(rhs.view(np.float64).ravel().copy()).cuda()
        dr = torch.zeros_like(dx)
        rel = np.zeros(ns)
        torch.cuda.synchronize()
        rc = L.sfdx_residual_noalloc(m.nx, m.ny, m.nz, capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                     ctypes.c_void_p(sig.data_ptr()), ns, capi.dptr(d(freqs)),
                                     ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(dx.data_ptr()),
                                     ctypes.c_void_p(dr.data_ptr()), capi.dptr(rel), None)
        assert rc == 0, capi.ERRORS.get(rc, rc)
        r = dr.cpu().numpy().view(np.complex128).reshape(m.nl, ns)
        # the same quantities from the regular entry point (it allocates)
        y = S.apply_operator(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, freqs, x)
        r_ref = rhs - y
        assert np.abs(r - r_ref).max() <= 1e-12 * np.abs(r_ref).max(), call
        rel_ref = np.linalg.norm(r_ref, axis=0) / np.linalg.norm(rhs, axis=0)
        np.testing.assert_allclose(rel, rel_ref, rtol=1e-12)


def test_residual_noalloc_rejects_sizes_above_its_limit():
    import torch

    from sfd_excmg_gb300 import capi

    L = capi.lib()
    one = np.ones(2000)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")  # never read: the size check comes first
    dummy = ctypes.c_void_p(buf.data_ptr())
    rel = np.zeros(1)
    rc = L.sfdx_residual_noalloc(2000, 4, 4, capi.dptr(one), capi.dptr(one), capi.dptr(one), dummy, 1,
                                 capi.dptr(np.ones(1)), dummy, dummy, dummy, capi.dptr(rel), None)
    assert rc == 10  # SFDX_ERR_NOMEM: above the fixed array's limit
