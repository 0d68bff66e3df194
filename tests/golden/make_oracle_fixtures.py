"""Oracle fixtures of the benchmark workloads: the exact discrete answer of each
(frequency, polarisation) system of a seeded synthetic model, for the GPU parity
tests and the benchmark's impedance error against the oracle.

For every frequency the oracle assembles the reference's system (fd_assemb +
dcfast with the 1-D boundary values of mt1d_anl) and solves both polarisations
to a relative residual of 1e-15 with its own converged-solution solver
(oracle.converged_solve: multigrid-preconditioned BiCGStab, checked against
the assembled matrix; on small meshes it agrees with SuperLU to ~1e-9 in the
impedances, tests/test_oracle.py).  Stored in tests/golden/<workload>_oracle.npz:

  freq[nf]                      frequencies (Hz)
  z[nf, nrec, 2]                Zxy, Zyx (complex) at the model's receivers,
                                post_process with rd = 2 (the reference's
                                receiver stencil)
  edges[ne]                     a deterministic sample of earth edges (every
                                stride-th edge below the air layers)
  fields[nf, 2, ne]             the solution on those edges (complex)
  relres[nf, 2]                 final relative residuals
  iters[nf, 2]                  BiCGStab iterations

Usage: python tests/golden/make_oracle_fixtures.py <workload> [processes]
workloads: halfspace-cube, aniso-hills, large-inclusions.
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from sfd_excmg_gb300 import synthetic as syn  # noqa: E402

BUILDERS = {"halfspace-cube": syn.halfspace_cube, "aniso-hills": lambda: syn.aniso_hills(seed=0),
            "large-inclusions": lambda: syn.large_inclusions(seed=0)}
TOL = 1e-15


def earth_edges(m, stride):
    """Every stride-th edge whose z position lies below the air layers."""
    nx, ny, nz, nair = m.nx, m.ny, m.nz, m.nair
    xnl, ynl = nx * (ny + 1) * (nz + 1), (nx + 1) * ny * (nz + 1)
    e = np.arange(0, m.nl, stride)
    k = np.where(e < xnl, e // (nx * (ny + 1)),
                 np.where(e < xnl + ynl, (e - xnl) // ((nx + 1) * ny), (e - xnl - ynl) // ((nx + 1) * (ny + 1))))
    return e[k > nair]


def one(args):
    name, k = args
    m = BUILDERS[name]()
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    t = time.time()
    x1, x2, r1, r2, its = O.converged_solve(om, float(m.freq[k]), tol=TOL)
    out, _, _ = O.post_process(om, x1, x2, float(m.freq[k]), out_type=1, rd=2)
    print(f"{name} f={m.freq[k]:g}: relres {r1:.1e} {r2:.1e}, iterations {its}, {time.time() - t:.0f} s", flush=True)
    stride = max(1, m.nl // 600)
    e = earth_edges(m, stride)
    return k, out, x1[e], x2[e], (r1, r2), its


def main():
    name = sys.argv[1]
    procs = int(sys.argv[2]) if len(sys.argv) > 2 else 1
    m = BUILDERS[name]()
    edges = earth_edges(m, max(1, m.nl // 600))
    nf = m.nf
    z = np.zeros((nf, m.recv.shape[0], 2), np.complex128)
    fields = np.zeros((nf, 2, edges.size), np.complex128)
    relres = np.zeros((nf, 2))
    iters = np.zeros((nf, 2), np.int32)
    jobs = [(name, k) for k in range(nf)]
    if procs > 1:
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(one, jobs)
    else:
        res = [one(j) for j in jobs]
    for k, out, f1, f2, rr, its in res:
        z[k, :, 0] = out[:, 0] + 1j * out[:, 1]
        z[k, :, 1] = out[:, 2] + 1j * out[:, 3]
        fields[k, 0], fields[k, 1] = f1, f2
        relres[k] = rr
        iters[k] = its
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name.replace("-", "_") + "_oracle.npz")
    np.savez_compressed(path, freq=np.asarray(m.freq), z=z, edges=edges, fields=fields, relres=relres, iters=iters)
    print("wrote", path, "max relres", relres.max())


if __name__ == "__main__":
    main()
