"""Runs the reference algorithm (oracle restatement: lexicographic SSOR-BiCGStab with the
divergence correction, fwd_acc=0 plain path from a zero guess, maxit 5000, tol 1e-8) on the
synthetic config-2 model for one frequency and writes iterations, residuals, CPU seconds and
impedances to tests/golden/aniso_hills_reference/f<k>.json.

Usage: python tests/golden/make_aniso_hills_reference.py <k> [maxit]
The CPU time per iteration and the iteration counts feed the CPU-baseline leg of bench.py.
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from sfd_excmg_gb300 import synthetic as syn  # noqa: E402


def main():
    k = int(sys.argv[1])
    maxit = int(sys.argv[2]) if len(sys.argv) > 2 else 5000
    m = syn.aniso_hills(seed=0)
    ff = float(m.freq[k])
    t0 = time.process_time()
    conv = O.column_conv(m.sigma, m.nx, m.ny, m.nz)
    edc, _, _ = O.mt1d_anl(ff, conv, m.c)
    K, p1, p2 = O.assemble(m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma, ff, edc)
    t_setup = time.process_time() - t0
    mesh = (m.nx, m.ny, m.nz, m.a, m.b, m.c, m.sigma)
    out = {"freq": ff, "nl": int(m.nl), "maxit": maxit, "tol": m.eps, "setup_cpu_s": t_setup, "pol": []}
    xs = []
    for p in (p1, p2):
        t1 = time.process_time()
        x, it, err = O.solve_krylov(1, mesh, K, p, np.zeros(m.nl), m.eps, maxit, O.OracleOpts())
        dt = time.process_time() - t1
        rr = float(np.linalg.norm(p - K @ x) / np.linalg.norm(p))
        out["pol"].append({"iters": int(it), "cpu_s": dt, "cpu_s_per_iter": dt / max(it, 1), "true_relres": rr,
                           "err_rec_tail": [float(e) for e in err[max(0, it - 5):it]]})
        xs.append(x)
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    z, _, _ = O.post_process(om, xs[0], xs[1], ff, 1, 2)
    out["Z"] = z.tolist()
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "aniso_hills_reference")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, f"f{k}.json"), "w") as f:
        json.dump(out, f)
    print(json.dumps({kk: v for kk, v in out.items() if kk != "Z"}))


if __name__ == "__main__":
    main()
