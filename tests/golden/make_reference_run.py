"""A complete run of the reference algorithm (the oracle's restatement of doublemode_acc with
the reference's compiled-in options, oracle.reference_frequency) on a benchmark workload at the
configuration's own tolerance: iterations per level and system, solve seconds on this machine,
final residuals and the impedance error against the oracle fixture of the same workload.
Written to tests/golden/<workload>_reference.json; bench.py scales its bounded CPU sample
(cpu_baseline) by these iteration counts.

Usage: python tests/golden/make_reference_run.py <workload> [processes]
"""
import json
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from sfd_excmg_gb300 import synthetic as syn  # noqa: E402

BUILDERS = {"halfspace-cube": syn.halfspace_cube, "aniso-hills": lambda: syn.aniso_hills(seed=0),
            "large-inclusions": lambda: syn.large_inclusions(seed=0)}


def one(args):
    name, k, pol = args
    m = BUILDERS[name]()
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv, m.level, m.eps, 1, 1)
    secs, u, rr, infos = O.reference_frequency(om, k, m.eps, pols=(pol,))
    its = [[lev, it[pol] if it else None] for lev, it in infos]
    print(f"{name} f={m.freq[k]:g} pol {pol}: {secs:.0f} s, levels {its}, relres {rr[pol]:.2e}", flush=True)
    return k, pol, secs, u[pol], rr[pol], its


def main():
    name = sys.argv[1]
    procs = int(sys.argv[2]) if len(sys.argv) > 2 else 1
    m = BUILDERS[name]()
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(one, [(name, k, pol) for k in range(m.nf) for pol in (0, 1)])
    by = {(r[0], r[1]): r for r in res}
    here = os.path.dirname(os.path.abspath(__file__))
    fxp = os.path.join(here, name.replace("-", "_") + "_oracle.npz")
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    zerr = None
    if os.path.exists(fxp):
        zref = np.load(fxp)["z"]
        zerr = []
        for k in range(m.nf):
            out, _, _ = O.post_process(om, by[(k, 0)][3], by[(k, 1)][3], float(m.freq[k]), out_type=1, rd=2)
            z = np.stack([out[:, 0] + 1j * out[:, 1], out[:, 2] + 1j * out[:, 3]], 1)
            zerr.append(float((np.abs(z - zref[k]) / np.abs(zref[k])).max()))
    doc = {"workload": name, "eps": m.eps, "freq": [float(f) for f in m.freq],
           "seconds": [[by[(k, p)][2] for p in (0, 1)] for k in range(m.nf)],
           "relres": [[by[(k, p)][4] for p in (0, 1)] for k in range(m.nf)],
           # per frequency: [[level, [xy, yx]], ...] (levels 1-2: exact solves, no iterations)
           "iterations": [[[lev, [by[(k, 0)][5][q][1], by[(k, 1)][5][q][1]] if by[(k, 0)][5][q][1] is not None
                            else []] for q, (lev, _) in enumerate(by[(k, 0)][5])] for k in range(m.nf)],
           "z_rel_err_vs_oracle_per_frequency": zerr,
           "machine": f"the x86 build container, {procs} processes of one system each"}
    path = os.path.join(here, name.replace("-", "_") + "_reference.json")
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
