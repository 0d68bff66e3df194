#!/usr/bin/env python3
"""Benchmark: MT forward solves/s of the GB300 solver on the anisotropic
topography workload.

Workload: anisotropic model with Gaussian hills, 64x64x48 core cells of 50 m
(80x80x80 with padding and air, 1,574,640 complex edge unknowns), 8
frequencies over 0.001-1000 Hz x 2 polarisations = 16 systems, EXCMG with 3
levels, finest tolerance 1e-10 (the tolerance at which the mixed-precision
impedances agree with the FP64 ones to ~1e-5), 32x32 receivers.  Solver:
GPBiCG with the multi-colour SSOR, complex64 iterations with FP64 reliable
residual updates, consistent gradient-space correction between restart
cycles of 40 iterations.  Synthetic, seeded (numpy default_rng(0)); the
reference publishes no model files for it.

A step = one complete forward solve of all 16 systems (both coarse levels,
prolongations, the finest level) followed by the impedances at the 1024
receivers.  `value` is solves/s with the conductivity resident in HBM;
`e2e` is the same through the C-ABI call sfdx_fwd_solve with host buffers
(H2D of sigma and D2H of all fields inside the timed region) followed by
sfdx_impedance.  The per-step working set (~4 GB) is far larger than L2, so
no flush is needed between steps.  The same solve in plain FP64 is timed
after the run (fp64_solves_per_s) and the impedances of the two compared.

The line also carries `adjoint`: the misfit-gradient case (the same mesh without
hills, isotropic log10 rho Gaussian random field, 6 frequencies, data from a
perturbed model with 2 % noise) -- forward solve + misfit and adjoint solves +
per-cell contraction timed with CUDA events, the ratio of the two, and the
mixed-precision gradient against the FP64 GPU adjoint (`--fd-cells N` adds
central differences at N random cells).  `--workload multi-model` times 8 models of
uneven meshes (256 systems) solved concurrently through sfdx_plan_solve_batch
against the same plans one after another.

`--impl reference` times the reference algorithm's CPU restatement (the
oracle: FP64 CSR, lexicographic SSOR-BiCGStab, serial per system) on the
host cores, one thread per system, as a bounded sample scaled to full solves
(see cpu_sample()).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
REF_SAMPLE_ITERS = 6


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        self.p = None
        self.index = index

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as td
        td.barrier()


def max_over_ranks(x, world):
    """The slowest rank's time (replicas run in step; the job takes the longest)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as td
    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step, steps, world, ms_max):
    """Units per second of the whole job: every rank processes its own replica of the
    step (weak scaling), timed by the slowest rank."""
    return units_per_rank_step * steps * world / (ms_max / 1e3)


SOLVER = {"bicgstab": 1, "tfqmr": 2, "gpbicg": 3, "bicg": 4, "cocr": 6}


# Divergence handling of the benchmark solves: the consistent gradient-space
# correction between GPBiCG restart cycles of 40 iterations (nodal PCG to 1e-2).
GC_OPTS = dict(div_cor=2, corr_intv=40, corr_tol=1e-2)


USE_GRAPHS = 1  # CUDA-graph capture of the Krylov check intervals (--no-graphs: 0)


def solve_opts(precision, solver="bicgstab", div_cor=2, eps=1e-10, corr_intv=None, level=3):
    import sfd_excmg_gb300 as S
    o = dict(excmg=1, level=level, eps=eps, precision=S.MIXED if precision == "mixed" else S.FP64,
             solver=SOLVER[solver], use_graphs=USE_GRAPHS)
    o.update(GC_OPTS if div_cor == 2 else dict(div_cor=div_cor))
    if corr_intv:
        o["corr_intv"] = corr_intv
    return o


# Workloads: the default anisotropic topography model, the large single model
# (128x128x96 core cells, 4 levels, tol 1e-7) and the reference's own DTM1
# example (4 levels, tol 1e-10) whose CPU times the reference publishes.
WORKLOADS = {
    "aniso-hills": ("aniso-hills: anisotropic 20-block model with Gaussian hills, 64x64x48 core cells of 50 m (80x80x80, "
             "1,574,640 edges), 8 freqs 1e-3..1e3 Hz x 2 pols, EXCMG 3 levels, tol {eps:g}, 32x32 receivers", 1e-10),
    "large-inclusions": ("large-inclusions: 128x128x96 core cells of 25 m + 16 padding per side, 12 bottom, 36 air (160x160x144, "
             "11,203,024 edges), 3 layers + 10 anisotropic boxes, 6 freqs 0.01..100 Hz x 2 pols, EXCMG 4 levels, "
             "tol {eps:g}", 1e-7),
    "multi-model": ("multi-model: 8 models per batch, cells per axis drawn from {{48,...,96}} (padding and air included), isotropic "
             "log10 rho GRF (mean 2, std 0.5, corr 5 cells), 16 freqs 1e-3..1e3 Hz x 2 pols = 256 systems, EXCMG 3 "
             "levels, tol {eps:g}, one host thread + stream per model", 1e-10),
    "dtm1": ("dtm1: the reference's DTM1.0 example (input.py), 128x128x192 cells incl. 64 air layers "
             "(9,568,704 edges), 4 freqs 0.001..1 Hz x 2 pols, EXCMG 4 levels, tol {eps:g}, 68 receivers", 1e-10),
}
# Reference CPU time for DTM1 (EXCMG, 4 levels, tol 1e-10; Xeon Gold 6248R, serial):
# 93.62 + 76.84 + 45.95 + 63.31 s for the four frequencies x two polarisations.
PUBLISHED_SOLVES_PER_S = {"dtm1": 8.0 / (93.62 + 76.84 + 45.95 + 63.31)}
# DRAM bytes (read + write) of one multi-colour SSOR application on the aniso-hills
# finest level, summed over its 11 colour launches from one ncu capture
# (profiles/mc_ssor_sweep_aniso_hills.md): 1528.6 MB read + 128.2 MB written.
SSOR_TRAFFIC = {"aniso-hills": 1656834048}


def make_workload(name):
    from sfd_excmg_gb300 import synthetic as syn
    if name == "large-inclusions":
        return syn.large_inclusions(seed=0)
    if name == "dtm1":
        return syn.dtm1()
    return syn.aniso_hills(seed=0)


def cpu_sample(model, freqs_idx, threads, iters=REF_SAMPLE_ITERS):
    """Bounded sample of the reference algorithm on the host cores.

    Per system (one thread each, the oracle releases the GIL): assembly of the
    finest-level CSR (fd_assemb + dcfast), then `iters` iterations of
    SSOR-BiCGStab (ssorfac + lusol + zamux, serial).  Returns the wall time of
    the parallel sample and the mean per-iteration / set-up seconds.
    """
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    import ctypes

    L = O.lib()

    def one(k):
        ff = float(model.freq[k])
        t0 = time.perf_counter()
        conv = O.column_conv(model.sigma, model.nx, model.ny, model.nz)
        edc, _, _ = O.mt1d_anl(ff, conv, model.c)
        K, p1, _ = O.assemble(model.nx, model.ny, model.nz, model.a, model.b, model.c, model.sigma, ff, edc)
        t1 = time.perf_counter()
        ia = np.ascontiguousarray(K.indptr, np.int64)
        ja = np.ascontiguousarray(K.indices, np.int32)
        km = np.ascontiguousarray(K.data)
        x = np.zeros(model.nl, np.complex128)
        L.orc_bicgstab_fixed(ctypes.c_int64(model.nl), km.ctypes.data_as(ctypes.c_void_p),
                             ia.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                             ja.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), p1.ctypes.data_as(ctypes.c_void_p),
                             x.ctypes.data_as(ctypes.c_void_p), iters)
        t2 = time.perf_counter()
        return t1 - t0, (t2 - t1) / iters

    t = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, freqs_idx))
    wall = time.perf_counter() - t
    return wall, float(np.mean([r[1] for r in res])), float(np.mean([r[0] for r in res]))


def reference_iterations():
    """Iterations the reference algorithm needs per aniso-hills system (tests/golden/aniso_hills_reference, made by
    tests/golden/make_aniso_hills_reference.py: plain path, zero guess, lexicographic SSOR + divergence correction)."""
    d = os.path.join(ROOT, "tests", "golden", "aniso_hills_reference")
    its = []
    if os.path.isdir(d):
        for fn in sorted(os.listdir(d)):
            if fn.endswith(".json"):
                with open(os.path.join(d, fn)) as f:
                    its += [p["iters"] for p in json.load(f)["pol"]]
    return its


def run_reference(args, rank, world):
    if rank != 0:
        return
    from sfd_excmg_gb300 import synthetic as syn
    m = syn.aniso_hills(seed=0)
    ns = 2 * m.nf
    threads = max(1, min(ns, os.cpu_count() or 1))
    its = reference_iterations()
    n_it = float(np.mean(its)) if its else float("nan")
    vals = []
    for _ in range(args.warmup):
        cpu_sample(m, list(range(m.nf)) * 2, threads, iters=2)
    samples = []
    for _ in range(args.steps):
        wall, t_it, t_setup = cpu_sample(m, list(range(m.nf)) * 2, threads)
        # projected time of the full solve of all systems on `threads` cores
        per_system = t_setup + n_it * t_it
        proj = per_system * ns / threads
        vals.append(ns / proj)
        samples.append((wall, t_it, t_setup))
    v = float(np.median(vals))
    line = {
        "impl": "reference", "metric": "MT solves/s", "value": v, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "ms_per_step": float(np.median([s[0] for s in samples]) * 1e3),
        "config": {"workload": WORKLOADS["aniso-hills"][0].format(eps=WORKLOADS["aniso-hills"][1]),
                   "solver": "SSOR-BiCGStab FP64 CSR (reference algorithm, oracle restatement)"},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": (f"per system: finest-level assembly + {REF_SAMPLE_ITERS} SSOR-BiCGStab iterations; "
                                    f"scaled by the reference algorithm's mean iteration count {n_it:.0f} "
                                    f"(tests/golden/aniso_hills_reference); {threads} systems in parallel")},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl")
    import sfd_excmg_gb300 as S
    from sfd_excmg_gb300 import capi
    from sfd_excmg_gb300 import synthetic as syn

    m = make_workload(args.workload)
    eps = args.eps if args.eps else WORKLOADS[args.workload][1]
    ns = 2 * m.nf
    opts = solve_opts(args.precision, args.solver, args.div_cor, eps, args.corr_intv, m.level)
    plan = S.Plan(m, **opts)
    stream = torch.cuda.Stream()
    plan.set_stream(stream.cuda_stream)
    sig = torch.from_numpy(np.ascontiguousarray(m.sigma)).to("cuda")
    fields = torch.empty((m.nf, 2, m.nl, 2), dtype=torch.float64, device="cuda")
    L = capi.lib()

    def step():
        plan.solve(sigma_device_ptr=sig.data_ptr(), out_device_ptr=fields.data_ptr(), allow_noconv=True)
        return plan.impedance()

    step()  # loads the conductivity
    vs = plan.autotune()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    clocks = Clocks(local)
    clocks.start()
    l0 = L.sfdx_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    z = None
    for _ in range(args.steps):
        z = step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = (L.sfdx_launch_count() - l0) / args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ms, world)
    barrier(world)
    value = whole_job_rate(ns, args.steps, world, ms)
    status, iters, relres, lt = plan.status, plan.iters.copy(), plan.relres.copy(), plan.level_times()

    # kernel rooflines on the finest level (CUDA events on the plan's stream)
    hbm, src = peaks()
    kern = {}
    for kid, name in ((2, "mc_ssor_c64"), (0, "operator_c64")):
        kms, kb = plan.kernel_time(kid, reps=10)
        kern[name] = {"ms": kms, "bytes": kb, "gbs": kb / (kms / 1e3) / 1e9}

    # end to end through the C ABI with host buffers
    e2e_steps = max(1, args.steps // 2)
    h2d = m.sigma.nbytes
    d2h = m.nf * 2 * m.nl * 16 + m.nf * m.recv.shape[0] * 4 * 8
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        ex, _, _ = S.fwd_solve(m, **opts) if args.e2e_allow_noconv is False else _fwd_noconv(S, m, opts)
        S.impedance(m, ex)
    e2e_s = (time.perf_counter() - t) / e2e_steps
    e2e_s = max_over_ranks(e2e_s, world)

    extra = {}
    if args.compare_fp64 and rank == 0:
        p64 = S.Plan(m, **solve_opts("fp64", args.solver, args.div_cor, eps, args.corr_intv, m.level))
        t = time.perf_counter()
        p64.solve(allow_noconv=True)
        t64 = time.perf_counter() - t
        z64 = p64.impedance()
        zc = z[..., 0::2] + 1j * z[..., 1::2]
        z64c = z64[..., 0::2] + 1j * z64[..., 1::2]
        rel = np.abs(zc - z64c) / np.abs(z64c)
        extra = {"z_rel_err_vs_fp64": float(rel.max()), "z_rel_err_vs_fp64_median": float(np.median(rel)),
                 "fp64_solves_per_s": ns / t64, "fp64_status": int(p64.status),
                 "fp64_fine_iters": p64.iters[:, :, -1].ravel().tolist()}
        p64.close()

    if rank == 0 and args.adjoint:
        extra["adjoint"] = adjoint_measure(S, syn, torch, stream, args.solver, 1e-10, fd_cells=args.fd_cells)

    if rank != 0:
        plan.close()
        return
    dom = kern["mc_ssor_c64"]
    cpu = None
    if args.cpu_baseline and args.workload == "aniso-hills":  # the reference's iteration counts are measured on this workload
        its = reference_iterations()
        _, t_it, t_setup = cpu_sample(m, [0], 1)
        n_it = float(np.mean(its)) if its else float("nan")
        cpu = {"value": 1.0 / (t_setup + n_it * t_it), "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": (f"one system: finest-level assembly + {REF_SAMPLE_ITERS} serial SSOR-BiCGStab iterations "
                          f"({t_it:.3f} s/it), scaled by the reference algorithm's mean iteration count {n_it:.0f}")}
    line = {
        "metric": "MT solves/s", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": (value / PUBLISHED_SOLVES_PER_S[args.workload]) if args.workload in PUBLISHED_SOLVES_PER_S else None,
        "dtype": "c64+c128" if args.precision == "mixed" else "c128", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload][0].format(eps=eps),
                   "precision": args.precision, "solver": args.solver, "div_cor": args.div_cor,
                   "systems_per_thread": {"c64": vs[0], "c128": vs[1]},
                   "systems_per_step": ns, "cuda_graphs": bool(USE_GRAPHS),
                   "l2": "working set > L2 (no flush)"},
        "e2e": {"value": ns / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "per_frequency": {"value": value / 2, "unit": "frequencies/s (both polarisations)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": dom["gbs"], "peak": hbm, "unit": "GB/s", "frac": dom["gbs"] / hbm,
                     "traffic": SSOR_TRAFFIC.get(args.workload), "kernel": "mc_ssor_c64 (11 colour sweeps)",
                     "peak_source": src},
        "kernels": kern,
        "cpu_baseline": cpu,
        "clocks": clk,
        "solve": {"status": int(status), "fine_iters": iters[:, :, -1].ravel().tolist(),
                  "relres_max": float(relres.max()), "level_ms": [float(x) for x in lt]},
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    plan.close()


def adjoint_measure(S, syn, torch, stream, solver, eps, fd_cells=0, reps=2, seed=0, adj_tol=1e-8):
    """Adjoint case: least-squares impedance misfit of an isotropic GRF model against data from a
    perturbed model (+2 % Gaussian noise, weights 1/(0.02|Z|)^2) and its gradient
    d misfit / d log sigma by one adjoint solve per frequency and polarisation.  Times the
    forward solve (+ misfit, tolerance eps) and the adjoint (+ per-cell contraction,
    tolerance adj_tol; once each at 1e-9 and eps for the accuracy they buy) with CUDA
    events on the plan's stream, compares the mixed-precision gradients with the FP64
    GPU adjoint at eps and,
    with fd_cells > 0, both with central differences (h = 1e-4 in log sigma) of FP64 GPU
    forward solves at that many random core cells (each perturbed solve starts from the base
    fields and solves the correction equation to a 1e-9 reduction, sfdx_plan_resolve)."""
    m, mt = syn.grf_inversion(seed), syn.grf_inversion_true(seed)
    opts = solve_opts("mixed", solver, 2, eps, None, m.level)
    opts64 = solve_opts("fp64", solver, 2, eps, None, m.level)
    with S.Plan(mt, **opts) as pt:
        pt.solve(fetch=False, allow_noconv=True)
        z = pt.impedance()
    rng = np.random.default_rng(seed + 7)
    zc = z[..., 0::2] + 1j * z[..., 1::2]
    sd = 0.02 * np.abs(zc)
    zn = zc + sd * (rng.standard_normal(zc.shape) + 1j * rng.standard_normal(zc.shape)) / np.sqrt(2)
    zobs = np.stack([zn.real[..., 0], zn.imag[..., 0], zn.real[..., 1], zn.imag[..., 1]], -1)
    wts = 1.0 / sd ** 2
    plan = S.Plan(m, **opts)
    plan.set_stream(stream.cuda_stream)
    sig = torch.from_numpy(np.ascontiguousarray(m.sigma)).to("cuda")
    g = torch.empty((6, m.ncell), dtype=torch.float64, device="cuda")

    def fwd():
        plan.solve(sigma_device_ptr=sig.data_ptr(), fetch=False, allow_noconv=True)
        return plan.misfit_grad(zobs, wts, with_grad=False)[0]

    def adj(tol):
        return plan.misfit_grad(zobs, wts, tol=tol, grad_device_ptr=g.data_ptr(), allow_noconv=True)

    def timed(fn):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(stream)
        out = fn()
        ev[1].record(stream)
        ev[1].synchronize()
        return out, ev[0].elapsed_time(ev[1])

    fwd()
    adj(adj_tol)
    tf, ta = [], []
    for _ in range(reps):
        mis, t = timed(fwd)
        tf.append(t)
        res, t = timed(lambda: adj(adj_tol))
        ta.append(t)
    fwd_iters = plan.iters[:, :, -1].ravel().tolist()
    adj_iters, adj_rr = res[3].ravel().tolist(), float(res[4].max())
    sg3 = m.sigma[0]
    dlog = sg3 * g[0:3].sum(0).cpu().numpy()
    sweep = {}
    for t_adj in (1e-9, eps):  # tighter adjoint tolerances, for the accuracy they buy
        if t_adj <= adj_tol:
            r_t, ms_t = timed(lambda: adj(t_adj))
            sweep[t_adj] = (r_t, ms_t, sg3 * g[0:3].sum(0).cpu().numpy())
    plan.close()
    p64 = S.Plan(m, **opts64)
    p64.solve(fetch=False, allow_noconv=True)
    mis64, g64, _, it64, _ = p64.misfit_grad(zobs, wts, allow_noconv=True)
    dlog64 = sg3 * g64[0:3].sum(0)
    out = {"workload": ("adjoint: the aniso-hills mesh without hills (80x80x80, 1,574,640 edges), isotropic log10 rho GRF "
                        "(mean 2, std 0.5, corr 5 cells), 6 freqs 1e-3..1e3 Hz x 2 pols, 32x32 receivers, data "
                        "from a perturbed GRF model + 2 % noise, EXCMG 3 levels, tol " + f"{eps:g}"),
           "precision": "mixed", "fwd_tol": eps, "adjoint_tol": adj_tol,
           "fwd_ms": float(np.median(tf)), "adjoint_ms": float(np.median(ta)),
           "grad_over_fwd": float(np.median(ta) / np.median(tf)),
           "fwd_plus_grad_over_fwd": float((np.median(tf) + np.median(ta)) / np.median(tf)),
           "misfit": mis, "misfit_fp64": mis64,
           "grad_rel_err_vs_fp64_adjoint": float(np.linalg.norm(dlog - dlog64) / np.linalg.norm(dlog64)),
           "fwd_fine_iters": fwd_iters, "adjoint_iters": adj_iters, "adjoint_relres_max": adj_rr,
           "tighter_adjoint_tol": [{"tol": t_adj, "adjoint_ms": ms_t, "grad_over_fwd": float(ms_t / np.median(tf)),
                                    "grad_rel_err_vs_fp64_adjoint": float(np.linalg.norm(dl - dlog64) /
                                                                          np.linalg.norm(dlog64)),
                                    "adjoint_iters": r_t[3].ravel().tolist()}
                                   for t_adj, (r_t, ms_t, dl) in sweep.items()],
           "fp64_adjoint": {"tol": eps, "iters": it64.ravel().tolist()}}
    if fd_cells:
        rs = np.random.default_rng(seed + 11)
        npad, nc, ncz = 8, 64, 48
        cells, fd = [], []
        for _ in range(fd_cells):
            i = rs.integers(npad, npad + nc)
            j = rs.integers(npad, npad + nc)
            k = rs.integers(m.nair, m.nair + ncz // 3)
            cells.append(int((k * m.ny + j) * m.nx + i))
        h = 1e-4
        for c in cells:
            f = []
            for sgn in (1, -1):
                s2 = m.sigma.copy()
                s2[0:3, c] *= np.exp(sgn * h)
                p64.resolve(sigma=s2, tol=-1e-9, allow_noconv=True)
                f.append(p64.misfit_grad(zobs, wts, with_grad=False)[0])
            fd.append((f[0] - f[1]) / (2 * h))
        fd = np.array(fd)
        a64 = dlog64[cells]
        am = dlog[cells]
        out["fd_check"] = {"cells": len(cells), "h_log_sigma": h, "forward": "fp64 GPU, correction equation from the base fields",
                           "max_rel_err_fp64_adjoint": float(np.max(np.abs(a64 - fd) / np.abs(fd))),
                           "median_rel_err_fp64_adjoint": float(np.median(np.abs(a64 - fd) / np.abs(fd))),
                           "max_rel_err_mixed_adjoint": float(np.max(np.abs(am - fd) / np.abs(fd))),
                           "median_rel_err_mixed_adjoint": float(np.median(np.abs(am - fd) / np.abs(fd))),
                           "fd": fd.tolist(), "adjoint_fp64": a64.tolist(), "adjoint_mixed": am.tolist()}
    p64.close()
    return out


def run_batch(args, rank, world, local):
    """multi-model: the 8 models solved together (sfdx_plan_solve_batch: one host thread and
    stream per model) -- value; the same plans one after another -- sequential_solves_per_s."""
    import torch
    torch.cuda.set_device(local)
    import sfd_excmg_gb300 as S
    from sfd_excmg_gb300 import capi
    from sfd_excmg_gb300 import synthetic as syn
    eps = args.eps if args.eps else WORKLOADS["multi-model"][1]
    models = syn.multi_model_batch(seed=rank)
    opts = solve_opts(args.precision, args.solver, args.div_cor, eps, args.corr_intv, 3)
    # the meshes are not square: receivers through the corrected (untransposed)
    # interpolation stencil (the reference's transposed one indexes past ny)
    opts["quirks"] = capi.QUIRKS_REFERENCE & ~4
    plans = [S.Plan(m, **opts) for m in models]
    sig = [torch.from_numpy(np.ascontiguousarray(m.sigma)).to("cuda") for m in models]
    ptrs = [t.data_ptr() for t in sig]
    ns = sum(2 * m.nf for m in models)
    L = capi.lib()

    def step():
        S.solve_batch(plans, sigma_device_ptrs=ptrs, allow_noconv=True)
        return [p.impedance() for p in plans]

    step()
    vs = [p.autotune() for p in plans]
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    clocks = Clocks(local)
    clocks.start()
    l0 = L.sfdx_launch_count()
    t = time.perf_counter()
    for _ in range(args.steps):
        z = step()
    torch.cuda.synchronize()
    sec = (time.perf_counter() - t) / args.steps
    launches = (L.sfdx_launch_count() - l0) / args.steps
    clk = clocks.stop()
    sec = max_over_ranks(sec, world)
    # the same plans one after another
    t = time.perf_counter()
    for p, ptr in zip(plans, ptrs):
        p.solve(sigma_device_ptr=ptr, fetch=False, allow_noconv=True)
        p.impedance()
    torch.cuda.synchronize()
    seq = time.perf_counter() - t
    # end to end: host conductivities in, impedances out
    t = time.perf_counter()
    S.solve_batch(plans, sigmas=[m.sigma for m in models], allow_noconv=True)
    zz = [p.impedance() for p in plans]
    e2e = time.perf_counter() - t
    h2d = sum(m.sigma.nbytes for m in models)
    d2h = sum(z_.nbytes for z_ in zz)
    status = [int(p.status) for p in plans]
    iters = [p.iters[:, :, -1].ravel().tolist() for p in plans]
    for p in plans:
        p.close()
    extra = {}
    if args.compare_fp64 and rank == 0:
        o64 = solve_opts("fp64", args.solver, args.div_cor, eps, args.corr_intv, 3)
        o64["quirks"] = opts["quirks"]
        p64 = [S.Plan(m, **o64) for m in models]
        t = time.perf_counter()
        S.solve_batch(p64, sigma_device_ptrs=ptrs, allow_noconv=True)
        t64 = time.perf_counter() - t
        rel = []
        for p, zm in zip(p64, z):
            z64 = p.impedance()
            a = zm[..., 0::2] + 1j * zm[..., 1::2]
            b = z64[..., 0::2] + 1j * z64[..., 1::2]
            rel.append((np.abs(a - b) / np.abs(b)).ravel())
            p.close()
        rel = np.concatenate(rel)
        extra = {"z_rel_err_vs_fp64": float(rel.max()), "z_rel_err_vs_fp64_median": float(np.median(rel)),
                 "fp64_solves_per_s": ns / t64}
    if rank != 0:
        return
    value = whole_job_rate(ns, 1, world, sec * 1e3)
    line = {
        "metric": "MT solves/s", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64+c128" if args.precision == "mixed" else "c128", "data": "synthetic",
        "config": {"workload": WORKLOADS["multi-model"][0].format(eps=eps),
                   "meshes": [[m.nx, m.ny, m.nz] for m in models], "edges": [int(m.nl) for m in models],
                   "precision": args.precision, "solver": args.solver, "div_cor": args.div_cor,
                   "systems_per_thread": vs, "systems_per_step": ns, "cuda_graphs": bool(USE_GRAPHS),
                   "l2": "working set > L2 (no flush)"},
        "e2e": {"value": ns / e2e, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches), "sequential_solves_per_s": ns / seq, "clocks": clk,
        "solve": {"status": status, "fine_iters": iters},
    }
    line.update(extra)
    print(json.dumps(line), flush=True)


def run_profile(args):
    """Kernel families on the finest level of the workload, CUDA-event timed (few launches)."""
    import sfd_excmg_gb300 as S
    from sfd_excmg_gb300 import synthetic as syn
    m = make_workload(args.workload)
    eps = args.eps if args.eps else WORKLOADS[args.workload][1]
    hbm, src = peaks()
    with S.Plan(m, **solve_opts(args.precision, args.solver, args.div_cor, eps, args.corr_intv, m.level)) as p:
        p.load()
        out = {}
        for kid, name in ((2, "mc_ssor_c64"), (0, "operator_c64"), (1, "operator_c128")):
            ms, b = p.kernel_time(kid, reps=2)
            out[name] = {"ms": ms, "alg_bytes": b, "gbs": b / (ms / 1e3) / 1e9, "frac_of_" + src: b / (ms / 1e3) / 1e9 / hbm}
    print(json.dumps(out), flush=True)


def _fwd_noconv(S, m, opts):
    with S.Plan(m, **opts) as p:
        ex = p.solve(allow_noconv=True)
    return ex, None, None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--solver", default="gpbicg", choices=list(SOLVER))
    ap.add_argument("--workload", default="aniso-hills", choices=list(WORKLOADS))
    ap.add_argument("--eps", type=float, default=None,
                    help="finest-level relative residual tolerance (default per workload; aniso-hills: 1e-10, the accuracy "
                         "at which the mixed-precision impedances agree with the FP64 ones to ~1e-5)")
    ap.add_argument("--corr-intv", dest="corr_intv", type=int, default=None,
                    help="Krylov iterations of the first restart cycle of the gradient correction (default 40; each "
                         "next cycle is 1.5x longer)")
    ap.add_argument("--div-cor", dest="div_cor", type=int, default=2, choices=[0, 1, 2],
                    help="0 none, 1 the reference's divergence correction, 2 consistent gradient-space correction")
    ap.add_argument("--no-compare-fp64", dest="compare_fp64", action="store_false")
    ap.add_argument("--no-graphs", dest="graphs", action="store_false",
                    help="launch the Krylov iterations one by one instead of replaying captured CUDA graphs")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false",
                    help="skip the misfit-gradient measurement (adjoint case: forward vs adjoint time, FP64 check)")
    ap.add_argument("--fd-cells", dest="fd_cells", type=int, default=0,
                    help="also check the gradient against central differences of FP64 forward solves at this many "
                         "random cells (the adjoint case asks for 20)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--e2e-strict", dest="e2e_allow_noconv", action="store_false")
    ap.add_argument("--profile", action="store_true",
                    help="only load the workload's conductivity and time each kernel family a few times "
                         "(a short launch sequence for ncu captures)")
    args = ap.parse_args()
    global USE_GRAPHS
    USE_GRAPHS = 1 if args.graphs else 0
    rank, world, local = dist()
    if args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "multi-model":
        run_batch(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
