// sfdx_solver.cu -- host drivers and the C ABI of the GB300 forward solver.
//
// One plan = one mesh hierarchy + one frequency list.  All 2*nf systems
// (frequency x polarisation) of a model are solved together: their vectors
// are interleaved innermost so that every kernel reads the shared
// conductivity and spacing tables once for the whole batch.
//
//  fwd_solver (fdfe_main.f90:1565)            -> sfdx_plan_solve
//    doublemode_nor (:892, fwd_acc = 0)       -> solve_plain
//    doublemode_acc (:1258, fwd_acc = 1)      -> solve_cascade
//      u1u2 + pardiso_spd (:1228, :765)       -> coarse levels: FP64 Krylov to coarse_tol
//      extint_v (excmg.f90:9)                 -> prolongate (k_interp, k_extrapolate)
//    Bicg_stab_p (solvers.f90:522)            -> bicgstab<T>   (sfdx_krylov.cuh)
//    pgpbicg (solvers.f90:137)                -> gpbicg<T>     (sfdx_krylov.cuh)
//    lusol/ssorfac (multi-colour)             -> precond       (sfdx_krylov.cuh)
//  mixed precision                            -> solve_level_mixed (FP64 residual,
//                                                complex64 inner BiCGStab)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <functional>
#include <memory>
#include <thread>
#include <type_traits>
#include <vector>

#include "sfdx.h"
#include "sfdx_divcorr.cuh"
#include "sfdx_excmg.cuh"
#include "sfdx_host.h"
#include "sfdx_kernels.cuh"
#include "sfdx_plan.h"
#include "sfdx_vkern.cuh"

using namespace sfdx;

namespace sfdx {

std::atomic<long long> g_launches{0};
thread_local int g_misaligned = 0;

static void axis_tables(const std::vector<double>& h, int stride, double* out) {
    const int n = (int)h.size();
    double* rh = out;
    double* lo = out + stride;
    double* hi = out + 2 * stride;
    double* rs = out + 3 * stride;
    double* wl = out + 4 * stride;
    double* wh = out + 5 * stride;
    for (int q = 0; q < 6 * stride; q++) out[q] = 0;
    for (int i = 0; i < n; i++) rh[i] = 1.0 / h[i];
    for (int m = 1; m < n; m++) {
        double s = h[m - 1] + h[m];
        lo[m] = -2 / (h[m - 1] * (h[m - 1] + h[m]));
        hi[m] = -2 / (h[m] * (h[m - 1] + h[m]));
        rs[m] = 1.0 / s;
        wl[m] = h[m - 1] / s;
        wh[m] = h[m] / s;
    }
}

static std::vector<double> node_coords(const std::vector<double>& h, int nair, bool is_z) {
    std::vector<double> X(h.size() + 1);
    double s = 0;
    if (is_z) {
        for (int i = 0; i < nair; i++) s += h[i];
        X[0] = -s;
    } else {
        for (double v : h) s += v;
        X[0] = -s / 2;
    }
    for (size_t i = 1; i <= h.size(); i++) X[i] = X[i - 1] + h[i - 1];
    return X;
}

static int upload_level_tables(Level& L, cudaStream_t st) {
    L.stride = std::max(L.nx, std::max(L.ny, L.nz)) + 2;
    std::vector<double> t64((size_t)18 * L.stride);
    axis_tables(L.a, L.stride, &t64[0]);
    axis_tables(L.b, L.stride, &t64[(size_t)6 * L.stride]);
    axis_tables(L.c, L.stride, &t64[(size_t)12 * L.stride]);
    std::vector<float> t32(t64.size());
    for (size_t q = 0; q < t64.size(); q++) t32[q] = (float)t64[q];
    RC(L.tab64.alloc(t64.size() * 8));
    RC(L.tab32.alloc(t32.size() * 4));
    CK(cudaMemcpyAsync(L.tab64.p, t64.data(), t64.size() * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(L.tab32.p, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice, st));
    std::vector<double> sp;
    sp.insert(sp.end(), L.a.begin(), L.a.end());
    sp.insert(sp.end(), L.b.begin(), L.b.end());
    sp.insert(sp.end(), L.c.begin(), L.c.end());
    RC(L.spac.alloc(sp.size() * 8));
    CK(cudaMemcpyAsync(L.spac.p, sp.data(), sp.size() * 8, cudaMemcpyHostToDevice, st));
    // coordinates for the prolongation INTO this level: cubic uses this
    // level's spacings; quad (into the next coarser level) uses the pairwise
    // sums of this level's spacings (extint_v excmg.f90:24-33).
    std::vector<double> cc;
    for (auto& v : node_coords(L.a, 0, false)) cc.push_back(v);
    for (auto& v : node_coords(L.b, 0, false)) cc.push_back(v);
    for (auto& v : node_coords(L.c, L.nair, true)) cc.push_back(v);
    RC(L.crd_cubic.alloc(cc.size() * 8));
    CK(cudaMemcpyAsync(L.crd_cubic.p, cc.data(), cc.size() * 8, cudaMemcpyHostToDevice, st));
    if (L.nx % 2 == 0 && L.ny % 2 == 0 && L.nz % 2 == 0) {
        std::vector<double> a2(L.nx / 2), b2(L.ny / 2), c2(L.nz / 2);
        for (int i = 0; i < L.nx / 2; i++) a2[i] = L.a[2 * i] + L.a[2 * i + 1];
        for (int i = 0; i < L.ny / 2; i++) b2[i] = L.b[2 * i] + L.b[2 * i + 1];
        for (int i = 0; i < L.nz / 2; i++) c2[i] = L.c[2 * i] + L.c[2 * i + 1];
        std::vector<double> cq;
        for (auto& v : node_coords(a2, 0, false)) cq.push_back(v);
        for (auto& v : node_coords(b2, 0, false)) cq.push_back(v);
        for (auto& v : node_coords(c2, L.nair / 2, true)) cq.push_back(v);
        RC(L.crd_quad.alloc(cq.size() * 8));
        CK(cudaMemcpyAsync(L.crd_quad.p, cq.data(), cq.size() * 8, cudaMemcpyHostToDevice, st));
    }
    return SFDX_OK;
}

// ------------------------------------------------------------------ divergence correction
static NodeGeo node_geo(const Level& LV) {
    NodeGeo G;
    G.nx = LV.nx; G.ny = LV.ny; G.nz = LV.nz;
    G.np = (int64_t)(LV.nx + 1) * (LV.ny + 1) * (LV.nz + 1);
    G.xnl = LV.xnl; G.ynl = LV.ynl; G.ncell = LV.ncell;
    const double* sp = LV.spac.as<double>();
    G.a = sp; G.b = sp + LV.nx; G.c = sp + LV.nx + LV.ny;
    G.sig = LV.sig64.as<double>();
    return G;
}

// x += grad(phi), P phi = T x  for the systems active in P.d_state
int div_correct(Plan& P, const Level& LV, double2* x) {
    const int ns = P.ns;
    const NodeGeo G = node_geo(LV);
    const size_t nb = (size_t)G.np * ns * sizeof(double2);
    for (int q = 0; q < 5; q++) RC(P.dcv[q].alloc(nb));
    RC(P.d_pst.alloc(sizeof(KState) * ns));
    double2 *t = P.dcv[0].as<double2>(), *r = P.dcv[1].as<double2>(), *p = P.dcv[2].as<double2>();
    double2 *v = P.dcv[3].as<double2>(), *phi = P.dcv[4].as<double2>();
    const int B = block_for(ns);
    const int G1 = grid_for(G.np * ns, B, 8);
    RC(P.d_part.alloc(std::max(P.d_part.bytes, (size_t)G1 * 2 * ns * sizeof(double2))));
    const size_t sm = 2 * B * sizeof(double2);
    KState* pst = P.d_pst.as<KState>();
    KL(k_dc_div<<<G1, B, sm, P.st>>>(G, P.d_state.as<KState>(), ns, x, t, r, p, phi, redbuf(P), pst));
    const int maxit = 2000;  // pcg itmax (div_correc.f90:57)
    int it = 0;
    std::vector<KState> h(ns);
    for (; it < maxit; it++) {
        KL(k_dc_Ap<<<G1, B, sm, P.st>>>(G, pst, ns, p, v, redbuf(P)));
        KL(k_dc_upd<<<G1, B, sm, P.st>>>(G, pst, ns, p, v, phi, r, redbuf(P), P.o.corr_tol, maxit));
        KL(k_dc_p<<<G1, B, 0, P.st>>>(G, pst, ns, r, p));
        if ((it + 1) % 16 == 0) {
            CK(cudaMemcpyAsync(h.data(), pst, sizeof(KState) * ns, cudaMemcpyDeviceToHost, P.st));
            CK(cudaStreamSynchronize(P.st));
            int act = 0;
            for (auto& q : h) act += q.active;
            if (!act) break;
        }
    }
    CK(cudaMemcpyAsync(h.data(), pst, sizeof(KState) * ns, cudaMemcpyDeviceToHost, P.st));
    KL(k_dc_grad<<<grid_for(LV.nl * ns, B, 16), B, 0, P.st>>>(G, P.d_state.as<KState>(), ns, phi, x));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(P.st));
    P.dc_calls++;
    P.dc_last_iters = h[0].iters;
    return SFDX_OK;
}

// true relative residual ||b - A x|| / ||b|| per system (FP64)
int true_residual(Plan& P, const Level& LV, const double2* b, const double2* x, double* rel, const int* mask) {
    const int ns = P.ns;
    std::vector<KState> init(ns);
    for (int q = 0; q < ns; q++) {
        KState S;
        memset(&S, 0, sizeof(S));
        S.wm = P.wm[q];
        S.active = mask ? mask[q] : 1;
        init[q] = S;
    }
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    const int B = block_for(ns);
    const int G = grid_for(LV.nl * ns, B, 8);
    RC(P.d_part.alloc((size_t)G * 2 * ns * sizeof(double2)));
    RC(P.r64.alloc((size_t)LV.nl * ns * sizeof(double2)));
    KL(k_residual<double, double, 2><<<G, B, 2 * B * sizeof(double2), P.st>>>(
        LV.lev<double>(), P.d_state.as<KState>(), ns, b, x, P.r64.as<double2>(), nullptr, redbuf(P), nullptr, 0));
    CK(cudaGetLastError());
    RC(sync_state(P));
    for (int q = 0; q < ns; q++) {
        double nb = P.hst[q].babs;
        rel[q] = (mask && !mask[q]) ? 0.0 : (nb > 0 ? P.hst[q].err / nb : P.hst[q].err);
    }
    return SFDX_OK;
}

// ------------------------------------------------------------------ level solves
// FP64 solve to `tol` with the reference's solver semantics.
static int solve_level_fp64(Plan& P, const Level& LV, double tol, int itmax, std::vector<int>& its,
                            std::vector<int>& status) {
    if (P.o.solver == SFDX_SOLVER_BICGSTAB)
        RC(bicgstab<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, nullptr));
    else if (P.o.solver == SFDX_SOLVER_GPBICG)
        RC(gpbicg<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, nullptr));
    else if (P.o.solver == SFDX_SOLVER_COCR)
        RC(cocr<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, nullptr));
    else if (P.o.solver == SFDX_SOLVER_TFQMR)
        RC(tfqmr<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, nullptr));
    else if (P.o.solver == SFDX_SOLVER_BICG)
        RC(bicg<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, nullptr));
    else
        return SFDX_ERR_UNSUPPORTED;
    its.resize(P.ns);
    status.resize(P.ns);
    for (int q = 0; q < P.ns; q++) {
        its[q] = P.hst[q].iters;
        status[q] = P.hst[q].status;
    }
    return SFDX_OK;
}

// Mixed precision: complex64 operator, smoother and Krylov recurrences;
// complex128 solution, residual and convergence test (reliable updates).
static int solve_level_mixed(Plan& P, const Level& LV, double tol, int itmax, std::vector<int>& its,
                             std::vector<int>& status) {
    const int ns = P.ns;
    const size_t n = (size_t)LV.nl * ns;
    DBuf& x32 = P.x32;
    RC(x32.alloc(n * sizeof(float2)));
    RC(P.xb.alloc(n * sizeof(double2)));
    Reliable rel{P.b64.as<double2>(), P.x64.as<double2>(), P.o.reliable_every > 0 ? P.o.reliable_every : 40,
                 P.xb.as<double2>()};
    if (P.o.solver == SFDX_SOLVER_GPBICG)
        RC(gpbicg<float>(P, LV, nullptr, x32.as<float2>(), nullptr, tol, itmax, nullptr, &rel));
    else if (P.o.solver == SFDX_SOLVER_BICGSTAB)
        RC(bicgstab<float>(P, LV, nullptr, x32.as<float2>(), nullptr, tol, itmax, nullptr, &rel));
    else if (P.o.solver == SFDX_SOLVER_COCR)
        RC(cocr<float>(P, LV, nullptr, x32.as<float2>(), nullptr, tol, itmax, nullptr, &rel));
    else
        return SFDX_ERR_UNSUPPORTED;
    its.resize(ns);
    status.resize(ns);
    std::vector<int> left(ns, 0);
    int nleft = 0, used_max = 0;
    for (int q = 0; q < ns; q++) {
        its[q] = P.hst[q].iters;
        int st = P.hst[q].status;
        status[q] = (st == ST_VCONV) ? ST_CONV : (st == ST_CONV || st == ST_RUN ? ST_MAXIT : st);
        // complex64 steps stalled (correction rejected) before the iteration
        // limit: finish this system in FP64 from its current FP64 iterate
        if (st == ST_BREAK && its[q] < itmax) {
            left[q] = 1;
            nleft++;
            used_max = std::max(used_max, its[q]);
        }
    }
    if (nleft) {
        std::vector<int> its64, st64;
        if (P.rec_on)
            for (int q = 0; q < ns; q++)
                if (left[q] && q < (int)P.rec_off.size()) P.rec_off[q] = its[q];
        const int save = P.o.div_cor;
        if (save == 1) P.o.div_cor = 0;  // the FP64 finish is a continuation, not a reference restart
        int rc;
        if (P.o.solver == SFDX_SOLVER_GPBICG)
            rc = gpbicg<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax - used_max,
                                left.data());
        else if (P.o.solver == SFDX_SOLVER_COCR)
            rc = cocr<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax - used_max,
                              left.data());
        else
            rc = bicgstab<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax - used_max,
                                  left.data());
        P.o.div_cor = save;
        RC(rc);
        for (int q = 0; q < ns; q++) {
            if (!left[q]) continue;
            its[q] += P.hst[q].iters;
            status[q] = P.hst[q].status;
        }
        if (P.o.verbose || getenv("SFDX_VERBOSE")) fprintf(stderr, "sfdx:   %d system(s) finished in FP64\n", nleft);
    }
    return SFDX_OK;
}

int solve_level(Plan& P, const Level& LV, double tol, int itmax, bool coarse, std::vector<int>& its,
                std::vector<int>& status) {
    // TFQMR and BiCG have no complex64 / reliable-update form: FP64 in every plan
    if (coarse || P.o.precision == SFDX_FP64 || P.o.solver == SFDX_SOLVER_TFQMR || P.o.solver == SFDX_SOLVER_BICG)
        return solve_level_fp64(P, LV, tol, itmax, its, status);
    // mixed precision with the multigrid preconditioner and the other solvers
    // (or SFDX_MG_SPLIT=0): complex128 Krylov vectors and operator, complex64
    // V-cycle (SFDX_MG_PF32=0: the complex64 Krylov iteration with FP64
    // reliable updates of the SSOR plans instead)
    // mixed precision, multigrid, BiCGStab: complex64 BiCGStab on split vectors
    // (y + G psi) under the split V-cycle, FP64 reliable updates
    // (SFDX_MG_SPLIT=0: the complex128 Krylov iteration below instead)
    static const bool split = [] {
        const char* e = getenv("SFDX_MG_SPLIT");
        return !(e && e[0] == '0');
    }();
    if (P.o.precond == 'G' && split && P.o.solver == SFDX_SOLVER_BICGSTAB) {
        P.split = true;
        const int rc = solve_level_mixed(P, LV, tol, itmax, its, status);
        P.split = false;
        return rc;
    }
    static const bool krylov64 = [] {
        const char* e = getenv("SFDX_MG_PF32");
        return !(e && e[0] == '0');
    }();
    if (P.o.precond == 'G' && krylov64) {
        // the starting iterate, for systems whose complex64 V-cycle fails them
        // (NaN or breakdown): those restart from it with the FP64 V-cycle
        const size_t n = (size_t)LV.nl * P.ns;
        RC(P.xb.alloc(n * sizeof(double2)));
        CK(cudaMemcpyAsync(P.xb.p, P.x64.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, P.st));
        P.pf32 = true;
        const int rc = solve_level_fp64(P, LV, tol, itmax, its, status);
        P.pf32 = false;
        RC(rc);
        std::vector<int> left(P.ns, 0);
        int nleft = 0;
        for (int q = 0; q < P.ns; q++)
            if (status[q] == ST_NAN || status[q] == ST_BREAK) {
                left[q] = 1;
                nleft++;
            }
        if (!nleft) return SFDX_OK;
        const int B = block_for(P.ns);
        RC(P.d_sel.alloc(sizeof(int) * P.ns));
        CK(cudaMemcpyAsync(P.d_sel.p, left.data(), sizeof(int) * P.ns, cudaMemcpyHostToDevice, P.st));
        KL(k_restore_sel<<<grid_for(n, B, 16), B, 0, P.st>>>(LV.nl, P.d_sel.as<int>(), P.ns, P.x64.as<double2>(),
                                                               P.xb.as<double2>()));
        CK(cudaGetLastError());
        if (P.rec_on)
            for (int q = 0; q < P.ns; q++)
                if (left[q] && q < (int)P.rec_off.size()) P.rec_off[q] = its[q];
        if (P.o.verbose || getenv("SFDX_VERBOSE"))
            fprintf(stderr, "sfdx:   %d system(s) restarted with the FP64 V-cycle\n", nleft);
        if (P.o.solver == SFDX_SOLVER_GPBICG)
            RC(gpbicg<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, left.data()));
        else if (P.o.solver == SFDX_SOLVER_COCR)
            RC(cocr<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, left.data()));
        else
            RC(bicgstab<double>(P, LV, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, itmax, left.data()));
        for (int q = 0; q < P.ns; q++) {
            if (!left[q]) continue;
            its[q] += P.hst[q].iters;
            status[q] = P.hst[q].status;
        }
        return SFDX_OK;
    }
    return solve_level_mixed(P, LV, tol, itmax, its, status);
}

// ------------------------------------------------------------------ per-level set-up
// 1-D background for every system of level LV (host, FP64), then the RHS.
static int level_rhs(Plan& P, const Level& LV, const std::vector<double>& col /*[nz][3]*/) {
    const int ns = P.ns, nz = LV.nz;
    P.edc_stride = 2 * nz + 2;
    std::vector<std::complex<double>> edc((size_t)ns * P.edc_stride);
    std::vector<double> conv((size_t)nz * 6, 0.0);
    for (int k = 0; k < nz; k++)
        for (int q = 0; q < 3; q++) conv[(size_t)q * nz + k] = col[(size_t)k * 3 + q];
    std::vector<int> pols(ns);
    for (int f = 0; f < P.nf; f++) {
        std::vector<std::complex<double>> e(2 * nz + 2);
        RC(mt1d_anl(P.freq[f], nz, conv.data(), LV.c.data(), e.data(), nullptr, nullptr));
        for (int pol = 0; pol < 2; pol++) {
            int s = 2 * f + pol;
            pols[s] = pol;
            std::copy(e.begin(), e.end(), edc.begin() + (size_t)s * P.edc_stride);
        }
    }
    RC(P.d_edc.alloc(edc.size() * sizeof(double2)));
    RC(P.d_pol.alloc(ns * sizeof(int)));
    CK(cudaMemcpyAsync(P.d_edc.p, edc.data(), edc.size() * sizeof(double2), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(P.d_pol.p, pols.data(), ns * sizeof(int), cudaMemcpyHostToDevice, P.st));
    const int B = block_for(ns);
    KL(k_build_rhs<<<grid_for(LV.nl * ns, B, 16), B, 0, P.st>>>(LV.lev<double>(), P.d_wm.as<double>(), P.d_pol.as<int>(),
                                                              P.d_edc.as<double2>(), P.edc_stride, ns, P.b64.as<double2>()));
    CK(cudaGetLastError());
    // NaN check of the right-hand side (fdfe_main.f90:1398-1403)
    RC(P.d_flag.alloc(sizeof(int)));
    CK(cudaMemsetAsync(P.d_flag.p, 0, sizeof(int), P.st));
    KL(k_nan_check<double><<<grid_for(LV.nl * ns, 256), 256, 0, P.st>>>(LV.nl * ns, P.b64.as<double2>(), P.d_flag.as<int>()));
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, P.d_flag.p, sizeof(int), cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return flag ? SFDX_ERR_NAN : SFDX_OK;
}

// conductivity column (i=1,j=1) of level LV, diagonal components (cont1,
// fdfe_main.f90:938-942 / 1376-1380)
static int level_column(Plan& P, const Level& LV, std::vector<double>& col) {
    col.assign((size_t)LV.nz * 3, 0.0);
    std::vector<double> tmp(LV.nz);
    for (int q = 0; q < 3; q++) {
        CK(cudaMemcpy2DAsync(tmp.data(), sizeof(double), LV.sig64.as<double>() + (size_t)q * LV.ncell,
                             sizeof(double) * (size_t)LV.nx * LV.ny, sizeof(double), LV.nz, cudaMemcpyDeviceToHost, P.st));
        CK(cudaStreamSynchronize(P.st));
        for (int k = 0; k < LV.nz; k++) col[(size_t)k * 3 + q] = tmp[k];
    }
    return SFDX_OK;
}

// mesh_coarsen's index shift (fdfe_main.f90:64) misplaces the coarse
// conductivity by one fine cell per coarsening; the EXCMG guesses tolerate it,
// the coarse-grid operators of the multigrid preconditioner do not (on the
// 160x160x144 model: 100-186 GPBiCG iterations with the shift, 23-45 without),
// so plans with precond 'G' always coarsen without it.
static bool coarsen_shift(const sfdx_opts& o) {
    return (o.quirks & SFDX_QUIRK_COARSEN_SHIFT) && o.precond != 'G';
}

static int set_conductivity(Plan& P, const double* sigma, bool on_device) {
    P.sigma_gen++;  // the last solution (if any) belongs to the previous conductivity
    Level& F = P.lev[P.nlev - 1];
    const size_t nb = (size_t)6 * F.ncell * sizeof(double);
    RC(F.sig64.alloc(nb));
    CK(cudaMemcpyAsync(F.sig64.p, sigma, nb, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, P.st));
    for (int l = P.nlev - 2; l >= 0; l--) {
        Level& C = P.lev[l];
        const int k = P.nlev - 1 - l;
        RC(C.sig64.alloc((size_t)6 * C.ncell * sizeof(double)));
        const double* fs = F.spac.as<double>();
        const double* cp = C.spac.as<double>();  // this level's a, b, c
        KL(k_coarsen<<<grid_for(C.ncell, 128, 32), 128, 0, P.st>>>(F.nx, F.ny, F.nz, fs, fs + F.nx, fs + F.nx + F.ny, cp,
                                                                cp + C.nx, cp + C.nx + C.ny, 1 << k,
                                                                coarsen_shift(P.o) ? 1 : 0,
                                                                F.sig64.as<double>(), C.sig64.as<double>()));
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(P.st));
    }
    for (int l = 0; l < P.nlev; l++) {
        Level& L = P.lev[l];
        L.gc_ok = false;
        RC(L.sig32.alloc((size_t)6 * L.ncell * sizeof(float)));
        // sigma is real: convert pairs as if complex (6*ncell is even)
        int64_t n2 = 3 * L.ncell;
        KL(k_convert<double, float><<<grid_for(n2, 256), 256, 0, P.st>>>(n2, L.sig64.as<double2>(), L.sig32.as<float2>()));
        RC(P.d_flag.alloc(sizeof(int)));
        CK(cudaMemsetAsync(P.d_flag.p, 0, sizeof(int), P.st));
        KL(k_any_offdiag<<<grid_for(3 * L.ncell, 256), 256, 0, P.st>>>(L.ncell, L.sig64.as<double>(), P.d_flag.as<int>()));
        int flag = 0;
        CK(cudaMemcpyAsync(&flag, P.d_flag.p, sizeof(int), cudaMemcpyDeviceToHost, P.st));
        CK(cudaStreamSynchronize(P.st));
        L.aniso = flag;
        // per-row coefficients of both precisions (SFDX_ROW_COEF=0: computed
        // in every row evaluation instead)
        L.rc_ok = false;
        const char* env = getenv("SFDX_ROW_COEF");
        if (!(env && env[0] == '0')) {
            RC(L.rc64.alloc((size_t)L.nl * 12 * sizeof(double)));
            RC(L.rc32.alloc((size_t)L.nl * 12 * sizeof(float)));
            KL(k_row_coef<double><<<grid_for(L.nl, 256, 16), 256, 0, P.st>>>(L.lev<double>(), L.mesh, L.rc64.as<double>()));
            KL(k_row_coef<float><<<grid_for(L.nl, 256, 16), 256, 0, P.st>>>(L.lev<float>(), L.mesh, L.rc32.as<float>()));
            CK(cudaGetLastError());
            L.rc_ok = true;
        }
    }
    return SFDX_OK;
}

// extint_v: x64 (level l) from u0 (level l-2) and u1 (level l-1)
static int prolongate(Plan& P, int l, const double2* u0, const double2* u1, double2* out) {
    const Level& F = P.lev[l];
    const Level& M = P.lev[l - 1];
    const int ns = P.ns;
    const int midq = (P.o.quirks & SFDX_QUIRK_EXCMG_MIDPOINT) ? 1 : 0;
    const int B = block_for(ns);
    // quad: level l-2 -> level l-1 (coordinates from pairwise sums of level l)
    const double* cq = F.crd_quad.as<double>();
    KL(k_interp<double, 2><<<grid_for(M.nl * ns, B, 16), B, 0, P.st>>>(M.nx, M.ny, M.nz, cq, cq + M.nx + 1,
                                                                     cq + M.nx + M.ny + 2, midq, ns, u0, P.ut.as<double2>()));
    KL(k_extrapolate<double><<<grid_for(M.nl * ns, 256), 256, 0, P.st>>>(M.nl * ns, u1, P.ut.as<double2>()));
    const double* cc = F.crd_cubic.as<double>();
    KL(k_interp<double, 4><<<grid_for(F.nl * ns, B, 16), B, 0, P.st>>>(F.nx, F.ny, F.nz, cc, cc + F.nx + 1,
                                                                     cc + F.nx + F.ny + 2, midq, ns, P.ut.as<double2>(), out));
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(P.d_flag.p, 0, sizeof(int), P.st));
    KL(k_nan_check<double><<<grid_for(F.nl * ns, 256), 256, 0, P.st>>>(F.nl * ns, out, P.d_flag.as<int>()));
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, P.d_flag.p, sizeof(int), cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return flag ? SFDX_ERR_NAN : SFDX_OK;
}

static int status_to_rc(const std::vector<int>& status) {
    int rc = SFDX_OK;
    for (int s : status) {
        if (s == ST_NAN) return SFDX_ERR_NAN;
        if (s == ST_MAXIT) rc = SFDX_ERR_NOCONV;
    }
    return rc;
}

static void record_iters(Plan& P, int level_slot, const std::vector<int>& its) {
    for (int s = 0; s < P.ns; s++) P.iters[(size_t)s * P.nlev + level_slot] = its[s];
}

static double now_ms() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static void log_level(Plan& P, int l, const std::vector<int>& its, const std::vector<int>& status, double ms) {
    if (!P.o.verbose && !getenv("SFDX_VERBOSE")) return;
    const Level& L = P.lev[l];
    int mn = 1 << 30, mx = 0, cnt[5] = {0, 0, 0, 0, 0};
    for (int q = 0; q < P.ns; q++) {
        mn = std::min(mn, its[q]);
        mx = std::max(mx, its[q]);
        if (status[q] >= 0 && status[q] < 5) cnt[status[q]]++;
    }
    fprintf(stderr, "sfdx: level %d (%dx%dx%d, nl=%lld) iters %d..%d conv %d maxit %d nan %d break %d  %.1f ms\n", l + 1,
            L.nx, L.ny, L.nz, (long long)L.nl, mn, mx, cnt[ST_CONV], cnt[ST_MAXIT], cnt[ST_NAN], cnt[ST_BREAK], ms);
}

// residual history of the next finest-level solve (sync_state records it)
static void history_start(Plan& P, int len) {
    P.rec_on = true;
    P.rec_len = len;
    P.rec_hist.assign((size_t)P.ns * len, 0.0);
    P.rec_off.assign(P.ns, 0);
    P.rec_map.clear();
}

// EXCMG cascade (doublemode_acc, fdfe_main.f90:1258-1563): levels 1 and 2
// solved tightly in FP64 from zero (u1u2, the PARDISO replacement), then on
// each finer level the extrapolated guess from the two previous solutions
// (extint_v) and a solve to eps 10^(l-N+1).  rhs(l) writes level l's
// right-hand side into P.b64.  record: keep iterations and times in the plan.
int excmg_cascade(Plan& P, const std::function<int(int)>& rhs, double eps, bool record, std::vector<int>& its,
                  std::vector<int>& status) {
    const int ns = P.ns, N = P.nlev;
    const size_t nfine = (size_t)P.lev[N - 1].nl * ns * sizeof(double2);
    RC(P.u0.alloc(nfine));
    RC(P.u1.alloc(nfine));
    RC(P.ut.alloc(nfine));
    double tol = eps * std::pow(10.0, -N + 1);
    for (int l = 0; l < 2; l++) {
        const double t0 = now_ms();
        const Level& L = P.lev[l];
        RC(rhs(l));
        CK(cudaMemsetAsync(P.x64.p, 0, (size_t)L.nl * ns * sizeof(double2), P.st));
        RC(solve_level(P, L, P.o.coarse_tol, P.o.coarse_maxit, true, its, status));
        double2* dst = l == 0 ? P.u0.as<double2>() : P.u1.as<double2>();
        CK(cudaMemcpyAsync(dst, P.x64.p, (size_t)L.nl * ns * sizeof(double2), cudaMemcpyDeviceToDevice, P.st));
        CK(cudaStreamSynchronize(P.st));
        if (record) {
            record_iters(P, l, its);
            P.level_ms[l] = now_ms() - t0;
            log_level(P, l, its, status, P.level_ms[l]);
        }
    }
    tol = tol * 10;
    for (int l = 2; l < N; l++) {
        tol = tol * 10;
        const double t0 = now_ms();
        const Level& L = P.lev[l];
        RC(prolongate(P, l, P.u0.as<double2>(), P.u1.as<double2>(), P.x64.as<double2>()));
        RC(rhs(l));
        if (record && l == N - 1) history_start(P, P.o.maxit_level);
        const int rcs = solve_level(P, L, tol, P.o.maxit_level, false, its, status);
        P.rec_on = false;
        RC(rcs);
        CK(cudaStreamSynchronize(P.st));
        if (record) {
            record_iters(P, l, its);
            P.level_ms[l] = now_ms() - t0;
            log_level(P, l, its, status, P.level_ms[l]);
        }
        if (l < N - 1) {
            std::swap(P.u0.p, P.u1.p);
            std::swap(P.u0.bytes, P.u1.bytes);
            CK(cudaMemcpyAsync(P.u1.p, P.x64.p, (size_t)L.nl * ns * sizeof(double2), cudaMemcpyDeviceToDevice, P.st));
        }
    }
    return SFDX_OK;
}

static int plan_solve(Plan& P) {
    const int ns = P.ns;
    const Level& F = P.lev[P.nlev - 1];
    P.iters.assign((size_t)ns * P.nlev, 0);
    P.relres.assign(ns, 0.0);
    std::vector<int> its, status;
    int rc_conv = SFDX_OK;
    const size_t nfine = (size_t)F.nl * ns * sizeof(double2);
    RC(P.x64.alloc(nfine));
    RC(P.b64.alloc(nfine));
    P.xf_valid = false;
    P.base_valid = false;
    std::vector<double> col;
    P.level_ms.assign(P.nlev, 0.0);
    if (!P.o.excmg) {
        double t0 = now_ms();
        RC(level_column(P, F, col));
        RC(level_rhs(P, F, col));
        CK(cudaMemsetAsync(P.x64.p, 0, nfine, P.st));
        history_start(P, P.o.maxit_plain);
        const int rcs = solve_level(P, F, P.o.eps, P.o.maxit_plain, false, its, status);
        P.rec_on = false;
        RC(rcs);
        record_iters(P, P.nlev - 1, its);
        rc_conv = status_to_rc(status);
        CK(cudaStreamSynchronize(P.st));
        P.level_ms[0] = now_ms() - t0;
        log_level(P, 0, its, status, P.level_ms[0]);
    } else {
        auto rhs = [&](int l) -> int {
            RC(level_column(P, P.lev[l], col));
            return level_rhs(P, P.lev[l], col);
        };
        RC(excmg_cascade(P, rhs, P.o.eps, true, its, status));
        rc_conv = status_to_rc(status);
        P.cascade_gen = P.sigma_gen;
    }
    RC(true_residual(P, F, P.b64.as<double2>(), P.x64.as<double2>(), P.relres.data(), nullptr));
    // de-interleave into [nf][2][nl] (system-major)
    RC(P.ex_out.alloc(nfine));
    const int B = block_for(ns);
    KL(k_scatter_sys<double><<<grid_for(F.nl * ns, B, 16), B, 0, P.st>>>(F.nl, ns, P.x64.as<double2>(), P.ex_out.as<double2>()));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(P.st));
    P.have_solution = true;
    P.sol_gen = P.sigma_gen;
    return rc_conv;
}

// x += a over n complex128 values
static __global__ void k_add_to(int64_t n, const double2* __restrict__ a, double2* __restrict__ x) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = x[g], w = a[g];
        x[g] = make_double2(v.x + w.x, v.y + w.y);
    }
}

// Finest level only, for a changed conductivity, from the fields x0 of the last
// full solve.  tol > 0: solve A x = b from x0 to relative residual tol.
// tol <= 0: solve the correction equation A d = b - A x0 from zero to a
// relative reduction |tol| (or eps) of that residual, then x = x0 + d -- the
// residual's own scale sets the tolerance, so a small perturbation of the
// model is resolved to the same relative accuracy as a full solve.
static int plan_resolve(Plan& P, double tol) {
    const int ns = P.ns;
    const Level& F = P.lev[P.nlev - 1];
    const int64_t n = F.nl * ns;
    const size_t nfine = (size_t)n * sizeof(double2);
    if (!P.base_valid) {
        RC(P.xbase.alloc(nfine));
        CK(cudaMemcpyAsync(P.xbase.p, (P.xf_valid ? P.xf : P.x64).p, nfine, cudaMemcpyDeviceToDevice, P.st));
        P.base_valid = true;
    }
    CK(cudaMemcpyAsync(P.x64.p, P.xbase.p, nfine, cudaMemcpyDeviceToDevice, P.st));
    P.xf_valid = false;
    std::vector<double> col;
    RC(level_column(P, F, col));
    RC(level_rhs(P, F, col));
    std::vector<int> its, status;
    const double t0 = now_ms();
    if (tol > 0) {
        RC(solve_level(P, F, tol, P.o.maxit_plain, false, its, status));
    } else {
        std::vector<double> r0(ns);
        RC(true_residual(P, F, P.b64.as<double2>(), P.x64.as<double2>(), r0.data(), nullptr));  // r64 = b - A x0
        CK(cudaMemcpyAsync(P.b64.p, P.r64.p, nfine, cudaMemcpyDeviceToDevice, P.st));
        CK(cudaMemsetAsync(P.x64.p, 0, nfine, P.st));
        RC(solve_level(P, F, tol < 0 ? -tol : P.o.eps, P.o.maxit_plain, false, its, status));
        KL(k_add_to<<<grid_for(n, 256, 16), 256, 0, P.st>>>(n, P.xbase.as<double2>(), P.x64.as<double2>()));
        CK(cudaGetLastError());
        RC(level_rhs(P, F, col));  // b again, for the reported residual
    }
    record_iters(P, P.nlev - 1, its);
    RC(true_residual(P, F, P.b64.as<double2>(), P.x64.as<double2>(), P.relres.data(), nullptr));
    const int B = block_for(ns);
    KL(k_scatter_sys<double><<<grid_for(F.nl * ns, B, 16), B, 0, P.st>>>(F.nl, ns, P.x64.as<double2>(), P.ex_out.as<double2>()));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(P.st));
    P.level_ms.assign(P.nlev, 0.0);
    P.level_ms[P.nlev - 1] = now_ms() - t0;
    P.have_solution = true;
    P.sol_gen = P.sigma_gen;
    return status_to_rc(status);
}

static int validate_opts(const sfdx_opts& o) {
    if (o.excmg && o.level < 3) return SFDX_ERR_ARG;
    if (o.precond == 'I') return SFDX_ERR_UNSUPPORTED;  // ILU(0), pre_type = 'I': not built
    if (o.precond != 'S' && o.precond != 'J' && o.precond != 'G') return SFDX_ERR_ARG;
    if (o.precision != SFDX_FP64 && o.precision != SFDX_MIXED) return SFDX_ERR_ARG;
    if (o.div_cor < 0 || o.div_cor > 2) return SFDX_ERR_ARG;
    if (o.div_cor == 2 && (o.corr_intv < 1 || !(o.corr_tol > 0))) return SFDX_ERR_ARG;
    if (o.solver != SFDX_SOLVER_BICGSTAB && o.solver != SFDX_SOLVER_GPBICG && o.solver != SFDX_SOLVER_TFQMR &&
        o.solver != SFDX_SOLVER_BICG && o.solver != SFDX_SOLVER_COCR)
        return SFDX_ERR_ARG;
    if (o.eps <= 0 || o.maxit_plain <= 0 || o.maxit_level <= 0) return SFDX_ERR_ARG;
    if (o.batch != 0) return SFDX_ERR_UNSUPPORTED;
    if (!(o.ssor_omega > 0 && o.ssor_omega < 2)) return SFDX_ERR_ARG;
    return SFDX_OK;
}

}  // namespace sfdx

// ====================================================================== C ABI
struct sfdx_plan {
    Plan P;
};

extern "C" void sfdx_default_opts(sfdx_opts* o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->level = 3;
    o->eps = 1e-8;
    o->solver = SFDX_SOLVER_BICGSTAB;
    o->excmg = 0;            // fwd_acc = 0 (global_para.f90:19)
    o->precond = 'S';        // pre_type = 'S' (global_para.f90:18)
    o->div_cor = 1;          // global_para.f90:8
    o->corr_intv = 200;      // global_para.f90:9
    o->corr_tol = 1e-3;      // global_para.f90:10
    o->ssor_omega = 1.0;     // solvers.f90:14
    o->sigma_air = 1e-9;     // global_para.f90:12
    o->maxit_plain = 5000;   // fdfe_main.f90:993
    o->maxit_level = 1000;   // fdfe_main.f90:1414
    o->precision = SFDX_FP64;
    o->quirks = SFDX_QUIRKS_REFERENCE;
    // The two coarsest levels only feed the extrapolated guess: its residual on
    // the next level is the same for a coarse solve to 1e-6 as for an exact
    // (direct) one, so 1e-6 in FP64 stands in for PARDISO.
    // levels 1-2 stand in for PARDISO's direct solves: near-exact, because the
    // relative residual is dominated by the Dirichlet rows of b (identity rows
    // solved after one preconditioner application) -- at 1e-6 the interior of the
    // coarse fields was barely solved
    o->coarse_tol = 1e-12;
    o->coarse_maxit = 3000;
    o->reliable_every = 40;
    o->batch = 0;
    o->verbose = 0;
    o->use_graphs = 1;
}

extern "C" const char* sfdx_strerror(int code) {
    switch (code) {
        case SFDX_OK: return "ok";
        case SFDX_ERR_ARG: return "invalid argument";
        case SFDX_ERR_MESH: return "mesh sizes not divisible by 2^level (or level too large)";
        case SFDX_ERR_CUDA: return "CUDA error or no CUDA device";
        case SFDX_ERR_NOCONV: return "iteration limit reached before the tolerance";
        case SFDX_ERR_NAN: return "NaN encountered";
        case SFDX_ERR_RECEIVER: return "receiver outside the interpolation stencil";
        case SFDX_ERR_IO: return "model/data file missing or malformed";
        case SFDX_ERR_UNSUPPORTED: return "option combination not implemented";
        case SFDX_ERR_TIMEOUT: return "bounded device wait ran out";
        case SFDX_ERR_NOMEM: return "device allocation failed or size above a fixed limit";
        default: return "unknown status";
    }
}

extern "C" int sfdx_version(void) { return 100; }

extern "C" int sfdx_plan_create(sfdx_plan** out, const sfdx_opts* opts, int nx, int ny, int nz, int nair,
                                const double* a, const double* b, const double* c, int nf, const double* freq) {
    if (!out || !a || !b || !c || !freq || nx < 2 || ny < 2 || nz < 2 || nf < 1 || nair < 0 || nair > nz)
        return SFDX_ERR_ARG;
    sfdx_opts o;
    if (opts) o = *opts;
    else sfdx_default_opts(&o);
    RC(validate_opts(o));
    std::unique_ptr<sfdx_plan> h(new sfdx_plan());
    Plan& P = h->P;
    P.o = o;
    P.nf = nf;
    P.ns = 2 * nf;
    if (P.ns > SFDX_MAX_SYSTEMS) return SFDX_ERR_UNSUPPORTED;
    P.freq.assign(freq, freq + nf);
    P.wm.resize(P.ns);
    for (int f = 0; f < nf; f++) {
        if (!(freq[f] > 0)) return SFDX_ERR_ARG;
        P.wm[2 * f] = P.wm[2 * f + 1] = 2 * kPi * freq[f] * kMu;
    }
    P.nlev = o.excmg ? o.level : 1;
    {  // the hot kernels index edge x system work items in 32 bits
        const int64_t nl = (int64_t)nx * (ny + 1) * (nz + 1) + (int64_t)(nx + 1) * ny * (nz + 1) +
                           (int64_t)(nx + 1) * (ny + 1) * nz;
        if (nl * P.ns >= (1LL << 31)) return SFDX_ERR_UNSUPPORTED;
    }
    if (o.excmg) {
        const int f = 1 << o.level;  // cubic_interp tiles 8 fine cells on level 3 and up
        if (nx % f || ny % f || nz % f) return SFDX_ERR_MESH;
        if (nx / f < 1 || ny / f < 1 || nz / f < 1) return SFDX_ERR_MESH;
    }
    // every argument check above runs before the first CUDA call
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return SFDX_ERR_CUDA;
    CK(cudaStreamCreateWithFlags(&P.own_st, cudaStreamNonBlocking));
    P.st = P.own_st;
    P.lev.resize(P.nlev);
    for (int l = 0; l < P.nlev; l++) {
        Level& L = P.lev[l];
        const int k = P.nlev - 1 - l, asf = 1 << k;
        L.set_dims(nx / asf, ny / asf, nz / asf);
        L.nair = nair / asf;
        L.a.resize(L.nx);
        L.b.resize(L.ny);
        L.c.resize(L.nz);
        // mesh_coarsen spacing sums (fdfe_main.f90:40-48)
        for (int i = 0; i < L.nx; i++) { double s = 0; for (int q = i * asf; q < (i + 1) * asf; q++) s += a[q]; L.a[i] = s; }
        for (int i = 0; i < L.ny; i++) { double s = 0; for (int q = i * asf; q < (i + 1) * asf; q++) s += b[q]; L.b[i] = s; }
        for (int i = 0; i < L.nz; i++) { double s = 0; for (int q = i * asf; q < (i + 1) * asf; q++) s += c[q]; L.c[i] = s; }
        RC(upload_level_tables(L, P.st));
    }
    RC(P.d_state.alloc(sizeof(KState) * P.ns));
    RC(P.d_wm.alloc(sizeof(double) * P.ns));
    CK(cudaMemcpyAsync(P.d_wm.p, P.wm.data(), sizeof(double) * P.ns, cudaMemcpyHostToDevice, P.st));
    RC(P.d_counter.alloc(sizeof(unsigned int)));
    CK(cudaMemsetAsync(P.d_counter.p, 0, sizeof(unsigned int), P.st));
    RC(P.d_flag.alloc(sizeof(int)));
    CK(cudaStreamSynchronize(P.st));
    *out = h.release();
    return SFDX_OK;
}

extern "C" int sfdx_plan_solve(sfdx_plan* plan, const double* sigma, int sigma_on_device, double* ex, int ex_on_device,
                               int* iters, double* relres) {
    if (!plan || !sigma) return SFDX_ERR_ARG;
    Plan& P = plan->P;
    RC(set_conductivity(P, sigma, sigma_on_device != 0));
    int rc = plan_solve(P);
    if (rc != SFDX_OK && rc != SFDX_ERR_NOCONV) return rc;
    const Level& F = P.lev[P.nlev - 1];
    if (ex) {
        CK(cudaMemcpyAsync(ex, P.ex_out.p, (size_t)F.nl * P.ns * sizeof(double2),
                           ex_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P.st));
        CK(cudaStreamSynchronize(P.st));
    }
    if (iters) memcpy(iters, P.iters.data(), P.iters.size() * sizeof(int));
    if (relres) memcpy(relres, P.relres.data(), P.relres.size() * sizeof(double));
    return rc;
}

// Several plans at once: each plan's solve runs on its own host thread and
// its own stream, so the GPU overlaps the models' kernels and one model's
// host synchronisations (convergence checks, restart cycles) do not stall
// the others.
extern "C" int sfdx_plan_solve_batch(int nplans, sfdx_plan* const* plans, const double* const* sigma,
                                     int sigma_on_device, double* const* ex, int ex_on_device, int* const* iters,
                                     double* const* relres, int* status) {
    if (nplans < 1 || !plans || !sigma) return SFDX_ERR_ARG;
    for (int q = 0; q < nplans; q++) {
        if (!plans[q] || !sigma[q]) return SFDX_ERR_ARG;
        for (int r = 0; r < q; r++)
            if (plans[r] == plans[q]) return SFDX_ERR_ARG;
    }
    int dev = 0;
    CK(cudaGetDevice(&dev));
    std::vector<int> rc(nplans, SFDX_OK);
    std::vector<std::thread> th;
    th.reserve(nplans);
    for (int q = 0; q < nplans; q++) {
        try {
            th.emplace_back([&, q] {
                try {
                    if (cudaSetDevice(dev) != cudaSuccess) {
                        rc[q] = SFDX_ERR_CUDA;
                        return;
                    }
                    rc[q] = sfdx_plan_solve(plans[q], sigma[q], sigma_on_device, ex ? ex[q] : nullptr, ex_on_device,
                                            iters ? iters[q] : nullptr, relres ? relres[q] : nullptr);
                } catch (...) {
                    rc[q] = SFDX_ERR_NOMEM;
                }
            });
        } catch (...) {  // no thread for this plan: report it, still join the others
            rc[q] = SFDX_ERR_NOMEM;
        }
    }
    for (auto& t : th) t.join();
    int out = SFDX_OK;
    for (int q = 0; q < nplans; q++) {
        if (status) status[q] = rc[q];
        if (rc[q] != SFDX_OK && (out == SFDX_OK || out == SFDX_ERR_NOCONV)) out = rc[q];
    }
    return out;
}

extern "C" int sfdx_plan_resolve(sfdx_plan* plan, const double* sigma, int sigma_on_device, double tol, int* iters,
                                 double* relres) {
    if (!plan || !sigma) return SFDX_ERR_ARG;
    Plan& P = plan->P;
    if (!P.have_solution) return SFDX_ERR_ARG;
    RC(set_conductivity(P, sigma, sigma_on_device != 0));
    const int rc = plan_resolve(P, tol);
    if (rc != SFDX_OK && rc != SFDX_ERR_NOCONV) return rc;
    if (iters) memcpy(iters, P.iters.data(), P.iters.size() * sizeof(int));
    if (relres) memcpy(relres, P.relres.data(), P.relres.size() * sizeof(double));
    return rc;
}

extern "C" int sfdx_plan_load(sfdx_plan* plan, const double* sigma, int sigma_on_device) {
    if (!plan || !sigma) return SFDX_ERR_ARG;
    RC(set_conductivity(plan->P, sigma, sigma_on_device != 0));
    CK(cudaStreamSynchronize(plan->P.st));
    return SFDX_OK;
}

extern "C" const double* sfdx_plan_fields(sfdx_plan* plan) {
    if (!plan || !plan->P.solution_current()) return nullptr;
    return plan->P.ex_out.as<double>();
}

extern "C" long long sfdx_plan_device_bytes(const sfdx_plan* plan) {
    if (!plan) return 0;
    const Plan& P = plan->P;
    long long s = 0;
    const DBuf* bufs[] = {&P.d_state, &P.d_wm, &P.d_pol, &P.d_edc, &P.d_part, &P.d_counter, &P.d_tol, &P.d_mask,
                          &P.d_scale, &P.d_flag, &P.x64, &P.b64, &P.r64, &P.u0, &P.u1, &P.ut, &P.ex_out, &P.errrec,
                          &P.xf, &P.x32, &P.xb, &P.cb64, &P.cx64, &P.d_idx, &P.d_pst, &P.xbase};
    for (auto* b : bufs) s += (long long)b->bytes;
    for (auto& b : P.kv) s += (long long)b.bytes;
    for (auto& b : P.dcv) s += (long long)b.bytes;
    for (auto& b : P.gcn) s += (long long)b.bytes;
    for (auto& b : P.gce) s += (long long)b.bytes;
    for (auto& L : P.lev) {
        s += (long long)(L.tab64.bytes + L.tab32.bytes + L.sig64.bytes + L.sig32.bytes + L.spac.bytes +
                         L.crd_cubic.bytes + L.crd_quad.bytes + L.rc64.bytes + L.rc32.bytes);
        for (auto& g : L.mg)
            s += (long long)(g.coef.bytes + g.dinv.bytes + g.x.bytes + g.b.bytes + g.t.bytes + g.r.bytes);
    }
    return s;
}

extern "C" void sfdx_plan_destroy(sfdx_plan* plan) { delete plan; }

extern "C" long long sfdx_launch_count(void) { return g_launches.load(); }

extern "C" int sfdx_plan_set_stream(sfdx_plan* plan, void* stream) {
    if (!plan) return SFDX_ERR_ARG;
    CK(cudaStreamSynchronize(plan->P.st));
    plan->P.st = stream ? (cudaStream_t)stream : plan->P.own_st;
    return SFDX_OK;
}

// Times `reps` launches of one kernel family on the plan's finest level
// with CUDA events on the plan's stream (the plan must have solved once so
// that the conductivity is resident).  kernel: 0 operator (complex64),
// 1 operator (complex128), 2 multi-colour SSOR application (complex64, all
// 11 colour launches), 3 multi-colour SSOR (complex128), 4 prolongation
// 2h->h (complex128).  bytes: algorithmic HBM bytes of one application.
extern "C" int sfdx_plan_kernel_time(sfdx_plan* plan, int kernel, int reps, double* ms, double* bytes) {
    if (!plan || !ms || reps < 1) return SFDX_ERR_ARG;
    Plan& P = plan->P;
    if (!P.lev[P.nlev - 1].sig64.p) return SFDX_ERR_ARG;  // conductivity not loaded yet
    const Level& F = P.lev[P.nlev - 1];
    const int ns = P.ns;
    const size_t n = (size_t)F.nl * ns;
    const bool f32 = (kernel == 0 || kernel == 2 || kernel == 4);
    const size_t es = f32 ? 8 : 16;
    for (int q = 0; q < 3; q++) RC(P.kv[q].alloc(n * es));
    std::vector<KState> init(ns);
    for (int q = 0; q < ns; q++) {
        memset(&init[q], 0, sizeof(KState));
        init[q].wm = P.wm[q];
        init[q].active = 1;
    }
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    // deterministic non-zero input
    if (f32) KL(k_pattern<float><<<grid_for(n, 256), 256, 0, P.st>>>(n, P.kv[0].as<float2>()));
    else KL(k_pattern<double><<<grid_for(n, 256), 256, 0, P.st>>>(n, P.kv[0].as<double2>()));
    const int B = block_for(ns);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // 2, 3: the multi-colour SSOR alone whatever the plan's preconditioner;
    // 4: one edge-multigrid V-cycle (complex64) over all levels
    const int save_pre = P.o.precond;
    auto launch = [&]() {
        switch (kernel) {
            case 0: apply_op<float>(P, F, P.kv[0].as<float2>(), P.kv[1].as<float2>()); break;
            case 1: apply_op<double>(P, F, P.kv[0].as<double2>(), P.kv[1].as<double2>()); break;
            case 2: P.o.precond = 'S'; precond_vec<float>(P, F, P.kv[1].as<float2>(), P.kv[0].as<float2>()); break;
            case 3: P.o.precond = 'S'; precond_vec<double>(P, F, P.kv[1].as<double2>(), P.kv[0].as<double2>()); break;
            case 4: P.o.precond = 'G'; precond_vec<float>(P, F, P.kv[1].as<float2>(), P.kv[0].as<float2>()); break;
            default: break;
        }
        P.o.precond = save_pre;
    };
    launch();
    CK(cudaEventRecord(e0, P.st));
    for (int r = 0; r < reps; r++) launch();
    CK(cudaEventRecord(e1, P.st));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaGetLastError());
    *ms = t / reps;
    // algorithmic bytes: read x, write y (complex, per edge and system) and
    // the six conductivities per cell once per launch
    const double p = f32 ? 4.0 : 8.0;
    double b1 = (double)F.nl * ns * 4 * p + (double)F.ncell * 6 * p;
    if (kernel == 2 || kernel == 3) b1 *= 2;  // forward + backward sweep
    if (kernel == 4) {
        // V-cycle: per level two SSOR applications (2 x 2 operator passes), five
        // residual-type passes (read x and b, write r: 6p per edge and system),
        // transfer and nodal passes (~4 vector passes); levels shrink 8x each
        double lev = (double)F.nl * ns * (4 * 4 * p + 5 * 6 * p + 4 * 2 * p);
        b1 = 0;
        for (int l = 0; l < P.nlev; l++, lev /= 8) b1 += lev;
    }
    if (bytes) *bytes = b1;
    return SFDX_OK;
}

// Pick the systems-per-thread grouping of the complex64 and complex128 hot
// kernels by timing one operator application plus one multi-colour SSOR
// application per candidate on the finest level.
extern "C" int sfdx_plan_autotune(sfdx_plan* plan, int reps, int* vs32, int* vs64) {
    if (!plan || reps < 1) return SFDX_ERR_ARG;
    Plan& P = plan->P;
    const Level& F = P.lev[P.nlev - 1];
    if (!F.sig64.p) return SFDX_ERR_ARG;  // conductivity not loaded yet
    const int ns = P.ns;
    const size_t n = (size_t)F.nl * ns;
    for (int q = 0; q < 3; q++) RC(P.kv[q].alloc(n * 16));
    std::vector<KState> init(ns);
    for (int q = 0; q < ns; q++) {
        memset(&init[q], 0, sizeof(KState));
        init[q].wm = P.wm[q];
        init[q].active = 1;
    }
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // complex64: eight iterations of the plan's Krylov solver (its fused
    // operator, sweep and update kernels, as a solve runs them) on a
    // deterministic right-hand side; complex128 (coarse levels, residual
    // replacements): an operator plus a preconditioner application
    DBuf tb, tx;
    const bool kry = P.o.solver == SFDX_SOLVER_GPBICG || P.o.solver == SFDX_SOLVER_BICGSTAB ||
                     P.o.solver == SFDX_SOLVER_COCR;
    if (kry) {
        RC(tb.alloc(n * sizeof(float2)));
        RC(tx.alloc(n * sizeof(float2)));
        KL(k_pattern<float><<<grid_for(n, 256), 256, 0, P.st>>>(n, tb.as<float2>()));
    }
    auto iterations = [&]() -> int {
        CK(cudaMemsetAsync(tx.p, 0, n * sizeof(float2), P.st));
        const float2* b = tb.as<float2>();
        float2* x = tx.as<float2>();
        if (P.o.solver == SFDX_SOLVER_GPBICG) return gpbicg<float>(P, F, b, x, nullptr, 1e-30, 8, nullptr);
        if (P.o.solver == SFDX_SOLVER_COCR) return cocr<float>(P, F, b, x, nullptr, 1e-30, 8, nullptr);
        return bicgstab<float>(P, F, b, x, nullptr, 1e-30, 8, nullptr);
    };
    int best[2] = {P.vs32, P.vs64};
    for (int prec = 0; prec < 2; prec++) {
        double tbest = 1e300;
        for (int cand : {4, 2, 1}) {
            if (vs_pick(ns, cand) != cand) continue;
            int& slot = prec == 0 ? P.vs32 : P.vs64;
            slot = cand;
            float t = 0;
            for (int r = 0; r <= reps; r++) {  // first pass warms up
                if (r == 1) CK(cudaEventRecord(e0, P.st));
                if (prec == 0 && kry) {
                    RC(iterations());
                } else if (prec == 0) {
                    RC(apply_op<float>(P, F, P.kv[0].as<float2>(), P.kv[1].as<float2>()));
                    RC(precond_vec<float>(P, F, P.kv[2].as<float2>(), P.kv[1].as<float2>()));
                } else {
                    RC(apply_op<double>(P, F, P.kv[0].as<double2>(), P.kv[1].as<double2>()));
                    RC(precond_vec<double>(P, F, P.kv[2].as<double2>(), P.kv[1].as<double2>()));
                }
            }
            CK(cudaEventRecord(e1, P.st));
            CK(cudaEventSynchronize(e1));
            CK(cudaEventElapsedTime(&t, e0, e1));
            if (t < tbest) {
                tbest = t;
                best[prec] = cand;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P.vs32 = best[0];
    P.vs64 = best[1];
    if (vs32) *vs32 = vs_pick(ns, P.vs32);
    if (vs64) *vs64 = vs_pick(ns, P.vs64);
    if (P.o.verbose || getenv("SFDX_VERBOSE"))
        fprintf(stderr, "sfdx: autotune: %d systems per thread (complex64), %d (complex128)\n", vs_pick(ns, P.vs32),
                vs_pick(ns, P.vs64));
    return SFDX_OK;
}

extern "C" int sfdx_plan_level_fields(sfdx_plan* plan, int level, double* ex) {
    if (!plan || !ex) return SFDX_ERR_ARG;
    Plan& P = plan->P;
    const int N = P.nlev;
    if (N < 3 || (level != N - 2 && level != N - 1) || P.cascade_gen != P.sigma_gen || !P.solution_current())
        return SFDX_ERR_ARG;
    const Level& L = P.lev[level - 1];
    const DBuf& src = level == N - 2 ? P.u0 : P.u1;  // excmg_cascade leaves levels N-2, N-1 there
    const int ns = P.ns;
    RC(P.ut.alloc((size_t)L.nl * ns * sizeof(double2)));
    const int B = block_for(ns);
    KL(k_scatter_sys<double><<<grid_for(L.nl * ns, B, 16), B, 0, P.st>>>(L.nl, ns, src.as<double2>(), P.ut.as<double2>()));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ex, P.ut.p, (size_t)L.nl * ns * sizeof(double2), cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

extern "C" int sfdx_plan_history(const sfdx_plan* plan, double* hist, int maxit) {
    if (!plan || !hist || maxit < 1) return SFDX_ERR_ARG;
    const Plan& P = plan->P;
    if (!P.solution_current() || P.rec_len < 1) return SFDX_ERR_ARG;
    for (int s = 0; s < P.ns; s++)
        for (int i = 0; i < maxit; i++)
            hist[(size_t)s * maxit + i] = i < P.rec_len ? P.rec_hist[(size_t)s * P.rec_len + i] : 0.0;
    return SFDX_OK;
}

extern "C" int sfdx_plan_level_times(const sfdx_plan* plan, double* ms, int n) {
    if (!plan || !ms) return SFDX_ERR_ARG;
    const Plan& P = plan->P;
    for (int l = 0; l < n; l++) ms[l] = l < (int)P.level_ms.size() ? P.level_ms[l] : 0.0;
    return SFDX_OK;
}

// impedance from the plan's device-resident solution: copy only the edge
// planes the evaluation reads.
// Impedances (and tippers) at the receivers from the plan's device fields:
// post_process + arho_interp2 (fdfe_main.f90:549-790) evaluated as
// impedance_from_fields does on the host (sfdx_host.cpp), one thread per
// (receiver, frequency).  The surface E and H of the nine stencil cells come
// straight from the edge planes nair and nair+1 of both polarisations.
struct ImpGeom {
    int nx, ny, nair, nrec, nf, out_type, ncomp;
    int64_t nl, xnl, ynl;
    double cz;
};
// surface E (x, y) and H (x, y, z) of one polarisation at cell (i, j)
__device__ __forceinline__ void imp_cell(const double2* __restrict__ x, const ImpGeom& g, const double* a,
                                         const double* b, double2 iwm, int i, int j, double2 E[2], double2 H[3]) {
    const int nx = g.nx, ny = g.ny;
    const int64_t pex = (int64_t)nx * (ny + 1), pey = (int64_t)(nx + 1) * ny, pez = (int64_t)(nx + 1) * (ny + 1);
    auto ex = [&](int pl, int ii, int jj) { return x[(int64_t)(g.nair + pl) * pex + (int64_t)jj * nx + ii]; };
    auto ey = [&](int pl, int ii, int jj) {
        return x[g.xnl + (int64_t)(g.nair + pl) * pey + (int64_t)jj * (nx + 1) + ii];
    };
    auto ez = [&](int ii, int jj) { return x[g.xnl + g.ynl + (int64_t)g.nair * pez + (int64_t)jj * (nx + 1) + ii]; };
    auto half = [](double2 u, double2 v) { return mk<double>((u.x + v.x) / 2.0, (u.y + v.y) / 2.0); };
    auto over = [](double2 u, double d) { return mk<double>(u.x / d, u.y / d); };
    const double2 ex0 = half(ex(0, i, j), ex(0, i, j + 1));
    const double2 ey0 = half(ey(0, i, j), ey(0, i + 1, j));
    E[0] = ex0;
    E[1] = ey0;
    const double2 exz = over(half(ex(1, i, j), ex(1, i, j + 1)) - ex0, g.cz);
    const double2 ezx = over(half(ez(i + 1, j), ez(i + 1, j + 1)) - half(ez(i, j + 1), ez(i, j)), a[i]);
    const double2 eyz = over(half(ey(1, i, j), ey(1, i + 1, j)) - ey0, g.cz);
    const double2 ezy = over(half(ez(i, j + 1), ez(i + 1, j + 1)) - half(ez(i, j), ez(i + 1, j)), b[j]);
    const double2 exy = over(ex(0, i, j + 1) - ex(0, i, j), b[j]);
    const double2 eyx = over(ey(0, i + 1, j) - ey(0, i, j), a[i]);
    H[1] = cdiv<double>(exz - ezx, iwm);
    H[0] = cdiv<double>(ezy - eyz, iwm);
    H[2] = cdiv<double>(exy - eyx, iwm);
}

static __global__ void k_impedance(ImpGeom g, const double2* __restrict__ fields, const double* __restrict__ a,
                                   const double* __restrict__ b, const double* __restrict__ wmu,
                                   const int* __restrict__ id, const int* __restrict__ idz,
                                   const double* __restrict__ w, double* __restrict__ out, double* __restrict__ tip) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nrec * g.nf) return;
    const int f = t / g.nrec, r = t - f * g.nrec;
    const double2 iwm = mk<double>(0.0, wmu[f]);
    double2 fr[2][5];
    for (int p = 0; p < 2; p++) {
        const double2* x = fields + (int64_t)(2 * f + p) * g.nl;
        for (int q = 0; q < 5; q++) fr[p][q] = zero<double>();
        for (int s = 0; s < 9; s++) {
            const double ws = w[r * 9 + s];
            double2 E[2], H[3];
            const int c = id[r * 9 + s];
            imp_cell(x, g, a, b, iwm, c % g.nx, c / g.nx, E, H);
            fr[p][0] = fr[p][0] + rmul<double>(ws, E[0]);
            fr[p][1] = fr[p][1] + rmul<double>(ws, E[1]);
            fr[p][2] = fr[p][2] + rmul<double>(ws, H[0]);
            fr[p][3] = fr[p][3] + rmul<double>(ws, H[1]);
            const int cz = idz[r * 9 + s];
            imp_cell(x, g, a, b, iwm, cz % g.nx, cz / g.nx, E, H);
            fr[p][4] = fr[p][4] + rmul<double>(ws, H[2]);
        }
    }
    const double2 det = cmul<double>(fr[0][2], fr[1][3]) - cmul<double>(fr[1][2], fr[0][3]);
    const double2 zxy = cdiv<double>(cmul<double>(fr[1][0], fr[0][2]) - cmul<double>(fr[0][0], fr[1][2]), det);
    const double2 zyx = cdiv<double>(cmul<double>(fr[0][1], fr[1][3]) - cmul<double>(fr[1][1], fr[0][3]), det);
    double* o = out + ((int64_t)f * g.nrec + r) * g.ncomp;
    if (g.out_type == 3) {
        // the full tensor Z = E H^-1 (the reference forms Zxy and Zyx only)
        const double2 zxx = cdiv<double>(cmul<double>(fr[0][0], fr[1][3]) - cmul<double>(fr[1][0], fr[0][3]), det);
        const double2 zyy = cdiv<double>(cmul<double>(fr[1][1], fr[0][2]) - cmul<double>(fr[0][1], fr[1][2]), det);
        const double2 zz[4] = {zxx, zxy, zyx, zyy};
        for (int q = 0; q < 4; q++) {
            o[2 * q] = zz[q].x;
            o[2 * q + 1] = zz[q].y;
        }
    } else if (g.out_type == 2) {
        const double2 a2 = cmul<double>(zxy, zxy), b2 = cmul<double>(zyx, zyx);
        o[0] = sqrt(cabs2<double>(a2)) / wmu[f];  // |i Z^2| = |Z^2|
        o[1] = sqrt(cabs2<double>(b2)) / wmu[f];
        o[2] = -atan(zxy.y / zxy.x) * 180.0 / 3.141592653589793238462643;
        o[3] = -atan(zyx.y / zyx.x) * 180.0 / 3.141592653589793238462643;
    } else {
        o[0] = zxy.x;
        o[1] = zxy.y;
        o[2] = zyx.x;
        o[3] = zyx.y;
    }
    if (tip) {
        const double2 tx = cdiv<double>(cmul<double>(fr[1][3], fr[0][4]) - cmul<double>(fr[0][3], fr[1][4]), det);
        const double2 ty = cdiv<double>(cmul<double>(fr[0][2], fr[1][4]) - cmul<double>(fr[1][2], fr[0][4]), det);
        double* tp = tip + ((int64_t)f * g.nrec + r) * 4;
        tp[0] = tx.x;
        tp[1] = tx.y;
        tp[2] = ty.x;
        tp[3] = ty.y;
    }
}

extern "C" int sfdx_plan_impedance(sfdx_plan* plan, int nrec, const double* recv, int out_type, double* out,
                                   double* tipper) {
    if (!plan || !recv || !out || nrec < 1) return SFDX_ERR_ARG;
    Plan& P = plan->P;
    if (!P.solution_current()) return SFDX_ERR_ARG;
    const Level& F = P.lev[P.nlev - 1];
    const int transpose = (P.o.quirks & SFDX_QUIRK_RX_TRANSPOSE) ? 1 : 0;
    const int ncomp = out_type == 3 ? 8 : 4;
    std::vector<int> id((size_t)nrec * 9), idz((size_t)nrec * 9);
    std::vector<double> w((size_t)nrec * 9), wmu(P.nf);
    RC(receiver_stencils(F.nx, F.ny, F.a.data(), F.b.data(), nrec, recv, transpose, id.data(), idz.data(), w.data()));
    const double pi = 3.141592653589793238462643, mu = 4.0 * pi * 1e-7;
    for (int f = 0; f < P.nf; f++) wmu[f] = 2.0 * pi * P.freq[f] * mu;
    // device workspace: a, b, wmu, w, out, tip (doubles), id, idz (ints)
    const size_t nd = (size_t)F.nx + F.ny + P.nf + w.size() + (size_t)P.nf * nrec * (ncomp + 4);
    RC(P.d_imp.alloc(nd * sizeof(double) + 2 * id.size() * sizeof(int)));
    double* da = P.d_imp.as<double>();
    double* db = da + F.nx;
    double* dwm = db + F.ny;
    double* dw = dwm + P.nf;
    double* dout = dw + w.size();
    double* dtip = dout + (size_t)P.nf * nrec * ncomp;
    int* did = reinterpret_cast<int*>(da + nd);
    int* didz = did + id.size();
    CK(cudaMemcpyAsync(da, F.a.data(), F.nx * sizeof(double), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(db, F.b.data(), F.ny * sizeof(double), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(dwm, wmu.data(), P.nf * sizeof(double), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(did, id.data(), id.size() * sizeof(int), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(didz, idz.data(), idz.size() * sizeof(int), cudaMemcpyHostToDevice, P.st));
    ImpGeom g;
    g.nx = F.nx; g.ny = F.ny; g.nair = F.nair; g.nrec = nrec; g.nf = P.nf; g.out_type = out_type; g.ncomp = ncomp;
    g.nl = F.nl; g.xnl = F.xnl; g.ynl = F.ynl;
    g.cz = F.c[F.nair];
    const int n = nrec * P.nf;
    KL(k_impedance<<<(n + 127) / 128, 128, 0, P.st>>>(g, P.ex_out.as<double2>(), da, db, dwm, did, didz, dw, dout,
                                                       tipper ? dtip : nullptr));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, (size_t)P.nf * nrec * ncomp * sizeof(double), cudaMemcpyDeviceToHost, P.st));
    if (tipper)
        CK(cudaMemcpyAsync(tipper, dtip, (size_t)P.nf * nrec * 4 * sizeof(double), cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

extern "C" int sfdx_plan_misfit_grad(sfdx_plan* plan, int nrec, const double* recv, const double* zobs,
                                     const double* wts, double tol, double* misfit, double* zpred, double* grad,
                                     int grad_on_device, int* adj_iters, double* adj_relres) {
    if (!plan || !recv || !zobs || !misfit || nrec < 1) return SFDX_ERR_ARG;
    if (grad && grad_on_device && (reinterpret_cast<uintptr_t>(grad) & 7)) return SFDX_ERR_ARG;  // stored as double
    return misfit_grad(plan->P, nrec, recv, zobs, wts, tol, misfit, zpred, grad, grad_on_device != 0, adj_iters,
                       adj_relres);
}

extern "C" int sfdx_fwd_solve(const sfdx_opts* o, int nx, int ny, int nz, int nair, const double* a, const double* b,
                              const double* c, const double* sigma, int nf, const double* freq, double* ex, int* iters,
                              double* relres) {
    sfdx_plan* p = nullptr;
    RC(sfdx_plan_create(&p, o, nx, ny, nz, nair, a, b, c, nf, freq));
    int rc = sfdx_plan_solve(p, sigma, 0, ex, 0, iters, relres);
    sfdx_plan_destroy(p);
    return rc;
}

extern "C" int sfdx_impedance(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c,
                              int nf, const double* freq, const double* ex, int nrec, const double* recv, int out_type,
                              int quirks, double* out, double* tipper) {
    if (!a || !b || !c || !freq || !ex || !recv || !out || nrec < 1 || nair < 0 || nair + 1 >= nz) return SFDX_ERR_ARG;
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1), ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    const size_t pex = (size_t)nx * (ny + 1), pey = (size_t)(nx + 1) * ny, pez = (size_t)(nx + 1) * (ny + 1);
    const std::complex<double>* X = reinterpret_cast<const std::complex<double>*>(ex);
    for (int f = 0; f < nf; f++) {
        SurfaceView sv;
        sv.nx = nx; sv.ny = ny; sv.nair = nair;
        for (int p = 0; p < 2; p++) {
            const std::complex<double>* x = X + (size_t)(2 * f + p) * nl;
            sv.exs[p] = x + (size_t)nair * pex;
            sv.eys[p] = x + xnl + (size_t)nair * pey;
            sv.ezs[p] = x + xnl + ynl + (size_t)nair * pez;
        }
        RC(impedance_from_surface(sv, a, b, c, freq[f], nrec, recv, out_type, (quirks & SFDX_QUIRK_RX_TRANSPOSE) ? 1 : 0,
                                  out + (size_t)f * nrec * (out_type == 3 ? 8 : 4),
                                  tipper ? tipper + (size_t)f * nrec * 4 : nullptr));
    }
    return SFDX_OK;
}

extern "C" int sfdx_impedance_topo(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c,
                                   int nf, const double* freq, const double* ex, int nrec, const double* recv,
                                   int out_type, int quirks, const int* abr, const double* topo, double* out,
                                   double* tipper) {
    if (!a || !b || !c || !freq || !ex || !recv || !out || !abr || !topo || nrec < 1 || nair < 0 || nair + 1 >= nz)
        return SFDX_ERR_ARG;
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1), ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    std::vector<int> mcol((size_t)nx * ny);
    std::vector<double> czcol((size_t)nx * ny);
    RC(receiver_planes(nx, ny, nz, nair, c, abr, topo, (quirks & SFDX_QUIRK_TOPO_PLANE) ? 1 : 0, mcol.data(),
                       czcol.data()));
    const std::complex<double>* X = reinterpret_cast<const std::complex<double>*>(ex);
    for (int f = 0; f < nf; f++)
        RC(impedance_topo(X + (size_t)(2 * f) * nl, X + (size_t)(2 * f + 1) * nl, nx, ny, nz, mcol.data(), czcol.data(),
                          a, b, freq[f], nrec, recv, out_type, (quirks & SFDX_QUIRK_RX_TRANSPOSE) ? 1 : 0,
                          out + (size_t)f * nrec * (out_type == 3 ? 8 : 4),
                          tipper ? tipper + (size_t)f * nrec * 4 : nullptr));
    return SFDX_OK;
}

extern "C" int sfdx_receiver_fields(int nx, int ny, int nz, int nair, const double* a, const double* b,
                                    const double* c, int nf, const double* freq, const double* ex, int nrec,
                                    const double* recv, int quirks, double* fields) {
    if (!a || !b || !c || !freq || !ex || !recv || !fields || nrec < 1 || nair < 0 || nair + 1 >= nz)
        return SFDX_ERR_ARG;
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1), ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    const size_t pex = (size_t)nx * (ny + 1), pey = (size_t)(nx + 1) * ny, pez = (size_t)(nx + 1) * (ny + 1);
    const std::complex<double>* X = reinterpret_cast<const std::complex<double>*>(ex);
    std::complex<double>* F = reinterpret_cast<std::complex<double>*>(fields);
    std::vector<double> z((size_t)nrec * 4);
    for (int f = 0; f < nf; f++) {
        SurfaceView sv;
        sv.nx = nx; sv.ny = ny; sv.nair = nair;
        for (int p = 0; p < 2; p++) {
            const std::complex<double>* x = X + (size_t)(2 * f + p) * nl;
            sv.exs[p] = x + (size_t)nair * pex;
            sv.eys[p] = x + xnl + (size_t)nair * pey;
            sv.ezs[p] = x + xnl + ynl + (size_t)nair * pez;
        }
        RC(impedance_from_surface(sv, a, b, c, freq[f], nrec, recv, 1, (quirks & SFDX_QUIRK_RX_TRANSPOSE) ? 1 : 0,
                                  z.data(), nullptr, F + (size_t)f * nrec * 10));
    }
    return SFDX_OK;
}

// ---------------------------------------------------------------- component entry points
namespace {
// A one-level plan over host inputs, ns systems at the given frequencies.
int component_plan(sfdx_plan** h, const sfdx_opts* o, int nx, int ny, int nz, const double* a, const double* b,
                   const double* c, const double* sigma, int ns, const double* freqs, int nair = 0,
                   int levels = 0) {
    if (ns < 1 || ns > SFDX_MAX_SYSTEMS || !freqs) return SFDX_ERR_ARG;
    sfdx_opts oo;
    if (o) oo = *o;
    else sfdx_default_opts(&oo);
    // one mesh level, or `levels` 2x-coarsened ones (the edge multigrid's)
    oo.excmg = levels > 1 ? 1 : 0;
    if (levels > 1) oo.level = levels;
    // nf systems pairs: reuse plan_create with one frequency per pair, then
    // override the per-system table with the requested frequencies.
    std::vector<double> fr((ns + 1) / 2, 1.0);
    RC(sfdx_plan_create(h, &oo, nx, ny, nz, nair, a, b, c, (int)fr.size(), fr.data()));
    Plan& P = (*h)->P;
    P.ns = ns;
    if (P.lev[0].nl * ns >= (1LL << 31)) return SFDX_ERR_UNSUPPORTED;
    P.wm.resize(ns);
    for (int s = 0; s < ns; s++) P.wm[s] = 2 * kPi * freqs[s] * kMu;
    RC(P.d_wm.alloc(sizeof(double) * ns));
    CK(cudaMemcpyAsync(P.d_wm.p, P.wm.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, P.st));
    RC(P.d_state.alloc(sizeof(KState) * ns));
    if (sigma) RC(set_conductivity(P, sigma, false));
    return SFDX_OK;
}
struct PlanGuard {
    sfdx_plan* p = nullptr;
    ~PlanGuard() { if (p) sfdx_plan_destroy(p); }
};
}  // namespace

extern "C" int sfdx_apply_operator(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                                   const double* sigma, int ns, const double* freqs, int precision, const double* x,
                                   double* y) {
    if (!sigma || !x || !y) return SFDX_ERR_ARG;
    PlanGuard g;
    RC(component_plan(&g.p, nullptr, nx, ny, nz, a, b, c, sigma, ns, freqs));
    Plan& P = g.p->P;
    const Level& L = P.lev[0];
    const size_t n = (size_t)L.nl * ns;
    DBuf dx, dy;
    RC(dx.alloc(n * 16));
    RC(dy.alloc(n * 16));
    CK(cudaMemcpyAsync(dx.p, x, n * 16, cudaMemcpyHostToDevice, P.st));
    const int B = block_for(ns);
    if (precision == SFDX_FP64) {
        RC(apply_op<double>(P, L, dx.as<double2>(), dy.as<double2>()));
    } else {
        DBuf fx, fy;
        RC(fx.alloc(n * 8));
        RC(fy.alloc(n * 8));
        KL(k_convert<double, float><<<grid_for(n, 256), 256, 0, P.st>>>(n, dx.as<double2>(), fx.as<float2>()));
        RC(apply_op<float>(P, L, fx.as<float2>(), fy.as<float2>()));
        KL(k_convert<float, double><<<grid_for(n, 256), 256, 0, P.st>>>(n, fy.as<float2>(), dy.as<double2>()));
        CK(cudaStreamSynchronize(P.st));
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(y, dy.p, n * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

extern "C" int sfdx_build_rhs(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                              const double* sigma, double freq, const double* edc, double* p1, double* p2) {
    if (!sigma || !edc || !p1 || !p2) return SFDX_ERR_ARG;
    PlanGuard g;
    double fr[2] = {freq, freq};
    RC(component_plan(&g.p, nullptr, nx, ny, nz, a, b, c, sigma, 2, fr));
    Plan& P = g.p->P;
    const Level& L = P.lev[0];
    P.edc_stride = 2 * nz + 2;
    std::vector<double2> e(2 * P.edc_stride);
    for (int q = 0; q < P.edc_stride; q++) e[q] = e[P.edc_stride + q] = make_double2(edc[2 * q], edc[2 * q + 1]);
    int pols[2] = {0, 1};
    RC(P.d_edc.alloc(e.size() * sizeof(double2)));
    RC(P.d_pol.alloc(2 * sizeof(int)));
    CK(cudaMemcpyAsync(P.d_edc.p, e.data(), e.size() * sizeof(double2), cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(P.d_pol.p, pols, 2 * sizeof(int), cudaMemcpyHostToDevice, P.st));
    RC(P.b64.alloc((size_t)L.nl * 2 * sizeof(double2)));
    const int B = block_for(2);
    KL(k_build_rhs<<<grid_for(L.nl * 2, B, 16), B, 0, P.st>>>(L.lev<double>(), P.d_wm.as<double>(), P.d_pol.as<int>(),
                                                            P.d_edc.as<double2>(), P.edc_stride, 2, P.b64.as<double2>()));
    RC(P.ex_out.alloc((size_t)L.nl * 2 * sizeof(double2)));
    KL(k_scatter_sys<double><<<grid_for(L.nl * 2, B, 16), B, 0, P.st>>>(L.nl, 2, P.b64.as<double2>(), P.ex_out.as<double2>()));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(p1, P.ex_out.p, L.nl * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaMemcpyAsync(p2, P.ex_out.as<double2>() + L.nl, L.nl * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

extern "C" int sfdx_precond_apply(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                                  const double* sigma, int ns, const double* freqs, int pc, int precision,
                                  const double* y, double* x) {
    if (!sigma || !y || !x) return SFDX_ERR_ARG;
    if (pc == 'I') return SFDX_ERR_UNSUPPORTED;
    if (pc != 'S' && pc != 'J') return SFDX_ERR_ARG;
    sfdx_opts o;
    sfdx_default_opts(&o);
    o.precond = pc;
    PlanGuard g;
    RC(component_plan(&g.p, &o, nx, ny, nz, a, b, c, sigma, ns, freqs));
    Plan& P = g.p->P;
    const Level& L = P.lev[0];
    const size_t n = (size_t)L.nl * ns;
    std::vector<KState> init(ns);
    for (int q = 0; q < ns; q++) {
        memset(&init[q], 0, sizeof(KState));
        init[q].wm = P.wm[q];
        init[q].active = 1;
    }
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    DBuf dy, dx;
    RC(dy.alloc(n * 16));
    RC(dx.alloc(n * 16));
    CK(cudaMemcpyAsync(dy.p, y, n * 16, cudaMemcpyHostToDevice, P.st));
    if (precision == SFDX_FP64) {
        RC(precond_vec<double>(P, L, dx.as<double2>(), dy.as<double2>()));
    } else {
        DBuf fy, fx;
        RC(fy.alloc(n * 8));
        RC(fx.alloc(n * 8));
        KL(k_convert<double, float><<<grid_for(n, 256), 256, 0, P.st>>>(n, dy.as<double2>(), fy.as<float2>()));
        RC(precond_vec<float>(P, L, fx.as<float2>(), fy.as<float2>()));
        KL(k_convert<float, double><<<grid_for(n, 256), 256, 0, P.st>>>(n, fx.as<float2>(), dx.as<double2>()));
        CK(cudaStreamSynchronize(P.st));
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(x, dx.p, n * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

extern "C" int sfdx_vcycle_apply(int nx, int ny, int nz, int nair, const double* a, const double* b, const double* c,
                                 const double* sigma, int ns, const double* freqs, int levels, int precision,
                                 const double* y, double* x) {
    if (!sigma || !y || !x || levels < 2 || nair < 0) return SFDX_ERR_ARG;
    if (precision != SFDX_FP64 && precision != SFDX_MIXED) return SFDX_ERR_ARG;
    sfdx_opts o;
    sfdx_default_opts(&o);
    o.precond = 'G';
    o.precision = precision;
    PlanGuard g;
    RC(component_plan(&g.p, &o, nx, ny, nz, a, b, c, sigma, ns, freqs, nair, levels));
    Plan& P = g.p->P;
    const Level& L = P.lev[P.nlev - 1];
    const size_t n = (size_t)L.nl * ns;
    std::vector<KState> init(ns);
    for (int q = 0; q < ns; q++) {
        memset(&init[q], 0, sizeof(KState));
        init[q].wm = P.wm[q];
        init[q].active = 1;
    }
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    DBuf dy, dx;
    RC(dy.alloc(n * 16));
    RC(dx.alloc(n * 16));
    CK(cudaMemcpyAsync(dy.p, y, n * 16, cudaMemcpyHostToDevice, P.st));
    if (precision == SFDX_FP64) {
        RC(precond_vec<double>(P, L, dx.as<double2>(), dy.as<double2>()));
    } else {
        DBuf fy, fx;
        RC(fy.alloc(n * 8));
        RC(fx.alloc(n * 8));
        KL(k_convert<double, float><<<grid_for(n, 256), 256, 0, P.st>>>(n, dy.as<double2>(), fy.as<float2>()));
        RC(precond_vec<float>(P, L, fx.as<float2>(), fy.as<float2>()));
        KL(k_convert<float, double><<<grid_for(n, 256), 256, 0, P.st>>>(n, fx.as<float2>(), dx.as<double2>()));
        CK(cudaStreamSynchronize(P.st));
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(x, dx.p, n * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

extern "C" int sfdx_mesh_coarsen(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                                 const double* sigma, int k, int quirks, double* a1, double* b1, double* c1,
                                 double* sigma1) {
    if (!a || !b || !c || !sigma || !a1 || !b1 || !c1 || !sigma1 || k < 0) return SFDX_ERR_ARG;
    const int asf = 1 << k;
    if (nx % asf || ny % asf || nz % asf) return SFDX_ERR_MESH;
    const int cx = nx / asf, cy = ny / asf, cz = nz / asf;
    for (int i = 0; i < cx; i++) { double s = 0; for (int q = i * asf; q < (i + 1) * asf; q++) s += a[q]; a1[i] = s; }
    for (int i = 0; i < cy; i++) { double s = 0; for (int q = i * asf; q < (i + 1) * asf; q++) s += b[q]; b1[i] = s; }
    for (int i = 0; i < cz; i++) { double s = 0; for (int q = i * asf; q < (i + 1) * asf; q++) s += c[q]; c1[i] = s; }
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t n0 = (size_t)nx * ny * nz, n1 = (size_t)cx * cy * cz;
    DBuf ds0, ds1, sp;
    int rc = ds0.alloc(n0 * 6 * 8);
    if (!rc) rc = ds1.alloc(n1 * 6 * 8);
    if (!rc) rc = sp.alloc((size_t)(nx + ny + nz + cx + cy + cz) * 8);
    if (rc) { cudaStreamDestroy(st); return rc; }
    std::vector<double> hs;
    hs.insert(hs.end(), a, a + nx);
    hs.insert(hs.end(), b, b + ny);
    hs.insert(hs.end(), c, c + nz);
    hs.insert(hs.end(), a1, a1 + cx);
    hs.insert(hs.end(), b1, b1 + cy);
    hs.insert(hs.end(), c1, c1 + cz);
    cudaMemcpyAsync(sp.p, hs.data(), hs.size() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(ds0.p, sigma, n0 * 48, cudaMemcpyHostToDevice, st);
    const double* s = sp.as<double>();
    KL(k_coarsen<<<grid_for(n1, 128, 32), 128, 0, st>>>(nx, ny, nz, s, s + nx, s + nx + ny, s + nx + ny + nz,
                                                     s + nx + ny + nz + cx, s + nx + ny + nz + cx + cy, asf,
                                                     (quirks & SFDX_QUIRK_COARSEN_SHIFT) ? 1 : 0, ds0.as<double>(),
                                                     ds1.as<double>()));
    cudaMemcpyAsync(sigma1, ds1.p, n1 * 48, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaStreamDestroy(st);
    return e == cudaSuccess ? SFDX_OK : SFDX_ERR_CUDA;
}

extern "C" int sfdx_prolongate(int nx, int ny, int nz, const double* a1, const double* b1, const double* c1, int nair,
                               int ns, const double* u0, const double* u1, double* u, int quirks) {
    if (!a1 || !b1 || !c1 || !u0 || !u1 || !u || ns < 1 || ns > SFDX_MAX_SYSTEMS) return SFDX_ERR_ARG;
    if (nx % 8 || ny % 8 || nz % 8) return SFDX_ERR_MESH;
    // a 3-level hierarchy whose finest level is this mesh
    sfdx_opts o;
    sfdx_default_opts(&o);
    o.excmg = 1;
    o.level = 3;
    o.quirks = quirks;
    std::vector<double> fr((ns + 1) / 2, 1.0);
    PlanGuard g;
    RC(sfdx_plan_create(&g.p, &o, nx, ny, nz, nair, a1, b1, c1, (int)fr.size(), fr.data()));
    Plan& P = g.p->P;
    P.ns = ns;
    const Level& F = P.lev[2];
    const Level& M = P.lev[1];
    const Level& C = P.lev[0];
    DBuf d0, d1, dout;
    RC(d0.alloc((size_t)C.nl * ns * 16));
    RC(d1.alloc((size_t)M.nl * ns * 16));
    RC(dout.alloc((size_t)F.nl * ns * 16));
    RC(P.ut.alloc((size_t)M.nl * ns * 16));
    CK(cudaMemcpyAsync(d0.p, u0, (size_t)C.nl * ns * 16, cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(d1.p, u1, (size_t)M.nl * ns * 16, cudaMemcpyHostToDevice, P.st));
    int rc = prolongate(P, 2, d0.as<double2>(), d1.as<double2>(), dout.as<double2>());
    if (rc && rc != SFDX_ERR_NAN) return rc;
    CK(cudaMemcpyAsync(u, dout.p, (size_t)F.nl * ns * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return rc;
}

extern "C" int sfdx_krylov_solve(const sfdx_opts* o, int nx, int ny, int nz, const double* a, const double* b,
                                 const double* c, const double* sigma, int ns, const double* freqs, const double* rhs,
                                 double* x, double tol, int itmax, int* iters, double* relres, double* history) {
    if (!sigma || !rhs || !x || itmax < 1) return SFDX_ERR_ARG;
    PlanGuard g;
    RC(component_plan(&g.p, o, nx, ny, nz, a, b, c, sigma, ns, freqs));
    Plan& P = g.p->P;
    const Level& L = P.lev[0];
    const size_t n = (size_t)L.nl * ns;
    RC(P.x64.alloc(n * 16));
    RC(P.b64.alloc(n * 16));
    CK(cudaMemcpyAsync(P.b64.p, rhs, n * 16, cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(P.x64.p, x, n * 16, cudaMemcpyHostToDevice, P.st));
    if (history) {
        RC(P.errrec.alloc((size_t)ns * itmax * sizeof(double)));
        CK(cudaMemsetAsync(P.errrec.p, 0, (size_t)ns * itmax * sizeof(double), P.st));
        P.hist = P.errrec.as<double>();
        P.hist_stride = itmax;
    }
    std::vector<int> its, status;
    RC(solve_level(P, L, tol, itmax, false, its, status));
    if (history) {
        CK(cudaMemcpyAsync(history, P.hist, (size_t)ns * itmax * sizeof(double), cudaMemcpyDeviceToHost, P.st));
        P.hist = nullptr;
    }
    std::vector<double> rel(ns);
    RC(true_residual(P, L, P.b64.as<double2>(), P.x64.as<double2>(), rel.data(), nullptr));
    CK(cudaMemcpyAsync(x, P.x64.p, n * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    if (iters) for (int q = 0; q < ns; q++) iters[q] = its[q];
    if (relres) for (int q = 0; q < ns; q++) relres[q] = rel[q];
    return status_to_rc(status);
}

extern "C" int sfdx_div_correct(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                                const double* sigma, int ns, double* x, double tol, int* pcg_iters) {
    if (!sigma || !x || ns < 1) return SFDX_ERR_ARG;
    std::vector<double> fr(ns, 1.0);
    sfdx_opts o;
    sfdx_default_opts(&o);
    o.corr_tol = tol;
    PlanGuard g;
    RC(component_plan(&g.p, &o, nx, ny, nz, a, b, c, sigma, ns, fr.data()));
    Plan& P = g.p->P;
    const Level& L = P.lev[0];
    const size_t n = (size_t)L.nl * ns;
    std::vector<KState> init(ns);
    for (int q = 0; q < ns; q++) {
        memset(&init[q], 0, sizeof(KState));
        init[q].active = 1;
    }
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    RC(P.x64.alloc(n * 16));
    CK(cudaMemcpyAsync(P.x64.p, x, n * 16, cudaMemcpyHostToDevice, P.st));
    RC(div_correct(P, L, P.x64.as<double2>()));
    CK(cudaMemcpyAsync(x, P.x64.p, n * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    if (pcg_iters) *pcg_iters = P.dc_last_iters;
    return SFDX_OK;
}

extern "C" int sfdx_grad_correct(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                                 const double* sigma, int ns, const double* freqs, const double* rhs, double* x,
                                 double tol, int maxit, int* pcg_iters) {
    if (!sigma || !rhs || !x || !(tol > 0) || maxit < 1) return SFDX_ERR_ARG;
    PlanGuard g;
    RC(component_plan(&g.p, nullptr, nx, ny, nz, a, b, c, sigma, ns, freqs));
    Plan& P = g.p->P;
    const Level& L = P.lev[0];
    const size_t n = (size_t)L.nl * ns;
    RC(P.x64.alloc(n * 16));
    RC(P.b64.alloc(n * 16));
    CK(cudaMemcpyAsync(P.b64.p, rhs, n * 16, cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(P.x64.p, x, n * 16, cudaMemcpyHostToDevice, P.st));
    int it = 0;
    RC(grad_correct(P, L, P.b64.as<double2>(), P.x64.as<double2>(), nullptr, tol, maxit, &it));
    CK(cudaMemcpyAsync(x, P.x64.p, n * 16, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    if (pcg_iters) *pcg_iters = it;
    return SFDX_OK;
}
