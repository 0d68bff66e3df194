// sfdx_krylov.cuh -- host drivers of the Krylov solves of one level (all
// systems of the batch at once): BiCGStab (Bicg_stab_p, solvers.f90:522-719),
// GPBiCG (pgpbicg, solvers.f90:137-315), the multi-colour SSOR / Jacobi
// preconditioner (lusol/ssorfac, diagcsr) and the reliable FP64 residual
// updates of the mixed-precision solve.  Included by sfdx_krylov_f32.cu and
// sfdx_krylov_f64.cu, which instantiate it per arithmetic type so that the
// two compile in parallel.
#pragma once
#include <chrono>

#include "sfdx_blas.cuh"
#include "sfdx_mgkern.cuh"
#include "sfdx_plan.h"
#include "sfdx_vkern.cuh"

namespace sfdx {

// ------------------------------------------------------------------ preconditioner
template <class T, int VS, int O, int PP, int MODE>
static void fwd_one(Plan& P, const Level& LV, const VCfg& c, cplx<T>* w, cplx<T>* q, const cplx<T>* r, const cplx<T>* v,
                    cplx<T>* aux) {
    const uint32_t W = mcolour_count(LV.mesh, O) * c.sg.G;
    vlaunch(k_fwd_v<T, VS, O, PP, MODE>, W, c.B, 0, P.st, LV.lev<T>(), LV.mesh, c.sg, P.d_state.as<KState>(), w, q, r, v,
            aux, (T)P.o.ssor_omega);
}
template <class T, int VS, int O, int PP>
static void bwd_one(Plan& P, const Level& LV, const VCfg& c, cplx<T>* x) {
    const uint32_t W = mcolour_count(LV.mesh, O) * c.sg.G;
    vlaunch(k_bwd_v<T, VS, O, PP>, W, c.B, 0, P.st, LV.lev<T>(), LV.mesh, c.sg, P.d_state.as<KState>(), x,
            (T)P.o.ssor_omega);
}

// out = M^{-1} rhs where rhs is produced by MODE (see k_fwd_v).  Multi-colour
// symmetric Gauss-Seidel: colours 0..5 forward, 4..0 backward (the backward
// step of the last colour is the identity).
template <class T, int VS, int MODE>
static void precond_ssor(Plan& P, const Level& LV, cplx<T>* out, cplx<T>* q, const cplx<T>* r, const cplx<T>* v,
                         cplx<T>* aux = nullptr) {
    const VCfg c = vcfg(P, LV.nl, 0, VS);
    fwd_one<T, VS, OX, 0, MODE>(P, LV, c, out, q, r, v, aux);
    fwd_one<T, VS, OX, 1, MODE>(P, LV, c, out, q, r, v, aux);
    fwd_one<T, VS, OY, 0, MODE>(P, LV, c, out, q, r, v, aux);
    fwd_one<T, VS, OY, 1, MODE>(P, LV, c, out, q, r, v, aux);
    fwd_one<T, VS, OZ, 0, MODE>(P, LV, c, out, q, r, v, aux);
    fwd_one<T, VS, OZ, 1, MODE>(P, LV, c, out, q, r, v, aux);
    bwd_one<T, VS, OZ, 0>(P, LV, c, out);
    bwd_one<T, VS, OY, 1>(P, LV, c, out);
    bwd_one<T, VS, OY, 0>(P, LV, c, out);
    bwd_one<T, VS, OX, 1>(P, LV, c, out);
    bwd_one<T, VS, OX, 0>(P, LV, c, out);
}

// ------------------------------------------------------------------ edge multigrid ('G')
// V-cycle over the plan's mesh levels (kernels and transfer operators in
// sfdx_mgkern.cuh).  Per level: pre-smoothing (multi-colour SSOR from zero,
// nodal step), residual, restriction, the coarser level's V-cycle,
// prolongation, post-smoothing (residual, SSOR, nodal step); on the coarsest
// level emg_coarse_sweeps() smoothing steps.  A fixed linear operator, so the
// Krylov methods see an ordinary (if strong) preconditioner.
// smoothing steps on the coarsest level and the damping of the nodal Jacobi
// step (SFDX_MG_COARSE, SFDX_MG_OMEGA override them)
static int emg_coarse_sweeps() {
    static const int v = [] {
        const char* e = getenv("SFDX_MG_COARSE");
        const int n = e ? atoi(e) : 0;
        return n > 0 ? n : 4;
    }();
    return v;
}
static double emg_nodal_omega() {
    static const double v = [] {
        const char* e = getenv("SFDX_MG_OMEGA");
        const double w = e ? atof(e) : 0.0;
        return w > 0 ? w : 0.7;
    }();
    return v;
}

// Nodal steps of complex64 V-cycles skip the nodes inside air (all eight
// cells below this conductivity, S/m; SFDX_MG_AIR overrides, 0 keeps them):
// there the step's gradient corrections scale like 1/(w mu sigma) and, stored
// in complex64 beside the field, swamp it; as near-null modes they barely
// change the residual, and the FP64 gradient correction after each restart
// cycle removes them where the impedances see them.
static double emg_air_cut() {
    static const double v = [] {
        const char* e = getenv("SFDX_MG_AIR");
        return e ? atof(e) : 1e-6;
    }();
    return v;
}

static int level_index(const Plan& P, const Level& LV) {
    for (int l = 0; l < P.nlev; l++)
        if (&P.lev[l] == &LV) return l;
    return -1;
}

// Work vectors of the V-cycle and the nodal operators of levels 0..l (sized
// for the plan's current batch); must run before any graph capture.
template <class T> static int emg_prepare(Plan& P, const Level& LV) {
    if (P.o.precond != 'G') return SFDX_OK;
    const int l = level_index(P, LV);
    if (l < 0) return SFDX_ERR_ARG;
    if (P.pf32) {  // complex64 copies of the preconditioner's input and output
        for (DBuf* b : {&P.emg_q32, &P.emg_o32}) {
            void* before = b->p;
            RC(b->alloc((size_t)LV.nl * P.ns * sizeof(float2)));
            if (b->p != before) P.emg_epoch++;
        }
    }
    if (P.split && std::is_same<T, float>::value) {
        for (int m = 0; m <= l; m++) {
            const Level& L = P.lev[m];
            const size_t ev = (size_t)L.nl * P.ns * sizeof(cplx<T>);
            const size_t nv = (size_t)(L.nx + 1) * (L.ny + 1) * (L.nz + 1) * P.ns * sizeof(cplx<T>);
            DBuf* bufs[3] = {&L.emg_g, &L.emg_t, &L.emg_psi};
            const size_t need[3] = {ev, ev, m < l ? nv : 0};
            for (int q = 0; q < 3; q++) {
                if (!need[q]) continue;
                void* before = bufs[q]->p;
                RC(bufs[q]->alloc(need[q]));
                if (bufs[q]->p != before) P.emg_epoch++;
            }
        }
    }
    for (int m = 0; m <= l; m++) {
        const Level& L = P.lev[m];
        RC(nodal_setup(P, L));
        const size_t ev = (size_t)L.nl * P.ns * sizeof(cplx<T>);
        const size_t nv = (size_t)(L.nx + 1) * (L.ny + 1) * (L.nz + 1) * P.ns * sizeof(cplx<T>);
        DBuf* bufs[5] = {&L.emg_r, &L.emg_z, &L.emg_phi, &L.emg_b, &L.emg_x};
        const size_t need[5] = {ev, ev, nv, m < l ? ev : 0, m < l ? ev : 0};
        for (int q = 0; q < 5; q++) {
            if (!need[q]) continue;
            void* before = bufs[q]->p;
            RC(bufs[q]->alloc(need[q]));
            if (bufs[q]->p != before) P.emg_epoch++;  // captured graphs hold the old address
        }
    }
    return SFDX_OK;
}

// nodal step: q = b + i wm Ms x (the gradient-space part of b - A x);
// phi = w D^-1 G^T V q; x += G phi
template <class T, int VS>
static void emg_nodal(Plan& P, const Level& L, const VCfg& c, const cplx<T>* b, cplx<T>* x) {
    const KState* dst = P.d_state.as<KState>();
    cplx<T>* r = L.emg_r.as<cplx<T>>();
    cplx<T>* phi = L.emg_phi.as<cplx<T>>();
    const uint32_t np = (uint32_t)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    vlaunch(k_mg_mres_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, b, (const cplx<T>*)x, r);
    vlaunch(k_mg_node_v<T, VS>, (int64_t)np * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, np, dst,
            (const cplx<T>*)r, L.mg[0].dinv.as<float>(), phi, (T)emg_nodal_omega(),
            (T)(sizeof(T) == 4 ? emg_air_cut() : 0.0));
    vlaunch(k_mg_gadd_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, (const cplx<T>*)phi, x);
}

// smoothing step from the current x: r = b - A x; z = S^-1 r; x += z; nodal step
template <class T, int VS>
static void emg_smooth(Plan& P, const Level& L, const VCfg& c, const cplx<T>* b, cplx<T>* x) {
    const KState* dst = P.d_state.as<KState>();
    cplx<T>* r = L.emg_r.as<cplx<T>>();
    cplx<T>* z = L.emg_z.as<cplx<T>>();
    vlaunch(k_mg_res_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, b, (const cplx<T>*)x, r);
    precond_ssor<T, VS, RHS_VEC>(P, L, z, r, nullptr, nullptr);
    vlaunch(k_mg_add_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.mesh, c.sg, dst, x, (const cplx<T>*)z);
    emg_nodal<T, VS>(P, L, c, b, x);
}

// x = V-cycle(b) on level l.  `pre`: x already holds S^-1 b (the caller fused
// its Krylov vector update into that first SSOR sweep).
template <class T, int VS>
static void emg_vcycle(Plan& P, int l, const cplx<T>* b, cplx<T>* x, bool pre) {
    const Level& L = P.lev[l];
    const VCfg c = vcfg(P, L.nl, 0, VS);
    const KState* dst = P.d_state.as<KState>();
    if (!pre) precond_ssor<T, VS, RHS_VEC>(P, L, x, const_cast<cplx<T>*>(b), nullptr, nullptr);
    emg_nodal<T, VS>(P, L, c, b, x);
    if (l == 0) {
        for (int s = 1; s < emg_coarse_sweeps(); s++) emg_smooth<T, VS>(P, L, c, b, x);
        return;
    }
    const Level& C = P.lev[l - 1];
    const VCfg cc = vcfg(P, C.nl, 0, VS);
    cplx<T>* r = L.emg_r.as<cplx<T>>();
    cplx<T>* bc = C.emg_b.as<cplx<T>>();
    cplx<T>* xc = C.emg_x.as<cplx<T>>();
    vlaunch(k_mg_res_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, b, (const cplx<T>*)x, r);
    vlaunch(k_mg_restrict_v<T, VS>, C.nl * cc.sg.G, cc.B, 0, P.st, L.lev<T>(), L.mesh, C.lev<T>(), C.mesh, cc.sg, dst,
            (const cplx<T>*)r, bc);
    emg_vcycle<T, VS>(P, l - 1, bc, xc, false);
    vlaunch(k_mg_prolong_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, C.mesh, c.sg, dst,
            (const cplx<T>*)xc, x);
    emg_smooth<T, VS>(P, L, c, b, x);
}

// ---- split V-cycle (P.split): x and the nodal potential psi of each level
// q = b + i wm Ms (x + G psi) ; phi = w D^-1 G^T V q ; psi += phi
template <class T, int VS>
static void emg_nodal_split(Plan& P, const Level& L, const VCfg& c, const cplx<T>* b, const cplx<T>* x, cplx<T>* psi) {
    const KState* dst = P.d_state.as<KState>();
    cplx<T>* xs = L.emg_g.as<cplx<T>>();
    cplx<T>* q = L.emg_r.as<cplx<T>>();
    cplx<T>* phi = L.emg_phi.as<cplx<T>>();
    const uint32_t np = (uint32_t)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    // the mass product has no curl-curl cancellation: x + G psi in one vector is fine here
    vlaunch(k_mg_xpg_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, x, (const cplx<T>*)psi, xs);
    vlaunch(k_mg_mres_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, b, (const cplx<T>*)xs, q);
    vlaunch(k_mg_node_v<T, VS>, (int64_t)np * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, np, dst,
            (const cplx<T>*)q, L.mg[0].dinv.as<float>(), phi, (T)emg_nodal_omega(), (T)0);
    vlaunch(k_mg_nadd_v<T, VS>, (int64_t)np * c.sg.G, c.B, 0, P.st, c.sg, dst, np, psi, (const cplx<T>*)phi);
}
// r = b - A x + i wm Ms G psi  (= b - A (x + G psi)) into L.emg_r
template <class T, int VS>
static void emg_res_split(Plan& P, const Level& L, const VCfg& c, const cplx<T>* b, const cplx<T>* x,
                          const cplx<T>* psi) {
    const KState* dst = P.d_state.as<KState>();
    cplx<T>* t = L.emg_t.as<cplx<T>>();
    cplx<T>* g = L.emg_g.as<cplx<T>>();
    vlaunch(k_mg_res_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, b, x, t);
    vlaunch(k_mg_xpg_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, (const cplx<T>*)nullptr,
            psi, g);
    vlaunch(k_mg_mres_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, c.sg, dst, (const cplx<T>*)t,
            (const cplx<T>*)g, L.emg_r.as<cplx<T>>());
}
// smoothing step: r = b - A(x + G psi); x += S^-1 r; nodal step
template <class T, int VS>
static void emg_smooth_split(Plan& P, const Level& L, const VCfg& c, const cplx<T>* b, cplx<T>* x, cplx<T>* psi) {
    const KState* dst = P.d_state.as<KState>();
    cplx<T>* z = L.emg_z.as<cplx<T>>();
    emg_res_split<T, VS>(P, L, c, b, x, psi);
    precond_ssor<T, VS, RHS_VEC>(P, L, z, L.emg_r.as<cplx<T>>(), nullptr, nullptr);
    vlaunch(k_mg_add_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.mesh, c.sg, dst, x, (const cplx<T>*)z);
    emg_nodal_split<T, VS>(P, L, c, b, x, psi);
}
// (x, psi) = V-cycle(b) on level l, psi from zero; `pre`: x already holds S^-1 b
template <class T, int VS>
static void emg_vcycle_split(Plan& P, int l, const cplx<T>* b, cplx<T>* x, cplx<T>* psi, bool pre) {
    const Level& L = P.lev[l];
    const VCfg c = vcfg(P, L.nl, 0, VS);
    const KState* dst = P.d_state.as<KState>();
    const uint32_t np = (uint32_t)(L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    vlaunch(k_psi_zero_v<T, VS, false>, (int64_t)np * c.sg.G, c.B, 0, P.st, c.sg, dst, np, psi);
    if (!pre) precond_ssor<T, VS, RHS_VEC>(P, L, x, const_cast<cplx<T>*>(b), nullptr, nullptr);
    emg_nodal_split<T, VS>(P, L, c, b, x, psi);
    if (l == 0) {
        for (int s = 1; s < emg_coarse_sweeps(); s++) emg_smooth_split<T, VS>(P, L, c, b, x, psi);
        return;
    }
    const Level& C = P.lev[l - 1];
    const VCfg cc = vcfg(P, C.nl, 0, VS);
    cplx<T>* bc = C.emg_b.as<cplx<T>>();
    cplx<T>* xc = C.emg_x.as<cplx<T>>();
    cplx<T>* pc = C.emg_psi.as<cplx<T>>();
    emg_res_split<T, VS>(P, L, c, b, x, psi);
    vlaunch(k_mg_restrict_v<T, VS>, C.nl * cc.sg.G, cc.B, 0, P.st, L.lev<T>(), L.mesh, C.lev<T>(), C.mesh, cc.sg, dst,
            (const cplx<T>*)L.emg_r.as<cplx<T>>(), bc);
    emg_vcycle_split<T, VS>(P, l - 1, bc, xc, pc, false);
    vlaunch(k_mg_prolong_v<T, VS>, L.nl * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, C.mesh, c.sg, dst,
            (const cplx<T>*)xc, x);
    vlaunch(k_mg_nprolong_v<T, VS>, (int64_t)np * c.sg.G, c.B, 0, P.st, L.lev<T>(), L.mesh, C.mesh, c.sg, dst, np,
            (const cplx<T>*)pc, psi);
    emg_smooth_split<T, VS>(P, L, c, b, x, psi);
}

// Complex64 V-cycle for a complex128 Krylov solve (P.pf32): MODE's vector
// update in FP64 with the result rounded to complex64, the V-cycle with the
// complex64 grouping of the plan, the output widened to FP64.  The Krylov
// vectors and the operator stay FP64, so the V-cycle's large discrete-gradient
// components (cheap in the operator's norm, costly under a rounded operator)
// never meet complex64 operator arithmetic.
template <int VS, int MODE>
static void emg_precond32(Plan& P, const Level& LV, double2* out, double2* q, const double2* r, const double2* v,
                          double2* aux) {
    const int l = level_index(P, LV);
    const VCfg c = vcfg(P, LV.nl, 0, VS);
    const KState* dst = P.d_state.as<KState>();
    float2* q32 = P.emg_q32.as<float2>();
    float2* o32 = P.emg_o32.as<float2>();
    vlaunch(k_mg_to32_v<VS, MODE>, LV.nl * c.sg.G, c.B, 0, P.st, LV.mesh, c.sg, dst, q, r, v, aux, q32);
    switch (plan_vs<float>(P)) {
        case 4: emg_vcycle<float, 4>(P, l, q32, o32, false); break;
        case 2: emg_vcycle<float, 2>(P, l, q32, o32, false); break;
        default: emg_vcycle<float, 1>(P, l, q32, o32, false); break;
    }
    vlaunch(k_mg_to64_v<VS>, LV.nl * c.sg.G, c.B, 0, P.st, LV.mesh, c.sg, dst, (const float2*)o32, out);
}

// out = M^{-1} rhs (rhs produced by MODE, see k_fwd_v): Jacobi, multi-colour
// SSOR, or the edge multigrid V-cycle whose first SSOR sweep carries MODE.
template <class T, int VS, int MODE>
static void precond(Plan& P, const Level& LV, cplx<T>* out, cplx<T>* q, const cplx<T>* r, const cplx<T>* v,
                    cplx<T>* aux = nullptr) {
    if constexpr (std::is_same<T, double>::value) {
        if (P.o.precond == 'G' && P.pf32) {
            emg_precond32<VS, MODE>(P, LV, out, q, r, v, aux);
            return;
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        if (P.o.precond == 'G' && P.split) {
            precond_ssor<T, VS, MODE>(P, LV, out, q, r, v, aux);
            emg_vcycle_split<T, VS>(P, level_index(P, LV), q, out, static_cast<cplx<T>*>(P.psi_out), true);
            return;
        }
    }
    if (P.o.precond == 'J') {
        const int B = block_for(P.ns);
        KL(k_jacobi<T, MODE><<<grid_for(LV.nl * P.ns, B, 16), B, 0, P.st>>>(LV.lev<T>(), P.d_state.as<KState>(), P.ns, out,
                                                                            q, r, v));
        return;
    }
    precond_ssor<T, VS, MODE>(P, LV, out, q, r, v, aux);
    if (P.o.precond == 'G') emg_vcycle<T, VS>(P, level_index(P, LV), q, out, true);
}

static void init_states(Plan& P, const double* tols_host, double tol, int itmax, const int* mask_host,
                        std::vector<KState>& init) {
    init.resize(P.ns);
    for (int q = 0; q < P.ns; q++) {
        KState S;
        memset(&S, 0, sizeof(S));
        S.wm = P.wm[q];
        S.tol = tols_host ? tols_host[q] : tol;
        S.itmax = itmax;
        S.active = mask_host ? mask_host[q] : 1;
        S.status = S.active ? ST_RUN : ST_SKIP;
        init[q] = S;
    }
}

// partial sums of the reducing kernels of one level (nq per system)
static int reserve_partials(Plan& P, const VCfg&, int nq) {
    return P.d_part.alloc(std::max(P.d_part.bytes, (size_t)max_resident_blocks() * nq * P.ns * sizeof(double2)));
}

// Graph key of one check interval (8 iterations): everything the captured
// launches bake in besides the caller's vectors in `extra`.
template <class T>
static std::vector<uintptr_t> interval_key(const Plan& P, const Level& LV, int solver, int VS,
                                           std::initializer_list<uintptr_t> extra) {
    std::vector<uintptr_t> k = {(uintptr_t)solver, sizeof(T), (uintptr_t)VS, (uintptr_t)&LV, (uintptr_t)P.ns,
                                (uintptr_t)LV.aniso, (uintptr_t)P.o.precond, (uintptr_t)P.d_state.p,
                                (uintptr_t)P.d_part.p, (uintptr_t)P.d_counter.p, (uintptr_t)P.hist,
                                (uintptr_t)P.hist_stride, (uintptr_t)LV.sig32.p, (uintptr_t)LV.sig64.p,
                                (uintptr_t)LV.tab32.p, (uintptr_t)LV.tab64.p, (uintptr_t)LV.rc_ok,
                                (uintptr_t)LV.rc32.p, (uintptr_t)LV.rc64.p,
                                (uintptr_t)(P.o.ssor_omega * 1e6), (uintptr_t)P.emg_epoch, (uintptr_t)P.pf32,
                                (uintptr_t)P.split, (uintptr_t)P.psi_y.p, (uintptr_t)P.psi_z.p, (uintptr_t)P.psi_x.p,
                                (uintptr_t)P.g_y.p, (uintptr_t)P.g_z.p};
    for (const DBuf& b : P.kv) k.push_back((uintptr_t)b.p);
    k.insert(k.end(), extra);
    return k;
}
// whether iterations it .. it+7 run as one captured graph: graphs enabled,
// a whole check interval, not the first one (it runs eagerly and fills the
// launch-shape cache), and no host work inside (the reference's divergence
// correction runs on the host every corr_intv iterations)
static bool graph_interval(const Plan& P, int it, int itmax, bool host_work) {
    return P.o.use_graphs && !host_work && it > 8 && (it - 1) % 8 == 0 && it + 7 <= itmax;
}

// x64 += G psi_x, psi_x = 0 (split Krylov vectors: the nodal part of the
// complex64 partial solution)
template <class T, int VS, bool ALL>
static void split_flush(Plan& P, const Level& LV, const VCfg& c, double2* x64) {
    if constexpr (std::is_same<T, float>::value) {
        const KState* dst = P.d_state.as<KState>();
        const uint32_t np = (uint32_t)(LV.nx + 1) * (LV.ny + 1) * (LV.nz + 1);
        cplx<T>* px = P.psi_x.as<cplx<T>>();
        vlaunch(k_flush_psi_v<T, VS, ALL>, LV.nl * c.sg.G, c.B, 0, P.st, LV.lev<double>(), LV.mesh, c.sg, dst, x64,
                (const cplx<T>*)px);
        vlaunch(k_psi_zero_v<T, VS, ALL>, (int64_t)np * c.sg.G, c.B, 0, P.st, c.sg, dst, np, px);
    }
}

// FP64 residual replacement for the systems still running or whose complex64
// recurrence claims convergence; returns the number of systems left active.
template <class T, int VS>
static int reliable_update(Plan& P, const Level& LV, const Reliable& rel, cplx<T>* x32, cplx<T>* r, const cplx<T>* rhat,
                           int solver, int& active) {
    constexpr int VSD = VS > 2 ? 2 : VS;  // systems per thread of the FP64 residual
    const int ns = P.ns;
    const VCfg c = vcfg(P, LV.nl, 2, VS);
    const VCfg cd = vcfg(P, LV.nl, 2, VSD);
    RC(reserve_partials(P, cd, 2));
    KState* dst = P.d_state.as<KState>();
    KL(k_reactivate<<<(ns + 127) / 128, 128, 0, P.st>>>(dst, ns));
    vlaunch(k_flush_v<T, VS, false>, LV.nl * c.sg.G, c.B, 0, P.st, LV.mesh, c.sg, dst, rel.x64, x32, rel.xb);
    if (P.split) split_flush<T, VS, false>(P, LV, c, rel.x64);
    vlaunch(k_reliable_v<T, VSD>, LV.nl * cd.sg.G, cd.B, cd.smem, P.st, LV.lev<double>(), LV.mesh, cd.sg, dst, rel.b64, rel.x64, r, rhat, solver, redbuf(P));
    CK(cudaGetLastError());
    RC(sync_state(P));
    active = 0;
    int rejected = 0;
    for (int q = 0; q < ns; q++) {
        active += P.hst[q].active;
        rejected += P.hst[q].status == ST_BREAK && P.hst[q].pad[0] == 1;
    }
    if (rejected) {
        const int B = block_for(ns);
        KL(k_restore<<<grid_for(LV.nl * ns, B, 16), B, 0, P.st>>>(LV.nl, dst, ns, rel.x64, rel.xb));
        CK(cudaGetLastError());
    }
    return SFDX_OK;
}

// Under the complex64 V-cycle (P.pf32) a system whose FP64 residual has grown
// 1e4-fold above the smallest it reached, or has not reached a new smallest
// residual for 160 iterations, met the V-cycle's rounding (gradient
// corrections of very low induction numbers, 1e-3 Hz in resistive ground;
// the multigrid iteration otherwise converges in tens of iterations): stop it
// as a breakdown, so that solve_level restarts it from its starting iterate
// with the FP64 V-cycle.  `emin` holds each system's smallest residual and the
// iteration that reached it.
struct ResMin {
    std::vector<double> e;
    std::vector<int> it;
};
static int pf32_divergence(Plan& P, ResMin& m) {
    if (!P.pf32) return SFDX_OK;
    if ((int)m.e.size() != P.ns) {
        m.e.assign(P.ns, INFINITY);
        m.it.assign(P.ns, 0);
    }
    KState* dst = P.d_state.as<KState>();
    bool sent = false;
    for (int q = 0; q < P.ns; q++) {
        KState& S = P.hst[q];
        if (!S.active) continue;
        if (!(S.err <= 1e4 * m.e[q]) || S.it - m.it[q] > 160) {  // also NaN
            S.active = 0;
            S.status = ST_BREAK;
            CK(cudaMemcpyAsync(dst + q, &S, sizeof(KState), cudaMemcpyHostToDevice, P.st));
            sent = true;
        } else if (S.err < m.e[q]) {
            m.e[q] = S.err;
            m.it[q] = S.it;
        }
    }
    if (sent) CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

// Bicg_stab_p (solvers.f90:522-719) for the ns systems of level LV: A x = b.
// Plain: x holds the initial guess (precision T).  With `rel` (mixed
// precision) b/x are the complex64 work vectors and the FP64 b64/x64 of
// `rel` define the system.
template <class T, int VS>
static int bicgstab_v(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol,
                      int itmax, const int* mask_host, const Reliable* rel) {
    const Lev<T> L = LV.lev<T>();
    const Mesh& M = LV.mesh;
    const int ns = P.ns;
    const size_t vb = (size_t)LV.nl * ns * sizeof(cplx<T>);
    for (int q = 0; q < 8; q++) RC(P.kv[q].alloc(vb));
    cplx<T>* r = P.kv[0].as<cplx<T>>();
    cplx<T>* rhat = P.kv[1].as<cplx<T>>();
    cplx<T>* p = P.kv[2].as<cplx<T>>();
    cplx<T>* v = P.kv[3].as<cplx<T>>();
    cplx<T>* y = P.kv[4].as<cplx<T>>();
    cplx<T>* s = P.kv[5].as<cplx<T>>();
    cplx<T>* z = P.kv[6].as<cplx<T>>();
    cplx<T>* t = P.kv[7].as<cplx<T>>();
    for (cplx<T>* q : {p, v, y, z}) CK(cudaMemsetAsync(q, 0, vb, P.st));
    std::vector<KState> init;
    init_states(P, tols_host, tol, itmax, mask_host, init);
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    constexpr int VSD = VS > 2 ? 2 : VS;  // systems per thread of FP64 residuals
    const VCfg c = vcfg(P, LV.nl, 2, VS);
    const VCfg cd = vcfg(P, LV.nl, 2, VSD);
    RC(reserve_partials(P, c, 2));
    RC(reserve_partials(P, cd, 2));
    KState* dst = P.d_state.as<KState>();
    if (rel) {
        CK(cudaMemsetAsync(x, 0, vb, P.st));
        vlaunch(k_residual_v<T, double, VSD, 0>, LV.nl * cd.sg.G, cd.B, cd.smem, P.st, LV.lev<double>(), M, cd.sg, dst, rel->b64, rel->x64, r, rhat, redbuf(P), P.hist, P.hist_stride);
    } else {
        vlaunch(k_residual_v<T, T, VS, 0>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, b, x, r, rhat, redbuf(P), P.hist, P.hist_stride);
    }
    CK(cudaGetLastError());
    const int check_every = 8;
    int last_rel = 0;
    ResMin emin;  // smallest residual per system (pf32_divergence)
    const bool div1 = !rel && std::is_same<T, double>::value && P.o.div_cor == 1;
    // split Krylov vectors (P.split, complex64 iteration under the split V-cycle):
    // y + G psi_y, z + G psi_z, partial solution x + G psi_x
    const bool split = rel && P.split && std::is_same<T, float>::value;
    const uint32_t npn = (uint32_t)(LV.nx + 1) * (LV.ny + 1) * (LV.nz + 1);
    cplx<T> *py = nullptr, *pz = nullptr, *px = nullptr, *gy = nullptr, *gz = nullptr;
    if (split) {
        const size_t nb = (size_t)npn * ns * sizeof(cplx<T>);
        for (DBuf* d : {&P.psi_y, &P.psi_z, &P.psi_x}) RC(d->alloc(nb));
        for (DBuf* d : {&P.g_y, &P.g_z}) RC(d->alloc(vb));
        py = P.psi_y.as<cplx<T>>();
        pz = P.psi_z.as<cplx<T>>();
        px = P.psi_x.as<cplx<T>>();
        gy = P.g_y.as<cplx<T>>();
        gz = P.g_z.as<cplx<T>>();
        CK(cudaMemsetAsync(px, 0, nb, P.st));
    }
    auto body = [&]() {
        if (split) {
            P.psi_out = py;
            precond<T, VS, RHS_PUPD>(P, LV, y, p, r, v);
            vlaunch(k_mg_xpg_v<T, VS>, LV.nl * c.sg.G, c.B, 0, P.st, L, M, c.sg, dst, (const cplx<T>*)nullptr,
                    (const cplx<T>*)py, gy);
            vlaunch(k_bicg_v_split_v<T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, y, gy, v, rhat,
                    redbuf(P));
            P.psi_out = pz;
            precond<T, VS, RHS_SUPD>(P, LV, z, s, r, v);
            vlaunch(k_mg_xpg_v<T, VS>, LV.nl * c.sg.G, c.B, 0, P.st, L, M, c.sg, dst, (const cplx<T>*)nullptr,
                    (const cplx<T>*)pz, gz);
            vlaunch(k_bicg_t_split_v<T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, z, gz, t, s,
                    redbuf(P));
            vlaunch(k_split_psi_upd_v<T, VS>, (int64_t)npn * c.sg.G, c.B, 0, P.st, c.sg, dst, npn, px,
                    (const cplx<T>*)py, (const cplx<T>*)pz);
            vlaunch(k_bicg_upd_v<T, T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, M, c.sg, dst, x, y, z, s, t, r, rhat, redbuf(P), P.hist, P.hist_stride);
            return;
        }
        precond<T, VS, RHS_PUPD>(P, LV, y, p, r, v);
        vlaunch(k_bicg_v_v<T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, y, v, rhat, redbuf(P));
        precond<T, VS, RHS_SUPD>(P, LV, z, s, r, v);
        vlaunch(k_bicg_t_v<T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, z, t, s, redbuf(P));
        vlaunch(k_bicg_upd_v<T, T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, M, c.sg, dst, x, y, z, s, t, r, rhat, redbuf(P), P.hist, P.hist_stride);
    };
    for (int it = 1; it <= itmax; it++) {
        // top of iteration `it` (solvers.f90:630-640): divergence correction and
        // residual restart every corr_intv iterations (FP64 solves only)
        if (div1 && it % P.o.corr_intv == 0) {
            RC(div_correct(P, LV, reinterpret_cast<double2*>(x)));
            vlaunch(k_residual_v<T, T, VS, 1>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, b, x, r, rhat, redbuf(P), nullptr, 0);
        }
        if (graph_interval(P, it, itmax, div1)) {
            RC(graph_run(P, interval_key<T>(P, LV, 1, VS, {(uintptr_t)x, (uintptr_t)b}), [&] {
                for (int q = 0; q < check_every; q++) body();
            }));
            it += check_every - 1;
        } else {
            body();
        }
        if (it % check_every == 0 || it == itmax) {
            CK(cudaGetLastError());
            RC(sync_state(P));
            RC(pf32_divergence(P, emin));
            int act = 0, cand = 0;
            for (int q = 0; q < ns; q++) {
                act += P.hst[q].active;
                cand += P.hst[q].status == ST_CONV;
            }
            if (rel && (cand || (act && (it - last_rel >= rel->every || it == itmax)))) {
                RC((reliable_update<T, VS>(P, LV, *rel, x, r, rhat, 1, act)));
                last_rel = it;
            }
            if (!act) break;
        }
    }
    if (rel) {
        vlaunch(k_flush_v<T, VS, true>, LV.nl * c.sg.G, c.B, 0, P.st, M, c.sg, dst, rel->x64, x, nullptr);
        if (split) split_flush<T, VS, true>(P, LV, c, rel->x64);
    }
    RC(sync_state(P));
    return SFDX_OK;
}

// pgpbicg (solvers.f90:137-315) for the ns systems of level LV (same calling
// convention as bicgstab).
template <class T, int VS>
static int gpbicg_v(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol,
                    int itmax, const int* mask_host, const Reliable* rel) {
    const Lev<T> L = LV.lev<T>();
    const Mesh& M = LV.mesh;
    const int ns = P.ns;
    const size_t vb = (size_t)LV.nl * ns * sizeof(cplx<T>);
    for (int q = 0; q < 14; q++) RC(P.kv[q].alloc(vb));
    cplx<T>* V[14];
    for (int q = 0; q < 14; q++) V[q] = P.kv[q].as<cplx<T>>();
    cplx<T> *r = V[0], *r0 = V[1], *rp = V[2], *y = V[3], *p = V[4], *u = V[5], *w = V[6], *t = V[7];
    cplx<T>* tp[2] = {V[8], V[9]};
    cplx<T> *ap = V[10], *at = V[11], *z = V[12], *tmp = V[13];
    for (cplx<T>* q : {u, w, t, tp[0], tp[1], z}) CK(cudaMemsetAsync(q, 0, vb, P.st));
    std::vector<KState> init;
    init_states(P, tols_host, tol, itmax, mask_host, init);
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    constexpr int VSD = VS > 2 ? 2 : VS;  // systems per thread of FP64 residuals
    const VCfg c = vcfg(P, LV.nl, 4, VS);
    const VCfg cd = vcfg(P, LV.nl, 2, VSD);
    RC(reserve_partials(P, c, 4));
    RC(reserve_partials(P, cd, 2));
    const int Ge = grid_for(LV.nl * c.sg.G, c.B, 16);
    KState* dst = P.d_state.as<KState>();
    if (rel) {
        CK(cudaMemsetAsync(x, 0, vb, P.st));
        vlaunch(k_residual_v<T, double, VSD, 3>, LV.nl * cd.sg.G, cd.B, cd.smem, P.st, LV.lev<double>(), M, cd.sg, dst, rel->b64, rel->x64, r, r0, redbuf(P), nullptr, 0);
    } else {
        vlaunch(k_residual_v<T, T, VS, 3>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, b, x, r, r0, redbuf(P), nullptr, 0);
    }
    precond<T, VS, RHS_VEC>(P, LV, rp, r, nullptr, nullptr);
    CK(cudaMemcpyAsync(p, rp, vb, cudaMemcpyDeviceToDevice, P.st));
    int cur = 0, last_rel = 0;
    ResMin emin;  // smallest residual per system (pf32_divergence)
    const bool div1 = !rel && std::is_same<T, double>::value && P.o.div_cor == 1;
    // one iteration up to the convergence check, with t' in tp[cc]
    auto body = [&](int cc) {
        vlaunch(k_gp_ap_v<T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, p, ap, r0, r, redbuf(P));
        vlaunch(k_gp_yt_v<T, VS>, LV.nl * c.sg.G, c.B, 0, P.st, M, c.sg, dst, y, t, r, w, ap);
        precond<T, VS, RHS_VEC>(P, LV, tmp, ap, nullptr, nullptr);
        vlaunch(k_gp_tp_v<T, VS>, LV.nl * c.sg.G, c.B, 0, P.st, M, c.sg, dst, tp[cc], rp, tmp);
        vlaunch(k_gp_at_v<T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, tp[cc], at, t, y, redbuf(P));
        vlaunch(k_gp_upd_v<T, T, VS>, LV.nl * c.sg.G, c.B, c.smem, P.st, M, c.sg, dst, u, z, x, r, tmp, tp[cc ^ 1], rp, p, t, y, at, r0, redbuf(P), P.hist, P.hist_stride);
    };
    // the rest of the iteration after the check
    auto tail = [&]() {
        precond<T, VS, RHS_VEC>(P, LV, rp, r, nullptr, nullptr);
        vlaunch(k_gp_pw_v<T, VS>, LV.nl * c.sg.G, c.B, 0, P.st, M, c.sg, dst, w, p, at, ap, rp, u);
    };
    for (int it = 1; it <= itmax; it++) {
        if (div1 && it % P.o.corr_intv == 0) {
            // solvers.f90:223-235: correct x, restart r and r0 (rp is kept)
            RC(div_correct(P, LV, reinterpret_cast<double2*>(x)));
            vlaunch(k_residual_v<T, T, VS, 4>, LV.nl * c.sg.G, c.B, c.smem, P.st, L, M, c.sg, dst, b, x, r, r0, redbuf(P), nullptr, 0);
        }
        if (graph_interval(P, it, itmax, div1)) {
            const int c0 = cur;
            RC(graph_run(P, interval_key<T>(P, LV, 3, VS, {(uintptr_t)x, (uintptr_t)b, (uintptr_t)c0}), [&] {
                int cc = c0;
                for (int q = 0; q < 8; q++) {
                    if (q) {
                        tail();
                        cc ^= 1;
                    }
                    body(cc);
                }
            }));
            it += 7;
            cur = c0 ^ 1;
        } else {
            body(cur);
        }
        bool stop = false;
        if (it % 8 == 0 || it == itmax) {
            CK(cudaGetLastError());
            RC(sync_state(P));
            RC(pf32_divergence(P, emin));
            int act = 0, cand = 0;
            for (int q = 0; q < ns; q++) {
                act += P.hst[q].active;
                cand += P.hst[q].status == ST_CONV;
            }
            if (rel && (cand || (act && (it - last_rel >= rel->every || it == itmax)))) {
                RC((reliable_update<T, VS>(P, LV, *rel, x, r, r0, 3, act)));
                last_rel = it;
            }
            stop = !act;
        }
        if (stop) break;
        tail();
        cur ^= 1;
    }
    if (rel) vlaunch(k_flush_v<T, VS, true>, LV.nl * c.sg.G, c.B, 0, P.st, M, c.sg, dst, rel->x64, x, nullptr);
    RC(sync_state(P));
    return SFDX_OK;
}

// Preconditioned COCR (SFDX_SOLVER_COCR; no working counterpart: pcocr,
// solvers.f90:58-135, divides by an unset m_j and is unreachable) for the ns
// systems of level LV, same calling convention as bicgstab.  The bilinear
// form and the kernels are in sfdx_vkern.cuh.  With `rel` the recurrence is
// restarted from the FP64 residual after every reliable update.
template <class T, int VS>
static int cocr_v(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
                  const int* mask_host, const Reliable* rel) {
    constexpr int VSD = VS > 2 ? 2 : VS;
    const Lev<T> L = LV.lev<T>();
    const Mesh& M = LV.mesh;
    const int ns = P.ns;
    const size_t vb = (size_t)LV.nl * ns * sizeof(cplx<T>);
    for (int k = 0; k < 6; k++) RC(P.kv[k].alloc(vb));
    cplx<T> *r = P.kv[0].as<cplx<T>>(), *z = P.kv[1].as<cplx<T>>(), *u = P.kv[2].as<cplx<T>>();
    cplx<T> *w = P.kv[3].as<cplx<T>>(), *p = P.kv[4].as<cplx<T>>(), *q = P.kv[5].as<cplx<T>>();
    std::vector<KState> init;
    init_states(P, tols_host, tol, itmax, mask_host, init);
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    const VCfg c = vcfg(P, LV.nl, 1, VS);
    const VCfg cd = vcfg(P, LV.nl, 2, VSD);
    RC(reserve_partials(P, c, 2));
    KState* dst = P.d_state.as<KState>();
    const int64_t W = LV.nl * c.sg.G, WD = LV.nl * cd.sg.G;
    if (rel) {
        vlaunch(k_fix_bnd<double, VSD>, WD, cd.B, 0, P.st, M, cd.sg, dst, rel->b64, rel->x64);
        CK(cudaMemsetAsync(x, 0, vb, P.st));
        vlaunch(k_residual_v<T, double, VSD, 3>, WD, cd.B, cd.smem, P.st, LV.lev<double>(), M, cd.sg, dst, rel->b64,
                rel->x64, r, (cplx<T>*)nullptr, redbuf(P), (double*)nullptr, 0);
    } else {
        vlaunch(k_fix_bnd<T, VS>, W, c.B, 0, P.st, M, c.sg, dst, b, x);
        vlaunch(k_residual_v<T, T, VS, 3>, W, c.B, c.smem, P.st, L, M, c.sg, dst, b, x, r, (cplx<T>*)nullptr, redbuf(P),
                (double*)nullptr, 0);
    }
    auto restart = [&]() -> int {  // z = M^-1 r ; p = w = 0 ; next beta = 0
        CK(cudaMemsetAsync(p, 0, vb, P.st));
        CK(cudaMemsetAsync(w, 0, vb, P.st));
        precond<T, VS, RHS_VEC>(P, LV, z, r, nullptr, nullptr);
        return SFDX_OK;
    };
    RC(restart());
    bool first = true;
    int last_rel = 0;
    ResMin emin;  // smallest residual per system (pf32_divergence)
    auto body = [&](bool fst) {
        if (fst)
            vlaunch(k_cocr_u<T, VS, true>, W, c.B, c.smem, P.st, L, M, c.sg, dst, (const cplx<T>*)z, u, redbuf(P));
        else
            vlaunch(k_cocr_u<T, VS, false>, W, c.B, c.smem, P.st, L, M, c.sg, dst, (const cplx<T>*)z, u, redbuf(P));
        if (P.o.precond == 'J') {
            vlaunch(k_cocr_dir<T, VS>, W, c.B, 0, P.st, M, c.sg, dst, (const cplx<T>*)u, w, (const cplx<T>*)z, p);
            precond<T, VS, RHS_VEC>(P, LV, q, w, nullptr, nullptr);
        } else {
            precond<T, VS, RHS_COCR>(P, LV, q, w, u, z, p);
        }
        vlaunch(k_cocr_alpha<T, VS>, W, c.B, c.smem, P.st, L, M, c.sg, dst, (const cplx<T>*)w, (const cplx<T>*)q,
                redbuf(P));
        vlaunch(k_cocr_upd<T, T, VS>, W, c.B, c.smem, P.st, M, c.sg, dst, x, r, z, (const cplx<T>*)p, (const cplx<T>*)w,
                (const cplx<T>*)q, redbuf(P), P.hist, P.hist_stride);
    };
    for (int it = 1; it <= itmax; it++) {
        if (graph_interval(P, it, itmax, false)) {
            const bool f0 = first;
            RC(graph_run(P, interval_key<T>(P, LV, 6, VS, {(uintptr_t)x, (uintptr_t)b, (uintptr_t)f0}), [&] {
                for (int k = 0; k < 8; k++) body(f0 && k == 0);
            }));
            it += 7;
        } else {
            body(first);
        }
        first = false;
        if (it % 8 == 0 || it == itmax) {
            CK(cudaGetLastError());
            RC(sync_state(P));
            RC(pf32_divergence(P, emin));
            int act = 0, cand = 0;
            for (int k = 0; k < ns; k++) {
                act += P.hst[k].active;
                cand += P.hst[k].status == ST_CONV;
            }
            if (rel && (cand || (act && (it - last_rel >= rel->every || it == itmax)))) {
                RC((reliable_update<T, VS>(P, LV, *rel, x, r, r, 6, act)));
                last_rel = it;
                if (act && it < itmax) {
                    RC(restart());
                    first = true;
                }
            }
            if (!act) break;
        }
    }
    if (rel) vlaunch(k_flush_v<T, VS, true>, W, c.B, 0, P.st, M, c.sg, dst, rel->x64, x, (double2*)nullptr);
    RC(sync_state(P));
    return SFDX_OK;
}

// Right-preconditioned TFQMR (Freund 1993; SFDX_SOLVER_TFQMR -- ptfqmr,
// solvers.f90:317-519, reads tmp, u and r0 before setting them) for the ns
// systems of level LV, same calling convention as bicgstab.  Per iteration two
// operator and two preconditioner applications, two quasi-minimisation
// half-steps; convergence on the residual bound tau sqrt(m+1).  FP64 only
// (mixed-precision plans run it in FP64).
template <class T, int VS>
static int tfqmr_v(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol,
                   int itmax, const int* mask_host, const Reliable* rel) {
    if (rel) return SFDX_ERR_UNSUPPORTED;
    const Lev<T> L = LV.lev<T>();
    const Mesh& M = LV.mesh;
    const int ns = P.ns;
    const size_t vb = (size_t)LV.nl * ns * sizeof(cplx<T>);
    for (int k = 0; k < 10; k++) RC(P.kv[k].alloc(vb));
    cplx<T>* V[10];
    for (int k = 0; k < 10; k++) V[k] = P.kv[k].as<cplx<T>>();
    cplx<T> *w = V[0], *rt = V[1], *u = V[2], *uh = V[3], *v = V[4], *q = V[5], *qh = V[6], *aq = V[7], *d = V[8];
    cplx<T>* au = V[9];
    std::vector<KState> init;
    init_states(P, tols_host, tol, itmax, mask_host, init);
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    const VCfg c = vcfg(P, LV.nl, 2, VS);
    RC(reserve_partials(P, c, 2));
    KState* dst = P.d_state.as<KState>();
    const int64_t W = LV.nl * c.sg.G;
    const double* wm = P.d_wm.as<double>();
    const cplx<T>* nul = nullptr;
    // out_h = M^-1 in, out_a = A out_h
    auto amv = [&](cplx<T>* out_h, cplx<T>* out_a, cplx<T>* in) {
        precond<T, VS, RHS_VEC>(P, LV, out_h, in, nullptr, nullptr);
        vlaunch(k_apply_v<T, VS>, W, c.B, 0, P.st, L, M, c.sg, wm, (const cplx<T>*)out_h, out_a);
    };
    auto xupd = [&]() {  // x += eta d, then stop the systems that met the test
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_ETA, BC_ZERO>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, x,
                (const cplx<T>*)x, (const cplx<T>*)d, nul);
        KL(k_bl_commit<<<(ns + 127) / 128, 128, 0, P.st>>>(dst, ns));
    };
    auto body = [&]() {
        vlaunch(k_bl_dot<T, VS, FIN_TFQ_SIGMA>, W, c.B, c.smem, P.st, M, c.sg, dst, (const cplx<T>*)rt,
                (const cplx<T>*)v, nul, nul, redbuf(P));
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_MALPHA, BC_ZERO>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, q,
                (const cplx<T>*)u, (const cplx<T>*)v, nul);
        amv(qh, aq, q);
        vlaunch(k_tfq_half<T, VS>, W, c.B, c.smem, P.st, M, c.sg, dst, w, (const cplx<T>*)v, d, (const cplx<T>*)uh,
                redbuf(P), P.hist, P.hist_stride);
        xupd();
        vlaunch(k_tfq_half<T, VS>, W, c.B, c.smem, P.st, M, c.sg, dst, w, (const cplx<T>*)aq, d, (const cplx<T>*)qh,
                redbuf(P), P.hist, P.hist_stride);
        xupd();
        vlaunch(k_bl_dot<T, VS, FIN_TFQ_RHO>, W, c.B, c.smem, P.st, M, c.sg, dst, (const cplx<T>*)rt,
                (const cplx<T>*)w, nul, nul, redbuf(P));
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_BETA, BC_ZERO>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, u,
                (const cplx<T>*)w, (const cplx<T>*)q, nul);
        amv(uh, au, u);
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_BETA, BC_BETA2>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, v,
                (const cplx<T>*)au, (const cplx<T>*)aq, (const cplx<T>*)v);
    };
    // The stopping test is the quasi-residual bound tau sqrt(m+1), which the
    // true residual can exceed once rounding has accumulated: systems that pass
    // it are checked against b - A x and restarted from their iterate if not
    // converged, within the iteration budget.
    std::vector<int> total(ns, 0);
    int used = 0;
    for (int round = 0; round < 32 && used < itmax; round++) {
        const int budget = itmax - used;
        CK(cudaMemsetAsync(d, 0, vb, P.st));
        vlaunch(k_residual_v<T, T, VS, 3>, W, c.B, c.smem, P.st, L, M, c.sg, dst, b, (const cplx<T>*)x, w, rt,
                redbuf(P), (double*)nullptr, 0);
        vlaunch(k_bl_dot<T, VS, FIN_TFQ_INIT>, W, c.B, c.smem, P.st, M, c.sg, dst, (const cplx<T>*)rt,
                (const cplx<T>*)w, (const cplx<T>*)w, (const cplx<T>*)w, redbuf(P));
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_ZERO, BC_ZERO>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, u,
                (const cplx<T>*)w, nul, nul);
        amv(uh, v, u);
        int done = 0;
        for (int it = 1; it <= budget; it++) {
            if (graph_interval(P, it, budget, false)) {
                RC(graph_run(P, interval_key<T>(P, LV, 2, VS, {(uintptr_t)x, (uintptr_t)b}), [&] {
                    for (int k = 0; k < 8; k++) body();
                }));
                it += 7;
            } else {
                body();
            }
            done = it;
            if (it % 8 == 0 || it == budget) {
                CK(cudaGetLastError());
                RC(sync_state(P));
                int act = 0;
                for (int k = 0; k < ns; k++) act += P.hst[k].active;
                if (!act) break;
            }
        }
        used += done;
        RC(sync_state(P));
        for (int k = 0; k < ns; k++) total[k] += P.hst[k].iters;
        // true residual of the systems that claim convergence
        KL(k_reactivate<<<(ns + 127) / 128, 128, 0, P.st>>>(dst, ns));
        vlaunch(k_residual_v<T, T, VS, 2>, W, c.B, c.smem, P.st, L, M, c.sg, dst, b, (const cplx<T>*)x, w,
                (cplx<T>*)nullptr, redbuf(P), (double*)nullptr, 0);
        RC(sync_state(P));
        int restart = 0;
        for (int k = 0; k < ns; k++) {
            KState& S = P.hst[k];
            if (!S.active) continue;  // not a convergence claim
            const double rel = S.babs > 0 ? S.err / S.babs : S.err;
            S.err = rel;
            S.iters = total[k];
            if (rel < S.tol) {
                S.active = 0;
                S.status = ST_CONV;
            } else {
                S.status = used < itmax ? ST_RUN : ST_MAXIT;
                S.active = used < itmax ? 1 : 0;
                restart += S.active;
            }
        }
        for (int k = 0; k < ns; k++) P.hst[k].iters = total[k];
        CK(cudaMemcpyAsync(P.d_state.p, P.hst.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
        if (!restart) break;
    }
    RC(sync_state(P));
    for (int k = 0; k < ns; k++) P.hst[k].iters = total[k];
    return SFDX_OK;
}

// Preconditioned two-sided BiCG for complex systems (Fletcher 1976, in the
// preconditioned form of the Templates book; SFDX_SOLVER_BICG -- pbicg,
// solvers.f90:878-1025, never forms zt with SSOR).  The shadow recurrence uses
// A^H and M^-H, formed through the dual-volume symmetry (k_bl_conj_vscale).
// FP64 only (mixed-precision plans run it in FP64).
template <class T, int VS>
static int bicg2_v(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol,
                   int itmax, const int* mask_host, const Reliable* rel) {
    if (rel) return SFDX_ERR_UNSUPPORTED;
    const Lev<T> L = LV.lev<T>();
    const Mesh& M = LV.mesh;
    const int ns = P.ns;
    const size_t vb = (size_t)LV.nl * ns * sizeof(cplx<T>);
    for (int k = 0; k < 10; k++) RC(P.kv[k].alloc(vb));
    cplx<T>* V[10];
    for (int k = 0; k < 10; k++) V[k] = P.kv[k].as<cplx<T>>();
    cplx<T> *r = V[0], *rt = V[1], *z = V[2], *zt = V[3], *p = V[4], *pt = V[5], *q = V[6], *qt = V[7], *t1 = V[8];
    cplx<T>* t2 = V[9];
    std::vector<KState> init;
    init_states(P, tols_host, tol, itmax, mask_host, init);
    CK(cudaMemcpyAsync(P.d_state.p, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    const VCfg c = vcfg(P, LV.nl, 2, VS);
    RC(reserve_partials(P, c, 2));
    KState* dst = P.d_state.as<KState>();
    const int64_t W = LV.nl * c.sg.G;
    const double* wm = P.d_wm.as<double>();
    const cplx<T>* nul = nullptr;
    CK(cudaMemsetAsync(p, 0, vb, P.st));
    CK(cudaMemsetAsync(pt, 0, vb, P.st));
    vlaunch(k_residual_v<T, T, VS, 3>, W, c.B, c.smem, P.st, L, M, c.sg, dst, b, (const cplx<T>*)x, r, rt, redbuf(P),
            (double*)nullptr, 0);
    vlaunch(k_bl_dot<T, VS, FIN_BICG_INIT>, W, c.B, c.smem, P.st, M, c.sg, dst, (const cplx<T>*)r, (const cplx<T>*)r,
            nul, nul, redbuf(P));
    // out = (op)^H in through V conj(op(V^-1 conj(in)))
    auto herm = [&](cplx<T>* out, const cplx<T>* in, bool prec) {
        vlaunch(k_bl_conj_vscale<T, VS, true>, W, c.B, 0, P.st, L, M, c.sg, (const KState*)dst, in, t1);
        if (prec)
            precond<T, VS, RHS_VEC>(P, LV, t2, t1, nullptr, nullptr);
        else
            vlaunch(k_apply_v<T, VS>, W, c.B, 0, P.st, L, M, c.sg, wm, (const cplx<T>*)t1, t2);
        vlaunch(k_bl_conj_vscale<T, VS, false>, W, c.B, 0, P.st, L, M, c.sg, (const KState*)dst, (const cplx<T>*)t2,
                out);
    };
    auto body = [&]() {
        precond<T, VS, RHS_VEC>(P, LV, z, r, nullptr, nullptr);
        herm(zt, rt, true);
        vlaunch(k_bl_dot<T, VS, FIN_BICG_RHO>, W, c.B, c.smem, P.st, M, c.sg, dst, (const cplx<T>*)rt,
                (const cplx<T>*)z, nul, nul, redbuf(P));
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_BETA, BC_ZERO>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, p,
                (const cplx<T>*)z, (const cplx<T>*)p, nul);
        vlaunch(k_bl_lincomb<T, VS, BC_ONE, BC_CBETA, BC_ZERO>, W, c.B, 0, P.st, M, c.sg, (const KState*)dst, pt,
                (const cplx<T>*)zt, (const cplx<T>*)pt, nul);
        vlaunch(k_apply_v<T, VS>, W, c.B, 0, P.st, L, M, c.sg, wm, (const cplx<T>*)p, q);
        herm(qt, pt, false);
        vlaunch(k_bl_dot<T, VS, FIN_BICG_ALPHA>, W, c.B, c.smem, P.st, M, c.sg, dst, (const cplx<T>*)pt,
                (const cplx<T>*)q, nul, nul, redbuf(P));
        vlaunch(k_bicg2_upd<T, VS>, W, c.B, c.smem, P.st, M, c.sg, dst, x, r, rt, (const cplx<T>*)p, (const cplx<T>*)q,
                (const cplx<T>*)qt, redbuf(P), P.hist, P.hist_stride);
    };
    for (int it = 1; it <= itmax; it++) {
        if (graph_interval(P, it, itmax, false)) {
            RC(graph_run(P, interval_key<T>(P, LV, 4, VS, {(uintptr_t)x, (uintptr_t)b}), [&] {
                for (int k = 0; k < 8; k++) body();
            }));
            it += 7;
        } else {
            body();
        }
        if (it % 8 == 0 || it == itmax) {
            CK(cudaGetLastError());
            RC(sync_state(P));
            int act = 0;
            for (int k = 0; k < ns; k++) act += P.hst[k].active;
            if (!act) break;
        }
    }
    RC(sync_state(P));
    return SFDX_OK;
}

// ------------------------------------------------------------------ corrected restart cycles
// dst[e][i] = src[e][idx[i]] (i < nd)  /  dst[e][idx[i]] = src[e][i]
static __global__ void k_gather_cols(int64_t nl, int ns, int nd, const int* __restrict__ idx,
                                     const double2* __restrict__ src, double2* __restrict__ dst) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nl * nd; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = g / nd;
        const int i = (int)(g - e * nd);
        dst[g] = src[e * ns + __ldg(idx + i)];
    }
}
static __global__ void k_scatter_cols(int64_t nl, int ns, int nd, const int* __restrict__ idx,
                                      const double2* __restrict__ src, double2* __restrict__ dst) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nl * nd; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = g / nd;
        const int i = (int)(g - e * nd);
        dst[e * ns + __ldg(idx + i)] = src[g];
    }
}

// div_cor = 2: the Krylov solve runs in cycles of corr_intv iterations; before
// every cycle and after the last one the FP64 iterate gets the consistent
// gradient-space correction (sfdx_gradcorr.cuh), and each cycle restarts the
// Krylov recurrences from the corrected iterate.  Because a cycle starts from
// the FP64 iterate alone, the systems still running are packed into a
// smaller batch for the cycle (FP64 right-hand side and iterate gathered,
// iterate scattered back): finished systems cost nothing, and the kernels'
// threads all work on running systems.  `run(itmax_cycle, b, x, rel)` is one
// Krylov solve from the current iterate of every system of the (possibly
// packed) batch; per-system iteration counts and statuses over all cycles are
// left in P.hst.
template <class T, class F>
static int corrected_cycles(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, int itmax, const int* mask_host,
                            const Reliable* rel, F run) {
    const int ns = P.ns;
    const double2* b64 = rel ? rel->b64 : reinterpret_cast<const double2*>(b);
    double2* x64 = rel ? rel->x64 : reinterpret_cast<double2*>(x);
    std::vector<int> mask(ns), part(ns), used(ns, 0), fin(ns, ST_CONV);
    for (int q = 0; q < ns; q++) part[q] = mask[q] = mask_host ? (mask_host[q] != 0) : 1;
    const int cyc0 = P.o.corr_intv > 0 ? P.o.corr_intv : 25;
    // cycle length grows by 1.5 per cycle (SFDX_CYCLE_GROWTH overrides): the
    // systems still running late (high frequencies) lose less Krylov history
    // to restarts, while the early cycles keep the correction frequent.  On the
    // 80x80x80 anisotropic model at 1e-10: 15.6 solves/s against 13.8 with fixed cycles (2.0: 14.9).
    // TFQMR keeps fixed cycles: it stagnates without frequent corrections.
    const char* gr_env = getenv("SFDX_CYCLE_GROWTH");
    const double growth =
        P.o.solver == SFDX_SOLVER_TFQMR ? 1.0 : gr_env ? std::max(1.0, atof(gr_env)) : 1.5;
    double cyc_f = cyc0;
    int cyc = cyc0;
    const int gc_maxit = 2000;  // pcg itmax (div_correc.f90:57)
    const std::vector<double> wm_all = P.wm;
    const bool can_pack = P.hist == nullptr;  // residual histories are indexed by the full batch
    std::vector<KState> hs(ns);
    for (;;) {
        std::vector<int> idx;
        for (int q = 0; q < ns; q++)
            if (mask[q]) idx.push_back(q);
        const int nd = (int)idx.size();
        const bool pack = can_pack && nd < ns;
        const double2* bc = b64;
        double2* xc = x64;
        if (pack) {  // the running systems become a batch of nd
            const size_t nb = (size_t)LV.nl * nd * sizeof(double2);
            RC(P.cb64.alloc(nb));
            RC(P.cx64.alloc(nb));
            RC(P.d_idx.alloc(sizeof(int) * ns));
            CK(cudaMemcpyAsync(P.d_idx.p, idx.data(), sizeof(int) * nd, cudaMemcpyHostToDevice, P.st));
            KL(k_gather_cols<<<grid_for(LV.nl * nd, 256, 16), 256, 0, P.st>>>(LV.nl, ns, nd, P.d_idx.as<int>(), b64,
                                                                              P.cb64.as<double2>()));
            KL(k_gather_cols<<<grid_for(LV.nl * nd, 256, 16), 256, 0, P.st>>>(LV.nl, ns, nd, P.d_idx.as<int>(), x64,
                                                                              P.cx64.as<double2>()));
            bc = P.cb64.as<double2>();
            xc = P.cx64.as<double2>();
            if (P.rec_on) P.rec_map = idx;
            P.ns = nd;
            P.wm.resize(nd);
            for (int i = 0; i < nd; i++) P.wm[i] = wm_all[idx[i]];
        }
        int room = 0;
        for (int q = 0; q < ns; q++)
            if (mask[q]) room = std::max(room, itmax - used[q]);
        const int* m = pack ? nullptr : mask.data();
        int gc_its = 0;
        const auto t0 = std::chrono::steady_clock::now();
        int rc = grad_correct(P, LV, bc, xc, m, P.o.corr_tol, gc_maxit, &gc_its);
        const auto t1 = std::chrono::steady_clock::now();
        if (rc == SFDX_OK) {
            if (rel) {
                Reliable rc_rel = *rel;
                rc_rel.b64 = bc;
                rc_rel.x64 = xc;
                rc = run(std::min(cyc, room), m, b, x, &rc_rel);
            } else {
                rc = run(std::min(cyc, room), m, reinterpret_cast<const cplx<T>*>(bc), reinterpret_cast<cplx<T>*>(xc),
                         nullptr);
            }
        }
        const auto t2 = std::chrono::steady_clock::now();
        if (pack) {  // back to the full batch
            KL(k_scatter_cols<<<grid_for(LV.nl * nd, 256, 16), 256, 0, P.st>>>(LV.nl, ns, nd, P.d_idx.as<int>(),
                                                                               P.cx64.as<double2>(), x64));
            P.ns = ns;
            P.wm = wm_all;
            P.rec_map.clear();
            if (rc == SFDX_OK)
                for (int i = 0; i < nd; i++) hs[idx[i]] = P.hst[i];
        } else if (rc == SFDX_OK) {
            for (int q = 0; q < ns; q++) hs[q] = P.hst[q];
        }
        RC(rc);
        if (P.o.verbose || getenv("SFDX_VERBOSE")) {
            double emin = 1e300, emax = 0;
            int cnt[6] = {0, 0, 0, 0, 0, 0};
            for (int q : idx) {
                emin = std::min(emin, hs[q].err);
                emax = std::max(emax, hs[q].err);
                if (hs[q].status >= 0 && hs[q].status < 6) cnt[hs[q].status]++;
            }
            const double ms_gc = std::chrono::duration<double, std::milli>(t1 - t0).count();
            const double ms_kr = std::chrono::duration<double, std::milli>(t2 - t1).count();
            fprintf(stderr,
                    "sfdx:   cycle (%s, %d of %d systems, %d its %.1f ms, nodal pcg %d its %.1f ms): err %.2e..%.2e  run %d "
                    "conv %d maxit %d nan %d break %d vconv %d\n",
                    rel ? "mixed" : "fp64", nd, ns, std::min(cyc, room), ms_kr, gc_its, ms_gc, emin, emax, cnt[0],
                    cnt[1], cnt[2], cnt[3], cnt[4], cnt[5]);
        }
        int left = 0;
        for (int q : idx) {
            const int st = hs[q].status;
            used[q] += std::max(1, hs[q].iters);
            if (P.rec_on && q < (int)P.rec_off.size()) P.rec_off[q] = used[q];
            // a breakdown under complex64 iterations or the complex64 V-cycle is
            // handed to the caller's FP64 finish / FP64 V-cycle restart
            if (st == ST_CONV || st == ST_VCONV || st == ST_NAN || (st == ST_BREAK && (rel || P.pf32))) {
                mask[q] = 0;  // converged, failed, or handed to the caller's FP64 finish
                fin[q] = st;
            } else if (used[q] >= itmax) {
                mask[q] = 0;
                fin[q] = ST_MAXIT;
            } else {
                left++;  // cycle limit reached (or an FP64 breakdown): restart
            }
        }
        if (!left) break;
        cyc_f *= growth;
        cyc = (int)std::min(cyc_f, 1e6);
    }
    std::vector<int> last(ns);
    for (int q = 0; q < ns; q++) last[q] = part[q] && fin[q] != ST_NAN && !(fin[q] == ST_BREAK && (rel || P.pf32));
    RC(grad_correct(P, LV, b64, x64, last.data(), P.o.corr_tol, gc_maxit, nullptr));
    P.hst.resize(ns);
    for (int q = 0; q < ns; q++) {
        P.hst[q] = hs[q];
        if (!part[q]) continue;
        P.hst[q].iters = used[q];
        P.hst[q].status = fin[q];
    }
    return SFDX_OK;
}

// ------------------------------------------------------------------ entry points (VS dispatch)
template <class T>
int bicgstab(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
             const int* mask_host, const Reliable* rel) {
    RC(emg_prepare<T>(P, LV));
    auto run = [&](int itc, const int* m, const cplx<T>* bb, cplx<T>* xx, const Reliable* rr) -> int {
        switch (plan_vs<T>(P)) {
            case 4: return bicgstab_v<T, 4>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            case 2: return bicgstab_v<T, 2>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            default: return bicgstab_v<T, 1>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
        }
    };
    if (P.o.div_cor == 2 && (rel || std::is_same<T, double>::value))
        return corrected_cycles<T>(P, LV, b, x, itmax, mask_host, rel, run);
    return run(itmax, mask_host, b, x, rel);
}
template <class T>
int gpbicg(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
           const int* mask_host, const Reliable* rel) {
    RC(emg_prepare<T>(P, LV));
    auto run = [&](int itc, const int* m, const cplx<T>* bb, cplx<T>* xx, const Reliable* rr) -> int {
        switch (plan_vs<T>(P)) {
            case 4: return gpbicg_v<T, 4>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            case 2: return gpbicg_v<T, 2>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            default: return gpbicg_v<T, 1>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
        }
    };
    if (P.o.div_cor == 2 && (rel || std::is_same<T, double>::value))
        return corrected_cycles<T>(P, LV, b, x, itmax, mask_host, rel, run);
    return run(itmax, mask_host, b, x, rel);
}
template <class T>
int cocr(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
         const int* mask_host, const Reliable* rel) {
    RC(emg_prepare<T>(P, LV));
    auto run = [&](int itc, const int* m, const cplx<T>* bb, cplx<T>* xx, const Reliable* rr) -> int {
        switch (plan_vs<T>(P)) {
            case 4: return cocr_v<T, 4>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            case 2: return cocr_v<T, 2>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            default: return cocr_v<T, 1>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
        }
    };
    if (P.o.div_cor == 2 && (rel || std::is_same<T, double>::value))
        return corrected_cycles<T>(P, LV, b, x, itmax, mask_host, rel, run);
    return run(itmax, mask_host, b, x, rel);
}
template <class T>
int tfqmr(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
          const int* mask_host, const Reliable* rel) {
    RC(emg_prepare<T>(P, LV));
    auto run = [&](int itc, const int* m, const cplx<T>* bb, cplx<T>* xx, const Reliable* rr) -> int {
        switch (plan_vs<T>(P)) {
            case 4: return tfqmr_v<T, 4>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            case 2: return tfqmr_v<T, 2>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            default: return tfqmr_v<T, 1>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
        }
    };
    if (P.o.div_cor == 2 && (rel || std::is_same<T, double>::value))
        return corrected_cycles<T>(P, LV, b, x, itmax, mask_host, rel, run);
    return run(itmax, mask_host, b, x, rel);
}
template <class T>
int bicg(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
         const int* mask_host, const Reliable* rel) {
    RC(emg_prepare<T>(P, LV));
    auto run = [&](int itc, const int* m, const cplx<T>* bb, cplx<T>* xx, const Reliable* rr) -> int {
        switch (plan_vs<T>(P)) {
            case 4: return bicg2_v<T, 4>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            case 2: return bicg2_v<T, 2>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
            default: return bicg2_v<T, 1>(P, LV, bb, xx, tols_host, tol, itc, m, rr);
        }
    };
    if (P.o.div_cor == 2 && (rel || std::is_same<T, double>::value))
        return corrected_cycles<T>(P, LV, b, x, itmax, mask_host, rel, run);
    return run(itmax, mask_host, b, x, rel);
}
template <class T> int precond_vec(Plan& P, const Level& LV, cplx<T>* out, cplx<T>* q) {
    RC(emg_prepare<T>(P, LV));
    switch (plan_vs<T>(P)) {
        case 4: precond<T, 4, RHS_VEC>(P, LV, out, q, nullptr, nullptr); break;
        case 2: precond<T, 2, RHS_VEC>(P, LV, out, q, nullptr, nullptr); break;
        default: precond<T, 1, RHS_VEC>(P, LV, out, q, nullptr, nullptr); break;
    }
    CK(cudaGetLastError());
    return SFDX_OK;
}
template <class T> int apply_op(Plan& P, const Level& LV, const cplx<T>* x, cplx<T>* y) {
    const VCfg c = vcfg(P, LV.nl, 0, plan_vs<T>(P), 16);
    const double* wm = P.d_wm.as<double>();
    switch (c.VS) {
        case 4: vlaunch(k_apply_v<T, 4>, LV.nl * c.sg.G, c.B, 0, P.st, LV.lev<T>(), LV.mesh, c.sg, wm, x, y); break;
        case 2: vlaunch(k_apply_v<T, 2>, LV.nl * c.sg.G, c.B, 0, P.st, LV.lev<T>(), LV.mesh, c.sg, wm, x, y); break;
        default: vlaunch(k_apply_v<T, 1>, LV.nl * c.sg.G, c.B, 0, P.st, LV.lev<T>(), LV.mesh, c.sg, wm, x, y); break;
    }
    CK(cudaGetLastError());
    return SFDX_OK;
}

#define SFDX_INSTANTIATE_KRYLOV(T)                                                                                      \
    template int bicgstab<T>(Plan&, const Level&, const cplx<T>*, cplx<T>*, const double*, double, int, const int*,    \
                             const Reliable*);                                                                          \
    template int gpbicg<T>(Plan&, const Level&, const cplx<T>*, cplx<T>*, const double*, double, int, const int*,      \
                           const Reliable*);                                                                            \
    template int cocr<T>(Plan&, const Level&, const cplx<T>*, cplx<T>*, const double*, double, int, const int*,        \
                         const Reliable*);                                                                              \
    template int tfqmr<T>(Plan&, const Level&, const cplx<T>*, cplx<T>*, const double*, double, int, const int*,       \
                          const Reliable*);                                                                             \
    template int bicg<T>(Plan&, const Level&, const cplx<T>*, cplx<T>*, const double*, double, int, const int*,        \
                         const Reliable*);                                                                              \
    template int precond_vec<T>(Plan&, const Level&, cplx<T>*, cplx<T>*);                                               \
    template int apply_op<T>(Plan&, const Level&, const cplx<T>*, cplx<T>*);

}  // namespace sfdx
