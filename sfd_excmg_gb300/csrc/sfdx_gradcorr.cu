// sfdx_gradcorr.cu -- host driver of the consistent gradient-space correction
// (kernels and derivation in sfdx_gradcorr.cuh; nodal multigrid in
// sfdx_nodemg.cuh).
#include "sfdx_gradcorr.cuh"
#include "sfdx_mgkern.cuh"
#include "sfdx_plan.h"

namespace sfdx {

// Assemble N = G^T V Ms G of level LV as a 27-point nodal stencil by probing
// the matrix-free product, then the Galerkin coarse stencils R N P of the
// nodal multigrid, also by probing; cached until the conductivity changes.
static int gc_assemble(Plan& P, const Level& LV) {
    const Mesh& M = LV.mesh;
    const Lev<double> L = LV.lev<double>();
    const int NPR = 27;
    LV.mg.clear();
    LV.mg.emplace_back();
    LV.mg[0].g = make_ngrid(LV.nx, LV.ny, LV.nz);
    while (true) {  // 2x coarsenings while every axis stays even with interior nodes
        const NGrid f = LV.mg.back().g;  // a copy: emplace_back may move the elements
        if (f.nx % 2 || f.ny % 2 || f.nz % 2 || f.nx < 4 || f.ny < 4 || f.nz < 4) break;
        LV.mg.emplace_back();
        LV.mg.back().g = make_ngrid(f.nx / 2, f.ny / 2, f.nz / 2);
    }
    const uint32_t np = LV.mg[0].g.np;
    for (auto& q : LV.mg) {
        RC(q.coef.alloc((size_t)27 * q.g.np * sizeof(float)));
        RC(q.dinv.alloc((size_t)q.g.np * sizeof(float)));
    }
    RC(P.gcn[0].alloc((size_t)np * NPR * sizeof(double2)));
    RC(P.gcn[1].alloc((size_t)np * NPR * sizeof(double2)));
    RC(P.gce[0].alloc((size_t)LV.nl * NPR * sizeof(double2)));
    RC(P.gce[1].alloc((size_t)LV.nl * NPR * sizeof(double2)));
    RC(P.d_pst.alloc(sizeof(KState) * std::max(P.ns, NPR)));
    std::vector<KState> init(NPR);
    for (auto& S : init) {
        memset(&S, 0, sizeof(S));
        S.active = 1;
    }
    KState* pst = P.d_pst.as<KState>();
    CK(cudaMemcpyAsync(pst, init.data(), sizeof(KState) * NPR, cudaMemcpyHostToDevice, P.st));
    const SysG sg = make_sysg(NPR, 1);
    const int B = vblock(sg.G);
    // finest: FP64 matrix-free product on the 27 probes
    {
        double2 *pr = P.gcn[0].as<double2>(), *Q = P.gcn[1].as<double2>();
        double2 *ge = P.gce[0].as<double2>(), *u = P.gce[1].as<double2>();
        KL(k_gc_probe<<<grid_for((int64_t)np * NPR, 256, 16), 256, 0, P.st>>>(M, np, pr));
        vlaunch(k_gc_grad<1>, LV.nl * sg.G, B, 0, P.st, L, M, sg, pst, pr, ge);
        vlaunch(k_gc_mass<1>, LV.nl * sg.G, B, 0, P.st, L, M, sg, pst, ge, u);
        vlaunch(k_gc_gtu<1>, np * sg.G, B, 0, P.st, L, M, sg, np, u, Q);
        const NGrid g0 = LV.mg[0].g;
        KL(k_mg_assemble<double2><<<grid_for(np, 256, 16), 256, 0, P.st>>>(g0, Q, LV.mg[0].coef.as<float>(),
                                                                             LV.mg[0].dinv.as<float>()));
    }
    // coarser: R N P on the 27 coarse probes (complex64 work vectors)
    for (size_t l = 1; l < LV.mg.size(); l++) {
        const NGrid gf = LV.mg[l - 1].g, gc = LV.mg[l].g;
        float2* pc = P.gcn[0].as<float2>();             // coarse probes   [np_c][27]
        // second arrays of each buffer start on a 32-byte boundary (vlaunch
        // requires aligned pointer arguments); the buffers hold 2 np 27 float2
        auto a32 = [](size_t n) { return (n + 3) / 4 * 4; };
        float2* xf = P.gcn[0].as<float2>() + a32((size_t)gc.np * NPR);  // prolonged [np_f][27]
        float2* yf = P.gcn[1].as<float2>();                             // N P probes [np_f][27]
        float2* Qc = P.gcn[1].as<float2>() + a32((size_t)gf.np * NPR);  // responses  [np_c][27]
        KL(k_mg_probe<<<grid_for((int64_t)gc.np * NPR, 256, 16), 256, 0, P.st>>>(gc, pc));
        CK(cudaMemsetAsync(xf, 0, (size_t)gf.np * NPR * sizeof(float2), P.st));
        vlaunch(k_mg_prolong<float, 1>, (int64_t)gf.np * sg.G, B, 0, P.st, gf, gc, sg, pst, pc, xf);
        vlaunch(k_mg_resid<float, 1>, (int64_t)gf.np * sg.G, B, 0, P.st, gf, sg, pst, LV.mg[l - 1].coef.as<float>(),
                (const float2*)nullptr, xf, yf);
        vlaunch(k_mg_restrict<float, 1>, (int64_t)gc.np * sg.G, B, 0, P.st, gc, gf, sg, pst, yf, Qc);
        KL(k_mg_assemble<float2><<<grid_for(gc.np, 256, 16), 256, 0, P.st>>>(gc, Qc, LV.mg[l].coef.as<float>(),
                                                                              LV.mg[l].dinv.as<float>()));
    }
    CK(cudaGetLastError());
    LV.gc_ok = true;
    return SFDX_OK;
}

// Jacobi damping and sweep counts of the V-cycle
static const float kMgOmega = 0.7f;
static const int kMgCoarseSweeps = 15;  // odd: the result ends in x

// x = V-cycle(b) on multigrid level l (complex64, systems active in pst)
template <int VS>
static void vcycle(Plan& P, const Level& LV, const SysG& sg, int B, const KState* pst, size_t l, const float2* b,
                   float2* x) {
    const NodeMG& Lv = LV.mg[l];
    const NGrid g = Lv.g;
    const int64_t W = (int64_t)g.np * sg.G;
    const float* coef = Lv.coef.as<float>();
    const float* dinv = Lv.dinv.as<float>();
    float2* t = Lv.t.as<float2>();
    if (l + 1 == LV.mg.size()) {
        vlaunch(k_mg_smooth<float, VS, true>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)nullptr, x,
                kMgOmega);
        for (int s = 1; s < kMgCoarseSweeps; s += 2) {
            vlaunch(k_mg_smooth<float, VS, false>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)x, t, kMgOmega);
            vlaunch(k_mg_smooth<float, VS, false>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)t, x, kMgOmega);
        }
        return;
    }
    const NodeMG& C = LV.mg[l + 1];
    float2* r = Lv.r.as<float2>();
    vlaunch(k_mg_smooth<float, VS, true>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)nullptr, t, kMgOmega);
    vlaunch(k_mg_smooth<float, VS, false>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)t, x, kMgOmega);
    vlaunch(k_mg_resid<float, VS>, W, B, 0, P.st, g, sg, pst, coef, b, (const float2*)x, r);
    vlaunch(k_mg_restrict<float, VS>, (int64_t)C.g.np * sg.G, B, 0, P.st, C.g, g, sg, pst, (const float2*)r,
            C.b.as<float2>());
    vcycle<VS>(P, LV, sg, B, pst, l + 1, C.b.as<float2>(), C.x.as<float2>());
    vlaunch(k_mg_prolong<float, VS>, W, B, 0, P.st, g, C.g, sg, pst, (const float2*)C.x.as<float2>(), x);
    vlaunch(k_mg_smooth<float, VS, false>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)x, t, kMgOmega);
    vlaunch(k_mg_smooth<float, VS, false>, W, B, 0, P.st, g, sg, pst, coef, dinv, b, (const float2*)t, x, kMgOmega);
}

template <int VS>
static int grad_correct_v(Plan& P, const Level& LV, const double2* b, double2* x, const int* mask, double tol, int maxit,
                          int* iters) {
    typedef float T;  // nodal PCG in complex64 (loose tolerance); r, t and x stay FP64
    const int ns = P.ns;
    const Mesh& M = LV.mesh;
    const Lev<double> L = LV.lev<double>();
    const uint32_t np = (uint32_t)(LV.nx + 1) * (LV.ny + 1) * (LV.nz + 1);
    if (iters) *iters = 0;
    std::vector<KState> init(ns);
    int any = 0;
    for (int s = 0; s < ns; s++) {
        KState S;
        memset(&S, 0, sizeof(S));
        S.wm = P.wm[s];
        S.tol = tol;
        S.itmax = maxit;
        S.active = mask ? mask[s] : 1;
        S.status = S.active ? ST_RUN : ST_SKIP;
        S.pad[1] = S.active;
        any += S.active;
        init[s] = S;
    }
    if (!any) return SFDX_OK;
    RC(nodal_setup(P, LV));
    const size_t nb = (size_t)np * ns * sizeof(cplx<T>), eb = (size_t)LV.nl * ns * sizeof(double2);
    for (int q = 0; q < 5; q++) RC(P.gcn[q].alloc(nb));
    for (size_t l = 0; l < LV.mg.size(); l++) {
        const size_t nbl = (size_t)LV.mg[l].g.np * ns * sizeof(cplx<T>);
        RC(LV.mg[l].t.alloc(nbl));
        RC(LV.mg[l].r.alloc(nbl));
        if (l) {
            RC(LV.mg[l].x.alloc(nbl));
            RC(LV.mg[l].b.alloc(nbl));
        }
    }
    RC(P.r64.alloc(eb));
    RC(P.d_pst.alloc(sizeof(KState) * std::max(ns, 27)));
    cplx<T> *phi = P.gcn[0].as<cplx<T>>(), *rn = P.gcn[1].as<cplx<T>>(), *z = P.gcn[2].as<cplx<T>>();
    cplx<T> *p = P.gcn[3].as<cplx<T>>(), *q = P.gcn[4].as<cplx<T>>();
    double2* re = P.r64.as<double2>();
    const float* coef = LV.mg[0].coef.as<float>();
    const float* dinv = LV.mg[0].dinv.as<float>();
    KState* pst = P.d_pst.as<KState>();
    CK(cudaMemcpyAsync(pst, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    constexpr int VSD = VS > 2 ? 2 : VS;  // systems per thread of the FP64 edge kernels
    const VCfg ce = vcfg(P, LV.nl, 2, VSD);
    const VCfg cnd = vcfg(P, np, 2, VSD);
    const VCfg cn = vcfg(P, np, 2, VS);
    RC(P.d_part.alloc(std::max(P.d_part.bytes, (size_t)max_resident_blocks() * 2 * ns * sizeof(double2))));
    // the gradient-space part of r = b - A x (FP64), formed as b + i w mu Ms x
    // (k_mg_mres_v: without the curl-curl terms, whose rounding noise the
    // nodal solve would amplify by 1/(w mu sigma) in air), then the nodal
    // right-hand side, z = M^{-1} r, p = z
    vlaunch(k_mg_mres_v<double, VSD>, LV.nl * ce.sg.G, ce.B, 0, P.st, L, M, ce.sg, (const KState*)pst, b,
            (const double2*)x, re);
    vlaunch(k_gc_rhs<T, VSD, false>, np * cnd.sg.G, cnd.B, cnd.smem, P.st, L, M, cnd.sg, np, pst, re, dinv, rn, z, p, phi,
            redbuf(P));
    vcycle<VS>(P, LV, cn.sg, cn.B, pst, 0, rn, z);
    vlaunch(k_gc_rz<T, VS, true>, np * cn.sg.G, cn.B, cn.smem, P.st, cn.sg, np, pst, rn, z, redbuf(P));
    vlaunch(k_gc_p<T, VS, true>, np * cn.sg.G, cn.B, 0, P.st, cn.sg, np, pst, z, p);
    CK(cudaGetLastError());
    std::vector<KState> h(ns);
    for (int it = 0; it < maxit; it++) {
        vlaunch(k_gc_Ap<T, VS>, np * cn.sg.G, cn.B, cn.smem, P.st, M, cn.sg, np, pst, coef, p, q, redbuf(P));
        vlaunch(k_gc_upd<T, VS, false>, np * cn.sg.G, cn.B, cn.smem, P.st, cn.sg, np, pst, dinv, p, q, phi, rn, z,
                redbuf(P));
        if ((it + 1) % 4 == 0) {
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(h.data(), pst, sizeof(KState) * ns, cudaMemcpyDeviceToHost, P.st));
            CK(cudaStreamSynchronize(P.st));
            int act = 0;
            for (auto& s : h) act += s.active;
            if (!act) break;
        }
        vcycle<VS>(P, LV, cn.sg, cn.B, pst, 0, rn, z);
        vlaunch(k_gc_rz<T, VS, false>, np * cn.sg.G, cn.B, cn.smem, P.st, cn.sg, np, pst, rn, z, redbuf(P));
        vlaunch(k_gc_p<T, VS, false>, np * cn.sg.G, cn.B, 0, P.st, cn.sg, np, pst, z, p);
    }
    vlaunch(k_gc_apply<T, VSD>, LV.nl * ce.sg.G, ce.B, 0, P.st, L, M, ce.sg, pst, phi, x);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h.data(), pst, sizeof(KState) * ns, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    int mx = 0;
    for (auto& s : h) mx = std::max(mx, s.iters);
    if (iters) *iters = mx;
    P.gc_calls++;
    P.gc_iters += mx;
    return SFDX_OK;
}

int nodal_setup(Plan& P, const Level& LV) {
    if (LV.gc_ok) return SFDX_OK;
    P.emg_epoch++;  // new stencil buffers: graphs that read the old ones are stale
    return gc_assemble(P, LV);
}

int grad_correct(Plan& P, const Level& LV, const double2* b, double2* x, const int* mask, double tol, int maxit,
                 int* iters) {
    switch (plan_vs<float>(P)) {
        case 4: return grad_correct_v<4>(P, LV, b, x, mask, tol, maxit, iters);
        case 2: return grad_correct_v<2>(P, LV, b, x, mask, tol, maxit, iters);
        default: return grad_correct_v<1>(P, LV, b, x, mask, tol, maxit, iters);
    }
}

}  // namespace sfdx
