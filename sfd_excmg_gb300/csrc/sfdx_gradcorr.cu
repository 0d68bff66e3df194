// sfdx_gradcorr.cu -- host driver of the consistent gradient-space correction
// (kernels and derivation in sfdx_gradcorr.cuh).
#include "sfdx_gradcorr.cuh"
#include "sfdx_plan.h"

namespace sfdx {

// Assemble N = G^T V Ms G of level LV as a 27-point nodal stencil (float
// coefficients + inverse diagonal) by probing; cached until the conductivity
// of the level changes.
static int gc_assemble(Plan& P, const Level& LV) {
    const Mesh& M = LV.mesh;
    const Lev<double> L = LV.lev<double>();
    const uint32_t np = (uint32_t)(LV.nx + 1) * (LV.ny + 1) * (LV.nz + 1);
    const int NPR = 27;
    RC(LV.gc_coef.alloc((size_t)27 * np * sizeof(float)));
    RC(LV.gc_dinv.alloc((size_t)np * sizeof(float)));
    RC(P.gcn[0].alloc((size_t)np * NPR * sizeof(double2)));  // probes
    RC(P.gcn[1].alloc((size_t)np * NPR * sizeof(double2)));  // responses
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
    double2 *pr = P.gcn[0].as<double2>(), *Q = P.gcn[1].as<double2>();
    double2 *ge = P.gce[0].as<double2>(), *u = P.gce[1].as<double2>();
    KL(k_gc_probe<<<grid_for((int64_t)np * NPR, 256, 16), 256, 0, P.st>>>(M, np, pr));
    vlaunch(k_gc_grad<1>, LV.nl * sg.G, B, 0, P.st, L, M, sg, pst, pr, ge);
    vlaunch(k_gc_mass<1>, LV.nl * sg.G, B, 0, P.st, L, M, sg, pst, ge, u);
    vlaunch(k_gc_gtu<1>, np * sg.G, B, 0, P.st, L, M, sg, np, u, Q);
    KL(k_gc_assemble<<<grid_for(np, 256, 16), 256, 0, P.st>>>(M, np, Q, LV.gc_coef.as<float>(), LV.gc_dinv.as<float>()));
    CK(cudaGetLastError());
    LV.gc_ok = true;
    return SFDX_OK;
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
    if (!LV.gc_ok) RC(gc_assemble(P, LV));
    const size_t nb = (size_t)np * ns * sizeof(cplx<T>), eb = (size_t)LV.nl * ns * sizeof(double2);
    for (int q = 0; q < 5; q++) RC(P.gcn[q].alloc(nb));
    RC(P.r64.alloc(eb));
    RC(P.d_pst.alloc(sizeof(KState) * std::max(ns, 27)));
    cplx<T> *phi = P.gcn[0].as<cplx<T>>(), *rn = P.gcn[1].as<cplx<T>>(), *z = P.gcn[2].as<cplx<T>>();
    cplx<T> *p = P.gcn[3].as<cplx<T>>(), *q = P.gcn[4].as<cplx<T>>();
    double2* re = P.r64.as<double2>();
    const float* coef = LV.gc_coef.as<float>();
    const float* dinv = LV.gc_dinv.as<float>();
    KState* pst = P.d_pst.as<KState>();
    CK(cudaMemcpyAsync(pst, init.data(), sizeof(KState) * ns, cudaMemcpyHostToDevice, P.st));
    constexpr int VSD = VS > 2 ? 2 : VS;  // systems per thread of the FP64 edge kernels
    const VCfg ce = vcfg(P, LV.nl, 2, VSD);
    const VCfg cnd = vcfg(P, np, 2, VSD);
    const VCfg cn = vcfg(P, np, 2, VS);
    RC(P.d_part.alloc(std::max(P.d_part.bytes, (size_t)max_resident_blocks() * 2 * ns * sizeof(double2))));
    // r = b - A x (FP64), then the nodal right-hand side and the PCG start
    vlaunch(k_residual_v<double, double, VSD, 2>, LV.nl * ce.sg.G, ce.B, ce.smem, P.st, L, M, ce.sg, pst, b, x, re, nullptr, redbuf(P), nullptr, 0);
    vlaunch(k_gc_rhs<T, VSD>, np * cnd.sg.G, cnd.B, cnd.smem, P.st, L, M, cnd.sg, np, pst, re, dinv, rn, z, p, phi, redbuf(P));
    CK(cudaGetLastError());
    std::vector<KState> h(ns);
    for (int it = 0; it < maxit; it++) {
        vlaunch(k_gc_Ap<T, VS>, np * cn.sg.G, cn.B, cn.smem, P.st, M, cn.sg, np, pst, coef, p, q, redbuf(P));
        vlaunch(k_gc_upd<T, VS>, np * cn.sg.G, cn.B, cn.smem, P.st, cn.sg, np, pst, dinv, p, q, phi, rn, z, redbuf(P));
        vlaunch(k_gc_p<T, VS>, np * cn.sg.G, cn.B, 0, P.st, cn.sg, np, pst, z, p);
        if ((it + 1) % 16 == 0) {
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(h.data(), pst, sizeof(KState) * ns, cudaMemcpyDeviceToHost, P.st));
            CK(cudaStreamSynchronize(P.st));
            int act = 0;
            for (auto& s : h) act += s.active;
            if (!act) break;
        }
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

int grad_correct(Plan& P, const Level& LV, const double2* b, double2* x, const int* mask, double tol, int maxit,
                 int* iters) {
    switch (plan_vs<float>(P)) {
        case 4: return grad_correct_v<4>(P, LV, b, x, mask, tol, maxit, iters);
        case 2: return grad_correct_v<2>(P, LV, b, x, mask, tol, maxit, iters);
        default: return grad_correct_v<1>(P, LV, b, x, mask, tol, maxit, iters);
    }
}

}  // namespace sfdx
