// sfdx_blas.cuh -- batched BLAS-1 building blocks with per-system scalar
// finalisers, for the Krylov methods that have no fused kernels of their own:
// TFQMR (Freund 1993) and the two-sided BiCG with conjugate-transpose products
// (ptfqmr solvers.f90:317-519 and pbicg :878-1025 are broken as written; these
// follow the published algorithms).  Scalars live in the per-system KState and
// are updated on the device by the last block of each reducing kernel, so a
// solve issues launches only and the host checks convergence every 8
// iterations, as for the other solvers.
#pragma once
#include "sfdx_vkern.cuh"

namespace sfdx {

// ------------------------------------------------------------------ coefficients
// Per-system coefficient of a linear combination, read from KState.
enum BlCoef {
    BC_ZERO, BC_ONE, BC_MONE,
    BC_ALPHA, BC_MALPHA, BC_MCALPHA,  // alpha, -alpha, -conj(alpha)
    BC_BETA, BC_CBETA, BC_BETA2,      // beta, conj(beta), beta^2
    BC_ETA, BC_DC                     // eta, the TFQMR direction coefficient (rhoold)
};
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv2(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ bool cfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }

template <int C> __device__ __forceinline__ double2 bl_coef(const KState& S) {
    switch (C) {
        case BC_ONE: return make_double2(1.0, 0.0);
        case BC_MONE: return make_double2(-1.0, 0.0);
        case BC_ALPHA: return S.alpha;
        case BC_MALPHA: return make_double2(-S.alpha.x, -S.alpha.y);
        case BC_MCALPHA: return make_double2(-S.alpha.x, S.alpha.y);
        case BC_BETA: return S.beta;
        case BC_CBETA: return make_double2(S.beta.x, -S.beta.y);
        case BC_BETA2: return cmul2(S.beta, S.beta);
        case BC_ETA: return S.eta;
        case BC_DC: return S.rhoold;
        default: return make_double2(0.0, 0.0);
    }
}

// out = c0 v0 + c1 v1 + c2 v2 for the active systems (zero terms skipped; out
// may be one of the inputs: every element is read and written by one thread)
template <class T, int VS, int C0, int C1, int C2>
__global__ void k_bl_lincomb(Mesh M, SysG sgp, const KState* st, cplx<T>* out, const cplx<T>* v0, const cplx<T>* v1,
                             const cplx<T>* v2) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> c[3][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        c[0][u] = cst<T>(bl_coef<C0>(st[s0 + u]));
        c[1][u] = cst<T>(bl_coef<C1>(st[s0 + u]));
        c[2][u] = cst<T>(bl_coef<C2>(st[s0 + u]));
    }
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> o, a;
        cvzero<T, VS>(o);
        if (C0 != BC_ZERO) {
            cvldw<T, VS>(a, v0 + g);
#pragma unroll
            for (int u = 0; u < VS; u++) o.v[u] = o.v[u] + cmul<T>(c[0][u], a.v[u]);
        }
        if (C1 != BC_ZERO) {
            cvldw<T, VS>(a, v1 + g);
#pragma unroll
            for (int u = 0; u < VS; u++) o.v[u] = o.v[u] + cmul<T>(c[1][u], a.v[u]);
        }
        if (C2 != BC_ZERO) {
            cvldw<T, VS>(a, v2 + g);
#pragma unroll
            for (int u = 0; u < VS; u++) o.v[u] = o.v[u] + cmul<T>(c[2][u], a.v[u]);
        }
        cvst_m<T, VS>(out + g, o, S.act);
    }
}

// out = conj(in) * V^s per edge (s = -1 with INV, +1 otherwise; V the dual
// volume, 1 on the Dirichlet edges).  With V A V^-1 = A^T (complex symmetry
// of the volume-weighted rows) a conjugate-transpose product is
// A^H y = V conj(A (V^-1 conj(y))), and the same holds for the multi-colour
// symmetric Gauss-Seidel preconditioner.
template <class T, int VS, bool INV>
__global__ void k_bl_conj_vscale(Lev<T> L, Mesh M, SysG sgp, const KState* st, const cplx<T>* __restrict__ in,
                                 cplx<T>* __restrict__ out) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        const T vol = edge_vol<T>(L, M, o, i, j, k);
        const T f = INV ? T(1) / vol : vol;
        CV<T, VS> a;
        cvld<T, VS>(a, in + g);
#pragma unroll
        for (int u = 0; u < VS; u++) a.v[u] = mk<T>(f * a.v[u].x, -f * a.v[u].y);
        cvst_m<T, VS>(out + g, a, S.act);
    }
}

// ------------------------------------------------------------------ finalisers
enum BlFin { FIN_TFQ_INIT, FIN_TFQ_SIGMA, FIN_TFQ_RHO, FIN_BICG_INIT, FIN_BICG_RHO, FIN_BICG_ALPHA };

__device__ __forceinline__ void bl_break(KState& Q) {
    Q.active = 0;
    Q.status = ST_BREAK;
}

// d0 = sum conj(a0) b0, d1 = sum conj(a1) b1 of system ss
template <int FIN> __device__ __forceinline__ void bl_finalise(KState& Q, double2 d0, double2 d1) {
    if (FIN == FIN_TFQ_INIT) {  // rho = <rt, r>, tau = ||r||
        Q.rho = d0;
        Q.tau = make_double2(sqrt(d1.x), 0.0);
        Q.omega = make_double2(0.0, 0.0);  // theta
        Q.eta = make_double2(0.0, 0.0);
        Q.rhoold = make_double2(0.0, 0.0);  // direction coefficient
        Q.it = 0;
        Q.iters = 0;
        Q.pad[2] = 0;
        if (Q.err < Q.tol) {
            Q.active = 0;
            Q.status = ST_CONV;
        } else if (!(d0.x != 0.0 || d0.y != 0.0)) {
            bl_break(Q);
        }
    } else if (FIN == FIN_TFQ_SIGMA) {  // sigma = <rt, v>: alpha, and theta^2 eta / alpha
        Q.alpha = cdiv2(Q.rho, d0);
        const double th = Q.omega.x;
        Q.rhoold = cdiv2(make_double2(th * th * Q.eta.x, th * th * Q.eta.y), Q.alpha);
        if (!cfinite(Q.alpha) || !cfinite(Q.rhoold)) bl_break(Q);
    } else if (FIN == FIN_TFQ_RHO) {  // rho_new = <rt, w>: beta
        Q.beta = cdiv2(d0, Q.rho);
        Q.rho = d0;
        if (!cfinite(Q.beta)) bl_break(Q);
    } else if (FIN == FIN_BICG_INIT) {  // the initial residual may already meet the tolerance
        Q.iters = 0;
        Q.it = 0;
        if (Q.err < Q.tol) {
            Q.active = 0;
            Q.status = ST_CONV;
        }
    } else if (FIN == FIN_BICG_RHO) {  // rho = <rt, z>: beta (0 on the first iteration)
        Q.beta = Q.iters == 0 ? make_double2(0.0, 0.0) : cdiv2(d0, Q.rho);
        Q.rho = d0;
        if (!cfinite(Q.beta) || !(d0.x != 0.0 || d0.y != 0.0)) bl_break(Q);
    } else if (FIN == FIN_BICG_ALPHA) {  // alpha = rho / <pt, q>
        Q.alpha = cdiv2(Q.rho, d0);
        if (!cfinite(Q.alpha)) bl_break(Q);
    }
}

// per system: d0 = <a0, b0> (and d1 = <a1, b1> when a1 is given), then FIN
template <class T, int VS, int FIN>
__global__ void k_bl_dot(Mesh M, SysG sgp, KState* st, const cplx<T>* a0, const cplx<T>* b0, const cplx<T>* a1,
                         const cplx<T>* b1, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A r0[VS], i0[VS], r1[VS], i1[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) r0[u] = i0[u] = r1[u] = i1[u] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> a, b;
            cvld<T, VS>(a, a0 + g);
            cvld<T, VS>(b, b0 + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                const cplx<T> z = cdot<T>(a.v[u], b.v[u]);
                r0[u] += z.x;
                i0[u] += z.y;
            }
            if (a1) {
                cvld<T, VS>(a, a1 + g);
                cvld<T, VS>(b, b1 + g);
#pragma unroll
                for (int u = 0; u < VS; u++) {
                    const cplx<T> z = cdot<T>(a.v[u], b.v[u]);
                    r1[u] += z.x;
                    i1[u] += z.y;
                }
            }
        }
    double2 acc[2][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        acc[0][u] = make_double2(r0[u], i0[u]);
        acc[1][u] = make_double2(r1[u], i1[u]);
    }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        bl_finalise<FIN>(Q, smem[B + ss], smem[B + ns + ss]);
    }
}

// ------------------------------------------------------------------ TFQMR
// One half-step of the quasi-minimisation: w -= alpha aw, d = dsrc + dc d,
// then theta = ||w|| / tau, c = (1 + theta^2)^-1/2, tau *= theta c,
// eta = c^2 alpha, the next direction coefficient theta^2 eta / alpha, and the
// residual bound tau sqrt(m+1) >= ||r_m|| as the convergence test.  A system
// that meets the tolerance (or the iteration limit) stops after the x update
// that follows (k_bl_commit).
template <class T, int VS>
__global__ void k_tfq_half(Mesh M, SysG sgp, KState* st, cplx<T>* w, const cplx<T>* __restrict__ aw, cplx<T>* d,
                           const cplx<T>* __restrict__ dsrc, RedBuf rb, double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    cplx<T> ma[VS], dc[VS];
    A nn[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        ma[u] = cst<T>(bl_coef<BC_MALPHA>(st[s0 + u]));
        dc[u] = cst<T>(bl_coef<BC_DC>(st[s0 + u]));
        nn[u] = 0;
    }
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> wv, av, dv, sv;
            cvldw<T, VS>(wv, w + g);
            cvld<T, VS>(av, aw + g);
            cvldw<T, VS>(dv, d + g);
            cvld<T, VS>(sv, dsrc + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                wv.v[u] = wv.v[u] + cmul<T>(ma[u], av.v[u]);
                dv.v[u] = sv.v[u] + cmul<T>(dc[u], dv.v[u]);
                nn[u] += (A)cabs2<T>(wv.v[u]);
            }
            cvst_m<T, VS>(w + g, wv, S.act);
            cvst_m<T, VS>(d + g, dv, S.act);
        }
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(nn[u], 0.0);
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        const double th = sqrt(smem[B + ss].x) / Q.tau.x;
        const double c = 1.0 / sqrt(1.0 + th * th);
        Q.tau.x = Q.tau.x * th * c;
        Q.omega = make_double2(th, 0.0);
        Q.eta = make_double2(c * c * Q.alpha.x, c * c * Q.alpha.y);
        Q.rhoold = cdiv2(make_double2(th * th * Q.eta.x, th * th * Q.eta.y), Q.alpha);
        Q.it += 1;
        Q.iters = (Q.it + 1) / 2;
        Q.err = Q.tau.x * sqrt((double)Q.it + 1.0) / Q.babs;
        if (err_rec && Q.iters < Q.itmax) err_rec[(size_t)ss * err_stride + Q.iters] = Q.err;
        if (!isfinite(Q.err) || !cfinite(Q.rhoold)) {
            bl_break(Q);
            Q.status = ST_NAN;
        } else if (Q.err < Q.tol) {
            Q.pad[2] = 1;
        } else if (Q.iters >= Q.itmax && (Q.it & 1) == 0) {
            Q.pad[2] = 2;
        }
    }
}

// systems whose last half-step met the test stop now (their x is updated)
static __global__ void k_bl_commit(KState* st, int ns) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    KState& Q = st[s];
    if (Q.active && Q.pad[2]) {
        Q.status = Q.pad[2] == 1 ? ST_CONV : ST_MAXIT;
        Q.active = 0;
        Q.pad[2] = 0;
    }
}

// ------------------------------------------------------------------ BiCG
// x += alpha p, r -= alpha q, rt -= conj(alpha) qt, then ||r|| / ||b|| as the
// convergence test (iteration count advanced here)
template <class T, int VS>
__global__ void k_bicg2_upd(Mesh M, SysG sgp, KState* st, cplx<T>* x, cplx<T>* r, cplx<T>* rt,
                            const cplx<T>* __restrict__ p, const cplx<T>* __restrict__ q, const cplx<T>* __restrict__ qt,
                            RedBuf rb, double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    cplx<T> al[VS], mal[VS], mcal[VS];
    A nn[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        al[u] = cst<T>(bl_coef<BC_ALPHA>(st[s0 + u]));
        mal[u] = cst<T>(bl_coef<BC_MALPHA>(st[s0 + u]));
        mcal[u] = cst<T>(bl_coef<BC_MCALPHA>(st[s0 + u]));
        nn[u] = 0;
    }
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> xv, rv, tv, pv, qv, uv;
            cvldw<T, VS>(xv, x + g);
            cvldw<T, VS>(rv, r + g);
            cvldw<T, VS>(tv, rt + g);
            cvld<T, VS>(pv, p + g);
            cvld<T, VS>(qv, q + g);
            cvld<T, VS>(uv, qt + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                xv.v[u] = xv.v[u] + cmul<T>(al[u], pv.v[u]);
                rv.v[u] = rv.v[u] + cmul<T>(mal[u], qv.v[u]);
                tv.v[u] = tv.v[u] + cmul<T>(mcal[u], uv.v[u]);
                nn[u] += (A)cabs2<T>(rv.v[u]);
            }
            cvst_m<T, VS>(x + g, xv, S.act);
            cvst_m<T, VS>(r + g, rv, S.act);
            cvst_m<T, VS>(rt + g, tv, S.act);
        }
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(nn[u], 0.0);
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        Q.iters += 1;
        Q.it += 1;
        Q.err = sqrt(smem[B + ss].x) / Q.babs;
        if (err_rec && Q.iters < Q.itmax) err_rec[(size_t)ss * err_stride + Q.iters] = Q.err;
        if (!isfinite(Q.err)) {
            Q.active = 0;
            Q.status = ST_NAN;
        } else if (Q.err < Q.tol) {
            Q.active = 0;
            Q.status = ST_CONV;
        } else if (Q.iters >= Q.itmax) {
            Q.active = 0;
            Q.status = ST_MAXIT;
        }
    }
}

}  // namespace sfdx
