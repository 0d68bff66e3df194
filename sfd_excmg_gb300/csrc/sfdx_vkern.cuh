// sfdx_vkern.cuh -- hot kernels of the Krylov solves in the system-group
// mapping of sfdx_stencil.cuh: operator, multi-colour SSOR sweeps, and the
// fused vector updates / inner products of BiCGStab (solvers.f90:522-719)
// and GPBiCG (solvers.f90:137-315).  Every kernel takes the template VS (systems per
// thread); the host picks VS = 4, 2 or 1 from the batch size.
#pragma once
#include "sfdx_kernels.cuh"
#include "sfdx_stencil.cuh"

namespace sfdx {

// per-thread system scalars
template <class T, int VS> struct SysV {
    unsigned act;  // bit v: system s0+v active
    T wm[VS];
};
template <class T, int VS> __device__ __forceinline__ SysV<T, VS> load_sys(const KState* st, int s0) {
    SysV<T, VS> S;
    S.act = 0;
#pragma unroll
    for (int v = 0; v < VS; v++) {
        S.act |= (st[s0 + v].active ? 1u : 0u) << v;
        S.wm[v] = (T)st[s0 + v].wm;
    }
    return S;
}
template <class T> __device__ __forceinline__ cplx<T> cst(const double2 z) { return mk<T>((T)z.x, (T)z.y); }

// ------------------------------------------------------------------ reduction
// acc[q][v] of each thread (systems s0+v) -> per-block partials part[block][q][ns];
// the last block sums the partials of every slot in a fixed order and leaves the
// totals at sm[blockDim + q*ns + s].  Shared memory: vred_smem_bytes() bytes.
// sum of p[b * pitch] for b = b0, b0 + step, ... < nb, in a fixed order with
// eight independent accumulators, so that eight L2 loads are in flight
__device__ __forceinline__ double2 sum_partials(const double2* p, size_t pitch, int b0, int step, int nb) {
    double2 a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = make_double2(0.0, 0.0);
    int b = b0;
    for (; b + 7 * step < nb; b += 8 * step) {
#pragma unroll
        for (int j = 0; j < 8; j++) a[j] = a[j] + __ldcg(p + (size_t)(b + j * step) * pitch);
    }
    for (int j = 0; b < nb; b += step, j++) a[j] = a[j] + __ldcg(p + (size_t)b * pitch);
    return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
}

template <int NQ, int VS>
__device__ __forceinline__ bool vreduce_last(double2 (&acc)[NQ][VS], const SysG& sgp, RedBuf rb, double2* sm) {
    const int t = threadIdx.x, B = blockDim.x, G = sgp.G, ns = sgp.ns;
    if ((G & (G - 1)) == 0 && G <= 32) {
        const int lane = t & 31, warp = t >> 5, nw = B >> 5;
#pragma unroll
        for (int q = 0; q < NQ; q++)
#pragma unroll
            for (int v = 0; v < VS; v++) {
                double2 a = acc[q][v];
                for (int off = 16; off >= G; off >>= 1) {
                    a.x += __shfl_xor_sync(0xffffffffu, a.x, off);
                    a.y += __shfl_xor_sync(0xffffffffu, a.y, off);
                }
                if (lane < G) sm[((size_t)warp * NQ + q) * ns + lane * VS + v] = a;
            }
        __syncthreads();
        for (int slot = t; slot < NQ * ns; slot += B) {
            const int q = slot / ns, s = slot - q * ns;
            double2 r = make_double2(0.0, 0.0);
            for (int w = 0; w < nw; w++) r = r + sm[((size_t)w * NQ + q) * ns + s];
            rb.part[((size_t)blockIdx.x * NQ + q) * ns + s] = r;
        }
    } else {
#pragma unroll
        for (int q = 0; q < NQ; q++)
#pragma unroll
            for (int v = 0; v < VS; v++) {
                sm[t] = acc[q][v];
                __syncthreads();
                for (int stride = B >> 1; stride >= G; stride >>= 1) {
                    if (t < stride) sm[t] = sm[t] + sm[t + stride];
                    __syncthreads();
                }
                if (t < G) rb.part[((size_t)blockIdx.x * NQ + q) * ns + t * VS + v] = sm[t];
                __syncthreads();
            }
    }
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (t == 0) {
        unsigned int prev = atomicAdd(rb.counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    const int slots = NQ * ns;
    if (slots * 2 > B) {  // one thread per slot, blocks summed in order
        __syncthreads();
        for (int slot = t; slot < slots; slot += B) {
            const int q = slot / ns, s = slot - q * ns;
            sm[B + slot] = sum_partials(rb.part + (size_t)q * ns + s, (size_t)NQ * ns, 0, 1, (int)gridDim.x);
        }
    } else {  // `per` threads per slot, each a fixed stride of blocks
        const int per = B / slots;
        const int slot = t / per, ln = t - slot * per;
        double2 a = make_double2(0.0, 0.0);
        if (slot < slots) {
            const int q = slot / ns, s = slot - q * ns;
            a = sum_partials(rb.part + (size_t)q * ns + s, (size_t)NQ * ns, ln, per, (int)gridDim.x);
        }
        __syncthreads();
        sm[t] = a;
        __syncthreads();
        double2 r = make_double2(0.0, 0.0);
        if (slot < slots && ln == 0)
            for (int l = 0; l < per; l++) r = r + sm[t + l];
        __syncthreads();
        if (slot < slots && ln == 0) sm[B + slot] = r;
    }
    if (t == 0) *rb.counter = 0u;
    __syncthreads();
    return true;
}

#define SFDX_GRID_LOOP(t, W) \
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < (W); t += gridDim.x * blockDim.x)

// ------------------------------------------------------------------ operator
template <class T, int VS>
__global__ void k_apply_v(Lev<T> L, Mesh M, SysG sgp, const double* wms, const cplx<T>* __restrict__ x,
                          cplx<T>* __restrict__ y) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    T wm[VS];
#pragma unroll
    for (int v = 0; v < VS; v++) wm[v] = (T)wms[s0 + v];
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        uint32_t e;
        int i, j, k;
        const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> xe, val;
        cvld<T, VS>(xe, x + g);
        row_apply<T, VS>(L, M, o, e, i, j, k, x, ns, s0, wm, xe, val);
        cvst<T, VS>(y + g, val);
    }
}

// ------------------------------------------------------------------ multi-colour SSOR
// Forward sweep of colour (O,P):  w_e = (rhs_e - sum_{earlier colours} K_en w_n) / D_e,
// rhs from MODE (RHS_PUPD: p = r + beta (p - omega v) stored in q; RHS_SUPD:
// s = r - alpha v stored in q; RHS_VEC: q; RHS_COCR: q = r + beta q stored in
// q (the operator image of the new search direction) and aux = v + beta aux
// (the search direction itself), rhs = q).
template <class T, int VS, int O, int P, int MODE>
__global__ void k_fwd_v(Lev<T> L, Mesh M, SysG sgp, const KState* st, cplx<T>* __restrict__ w, cplx<T>* __restrict__ q,
                        const cplx<T>* __restrict__ r, const cplx<T>* __restrict__ v, cplx<T>* __restrict__ aux,
                        T omega) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> c1[VS], c2[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        if (MODE == RHS_PUPD) {
            c1[u] = cst<T>(st[s0 + u].beta);
            c2[u] = cst<T>(st[s0 + u].omega);
        } else if (MODE == RHS_SUPD) {
            c1[u] = cst<T>(st[s0 + u].alpha);
        } else if (MODE == RHS_COCR) {
            c1[u] = cst<T>(st[s0 + u].beta);
        }
    }
    SFDX_GRID_LOOP(t, mcolour_count(M, O) * sgp.G) {
        int i, j, k;
        if (!mcolour<O>(M, P, fdiv(sgp.fG, t), i, j, k)) continue;
        const uint32_t e = medge(M, O, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> rhs;
        if (MODE == RHS_PUPD) {
            CV<T, VS> rr, qq, vv;
            cvld<T, VS>(rr, r + g);
            cvldw<T, VS>(qq, q + g);
            cvld<T, VS>(vv, v + g);
#pragma unroll
            for (int u = 0; u < VS; u++) rhs.v[u] = rr.v[u] + cmul<T>(c1[u], qq.v[u] - cmul<T>(c2[u], vv.v[u]));
            cvst_m<T, VS>(q + g, rhs, S.act);
        } else if (MODE == RHS_SUPD) {
            CV<T, VS> rr, vv;
            cvld<T, VS>(rr, r + g);
            cvld<T, VS>(vv, v + g);
#pragma unroll
            for (int u = 0; u < VS; u++) rhs.v[u] = rr.v[u] - cmul<T>(c1[u], vv.v[u]);
            cvst_m<T, VS>(q + g, rhs, S.act);
        } else if (MODE == RHS_COCR) {
            CV<T, VS> uu, qq, zz, pp;
            cvld<T, VS>(uu, r + g);
            cvldw<T, VS>(qq, q + g);
            cvld<T, VS>(zz, v + g);
            cvldw<T, VS>(pp, aux + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                rhs.v[u] = uu.v[u] + cmul<T>(c1[u], qq.v[u]);
                pp.v[u] = zz.v[u] + cmul<T>(c1[u], pp.v[u]);
            }
            cvst_m<T, VS>(q + g, rhs, S.act);
            cvst_m<T, VS>(aux + g, pp, S.act);
        } else {
            cvld<T, VS>(rhs, q + g);
        }
        if (mbnd(M, O, i, j, k)) {
            cvst_m<T, VS>(w + g, rhs, S.act);
            continue;
        }
        const RowK<T> K = row_k_e<T, O, P == 1, (O >= OY), (O == OZ)>(L, e, i, j, k);
        const RowN N = row_n<O>(M, e, i, j, k);
        CV<T, VS> C, Mm, out;
        row_off<T, VS, O, P == 1, (O >= OY), (O == OZ), true>(K, N, w, ns, s0, C, Mm);
#pragma unroll
        for (int u = 0; u < VS; u++) {
            const cplx<T> cm = cm_combine<T>(C.v[u], Mm.v[u], S.wm[u]);
            out.v[u] = cdiv<T>(rhs.v[u] - mk<T>(omega * cm.x, omega * cm.y), row_dia<T>(K, S.wm[u]));
        }
        cvst_m<T, VS>(w + g, out, S.act);
    }
}

// Backward sweep of colour (O,P), in place:  x_e -= omega D_e^{-1} sum_{later colours} K_en x_n.
// With the forward sweep's w_e = (rhs_e - omega sum_{earlier} K_en w_n) / D_e this
// applies M^-1 for M = (D + omega L) D^-1 (D + omega U), the SSOR preconditioner
// up to the constant factor omega (2 - omega) that Krylov methods do not see.
template <class T, int VS, int O, int P>
__global__ void k_bwd_v(Lev<T> L, Mesh M, SysG sgp, const KState* st, cplx<T>* __restrict__ x, T omega) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, mcolour_count(M, O) * sgp.G) {
        int i, j, k;
        if (!mcolour<O>(M, P, fdiv(sgp.fG, t), i, j, k)) continue;
        if (mbnd(M, O, i, j, k)) continue;
        const uint32_t e = medge(M, O, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        const RowK<T> K = row_k_e<T, O, P == 0, (O == OX), (O <= OY)>(L, e, i, j, k);
        const RowN N = row_n<O>(M, e, i, j, k);
        CV<T, VS> C, Mm, xe;
        row_off<T, VS, O, P == 0, (O == OX), (O <= OY), true>(K, N, x, ns, s0, C, Mm);
        cvldw<T, VS>(xe, x + g);
#pragma unroll
        for (int u = 0; u < VS; u++) {
            const cplx<T> cm = cm_combine<T>(C.v[u], Mm.v[u], S.wm[u]);
            xe.v[u] = xe.v[u] - cdiv<T>(mk<T>(omega * cm.x, omega * cm.y), row_dia<T>(K, S.wm[u]));
        }
        cvst_m<T, VS>(x + g, xe, S.act);
    }
}

// ------------------------------------------------------------------ residual
// r = b - A x (x, b in XT; r, rhat in T).  MODE as k_residual (sfdx_kernels.cuh):
// 0 BiCGStab start, 1 BiCGStab restart, 2 absolute residual, 3 GPBiCG start,
// 4 residual restart only.
template <class T, class XT, int VS, int MODE>
__global__ void k_residual_v(Lev<XT> L, Mesh M, SysG sgp, KState* st, const cplx<XT>* __restrict__ bvec,
                             const cplx<XT>* __restrict__ x, cplx<T>* __restrict__ r, cplx<T>* __restrict__ rhat, RedBuf rb,
                             double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<XT, VS> S = load_sys<XT, VS>(st, s0);
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(0.0, 0.0);
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<XT, VS> xe, ax, bv;
            cvld<XT, VS>(xe, x + g);
            row_apply<XT, VS>(L, M, o, e, i, j, k, x, ns, s0, S.wm, xe, ax);
            cvld<XT, VS>(bv, bvec + g);
            CV<T, VS> rt;
#pragma unroll
            for (int u = 0; u < VS; u++) {
                cplx<XT> rv = bv.v[u] - ax.v[u];
                rt.v[u] = mk<T>((T)rv.x, (T)rv.y);
                acc[0][u].x += (double)cabs2<XT>(rv);
                acc[0][u].y += (double)cabs2<XT>(bv.v[u]);
            }
            cvst_m<T, VS>(r + g, rt, S.act);
            if (rhat) cvst_m<T, VS>(rhat + g, rt, S.act);
        }
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        double2 v = smem[B + ss];
        double nr = sqrt(v.x);
        if (MODE == 0) {
            Q.babs = sqrt(v.y);
            Q.err = nr / Q.babs;
            Q.errv = Q.err;
            Q.rho = make_double2(1.0, 0.0);
            Q.alpha = make_double2(1.0, 0.0);
            Q.omega = make_double2(1.0, 0.0);
            Q.it = 1;
            Q.iters = 1;
            if (err_rec) err_rec[(size_t)ss * err_stride] = Q.err;
            if (isnan(Q.err)) {  // solvers.f90:619
                Q.status = ST_NAN;
                Q.active = 0;
                Q.iters = 0;
                continue;
            }
            if (Q.err < Q.tol) {
                Q.status = ST_CONV;
                Q.active = 0;
                continue;
            }
            Q.rhoold = Q.rho;
            Q.rho = make_double2(v.x, 0.0);  // rhat == r
            Q.beta = Q.rho;
        } else if (MODE == 1) {
            Q.rho = make_double2(v.x, 0.0);
            double2 a = Q.rho, b = Q.rhoold, al2 = Q.alpha, om2 = Q.omega;
            double bd = b.x * b.x + b.y * b.y, od = om2.x * om2.x + om2.y * om2.y;
            double2 q1 = make_double2((a.x * b.x + a.y * b.y) / bd, (a.y * b.x - a.x * b.y) / bd);
            double2 q2 = make_double2((al2.x * om2.x + al2.y * om2.y) / od, (al2.y * om2.x - al2.x * om2.y) / od);
            Q.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        } else if (MODE == 2) {
            Q.err = nr;
            Q.babs = sqrt(v.y);
        } else if (MODE == 3) {  // GPBiCG start (solvers.f90:203-221)
            Q.babs = sqrt(v.y);
            Q.err = nr / Q.babs;
            Q.errv = Q.err;
            Q.it = 1;
            Q.iters = 0;
            Q.beta = make_double2(0.0, 0.0);
            if (isnan(Q.err)) {
                Q.status = ST_NAN;
                Q.active = 0;
            }
        }
    }
}

// ------------------------------------------------------------------ BiCGStab
// v = A y ; alpha = rho / <rhat, v>
template <class T, int VS>
__global__ void k_bicg_v_v(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ y, cplx<T>* __restrict__ v,
                           const cplx<T>* __restrict__ rhat, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A ar[VS], ai[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) ar[u] = ai[u] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<T, VS> ye, val, h;
            cvld<T, VS>(ye, y + g);
            row_apply<T, VS>(L, M, o, e, i, j, k, y, ns, s0, S.wm, ye, val);
            cvst_m<T, VS>(v + g, val, S.act);
            cvld<T, VS>(h, rhat + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                cplx<T> d = cdot<T>(h.v[u], val.v[u]);
                ar[u] += d.x;
                ai[u] += d.y;
            }
        }
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(ar[u], ai[u]);
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        if (!st[ss].active) continue;
        double2 d = smem[B + ss];
        double2 rho = st[ss].rho;
        double den = d.x * d.x + d.y * d.y;
        st[ss].alpha = make_double2((rho.x * d.x + rho.y * d.y) / den, (rho.y * d.x - rho.x * d.y) / den);
        if (!isfinite(st[ss].alpha.x) || !isfinite(st[ss].alpha.y)) {  // breakdown: keep the last iterate
            st[ss].active = 0;
            st[ss].status = ST_BREAK;
        }
    }
}

// t = A z ; omega = <t,s>/<t,t>
template <class T, int VS>
__global__ void k_bicg_t_v(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ z, cplx<T>* __restrict__ tv,
                           const cplx<T>* __restrict__ sv, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A a0r[VS], a0i[VS], a1[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) a0r[u] = a0i[u] = a1[u] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<T, VS> ze, val, ss;
            cvld<T, VS>(ze, z + g);
            row_apply<T, VS>(L, M, o, e, i, j, k, z, ns, s0, S.wm, ze, val);
            cvst_m<T, VS>(tv + g, val, S.act);
            cvld<T, VS>(ss, sv + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                cplx<T> d = cdot<T>(val.v[u], ss.v[u]);
                a0r[u] += d.x;
                a0i[u] += d.y;
                a1[u] += cabs2<T>(val.v[u]);
            }
        }
    double2 acc[2][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        acc[0][u] = make_double2(a0r[u], a0i[u]);
        acc[1][u] = make_double2(a1[u], 0.0);
    }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        if (!st[ss].active) continue;
        double2 ts = smem[B + ss];
        double tt = smem[B + ns + ss].x;
        st[ss].omega = make_double2(ts.x / tt, ts.y / tt);
        if (!isfinite(st[ss].omega.x) || !isfinite(st[ss].omega.y) || (st[ss].omega.x == 0.0 && st[ss].omega.y == 0.0)) {
            st[ss].active = 0;
            st[ss].status = ST_BREAK;
        }
    }
}

// x += alpha y + omega z ; r = s - omega t ; err = |r|/|b| ; rho, beta of the
// next iteration, stopping tests (solvers.f90:655-685)
template <class T, class XT, int VS>
__global__ void k_bicg_upd_v(Mesh M, SysG sgp, KState* st, cplx<XT>* __restrict__ x, const cplx<T>* __restrict__ y,
                             const cplx<T>* __restrict__ z, const cplx<T>* __restrict__ sv, const cplx<T>* __restrict__ tv,
                             cplx<T>* __restrict__ r, const cplx<T>* __restrict__ rhat, RedBuf rb, double* err_rec,
                             int err_stride) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    cplx<T> om[VS];
    cplx<XT> alx[VS], omx[VS];
    A rr[VS], hr[VS], hi[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        om[u] = cst<T>(st[s0 + u].omega);
        alx[u] = cst<XT>(st[s0 + u].alpha);
        omx[u] = cst<XT>(st[s0 + u].omega);
        rr[u] = hr[u] = hi[u] = 0;
    }
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> yy, zz, s_, t_, h;
            CV<XT, VS> xx;
            cvld<T, VS>(yy, y + g);
            cvld<T, VS>(zz, z + g);
            cvldw<XT, VS>(xx, x + g);
            cvld<T, VS>(s_, sv + g);
            cvld<T, VS>(t_, tv + g);
            cvld<T, VS>(h, rhat + g);
            CV<T, VS> rn;
#pragma unroll
            for (int u = 0; u < VS; u++) {
                cplx<XT> y2 = mk<XT>((XT)yy.v[u].x, (XT)yy.v[u].y), z2 = mk<XT>((XT)zz.v[u].x, (XT)zz.v[u].y);
                xx.v[u] = xx.v[u] + cmul<XT>(alx[u], y2) + cmul<XT>(omx[u], z2);
                rn.v[u] = s_.v[u] - cmul<T>(om[u], t_.v[u]);
                rr[u] += cabs2<T>(rn.v[u]);
                cplx<T> d = cdot<T>(h.v[u], rn.v[u]);
                hr[u] += d.x;
                hi[u] += d.y;
            }
            cvst_m<XT, VS>(x + g, xx, S.act);
            cvst_m<T, VS>(r + g, rn, S.act);
        }
    double2 acc[2][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        acc[0][u] = make_double2(rr[u], 0.0);
        acc[1][u] = make_double2(hr[u], hi[u]);
    }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        double nr = sqrt(smem[B + ss].x);
        double2 rh = smem[B + ns + ss];
        Q.err = nr / Q.babs;
        Q.it += 1;
        if (err_rec && Q.it <= Q.itmax) err_rec[(size_t)ss * err_stride + Q.it - 1] = Q.err;
        // scalars of the next iteration first: a system stopped below may be
        // resumed (mixed precision re-check) and must continue consistently
        Q.rhoold = Q.rho;
        Q.rho = rh;
        double2 a = Q.rho, b = Q.rhoold, al2 = Q.alpha, om2 = Q.omega;
        double bd = b.x * b.x + b.y * b.y, od = om2.x * om2.x + om2.y * om2.y;
        double2 q1 = make_double2((a.x * b.x + a.y * b.y) / bd, (a.y * b.x - a.x * b.y) / bd);
        double2 q2 = make_double2((al2.x * om2.x + al2.y * om2.y) / od, (al2.y * om2.x - al2.x * om2.y) / od);
        Q.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        if (isnan(Q.err)) {  // solvers.f90:683
            Q.status = ST_NAN;
            Q.active = 0;
            Q.iters = Q.it - 1;
            continue;
        }
        if (Q.it > Q.itmax) {
            Q.status = ST_MAXIT;
            Q.active = 0;
            Q.iters = Q.itmax;
            continue;
        }
        Q.iters = Q.it;
        if (Q.err < Q.tol) {  // solvers.f90:625
            Q.status = ST_CONV;
            Q.active = 0;
            continue;
        }
    }
}

// ------------------------------------------------------------------ GPBiCG
// ap = A p ; alpha = <r0, r> / <r0, ap>
template <class T, int VS>
__global__ void k_gp_ap_v(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ p, cplx<T>* __restrict__ ap,
                          const cplx<T>* __restrict__ r0, const cplx<T>* __restrict__ r, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A a0r[VS], a0i[VS], a1r[VS], a1i[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) a0r[u] = a0i[u] = a1r[u] = a1i[u] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<T, VS> pe, val, q0, rr;
            cvld<T, VS>(pe, p + g);
            row_apply<T, VS>(L, M, o, e, i, j, k, p, ns, s0, S.wm, pe, val);
            cvst_m<T, VS>(ap + g, val, S.act);
            cvld<T, VS>(q0, r0 + g);
            cvld<T, VS>(rr, r + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                cplx<T> d0 = cdot<T>(q0.v[u], val.v[u]), d1 = cdot<T>(q0.v[u], rr.v[u]);
                a0r[u] += d0.x; a0i[u] += d0.y; a1r[u] += d1.x; a1i[u] += d1.y;
            }
        }
    double2 acc[2][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        acc[0][u] = make_double2(a0r[u], a0i[u]);
        acc[1][u] = make_double2(a1r[u], a1i[u]);
    }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        double2 d = smem[B + ss], n = smem[B + ns + ss];
        double den = d.x * d.x + d.y * d.y;
        Q.rho = n;  // <r0, r>, the "rold" inner product of the beta update
        Q.alpha = make_double2((n.x * d.x + n.y * d.y) / den, (n.y * d.x - n.x * d.y) / den);
        if (!isfinite(Q.alpha.x) || !isfinite(Q.alpha.y)) {
            Q.active = 0;
            Q.status = ST_BREAK;
        }
    }
}

// y = t - r - alpha w + alpha ap ; t = r - alpha ap
template <class T, int VS>
__global__ void k_gp_yt_v(Mesh M, SysG sgp, const KState* st, cplx<T>* __restrict__ y, cplx<T>* __restrict__ tv,
                          const cplx<T>* __restrict__ r, const cplx<T>* __restrict__ w, const cplx<T>* __restrict__ ap) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> al[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) al[u] = cst<T>(st[s0 + u].alpha);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> tt, rr, ww, aa, yn;
        cvldw<T, VS>(tt, tv + g);
        cvld<T, VS>(rr, r + g);
        cvld<T, VS>(ww, w + g);
        cvld<T, VS>(aa, ap + g);
#pragma unroll
        for (int u = 0; u < VS; u++) {
            cplx<T> aap = cmul<T>(al[u], aa.v[u]);
            yn.v[u] = (tt.v[u] - rr.v[u]) - cmul<T>(al[u], ww.v[u]) + aap;
            tt.v[u] = rr.v[u] - aap;
        }
        cvst_m<T, VS>(y + g, yn, S.act);
        cvst_m<T, VS>(tv + g, tt, S.act);
    }
}

// tp = rp - alpha tmp
template <class T, int VS>
__global__ void k_gp_tp_v(Mesh M, SysG sgp, const KState* st, cplx<T>* __restrict__ tp, const cplx<T>* __restrict__ rp,
                          const cplx<T>* __restrict__ tmp) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> al[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) al[u] = cst<T>(st[s0 + u].alpha);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> a, b, o;
        cvld<T, VS>(a, rp + g);
        cvld<T, VS>(b, tmp + g);
#pragma unroll
        for (int u = 0; u < VS; u++) o.v[u] = a.v[u] - cmul<T>(al[u], b.v[u]);
        cvst_m<T, VS>(tp + g, o, S.act);
    }
}

// at = A tp ; omega, eta from <at,t>, <at,at>, <y,y>, <y,t>, <at,y>
template <class T, int VS>
__global__ void k_gp_at_v(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ tp, cplx<T>* __restrict__ at,
                          const cplx<T>* __restrict__ tv, const cplx<T>* __restrict__ y, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A c0r[VS], c0i[VS], c1[VS], c2[VS], c3r[VS], c3i[VS], c4r[VS], c4i[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) c0r[u] = c0i[u] = c1[u] = c2[u] = c3r[u] = c3i[u] = c4r[u] = c4i[u] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<T, VS> pe, val, tt, yy;
            cvld<T, VS>(pe, tp + g);
            row_apply<T, VS>(L, M, o, e, i, j, k, tp, ns, s0, S.wm, pe, val);
            cvst_m<T, VS>(at + g, val, S.act);
            cvld<T, VS>(tt, tv + g);
            cvld<T, VS>(yy, y + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                cplx<T> d0 = cdot<T>(val.v[u], tt.v[u]), d3 = cdot<T>(yy.v[u], tt.v[u]), d4 = cdot<T>(val.v[u], yy.v[u]);
                c0r[u] += d0.x; c0i[u] += d0.y;
                c1[u] += cabs2<T>(val.v[u]);
                c2[u] += cabs2<T>(yy.v[u]);
                c3r[u] += d3.x; c3i[u] += d3.y;
                c4r[u] += d4.x; c4i[u] += d4.y;
            }
        }
    double2 acc[4][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        acc[0][u] = make_double2(c0r[u], c0i[u]);
        acc[1][u] = make_double2(c1[u], c2[u]);
        acc[2][u] = make_double2(c3r[u], c3i[u]);
        acc[3][u] = make_double2(c4r[u], c4i[u]);
    }
    if (!vreduce_last<4, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        typedef double2 Z;
        Z att = smem[B + ss];
        double atat = smem[B + ns + ss].x, yyv = smem[B + ns + ss].y;
        Z yt = smem[B + 2 * ns + ss], aty = smem[B + 3 * ns + ss];
        Z yat = make_double2(aty.x, -aty.y);  // <y, at> = conj(<at, y>)
        auto mul = [](Z a, Z b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
        auto sub = [](Z a, Z b) { return make_double2(a.x - b.x, a.y - b.y); };
        auto dv = [](Z a, Z b) {
            double d = b.x * b.x + b.y * b.y;
            return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
        };
        Z om, et;
        if (Q.it == 1) {
            om = make_double2(att.x / atat, att.y / atat);
            et = make_double2(0.0, 0.0);
        } else {
            Z Yy = make_double2(yyv, 0.0), Atat = make_double2(atat, 0.0);
            Z den = sub(mul(Atat, Yy), mul(yat, aty));
            om = dv(sub(mul(Yy, att), mul(yt, aty)), den);
            et = dv(sub(mul(Atat, yt), mul(yat, att)), den);
        }
        Q.omega = om;
        Q.eta = et;
        if (!isfinite(om.x) || !isfinite(om.y) || !isfinite(et.x) || !isfinite(et.y) || (om.x == 0.0 && om.y == 0.0)) {
            Q.active = 0;
            Q.status = ST_BREAK;
        }
    }
}

// u = omega tmp + eta (tpold - rp + beta u) ; z = omega rp + eta z - alpha u ;
// x += alpha p + z ; r = t - eta y - omega at ; err, convergence, beta
template <class T, class XT, int VS>
__global__ void k_gp_upd_v(Mesh M, SysG sgp, KState* st, cplx<T>* __restrict__ u, cplx<T>* __restrict__ z,
                           cplx<XT>* __restrict__ x, cplx<T>* __restrict__ r, const cplx<T>* __restrict__ tmp,
                           const cplx<T>* __restrict__ tpold, const cplx<T>* __restrict__ rp, const cplx<T>* __restrict__ p,
                           const cplx<T>* __restrict__ tv, const cplx<T>* __restrict__ y, const cplx<T>* __restrict__ at,
                           const cplx<T>* __restrict__ r0, RedBuf rb, double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    cplx<T> al[VS], om[VS], et[VS], be[VS];
    cplx<XT> alx[VS];
    A rr[VS], hr[VS], hi[VS];
#pragma unroll
    for (int q = 0; q < VS; q++) {
        al[q] = cst<T>(st[s0 + q].alpha);
        om[q] = cst<T>(st[s0 + q].omega);
        et[q] = cst<T>(st[s0 + q].eta);
        be[q] = cst<T>(st[s0 + q].beta);
        alx[q] = cst<XT>(st[s0 + q].alpha);
        rr[q] = hr[q] = hi[q] = 0;
    }
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> rpg, tm, tpo, uu, zz, pp, tt, yy, aa, q0;
            CV<XT, VS> xx;
            cvld<T, VS>(rpg, rp + g);
            cvld<T, VS>(tm, tmp + g);
            cvld<T, VS>(tpo, tpold + g);
            cvldw<T, VS>(uu, u + g);
            cvldw<T, VS>(zz, z + g);
            cvld<T, VS>(pp, p + g);
            cvldw<XT, VS>(xx, x + g);
            cvld<T, VS>(tt, tv + g);
            cvld<T, VS>(yy, y + g);
            cvld<T, VS>(aa, at + g);
            cvld<T, VS>(q0, r0 + g);
            CV<T, VS> rn;
#pragma unroll
            for (int q = 0; q < VS; q++) {
                cplx<T> un = cmul<T>(om[q], tm.v[q]) + cmul<T>(et[q], (tpo.v[q] - rpg.v[q]) + cmul<T>(be[q], uu.v[q]));
                uu.v[q] = un;
                cplx<T> zn = cmul<T>(om[q], rpg.v[q]) + cmul<T>(et[q], zz.v[q]) - cmul<T>(al[q], un);
                zz.v[q] = zn;
                cplx<XT> p2 = mk<XT>((XT)pp.v[q].x, (XT)pp.v[q].y), z2 = mk<XT>((XT)zn.x, (XT)zn.y);
                xx.v[q] = xx.v[q] + cmul<XT>(alx[q], p2) + z2;
                rn.v[q] = (tt.v[q] - cmul<T>(et[q], yy.v[q])) - cmul<T>(om[q], aa.v[q]);
                rr[q] += cabs2<T>(rn.v[q]);
                cplx<T> d = cdot<T>(q0.v[q], rn.v[q]);
                hr[q] += d.x;
                hi[q] += d.y;
            }
            cvst_m<T, VS>(u + g, uu, S.act);
            cvst_m<T, VS>(z + g, zz, S.act);
            cvst_m<XT, VS>(x + g, xx, S.act);
            cvst_m<T, VS>(r + g, rn, S.act);
        }
    double2 acc[2][VS];
#pragma unroll
    for (int q = 0; q < VS; q++) {
        acc[0][q] = make_double2(rr[q], 0.0);
        acc[1][q] = make_double2(hr[q], hi[q]);
    }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        double nr = sqrt(smem[B + ss].x);
        double2 rn = smem[B + ns + ss];
        Q.err = nr / Q.babs;
        if (err_rec && Q.it <= Q.itmax) err_rec[(size_t)ss * err_stride + Q.it - 1] = Q.err;
        Q.iters = Q.it;
        // beta = alpha/omega * <r0, r_new> / <r0, r_old>, computed before the
        // stopping tests so that a resumed system (mixed precision re-check)
        // continues with consistent scalars
        double2 a = Q.alpha, o = Q.omega, ro = Q.rho;
        double od = o.x * o.x + o.y * o.y, rd = ro.x * ro.x + ro.y * ro.y;
        double2 q1 = make_double2((a.x * o.x + a.y * o.y) / od, (a.y * o.x - a.x * o.y) / od);
        double2 q2 = make_double2((rn.x * ro.x + rn.y * ro.y) / rd, (rn.y * ro.x - rn.x * ro.y) / rd);
        Q.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        Q.it += 1;
        if (isnan(Q.err)) {
            Q.status = ST_NAN;
            Q.active = 0;
            continue;
        }
        if (Q.err <= Q.tol) {  // solvers.f90:272
            Q.status = ST_CONV;
            Q.active = 0;
            continue;
        }
        if (Q.iters >= Q.itmax) {
            Q.status = ST_MAXIT;
            Q.active = 0;
            continue;
        }
    }
}

// w = at + beta ap ; p = rp + beta (p - u)
template <class T, int VS>
__global__ void k_gp_pw_v(Mesh M, SysG sgp, const KState* st, cplx<T>* __restrict__ w, cplx<T>* __restrict__ p,
                          const cplx<T>* __restrict__ at, const cplx<T>* __restrict__ ap, const cplx<T>* __restrict__ rp,
                          const cplx<T>* __restrict__ u) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> be[VS];
#pragma unroll
    for (int q = 0; q < VS; q++) be[q] = cst<T>(st[s0 + q].beta);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> a, b, c, d, pp, wn;
        cvld<T, VS>(a, at + g);
        cvld<T, VS>(b, ap + g);
        cvld<T, VS>(c, rp + g);
        cvld<T, VS>(d, u + g);
        cvldw<T, VS>(pp, p + g);
#pragma unroll
        for (int q = 0; q < VS; q++) {
            wn.v[q] = a.v[q] + cmul<T>(be[q], b.v[q]);
            pp.v[q] = c.v[q] + cmul<T>(be[q], pp.v[q] - d.v[q]);
        }
        cvst_m<T, VS>(w + g, wn, S.act);
        cvst_m<T, VS>(p + g, pp, S.act);
    }
}

// ------------------------------------------------------------------ reliable updates
// x64 += x32 ; x32 = 0 (xb keeps x64 before the update).  ALL = false: the
// active systems (a reliable update in the middle of a solve); ALL = true:
// every system without a NaN (the end of a solve, including systems stopped by
// the iteration limit or a breakdown, whose partial solution would otherwise
// be lost; systems already flushed hold x32 = 0)
template <class T, int VS, bool ALL>
__global__ void k_flush_v(Mesh M, SysG sgp, const KState* st, double2* __restrict__ x64, cplx<T>* __restrict__ x32,
                          double2* __restrict__ xb) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (ALL) {
        S.act = 0;
#pragma unroll
        for (int v = 0; v < VS; v++) S.act |= (st[s0 + v].status != ST_NAN ? 1u : 0u) << v;
    }
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> d, zz;
        CV<double, VS> xv;
        cvldw<T, VS>(d, x32 + g);
        cvldw<double, VS>(xv, x64 + g);
        if (xb) cvst_m<double, VS>(xb + g, xv, S.act);
#pragma unroll
        for (int q = 0; q < VS; q++) xv.v[q] = make_double2(xv.v[q].x + (double)d.v[q].x, xv.v[q].y + (double)d.v[q].y);
        cvzero<T, VS>(zz);
        cvst_m<double, VS>(x64 + g, xv, S.act);
        cvst_m<T, VS>(x32 + g, zz, S.act);
    }
}

// r32 = b64 - A64 x64 ; FP64 convergence test with rejection of updates that
// made the FP64 residual worse ; scalars re-synchronised with the new residual
// (1 BiCGStab: rho = <rhat, r>, beta = rho/rhoold * alpha/omega; 3 GPBiCG:
// beta = alpha/omega * <r0, r>/<r0, r_old>).
template <class T, int VS>
__global__ void k_reliable_v(Lev<double> L, Mesh M, SysG sgp, KState* st, const double2* __restrict__ b,
                             const double2* __restrict__ x, cplx<T>* __restrict__ r, const cplx<T>* __restrict__ rhat,
                             int solver, RedBuf rb) {
    extern __shared__ double2 smem[];
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<double, VS> S = load_sys<double, VS>(st, s0);
    double2 acc[2][VS];
#pragma unroll
    for (int q = 0; q < VS; q++) acc[0][q] = acc[1][q] = make_double2(0.0, 0.0);
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<double, VS> xe, ax, bv;
            cvld<double, VS>(xe, x + g);
            row_apply<double, VS>(L, M, o, e, i, j, k, x, ns, s0, S.wm, xe, ax);
            cvld<double, VS>(bv, b + g);
            CV<T, VS> rt, h;
            cvld<T, VS>(h, rhat + g);
#pragma unroll
            for (int q = 0; q < VS; q++) {
                double2 rv = bv.v[q] - ax.v[q];
                rt.v[q] = mk<T>((T)rv.x, (T)rv.y);
                acc[0][q].x += rv.x * rv.x + rv.y * rv.y;
                acc[1][q].x += (double)h.v[q].x * rv.x + (double)h.v[q].y * rv.y;
                acc[1][q].y += (double)h.v[q].x * rv.y - (double)h.v[q].y * rv.x;
            }
            cvst_m<T, VS>(r + g, rt, S.act);
        }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        Q.err = sqrt(smem[B + ss].x) / Q.babs;
        double2 h = smem[B + ns + ss];
        if (isnan(Q.err) || (Q.errv > 0 && Q.err > 10.0 * Q.errv)) {
            // the complex64 correction made the FP64 residual worse (kappa * eps32 > 1
            // for this system): take it back (k_restore) and stop the mixed iteration
            Q.status = ST_BREAK;
            Q.active = 0;
            Q.pad[0] = 1;
            Q.err = Q.errv;
            continue;
        }
        Q.errv = Q.err;
        if (Q.err < Q.tol) {
            Q.status = ST_VCONV;
            Q.active = 0;
            continue;
        }
        if (Q.it > Q.itmax) {
            Q.status = ST_MAXIT;
            Q.active = 0;
            continue;
        }
        if (solver == 6) {
            // COCR: the driver restarts the recurrence from the new residual
        } else if (solver == 3) {
            double2 a = Q.alpha, o = Q.omega, ro = Q.rho;
            double od = o.x * o.x + o.y * o.y, rd = ro.x * ro.x + ro.y * ro.y;
            double2 q1 = make_double2((a.x * o.x + a.y * o.y) / od, (a.y * o.x - a.x * o.y) / od);
            double2 q2 = make_double2((h.x * ro.x + h.y * ro.y) / rd, (h.y * ro.x - h.x * ro.y) / rd);
            Q.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        } else {
            Q.rho = h;
            double2 a = Q.rho, bb = Q.rhoold, al2 = Q.alpha, om2 = Q.omega;
            double bd = bb.x * bb.x + bb.y * bb.y, od = om2.x * om2.x + om2.y * om2.y;
            double2 q1 = make_double2((a.x * bb.x + a.y * bb.y) / bd, (a.y * bb.x - a.x * bb.y) / bd);
            double2 q2 = make_double2((al2.x * om2.x + al2.y * om2.y) / od, (al2.y * om2.x - al2.x * om2.y) / od);
            Q.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        }
    }
}

// ------------------------------------------------------------------ COCR
// Preconditioned COCR (Sogabe & Zhang 2007) in the bilinear form
// B(u, v) = sum_e u_e V_e v_e (no conjugation): V K and V M are complex
// symmetric for the operator K of fd_assemb/dcfast and its multi-colour SSOR M
// (V the edge dual volumes), so the short recurrence of COCR applies.  Per
// iteration one operator application (u = K z) and one preconditioner
// application (q = M^-1 w); the direction updates p = z + beta p and
// w = u + beta w ride on the first sweep (RHS_COCR).

// x_b = b_b on the boundary edges (identity rows), so that the boundary
// residual is zero before the recurrence starts and stays zero
template <class XT, int VS>
__global__ void k_fix_bnd(Mesh M, SysG sgp, const KState* st, const cplx<XT>* __restrict__ b, cplx<XT>* __restrict__ x) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<XT, VS> S = load_sys<XT, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        if (!mbnd(M, o, i, j, k)) continue;
        const size_t g = (size_t)e * ns + s0;
        CV<XT, VS> bv;
        cvld<XT, VS>(bv, b + g);
        cvst_m<XT, VS>(x + g, bv, S.act);
    }
}

// u = K z ; rho_new = B(z, u) ; beta = rho_new / rho (FIRST: 0) ; rho = rho_new
template <class T, int VS, bool FIRST>
__global__ void k_cocr_u(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ z, cplx<T>* __restrict__ u,
                         RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef double A;  // the dual volumes span many orders of magnitude
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A ar[VS], ai[VS];
#pragma unroll
    for (int q = 0; q < VS; q++) ar[q] = ai[q] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            uint32_t e;
            int i, j, k;
            const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<T, VS> ze, val;
            cvld<T, VS>(ze, z + g);
            row_apply<T, VS>(L, M, o, e, i, j, k, z, ns, s0, S.wm, ze, val);
            cvst_m<T, VS>(u + g, val, S.act);
            const A vol = (A)edge_vol<T>(L, M, o, i, j, k);
#pragma unroll
            for (int q = 0; q < VS; q++) {
                ar[q] += vol * ((A)ze.v[q].x * val.v[q].x - (A)ze.v[q].y * val.v[q].y);
                ai[q] += vol * ((A)ze.v[q].x * val.v[q].y + (A)ze.v[q].y * val.v[q].x);
            }
        }
    double2 acc[1][VS];
#pragma unroll
    for (int q = 0; q < VS; q++) acc[0][q] = make_double2(ar[q], ai[q]);
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        const double2 rn = smem[B + ss], ro = Q.rho;
        if (FIRST) {
            Q.beta = make_double2(0.0, 0.0);
        } else {
            const double rd = ro.x * ro.x + ro.y * ro.y;
            Q.beta = make_double2((rn.x * ro.x + rn.y * ro.y) / rd, (rn.y * ro.x - rn.x * ro.y) / rd);
        }
        Q.rho = rn;
        if (!isfinite(Q.beta.x) || !isfinite(Q.beta.y) || (rn.x == 0.0 && rn.y == 0.0)) {
            Q.active = 0;
            Q.status = ST_BREAK;
        }
    }
}

// w = u + beta w ; p = z + beta p  (the direction update when the
// preconditioner is not the SSOR sweep that fuses it)
template <class T, int VS>
__global__ void k_cocr_dir(Mesh M, SysG sgp, const KState* st, const cplx<T>* __restrict__ u, cplx<T>* __restrict__ w,
                           const cplx<T>* __restrict__ z, cplx<T>* __restrict__ p) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> be[VS];
#pragma unroll
    for (int q = 0; q < VS; q++) be[q] = cst<T>(st[s0 + q].beta);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> uu, ww, zz, pp;
        cvld<T, VS>(uu, u + g);
        cvldw<T, VS>(ww, w + g);
        cvld<T, VS>(zz, z + g);
        cvldw<T, VS>(pp, p + g);
#pragma unroll
        for (int q = 0; q < VS; q++) {
            ww.v[q] = uu.v[q] + cmul<T>(be[q], ww.v[q]);
            pp.v[q] = zz.v[q] + cmul<T>(be[q], pp.v[q]);
        }
        cvst_m<T, VS>(w + g, ww, S.act);
        cvst_m<T, VS>(p + g, pp, S.act);
    }
}

// alpha = rho / B(w, q)
template <class T, int VS>
__global__ void k_cocr_alpha(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ w,
                             const cplx<T>* __restrict__ q, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef double A;  // the dual volumes span many orders of magnitude
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    A ar[VS], ai[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) ar[u] = ai[u] = 0;
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const uint32_t e = fdiv(sgp.fG, t);
            int i, j, k;
            const int o = mdecode(M, e, i, j, k);
            const size_t g = (size_t)e * ns + s0;
            CV<T, VS> wv, qv;
            cvld<T, VS>(wv, w + g);
            cvld<T, VS>(qv, q + g);
            const A vol = (A)edge_vol<T>(L, M, o, i, j, k);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                ar[u] += vol * ((A)wv.v[u].x * qv.v[u].x - (A)wv.v[u].y * qv.v[u].y);
                ai[u] += vol * ((A)wv.v[u].x * qv.v[u].y + (A)wv.v[u].y * qv.v[u].x);
            }
        }
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(ar[u], ai[u]);
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        const double2 d = smem[B + ss], n = Q.rho;
        const double den = d.x * d.x + d.y * d.y;
        Q.alpha = make_double2((n.x * d.x + n.y * d.y) / den, (n.y * d.x - n.x * d.y) / den);
        if (!isfinite(Q.alpha.x) || !isfinite(Q.alpha.y)) {
            Q.active = 0;
            Q.status = ST_BREAK;
        }
    }
}

// x += alpha p ; r -= alpha w ; z -= alpha q ; err = |r| / |b| and the
// stopping tests (as GPBiCG: solvers.f90:272 semantics)
template <class T, class XT, int VS>
__global__ void k_cocr_upd(Mesh M, SysG sgp, KState* st, cplx<XT>* __restrict__ x, cplx<T>* __restrict__ r,
                           cplx<T>* __restrict__ z, const cplx<T>* __restrict__ p, const cplx<T>* __restrict__ w,
                           const cplx<T>* __restrict__ q, RedBuf rb, double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    cplx<T> al[VS];
    cplx<XT> alx[VS];
    A rr[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        al[u] = cst<T>(st[s0 + u].alpha);
        alx[u] = cst<XT>(st[s0 + u].alpha);
        rr[u] = 0;
    }
    if (S.act)
        SFDX_GRID_LOOP(t, M.nl * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> rv, zv, pv, wv, qv;
            CV<XT, VS> xv;
            cvldw<T, VS>(rv, r + g);
            cvldw<T, VS>(zv, z + g);
            cvld<T, VS>(pv, p + g);
            cvld<T, VS>(wv, w + g);
            cvld<T, VS>(qv, q + g);
            cvldw<XT, VS>(xv, x + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                const cplx<XT> p2 = mk<XT>((XT)pv.v[u].x, (XT)pv.v[u].y);
                xv.v[u] = xv.v[u] + cmul<XT>(alx[u], p2);
                rv.v[u] = rv.v[u] - cmul<T>(al[u], wv.v[u]);
                zv.v[u] = zv.v[u] - cmul<T>(al[u], qv.v[u]);
                rr[u] += cabs2<T>(rv.v[u]);
            }
            cvst_m<XT, VS>(x + g, xv, S.act);
            cvst_m<T, VS>(r + g, rv, S.act);
            cvst_m<T, VS>(z + g, zv, S.act);
        }
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(rr[u], 0.0);
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = st[ss];
        if (!Q.active) continue;
        Q.err = sqrt(smem[B + ss].x) / Q.babs;
        if (err_rec && Q.it <= Q.itmax) err_rec[(size_t)ss * err_stride + Q.it - 1] = Q.err;
        Q.iters = Q.it;
        Q.it += 1;
        if (isnan(Q.err)) {
            Q.status = ST_NAN;
            Q.active = 0;
        } else if (Q.err <= Q.tol) {
            Q.status = ST_CONV;
            Q.active = 0;
        } else if (Q.iters >= Q.itmax) {
            Q.status = ST_MAXIT;
            Q.active = 0;
        }
    }
}

// ------------------------------------------------------------------ row coefficients
// rc[e][12] = the coefficients row_k computes for interior row e (zero for the
// Dirichlet rows); built after every conductivity change, per level and
// precision.  L.rc must be null here.
template <class T>
__global__ void k_row_coef(Lev<T> L, Mesh M, T* __restrict__ rc) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < M.nl; e += gridDim.x * blockDim.x) {
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        T v[12];
#pragma unroll
        for (int q = 0; q < 12; q++) v[q] = T(0);
        if (!mbnd(M, o, i, j, k)) {
            RowK<T> K;
            if (o == OX) K = row_k<T, OX, true, true, true>(L, i, j, k);
            else if (o == OY) K = row_k<T, OY, true, true, true>(L, i, j, k);
            else K = row_k<T, OZ, true, true, true>(L, i, j, k);
            v[0] = K.cs[0]; v[1] = K.cs[1]; v[2] = K.cs[2]; v[3] = K.cs[3];
            v[4] = K.dre; v[5] = K.sbar;
            v[6] = K.gA; v[7] = K.sA1; v[8] = K.sA2;
            v[9] = K.gB; v[10] = K.sB1; v[11] = K.sB2;
        }
#pragma unroll
        for (int q = 0; q < 12; q++) rc[(size_t)e * 12 + q] = v[q];
    }
}

}  // namespace sfdx
