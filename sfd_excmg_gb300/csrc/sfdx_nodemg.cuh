// sfdx_nodemg.cuh -- geometric multigrid for the nodal operator of the
// gradient-space correction (sfdx_gradcorr.cuh), used as the preconditioner of
// its conjugate-gradient solve.
//
// Levels: the node grid of the mesh level and its 2x coarsenings (coarse node
// I sits on fine node 2I).  Transfer: trilinear prolongation P with index
// weights 1, 1/2, 1/4, 1/8 (interior nodes only, boundary nodes are held at
// zero) and restriction R = P^T.  Coarse operators are Galerkin products
// R N P, assembled as 27-point stencils by probing (the same colour trick as
// the finest stencil).  Smoother: damped Jacobi, two sweeps before and after
// the coarse-grid correction, a fixed number of sweeps on the coarsest grid;
// with R = P^T and equal pre/post sweeps the V-cycle is a symmetric positive
// definite preconditioner, as conjugate gradients needs.
//
// Vectors are complex64 [node][ns] (ns systems, VS per thread), stencils float.
#pragma once
#include "sfdx_vkern.cuh"

namespace sfdx {

struct NGrid {
    int nx, ny, nz;  // cells; nodes are (nx+1)(ny+1)(nz+1)
    uint32_t np;
    FastDiv fnx1, fny1;
};
inline NGrid make_ngrid(int nx, int ny, int nz) {
    NGrid g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.np = (uint32_t)(nx + 1) * (ny + 1) * (nz + 1);
    g.fnx1 = make_fastdiv(nx + 1);
    g.fny1 = make_fastdiv(ny + 1);
    return g;
}
__device__ __forceinline__ void ng_ijk(const NGrid& G, uint32_t n, int& i, int& j, int& k) {
    uint32_t q = fdiv(G.fnx1, n);
    i = (int)(n - q * (uint32_t)(G.nx + 1));
    uint32_t kk = fdiv(G.fny1, q);
    j = (int)(q - kk * (uint32_t)(G.ny + 1));
    k = (int)kk;
}
__device__ __forceinline__ bool ng_bnd(const NGrid& G, int i, int j, int k) {
    return i == 0 || i == G.nx || j == 0 || j == G.ny || k == 0 || k == G.nz;
}
__device__ __forceinline__ uint32_t ng_id(const NGrid& G, int i, int j, int k) {
    return ((uint32_t)k * (G.ny + 1) + j) * (G.nx + 1) + i;
}

// sum_d coef[d][n] x[n + off(d)] for VS systems (interior node n)
template <class T, int VS>
__device__ __forceinline__ void ng_stencil(const NGrid& G, const float* coef, uint32_t n, const cplx<T>* x, int ns, int s0,
                                           CV<T, VS>& y) {
    const int nx1 = G.nx + 1, pl = nx1 * (G.ny + 1);
    cvzero<T, VS>(y);
#pragma unroll
    for (int d = 0; d < 27; d++) {
        const int off = (d % 3 - 1) + ((d / 3) % 3 - 1) * nx1 + (d / 9 - 1) * pl;
        const T cf = (T)__ldg(coef + (size_t)d * G.np + n);
        CV<T, VS> a;
        cvld<T, VS>(a, x + (size_t)((int64_t)n + off) * ns + s0);
#pragma unroll
        for (int u = 0; u < VS; u++) {
            y.v[u].x += cf * a.v[u].x;
            y.v[u].y += cf * a.v[u].y;
        }
    }
}

// Damped Jacobi sweep: xout = xin + w dinv (b - N xin); FIRST: xout = w dinv b.
// Boundary nodes: 0.
template <class T, int VS, bool FIRST>
__global__ void k_mg_smooth(NGrid G, SysG sgp, const KState* st, const float* __restrict__ coef,
                            const float* __restrict__ dinv, const cplx<T>* __restrict__ b, const cplx<T>* __restrict__ xin,
                            cplx<T>* __restrict__ xout, float w) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, G.np * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        const size_t g = (size_t)n * ns + s0;
        int i, j, k;
        ng_ijk(G, n, i, j, k);
        CV<T, VS> o;
        if (ng_bnd(G, i, j, k)) {
            cvzero<T, VS>(o);
        } else {
            CV<T, VS> bv;
            cvld<T, VS>(bv, b + g);
            const T wd = (T)w * (T)__ldg(dinv + n);
            if (FIRST) {
#pragma unroll
                for (int u = 0; u < VS; u++) o.v[u] = mk<T>(wd * bv.v[u].x, wd * bv.v[u].y);
            } else {
                CV<T, VS> ax, xv;
                ng_stencil<T, VS>(G, coef, n, xin, ns, s0, ax);
                cvld<T, VS>(xv, xin + g);
#pragma unroll
                for (int u = 0; u < VS; u++)
                    o.v[u] = mk<T>(xv.v[u].x + wd * (bv.v[u].x - ax.v[u].x), xv.v[u].y + wd * (bv.v[u].y - ax.v[u].y));
            }
        }
        cvst_m<T, VS>(xout + g, o, S.act);
    }
}

// r = b - N x  (b == nullptr: r = N x); boundary nodes 0
template <class T, int VS>
__global__ void k_mg_resid(NGrid G, SysG sgp, const KState* st, const float* __restrict__ coef,
                           const cplx<T>* __restrict__ b, const cplx<T>* __restrict__ x, cplx<T>* __restrict__ r) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, G.np * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        const size_t g = (size_t)n * ns + s0;
        int i, j, k;
        ng_ijk(G, n, i, j, k);
        CV<T, VS> o;
        if (ng_bnd(G, i, j, k)) {
            cvzero<T, VS>(o);
        } else {
            ng_stencil<T, VS>(G, coef, n, x, ns, s0, o);
            if (b) {
                CV<T, VS> bv;
                cvld<T, VS>(bv, b + g);
#pragma unroll
                for (int u = 0; u < VS; u++) o.v[u] = bv.v[u] - o.v[u];
            }
        }
        cvst_m<T, VS>(r + g, o, S.act);
    }
}

// bc = R rf = P^T rf on the interior coarse nodes (weights 1/2 per unit of
// distance along each axis over the 27 fine nodes around 2I)
template <class T, int VS>
__global__ void k_mg_restrict(NGrid Gc, NGrid Gf, SysG sgp, const KState* st, const cplx<T>* __restrict__ rf,
                              cplx<T>* __restrict__ bc) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, Gc.np * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        int I, J, K;
        ng_ijk(Gc, n, I, J, K);
        CV<T, VS> o;
        cvzero<T, VS>(o);
        if (!ng_bnd(Gc, I, J, K)) {
            const uint32_t f0 = ng_id(Gf, 2 * I, 2 * J, 2 * K);
            const int nx1 = Gf.nx + 1, pl = nx1 * (Gf.ny + 1);
#pragma unroll
            for (int d = 0; d < 27; d++) {
                const int di = d % 3 - 1, dj = (d / 3) % 3 - 1, dk = d / 9 - 1;
                const T wgt = (T)(1.0f / (float)(1 << ((di != 0) + (dj != 0) + (dk != 0))));
                CV<T, VS> a;
                cvld<T, VS>(a, rf + (size_t)((int64_t)f0 + di + dj * nx1 + dk * pl) * ns + s0);
#pragma unroll
                for (int u = 0; u < VS; u++) {
                    o.v[u].x += wgt * a.v[u].x;
                    o.v[u].y += wgt * a.v[u].y;
                }
            }
        }
        cvst_m<T, VS>(bc + (size_t)n * ns + s0, o, S.act);
    }
}

// xf += P xc on the interior fine nodes
template <class T, int VS>
__global__ void k_mg_prolong(NGrid Gf, NGrid Gc, SysG sgp, const KState* st, const cplx<T>* __restrict__ xc,
                             cplx<T>* __restrict__ xf) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, Gf.np * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        int i, j, k;
        ng_ijk(Gf, n, i, j, k);
        if (ng_bnd(Gf, i, j, k)) continue;
        const size_t g = (size_t)n * ns + s0;
        CV<T, VS> o;
        cvldw<T, VS>(o, xf + g);
        const int i0 = i >> 1, j0 = j >> 1, k0 = k >> 1;
        const int i1 = i0 + (i & 1), j1 = j0 + (j & 1), k1 = k0 + (k & 1);
        const T wgt = (T)(1.0f / (float)(1 << ((i & 1) + (j & 1) + (k & 1))));
        for (int kk = k0; kk <= k1; kk++)
            for (int jj = j0; jj <= j1; jj++)
                for (int ii = i0; ii <= i1; ii++) {
                    CV<T, VS> a;
                    cvld<T, VS>(a, xc + (size_t)ng_id(Gc, ii, jj, kk) * ns + s0);
#pragma unroll
                    for (int u = 0; u < VS; u++) {
                        o.v[u].x += wgt * a.v[u].x;
                        o.v[u].y += wgt * a.v[u].y;
                    }
                }
        cvst_m<T, VS>(xf + g, o, S.act);
    }
}

// 27 probe vectors on grid G (systems c = 0..26): 1 on interior nodes of colour c
__device__ __forceinline__ int ng_colour27(int i, int j, int k) { return i % 3 + 3 * (j % 3) + 9 * (k % 3); }
static __global__ void k_mg_probe(NGrid G, float2* __restrict__ pr) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < G.np * 27u; t += gridDim.x * blockDim.x) {
        const uint32_t n = t / 27u;
        const int c = (int)(t - n * 27u);
        int i, j, k;
        ng_ijk(G, n, i, j, k);
        pr[t] = make_float2(!ng_bnd(G, i, j, k) && ng_colour27(i, j, k) == c ? 1.f : 0.f, 0.f);
    }
}
// stencil from the 27 probe responses Q[n][c]; boundary nodes identity rows
template <class QT>
__global__ void k_mg_assemble(NGrid G, const QT* __restrict__ Q, float* __restrict__ coef, float* __restrict__ dinv) {
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < G.np; n += gridDim.x * blockDim.x) {
        int i, j, k;
        ng_ijk(G, n, i, j, k);
        const bool bnd = ng_bnd(G, i, j, k);
        for (int d = 0; d < 27; d++) {
            const int di = d % 3 - 1, dj = (d / 3) % 3 - 1, dk = d / 9 - 1;
            float v;
            if (bnd) v = d == 13 ? 1.f : 0.f;
            else v = (float)Q[(size_t)n * 27 + ng_colour27(i + di, j + dj, k + dk)].x;
            coef[(size_t)d * G.np + n] = v;
        }
        const float dg = bnd ? 1.f : (float)Q[(size_t)n * 27 + ng_colour27(i, j, k)].x;
        dinv[n] = dg > 0.f ? 1.f / dg : 1.f;
    }
}

}  // namespace sfdx
