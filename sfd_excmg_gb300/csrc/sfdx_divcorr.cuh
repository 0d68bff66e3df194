// sfdx_divcorr.cuh -- divergence correction of the edge field
// (div_correc, div_correc.f90:11-147) with the isotropic scheme of
// fddc_assemb (:548-884, iso branches) and the Jacobi-CG of pcg (:343-402):
//   t = T x           nodal sigma-weighted divergence (6 edges per node),
//   P phi = t         7-point nodal sigma-Laplacian, Jacobi-CG to corr_tol,
//   x += grad phi     (phi(end) - phi(start)) / length, except edges with
//                     both end nodes on the outer boundary.
// Boundary nodes carry identity rows in P and zero divergence, so phi = 0
// there.  All of it matrix-free on the cell conductivities, FP64, for ns
// interleaved systems.
#pragma once
#include "sfdx_kernels.cuh"

namespace sfdx {

struct NodeGeo {
    int nx, ny, nz;
    int64_t np, xnl, ynl, ncell;
    const double* a;  // cell sizes (device)
    const double* b;
    const double* c;
    const double* sig;  // [6][ncell]
};

__device__ __forceinline__ bool node_bnd(const NodeGeo& G, int i, int j, int k) {
    return i == 0 || i == G.nx || j == 0 || j == G.ny || k == 0 || k == G.nz;
}
__device__ __forceinline__ double sgn(const NodeGeo& G, int comp, int i, int j, int k) {
    return __ldg(G.sig + (int64_t)comp * G.ncell + ((int64_t)k * G.ny + j) * G.nx + i);
}

// Face fluxes around interior node (i,j,k):  f[0..5] = x-left, x-right,
// y-left, y-right, z-left, z-right sums  sigma*area*2 (no sign), i.e. the
// magnitudes of the T-row entries of fddc_assemb.
__device__ __forceinline__ void node_fluxes(const NodeGeo& G, int i, int j, int k, double* f) {
    const double a0 = __ldg(G.a + i - 1), a1 = __ldg(G.a + i), b0 = __ldg(G.b + j - 1), b1 = __ldg(G.b + j);
    const double c0 = __ldg(G.c + k - 1), c1 = __ldg(G.c + k);
    f[0] = (sgn(G, 0, i - 1, j - 1, k - 1) * b0 * c0 + sgn(G, 0, i - 1, j, k - 1) * b1 * c0 +
            sgn(G, 0, i - 1, j - 1, k) * b0 * c1 + sgn(G, 0, i - 1, j, k) * b1 * c1) * 2;
    f[1] = (sgn(G, 0, i, j - 1, k - 1) * b0 * c0 + sgn(G, 0, i, j, k - 1) * b1 * c0 + sgn(G, 0, i, j - 1, k) * b0 * c1 +
            sgn(G, 0, i, j, k) * b1 * c1) * 2;
    f[2] = (sgn(G, 1, i - 1, j - 1, k - 1) * a0 * c0 + sgn(G, 1, i, j - 1, k - 1) * a1 * c0 +
            sgn(G, 1, i - 1, j - 1, k) * a0 * c1 + sgn(G, 1, i, j - 1, k) * a1 * c1) * 2;
    f[3] = (sgn(G, 1, i - 1, j, k - 1) * a0 * c0 + sgn(G, 1, i, j, k - 1) * a1 * c0 + sgn(G, 1, i - 1, j, k) * a0 * c1 +
            sgn(G, 1, i, j, k) * a1 * c1) * 2;
    f[4] = (sgn(G, 2, i - 1, j - 1, k - 1) * a0 * b0 + sgn(G, 2, i, j - 1, k - 1) * a1 * b0 +
            sgn(G, 2, i - 1, j, k - 1) * a0 * b1 + sgn(G, 2, i, j, k - 1) * a1 * b1) * 2;
    f[5] = (sgn(G, 2, i - 1, j - 1, k) * a0 * b0 + sgn(G, 2, i, j - 1, k) * a1 * b0 + sgn(G, 2, i - 1, j, k) * a0 * b1 +
            sgn(G, 2, i, j, k) * a1 * b1) * 2;
}
// P-row weights: flux / edge length
__device__ __forceinline__ void node_weights(const NodeGeo& G, int i, int j, int k, double* q) {
    double f[6];
    node_fluxes(G, i, j, k, f);
    q[0] = f[0] / __ldg(G.a + i - 1);
    q[1] = f[1] / __ldg(G.a + i);
    q[2] = f[2] / __ldg(G.b + j - 1);
    q[3] = f[3] / __ldg(G.b + j);
    q[4] = f[4] / __ldg(G.c + k - 1);
    q[5] = f[5] / __ldg(G.c + k);
}
__device__ __forceinline__ void node_decode(const NodeGeo& G, int64_t n, int& i, int& j, int& k) {
    i = (int)(n % (G.nx + 1));
    int64_t r = n / (G.nx + 1);
    j = (int)(r % (G.ny + 1));
    k = (int)(r / (G.ny + 1));
}
__device__ __forceinline__ int64_t node_id(const NodeGeo& G, int i, int j, int k) {
    return ((int64_t)k * (G.ny + 1) + j) * (G.nx + 1) + i;
}

// t = T x (boundary nodes 0); also r = t, p = r/m and the PCG start-up sums.
static __global__ void k_dc_div(NodeGeo G, const KState* st, int ns, const double2* __restrict__ x, double2* __restrict__ t,
                         double2* __restrict__ r, double2* __restrict__ p, double2* __restrict__ u, RedBuf rb,
                         KState* pst) {
    extern __shared__ double2 smem[];
    const int s = threadIdx.x % ns;
    const bool act = st[s].active;
    double tt = 0, rz = 0;
    const int64_t W = G.np * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            int i, j, k;
            node_decode(G, g / ns, i, j, k);
            double2 v = make_double2(0.0, 0.0);
            double m = 1.0;
            if (!node_bnd(G, i, j, k)) {
                double f[6];
                node_fluxes(G, i, j, k, f);
                // entry order of the T row: x-left, x-right, y-left, y-right, z-left, z-right
                double2 e0 = x[(((int64_t)k * (G.ny + 1) + j) * G.nx + (i - 1)) * ns + s];
                double2 e1 = x[(((int64_t)k * (G.ny + 1) + j) * G.nx + i) * ns + s];
                double2 e2 = x[(G.xnl + ((int64_t)k * G.ny + (j - 1)) * (G.nx + 1) + i) * ns + s];
                double2 e3 = x[(G.xnl + ((int64_t)k * G.ny + j) * (G.nx + 1) + i) * ns + s];
                double2 e4 = x[(G.xnl + G.ynl + ((int64_t)(k - 1) * (G.ny + 1) + j) * (G.nx + 1) + i) * ns + s];
                double2 e5 = x[(G.xnl + G.ynl + ((int64_t)k * (G.ny + 1) + j) * (G.nx + 1) + i) * ns + s];
                v.x = -f[0] * e0.x + f[1] * e1.x - f[2] * e2.x + f[3] * e3.x - f[4] * e4.x + f[5] * e5.x;
                v.y = -f[0] * e0.y + f[1] * e1.y - f[2] * e2.y + f[3] * e3.y - f[4] * e4.y + f[5] * e5.y;
                double q[6];
                node_weights(G, i, j, k, q);
                m = q[4] + q[2] + q[0] + q[1] + q[3] + q[5];
            }
            t[g] = v;
            r[g] = v;
            u[g] = make_double2(0.0, 0.0);
            p[g] = make_double2(v.x / m, v.y / m);
            tt += v.x * v.x + v.y * v.y;
            rz += (v.x * v.x + v.y * v.y) / m;
        }
    double2 acc[1] = {make_double2(tt, rz)};
    if (!block_reduce_and_last<1, double>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = pst[ss];
        S.active = st[ss].active;
        S.it = 0;
        S.iters = 0;
        S.status = ST_RUN;
        if (!S.active) continue;
        double2 v = smem[B + ss];
        S.babs = sqrt(v.x);
        S.err = 1.0;
        S.rho = make_double2(v.y, 0.0);
        if (!(S.babs > 0)) {  // divergence-free already: phi = 0
            S.active = 0;
            S.status = ST_CONV;
        }
    }
}

// v = P p ; alpha = rho / <p, v>
static __global__ void k_dc_Ap(NodeGeo G, KState* pst, int ns, const double2* __restrict__ p, double2* __restrict__ v,
                        RedBuf rb) {
    extern __shared__ double2 smem[];
    const int s = threadIdx.x % ns;
    const bool act = pst[s].active;
    double ar = 0, ai = 0;
    const int64_t W = G.np * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            int i, j, k;
            node_decode(G, g / ns, i, j, k);
            double2 pv = p[g], out = pv;
            if (!node_bnd(G, i, j, k)) {
                double q[6];
                node_weights(G, i, j, k, q);
                const int64_t n = g / ns;
                const int64_t n2 = (int64_t)(G.nx + 1) * (G.ny + 1);
                double2 pzl = p[(n - n2) * ns + s], pyl = p[(n - G.nx - 1) * ns + s], pxl = p[(n - 1) * ns + s];
                double2 pxr = p[(n + 1) * ns + s], pyr = p[(n + G.nx + 1) * ns + s], pzr = p[(n + n2) * ns + s];
                double d = q[4] + q[2] + q[0] + q[1] + q[3] + q[5];
                out.x = -q[4] * pzl.x - q[2] * pyl.x - q[0] * pxl.x + d * pv.x - q[1] * pxr.x - q[3] * pyr.x - q[5] * pzr.x;
                out.y = -q[4] * pzl.y - q[2] * pyl.y - q[0] * pxl.y + d * pv.y - q[1] * pxr.y - q[3] * pyr.y - q[5] * pzr.y;
            }
            v[g] = out;
            ar += pv.x * out.x + pv.y * out.y;  // conj(p) v
            ai += pv.x * out.y - pv.y * out.x;
        }
    double2 acc[1] = {make_double2(ar, ai)};
    if (!block_reduce_and_last<1, double>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = pst[ss];
        if (!S.active) continue;
        double2 d = smem[B + ss];
        double den = d.x * d.x + d.y * d.y;
        double2 rho = S.rho;
        S.alpha = make_double2((rho.x * d.x + rho.y * d.y) / den, (rho.y * d.x - rho.x * d.y) / den);
        if (!isfinite(S.alpha.x) || !isfinite(S.alpha.y)) {
            S.active = 0;
            S.status = ST_BREAK;
        }
    }
}

// u += alpha p ; r -= alpha v ; rho_new = <r/m, r> ; err = |r|/|t| ; beta
static __global__ void k_dc_upd(NodeGeo G, KState* pst, int ns, const double2* __restrict__ p, const double2* __restrict__ v,
                         double2* __restrict__ u, double2* __restrict__ r, RedBuf rb, double tol, int maxit) {
    extern __shared__ double2 smem[];
    const int s = threadIdx.x % ns;
    const bool act = pst[s].active;
    const double2 al = pst[s].alpha;
    double rr = 0, rz = 0;
    const int64_t W = G.np * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            int i, j, k;
            node_decode(G, g / ns, i, j, k);
            double2 pv = p[g], vv = v[g], uu = u[g], rv = r[g];
            uu.x += al.x * pv.x - al.y * pv.y;
            uu.y += al.x * pv.y + al.y * pv.x;
            rv.x -= al.x * vv.x - al.y * vv.y;
            rv.y -= al.x * vv.y + al.y * vv.x;
            u[g] = uu;
            r[g] = rv;
            double m = 1.0;
            if (!node_bnd(G, i, j, k)) {
                double q[6];
                node_weights(G, i, j, k, q);
                m = q[4] + q[2] + q[0] + q[1] + q[3] + q[5];
            }
            double a2 = rv.x * rv.x + rv.y * rv.y;
            rr += a2;
            rz += a2 / m;
        }
    double2 acc[1] = {make_double2(rr, rz)};
    if (!block_reduce_and_last<1, double>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = pst[ss];
        if (!S.active) continue;
        double2 vv = smem[B + ss];
        S.it += 1;
        S.iters = S.it;
        S.err = sqrt(vv.x) / S.babs;
        double rold = S.rho.x;
        S.rho = make_double2(vv.y, 0.0);
        S.beta = make_double2(vv.y / rold, 0.0);
        if (isnan(S.err)) {
            S.active = 0;
            S.status = ST_NAN;
        } else if (S.err < tol && S.err > 0) {  // pcg stopping test (div_correc.f90:383)
            S.active = 0;
            S.status = ST_CONV;
        } else if (S.it >= maxit) {
            S.active = 0;
            S.status = ST_MAXIT;
        }
    }
}

// p = r/m + beta p
static __global__ void k_dc_p(NodeGeo G, const KState* pst, int ns, const double2* __restrict__ r, double2* __restrict__ p) {
    const int64_t W = G.np * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (!pst[s].active) continue;
        int i, j, k;
        node_decode(G, g / ns, i, j, k);
        double m = 1.0;
        if (!node_bnd(G, i, j, k)) {
            double q[6];
            node_weights(G, i, j, k, q);
            m = q[4] + q[2] + q[0] + q[1] + q[3] + q[5];
        }
        double2 rv = r[g], pv = p[g];
        double be = pst[s].beta.x;
        p[g] = make_double2(rv.x / m + be * pv.x, rv.y / m + be * pv.y);
    }
}

// x_e += (phi(end) - phi(start)) / len_e  unless both ends are boundary nodes
static __global__ void k_dc_grad(NodeGeo G, const KState* st, int ns, const double2* __restrict__ phi, double2* __restrict__ x) {
    const int64_t nl = G.xnl + G.ynl + (int64_t)(G.nx + 1) * (G.ny + 1) * G.nz;
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (!st[s].active) continue;
        const int64_t e = g / ns;
        int i, j, k, i2, j2, k2;
        double len;
        if (e < G.xnl) {
            i = (int)(e % G.nx); int64_t r = e / G.nx; j = (int)(r % (G.ny + 1)); k = (int)(r / (G.ny + 1));
            i2 = i + 1; j2 = j; k2 = k; len = __ldg(G.a + i);
        } else if (e < G.xnl + G.ynl) {
            int64_t f = e - G.xnl;
            i = (int)(f % (G.nx + 1)); int64_t r = f / (G.nx + 1); j = (int)(r % G.ny); k = (int)(r / G.ny);
            i2 = i; j2 = j + 1; k2 = k; len = __ldg(G.b + j);
        } else {
            int64_t f = e - G.xnl - G.ynl;
            i = (int)(f % (G.nx + 1)); int64_t r = f / (G.nx + 1); j = (int)(r % (G.ny + 1)); k = (int)(r / (G.ny + 1));
            i2 = i; j2 = j; k2 = k + 1; len = __ldg(G.c + k);
        }
        if (node_bnd(G, i, j, k) && node_bnd(G, i2, j2, k2)) continue;
        double2 p1 = phi[node_id(G, i, j, k) * ns + s], p2 = phi[node_id(G, i2, j2, k2) * ns + s];
        double2 xv = x[g];
        x[g] = make_double2(xv.x + (p2.x - p1.x) / len, xv.y + (p2.y - p1.y) / len);
    }
}

}  // namespace sfdx
