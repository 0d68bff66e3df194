// sfdx_gradcorr.cuh -- consistent gradient-space (nodal) correction of the
// edge field.
//
// The reference corrects the field every corr_intv Krylov iterations by
// removing the nodal sigma-weighted divergence of x (div_correc,
// div_correc.f90:11-147).  That step ignores the right-hand side, so it
// moves x away from the discrete solution whenever the Dirichlet-eliminated
// right-hand side has a divergence (it always does next to the boundary).
// This module implements the same idea consistently with the discrete
// system A = C - i*w*mu*Ms (curl-curl part C, mass part Ms, rows of
// fd_assemb fdfe_main.f90:248-393):
//
//   x <- x + G phi,    (G^T V Ms G) phi = G^T V r / (-i w mu),   r = b - A x
//
// with G the nodal gradient (interior nodes; edge value (phi_end -
// phi_start) / length) and V the dual volume of each edge.  V*C is
// symmetric and C G = 0, so G^T V A = -i w mu G^T V Ms: the correction is the
// Galerkin projection of the error onto the gradient space, which leaves the
// exact solution unchanged and removes exactly the error components the
// Krylov iteration controls worst (discrete gradients: near-null space of A
// at low frequency and in air).  N = G^T V Ms G is real, symmetric and
// positive definite (the nodal sigma-Laplacian of the operator's own
// conductivity averaging, anisotropic terms included) and frequency
// independent.  It is assembled once per conductivity as a 27-point nodal
// stencil by probing: the matrix-free product (edge gradient, edge mass,
// nodal divergence; FP64) applied to 27 colour-indicator vectors, one per
// residue class of (i mod 3, j mod 3, k mod 3), gives every stencil entry.
// The correction itself is a Jacobi-preconditioned CG on the assembled
// stencil for the ns interleaved systems (complex64 vectors, FP64 inner
// products), to a loose relative tolerance; residual, right-hand side and the
// update of the FP64 field stay FP64.
#pragma once
#include "sfdx_nodemg.cuh"

namespace sfdx {

// dual volume / length of an interior edge (V_e / len_e): the two transverse
// half-spacing sums, e.g. Ex(i,j,k): (b(j-1)+b(j))/2 * (c(k-1)+c(k))/2
__device__ __forceinline__ double vlen(double rs1, double rs2) { return 0.25 / (rs1 * rs2); }

__device__ __forceinline__ void node_ijk(const Mesh& M, uint32_t n, int& i, int& j, int& k) {
    uint32_t q = fdiv(M.fnx1, n);
    i = (int)(n - q * (uint32_t)(M.nx + 1));
    uint32_t kk = fdiv(M.fny1, q);
    j = (int)(q - kk * (uint32_t)(M.ny + 1));
    k = (int)kk;
}
__device__ __forceinline__ bool node_bnd(const Mesh& M, int i, int j, int k) {
    return i == 0 || i == M.nx || j == 0 || j == M.ny || k == 0 || k == M.nz;
}

// The six edges of interior node (i,j,k): [0] Ex(i-1) end, [1] Ex(i) start,
// [2] Ey(j-1) end, [3] Ey(j) start, [4] Ez(k-1) end, [5] Ez(k) start; and the
// weight V/len shared by each pair.
struct NodeEdges {
    uint32_t e[6];
    double w[3];
};
__device__ __forceinline__ NodeEdges node_edges(const Lev<double>& L, const Mesh& M, int i, int j, int k) {
    NodeEdges N;
    const uint32_t nx = M.nx, ny = M.ny, nx1 = nx + 1, ny1 = ny + 1;
    const uint32_t ex = ((uint32_t)k * ny1 + j) * nx + i;
    N.e[0] = ex - 1;
    N.e[1] = ex;
    const uint32_t ey = M.xnl + ((uint32_t)k * ny + j) * nx1 + i;
    N.e[2] = ey - nx1;
    N.e[3] = ey;
    const uint32_t ez = M.xnl + M.ynl + ((uint32_t)k * ny1 + j) * nx1 + i;
    N.e[4] = ez - nx1 * ny1;
    N.e[5] = ez;
    const double rx = __ldg(L.ax.rs + i), ry = __ldg(L.ay.rs + j), rz = __ldg(L.az.rs + k);
    N.w[0] = vlen(ry, rz);
    N.w[1] = vlen(rx, rz);
    N.w[2] = vlen(rx, ry);
    return N;
}

// ge = G p on every edge ((p_end - p_start) / len; boundary edges get 0
// because p = 0 on boundary nodes)
template <int VS>
__global__ void k_gc_grad(Lev<double> L, Mesh M, SysG sgp, const KState* pst, const double2* __restrict__ p,
                          double2* __restrict__ ge) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<double, VS> S = load_sys<double, VS>(pst, s0);
    if (!S.act) return;
    const uint32_t nx1 = M.nx + 1, pl = nx1 * (M.ny + 1);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        const uint32_t n0 = ((uint32_t)k * (M.ny + 1) + j) * nx1 + i;
        uint32_t n1;
        double rl;
        if (o == OX) { n1 = n0 + 1; rl = __ldg(L.ax.rh + i); }
        else if (o == OY) { n1 = n0 + nx1; rl = __ldg(L.ay.rh + j); }
        else { n1 = n0 + pl; rl = __ldg(L.az.rh + k); }
        CV<double, VS> a, b, o2;
        cvld<double, VS>(a, p + (size_t)n0 * ns + s0);
        cvld<double, VS>(b, p + (size_t)n1 * ns + s0);
#pragma unroll
        for (int u = 0; u < VS; u++) o2.v[u] = make_double2(rl * (b.v[u].x - a.v[u].x), rl * (b.v[u].y - a.v[u].y));
        cvst_m<double, VS>(ge + (size_t)e * ns + s0, o2, S.act);
    }
}

// u = (V/len) * Ms ge on interior edges (mass part of the operator row:
// sbar on the diagonal, the anisotropic cross couplings off it), 0 on
// boundary edges
template <int VS, int O>
__device__ __forceinline__ void gc_mass_row(const Lev<double>& L, const Mesh& M, uint32_t e, int i, int j, int k,
                                            const double2* ge, int ns, int s0, CV<double, VS>& out) {
    if (mbnd(M, O, i, j, k)) {
        cvzero<double, VS>(out);
        return;
    }
    const RowK<double> K = row_k<double, O, false, true, true>(L, i, j, k);
    const RowN N = row_n<O>(M, e, i, j, k);
    CV<double, VS> C, Mm, g;
    row_off<double, VS, O, false, true, true, true>(K, N, ge, ns, s0, C, Mm);
    cvld<double, VS>(g, ge + (size_t)e * ns + s0);
    double w;
    if (O == OX) w = vlen(__ldg(L.ay.rs + j), __ldg(L.az.rs + k));
    else if (O == OY) w = vlen(__ldg(L.ax.rs + i), __ldg(L.az.rs + k));
    else w = vlen(__ldg(L.ax.rs + i), __ldg(L.ay.rs + j));
#pragma unroll
    for (int u = 0; u < VS; u++)
        out.v[u] = make_double2(w * (Mm.v[u].x + K.sbar * g.v[u].x), w * (Mm.v[u].y + K.sbar * g.v[u].y));
}
template <int VS>
__global__ void k_gc_mass(Lev<double> L, Mesh M, SysG sgp, const KState* pst, const double2* __restrict__ ge,
                          double2* __restrict__ u) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<double, VS> S = load_sys<double, VS>(pst, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        CV<double, VS> out;
        if (o == OX) gc_mass_row<VS, OX>(L, M, e, i, j, k, ge, ns, s0, out);
        else if (o == OY) gc_mass_row<VS, OY>(L, M, e, i, j, k, ge, ns, s0, out);
        else gc_mass_row<VS, OZ>(L, M, e, i, j, k, ge, ns, s0, out);
        cvst_m<double, VS>(u + (size_t)e * ns + s0, out, S.act);
    }
}

// q = G^T u at interior nodes (u carries V/len: G^T V w = sum of +-(V/len) w
// over the six edges), 0 on boundary nodes
template <int VS>
__global__ void k_gc_gtu(Lev<double> L, Mesh M, SysG sgp, uint32_t np, const double2* __restrict__ uedge,
                         double2* __restrict__ q) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    SFDX_GRID_LOOP(t, np * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        int i, j, k;
        node_ijk(M, n, i, j, k);
        CV<double, VS> qv;
        cvzero<double, VS>(qv);
        if (!node_bnd(M, i, j, k)) {
            const NodeEdges E = node_edges(L, M, i, j, k);
#pragma unroll
            for (int m = 0; m < 6; m++) {
                CV<double, VS> a;
                cvld<double, VS>(a, uedge + (size_t)E.e[m] * ns + s0);
                const double sg_ = (m & 1) ? -1.0 : 1.0;
#pragma unroll
                for (int u = 0; u < VS; u++) {
                    qv.v[u].x += sg_ * a.v[u].x;
                    qv.v[u].y += sg_ * a.v[u].y;
                }
            }
        }
        cvst<double, VS>(q + (size_t)n * ns + s0, qv);
    }
}

// 27 probe vectors (systems c = 0..26): 1 on the interior nodes whose
// (i mod 3) + 3 (j mod 3) + 9 (k mod 3) equals c, 0 elsewhere
__device__ __forceinline__ int node_colour27(int i, int j, int k) { return i % 3 + 3 * (j % 3) + 9 * (k % 3); }
static __global__ void k_gc_probe(Mesh M, uint32_t np, double2* __restrict__ pr) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < np * 27u; t += gridDim.x * blockDim.x) {
        const uint32_t n = t / 27u;
        const int c = (int)(t - n * 27u);
        int i, j, k;
        node_ijk(M, n, i, j, k);
        pr[t] = make_double2(!node_bnd(M, i, j, k) && node_colour27(i, j, k) == c ? 1.0 : 0.0, 0.0);
    }
}
// Start of the nodal PCG: t = i/(w mu) G^T V r (interior nodes; r the FP64
// edge residual), r_n = t, phi = 0, |t|^2; with JAC also z = dinv r, p = z and
// <r, z> (Jacobi preconditioner; otherwise the multigrid V-cycle makes z).
template <class T, int VS, bool JAC>
__global__ void k_gc_rhs(Lev<double> L, Mesh M, SysG sgp, uint32_t np, KState* pst, const double2* __restrict__ redge,
                         const float* __restrict__ dinv, cplx<T>* __restrict__ rn, cplx<T>* __restrict__ z,
                         cplx<T>* __restrict__ p, cplx<T>* __restrict__ phi, RedBuf rb) {
    extern __shared__ double2 smem[];
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<double, VS> S = load_sys<double, VS>(pst, s0);
    double2 acc[2][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = acc[1][u] = make_double2(0.0, 0.0);
    if (S.act)
        SFDX_GRID_LOOP(t, np * sgp.G) {
            const uint32_t n = fdiv(sgp.fG, t);
            const size_t g = (size_t)n * ns + s0;
            int i, j, k;
            node_ijk(M, n, i, j, k);
            CV<double, VS> tv;
            cvzero<double, VS>(tv);
            if (!node_bnd(M, i, j, k)) {
                const NodeEdges E = node_edges(L, M, i, j, k);
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    CV<double, VS> a, b;
                    cvld<double, VS>(a, redge + (size_t)E.e[2 * q] * ns + s0);
                    cvld<double, VS>(b, redge + (size_t)E.e[2 * q + 1] * ns + s0);
#pragma unroll
                    for (int u = 0; u < VS; u++) {
                        tv.v[u].x += E.w[q] * (a.v[u].x - b.v[u].x);
                        tv.v[u].y += E.w[q] * (a.v[u].y - b.v[u].y);
                    }
                }
#pragma unroll
                for (int u = 0; u < VS; u++) tv.v[u] = make_double2(-tv.v[u].y / S.wm[u], tv.v[u].x / S.wm[u]);
            }
            const double di = (double)__ldg(dinv + n);
            CV<T, VS> tt, zz, zero;
            cvzero<T, VS>(zero);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                tt.v[u] = mk<T>((T)tv.v[u].x, (T)tv.v[u].y);
                zz.v[u] = mk<T>((T)(di * tv.v[u].x), (T)(di * tv.v[u].y));
                acc[0][u].x += tv.v[u].x * tv.v[u].x + tv.v[u].y * tv.v[u].y;
                acc[1][u].x += di * (tv.v[u].x * tv.v[u].x + tv.v[u].y * tv.v[u].y);
            }
            cvst_m<T, VS>(rn + g, tt, S.act);
            if (JAC) {
                cvst_m<T, VS>(z + g, zz, S.act);
                cvst_m<T, VS>(p + g, zz, S.act);
            }
            cvst_m<T, VS>(phi + g, zero, S.act);
        }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = pst[ss];
        if (!Q.active) continue;
        Q.babs = sqrt(smem[B + ss].x);
        Q.rho = smem[B + ns + ss];
        Q.err = Q.babs > 0 ? 1.0 : 0.0;
        Q.it = 0;
        Q.iters = 0;
        if (!(Q.babs > 0) || !isfinite(Q.babs)) {  // nothing to correct (or NaN input)
            Q.active = 0;
            Q.status = isfinite(Q.babs) ? ST_CONV : ST_NAN;
        }
    }
}

// q = N p (27-point stencil; boundary rows are identity rows on p = 0);
// alpha = <r,z> / <p,q>
template <class T, int VS>
__global__ void k_gc_Ap(Mesh M, SysG sgp, uint32_t np, KState* pst, const float* __restrict__ coef,
                        const cplx<T>* __restrict__ p, cplx<T>* __restrict__ q, RedBuf rb) {
    extern __shared__ double2 smem[];
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(pst, s0);
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(0.0, 0.0);
    const int nx1 = M.nx + 1, pl = nx1 * (M.ny + 1);
    if (S.act)
        SFDX_GRID_LOOP(t, np * sgp.G) {
            const uint32_t n = fdiv(sgp.fG, t);
            const size_t g = (size_t)n * ns + s0;
            int i, j, k;
            node_ijk(M, n, i, j, k);
            CV<T, VS> qv;
            cvzero<T, VS>(qv);
            if (!node_bnd(M, i, j, k)) {
#pragma unroll
                for (int d = 0; d < 27; d++) {
                    const int off = (d % 3 - 1) + ((d / 3) % 3 - 1) * nx1 + (d / 9 - 1) * pl;
                    const T cf = (T)__ldg(coef + (size_t)d * np + n);
                    CV<T, VS> a;
                    cvld<T, VS>(a, p + (size_t)((int64_t)n + off) * ns + s0);
#pragma unroll
                    for (int u = 0; u < VS; u++) {
                        qv.v[u].x += cf * a.v[u].x;
                        qv.v[u].y += cf * a.v[u].y;
                    }
                }
                CV<T, VS> pv;
                cvld<T, VS>(pv, p + g);
#pragma unroll
                for (int u = 0; u < VS; u++) {
                    acc[0][u].x += (double)pv.v[u].x * qv.v[u].x + (double)pv.v[u].y * qv.v[u].y;
                    acc[0][u].y += (double)pv.v[u].x * qv.v[u].y - (double)pv.v[u].y * qv.v[u].x;
                }
            }
            cvst_m<T, VS>(q + g, qv, S.act);
        }
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = pst[ss];
        if (!Q.active) continue;
        const double2 pq = smem[B + ss], rz = Q.rho;
        const double den = pq.x * pq.x + pq.y * pq.y;
        Q.alpha = make_double2((rz.x * pq.x + rz.y * pq.y) / den, (rz.y * pq.x - rz.x * pq.y) / den);
        if (!isfinite(Q.alpha.x) || !isfinite(Q.alpha.y)) {  // breakdown: keep phi so far
            Q.active = 0;
            Q.status = ST_BREAK;
        }
    }
}

// phi += alpha p ; r -= alpha q ; |r|^2 and the stopping test; with JAC also
// z = dinv r, <r,z> and beta (otherwise k_gc_rz after the V-cycle)
template <class T, int VS, bool JAC>
__global__ void k_gc_upd(SysG sgp, uint32_t np, KState* pst, const float* __restrict__ dinv,
                         const cplx<T>* __restrict__ p, const cplx<T>* __restrict__ q, cplx<T>* __restrict__ phi,
                         cplx<T>* __restrict__ rn, cplx<T>* __restrict__ z, RedBuf rb) {
    extern __shared__ double2 smem[];
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(pst, s0);
    cplx<T> al[VS];
    double2 acc[2][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        al[u] = cst<T>(pst[s0 + u].alpha);
        acc[0][u] = acc[1][u] = make_double2(0.0, 0.0);
    }
    if (S.act)
        SFDX_GRID_LOOP(t, np * sgp.G) {
            const uint32_t n = fdiv(sgp.fG, t);
            const size_t g = (size_t)n * ns + s0;
            CV<T, VS> pv, qv, fv, rv, zv;
            cvld<T, VS>(pv, p + g);
            cvld<T, VS>(qv, q + g);
            cvldw<T, VS>(fv, phi + g);
            cvldw<T, VS>(rv, rn + g);
            const T di = (T)__ldg(dinv + n);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                fv.v[u] = fv.v[u] + cmul<T>(al[u], pv.v[u]);
                rv.v[u] = rv.v[u] - cmul<T>(al[u], qv.v[u]);
                zv.v[u] = mk<T>(di * rv.v[u].x, di * rv.v[u].y);
                const double r2 = (double)rv.v[u].x * rv.v[u].x + (double)rv.v[u].y * rv.v[u].y;
                acc[0][u].x += (double)di * r2;
                acc[1][u].x += r2;
            }
            cvst_m<T, VS>(phi + g, fv, S.act);
            cvst_m<T, VS>(rn + g, rv, S.act);
            if (JAC) cvst_m<T, VS>(z + g, zv, S.act);
        }
    if (!vreduce_last<2, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = pst[ss];
        if (!Q.active) continue;
        if (JAC) {
            const double2 rz = smem[B + ss], ro = Q.rho;
            const double rd = ro.x * ro.x + ro.y * ro.y;
            Q.beta = make_double2((rz.x * ro.x + rz.y * ro.y) / rd, (rz.y * ro.x - rz.x * ro.y) / rd);
            Q.rho = rz;
        }
        Q.err = sqrt(smem[B + ns + ss].x) / Q.babs;
        Q.it += 1;
        Q.iters = Q.it;
        if (isnan(Q.err)) {
            Q.active = 0;
            Q.status = ST_NAN;
        } else if (Q.err < Q.tol) {
            Q.active = 0;
            Q.status = ST_CONV;
        } else if (Q.it >= Q.itmax) {
            Q.active = 0;
            Q.status = ST_MAXIT;
        }
    }
}

// <r, z> after the preconditioner: rho, and beta = rho_new / rho_old unless FIRST
template <class T, int VS, bool FIRST>
__global__ void k_gc_rz(SysG sgp, uint32_t np, KState* pst, const cplx<T>* __restrict__ rn, const cplx<T>* __restrict__ z,
                        RedBuf rb) {
    extern __shared__ double2 smem[];
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(pst, s0);
    double2 acc[1][VS];
#pragma unroll
    for (int u = 0; u < VS; u++) acc[0][u] = make_double2(0.0, 0.0);
    if (S.act)
        SFDX_GRID_LOOP(t, np * sgp.G) {
            const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
            CV<T, VS> rv, zv;
            cvld<T, VS>(rv, rn + g);
            cvld<T, VS>(zv, z + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                acc[0][u].x += (double)rv.v[u].x * zv.v[u].x + (double)rv.v[u].y * zv.v[u].y;
                acc[0][u].y += (double)rv.v[u].x * zv.v[u].y - (double)rv.v[u].y * zv.v[u].x;
            }
        }
    if (!vreduce_last<1, VS>(acc, sgp, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& Q = pst[ss];
        if (!Q.active) continue;
        const double2 rz = smem[B + ss];
        if (!FIRST) {
            const double2 ro = Q.rho;
            const double rd = ro.x * ro.x + ro.y * ro.y;
            Q.beta = make_double2((rz.x * ro.x + rz.y * ro.y) / rd, (rz.y * ro.x - rz.x * ro.y) / rd);
        }
        Q.rho = rz;
        if (!isfinite(rz.x) || !isfinite(rz.y)) {
            Q.active = 0;
            Q.status = ST_BREAK;
        }
    }
}

// p = z + beta p  (FIRST: p = z)
template <class T, int VS, bool FIRST>
__global__ void k_gc_p(SysG sgp, uint32_t np, const KState* pst, const cplx<T>* __restrict__ z, cplx<T>* __restrict__ p) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(pst, s0);
    if (!S.act) return;
    cplx<T> be[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) be[u] = cst<T>(pst[s0 + u].beta);
    SFDX_GRID_LOOP(t, np * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> zv, pv;
        cvld<T, VS>(zv, z + g);
        if (FIRST) {
            pv = zv;
        } else {
            cvldw<T, VS>(pv, p + g);
#pragma unroll
            for (int u = 0; u < VS; u++) pv.v[u] = zv.v[u] + cmul<T>(be[u], pv.v[u]);
        }
        cvst_m<T, VS>(p + g, pv, S.act);
    }
}

// x += G phi (FP64 accumulation) for the systems that took part (pad[1] == 1)
template <class T, int VS>
__global__ void k_gc_apply(Lev<double> L, Mesh M, SysG sgp, const KState* pst, const cplx<T>* __restrict__ phi,
                           double2* __restrict__ x) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    unsigned act = 0;
#pragma unroll
    for (int u = 0; u < VS; u++) act |= (pst[s0 + u].pad[1] == 1 ? 1u : 0u) << u;
    if (!act) return;
    const uint32_t nx1 = M.nx + 1, pl = nx1 * (M.ny + 1);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        const uint32_t n0 = ((uint32_t)k * (M.ny + 1) + j) * nx1 + i;
        uint32_t n1;
        double rl;
        if (o == OX) { n1 = n0 + 1; rl = __ldg(L.ax.rh + i); }
        else if (o == OY) { n1 = n0 + nx1; rl = __ldg(L.ay.rh + j); }
        else { n1 = n0 + pl; rl = __ldg(L.az.rh + k); }
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> a, b;
        CV<double, VS> xv;
        cvld<T, VS>(a, phi + (size_t)n0 * ns + s0);
        cvld<T, VS>(b, phi + (size_t)n1 * ns + s0);
        cvldw<double, VS>(xv, x + g);
#pragma unroll
        for (int u = 0; u < VS; u++)
            xv.v[u] = make_double2(xv.v[u].x + rl * ((double)b.v[u].x - (double)a.v[u].x),
                                   xv.v[u].y + rl * ((double)b.v[u].y - (double)a.v[u].y));
        cvst_m<double, VS>(x + g, xv, act);
    }
}

}  // namespace sfdx
