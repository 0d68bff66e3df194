// sfdx_mgkern.cuh -- kernels of the edge multigrid preconditioner
// (precond = 'G'; no counterpart in the reference, whose pre_type offers
// SSOR, Jacobi and ILU(0) only, global_para.f90:18).
//
// The V-cycle runs on the mesh levels the EXCMG cascade already holds (level
// l-1 is level l with every pair of cells merged, mesh_coarsen
// fdfe_main.f90:18-84), each with its own rediscretised operator:
//   * smoother: the multi-colour SSOR of the Krylov solves, followed by a
//     nodal (gradient-space) step: phi = w D^-1 G^T V r with r = b - A x (formed
//     as b + i w mu Ms x, see k_mg_mres_v) and D
//     the diagonal of G^T V A G = -i w mu N (N the nodal operator of the
//     gradient correction), x += G phi.  Point smoothers cannot reduce the
//     error in the near-null space of the curl-curl operator (discrete
//     gradients: air cells and low frequencies); the nodal step does.
//   * prolongation P: the lowest-order edge interpolation on nested
//     non-uniform meshes -- a fine edge takes the coarse edges parallel to it
//     with weight 1 along the edge and the linear interpolation weights of its
//     transverse node positions (1 on a coarse node, h-/(h-+h+) and
//     h+/(h-+h+) between two);
//   * restriction R = V_c^-1 P^T V_f (V the edge dual volumes), the transpose
//     with respect to the inner product in which the operator is symmetric.
// Vectors are [edge][ns] (nodal: [node][ns]) in the precision of the solve;
// VS systems per thread as in sfdx_vkern.cuh.
#pragma once
#include "sfdx_gradcorr.cuh"

namespace sfdx {

// r = b - A x for the active systems (boundary rows: identity)
template <class T, int VS>
__global__ void k_mg_res_v(Lev<T> L, Mesh M, SysG sgp, const KState* st, const cplx<T>* __restrict__ b,
                           const cplx<T>* __restrict__ x, cplx<T>* __restrict__ r) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        uint32_t e;
        int i, j, k;
        const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> xe, ax, bv;
        cvld<T, VS>(xe, x + g);
        row_apply<T, VS>(L, M, o, e, i, j, k, x, ns, s0, S.wm, xe, ax);
        cvld<T, VS>(bv, b + g);
#pragma unroll
        for (int u = 0; u < VS; u++) ax.v[u] = bv.v[u] - ax.v[u];
        cvst_m<T, VS>(r + g, ax, S.act);
    }
}

// Gradient-space residual of the nodal step, q = b + i wm Ms x on interior
// edges (0 on boundary edges).  G^T V A = -i wm G^T V Ms exactly (V C is
// symmetric and C G = 0), so G^T V q equals G^T V (b - A x) without the
// curl-curl terms: the full residual r = b - A x carries rounding noise of the
// size eps |C x|, which the nodal step divides by wm sigma -- in air (sigma
// 1e-8) a complex64 V-cycle turned that noise into gradient fields of order
// one and diverged.
template <class T, int VS, int O>
__device__ __forceinline__ void mg_mass_row(const Lev<T>& L, const Mesh& M, uint32_t e, int i, int j, int k,
                                            const cplx<T>* x, int ns, int s0, const T (&wm)[VS], const CV<T, VS>& bv,
                                            CV<T, VS>& q) {
    if (mbnd(M, O, i, j, k)) {
        cvzero<T, VS>(q);
        return;
    }
    const RowK<T> K = row_k_e<T, O, false, true, true>(L, e, i, j, k);
    CV<T, VS> Mm, xe;
    if (both_zero(K.sA1, K.sA2) && both_zero(K.sB1, K.sB2)) {
        cvzero<T, VS>(Mm);  // isotropic cells around the edge: diagonal mass only, no neighbour reads
    } else {
        const RowN N = row_n<O>(M, e, i, j, k);
        CV<T, VS> C;
        row_off<T, VS, O, false, true, true, true>(K, N, x, ns, s0, C, Mm);
    }
    cvld<T, VS>(xe, x + (size_t)e * ns + s0);
#pragma unroll
    for (int u = 0; u < VS; u++) {
        const T mx = Mm.v[u].x + K.sbar * xe.v[u].x, my = Mm.v[u].y + K.sbar * xe.v[u].y;
        q.v[u] = mk<T>(bv.v[u].x - wm[u] * my, bv.v[u].y + wm[u] * mx);
    }
}
template <class T, int VS>
__global__ void k_mg_mres_v(Lev<T> L, Mesh M, SysG sgp, const KState* st, const cplx<T>* __restrict__ b,
                            const cplx<T>* __restrict__ x, cplx<T>* __restrict__ q) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        uint32_t e;
        int i, j, k;
        const int o = mdecode_plane(M, fdiv(sgp.fG, t), e, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> bv, qv;
        cvld<T, VS>(bv, b + g);
        if (o == OX) mg_mass_row<T, VS, OX>(L, M, e, i, j, k, x, ns, s0, S.wm, bv, qv);
        else if (o == OY) mg_mass_row<T, VS, OY>(L, M, e, i, j, k, x, ns, s0, S.wm, bv, qv);
        else mg_mass_row<T, VS, OZ>(L, M, e, i, j, k, x, ns, s0, S.wm, bv, qv);
        cvst_m<T, VS>(q + g, qv, S.act);
    }
}

// Complex64 preconditioning of a complex128 Krylov solve: the vector update
// of MODE (as the first sweep of k_fwd_v applies it) in FP64, its result
// rounded to complex64 for the V-cycle; and the V-cycle's output widened back.
template <int VS, int MODE>
__global__ void k_mg_to32_v(Mesh M, SysG sgp, const KState* st, double2* __restrict__ q, const double2* __restrict__ r,
                            const double2* __restrict__ v, double2* __restrict__ aux, float2* __restrict__ q32) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<double, VS> S = load_sys<double, VS>(st, s0);
    if (!S.act) return;
    double2 c1[VS], c2[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        c1[u] = MODE == RHS_PUPD || MODE == RHS_COCR ? st[s0 + u].beta : st[s0 + u].alpha;
        c2[u] = st[s0 + u].omega;
    }
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<double, VS> rhs;
        if (MODE == RHS_PUPD) {
            CV<double, VS> rr, qq, vv;
            cvld<double, VS>(rr, r + g);
            cvldw<double, VS>(qq, q + g);
            cvld<double, VS>(vv, v + g);
#pragma unroll
            for (int u = 0; u < VS; u++) rhs.v[u] = rr.v[u] + cmul<double>(c1[u], qq.v[u] - cmul<double>(c2[u], vv.v[u]));
            cvst_m<double, VS>(q + g, rhs, S.act);
        } else if (MODE == RHS_SUPD) {
            CV<double, VS> rr, vv;
            cvld<double, VS>(rr, r + g);
            cvld<double, VS>(vv, v + g);
#pragma unroll
            for (int u = 0; u < VS; u++) rhs.v[u] = rr.v[u] - cmul<double>(c1[u], vv.v[u]);
            cvst_m<double, VS>(q + g, rhs, S.act);
        } else if (MODE == RHS_COCR) {
            CV<double, VS> uu, qq, zz, pp;
            cvld<double, VS>(uu, r + g);
            cvldw<double, VS>(qq, q + g);
            cvld<double, VS>(zz, v + g);
            cvldw<double, VS>(pp, aux + g);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                rhs.v[u] = uu.v[u] + cmul<double>(c1[u], qq.v[u]);
                pp.v[u] = zz.v[u] + cmul<double>(c1[u], pp.v[u]);
            }
            cvst_m<double, VS>(q + g, rhs, S.act);
            cvst_m<double, VS>(aux + g, pp, S.act);
        } else {
            cvldw<double, VS>(rhs, q + g);
        }
        CV<float, VS> f;
#pragma unroll
        for (int u = 0; u < VS; u++) f.v[u] = make_float2((float)rhs.v[u].x, (float)rhs.v[u].y);
        cvst_m<float, VS>(q32 + g, f, S.act);
    }
}
template <int VS>
__global__ void k_mg_to64_v(Mesh M, SysG sgp, const KState* st, const float2* __restrict__ x32, double2* __restrict__ x) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<double, VS> S = load_sys<double, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<float, VS> f;
        cvld<float, VS>(f, x32 + g);
        CV<double, VS> d;
#pragma unroll
        for (int u = 0; u < VS; u++) d.v[u] = make_double2((double)f.v[u].x, (double)f.v[u].y);
        cvst_m<double, VS>(x + g, d, S.act);
    }
}

// x += z for the active systems
template <class T, int VS>
__global__ void k_mg_add_v(Mesh M, SysG sgp, const KState* st, cplx<T>* __restrict__ x, const cplx<T>* __restrict__ z) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> a, d;
        cvldw<T, VS>(a, x + g);
        cvld<T, VS>(d, z + g);
#pragma unroll
        for (int u = 0; u < VS; u++) a.v[u] = a.v[u] + d.v[u];
        cvst_m<T, VS>(x + g, a, S.act);
    }
}

// Nodal step, part 1: phi = w D^-1 G^T V r at interior nodes (0 on boundary
// nodes), D = -i wm N_nn, so phi = (w dinv / wm) * i * (G^T V r).
// G^T V r at node (i,j,k) = sum over its six edges of +-(V/len) r: + for the
// edge that ends at the node, - for the one that starts there.
// air_max > 0: nodes whose eight cells all have sigma_xx below air_max get no
// correction (their gradients are near-null modes of any size -- see
// emg_air_cut).
template <class T, int VS>
__global__ void k_mg_node_v(Lev<T> L, Mesh M, SysG sgp, uint32_t np, const KState* st, const cplx<T>* __restrict__ r,
                            const float* __restrict__ dinv, cplx<T>* __restrict__ phi, T omega, T air_max) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    const uint32_t nx1 = M.nx + 1, ny1 = M.ny + 1;
    SFDX_GRID_LOOP(t, np * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        int i, j, k;
        node_ijk(M, n, i, j, k);
        CV<T, VS> out;
        cvzero<T, VS>(out);
        bool air = false;
        if (air_max > T(0) && !node_bnd(M, i, j, k)) {
            T smax = T(0);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int64_t cidx = ((int64_t)(k - 1 + (q >> 2)) * M.ny + (j - 1 + ((q >> 1) & 1))) * M.nx + (i - 1 + (q & 1));
                smax = fmax(smax, __ldg(L.sig + cidx));
            }
            air = smax < air_max;
        }
        if (!node_bnd(M, i, j, k) && !air) {
            const uint32_t ex = ((uint32_t)k * ny1 + j) * M.nx + i;
            const uint32_t ey = M.xnl + ((uint32_t)k * M.ny + j) * nx1 + i;
            const uint32_t ez = M.xnl + M.ynl + ((uint32_t)k * ny1 + j) * nx1 + i;
            const uint32_t es[6] = {ex - 1, ex, ey - nx1, ey, ez - nx1 * ny1, ez};
            const T rx = __ldg(L.ax.rs + i), ry = __ldg(L.ay.rs + j), rz = __ldg(L.az.rs + k);
            const T w[3] = {T(0.25) / (ry * rz), T(0.25) / (rx * rz), T(0.25) / (rx * ry)};
            CV<T, VS> tn;
            cvzero<T, VS>(tn);
#pragma unroll
            for (int m = 0; m < 6; m++) {
                CV<T, VS> a;
                cvld<T, VS>(a, r + (size_t)es[m] * ns + s0);
                const T f = (m & 1) ? -w[m >> 1] : w[m >> 1];
#pragma unroll
                for (int u = 0; u < VS; u++) {
                    tn.v[u].x += f * a.v[u].x;
                    tn.v[u].y += f * a.v[u].y;
                }
            }
            const T d = omega * (T)__ldg(dinv + n);
#pragma unroll
            for (int u = 0; u < VS; u++) {
                const T s = d / S.wm[u];
                out.v[u] = mk<T>(-s * tn.v[u].y, s * tn.v[u].x);
            }
        }
        cvst_m<T, VS>(phi + (size_t)n * ns + s0, out, S.act);
    }
}

// Nodal step, part 2: x += G phi on interior edges ((phi_end - phi_start) / len)
template <class T, int VS>
__global__ void k_mg_gadd_v(Lev<T> L, Mesh M, SysG sgp, const KState* st, const cplx<T>* __restrict__ phi,
                            cplx<T>* __restrict__ x) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    const uint32_t nx1 = M.nx + 1, pl = nx1 * (M.ny + 1);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        if (mbnd(M, o, i, j, k)) continue;
        const uint32_t n0 = ((uint32_t)k * (M.ny + 1) + j) * nx1 + i;
        uint32_t n1;
        T rl;
        if (o == OX) { n1 = n0 + 1; rl = __ldg(L.ax.rh + i); }
        else if (o == OY) { n1 = n0 + nx1; rl = __ldg(L.ay.rh + j); }
        else { n1 = n0 + pl; rl = __ldg(L.az.rh + k); }
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> a, b, xv;
        cvld<T, VS>(a, phi + (size_t)n0 * ns + s0);
        cvld<T, VS>(b, phi + (size_t)n1 * ns + s0);
        cvldw<T, VS>(xv, x + g);
#pragma unroll
        for (int u = 0; u < VS; u++)
            xv.v[u] = mk<T>(xv.v[u].x + rl * (b.v[u].x - a.v[u].x), xv.v[u].y + rl * (b.v[u].y - a.v[u].y));
        cvst_m<T, VS>(x + g, xv, S.act);
    }
}

// Transverse interpolation of one fine node index m onto the coarse nodes
// of an axis (fine node 2I is coarse node I): 1 or 2 terms (coarse node,
// weight).  Between two coarse nodes the weights are linear in position:
// whi(m) = h(m)/(h(m-1)+h(m)) towards the lower one, wlo(m) towards the upper.
template <class T>
__device__ __forceinline__ int mg_node_terms(const AxisT<T>& A, int m, int (&c)[2], T (&w)[2]) {
    if ((m & 1) == 0) {
        c[0] = m >> 1;
        w[0] = T(1);
        return 1;
    }
    c[0] = m >> 1;
    c[1] = (m >> 1) + 1;
    w[0] = __ldg(A.whi + m);
    w[1] = __ldg(A.wlo + m);
    return 2;
}

// Prolongation with addition: xf += P ec on the interior fine edges.
template <class T, int VS>
__global__ void k_mg_prolong_v(Lev<T> Lf, Mesh Mf, Mesh Mc, SysG sgp, const KState* st, const cplx<T>* __restrict__ ec,
                               cplx<T>* __restrict__ xf) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, Mf.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(Mf, e, i, j, k);
        if (mbnd(Mf, o, i, j, k)) continue;
        int ca[2], cb[2];
        T wa[2], wb[2];
        int na, nb;
        if (o == OX) {
            na = mg_node_terms<T>(Lf.ay, j, ca, wa);
            nb = mg_node_terms<T>(Lf.az, k, cb, wb);
        } else if (o == OY) {
            na = mg_node_terms<T>(Lf.ax, i, ca, wa);
            nb = mg_node_terms<T>(Lf.az, k, cb, wb);
        } else {
            na = mg_node_terms<T>(Lf.ax, i, ca, wa);
            nb = mg_node_terms<T>(Lf.ay, j, cb, wb);
        }
        CV<T, VS> acc;
        cvzero<T, VS>(acc);
        for (int p = 0; p < na; p++)
            for (int q = 0; q < nb; q++) {
                uint32_t c;
                if (o == OX) c = medge(Mc, OX, i >> 1, ca[p], cb[q]);
                else if (o == OY) c = medge(Mc, OY, ca[p], j >> 1, cb[q]);
                else c = medge(Mc, OZ, ca[p], cb[q], k >> 1);
                CV<T, VS> v;
                cvld<T, VS>(v, ec + (size_t)c * ns + s0);
                const T w = wa[p] * wb[q];
#pragma unroll
                for (int u = 0; u < VS; u++) {
                    acc.v[u].x += w * v.v[u].x;
                    acc.v[u].y += w * v.v[u].y;
                }
            }
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> xv;
        cvldw<T, VS>(xv, xf + g);
#pragma unroll
        for (int u = 0; u < VS; u++) xv.v[u] = xv.v[u] + acc.v[u];
        cvst_m<T, VS>(xf + g, xv, S.act);
    }
}

// Restriction bc = V_c^-1 P^T V_f rf on the interior coarse edges (0 on the
// coarse boundary edges, whose rows are identity rows).  A coarse edge
// gathers the two fine edges along it and their parallel neighbours at the
// fine nodes 2J-1, 2J, 2J+1 of each transverse axis (18 fine edges, all
// interior when the coarse edge is).
template <class T>
__device__ __forceinline__ void mg_gather_terms(const AxisT<T>& A, int J, int (&m)[3], T (&w)[3]) {
    m[0] = 2 * J - 1;
    m[1] = 2 * J;
    m[2] = 2 * J + 1;
    w[0] = __ldg(A.wlo + m[0]);  // fine node 2J-1 towards its upper coarse node J
    w[1] = T(1);
    w[2] = __ldg(A.whi + m[2]);  // fine node 2J+1 towards its lower coarse node J
}
template <class T, int VS>
__global__ void k_mg_restrict_v(Lev<T> Lf, Mesh Mf, Lev<T> Lc, Mesh Mc, SysG sgp, const KState* st,
                                const cplx<T>* __restrict__ rf, cplx<T>* __restrict__ bc) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, Mc.nl * sgp.G) {
        const uint32_t ec = fdiv(sgp.fG, t);
        int I, J, K;
        const int o = mdecode(Mc, ec, I, J, K);
        CV<T, VS> acc;
        cvzero<T, VS>(acc);
        if (!mbnd(Mc, o, I, J, K)) {
            int ma[3], mb[3];
            T wa[3], wb[3];
            // transverse weights; the fine dual volume is length x 1/4 (h-+h+)(h-+h+) of the two
            // transverse axes, 1/(rs rs) / 4
            T ra[3], rb[3];
            if (o == OX) {
                mg_gather_terms<T>(Lf.ay, J, ma, wa);
                mg_gather_terms<T>(Lf.az, K, mb, wb);
                for (int q = 0; q < 3; q++) { ra[q] = __ldg(Lf.ay.rs + ma[q]); rb[q] = __ldg(Lf.az.rs + mb[q]); }
            } else if (o == OY) {
                mg_gather_terms<T>(Lf.ax, I, ma, wa);
                mg_gather_terms<T>(Lf.az, K, mb, wb);
                for (int q = 0; q < 3; q++) { ra[q] = __ldg(Lf.ax.rs + ma[q]); rb[q] = __ldg(Lf.az.rs + mb[q]); }
            } else {
                mg_gather_terms<T>(Lf.ax, I, ma, wa);
                mg_gather_terms<T>(Lf.ay, J, mb, wb);
                for (int q = 0; q < 3; q++) { ra[q] = __ldg(Lf.ax.rs + ma[q]); rb[q] = __ldg(Lf.ay.rs + mb[q]); }
            }
            const AxisT<T>& Al = o == OX ? Lf.ax : (o == OY ? Lf.ay : Lf.az);
            const int l0 = o == OX ? 2 * I : (o == OY ? 2 * J : 2 * K);
            const T len0 = T(1) / __ldg(Al.rh + l0), len1 = T(1) / __ldg(Al.rh + l0 + 1);
            for (int h = 0; h < 2; h++) {
                const T len = h ? len1 : len0;
                const int l = l0 + h;
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        uint32_t f;
                        if (o == OX) f = medge(Mf, OX, l, ma[p], mb[q]);
                        else if (o == OY) f = medge(Mf, OY, ma[p], l, mb[q]);
                        else f = medge(Mf, OZ, ma[p], mb[q], l);
                        const T w = wa[p] * wb[q] * len * T(0.25) / (ra[p] * rb[q]);
                        CV<T, VS> v;
                        cvld<T, VS>(v, rf + (size_t)f * ns + s0);
#pragma unroll
                        for (int u = 0; u < VS; u++) {
                            acc.v[u].x += w * v.v[u].x;
                            acc.v[u].y += w * v.v[u].y;
                        }
                    }
            }
            const T iv = T(1) / edge_vol<T>(Lc, Mc, o, I, J, K);
#pragma unroll
            for (int u = 0; u < VS; u++) acc.v[u] = mk<T>(acc.v[u].x * iv, acc.v[u].y * iv);
        }
        cvst_m<T, VS>(bc + (size_t)ec * ns + s0, acc, S.act);
    }
}

// ------------------------------------------------------------------ split V-cycle
// For a complex64 Krylov iteration under the multigrid (SFDX_MG_SPLIT): the
// V-cycle carries its nodal corrections as a potential psi beside x instead
// of adding G phi into x, and A(x + G psi) = A x - i wm Ms G psi (C G = 0), so
// no complex64 vector holds a curl part beside a much larger gradient part.

// out = x + G psi on interior edges, x on boundary edges (x == nullptr: 0)
template <class T, int VS>
__global__ void k_mg_xpg_v(Lev<T> L, Mesh M, SysG sgp, const KState* st, const cplx<T>* __restrict__ x,
                           const cplx<T>* __restrict__ psi, cplx<T>* __restrict__ out) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    const uint32_t nx1 = M.nx + 1, pl = nx1 * (M.ny + 1);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> xv;
        if (x) cvld<T, VS>(xv, x + g);
        else cvzero<T, VS>(xv);
        if (!mbnd(M, o, i, j, k)) {
            const uint32_t n0 = ((uint32_t)k * (M.ny + 1) + j) * nx1 + i;
            uint32_t n1;
            T rl;
            if (o == OX) { n1 = n0 + 1; rl = __ldg(L.ax.rh + i); }
            else if (o == OY) { n1 = n0 + nx1; rl = __ldg(L.ay.rh + j); }
            else { n1 = n0 + pl; rl = __ldg(L.az.rh + k); }
            CV<T, VS> a, b;
            cvld<T, VS>(a, psi + (size_t)n0 * ns + s0);
            cvld<T, VS>(b, psi + (size_t)n1 * ns + s0);
#pragma unroll
            for (int u = 0; u < VS; u++)
                xv.v[u] = mk<T>(xv.v[u].x + rl * (b.v[u].x - a.v[u].x), xv.v[u].y + rl * (b.v[u].y - a.v[u].y));
        }
        cvst_m<T, VS>(out + g, xv, S.act);
    }
}

// psi += phi (node vectors [node][ns])
template <class T, int VS>
__global__ void k_mg_nadd_v(SysG sgp, const KState* st, uint32_t np, cplx<T>* __restrict__ psi,
                            const cplx<T>* __restrict__ phi) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    SFDX_GRID_LOOP(t, np * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> a, d;
        cvldw<T, VS>(a, psi + g);
        cvld<T, VS>(d, phi + g);
#pragma unroll
        for (int u = 0; u < VS; u++) a.v[u] = a.v[u] + d.v[u];
        cvst_m<T, VS>(psi + g, a, S.act);
    }
}

// psi_f += Pn psi_c at the interior fine nodes: the trilinear interpolation on
// the nested non-uniform node grids (the node terms of the edge prolongation,
// with which it commutes: P G_c = G_f Pn)
template <class T, int VS>
__global__ void k_mg_nprolong_v(Lev<T> Lf, Mesh Mf, Mesh Mc, SysG sgp, const KState* st, uint32_t npf,
                                const cplx<T>* __restrict__ psic, cplx<T>* __restrict__ psif) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    const uint32_t cx1 = Mc.nx + 1, cy1 = Mc.ny + 1;
    SFDX_GRID_LOOP(t, npf * sgp.G) {
        const uint32_t n = fdiv(sgp.fG, t);
        int i, j, k;
        node_ijk(Mf, n, i, j, k);
        if (node_bnd(Mf, i, j, k)) continue;
        int ca[2], cb[2], cc[2];
        T wa[2], wb[2], wc[2];
        const int na = mg_node_terms<T>(Lf.ax, i, ca, wa);
        const int nb = mg_node_terms<T>(Lf.ay, j, cb, wb);
        const int nc = mg_node_terms<T>(Lf.az, k, cc, wc);
        CV<T, VS> acc;
        cvzero<T, VS>(acc);
        for (int c = 0; c < nc; c++)
            for (int b = 0; b < nb; b++)
                for (int a = 0; a < na; a++) {
                    const uint32_t cn = ((uint32_t)cc[c] * cy1 + (uint32_t)cb[b]) * cx1 + (uint32_t)ca[a];
                    const T w = wa[a] * wb[b] * wc[c];
                    CV<T, VS> v;
                    cvld<T, VS>(v, psic + (size_t)cn * ns + s0);
#pragma unroll
                    for (int u = 0; u < VS; u++) {
                        acc.v[u].x += w * v.v[u].x;
                        acc.v[u].y += w * v.v[u].y;
                    }
                }
        const size_t g = (size_t)n * ns + s0;
        CV<T, VS> pv;
        cvldw<T, VS>(pv, psif + g);
#pragma unroll
        for (int u = 0; u < VS; u++) pv.v[u] = pv.v[u] + acc.v[u];
        cvst_m<T, VS>(psif + g, pv, S.act);
    }
}

// Krylov side of the split: psi_x += alpha psi_y + omega psi_z (this
// iteration's BiCGStab scalars; before k_bicg_upd_v retires converged systems)
template <class T, int VS>
__global__ void k_split_psi_upd_v(SysG sgp, const KState* st, uint32_t np, cplx<T>* __restrict__ px,
                                  const cplx<T>* __restrict__ py, const cplx<T>* __restrict__ pz) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    const SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (!S.act) return;
    cplx<T> al[VS], om[VS];
#pragma unroll
    for (int u = 0; u < VS; u++) {
        al[u] = cst<T>(st[s0 + u].alpha);
        om[u] = cst<T>(st[s0 + u].omega);
    }
    SFDX_GRID_LOOP(t, np * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> a, y, z;
        cvldw<T, VS>(a, px + g);
        cvld<T, VS>(y, py + g);
        cvld<T, VS>(z, pz + g);
#pragma unroll
        for (int u = 0; u < VS; u++) a.v[u] = a.v[u] + cmul<T>(al[u], y.v[u]) + cmul<T>(om[u], z.v[u]);
        cvst_m<T, VS>(px + g, a, S.act);
    }
}

// x64 += G psi (FP64) on interior edges: the nodal part of the complex64
// partial solution folded into the FP64 solution.  ALL: every system that is
// not NaN (the final fold), else the active ones (reliable updates), as k_flush_v.
template <class T, int VS, bool ALL>
__global__ void k_flush_psi_v(Lev<double> L, Mesh M, SysG sgp, const KState* st, double2* __restrict__ x64,
                              const cplx<T>* __restrict__ psi) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (ALL) {
        S.act = 0;
#pragma unroll
        for (int v = 0; v < VS; v++) S.act |= (st[s0 + v].status != ST_NAN ? 1u : 0u) << v;
    }
    if (!S.act) return;
    const uint32_t nx1 = M.nx + 1, pl = nx1 * (M.ny + 1);
    SFDX_GRID_LOOP(t, M.nl * sgp.G) {
        const uint32_t e = fdiv(sgp.fG, t);
        int i, j, k;
        const int o = mdecode(M, e, i, j, k);
        if (mbnd(M, o, i, j, k)) continue;
        const uint32_t n0 = ((uint32_t)k * (M.ny + 1) + j) * nx1 + i;
        uint32_t n1;
        double rl;
        if (o == OX) { n1 = n0 + 1; rl = __ldg(L.ax.rh + i); }
        else if (o == OY) { n1 = n0 + nx1; rl = __ldg(L.ay.rh + j); }
        else { n1 = n0 + pl; rl = __ldg(L.az.rh + k); }
        const size_t g = (size_t)e * ns + s0;
        CV<T, VS> a, b;
        cvld<T, VS>(a, psi + (size_t)n0 * ns + s0);
        cvld<T, VS>(b, psi + (size_t)n1 * ns + s0);
        CV<double, VS> xv;
        cvldw<double, VS>(xv, x64 + g);
#pragma unroll
        for (int u = 0; u < VS; u++)
            xv.v[u] = make_double2(xv.v[u].x + rl * ((double)b.v[u].x - (double)a.v[u].x),
                                   xv.v[u].y + rl * ((double)b.v[u].y - (double)a.v[u].y));
        cvst_m<double, VS>(x64 + g, xv, S.act);
    }
}
// psi = 0 for the systems k_flush_psi_v<T, VS, ALL> folded
template <class T, int VS, bool ALL>
__global__ void k_psi_zero_v(SysG sgp, const KState* st, uint32_t np, cplx<T>* __restrict__ psi) {
    const int ns = sgp.ns, s0 = (threadIdx.x % sgp.G) * VS;
    SysV<T, VS> S = load_sys<T, VS>(st, s0);
    if (ALL) {
        S.act = 0;
#pragma unroll
        for (int v = 0; v < VS; v++) S.act |= (st[s0 + v].status != ST_NAN ? 1u : 0u) << v;
    }
    if (!S.act) return;
    SFDX_GRID_LOOP(t, np * sgp.G) {
        const size_t g = (size_t)fdiv(sgp.fG, t) * ns + s0;
        CV<T, VS> z;
        cvzero<T, VS>(z);
        cvst_m<T, VS>(psi + g, z, S.act);
    }
}

// A (y + G psi) = A y - i wm Ms g with g = G psi materialised (k_mg_xpg_v):
// the row's operator on y plus the mass row on g, boundary rows y
template <class T, int VS>
__device__ __forceinline__ void split_row(const Lev<T>& L, const Mesh& M, int o, uint32_t e, int i, int j, int k,
                                          const cplx<T>* y, const cplx<T>* gv, int ns, int s0, const T (&wm)[VS],
                                          CV<T, VS>& val) {
    CV<T, VS> ye, mq, zb;
    cvld<T, VS>(ye, y + (size_t)e * ns + s0);
    row_apply<T, VS>(L, M, o, e, i, j, k, y, ns, s0, wm, ye, val);
    cvzero<T, VS>(zb);
    if (o == OX) mg_mass_row<T, VS, OX>(L, M, e, i, j, k, gv, ns, s0, wm, zb, mq);
    else if (o == OY) mg_mass_row<T, VS, OY>(L, M, e, i, j, k, gv, ns, s0, wm, zb, mq);
    else mg_mass_row<T, VS, OZ>(L, M, e, i, j, k, gv, ns, s0, wm, zb, mq);
#pragma unroll
    for (int u = 0; u < VS; u++) val.v[u] = val.v[u] - mq.v[u];  // mq = i wm Ms g
}

// k_bicg_v_v on the split vector: v = A (y + G psi_y) ; alpha = rho / <rhat, v>
template <class T, int VS>
__global__ void k_bicg_v_split_v(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ y,
                                 const cplx<T>* __restrict__ gy, cplx<T>* __restrict__ v,
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
            CV<T, VS> val, h;
            split_row<T, VS>(L, M, o, e, i, j, k, y, gy, ns, s0, S.wm, val);
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
        if (!isfinite(st[ss].alpha.x) || !isfinite(st[ss].alpha.y)) {
            st[ss].active = 0;
            st[ss].status = ST_BREAK;
        }
    }
}

// k_bicg_t_v on the split vector: t = A (z + G psi_z) ; omega = <t,s>/<t,t>
template <class T, int VS>
__global__ void k_bicg_t_split_v(Lev<T> L, Mesh M, SysG sgp, KState* st, const cplx<T>* __restrict__ z,
                                 const cplx<T>* __restrict__ gz, cplx<T>* __restrict__ tv,
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
            CV<T, VS> val, ss;
            split_row<T, VS>(L, M, o, e, i, j, k, z, gz, ns, s0, S.wm, val);
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

}  // namespace sfdx
