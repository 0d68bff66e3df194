// sfdx_excmg.cuh -- EXCMG transfer kernels: conductivity coarsening
// (mesh_coarsen, fdfe_main.f90:18-84) and the extrapolation-interpolation
// guess (extint_v / quad_interp_e / cubic_interp / cal_coef / lbf,
// excmg.f90:9-77, 357-772).
//
// The reference builds, for every 2m-cell block of the output mesh, the dense
// ((2m+1)^2*2m) x ((m+1)^2*m) matrix of tensor-product Lagrange weights.
// Here each output edge evaluates its three 1-D Lagrange bases (degree m
// across the edge, m-1 along it) directly from the node coordinates, and the
// sum over the block's coarse edges runs in the reference's column order.
#pragma once
#include "sfdx_device.cuh"

namespace sfdx {

// mesh_coarsen: ncont(coarse cell) = sum_fine sigma * v_fine / v_coarse.
// quirk: fine index ((m-1)asf+r)*..+((j-1)asf+s)*.. as in the reference (one
// plane and one row too far; row overflow wraps into the next plane, a read
// past the last plane is clamped back into it).
static __global__ void k_coarsen(int nx0, int ny0, int nz0, const double* __restrict__ a, const double* __restrict__ b,
                          const double* __restrict__ c, const double* __restrict__ a1, const double* __restrict__ b1,
                          const double* __restrict__ c1, int asf, int quirk, const double* __restrict__ sig0,
                          double* __restrict__ sig1) {
    const int nx = nx0 / asf, ny = ny0 / asf, nz = nz0 / asf;
    const int64_t ne = (int64_t)nx * ny * nz, ncell0 = (int64_t)nx0 * ny0 * nz0, plane0 = (int64_t)nx0 * ny0;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < ne; q += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(q % nx) + 1;
        int j = (int)((q / nx) % ny) + 1;
        int m = (int)(q / ((int64_t)nx * ny)) + 1;
        double vbig = a1[i - 1] * b1[j - 1] * c1[m - 1];
        double t[6] = {0, 0, 0, 0, 0, 0};
        for (int r = 1; r <= asf; r++)
            for (int s = 1; s <= asf; s++)
                for (int tt = 1; tt <= asf; tt++) {
                    int64_t ind;
                    if (quirk) {
                        ind = ((int64_t)(m - 1) * asf + r) * nx * ny * asf * asf + ((int64_t)(j - 1) * asf + s) * nx * asf +
                              (int64_t)(i - 1) * asf + tt;
                        while (ind > ncell0) ind -= plane0;
                    } else {
                        ind = ((int64_t)(m - 1) * asf + r - 1) * plane0 + ((int64_t)(j - 1) * asf + s - 1) * nx0 +
                              (int64_t)(i - 1) * asf + tt;
                    }
                    double vs = a[(i - 1) * asf + tt - 1] * b[(j - 1) * asf + s - 1] * c[(m - 1) * asf + r - 1];
                    for (int cc = 0; cc < 6; cc++) t[cc] += sig0[(int64_t)cc * ncell0 + ind - 1] * vs;
                }
        for (int cc = 0; cc < 6; cc++) sig1[(int64_t)cc * ne + q] = t[cc] / vbig;
    }
}

// Lagrange basis (lbf, excmg.f90:754-772)
template <int NP>
__device__ __forceinline__ void lagrange(const double* cx, double x, double* w) {
#pragma unroll
    for (int id = 0; id < NP; id++) {
        double num = 1.0, den = 1.0;
#pragma unroll
        for (int q = 0; q < NP; q++)
            if (q != id) {
                num = num * (x - cx[q]);
                den = den * (cx[id] - cx[q]);
            }
        w[id] = num / den;
    }
}

// Node block of node position p: the later block owns a shared face (the
// reference writes blocks in increasing order); -1 if not covered.
__device__ __forceinline__ int node_block(int p, int bs, int nb) {
    int bI = p / bs;
    if (bI < nb) return bI;
    return (p == nb * bs) ? nb - 1 : -1;
}

// Interpolate the coarse-mesh edge field uc (mesh nx/2 x ny/2 x nz/2) to the
// fine mesh (nx, ny, nz) with blocks of 2M fine cells.  X, Y, Z: fine node
// coordinates.  Fine edges outside complete blocks are set to zero (the
// reference leaves them at their initial zero).
template <class T, int M>
__global__ void k_interp(int nx, int ny, int nz, const double* __restrict__ X, const double* __restrict__ Y,
                         const double* __restrict__ Z, int mid_quirk, int ns, const cplx<T>* __restrict__ uc,
                         cplx<T>* __restrict__ uf) {
    const int bs = 2 * M;
    const int nbx = nx / bs, nby = ny / bs, nbz = nz / bs;
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1), ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    const int64_t cxnl = (int64_t)cx * (cy + 1) * (cz + 1), cynl = (int64_t)(cx + 1) * cy * (cz + 1);
    // one thread per fine edge and group of up to SG systems: the Lagrange
    // weights are computed once per group (the same products, in the same
    // order, for every system: results do not depend on the grouping)
    constexpr int SG = 4;
    const int ngrp = (ns + SG - 1) / SG;
    const int64_t W = nl * ngrp;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s0 = (int)(g % ngrp) * SG;
        const int cnt = min(SG, ns - s0);
        const int64_t e = g / ngrp;
        cplx<T>* out = uf + e * ns + s0;
        int o, i, j, k;
        if (e < xnl) {
            o = 0; i = (int)(e % nx); int64_t r = e / nx; j = (int)(r % (ny + 1)); k = (int)(r / (ny + 1));
        } else if (e < xnl + ynl) {
            int64_t f = e - xnl; o = 1; i = (int)(f % (nx + 1)); int64_t r = f / (nx + 1); j = (int)(r % ny); k = (int)(r / ny);
        } else {
            int64_t f = e - xnl - ynl; o = 2; i = (int)(f % (nx + 1)); int64_t r = f / (nx + 1); j = (int)(r % (ny + 1)); k = (int)(r / (ny + 1));
        }
        // along-edge position/axis and the two transverse node positions
        int pe, p1, p2, nbe, nb1, nb2;
        const double *Ce, *C1, *C2;
        if (o == 0) { pe = i; p1 = j; p2 = k; nbe = nbx; nb1 = nby; nb2 = nbz; Ce = X; C1 = Y; C2 = Z; }
        else if (o == 1) { pe = j; p1 = i; p2 = k; nbe = nby; nb1 = nbx; nb2 = nbz; Ce = Y; C1 = X; C2 = Z; }
        else { pe = k; p1 = i; p2 = j; nbe = nbz; nb1 = nbx; nb2 = nby; Ce = Z; C1 = X; C2 = Y; }
        int be = pe / bs;
        int b1 = node_block(p1, bs, nb1), b2 = node_block(p2, bs, nb2);
        if (be >= nbe || b1 < 0 || b2 < 0) {
            for (int u = 0; u < cnt; u++) out[u] = zero<T>();
            continue;
        }
        double cx1[M + 1], cx2[M + 1], cx3[M];
        for (int q = 0; q <= M; q++) {
            cx1[q] = C1[b1 * bs + 2 * q];
            cx2[q] = C2[b2 * bs + 2 * q];
        }
        for (int q = 0; q < M; q++)
            cx3[q] = mid_quirk ? (Ce[be * bs + 2 * q] + Ce[be * bs + 2 * q + 1]) / 2
                               : (Ce[be * bs + 2 * q] + Ce[be * bs + 2 * q + 2]) / 2;
        double w1[M + 1], w2[M + 1], w3[M];
        lagrange<M + 1>(cx1, C1[p1], w1);
        lagrange<M + 1>(cx2, C2[p2], w2);
        lagrange<M>(cx3, (Ce[pe] + Ce[pe + 1]) / 2, w3);
        // coarse edge (ce along, c1 across-1, c2 across-2) -> coarse index
        const int ce0 = be * M, c10 = b1 * M, c20 = b2 * M;
        double ar[SG], ai[SG];
#pragma unroll
        for (int u = 0; u < SG; u++) ar[u] = ai[u] = 0.0;
        for (int kk = 0; kk < M; kk++)
            for (int jj = 0; jj <= M; jj++)
                for (int ii = 0; ii <= M; ii++) {
                    double w = w1[ii] * w2[jj] * w3[kk];
                    int64_t ci;
                    if (o == 0)
                        ci = ((int64_t)(c20 + jj) * (cy + 1) + (c10 + ii)) * cx + (ce0 + kk);
                    else if (o == 1)
                        ci = cxnl + ((int64_t)(c20 + jj) * cy + (ce0 + kk)) * (cx + 1) + (c10 + ii);
                    else
                        ci = cxnl + cynl + ((int64_t)(ce0 + kk) * (cy + 1) + (c20 + jj)) * (cx + 1) + (c10 + ii);
                    const cplx<T>* up = uc + ci * ns + s0;
#pragma unroll
                    for (int u = 0; u < SG; u++)
                        if (u < cnt) {
                            const cplx<T> v = up[u];
                            ar[u] += w * (double)v.x;
                            ai[u] += w * (double)v.y;
                        }
                }
        for (int u = 0; u < cnt; u++) out[u] = mk<T>((T)ar[u], (T)ai[u]);
    }
}

// Richardson step of extint_v: u = (1 + 2^-2) u1 - 2^-2 u  (order = 2)
template <class T>
__global__ void k_extrapolate(int64_t n, const cplx<T>* __restrict__ u1, cplx<T>* __restrict__ u) {
    const double co1 = 1.25, co2 = 0.25;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
        cplx<T> a = u1[g], b = u[g];
        u[g] = mk<T>((T)(co1 * a.x - co2 * b.x), (T)(co1 * a.y - co2 * b.y));
    }
}

// Flags any non-zero off-diagonal conductivity (selects the anisotropic
// cross terms of the operator).
static __global__ void k_any_offdiag(int64_t ncell, const double* __restrict__ sig, int* flag) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * ncell; q += (int64_t)gridDim.x * blockDim.x)
        if (sig[3 * ncell + q] != 0.0) {
            *flag = 1;
            return;
        }
}

// NaN check of a vector (extint_v excmg.f90:73-75 / the RHS check at
// fdfe_main.f90:1398-1403).
template <class T>
__global__ void k_nan_check(int64_t n, const cplx<T>* __restrict__ v, int* flag) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
        cplx<T> a = v[g];
        if (isnan(a.x) || isnan(a.y)) {
            *flag = 1;
            return;
        }
    }
}

}  // namespace sfdx
