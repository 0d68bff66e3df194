// sfdx_adjoint.cu -- gradient of the impedance misfit with respect to the cell
// conductivities: one adjoint solve per frequency and polarisation (all in one
// batch, through the same Krylov / multigrid machinery as the forward solve)
// and a fused per-cell kernel that contracts forward and adjoint fields.
//
// The reference has no inversion path; this is the differentiation part of
// the forward-solve interface.  Derivation (interior rows I, Dirichlet edges
// B held at the 1-D background values):
//   K_II(s) x_I + K_IB(s) p_B = 0,   phi = phi(x),   d phi = 2 Re(g^T dx)
//   => d phi / d s = -2 Re( lambda^T (dK/ds) x ),   K_II^T lambda = g_I.
// The interior rows are complex symmetric after weighting with the edge dual
// volumes V (V K_II = K_II^T V), so lambda = V mu with K_II mu = V^-1 g_I: the
// adjoint system is the forward operator with a right-hand side on the
// receiver planes and zero Dirichlet data.  dK/ds = -i w mu0 dM/ds, and V dM/ds
// for one cell and component is a small symmetric matrix over the cell's 12
// edges (vol/4 on the diagonal for xx, yy, zz; vol/8 between each pair of
// differently oriented edges that share a face level for xy, xz, yz), which
// is the conductivity part of the rows of fd_assemb (fdfe_main.f90:248-393)
// weighted by V.
#include <cuda_runtime.h>

#include <complex>
#include <cstring>
#include <vector>

#include "sfdx.h"
#include "sfdx_host.h"
#include "sfdx_kernels.cuh"
#include "sfdx_plan.h"

namespace sfdx {

// grad[q][c] = -2 sum_s wm_s Im( S_q,s(c) ),  S = sum over the cell's edge pairs
// of (V dM/ds_q)_{ee'} mu_e x_e'  (mu zero on the Dirichlet edges)
__global__ void k_sigma_grad(Lev<double> L, int ns, const double* __restrict__ wm, const double2* __restrict__ xf,
                             const double2* __restrict__ mu, double* __restrict__ grad) {
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < L.ncell;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int ci = (int)(c % nx);
        const int64_t r = c / nx;
        const int cj = (int)(r % ny), ck = (int)(r / ny);
        const double vol = 1.0 / (__ldg(L.ax.rh + ci) * __ldg(L.ay.rh + cj) * __ldg(L.az.rh + ck));
        // edges of the cell: ex[dj][dk], ey[di][dk], ez[di][dj]; interior flags
        int64_t ex[2][2], ey[2][2], ez[2][2];
        bool ix[2][2], iy[2][2], iz[2][2];
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int v = 0; v < 2; v++) {
                ex[u][v] = eidx(L, OX, ci, cj + u, ck + v);
                ix[u][v] = !(cj + u == 0 || cj + u == ny || ck + v == 0 || ck + v == nz);
                ey[u][v] = eidx(L, OY, ci + u, cj, ck + v);
                iy[u][v] = !(ci + u == 0 || ci + u == nx || ck + v == 0 || ck + v == nz);
                ez[u][v] = eidx(L, OZ, ci + u, cj + v, ck);
                iz[u][v] = !(ci + u == 0 || ci + u == nx || cj + v == 0 || cj + v == ny);
            }
        double g[6] = {0, 0, 0, 0, 0, 0};
        for (int s = 0; s < ns; s++) {
            double2 Xx[2][2], Xy[2][2], Xz[2][2], Mx[2][2], My[2][2], Mz[2][2];
            const double2 z0 = make_double2(0.0, 0.0);
#pragma unroll
            for (int u = 0; u < 2; u++)
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    Xx[u][v] = __ldg(xf + ex[u][v] * ns + s);
                    Xy[u][v] = __ldg(xf + ey[u][v] * ns + s);
                    Xz[u][v] = __ldg(xf + ez[u][v] * ns + s);
                    Mx[u][v] = ix[u][v] ? __ldg(mu + ex[u][v] * ns + s) : z0;
                    My[u][v] = iy[u][v] ? __ldg(mu + ey[u][v] * ns + s) : z0;
                    Mz[u][v] = iz[u][v] ? __ldg(mu + ez[u][v] * ns + s) : z0;
                }
            double2 S[6];
#pragma unroll
            for (int q = 0; q < 6; q++) S[q] = z0;
#pragma unroll
            for (int u = 0; u < 2; u++)
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    S[0] = S[0] + cmul<double>(Mx[u][v], Xx[u][v]);
                    S[1] = S[1] + cmul<double>(My[u][v], Xy[u][v]);
                    S[2] = S[2] + cmul<double>(Mz[u][v], Xz[u][v]);
                }
            // xy: Ex (dj, dk) with Ey (di, dk) on the same z level dk
#pragma unroll
            for (int v = 0; v < 2; v++) {
                const double2 mxs = Mx[0][v] + Mx[1][v], xxs = Xx[0][v] + Xx[1][v];
                const double2 mys = My[0][v] + My[1][v], xys = Xy[0][v] + Xy[1][v];
                S[3] = S[3] + cmul<double>(mxs, xys) + cmul<double>(mys, xxs);
            }
            // xz: Ex (dj, dk) with Ez (di, dj) on the same y level dj
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const double2 mxs = Mx[u][0] + Mx[u][1], xxs = Xx[u][0] + Xx[u][1];
                const double2 mzs = Mz[0][u] + Mz[1][u], xzs = Xz[0][u] + Xz[1][u];
                S[4] = S[4] + cmul<double>(mxs, xzs) + cmul<double>(mzs, xxs);
            }
            // yz: Ey (di, dk) with Ez (di, dj) on the same x level di
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const double2 mys = My[u][0] + My[u][1], xys = Xy[u][0] + Xy[u][1];
                const double2 mzs = Mz[u][0] + Mz[u][1], xzs = Xz[u][0] + Xz[u][1];
                S[5] = S[5] + cmul<double>(mys, xzs) + cmul<double>(mzs, xys);
            }
            const double w = -2.0 * __ldg(wm + s);
#pragma unroll
            for (int q = 0; q < 6; q++) g[q] += w * S[q].y;
        }
#pragma unroll
        for (int q = 0; q < 6; q++) grad[(size_t)q * L.ncell + c] = g[q] * vol * (q < 3 ? 0.25 : 0.125);
    }
}

// dual volume of an interior edge (0 on the Dirichlet faces): length x the two
// transverse half-spacing sums
static double dual_volume(const std::vector<double>& h0, const std::vector<double>& h1, const std::vector<double>& h2,
                          int i, int j, int k) {
    const int n1 = (int)h1.size(), n2 = (int)h2.size();
    if (j == 0 || j == n1 || k == 0 || k == n2) return 0.0;
    return h0[i] * (h1[j - 1] + h1[j]) * 0.5 * (h2[k - 1] + h2[k]) * 0.5;
}

// V^-1 g of the adjoint source on the receiver planes of level L (interior
// edges), written interleaved [edge][system] into P.b64 (zero elsewhere).
// cf: [nf][nrec][2][4] receiver cotangents.
static int adjoint_rhs(Plan& P, const Level& L, int nrec, const double* recv, int transpose,
                       const std::vector<std::complex<double>>& cf) {
    const int ns = P.ns, nx = L.nx, ny = L.ny, m = L.nair;
    const size_t pex = (size_t)nx * (ny + 1), pey = (size_t)(nx + 1) * ny, pez = (size_t)(nx + 1) * (ny + 1);
    const size_t per = 2 * pex + 2 * pey + pez;
    std::vector<std::complex<double>> gs(per * ns, 0.0);
    for (int f = 0; f < P.nf; f++) {
        SurfaceGrad sg;
        sg.nx = nx;
        sg.ny = ny;
        for (int p = 0; p < 2; p++) {
            const size_t o = (size_t)(2 * f + p) * per;
            sg.exs[p] = gs.data() + o;
            sg.eys[p] = gs.data() + o + 2 * pex;
            sg.ezs[p] = gs.data() + o + 2 * pex + 2 * pey;
        }
        RC(impedance_adjoint_source(sg, m, L.a.data(), L.b.data(), L.c.data(), P.freq[f], nrec, recv, transpose,
                                    cf.data() + (size_t)f * nrec * 8));
    }
    std::vector<std::complex<double>> rx(2 * pex * ns), ry(2 * pey * ns), rz(pez * ns);
    for (int s = 0; s < ns; s++) {
        const std::complex<double>* g = gs.data() + (size_t)s * per;
        for (int pl = 0; pl < 2; pl++)
            for (int j = 0; j <= ny; j++)
                for (int i = 0; i < nx; i++) {
                    const size_t q = (size_t)pl * pex + (size_t)j * nx + i;
                    const double v = dual_volume(L.a, L.b, L.c, i, j, m + pl);
                    rx[q * ns + s] = v > 0 ? g[q] / v : 0.0;
                }
        for (int pl = 0; pl < 2; pl++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i <= nx; i++) {
                    const size_t q = (size_t)pl * pey + (size_t)j * (nx + 1) + i;
                    const double v = dual_volume(L.b, L.a, L.c, j, i, m + pl);
                    ry[q * ns + s] = v > 0 ? g[2 * pex + q] / v : 0.0;
                }
        for (int j = 0; j <= ny; j++)
            for (int i = 0; i <= nx; i++) {
                const size_t q = (size_t)j * (nx + 1) + i;
                const double v = dual_volume(L.c, L.a, L.b, m, i, j);
                rz[q * ns + s] = v > 0 ? g[2 * pex + 2 * pey + q] / v : 0.0;
            }
    }
    double2* b = P.b64.as<double2>();
    CK(cudaMemsetAsync(P.b64.p, 0, (size_t)L.nl * ns * sizeof(double2), P.st));
    CK(cudaMemcpyAsync(b + (size_t)m * pex * ns, rx.data(), rx.size() * 16, cudaMemcpyHostToDevice, P.st));
    CK(cudaMemcpyAsync(b + ((size_t)L.xnl + (size_t)m * pey) * ns, ry.data(), ry.size() * 16, cudaMemcpyHostToDevice,
                       P.st));
    CK(cudaMemcpyAsync(b + ((size_t)L.xnl + L.ynl + (size_t)m * pez) * ns, rz.data(), rz.size() * 16,
                       cudaMemcpyHostToDevice, P.st));
    // the host staging vectors go out of scope: finish the copies first
    CK(cudaStreamSynchronize(P.st));
    return SFDX_OK;
}

int misfit_grad(Plan& P, int nrec, const double* recv, const double* zobs, const double* wts, double tol,
                double* misfit, double* zpred, double* grad, bool grad_on_device, int* adj_iters, double* adj_relres) {
    if (!P.solution_current()) return SFDX_ERR_ARG;  // no solve since the conductivity changed
    const Level& F = P.lev[P.nlev - 1];
    const int ns = P.ns, nx = F.nx, ny = F.ny, nz = F.nz, m = F.nair;
    if (m < 1 || m + 2 > nz) return SFDX_ERR_MESH;
    const size_t nfine = (size_t)F.nl * ns * sizeof(double2);
    // surface planes of every system (system-major copy of the solution)
    const size_t pex = (size_t)nx * (ny + 1), pey = (size_t)(nx + 1) * ny, pez = (size_t)(nx + 1) * (ny + 1);
    const size_t per = 2 * pex + 2 * pey + pez;
    std::vector<std::complex<double>> surf(per * ns);
    const std::complex<double>* dev = reinterpret_cast<const std::complex<double>*>(P.ex_out.p);
    for (int s = 0; s < ns; s++) {
        const std::complex<double>* x = dev + (size_t)s * F.nl;
        std::complex<double>* base = surf.data() + (size_t)s * per;
        CK(cudaMemcpyAsync(base, x + (size_t)m * pex, 2 * pex * 16, cudaMemcpyDeviceToHost, P.st));
        CK(cudaMemcpyAsync(base + 2 * pex, x + F.xnl + (size_t)m * pey, 2 * pey * 16, cudaMemcpyDeviceToHost, P.st));
        CK(cudaMemcpyAsync(base + 2 * pex + 2 * pey, x + F.xnl + F.ynl + (size_t)m * pez, pez * 16,
                           cudaMemcpyDeviceToHost, P.st));
    }
    CK(cudaStreamSynchronize(P.st));
    double phi = 0;
    const int transpose = (P.o.quirks & SFDX_QUIRK_RX_TRANSPOSE) ? 1 : 0;
    std::vector<std::complex<double>> cf((size_t)P.nf * nrec * 8);
    for (int f = 0; f < P.nf; f++) {
        SurfaceView sv;
        sv.nx = nx;
        sv.ny = ny;
        sv.nair = m;
        for (int p = 0; p < 2; p++) {
            const size_t o = (size_t)(2 * f + p) * per;
            sv.exs[p] = surf.data() + o;
            sv.eys[p] = surf.data() + o + 2 * pex;
            sv.ezs[p] = surf.data() + o + 2 * pex + 2 * pey;
        }
        RC(impedance_cotangents(sv, F.a.data(), F.b.data(), F.c.data(), P.freq[f], nrec, recv, transpose,
                                zobs + (size_t)f * nrec * 4, wts ? wts + (size_t)f * nrec * 2 : nullptr, &phi,
                                zpred ? zpred + (size_t)f * nrec * 4 : nullptr, cf.data() + (size_t)f * nrec * 8));
    }
    *misfit = phi;
    if (!grad) return SFDX_OK;  // misfit (and predicted impedances) only
    // forward fields of the last solve (x64 is about to hold the adjoint)
    if (!P.xf_valid) {
        RC(P.xf.alloc(nfine));
        CK(cudaMemcpyAsync(P.xf.p, P.x64.p, nfine, cudaMemcpyDeviceToDevice, P.st));
        P.xf_valid = true;
    }
    // Adjoint solve on the finest mesh from zero.  (An EXCMG cascade with the
    // same receiver functional on the coarse meshes gives a worse start: the
    // extrapolation amplifies the coarse-grid error of the point-like receiver
    // sources -- on the 80x80x80 GRF adjoint case it needed more iterations than the zero guess.)
    std::vector<int> its, status;
    RC(adjoint_rhs(P, F, nrec, recv, transpose, cf));
    CK(cudaMemsetAsync(P.x64.p, 0, nfine, P.st));
    RC(solve_level(P, F, tol > 0 ? tol : P.o.eps, P.o.maxit_plain, false, its, status));
    int rc_conv = SFDX_OK;
    for (int s = 0; s < ns; s++) {
        if (adj_iters) adj_iters[s] = its[s];
        if (status[s] != ST_CONV) rc_conv = status[s] == ST_NAN ? SFDX_ERR_NAN : SFDX_ERR_NOCONV;
    }
    if (adj_relres) {
        std::vector<double> rel(ns);
        RC(true_residual(P, F, P.b64.as<double2>(), P.x64.as<double2>(), rel.data(), nullptr));
        for (int s = 0; s < ns; s++) adj_relres[s] = rel[s];
    }
    // per-cell contraction
    DBuf gd;
    double* gout = grad;
    if (!grad_on_device) {
        RC(gd.alloc((size_t)6 * F.ncell * sizeof(double)));
        gout = gd.as<double>();
    }
    KL(k_sigma_grad<<<grid_for(F.ncell, 128, 8), 128, 0, P.st>>>(F.lev<double>(), ns, P.d_wm.as<double>(),
                                                                 P.xf.as<double2>(), P.x64.as<double2>(), gout));
    CK(cudaGetLastError());
    if (!grad_on_device)
        CK(cudaMemcpyAsync(grad, gout, (size_t)6 * F.ncell * sizeof(double), cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    return rc_conv;
}

}  // namespace sfdx
