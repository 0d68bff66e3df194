// sfdx_host.cpp -- host-side parts of the forward-solve path that are O(nz)
// or O(nx*ny) and stay in FP64 on the CPU:
//   * the analytic 1-D anisotropic layered field (mt1d_anl,
//     model_selec.f90:266-401) that feeds the Dirichlet boundary values,
//   * the impedance evaluation (post_process + arho_interp2,
//     fdfe_main.f90:549-790),
//   * the reference's model/data/result file formats (file_opt.f90:8-158).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sfdx.h"
#include "sfdx_host.h"

namespace sfdx {

typedef std::complex<double> zd;
static const double kPi = 3.141592653589793238462643;
static const double kMu = 4.0 * 3.141592653589793238462643 * 1e-7;
#define HRC(x)                   \
    do {                         \
        int rc_ = (x);           \
        if (rc_) return rc_;     \
    } while (0)

// -------------------------------------------------------------------- mt1d
// Propagator form of Pek & Santos (2002) for a stack of anisotropic layers:
// a 4x4 layer matrix S_i maps (Ex, Ey, Hx, Hy)-like field vectors from the
// bottom of layer i to its top; the bottom half-space fixes the two decaying
// modes and the top E is normalised to (1,0) (xy) or (0,1) (yx).
static void mat4(const zd* A, const zd* B, zd* C) {
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            zd s = 0;
            for (int k = 0; k < 4; k++) s += A[i * 4 + k] * B[k * 4 + j];
            C[i * 4 + j] = s;
        }
}

int mt1d_anl(double ff, int nz, const double* conv, const double* c, zd* ex, zd* hx, zd* imp) {
    if (nz <= 0 || !conv || !c || !ex) return SFDX_ERR_ARG;
    auto CV = [&](int i, int m) { return conv[(size_t)(m - 1) * nz + (i - 1)]; };
    std::vector<zd> sprod((size_t)16 * (nz + 1), zd(0, 0));
    zd m[16];
    for (auto& q : m) q = 0;
    const double w = 2 * kPi * ff;
    const zd iwm = zd(0, 1) * w * kMu;
    for (int i = 0; i < 4; i++) sprod[(size_t)nz * 16 + i * 4 + i] = 1.0;
    for (int i = nz; i >= 1; i--) {
        double axx = CV(i, 1) - CV(i, 5) * CV(i, 5) / CV(i, 3);
        double ayy = CV(i, 2) - CV(i, 6) * CV(i, 6) / CV(i, 3);
        double axy = CV(i, 4) - CV(i, 5) * CV(i, 6) / CV(i, 3);
        double ada = axx + ayy, add = axx - ayy;
        double da12 = std::sqrt(add * add + 4 * axy * axy);
        if (add < 0) da12 = -da12;
        double a1 = (ada + da12) / 2, a2 = (ada - da12) / 2;
        zd kp = std::sqrt(-iwm) * std::sqrt(a1), km = std::sqrt(-iwm) * std::sqrt(a2);
        zd xp = -kp / iwm, xm = -km / iwm;
        double qp = 0, qm = 0;
        if (axy != 0) {
            qp = 2 * axy / (add + da12);
            qm = (add - da12) / axy / 2;
        }
        double qdq = qp * qm, dq = 1 - qdq;
        if (i == nz) {  // bottom half-space: the two downward-decaying modes
            m[0 * 4 + 1] = 1.0;
            m[1 * 4 + 1] = qp;
            m[2 * 4 + 1] = -xp * qp;
            m[3 * 4 + 1] = xp;
            m[0 * 4 + 3] = qm;
            m[1 * 4 + 3] = 1.0;
            m[2 * 4 + 3] = -xm;
            m[3 * 4 + 3] = xm * qm;
        }
        zd t = kp * c[i - 1];
        zd sp = (std::exp(t) - std::exp(-t)) / 2.0, cp = (std::exp(t) + std::exp(-t)) / 2.0;
        t = km * c[i - 1];
        zd sm = (std::exp(t) - std::exp(-t)) / 2.0, cm = (std::exp(t) + std::exp(-t)) / 2.0;
        zd s[16] = {cp - qdq * cm,           -qm * (cp - cm),          qm * (sp / xp - sm / xm), sp / xp - qdq * sm / xm,
                    qp * (cp - cm),          -qdq * cp + cm,           qdq * sp / xp - sm / xm,  qp * (sp / xp - sm / xm),
                    -qp * (xp * sp - xm * sm), qdq * xp * sp - xm * sm, -qdq * cp + cm,          -qp * (cp - cm),
                    xp * sp - qdq * xm * sm, -qm * (xp * sp - xm * sm), qm * (cp - cm),           cp - qdq * cm};
        for (auto& q : s) q /= dq;
        mat4(s, &sprod[(size_t)i * 16], &sprod[(size_t)(i - 1) * 16]);
    }
    zd sm4[16];
    mat4(&sprod[0], m, sm4);
    zd bot[8];
    for (int mode = 0; mode < 2; mode++) {
        zd e0 = mode == 0 ? zd(1, 0) : zd(0, 1);
        zd g11 = sm4[1], g21 = sm4[5], g12 = sm4[3], g22 = sm4[7];
        zd det = g11 * g22 - g12 * g21;
        zd cb[4] = {0, (g22 * e0.real() - g12 * e0.imag()) / det, 0, (-g21 * e0.real() + g11 * e0.imag()) / det};
        zd mc[4];
        for (int r = 0; r < 4; r++) {
            zd a = 0;
            for (int q = 0; q < 4; q++) a += m[r * 4 + q] * cb[q];
            mc[r] = a;
        }
        for (int i = 1; i <= nz + 1; i++) {
            zd f[4];
            for (int r = 0; r < 4; r++) {
                zd a = 0;
                for (int q = 0; q < 4; q++) a += sprod[(size_t)(i - 1) * 16 + r * 4 + q] * mc[q];
                f[r] = a;
            }
            if (mode == 0) {
                ex[i - 1] = f[0];
                if (hx) hx[i - 1] = f[3];
            } else {
                ex[i + nz] = f[1];
                if (hx) hx[i + nz] = f[2];
            }
            if (i == nz + 1)
                for (int r = 0; r < 4; r++) bot[mode * 4 + r] = f[r];
        }
    }
    if (imp) {
        zd t = bot[2] * bot[7] - bot[3] * bot[6];
        imp[0] = (bot[0] * bot[7] - bot[4] * bot[3]) / t;
        imp[1] = (bot[4] * bot[2] - bot[0] * bot[6]) / t;
        imp[2] = (bot[1] * bot[7] - bot[5] * bot[3]) / t;
        imp[3] = (bot[5] * bot[2] - bot[1] * bot[6]) / t;
    }
    for (int q = 0; q < 2 * nz + 2; q++)
        if (std::isnan(std::abs(ex[q]))) return SFDX_ERR_NAN;
    return SFDX_OK;
}

// -------------------------------------------------------------------- impedance
// Surface fields at cell centres of node plane nair+1 from the edge solution
// (fdfe_main.f90:601-683), then a 3x3 quadratic Lagrange interpolation to the
// receivers (arho_interp2, :718-790) and Z from the two polarisations
// (:687-705).  `surf` supplies the few edge planes the evaluation reads.
static double qcoef(double x, const double* x0, int q) {
    if (q == 0) return (x - x0[1]) * (x - x0[2]) / (x0[0] - x0[1]) / (x0[0] - x0[2]);
    if (q == 1) return (x - x0[0]) * (x - x0[2]) / (x0[1] - x0[0]) / (x0[1] - x0[2]);
    return (x - x0[0]) * (x - x0[1]) / (x0[2] - x0[0]) / (x0[2] - x0[1]);
}

// E (x, y) and H (x, y, z) of one polarisation at the cell centres (i, j) of
// the surface, [j*nx + i]: E is the mean of the two surface edges, H = curl E
// / (i w mu) from one-sided differences into the first earth layer.
struct SurfFields {
    std::vector<zd> E[2], H[3];
    void init(size_t n) {
        for (auto& v : E) v.assign(n, 0);
        for (auto& v : H) v.assign(n, 0);
    }
};
static void surface_fields(const SurfaceView& sv, int p, const double* a, const double* b, double cz, zd iwm,
                           SurfFields& F) {
    const int nx = sv.nx, ny = sv.ny;
    F.init((size_t)nx * ny);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t id = (size_t)j * nx + i;
            zd ex0 = (sv.ex(p, 0, i, j) + sv.ex(p, 0, i, j + 1)) / 2.0;
            zd ey0 = (sv.ey(p, 0, i, j) + sv.ey(p, 0, i + 1, j)) / 2.0;
            F.E[0][id] = ex0;
            F.E[1][id] = ey0;
            zd exz = ((sv.ex(p, 1, i, j) + sv.ex(p, 1, i, j + 1)) / 2.0 - ex0) / cz;
            zd ezx = ((sv.ez(p, i + 1, j) + sv.ez(p, i + 1, j + 1)) / 2.0 - (sv.ez(p, i, j + 1) + sv.ez(p, i, j)) / 2.0) / a[i];
            zd eyz = ((sv.ey(p, 1, i, j) + sv.ey(p, 1, i + 1, j)) / 2.0 - ey0) / cz;
            zd ezy = (-(sv.ez(p, i, j) + sv.ez(p, i + 1, j)) / 2.0 + (sv.ez(p, i, j + 1) + sv.ez(p, i + 1, j + 1)) / 2.0) / b[j];
            zd exy = (sv.ex(p, 0, i, j + 1) - sv.ex(p, 0, i, j)) / b[j];
            zd eyx = (sv.ey(p, 0, i + 1, j) - sv.ey(p, 0, i, j)) / a[i];
            F.H[1][id] = (exz - ezx) / iwm;
            F.H[0][id] = (ezy - eyz) / iwm;
            F.H[2][id] = (exy - eyx) / iwm;
        }
}
// Transpose of surface_fields: cotangents dF at the cell centres are
// accumulated onto the edge planes of polarisation p in g (the linear map is
// holomorphic, so no conjugation).
static void surface_fields_adjoint(SurfaceGrad& g, int p, const double* a, const double* b, double cz, zd iwm,
                                   const SurfFields& dF) {
    const int nx = g.nx, ny = g.ny;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t id = (size_t)j * nx + i;
            const zd hx = dF.H[0][id] / iwm, hy = dF.H[1][id] / iwm, hz = dF.H[2][id] / iwm;
            // H_y = (exz - ezx), H_x = (ezy - eyz), H_z = (exy - eyx)
            const zd dexz = hy, dezx = -hy, dezy = hx, deyz = -hx, dexy = hz, deyx = -hz;
            const zd dex0 = dF.E[0][id] - dexz / cz, dey0 = dF.E[1][id] - deyz / cz;
            g.ex(p, 1, i, j) += dexz / cz / 2.0;
            g.ex(p, 1, i, j + 1) += dexz / cz / 2.0;
            g.ey(p, 1, i, j) += deyz / cz / 2.0;
            g.ey(p, 1, i + 1, j) += deyz / cz / 2.0;
            g.ez(p, i + 1, j) += dezx / a[i] / 2.0;
            g.ez(p, i + 1, j + 1) += dezx / a[i] / 2.0;
            g.ez(p, i, j) -= dezx / a[i] / 2.0;
            g.ez(p, i, j + 1) -= dezx / a[i] / 2.0;
            g.ez(p, i, j + 1) += dezy / b[j] / 2.0;
            g.ez(p, i + 1, j + 1) += dezy / b[j] / 2.0;
            g.ez(p, i, j) -= dezy / b[j] / 2.0;
            g.ez(p, i + 1, j) -= dezy / b[j] / 2.0;
            g.ex(p, 0, i, j + 1) += dexy / b[j];
            g.ex(p, 0, i, j) -= dexy / b[j];
            g.ey(p, 0, i + 1, j) += deyx / a[i];
            g.ey(p, 0, i, j) -= deyx / a[i];
            g.ex(p, 0, i, j) += dex0 / 2.0;
            g.ex(p, 0, i, j + 1) += dex0 / 2.0;
            g.ey(p, 0, i, j) += dey0 / 2.0;
            g.ey(p, 0, i + 1, j) += dey0 / 2.0;
        }
}

// cell-centre coordinates (arho_interp2 :729-735)
static void cell_centres(int nx, int ny, const double* a, const double* b, std::vector<double>& aax,
                         std::vector<double>& bby) {
    aax.assign(nx, 0.0);
    bby.assign(ny, 0.0);
    double sa = 0, sb = 0;
    for (int i = 0; i < nx; i++) sa += a[i];
    for (int i = 0; i < ny; i++) sb += b[i];
    aax[0] = (a[0] - sa) / 2;
    bby[0] = (b[0] - sb) / 2;
    for (int i = 2; i <= nx; i++) {
        double s = 0;
        for (int q = 0; q < i - 1; q++) s += a[q];
        aax[i - 1] = -sa / 2 + s + a[i - 1] / 2;
    }
    for (int i = 2; i <= ny; i++) {
        double s = 0;
        for (int q = 0; q < i - 1; q++) s += b[q];
        bby[i - 1] = -sb / 2 + s + b[i - 1] / 2;
    }
}

// The 9 cell centres and weights that interpolate a receiver: id[] for E, Hx
// and Hy (transposed stencil with rd=2), idz[] for Hz.
struct RecvStencil {
    size_t id[9], idz[9];
    double w[9];
};
static int receiver_stencil(int nx, int ny, const std::vector<double>& aax, const std::vector<double>& bby, double xr,
                            double yr, int transpose, RecvStencil& S) {
    int irec = -1, jrec = -1;
    for (int j = 1; j <= nx - 1; j++)
        if (xr >= aax[j - 1] && xr <= aax[j]) { irec = j; break; }
    for (int j = 1; j <= ny - 1; j++)
        if (yr >= bby[j - 1] && yr <= bby[j]) { jrec = j; break; }
    if (irec < 2 || jrec < 2 || irec + 1 > nx || jrec + 1 > ny) return SFDX_ERR_RECEIVER;
    if (transpose && (jrec + 1 > nx || irec + 1 > ny)) return SFDX_ERR_RECEIVER;
    double c1[3], c2[3];
    for (int q = 0; q < 3; q++) c1[q] = qcoef(xr, &aax[irec - 2], q);
    for (int q = 0; q < 3; q++) c2[q] = qcoef(yr, &bby[jrec - 2], q);
    int t = 0;
    for (int mm = 1; mm <= 3; mm++)
        for (int nn = 1; nn <= 3; nn++, t++) {
            S.w[t] = c1[mm - 1] * c2[nn - 1];
            // 1-based (I,J) of the field array
            int I = transpose ? mm + jrec - 2 : mm + irec - 2;
            int J = transpose ? nn + irec - 2 : nn + jrec - 2;
            S.id[t] = (size_t)(J - 1) * nx + (I - 1);
            S.idz[t] = (size_t)(nn + jrec - 3) * nx + (mm + irec - 3);
        }
    return SFDX_OK;
}

// f[p][0..4] = (Ex, Ey, Hx, Hy, Hz) of polarisation p at the receiver
static void receiver_fields(const SurfFields* F, const RecvStencil& S, zd f[2][5]) {
    for (int p = 0; p < 2; p++) {
        for (int q = 0; q < 5; q++) f[p][q] = 0;
        for (int t = 0; t < 9; t++) {
            f[p][0] += S.w[t] * F[p].E[0][S.id[t]];
            f[p][1] += S.w[t] * F[p].E[1][S.id[t]];
            f[p][2] += S.w[t] * F[p].H[0][S.id[t]];
            f[p][3] += S.w[t] * F[p].H[1][S.id[t]];
            f[p][4] += S.w[t] * F[p].H[2][S.idz[t]];
        }
    }
}

static int impedance_from_fields(const SurfFields (&F)[2], int nx, int ny, const double* a, const double* b,
                                 double ff, int nrec, const double* recv, int out_type, int transpose, double* out,
                                 double* tip, zd* fields);

int receiver_stencils(int nx, int ny, const double* a, const double* b, int nrec, const double* recv, int transpose,
                      int* id, int* idz, double* w) {
    std::vector<double> aax, bby;
    cell_centres(nx, ny, a, b, aax, bby);
    for (int r = 0; r < nrec; r++) {
        RecvStencil S;
        HRC(receiver_stencil(nx, ny, aax, bby, recv[r], recv[(size_t)nrec + r], transpose, S));
        for (int t = 0; t < 9; t++) {
            id[(size_t)r * 9 + t] = (int)S.id[t];
            idz[(size_t)r * 9 + t] = (int)S.idz[t];
            w[(size_t)r * 9 + t] = S.w[t];
        }
    }
    return SFDX_OK;
}

int impedance_from_surface(const SurfaceView& sv, const double* a, const double* b, const double* c, double ff,
                           int nrec, const double* recv, int out_type, int transpose, double* out, double* tip,
                           zd* fields) {
    const zd iwm = zd(0, 1) * 2.0 * kPi * ff * kMu;
    SurfFields F[2];
    for (int p = 0; p < 2; p++) surface_fields(sv, p, a, b, c[sv.nair], iwm, F[p]);
    return impedance_from_fields(F, sv.nx, sv.ny, a, b, ff, nrec, recv, out_type, transpose, out, tip, fields);
}

// Receiver plane per surface column with topography (post_process,
// fdfe_main.f90:604-616): inside the window abr = (i1, i2, j1, j2, k1, k2)
// (1-based) the first cell k of k1..k2 whose centre lies at or below the
// surface -topo (elevation, positive up) marks the column's plane; outside the
// window, or with no such cell, the plane is nair.  `reference`: the cell's
// lower node plane (m = k) and the vertical step c(nair+1) for every column, as
// the reference computes them; otherwise its upper plane (m = k - 1, the top of
// the first earth cell, nair on flat ground) and the cell below it (c(m+1)).
int receiver_planes(int nx, int ny, int nz, int nair, const double* c, const int* abr, const double* topo,
                    int reference, int* mcol, double* czcol) {
    if (abr[0] < 1 || abr[1] > nx || abr[0] > abr[1] || abr[2] < 1 || abr[3] > ny || abr[2] > abr[3] ||
        abr[4] < 1 || abr[5] >= nz || abr[4] > abr[5])
        return SFDX_ERR_ARG;
    std::vector<double> ccz(nz);
    double air = 0, acc = 0;
    for (int k = 0; k < nair; k++) air += c[k];
    for (int k = 0; k < nz; k++) {
        acc += c[k];
        ccz[k] = -air + acc - c[k] / 2;
    }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            const size_t id = (size_t)(j - 1) * nx + i - 1;
            mcol[id] = nair;
            czcol[id] = c[nair];
            if (i < abr[0] || i > abr[1] || j < abr[2] || j > abr[3]) continue;
            const double t = topo[(size_t)(j - abr[2]) * (abr[1] - abr[0] + 1) + i - abr[0]];
            for (int k = abr[4]; k <= abr[5]; k++)
                if (ccz[k - 1] >= -t) {
                    mcol[id] = reference ? k : k - 1;
                    if (!reference) czcol[id] = c[k - 1];
                    break;
                }
        }
    return SFDX_OK;
}

// surface_fields with a plane per column: x is the whole field of one
// polarisation (Ex, Ey, Ez blocks of the reference order)
static void surface_fields_cols(const zd* x, int nx, int ny, int nz, const int* mcol, const double* czcol,
                                const double* a, const double* b, zd iwm, SurfFields& F) {
    const size_t xnl = (size_t)nx * (ny + 1) * (nz + 1), ynl = (size_t)(nx + 1) * ny * (nz + 1);
    auto EX = [&](int k, int i, int j) { return x[((size_t)k * (ny + 1) + j) * nx + i]; };
    auto EY = [&](int k, int i, int j) { return x[xnl + ((size_t)k * ny + j) * (nx + 1) + i]; };
    auto EZ = [&](int k, int i, int j) { return x[xnl + ynl + ((size_t)k * (ny + 1) + j) * (nx + 1) + i]; };
    F.init((size_t)nx * ny);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t id = (size_t)j * nx + i;
            const int m = mcol[id];
            const double cz = czcol[id];
            zd ex0 = (EX(m, i, j) + EX(m, i, j + 1)) / 2.0;
            zd ey0 = (EY(m, i, j) + EY(m, i + 1, j)) / 2.0;
            F.E[0][id] = ex0;
            F.E[1][id] = ey0;
            zd exz = ((EX(m + 1, i, j) + EX(m + 1, i, j + 1)) / 2.0 - ex0) / cz;
            zd ezx = ((EZ(m, i + 1, j) + EZ(m, i + 1, j + 1)) / 2.0 - (EZ(m, i, j + 1) + EZ(m, i, j)) / 2.0) / a[i];
            zd eyz = ((EY(m + 1, i, j) + EY(m + 1, i + 1, j)) / 2.0 - ey0) / cz;
            zd ezy = (-(EZ(m, i, j) + EZ(m, i + 1, j)) / 2.0 + (EZ(m, i, j + 1) + EZ(m, i + 1, j + 1)) / 2.0) / b[j];
            zd exy = (EX(m, i, j + 1) - EX(m, i, j)) / b[j];
            zd eyx = (EY(m, i + 1, j) - EY(m, i, j)) / a[i];
            F.H[1][id] = (exz - ezx) / iwm;
            F.H[0][id] = (ezy - eyz) / iwm;
            F.H[2][id] = (exy - eyx) / iwm;
        }
}

int impedance_topo(const zd* x1, const zd* x2, int nx, int ny, int nz, const int* mcol, const double* czcol,
                   const double* a, const double* b, double ff, int nrec, const double* recv, int out_type,
                   int transpose, double* out, double* tip) {
    const zd iwm = zd(0, 1) * 2.0 * kPi * ff * kMu;
    SurfFields F[2];
    surface_fields_cols(x1, nx, ny, nz, mcol, czcol, a, b, iwm, F[0]);
    surface_fields_cols(x2, nx, ny, nz, mcol, czcol, a, b, iwm, F[1]);
    return impedance_from_fields(F, nx, ny, a, b, ff, nrec, recv, out_type, transpose, out, tip, nullptr);
}

static int impedance_from_fields(const SurfFields (&F)[2], int nx, int ny, const double* a, const double* b,
                                 double ff, int nrec, const double* recv, int out_type, int transpose, double* out,
                                 double* tip, zd* fields) {
    std::vector<double> aax, bby;
    cell_centres(nx, ny, a, b, aax, bby);
    for (int r = 0; r < nrec; r++) {
        RecvStencil S;
        HRC(receiver_stencil(nx, ny, aax, bby, recv[r], recv[(size_t)nrec + r], transpose, S));
        zd f[2][5];
        receiver_fields(F, S, f);
        if (fields)
            for (int p = 0; p < 2; p++)
                for (int q = 0; q < 5; q++) fields[(size_t)r * 10 + p * 5 + q] = f[p][q];
        zd det = f[0][2] * f[1][3] - f[1][2] * f[0][3];
        zd zxy = (f[1][0] * f[0][2] - f[0][0] * f[1][2]) / det;
        zd zyx = (f[0][1] * f[1][3] - f[1][1] * f[0][3]) / det;
        double* o = out + (size_t)r * (out_type == 3 ? 8 : 4);
        if (out_type == 3) {
            // the full tensor Z = E H^-1 of the two polarisations (E, H columns xy, yx);
            // the reference forms only Zxy and Zyx (fdfe_main.f90:688-705)
            const zd zxx = (f[0][0] * f[1][3] - f[1][0] * f[0][3]) / det;
            const zd zyy = (f[1][1] * f[0][2] - f[0][1] * f[1][2]) / det;
            const zd zz[4] = {zxx, zxy, zyx, zyy};
            for (int q = 0; q < 4; q++) {
                o[2 * q] = zz[q].real();
                o[2 * q + 1] = zz[q].imag();
            }
        } else if (out_type == 2) {
            double wmu = 2.0 * kPi * ff * kMu;
            o[0] = std::abs(zxy * zxy * zd(0, 1)) / wmu;
            o[1] = std::abs(zyx * zyx * zd(0, 1)) / wmu;
            o[2] = -std::atan(zxy.imag() / zxy.real()) * 180.0 / kPi;
            o[3] = -std::atan(zyx.imag() / zyx.real()) * 180.0 / kPi;
        } else {
            o[0] = zxy.real();
            o[1] = zxy.imag();
            o[2] = zyx.real();
            o[3] = zyx.imag();
        }
        if (tip) {
            zd tx = (f[1][3] * f[0][4] - f[0][3] * f[1][4]) / det;
            zd ty = (f[0][2] * f[1][4] - f[1][2] * f[0][4]) / det;
            double* t = tip + (size_t)r * 4;
            t[0] = tx.real();
            t[1] = tx.imag();
            t[2] = ty.real();
            t[3] = ty.imag();
        }
    }
    return SFDX_OK;
}

// Least-squares impedance misfit of one frequency and its derivative with
// respect to the receiver fields (reverse mode through Z):
// phi = sum_r wxy |Zxy - dxy|^2 + wyx |Zyx - dyx|^2, cf[r][p][q] = d phi / d
// f[p][q] (q = Ex, Ey, Hx, Hy of polarisation p at receiver r) in the
// holomorphic (Wirtinger) sense, so that d phi = 2 Re(sum cf df).
int impedance_cotangents(const SurfaceView& sv, const double* a, const double* b, const double* c, double ff,
                         int nrec, const double* recv, int transpose, const double* zobs, const double* wts,
                         double* misfit, double* zpred, std::complex<double>* cf_out) {
    const int nx = sv.nx, ny = sv.ny;
    const zd iwm = zd(0, 1) * 2.0 * kPi * ff * kMu;
    SurfFields F[2];
    for (int p = 0; p < 2; p++) surface_fields(sv, p, a, b, c[sv.nair], iwm, F[p]);
    std::vector<double> aax, bby;
    cell_centres(nx, ny, a, b, aax, bby);
    double phi = 0;
    for (int r = 0; r < nrec; r++) {
        RecvStencil S;
        HRC(receiver_stencil(nx, ny, aax, bby, recv[r], recv[(size_t)nrec + r], transpose, S));
        zd f[2][5];
        receiver_fields(F, S, f);
        const zd Ex1 = f[0][0], Ex2 = f[1][0], Ey1 = f[0][1], Ey2 = f[1][1];
        const zd Hx1 = f[0][2], Hy1 = f[0][3], Hx2 = f[1][2], Hy2 = f[1][3];
        const zd det = Hx1 * Hy2 - Hx2 * Hy1;
        const zd zxy = (Ex2 * Hx1 - Ex1 * Hx2) / det;
        const zd zyx = (Ey1 * Hy2 - Ey2 * Hy1) / det;
        const double* d = zobs + (size_t)r * 4;
        const double wxy = wts ? wts[(size_t)r * 2] : 1.0, wyx = wts ? wts[(size_t)r * 2 + 1] : 1.0;
        const zd rxy = zxy - zd(d[0], d[1]), ryx = zyx - zd(d[2], d[3]);
        phi += wxy * std::norm(rxy) + wyx * std::norm(ryx);
        if (zpred) {
            double* o = zpred + (size_t)r * 4;
            o[0] = zxy.real(); o[1] = zxy.imag(); o[2] = zyx.real(); o[3] = zyx.imag();
        }
        // d phi / dZ, then through Z(E, H)
        const zd cxy = wxy * std::conj(rxy), cyx = wyx * std::conj(ryx);
        zd* cf = cf_out + (size_t)r * 8;  // [p][q]
        cf[0] = cxy * (-Hx2 / det);                                         // Ex1
        cf[4] = cxy * (Hx1 / det);                                          // Ex2
        cf[1] = cyx * (Hy2 / det);                                          // Ey1
        cf[5] = cyx * (-Hy1 / det);                                         // Ey2
        cf[2] = cxy * ((Ex2 - zxy * Hy2) / det) + cyx * (-zyx * Hy2 / det); // Hx1
        cf[6] = cxy * ((-Ex1 + zxy * Hy1) / det) + cyx * (zyx * Hy1 / det); // Hx2
        cf[3] = cxy * (zxy * Hx2 / det) + cyx * ((-Ey2 + zyx * Hx2) / det); // Hy1
        cf[7] = cxy * (-zxy * Hx1 / det) + cyx * ((Ey1 - zyx * Hx1) / det); // Hy2
    }
    *misfit += phi;
    return SFDX_OK;
}

// The adjoint source of those cotangents on the surface edge planes of a mesh
// (the transpose of the receiver interpolation and of surface_fields); g is
// accumulated.  Evaluated on the coarse meshes too, where it is the same
// functional of the coarse fields.
int impedance_adjoint_source(SurfaceGrad& g, int nair, const double* a, const double* b, const double* c, double ff,
                             int nrec, const double* recv, int transpose, const std::complex<double>* cf_in) {
    const int nx = g.nx, ny = g.ny;
    const size_t n = (size_t)nx * ny;
    const zd iwm = zd(0, 1) * 2.0 * kPi * ff * kMu;
    SurfFields dF[2];
    for (int p = 0; p < 2; p++) dF[p].init(n);
    std::vector<double> aax, bby;
    cell_centres(nx, ny, a, b, aax, bby);
    for (int r = 0; r < nrec; r++) {
        RecvStencil S;
        HRC(receiver_stencil(nx, ny, aax, bby, recv[r], recv[(size_t)nrec + r], transpose, S));
        const zd* cf = cf_in + (size_t)r * 8;
        for (int p = 0; p < 2; p++)
            for (int t = 0; t < 9; t++) {
                dF[p].E[0][S.id[t]] += S.w[t] * cf[4 * p + 0];
                dF[p].E[1][S.id[t]] += S.w[t] * cf[4 * p + 1];
                dF[p].H[0][S.id[t]] += S.w[t] * cf[4 * p + 2];
                dF[p].H[1][S.id[t]] += S.w[t] * cf[4 * p + 3];
            }
    }
    for (int p = 0; p < 2; p++) surface_fields_adjoint(g, p, a, b, c[nair], iwm, dF[p]);
    return SFDX_OK;
}

// -------------------------------------------------------------------- files
// read_input (file_opt.f90:8-95) + read_topo (:97-128): list-directed reads
// are whitespace-separated numbers; the first line is a free-text title.
// Values of Fortran list-directed input (the reference reads its files with
// read(unit,*)): separated by blanks, line ends or commas; D or d as the
// exponent letter; r*c repeats the constant c r times.
struct Tok {
    FILE* f;
    double rep_val = 0;
    long rep_left = 0;  // values of an r*c item still to hand out
    explicit Tok(FILE* ff) : f(ff) {}
    bool skip_line() {
        rep_left = 0;
        int ch;
        while ((ch = fgetc(f)) != EOF && ch != '\n') {
        }
        return ch != EOF;
    }
    static bool parse(char* s, double& v) {
        for (char* p = s; *p; p++)
            if (*p == 'd' || *p == 'D') *p = 'e';  // Fortran exponent letter
        char* end;
        v = strtod(s, &end);
        return end != s && *end == '\0';
    }
    bool token(char* buf, int cap) {
        int ch, n = 0;
        while ((ch = fgetc(f)) != EOF && (isspace(ch) || ch == ','))
            ;
        while (ch != EOF && !isspace(ch) && ch != ',') {
            if (n + 1 >= cap) return false;
            buf[n++] = (char)ch;
            ch = fgetc(f);
        }
        buf[n] = '\0';
        return n > 0;
    }
    bool num(double& v) {
        if (rep_left > 0) {
            rep_left--;
            v = rep_val;
            return true;
        }
        char buf[128];
        if (!token(buf, (int)sizeof buf)) return false;
        if (char* star = strchr(buf, '*')) {  // r*c
            *star = '\0';
            char* end;
            const long r = strtol(buf, &end, 10);
            if (end == buf || *end != '\0' || r < 1 || !parse(star + 1, rep_val)) return false;
            rep_left = r - 1;
            v = rep_val;
            return true;
        }
        return parse(buf, v);
    }
    bool inum(int& v) {  // an integer item: a whole number within the range of int
        double d;
        if (!num(d) || !(d >= -2147483648.0 && d <= 2147483647.0) || d != std::floor(d)) return false;
        v = (int)d;
        return true;
    }
};

struct ModelHeader {
    int level, solver, out_type, nx, ny, nz, nair, topo, conduc_type, nf, nrec;
    double eps, ext[2];
    int abu[6];
};

static int read_header(Tok& t, ModelHeader& h) {
    if (!t.skip_line()) return SFDX_ERR_IO;
    if (!t.inum(h.level) || !t.num(h.eps) || !t.inum(h.solver) || !t.inum(h.out_type)) return SFDX_ERR_IO;
    if (!t.inum(h.nx) || !t.inum(h.ny) || !t.inum(h.nz) || !t.inum(h.nair) || !t.inum(h.topo)) return SFDX_ERR_IO;
    return SFDX_OK;
}

}  // namespace sfdx

using namespace sfdx;

extern "C" int sfdx_read_sizes(const char* name, int* nx, int* ny, int* nz, int* nair, int* nf, int* nrec) {
    if (!name) return SFDX_ERR_ARG;
    std::string base(name);
    FILE* f = fopen((base + ".fwd").c_str(), "r");
    if (!f) return SFDX_ERR_IO;
    Tok t(f);
    ModelHeader h{};
    int rc = read_header(t, h);
    fclose(f);
    if (rc) return rc;
    FILE* g = fopen((base + ".dat").c_str(), "r");
    if (!g) return SFDX_ERR_IO;
    Tok u(g);
    int nfr = 0, nr = 0;
    double d;
    if (!u.inum(nfr)) { fclose(g); return SFDX_ERR_IO; }
    for (int i = 0; i < nfr; i++)
        if (!u.num(d)) { fclose(g); return SFDX_ERR_IO; }
    if (!u.inum(nr)) { fclose(g); return SFDX_ERR_IO; }
    fclose(g);
    // sizes the caller allocates from: reject what no model can have
    if (h.nx < 1 || h.ny < 1 || h.nz < 1 || h.nair < 0 || nfr < 1 || nr < 0) return SFDX_ERR_IO;
    if ((double)h.nx * h.ny * (double)(h.nz + h.nair) * 6.0 > 9.0e15) return SFDX_ERR_IO;
    if (nx) *nx = h.nx;
    if (ny) *ny = h.ny;
    if (nz) *nz = h.nz + h.nair;  // total z cells, air included
    if (nair) *nair = h.nair;
    if (nf) *nf = nfr;
    if (nrec) *nrec = nr;
    return SFDX_OK;
}

extern "C" int sfdx_read_model(const char* name, const sfdx_opts* o, int* level, double* eps, int* solver,
                               int* out_type, double* a, double* b, double* c, double* sigma, double* freq,
                               double* recv, int* abu) {
    if (!name || !a || !b || !c || !sigma || !freq || !recv) return SFDX_ERR_ARG;
    sfdx_opts def;
    sfdx_default_opts(&def);
    if (!o) o = &def;
    std::string base(name);
    FILE* f = fopen((base + ".fwd").c_str(), "r");
    if (!f) return SFDX_ERR_IO;
    Tok t(f);
    ModelHeader h{};
    int rc = read_header(t, h);
    if (rc) { fclose(f); return rc; }
    // range checks of read_input (file_opt.f90:22-39)
    if (h.level < 3 || h.solver < 0 || h.solver >= 5 || h.out_type < 0 || h.out_type >= 3 ||
        h.nx / (1 << h.level) < 2) {
        fclose(f);
        return SFDX_ERR_ARG;
    }
    const int nx = h.nx, ny = h.ny, nze = h.nz, nair = h.nair, nzt = nze + nair;
    for (int i = 0; i < nx; i++) if (!t.num(a[i])) { fclose(f); return SFDX_ERR_IO; }
    for (int i = 0; i < ny; i++) if (!t.num(b[i])) { fclose(f); return SFDX_ERR_IO; }
    for (int i = 0; i < nze; i++) if (!t.num(c[nair + i])) { fclose(f); return SFDX_ERR_IO; }
    if (!t.num(h.ext[0]) || !t.num(h.ext[1])) { fclose(f); return SFDX_ERR_IO; }
    for (int q = 0; q < 6; q++) if (!t.inum(h.abu[q])) { fclose(f); return SFDX_ERR_IO; }
    for (int i = 0; i < nair; i++) c[i] = c[nzt - 1 - i];  // c(1:nair) = c(nz+nair:nz+1:-1)
    if (!t.inum(h.conduc_type)) { fclose(f); return SFDX_ERR_IO; }
    const size_t ncell = (size_t)nx * ny * nzt;
    for (size_t q = 0; q < 6 * ncell; q++) sigma[q] = 0;
    for (int k = 1; k <= nze; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                size_t id = (size_t)(nair + k - 1) * nx * ny + (size_t)(j - 1) * nx + (i - 1);
                double v[6] = {0, 0, 0, 0, 0, 0};
                int nv = h.conduc_type == 1 ? 1 : (h.conduc_type == 2 ? 3 : 6);
                for (int q = 0; q < nv; q++) if (!t.num(v[q])) { fclose(f); return SFDX_ERR_IO; }
                if (h.conduc_type == 1) v[1] = v[2] = v[0];
                for (int q = 0; q < 6; q++) sigma[q * ncell + id] = v[q];
            }
    fclose(f);
    for (size_t id = 0; id < (size_t)nair * nx * ny; id++)
        for (int q = 0; q < 3; q++) sigma[q * ncell + id] = o->sigma_air;
    if (h.topo != 0) {
        // read_topo (file_opt.f90:97-128): air cells below the local surface
        // take the earth conductivity sigma_hhs; the reference writes it into
        // components 1, 4 and 6 (xx, xy, yz), kept here as written.
        FILE* g = fopen((base + ".topo").c_str(), "r");
        if (!g) return SFDX_ERR_IO;
        Tok u(g);
        int n1, n2;
        if (!u.inum(n1) || !u.inum(n2)) { fclose(g); return SFDX_ERR_IO; }
        const double cstep = c[nair];
        const double sigma_hhs = 1e-2;  // global_para.f90:12
        for (int j = n1; j <= n2; j++)
            for (int i = n1; i <= n2; i++) {
                double tv;
                if (!u.num(tv)) { fclose(g); return SFDX_ERR_IO; }
                int n3 = (int)(tv / cstep);
                for (int k = 1; k <= n3; k++) {
                    long long id = (long long)(nair - n3 + k - 1) * nx * ny + (long long)(j - 1) * nx + (i - 1);
                    if (id < 0 || id >= (long long)ncell) continue;
                    sigma[0 * ncell + id] = sigma_hhs;
                    sigma[3 * ncell + id] = sigma_hhs;
                    sigma[5 * ncell + id] = sigma_hhs;
                }
            }
        fclose(g);
    }
    FILE* g = fopen((base + ".dat").c_str(), "r");
    if (!g) return SFDX_ERR_IO;
    Tok u(g);
    int nf, nrec;
    if (!u.inum(nf)) { fclose(g); return SFDX_ERR_IO; }
    for (int i = 0; i < nf; i++) if (!u.num(freq[i])) { fclose(g); return SFDX_ERR_IO; }
    if (!u.inum(nrec)) { fclose(g); return SFDX_ERR_IO; }
    for (int i = 0; i < nrec; i++)
        for (int q = 0; q < 3; q++) if (!u.num(recv[(size_t)q * nrec + i])) { fclose(g); return SFDX_ERR_IO; }
    fclose(g);
    if (level) *level = h.level;
    if (eps) *eps = h.eps;
    if (solver) *solver = h.solver;
    if (out_type) *out_type = h.out_type;
    if (abu) for (int q = 0; q < 6; q++) abu[q] = h.abu[q];
    return SFDX_OK;
}

// output_data (file_opt.f90:131-158): format 4(e12.5,2x),i1,2x,4(e12.5,2x).
// The reference prints an unset loop variable in the i1 field; 0 is written.
// Fortran Ew.d edit descriptor: [-]0.d...dE[+-]xx, right-justified in w columns
static void fortran_e(char* buf, size_t cap, int w, int d, double v) {
    char body[64];
    if (v == 0) {
        snprintf(body, sizeof body, "0.%0*dE+00", d, 0);
    } else {
        int ex = (int)std::floor(std::log10(std::fabs(v))) + 1;
        double m = std::fabs(v) / std::pow(10.0, ex);
        if (m < 0.1) { m *= 10; ex -= 1; }
        if (m >= 1.0) { m /= 10; ex += 1; }
        const double top = 1.0 - 0.5 * std::pow(10.0, -d);  // would print as 1.0...
        if (m >= top) { m /= 10; ex += 1; }
        char mant[32];
        snprintf(mant, sizeof mant, "%.*f", d, m);
        snprintf(body, sizeof body, "%s%sE%c%02d", v < 0 ? "-" : "", mant, ex < 0 ? '-' : '+', std::abs(ex) % 100);
    }
    snprintf(buf, cap, "%*s", w, body);
}
static void fortran_e12_5(char* buf, double v) { fortran_e(buf, 32, 12, 5, v); }

// output_data (file_opt.f90:131-158): one row per (frequency, receiver) with
// the receiver position, the frequency, the loop variable the reference prints
// uninitialised (written as 0) and four values, in format 4(e12.5,2x),i1,2x,4(e12.5,2x).
static void write_res_rows(FILE* f, int nf, const double* freq, int nrec, const double* recv, const double* v) {
    char b[32];
    for (int k = 0; k < nf; k++)
        for (int i = 0; i < nrec; i++) {
            for (int q = 0; q < 3; q++) { fortran_e12_5(b, recv[(size_t)q * nrec + i]); fprintf(f, "%s  ", b); }
            fortran_e12_5(b, freq[k]);
            fprintf(f, "%s  0  ", b);
            for (int q = 0; q < 4; q++) {
                fortran_e12_5(b, v[((size_t)k * nrec + i) * 4 + q]);
                fprintf(f, "%s  ", b);
            }
            fprintf(f, "\n");
        }
}

extern "C" int sfdx_write_res_tipper(const char* name, int nf, const double* freq, int nrec, const double* recv,
                                     const double* out, const double* tipper) {
    if (!name || !freq || !recv || !out || nf < 0 || nrec < 0) return SFDX_ERR_ARG;
    FILE* f = fopen((std::string(name) + ".res").c_str(), "w");
    if (!f) return SFDX_ERR_IO;
    write_res_rows(f, nf, freq, nrec, recv, out);
    // output_tipper (global_para.f90:7): the tipper block follows the impedance block
    if (tipper) write_res_rows(f, nf, freq, nrec, recv, tipper);
    const bool bad = ferror(f) != 0;
    return (fclose(f) != 0 || bad) ? SFDX_ERR_IO : SFDX_OK;
}

extern "C" int sfdx_write_res(const char* name, int nf, const double* freq, int nrec, const double* recv,
                              const double* out) {
    return sfdx_write_res_tipper(name, nf, freq, nrec, recv, out, nullptr);
}

// Misfit of host fields and its derivative with respect to every edge value
// (zero away from the receiver planes): the host part of the adjoint gradient,
// for callers that run their own adjoint solves.
extern "C" int sfdx_impedance_misfit(int nx, int ny, int nz, int nair, const double* a, const double* b,
                                     const double* c, int nf, const double* freq, const double* ex, int nrec,
                                     const double* recv, int quirks, const double* zobs, const double* wts,
                                     double* misfit, double* grad) {
    if (!a || !b || !c || !freq || !ex || !recv || !zobs || !misfit || nrec < 1 || nf < 1 || nair < 1 ||
        nair + 2 > nz)
        return SFDX_ERR_ARG;
    const size_t xnl = (size_t)nx * (ny + 1) * (nz + 1), ynl = (size_t)(nx + 1) * ny * (nz + 1);
    const size_t nl = xnl + ynl + (size_t)(nx + 1) * (ny + 1) * nz;
    const size_t pex = (size_t)nx * (ny + 1), pey = (size_t)(nx + 1) * ny, pez = (size_t)(nx + 1) * (ny + 1);
    const int transpose = (quirks & SFDX_QUIRK_RX_TRANSPOSE) ? 1 : 0;
    const zd* x = reinterpret_cast<const zd*>(ex);
    zd* g = reinterpret_cast<zd*>(grad);
    if (g) std::fill(g, g + (size_t)nf * 2 * nl, zd(0.0));
    double phi = 0;
    std::vector<zd> cf((size_t)nrec * 8);
    for (int f = 0; f < nf; f++) {
        SurfaceView sv;
        sv.nx = nx; sv.ny = ny; sv.nair = nair;
        for (int p = 0; p < 2; p++) {
            const zd* xp = x + ((size_t)f * 2 + p) * nl;
            sv.exs[p] = xp + (size_t)nair * pex;
            sv.eys[p] = xp + xnl + (size_t)nair * pey;
            sv.ezs[p] = xp + xnl + ynl + (size_t)nair * pez;
        }
        HRC(impedance_cotangents(sv, a, b, c, freq[f], nrec, recv, transpose, zobs + (size_t)f * nrec * 4,
                                 wts ? wts + (size_t)f * nrec * 2 : nullptr, &phi, nullptr, cf.data()));
        if (!g) continue;
        SurfaceGrad sg;
        sg.nx = nx; sg.ny = ny;
        for (int p = 0; p < 2; p++) {
            zd* gp = g + ((size_t)f * 2 + p) * nl;
            sg.exs[p] = gp + (size_t)nair * pex;
            sg.eys[p] = gp + xnl + (size_t)nair * pey;
            sg.ezs[p] = gp + xnl + ynl + (size_t)nair * pez;
        }
        HRC(impedance_adjoint_source(sg, nair, a, b, c, freq[f], nrec, recv, transpose, cf.data()));
    }
    *misfit = phi;
    return SFDX_OK;
}

// Convergence history file of one solve (Bicg_stab_p / pgpbicg with
// output_ccv, solvers.f90:687-704, :289-305): named
// <model>_<freq as e9.2>_<polar>_<tag>.ccv, the iteration count on the first
// line, then every non-zero relative residual as e9.2.
extern "C" int sfdx_write_ccv(const char* name, double freq, const char* polar, const char* tag, int iters,
                              const double* history, int n) {
    if (!name || !polar || !tag || (n > 0 && !history) || n < 0) return SFDX_ERR_ARG;
    char fb[32];
    fortran_e(fb, sizeof fb, 9, 2, freq);
    const char* ft = fb;
    while (*ft == ' ') ft++;
    FILE* f = fopen((std::string(name) + "_" + ft + "_" + polar + "_" + tag + ".ccv").c_str(), "w");
    if (!f) return SFDX_ERR_IO;
    fprintf(f, "%12d\n", iters);
    char b[32];
    for (int j = 0; j < n; j++)
        if (history[j] != 0) {
            fortran_e(b, sizeof b, 9, 2, history[j]);
            fprintf(f, "%s\n", b);
        }
    fclose(f);
    return SFDX_OK;
}

extern "C" int sfdx_mt1d(double freq, int nz, const double* conv, const double* c, double* edc, double* hx,
                         double* imp) {
    if (!conv || !c || !edc || nz <= 0) return SFDX_ERR_ARG;
    return sfdx::mt1d_anl(freq, nz, conv, c, reinterpret_cast<zd*>(edc), reinterpret_cast<zd*>(hx),
                          reinterpret_cast<zd*>(imp));
}
