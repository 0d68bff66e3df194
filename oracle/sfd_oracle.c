/*
 * sfd_oracle.c -- CPU restatement of the SFD_EXCMG forward-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it, to check results.
 * Nothing in the shipped library links, loads or calls it.
 *
 * Parity status: unpinned against reference outputs.  The reference Fortran
 * (sfd_excmg/src, Fortran 90) needs ifort + MKL, does not compile as committed, and
 * ships no golden vectors; this restatement follows its source index for index
 * and is pinned instead by known-answer tests (1-D layered earth, homogeneous
 * half-space, polynomial-exact prolongation) in tests/.
 *
 * All index arithmetic below is written 1-based, exactly as in the Fortran
 * source it restates, through the E1/S1 helper macros; storage is 0-based.
 * Complex numbers are C99 double complex (same memory layout as Fortran
 * complex(8)).  sigma is Fortran sigma(ncell,6), i.e. [6][ncell] in C order.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zc;

static const double PI = 3.141592653589793238462643;
static const double MU = 4.0 * 3.141592653589793238462643 * 1e-7;

#define SG(ie, comp) sig[(size_t)((comp)-1) * (size_t)ncell + (size_t)((ie)-1)]

/* ------------------------------------------------------------------------ */
/* fd_assemb (fdfe_main.f90:226-396): 13 COO entries per interior edge row.  */
/* v/vc are 13*nl arrays; vc==0 marks "not assembled" (boundary rows).        */
/* ------------------------------------------------------------------------ */
static void fd_assemb(int nx, int ny, int nz, const double *a, const double *b,
                      const double *c, const double *sig, double ff, zc *v,
                      int64_t *vc) {
    const int64_t ncell = (int64_t)nx * ny * nz;
    const double w = 2 * PI * ff;
    const zc coef = I * w * MU; /* cmplx(0,1)*w*mu  (:238) */
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1);
    const int64_t ynl = (int64_t)ny * (nz + 1) * (nx + 1);
    const int64_t nl = xnl + ynl + (int64_t)nz * (nx + 1) * (ny + 1);
    memset(v, 0, sizeof(zc) * 13 * nl);
    memset(vc, 0, sizeof(int64_t) * 13 * nl);
#define A(i) a[(i)-1]
#define B(j) b[(j)-1]
#define C(k) c[(k)-1]
#define V(n) v[(ind - 1) * 13 + (n)-1]
#define VC(n) vc[(ind - 1) * 13 + (n)-1]
    /* Ex rows (:248-295) */
    for (int k = 2; k <= nz; k++)
        for (int j = 2; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                int64_t ie = (int64_t)(k - 2) * nx * ny + (int64_t)(j - 2) * nx + i;
                double sigmas = (SG(ie, 1) * B(j - 1) * C(k - 1) + SG(ie + nx, 1) * B(j) * C(k - 1) +
                                 SG(ie + (int64_t)nx * ny, 1) * B(j - 1) * C(k) +
                                 SG(ie + (int64_t)nx * ny + nx, 1) * B(j) * C(k)) /
                                ((B(j - 1) + B(j)) * (C(k - 1) + C(k)));
                double den = (B(j - 1) + B(j)) * (C(k - 1) + C(k));
                double sv1 = (SG(ie, 4) * B(j - 1) * C(k - 1) + SG(ie + (int64_t)nx * ny, 4) * B(j - 1) * C(k)) / 2 / den;
                double sv2 = (SG(ie + nx, 4) * B(j) * C(k - 1) + SG(ie + (int64_t)nx * ny + nx, 4) * B(j) * C(k)) / 2 / den;
                double sv3 = (SG(ie, 5) * B(j - 1) * C(k - 1) + SG(ie + nx, 5) * B(j) * C(k - 1)) / 2 / den;
                double sv4 = (SG(ie + (int64_t)nx * ny, 5) * B(j - 1) * C(k) + SG(ie + nx + (int64_t)nx * ny, 5) * B(j) * C(k)) / 2 / den;
                int64_t ind = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i;
                V(1) = -2 / (C(k - 1) * (C(k - 1) + C(k)));
                VC(1) = ind - (int64_t)nx * (ny + 1);
                V(2) = -2 / (B(j - 1) * (B(j - 1) + B(j)));
                VC(2) = ind - nx;
                V(4) = -2 / (B(j) * (B(j - 1) + B(j)));
                VC(4) = ind + nx;
                V(5) = -2 / (C(k) * (C(k - 1) + C(k)));
                VC(5) = ind + (int64_t)nx * (ny + 1);
                V(3) = -(V(1) + V(2) + V(3) + V(4) + V(5)) - coef * sigmas;
                VC(3) = ind;
                V(6) = 2 / (A(i) * (B(j - 1) + B(j)));
                VC(6) = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 2) * (nx + 1) + i;
                V(8) = -V(6);
                V(7) = -V(6);
                V(9) = V(6);
                V(6) -= coef * sv1;
                V(7) -= coef * sv1;
                V(8) -= coef * sv2;
                V(9) -= coef * sv2;
                VC(7) = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 2) * (nx + 1) + i + 1;
                VC(8) = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i;
                VC(9) = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i + 1;
                V(10) = 2 / (A(i) * (C(k - 1) + C(k)));
                VC(10) = xnl + ynl + (int64_t)(k - 2) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                V(12) = -V(10);
                V(11) = -V(10);
                V(13) = V(10);
                VC(11) = xnl + ynl + (int64_t)(k - 2) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i + 1;
                VC(12) = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                VC(13) = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i + 1;
                V(10) -= coef * sv3;
                V(11) -= coef * sv3;
                V(12) -= coef * sv4;
                V(13) -= coef * sv4;
            }
    /* Ey rows (:297-344) */
    for (int k = 2; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 2; i <= nx; i++) {
                int64_t ie = (int64_t)(k - 2) * nx * ny + (int64_t)(j - 1) * nx + i - 1;
                int64_t nxy = (int64_t)nx * ny;
                double den = (A(i - 1) + A(i)) * (C(k - 1) + C(k));
                double sigmas = (SG(ie, 2) * A(i - 1) * C(k - 1) + SG(ie + 1, 2) * A(i) * C(k - 1) +
                                 SG(ie + nxy, 2) * A(i - 1) * C(k) + SG(ie + nxy + 1, 2) * A(i) * C(k)) / den;
                double sv1 = (SG(ie, 4) * A(i - 1) * C(k - 1) + SG(ie + nxy, 4) * A(i - 1) * C(k)) / 2 / den;
                double sv2 = (SG(ie + 1, 4) * A(i) * C(k - 1) + SG(ie + nxy + 1, 4) * A(i) * C(k)) / 2 / den;
                double sv3 = (SG(ie, 6) * A(i - 1) * C(k - 1) + SG(ie + 1, 6) * A(i) * C(k - 1)) / 2 / den;
                double sv4 = (SG(ie + nxy, 6) * A(i - 1) * C(k) + SG(ie + nxy + 1, 6) * A(i) * C(k)) / 2 / den;
                int64_t ind = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i;
                V(1) = 2 / (B(j) * (A(i - 1) + A(i)));
                VC(1) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i - 1;
                V(2) = -V(1);
                V(3) = -V(1);
                V(4) = V(1);
                VC(2) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i;
                VC(3) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i - 1 + nx;
                VC(4) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i + nx;
                V(1) -= coef * sv1;
                V(3) -= coef * sv1;
                V(2) -= coef * sv2;
                V(4) -= coef * sv2;
                V(5) = -2 / (C(k - 1) * (C(k - 1) + C(k)));
                VC(5) = ind - (int64_t)(nx + 1) * ny;
                V(6) = -2 / (A(i - 1) * (A(i - 1) + A(i)));
                VC(6) = ind - 1;
                V(8) = -2 / (A(i) * (A(i - 1) + A(i)));
                VC(8) = ind + 1;
                V(9) = -2 / (C(k) * (C(k - 1) + C(k)));
                VC(9) = ind + (int64_t)(nx + 1) * ny;
                V(7) = -(V(5) + V(6) + V(7) + V(8) + V(9)) - coef * sigmas;
                VC(7) = ind;
                V(10) = 2 / (B(j) * (C(k - 1) + C(k)));
                VC(10) = xnl + ynl + (int64_t)(k - 2) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                V(12) = -V(10);
                V(11) = -V(10);
                V(13) = V(10);
                VC(11) = xnl + ynl + (int64_t)(k - 2) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i + nx + 1;
                VC(12) = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                VC(13) = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i + nx + 1;
                V(10) -= coef * sv3;
                V(11) -= coef * sv3;
                V(12) -= coef * sv4;
                V(13) -= coef * sv4;
            }
    /* Ez rows (:346-393) */
    for (int k = 1; k <= nz; k++)
        for (int j = 2; j <= ny; j++)
            for (int i = 2; i <= nx; i++) {
                int64_t ie = (int64_t)(k - 1) * nx * ny + (int64_t)(j - 2) * nx + i - 1;
                double den = (B(j - 1) + B(j)) * (A(i - 1) + A(i));
                double sigmas = (SG(ie, 3) * B(j - 1) * A(i - 1) + SG(ie + nx, 3) * B(j) * A(i - 1) +
                                 SG(ie + 1, 3) * B(j - 1) * A(i) + SG(ie + nx + 1, 3) * B(j) * A(i)) / den;
                double sv1 = (SG(ie, 5) * B(j - 1) * A(i - 1) + SG(ie + nx, 5) * B(j) * A(i - 1)) / 2 / den;
                double sv2 = (SG(ie + 1, 5) * B(j - 1) * A(i) + SG(ie + nx + 1, 5) * B(j) * A(i)) / 2 / den;
                double sv3 = (SG(ie, 6) * B(j - 1) * A(i - 1) + SG(ie + 1, 6) * B(j - 1) * A(i)) / 2 / den;
                double sv4 = (SG(ie + nx, 6) * B(j) * A(i - 1) + SG(ie + nx + 1, 6) * B(j) * A(i)) / 2 / den;
                int64_t ind = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                V(1) = 2 / (C(k) * (A(i - 1) + A(i)));
                VC(1) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i - 1;
                V(2) = -V(1);
                V(3) = -V(1);
                V(4) = V(1);
                VC(2) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i;
                VC(3) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i - 1 + (int64_t)nx * (ny + 1);
                VC(4) = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i + (int64_t)nx * (ny + 1);
                V(1) -= coef * sv1;
                V(3) -= coef * sv1;
                V(2) -= coef * sv2;
                V(4) -= coef * sv2;
                V(5) = 2 / (C(k) * (B(j - 1) + B(j)));
                VC(5) = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 2) * (nx + 1) + i;
                V(6) = -V(5);
                V(7) = -V(5);
                V(8) = V(5);
                VC(6) = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i;
                VC(7) = xnl + (int64_t)k * (nx + 1) * ny + (int64_t)(j - 2) * (nx + 1) + i;
                VC(8) = xnl + (int64_t)k * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i;
                V(5) -= coef * sv3;
                V(7) -= coef * sv3;
                V(6) -= coef * sv4;
                V(8) -= coef * sv4;
                V(9) = -2 / (B(j - 1) * (B(j - 1) + B(j)));
                VC(9) = ind - (nx + 1);
                V(10) = -2 / (A(i - 1) * (A(i - 1) + A(i)));
                VC(10) = ind - 1;
                V(12) = -2 / (A(i) * (A(i - 1) + A(i)));
                VC(12) = ind + 1;
                V(13) = -2 / (B(j) * (B(j - 1) + B(j)));
                VC(13) = ind + (nx + 1);
                V(11) = -(V(9) + V(10) + V(11) + V(12) + V(13)) - coef * sigmas;
                VC(11) = ind;
            }
#undef V
#undef VC
}

/* Boundary-edge flags of dcfast (fdfe_main.f90:436-468); bori is 1-based. */
static void boundary_flags(int nx, int ny, int nz, unsigned char *bori) {
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1);
    const int64_t ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    memset(bori, 0, (size_t)nl + 1);
    for (int k = 1; k <= nz + 1; k++)
        for (int j = 1; j <= ny + 1; j++)
            for (int i = 1; i <= nx; i++) {
                int64_t ind = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i;
                if (k == 1 || k == nz + 1 || j == 1 || j == ny + 1) bori[ind] = 1;
            }
    for (int k = 1; k <= nz + 1; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx + 1; i++) {
                int64_t ind = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i;
                if (k == 1 || k == nz + 1 || i == 1 || i == nx + 1) bori[ind] = 1;
            }
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny + 1; j++)
            for (int i = 1; i <= nx + 1; i++) {
                int64_t ind = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                if (i == 1 || i == nx + 1 || j == 1 || j == ny + 1) bori[ind] = 1;
            }
}

/* Dirichlet vectors p1 (xy) and p2 (yx) of dcfast (fdfe_main.f90:470-494).
 * ex is e_dc(2nz+2) from mt1d_anl; p1/p2 are 0-based arrays of length nl. */
static void dirichlet(int nx, int ny, int nz, const zc *ex, zc *p1, zc *p2) {
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1);
    const int64_t ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
#define P1(n) p1[(n)-1]
#define P2(n) p2[(n)-1]
#define EX(n) ex[(n)-1]
    for (int64_t n = 0; n < nl; n++) p1[n] = p2[n] = 0;
    for (int i = 1; i <= ny + 1; i++)
        for (int64_t n = (int64_t)(i - 1) * nx + 1; n <= (int64_t)i * nx; n++) P1(n) = 1.0;
    for (int k = 1; k <= nz; k++) {
        for (int64_t n = (int64_t)k * nx * (ny + 1) + 1; n <= (int64_t)k * nx * (ny + 1) + nx; n++) P1(n) = EX(k + 1);
        for (int64_t n = (int64_t)(k + 1) * nx * (ny + 1) - nx + 1; n <= (int64_t)(k + 1) * nx * (ny + 1); n++)
            P1(n) = EX(k + 1);
    }
    for (int64_t n = xnl - (int64_t)nx * (ny + 1) + 1; n <= xnl; n++) P1(n) = EX(nz + 1);
    for (int i = 1; i <= ny; i++)
        for (int64_t n = xnl + (int64_t)(i - 1) * (nx + 1) + 1; n <= xnl + (int64_t)i * (nx + 1); n++) P2(n) = 1.0;
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= ny; i++) {
            P2(xnl + (int64_t)k * (nx + 1) * ny + (int64_t)(i - 1) * (nx + 1) + 1) = EX(nz + 1 + k + 1);
            P2(xnl + (int64_t)k * (nx + 1) * ny + (int64_t)i * (nx + 1)) = EX(nz + 1 + k + 1);
        }
    for (int64_t n = xnl + ynl - (int64_t)(nx + 1) * ny + 1; n <= xnl + ynl; n++) P2(n) = EX(2 * nz + 2);
#undef P1
#undef P2
#undef EX
}

/*
 * orc_assemble: fd_assemb + dcfast (fdfe_main.f90:226-546).
 * Outputs a 0-based CSR (ia[nl+1], ja, kmat) in the reference's entry order
 * (row-major, the 13 entries in assembly order, zero and boundary columns
 * removed) plus the two right-hand sides p1, p2.  ja/kmat need 13*nl slots.
 * Returns nnz.
 */
int64_t orc_assemble(int nx, int ny, int nz, const double *a, const double *b, const double *c,
                     const double *sig, double ff, const zc *edc, int64_t *ia, int32_t *ja, zc *kmat,
                     zc *p1, zc *p2) {
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1);
    const int64_t ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    zc *v = (zc *)malloc(sizeof(zc) * 13 * nl);
    int64_t *vc = (int64_t *)malloc(sizeof(int64_t) * 13 * nl);
    unsigned char *bori = (unsigned char *)malloc((size_t)nl + 1);
    fd_assemb(nx, ny, nz, a, b, c, sig, ff, v, vc);
    boundary_flags(nx, ny, nz, bori);
    dirichlet(nx, ny, nz, edc, p1, p2);
    int64_t k = 0;
    ia[0] = 0;
    for (int64_t i = 1; i <= nl; i++) {
        zc tmp = 0, tmp2 = 0;
        if (!bori[i]) {
            for (int j = 1; j <= 13; j++) {
                int64_t ind = (i - 1) * 13 + j;
                int64_t col = vc[ind - 1];
                if (col > 0) {
                    if (!bori[col] && v[ind - 1] != 0) {
                        kmat[k] = v[ind - 1];
                        ja[k] = (int32_t)(col - 1);
                        k++;
                    } else {
                        tmp += v[ind - 1] * p1[col - 1];
                        tmp2 += v[ind - 1] * p2[col - 1];
                    }
                }
            }
            p1[i - 1] -= tmp;
            p2[i - 1] -= tmp2;
        } else {
            kmat[k] = 1.0;
            ja[k] = (int32_t)(i - 1);
            k++;
        }
        ia[i] = k;
    }
    free(v);
    free(vc);
    free(bori);
    return k;
}

/* Boundary flags exported for tests (0-based, length nl). */
void orc_boundary_flags(int nx, int ny, int nz, unsigned char *flags0) {
    const int64_t nl = (int64_t)nx * (ny + 1) * (nz + 1) + (int64_t)(nx + 1) * ny * (nz + 1) +
                       (int64_t)(nx + 1) * (ny + 1) * nz;
    unsigned char *bori = (unsigned char *)malloc((size_t)nl + 1);
    boundary_flags(nx, ny, nz, bori);
    memcpy(flags0, bori + 1, (size_t)nl);
    free(bori);
}

/* ------------------------------------------------------------------------ */
/* mt1d_anl (model_selec.f90:266-401): analytic 1-D anisotropic layered field */
/* conv is Fortran conv(nz,6) (column-major); ex, hx have 2nz+2 entries.      */
/* ------------------------------------------------------------------------ */
static void mat4mul(const zc *A, const zc *B, zc *Cm) { /* row-major 4x4 */
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            zc s = 0;
            for (int k = 0; k < 4; k++) s += A[i * 4 + k] * B[k * 4 + j];
            Cm[i * 4 + j] = s;
        }
}

void orc_mt1d_anl(double ff, int nz, const double *conv, const double *c, zc *ex, zc *hx, zc *imp) {
#define CV(i, m) conv[(size_t)((m)-1) * nz + (i)-1]
    zc *sprod = (zc *)calloc((size_t)16 * (nz + 1), sizeof(zc)); /* sprod(:,:,i) at [(i-1)*16] */
    zc *xip = (zc *)calloc((size_t)nz + 1, sizeof(zc));
    zc *xim = (zc *)calloc((size_t)nz + 1, sizeof(zc));
    double *qp = (double *)calloc((size_t)nz + 1, sizeof(double));
    double *qm = (double *)calloc((size_t)nz + 1, sizeof(double));
    zc m[16] = {0};
    const double w = 2 * PI * ff;
    for (int i = 0; i < 4; i++) sprod[(size_t)nz * 16 + i * 4 + i] = 1.0;
    for (int i = nz; i >= 1; i--) {
        double axx = CV(i, 1) - CV(i, 5) * CV(i, 5) / CV(i, 3);
        double ayy = CV(i, 2) - CV(i, 6) * CV(i, 6) / CV(i, 3);
        double axy = CV(i, 4) - CV(i, 5) * CV(i, 6) / CV(i, 3);
        double ada = axx + ayy, add = axx - ayy, da12;
        if (add >= 0)
            da12 = sqrt(add * add + 4 * axy * axy);
        else
            da12 = -sqrt(add * add + 4 * axy * axy);
        double a1 = (ada + da12) / 2, a2 = (ada - da12) / 2;
        zc iwm = I * w * MU;
        zc kp = csqrt(-iwm) * sqrt(a1);
        zc km = csqrt(-iwm) * sqrt(a2);
        xip[i - 1] = -kp / iwm;
        xim[i - 1] = -km / iwm;
        if (axy == 0) {
            qp[i - 1] = 0;
            qm[i - 1] = 0;
        } else {
            qp[i - 1] = 2 * axy / (add + da12);
            qm[i - 1] = (add - da12) / axy / 2;
        }
        double qdq = qp[i - 1] * qm[i - 1];
        double dq = 1 - qdq;
        if (i == nz) {
            m[0 * 4 + 1] = 1.0;
            m[1 * 4 + 1] = qp[i - 1];
            m[2 * 4 + 1] = -xip[i - 1] * qp[i - 1];
            m[3 * 4 + 1] = xip[i - 1];
            m[0 * 4 + 3] = qm[i - 1];
            m[1 * 4 + 3] = 1.0;
            m[2 * 4 + 3] = -xim[i - 1];
            m[3 * 4 + 3] = xim[i - 1] * qm[i - 1];
        }
        zc tmp = kp * c[i - 1];
        zc sp = (cexp(tmp) - cexp(-tmp)) / 2.0, cp = (cexp(tmp) + cexp(-tmp)) / 2.0;
        tmp = km * c[i - 1];
        zc sm = (cexp(tmp) - cexp(-tmp)) / 2.0, cm = (cexp(tmp) + cexp(-tmp)) / 2.0;
        zc xp = xip[i - 1], xm = xim[i - 1];
        double qpi = qp[i - 1], qmi = qm[i - 1];
        zc s[16] = {
            cp - qdq * cm, -qmi * (cp - cm), qmi * (sp / xp - sm / xm), sp / xp - qdq * sm / xm,
            qpi * (cp - cm), -qdq * cp + cm, qdq * sp / xp - sm / xm, qpi * (sp / xp - sm / xm),
            -qpi * (xp * sp - xm * sm), qdq * xp * sp - xm * sm, -qdq * cp + cm, -qpi * (cp - cm),
            xp * sp - qdq * xm * sm, -qmi * (xp * sp - xm * sm), qmi * (cp - cm), cp - qdq * cm};
        for (int q = 0; q < 16; q++) s[q] = s[q] / dq;
        mat4mul(s, &sprod[(size_t)i * 16], &sprod[(size_t)(i - 1) * 16]);
    }
    zc s_m[16];
    mat4mul(&sprod[0], m, s_m);
    zc atmp[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int mode = 0; mode < 2; mode++) {
        zc e0 = mode == 0 ? (zc)1.0 : (zc)I;
        /* g = reshape((/s_m(1,2),s_m(2,2),s_m(1,4),s_m(2,4)/),(/2,2/)) */
        zc g11 = s_m[0 * 4 + 1], g21 = s_m[1 * 4 + 1], g12 = s_m[0 * 4 + 3], g22 = s_m[1 * 4 + 3];
        zc detg = g11 * g22 - g12 * g21;
        zc cbot[4] = {0, 0, 0, 0};
        cbot[1] = (g22 * creal(e0) - g12 * cimag(e0)) / detg;
        cbot[3] = (-g21 * creal(e0) + g11 * cimag(e0)) / detg;
        zc mc[4];
        for (int r = 0; r < 4; r++) {
            zc sacc = 0;
            for (int q = 0; q < 4; q++) sacc += m[r * 4 + q] * cbot[q];
            mc[r] = sacc;
        }
        for (int i = 1; i <= nz + 1; i++) {
            zc f[4];
            for (int r = 0; r < 4; r++) {
                zc sacc = 0;
                for (int q = 0; q < 4; q++) sacc += sprod[(size_t)(i - 1) * 16 + r * 4 + q] * mc[q];
                f[r] = sacc;
            }
            if (mode == 0) {
                ex[i - 1] = f[0];
                hx[i - 1] = f[3];
                if (i == nz + 1) memcpy(atmp, f, sizeof(f));
            } else {
                ex[i + nz] = f[1];
                hx[i + nz] = f[2];
                if (i == nz + 1) memcpy(atmp + 4, f, sizeof(f));
            }
        }
    }
    zc tmp = atmp[2] * atmp[7] - atmp[3] * atmp[6];
    imp[0] = (atmp[0] * atmp[7] - atmp[4] * atmp[3]) / tmp;
    imp[1] = (atmp[4] * atmp[2] - atmp[0] * atmp[6]) / tmp;
    imp[2] = (atmp[1] * atmp[7] - atmp[5] * atmp[3]) / tmp;
    imp[3] = (atmp[5] * atmp[2] - atmp[1] * atmp[6]) / tmp;
    free(sprod);
    free(xip);
    free(xim);
    free(qp);
    free(qm);
#undef CV
}

/* ------------------------------------------------------------------------ */
/* mesh_coarsen (fdfe_main.f90:18-84).  quirk=1 keeps the reference's fine-  */
/* cell index ((m-1)asf+r)*.. which is shifted by one plane and one row; the */
/* row overflow wraps into the next plane as in the reference, and a read    */
/* past the last plane (undefined in the reference) is clamped to the last   */
/* plane.  quirk=0 uses the intended index.                                  */
/* ------------------------------------------------------------------------ */
void orc_mesh_coarsen(int nx0, int ny0, int nz0, const double *a, const double *b, const double *c,
                      const double *cont, int k, int quirk, double *a1, double *b1, double *c1, double *ncont) {
    const int asf = 1 << k;
    const int nx = nx0 / asf, ny = ny0 / asf, nz = nz0 / asf;
    const int64_t ncell0 = (int64_t)nx0 * ny0 * nz0;
    const int64_t ne = (int64_t)nx * ny * nz;
    for (int i = 1; i <= nx; i++) {
        double s = 0;
        for (int q = (i - 1) * asf + 1; q <= i * asf; q++) s += a[q - 1];
        a1[i - 1] = s;
    }
    for (int i = 1; i <= ny; i++) {
        double s = 0;
        for (int q = (i - 1) * asf + 1; q <= i * asf; q++) s += b[q - 1];
        b1[i - 1] = s;
    }
    for (int i = 1; i <= nz; i++) {
        double s = 0;
        for (int q = (i - 1) * asf + 1; q <= i * asf; q++) s += c[q - 1];
        c1[i - 1] = s;
    }
    for (int m = 1; m <= nz; m++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double vbig = a1[i - 1] * b1[j - 1] * c1[m - 1];
                double tmp[6] = {0, 0, 0, 0, 0, 0};
                for (int r = 1; r <= asf; r++)
                    for (int s = 1; s <= asf; s++)
                        for (int t = 1; t <= asf; t++) {
                            int64_t ind;
                            if (quirk) {
                                ind = ((int64_t)(m - 1) * asf + r) * nx * ny * asf * asf +
                                      ((int64_t)(j - 1) * asf + s) * nx * asf + (int64_t)(i - 1) * asf + t;
                                while (ind > ncell0) ind -= (int64_t)nx0 * ny0;
                            } else {
                                ind = ((int64_t)(m - 1) * asf + r - 1) * nx0 * ny0 +
                                      ((int64_t)(j - 1) * asf + s - 1) * nx0 + (int64_t)(i - 1) * asf + t;
                            }
                            double vsmall = a[(i - 1) * asf + t - 1] * b[(j - 1) * asf + s - 1] * c[(m - 1) * asf + r - 1];
                            for (int q = 0; q < 6; q++) tmp[q] += cont[(size_t)q * ncell0 + ind - 1] * vsmall;
                        }
                int64_t o = (int64_t)(m - 1) * nx * ny + (int64_t)(j - 1) * nx + i;
                for (int q = 0; q < 6; q++) ncont[(size_t)q * ne + o - 1] = tmp[q] / vbig;
            }
}

/* ------------------------------------------------------------------------ */
/* CSR helpers: zamux (div_correc.f90:431-449), vnorm (model_selec.f90:631) */
/* ------------------------------------------------------------------------ */
static void zamux(int64_t n, const zc *x, zc *y, const zc *a, const int32_t *ja, const int64_t *ia) {
    for (int64_t i = 0; i < n; i++) {
        zc t = 0;
        for (int64_t k = ia[i]; k < ia[i + 1]; k++) t += a[k] * x[ja[k]];
        y[i] = t;
    }
}
static double vnorm(const zc *z, int64_t n) {
    double s = 0;
    for (int64_t i = 0; i < n; i++) {
        double ab = cabs(z[i]);
        s += ab * ab;
    }
    return sqrt(s);
}
static zc dotc(const zc *a, const zc *b, int64_t n) { /* Fortran dot_product: sum(conjg(a)*b) */
    zc s = 0;
    for (int64_t i = 0; i < n; i++) s += conj(a[i]) * b[i];
    return s;
}

void orc_zamux(int64_t n, const zc *x, zc *y, const zc *a, const int32_t *ja, const int64_t *ia) {
    zamux(n, x, y, a, ja, ia);
}

/* ------------------------------------------------------------------------ */
/* ssorfac (div_correc.f90:171-220) + lusol (solvers.f90:721-762), MSR form. */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t n;
    zc *alu;      /* 1-based MSR values, size nnz+2 */
    int64_t *jlu; /* 1-based */
    int64_t *ju;  /* 1-based */
    double w;
    char pre; /* 'S', 'J' or 'M' */
    zc *mj;   /* Jacobi diagonal */
    void *mc; /* multi-colour data ('M') */
} precond_t;

static int ssorfac(int64_t n, const zc *a, const int64_t *ia0, const int32_t *ja0, double omega, precond_t *P) {
    int64_t nnz = ia0[n];
    P->n = n;
    P->w = omega;
    P->pre = 'S';
    P->alu = (zc *)calloc((size_t)(nnz + n + 2), sizeof(zc));
    P->jlu = (int64_t *)calloc((size_t)(nnz + n + 2), sizeof(int64_t));
    P->ju = (int64_t *)calloc((size_t)(n + 2), sizeof(int64_t));
    P->mj = NULL;
    P->mc = NULL;
    int64_t ju0 = n + 2;
    P->jlu[1] = ju0;
    for (int64_t ii = 1; ii <= n; ii++) {
        for (int64_t j = ia0[ii - 1] + 1; j <= ia0[ii]; j++) {
            int64_t jcol = (int64_t)ja0[j - 1] + 1;
            if (jcol == ii) {
                P->alu[ii] = a[j - 1];
                P->ju[ii] = ju0;
            } else {
                P->alu[ju0] = a[j - 1];
                P->jlu[ju0] = jcol;
                ju0++;
            }
        }
        P->jlu[ii + 1] = ju0;
        if (P->alu[ii] == 0) return (int)ii;
        P->alu[ii] = 1.0 / P->alu[ii];
    }
    return 0;
}

static void jacobifac(int64_t n, const zc *a, const int64_t *ia0, const int32_t *ja0, precond_t *P) {
    P->n = n;
    P->pre = 'J';
    P->alu = NULL;
    P->jlu = P->ju = NULL;
    P->mc = NULL;
    P->mj = (zc *)calloc((size_t)n, sizeof(zc));
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = ia0[i]; j < ia0[i + 1]; j++)
            if (ja0[j] == i) P->mj[i] = a[j];
}

/* zilu0 (div_correc.f90:223-317): ILU(0) in MSR form, pre_type = 'I'.  Only
 * columns within the band |jcol - ii - idd(1)| <= idd(2), idd(1) <= jcol <=
 * idd(3) enter the factor (:258).  The solvers receive idd = (1, nl, nl, ...)
 * from doublemode_nor (fdfe_main.f90:994: every entry kept) and (1, np, nl,
 * ...) from doublemode_acc (:1413: couplings more than np columns apart, the
 * Ex-Ez blocks, are left out).  band <= 0 keeps every entry.  The elimination
 * runs over the entries stored before the diagonal in CSR order, which are the
 * columns < ii because dcfast writes sorted rows.  Returns the zero-pivot row
 * (1-based) or 0. */
static int zilu0(int64_t n, int64_t band, const zc *a, const int64_t *ia0, const int32_t *ja0, precond_t *P) {
    int64_t nnz = ia0[n];
    if (band <= 0) band = n;
    P->n = n;
    P->w = 1.0;
    P->pre = 'I';
    P->mj = NULL;
    P->mc = NULL;
    P->alu = (zc *)calloc((size_t)(nnz + n + 2), sizeof(zc));
    P->jlu = (int64_t *)calloc((size_t)(nnz + n + 2), sizeof(int64_t));
    P->ju = (int64_t *)calloc((size_t)(n + 2), sizeof(int64_t));
    int64_t *iw = (int64_t *)calloc((size_t)(n + 2), sizeof(int64_t));
    zc *alu = P->alu;
    int64_t *jlu = P->jlu, *ju = P->ju;
    int64_t ju0 = n + 2;
    jlu[1] = ju0;
    int ierr = 0;
    for (int64_t ii = 1; ii <= n && !ierr; ii++) {
        const int64_t js = ju0;
        for (int64_t j = ia0[ii - 1] + 1; j <= ia0[ii]; j++) {
            const int64_t jcol = (int64_t)ja0[j - 1] + 1;
            const int64_t off = jcol - ii - 1;
            if (!((off < 0 ? -off : off) <= band && jcol <= n && jcol >= 1)) continue;
            if (jcol == ii) {
                alu[ii] = a[j - 1];
                iw[jcol] = ii;
                ju[ii] = ju0;
            } else {
                alu[ju0] = a[j - 1];
                jlu[ju0] = jcol;
                iw[jcol] = ju0;
                ju0++;
            }
        }
        jlu[ii + 1] = ju0;
        const int64_t jf = ju0 - 1, jm = ju[ii] - 1;
        for (int64_t j = js; j <= jm; j++) {  /* row ii of L: eliminate with the rows above */
            const int64_t jrow = jlu[j];
            const zc tl = alu[j] * alu[jrow];
            alu[j] = tl;
            for (int64_t jj = ju[jrow]; jj <= jlu[jrow + 1] - 1; jj++) {
                const int64_t jw = iw[jlu[jj]];
                if (jw != 0) alu[jw] = alu[jw] - tl * alu[jj];
            }
        }
        if (alu[ii] == 0) {
            ierr = (int)ii;
            break;
        }
        alu[ii] = 1.0 / alu[ii];
        iw[ii] = 0;
        for (int64_t i = js; i <= jf; i++) iw[jlu[i]] = 0;
    }
    free(iw);
    return ierr;
}

static void precond_free(precond_t *P) {
    free(P->alu);
    free(P->jlu);
    free(P->ju);
    free(P->mj);
    P->alu = NULL;
    P->jlu = P->ju = NULL;
    P->mj = NULL;
}

/* Multi-colour symmetric Gauss-Seidel ('M'): the GPU's preconditioner,
 * restated on the assembled CSR.  colour[i] in 0..5 (Ex (j+k)&1, Ey (i+k)&1,
 * Ez (i+j)&1, orientation-major); forward sweep in increasing colour,
 * backward in decreasing colour, x = (D+U)^{-1} D (D+L)^{-1} y with L, U the
 * parts coupling to earlier / later colours.  Not part of the reference: it
 * is the oracle of the multi-colour kernels. */
typedef struct {
    int64_t n;
    const zc *a;
    const int64_t *ia;
    const int32_t *ja;
    unsigned char *col;
    zc *diag;
} mcpre_t;

static void mc_colours(int nx, int ny, int nz, unsigned char *col) {
    int64_t q = 0;
    for (int k = 0; k <= nz; k++)
        for (int j = 0; j <= ny; j++)
            for (int i = 0; i < nx; i++) col[q++] = (unsigned char)((j + k) & 1);
    for (int k = 0; k <= nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i <= nx; i++) col[q++] = (unsigned char)(2 + ((i + k) & 1));
    for (int k = 0; k < nz; k++)
        for (int j = 0; j <= ny; j++)
            for (int i = 0; i <= nx; i++) col[q++] = (unsigned char)(4 + ((i + j) & 1));
}

static void mc_psolve(const mcpre_t *M, const zc *y, zc *x) {
    int64_t n = M->n;
    for (int c = 0; c < 6; c++)
        for (int64_t i = 0; i < n; i++) {
            if (M->col[i] != c) continue;
            zc s = y[i];
            for (int64_t k = M->ia[i]; k < M->ia[i + 1]; k++) {
                int32_t j = M->ja[k];
                if (M->col[j] < c) s -= M->a[k] * x[j];
            }
            x[i] = s / M->diag[i];
        }
    for (int c = 5; c >= 0; c--)
        for (int64_t i = 0; i < n; i++) {
            if (M->col[i] != c) continue;
            zc s = 0;
            for (int64_t k = M->ia[i]; k < M->ia[i + 1]; k++) {
                int32_t j = M->ja[k];
                if (M->col[j] > c) s += M->a[k] * x[j];
            }
            x[i] = x[i] - s / M->diag[i];
        }
}

/* x = M^{-1} y.  For 'S' this is lusol with pre_type='S' including the
 * -(2-w)/w scaling of solvers.f90:743-747 (the sign is kept so iterates match
 * the reference bit for bit in exact arithmetic).  x keeps its previous
 * contents on entry only as storage, exactly like the reference. */
static void psolve(const precond_t *P, const zc *y, zc *xo) {
    int64_t n = P->n;
    if (P->pre == 'J') {
        for (int64_t i = 0; i < n; i++) xo[i] = y[i] / P->mj[i];
        return;
    }
    if (P->pre == 'M') {
        mc_psolve((const mcpre_t *)P->mc, y, xo);
        return;
    }
    const zc *alu = P->alu;
    const int64_t *jlu = P->jlu, *ju = P->ju;
    double w = P->w;
    zc *x = xo - 1; /* 1-based view */
    if (P->pre == 'I') {  /* lusol with pre_type = 'I': unit L, then U with the inverted pivots */
        for (int64_t i = 1; i <= n; i++) {
            zc xi = y[i - 1];
            for (int64_t k = jlu[i]; k <= ju[i] - 1; k++) xi = xi - alu[k] * x[jlu[k]];
            x[i] = xi;
        }
        for (int64_t i = n; i >= 1; i--) {
            zc xi = x[i];
            for (int64_t k = ju[i]; k <= jlu[i + 1] - 1; k++) xi = xi - alu[k] * x[jlu[k]];
            x[i] = alu[i] * xi;
        }
        return;
    }
    for (int64_t i = 1; i <= n; i++) {
        zc xi = y[i - 1];
        for (int64_t k = jlu[i]; k <= ju[i] - 1; k++) xi = xi - alu[k] * x[jlu[k]];
        x[i] = xi * alu[i] * w;
    }
    for (int64_t i = 1; i <= n; i++) x[i] = -x[i] / alu[i] * (2 - w) / w;
    for (int64_t i = n; i >= 1; i--) {
        zc xi = x[i];
        for (int64_t k = ju[i]; k <= jlu[i + 1] - 1; k++) xi = xi - alu[k] * x[jlu[k]];
        x[i] = alu[i] * xi * w;
    }
}

/* Exported single application of the ILU(0) preconditioner (tests). */
int orc_ilu_apply(int64_t n, const zc *a, const int64_t *ia, const int32_t *ja, int64_t band, const zc *y, zc *x) {
    precond_t P;
    int ierr = zilu0(n, band, a, ia, ja, &P);
    if (ierr == 0) psolve(&P, y, x);
    precond_free(&P);
    return ierr;
}

/* Exported single application of the SSOR preconditioner (tests). */
int orc_ssor_apply(int64_t n, const zc *a, const int64_t *ia, const int32_t *ja, double omega, const zc *y, zc *x) {
    precond_t P;
    int ierr = ssorfac(n, a, ia, ja, omega, &P);
    if (ierr == 0) psolve(&P, y, x);
    precond_free(&P);
    return ierr;
}

/* ------------------------------------------------------------------------ */
/* Divergence correction, isotropic scheme of fddc_assemb                    */
/* (div_correc.f90:548-884, iso==1 branches), pcg (:343-402),               */
/* div_correc (:11-147).                                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t np, nl;
    int64_t *pia;
    int32_t *pja;
    zc *pmat;
    int64_t *tia;
    int32_t *tja;
    zc *tmat;
    double *el;
    int64_t *emap; /* 2*nl, 1-based node ids */
    unsigned char *dc;
} divcorr_t;

static void fddc_assemb_iso(int nx, int ny, int nz, const double *a, const double *b, const double *c,
                            const double *sig, divcorr_t *D) {
    const int64_t ncell = (int64_t)nx * ny * nz;
    const int64_t np = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    const int64_t xnl = (int64_t)nx * (ny + 1) * (nz + 1);
    const int64_t ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    const int64_t n1 = (int64_t)nx * ny, n2 = (int64_t)(nx + 1) * (ny + 1);
    D->np = np;
    D->nl = nl;
    D->el = (double *)calloc((size_t)nl, sizeof(double));
    D->emap = (int64_t *)calloc((size_t)2 * nl, sizeof(int64_t));
    D->dc = (unsigned char *)calloc((size_t)np + 1, 1);
    zc *v = (zc *)calloc((size_t)np * 7, sizeof(zc));
    int64_t *vc = (int64_t *)calloc((size_t)np * 7, sizeof(int64_t));
    for (int k = 1; k <= nz + 1; k++)
        for (int j = 1; j <= ny + 1; j++)
            for (int i = 1; i <= nx + 1; i++) {
                int64_t ind = (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i;
                int64_t ie = (int64_t)(k - 1) * n1 + (int64_t)(j - 1) * nx + i;
                if (k != 1 && k != nz + 1 && j != 1 && j != ny + 1 && i != 1 && i != nx + 1) {
                    double s[6];
                    s[0] = (SG(ie - n1 - nx - 1, 3) * a[i - 2] * b[j - 2] + SG(ie - n1 - nx, 3) * a[i - 1] * b[j - 2] +
                            SG(ie - n1 - 1, 3) * a[i - 2] * b[j - 1] + SG(ie - n1, 3) * a[i - 1] * b[j - 1]) / c[k - 2] * 2;
                    s[1] = (SG(ie - n1 - nx - 1, 2) * a[i - 2] * c[k - 2] + SG(ie - n1 - nx, 2) * a[i - 1] * c[k - 2] +
                            SG(ie - nx - 1, 2) * a[i - 2] * c[k - 1] + SG(ie - nx, 2) * a[i - 1] * c[k - 1]) / b[j - 2] * 2;
                    s[2] = (SG(ie - n1 - nx - 1, 1) * b[j - 2] * c[k - 2] + SG(ie - n1 - 1, 1) * b[j - 1] * c[k - 2] +
                            SG(ie - nx - 1, 1) * b[j - 2] * c[k - 1] + SG(ie - 1, 1) * b[j - 1] * c[k - 1]) / a[i - 2] * 2;
                    s[3] = (SG(ie - n1 - nx, 1) * b[j - 2] * c[k - 2] + SG(ie - n1, 1) * b[j - 1] * c[k - 2] +
                            SG(ie - nx, 1) * b[j - 2] * c[k - 1] + SG(ie, 1) * b[j - 1] * c[k - 1]) / a[i - 1] * 2;
                    s[4] = (SG(ie - n1 - 1, 2) * a[i - 2] * c[k - 2] + SG(ie - n1, 2) * a[i - 1] * c[k - 2] +
                            SG(ie - 1, 2) * a[i - 2] * c[k - 1] + SG(ie, 2) * a[i - 1] * c[k - 1]) / b[j - 1] * 2;
                    s[5] = (SG(ie - nx - 1, 3) * a[i - 2] * b[j - 2] + SG(ie - nx, 3) * a[i - 1] * b[j - 2] +
                            SG(ie - 1, 3) * a[i - 2] * b[j - 1] + SG(ie, 3) * a[i - 1] * b[j - 1]) / c[k - 1] * 2;
                    zc *vv = &v[(ind - 1) * 7];
                    int64_t *cc = &vc[(ind - 1) * 7];
                    vv[0] = -s[0];
                    vv[1] = -s[1];
                    vv[2] = -s[2];
                    vv[4] = -s[3];
                    vv[5] = -s[4];
                    vv[6] = -s[5];
                    vv[3] = s[0] + s[1] + s[2] + s[3] + s[4] + s[5];
                    cc[0] = ind - n2;
                    cc[1] = ind - nx - 1;
                    cc[2] = ind - 1;
                    cc[3] = ind;
                    cc[4] = ind + 1;
                    cc[5] = ind + nx + 1;
                    cc[6] = ind + n2;
                } else {
                    v[(ind - 1) * 7] = 1.0;
                    vc[(ind - 1) * 7] = ind;
                    D->dc[ind] = 1;
                }
            }
    D->pia = (int64_t *)calloc((size_t)np + 1, sizeof(int64_t));
    D->pja = (int32_t *)calloc((size_t)np * 7, sizeof(int32_t));
    D->pmat = (zc *)calloc((size_t)np * 7, sizeof(zc));
    int64_t kk = 0;
    for (int64_t i = 1; i <= np; i++) {
        for (int j = 1; j <= 7; j++) {
            int64_t ind = 7 * (i - 1) + j;
            if (v[ind - 1] != 0 && vc[ind - 1] != 0) {
                D->pmat[kk] = v[ind - 1];
                D->pja[kk] = (int32_t)(vc[ind - 1] - 1);
                kk++;
            }
        }
        D->pia[i] = kk;
    }
    free(v);
    free(vc);
    /* divergence operator T (6 entries per interior node; boundary rows empty) */
    v = (zc *)calloc((size_t)np * 6, sizeof(zc));
    vc = (int64_t *)calloc((size_t)np * 6, sizeof(int64_t));
    for (int k = 1; k <= nz + 1; k++)
        for (int j = 1; j <= ny + 1; j++)
            for (int i = 1; i <= nx + 1; i++) {
                int64_t ind = (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i;
                int64_t ie = (int64_t)(k - 1) * n1 + (int64_t)(j - 1) * nx + i;
                if (k != 1 && k != nz + 1 && j != 1 && j != ny + 1 && i != 1 && i != nx + 1) {
                    double s[6];
                    s[0] = -(SG(ie - n1 - nx - 1, 3) * a[i - 2] * b[j - 2] + SG(ie - n1 - nx, 3) * a[i - 1] * b[j - 2] +
                             SG(ie - n1 - 1, 3) * a[i - 2] * b[j - 1] + SG(ie - n1, 3) * a[i - 1] * b[j - 1]) * 2;
                    s[1] = -(SG(ie - n1 - nx - 1, 2) * a[i - 2] * c[k - 2] + SG(ie - n1 - nx, 2) * a[i - 1] * c[k - 2] +
                             SG(ie - nx - 1, 2) * a[i - 2] * c[k - 1] + SG(ie - nx, 2) * a[i - 1] * c[k - 1]) * 2;
                    s[2] = -(SG(ie - n1 - nx - 1, 1) * b[j - 2] * c[k - 2] + SG(ie - n1 - 1, 1) * b[j - 1] * c[k - 2] +
                             SG(ie - nx - 1, 1) * b[j - 2] * c[k - 1] + SG(ie - 1, 1) * b[j - 1] * c[k - 1]) * 2;
                    s[3] = (SG(ie - n1 - nx, 1) * b[j - 2] * c[k - 2] + SG(ie - n1, 1) * b[j - 1] * c[k - 2] +
                            SG(ie - nx, 1) * b[j - 2] * c[k - 1] + SG(ie, 1) * b[j - 1] * c[k - 1]) * 2;
                    s[4] = (SG(ie - n1 - 1, 2) * a[i - 2] * c[k - 2] + SG(ie - n1, 2) * a[i - 1] * c[k - 2] +
                            SG(ie - 1, 2) * a[i - 2] * c[k - 1] + SG(ie, 2) * a[i - 1] * c[k - 1]) * 2;
                    s[5] = (SG(ie - nx - 1, 3) * a[i - 2] * b[j - 2] + SG(ie - nx, 3) * a[i - 1] * b[j - 2] +
                            SG(ie - 1, 3) * a[i - 2] * b[j - 1] + SG(ie, 3) * a[i - 1] * b[j - 1]) * 2;
                    static const int idx[6] = {3, 4, 2, 5, 1, 6};
                    zc *vv = &v[(ind - 1) * 6];
                    int64_t *cc = &vc[(ind - 1) * 6];
                    for (int q = 0; q < 6; q++) vv[q] = s[idx[q] - 1];
                    cc[0] = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i - 1;
                    cc[1] = (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i;
                    cc[2] = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 2) * (nx + 1) + i;
                    cc[3] = xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i;
                    cc[4] = xnl + ynl + (int64_t)(k - 2) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                    cc[5] = xnl + ynl + (int64_t)(k - 1) * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                } else {
                    v[(ind - 1) * 6] = 0;
                    vc[(ind - 1) * 6] = ind;
                }
            }
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                int64_t eid[12] = {
                    (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)(j - 1) * nx + i, (int64_t)(k - 1) * nx * (ny + 1) + (int64_t)j * nx + i,
                    (int64_t)k * nx * (ny + 1) + (int64_t)(j - 1) * nx + i, (int64_t)k * nx * (ny + 1) + (int64_t)j * nx + i,
                    xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i,
                    xnl + (int64_t)k * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i,
                    xnl + (int64_t)(k - 1) * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i + 1,
                    xnl + (int64_t)k * (nx + 1) * ny + (int64_t)(j - 1) * (nx + 1) + i + 1,
                    xnl + ynl + (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i,
                    xnl + ynl + (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i + 1,
                    xnl + ynl + (int64_t)(k - 1) * n2 + (int64_t)j * (nx + 1) + i,
                    xnl + ynl + (int64_t)(k - 1) * n2 + (int64_t)j * (nx + 1) + i + 1};
                int64_t nid1[12] = {(int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i,
                                    (int64_t)(k - 1) * n2 + (int64_t)j * (nx + 1) + i,
                                    (int64_t)k * n2 + (int64_t)(j - 1) * (nx + 1) + i,
                                    (int64_t)k * n2 + (int64_t)j * (nx + 1) + i,
                                    (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i,
                                    (int64_t)k * n2 + (int64_t)(j - 1) * (nx + 1) + i,
                                    (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i + 1,
                                    (int64_t)k * n2 + (int64_t)(j - 1) * (nx + 1) + i + 1,
                                    (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i,
                                    (int64_t)(k - 1) * n2 + (int64_t)(j - 1) * (nx + 1) + i + 1,
                                    (int64_t)(k - 1) * n2 + (int64_t)j * (nx + 1) + i,
                                    (int64_t)(k - 1) * n2 + (int64_t)j * (nx + 1) + i + 1};
                for (int q = 0; q < 12; q++) {
                    int64_t nid2 = q < 4 ? nid1[q] + 1 : (q < 8 ? nid1[q] + nx + 1 : nid1[q] + n2);
                    D->emap[(eid[q] - 1) * 2 + 0] = nid1[q];
                    D->emap[(eid[q] - 1) * 2 + 1] = nid2;
                    D->el[eid[q] - 1] = q < 4 ? a[i - 1] : (q < 8 ? b[j - 1] : c[k - 1]);
                }
            }
    D->tia = (int64_t *)calloc((size_t)np + 1, sizeof(int64_t));
    D->tja = (int32_t *)calloc((size_t)np * 6, sizeof(int32_t));
    D->tmat = (zc *)calloc((size_t)np * 6, sizeof(zc));
    kk = 0;
    for (int64_t i = 1; i <= np; i++) {
        for (int j = 1; j <= 6; j++) {
            int64_t ind = 6 * (i - 1) + j;
            if (v[ind - 1] != 0 && vc[ind - 1] != 0) {
                D->tmat[kk] = v[ind - 1];
                D->tja[kk] = (int32_t)(vc[ind - 1] - 1);
                kk++;
            }
        }
        D->tia[i] = kk;
    }
    free(v);
    free(vc);
}

static void divcorr_free(divcorr_t *D) {
    free(D->pia);
    free(D->pja);
    free(D->pmat);
    free(D->tia);
    free(D->tja);
    free(D->tmat);
    free(D->el);
    free(D->emap);
    free(D->dc);
}

/* Jacobi-CG (div_correc.f90:343-402) */
static int pcg(const zc *kmat, const int64_t *ia, const int32_t *ja, int64_t nl, const zc *b, zc *u, double tol,
               int maxit) {
    zc *r = (zc *)malloc(sizeof(zc) * nl), *rold = (zc *)malloc(sizeof(zc) * nl);
    zc *p = (zc *)malloc(sizeof(zc) * nl), *v = (zc *)malloc(sizeof(zc) * nl);
    zc *mj = (zc *)calloc((size_t)nl, sizeof(zc));
    for (int64_t i = 0; i < nl; i++)
        for (int64_t j = ia[i]; j < ia[i + 1]; j++)
            if (ja[j] == i) mj[i] = kmat[j];
    zamux(nl, u, r, kmat, ja, ia);
    for (int64_t i = 0; i < nl; i++) r[i] = b[i] - r[i];
    double babs = vnorm(b, nl);
    double error = vnorm(r, nl) / babs;
    int k = 0;
    for (int64_t i = 0; i < nl; i++) p[i] = r[i] / mj[i];
    for (int it = 1; it <= maxit; it++) {
        memcpy(rold, r, sizeof(zc) * nl);
        if (error < tol && error > 0) break;
        zamux(nl, p, v, kmat, ja, ia);
        zc num = 0, den = 0;
        for (int64_t i = 0; i < nl; i++) num += conj(r[i] / mj[i]) * r[i];
        for (int64_t i = 0; i < nl; i++) den += conj(p[i]) * v[i];
        zc alpha = num / den;
        for (int64_t i = 0; i < nl; i++) u[i] += alpha * p[i];
        for (int64_t i = 0; i < nl; i++) r[i] -= alpha * v[i];
        zc bn = 0, bd = 0;
        for (int64_t i = 0; i < nl; i++) bn += conj(r[i] / mj[i]) * r[i];
        for (int64_t i = 0; i < nl; i++) bd += conj(rold[i] / mj[i]) * rold[i];
        zc beta = bn / bd;
        for (int64_t i = 0; i < nl; i++) p[i] = r[i] / mj[i] + beta * p[i];
        error = vnorm(r, nl) / babs;
        k++;
    }
    free(r);
    free(rold);
    free(p);
    free(v);
    free(mj);
    return k;
}

/* div_correc (div_correc.f90:11-147): x += grad(phi), P phi = T x. */
static int div_correc(const divcorr_t *D, zc *x, double tol_cor) {
    int64_t np = D->np;
    zc *t = (zc *)calloc((size_t)np, sizeof(zc));
    zc *phi = (zc *)calloc((size_t)np, sizeof(zc));
    zamux(np, x, t, D->tmat, D->tja, D->tia);
    for (int64_t i = 0; i < np; i++)
        if (D->dc[i + 1]) t[i] = 0;
    int it = pcg(D->pmat, D->pia, D->pja, np, t, phi, tol_cor, 2000);
    for (int64_t i = 0; i < D->nl; i++) {
        int64_t n1 = D->emap[2 * i], n2 = D->emap[2 * i + 1];
        if (!(D->dc[n1] && D->dc[n2])) x[i] = x[i] + (phi[n2 - 1] - phi[n1 - 1]) / D->el[i];
    }
    free(t);
    free(phi);
    return it;
}

/* Exported: one divergence correction of x in place (tests). */
int orc_div_correc(int nx, int ny, int nz, const double *a, const double *b, const double *c, const double *sig, zc *x,
                   double tol_cor) {
    divcorr_t D;
    fddc_assemb_iso(nx, ny, nz, a, b, c, sig, &D);
    int it = div_correc(&D, x, tol_cor);
    divcorr_free(&D);
    return it;
}

/* Exported: T x (nodal divergence, boundary nodes zeroed) for tests. */
void orc_divergence(int nx, int ny, int nz, const double *a, const double *b, const double *c, const double *sig,
                    const zc *x, zc *t) {
    divcorr_t D;
    fddc_assemb_iso(nx, ny, nz, a, b, c, sig, &D);
    zamux(D.np, x, t, D.tmat, D.tja, D.tia);
    for (int64_t i = 0; i < D.np; i++)
        if (D.dc[i + 1]) t[i] = 0;
    divcorr_free(&D);
}

/* ------------------------------------------------------------------------ */
/* Krylov solvers.                                                          */
/* opts: pre ('S'|'J'), div_cor (0/1), corr_intv, corr_tol, omega.          */
/* The mesh arguments are only used by the divergence correction.           */
/* ------------------------------------------------------------------------ */
typedef struct {
    int nx, ny, nz;
    const double *a, *b, *c, *sig;
    char pre;
    int div_cor, corr_intv;
    double corr_tol, omega;
    int64_t ilu_band; /* pre = 'I': idd(2) of the caller; 0 keeps every entry */
} korc_opts;

/* multi-colour preconditioner data: one per calling thread, colour buffer reused across solves */
static __thread mcpre_t t_mc;
static __thread int64_t t_mc_cap;

static int make_precond(const korc_opts *o, int64_t n, const zc *K, const int64_t *ia, const int32_t *ja, precond_t *P) {
    if (o->pre == 'J') {
        jacobifac(n, K, ia, ja, P);
        return 0;
    }
    if (o->pre == 'M') {
        jacobifac(n, K, ia, ja, P); /* diagonal */
        P->pre = 'M';
        t_mc.n = n;
        t_mc.a = K;
        t_mc.ia = ia;
        t_mc.ja = ja;
        if (t_mc_cap < n) {
            free(t_mc.col);
            t_mc.col = (unsigned char *)malloc((size_t)n);
            t_mc_cap = n;
        }
        mc_colours(o->nx, o->ny, o->nz, t_mc.col);
        t_mc.diag = P->mj;
        P->mc = &t_mc;
        return 0;
    }
    if (o->pre == 'I') return zilu0(n, o->ilu_band, K, ia, ja, P);
    return ssorfac(n, K, ia, ja, o->omega, P);
}

/*
 * Bicg_stab_p (solvers.f90:522-719).  Returns the reference's iters(1): the
 * loop index at which the stopping test fired (or itmax).  err_rec[itmax]
 * receives the relative residual recorded at the top of each iteration.
 */
int orc_bicgstab(const korc_opts *o, int64_t n, const zc *K, const int64_t *ia, const int32_t *ja, const zc *b, zc *x,
                 double eps, int itmax, double *err_rec) {
    precond_t P;
    divcorr_t D;
    int iters = 0;
    if (o->div_cor) fddc_assemb_iso(o->nx, o->ny, o->nz, o->a, o->b, o->c, o->sig, &D);
    make_precond(o, n, K, ia, ja, &P);
    size_t sz = sizeof(zc) * (size_t)n;
    zc *r = (zc *)malloc(sz), *rhat = (zc *)malloc(sz), *p = (zc *)calloc((size_t)n, sizeof(zc));
    zc *y = (zc *)calloc((size_t)n, sizeof(zc)), *s = (zc *)malloc(sz), *z = (zc *)calloc((size_t)n, sizeof(zc));
    zc *vk = (zc *)calloc((size_t)n, sizeof(zc)), *t = (zc *)malloc(sz), *xmin = (zc *)calloc((size_t)n, sizeof(zc));
    for (int i = 0; i < itmax; i++) err_rec[i] = 0;
    zamux(n, x, r, K, ja, ia);
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - r[i];
    memcpy(rhat, r, sz);
    zc rho = 1.0, alpha = 1.0, omega = 1.0, rhoold;
    double babs = vnorm(b, n);
    double error = vnorm(r, n) / babs;
    if (isnan(error)) goto done;
    for (int i = 1; i <= itmax; i++) {
        iters = i;
        err_rec[i - 1] = error;
        if (error < eps) {
            if (i == itmax) memcpy(x, xmin, sz);
            break;
        }
        if (i % o->corr_intv == 0) {
            if (o->div_cor) {
                div_correc(&D, x, o->corr_tol);
                zamux(n, x, r, K, ja, ia);
                for (int64_t q = 0; q < n; q++) r[q] = b[q] - r[q];
                memcpy(rhat, r, sz);
            }
            memcpy(xmin, x, sz);
        }
        rhoold = rho;
        rho = dotc(rhat, r, n);
        zc beta = (rho / rhoold) * (alpha / omega);
        for (int64_t q = 0; q < n; q++) p[q] = r[q] + beta * (p[q] - omega * vk[q]);
        psolve(&P, p, y);
        zamux(n, y, vk, K, ja, ia);
        alpha = rho / dotc(rhat, vk, n);
        for (int64_t q = 0; q < n; q++) s[q] = r[q] - alpha * vk[q];
        psolve(&P, s, z);
        zamux(n, z, t, K, ja, ia);
        omega = dotc(t, s, n) / dotc(t, t, n);
        for (int64_t q = 0; q < n; q++) x[q] = x[q] + alpha * y[q] + omega * z[q];
        for (int64_t q = 0; q < n; q++) r[q] = s[q] - omega * t[q];
        error = vnorm(r, n) / babs;
        if (isnan(error)) break;
    }
done:
    free(r);
    free(rhat);
    free(p);
    free(y);
    free(s);
    free(z);
    free(vk);
    free(t);
    free(xmin);
    precond_free(&P);
    if (o->div_cor) divcorr_free(&D);
    return iters;
}

/*
 * pgpbicg (solvers.f90:137-315), right-preconditioned GPBiCG.  Returns the
 * iteration at which ||r||/||b|| <= tol (iters(1)), or maxit+1 when the loop
 * ran out (the reference leaves iters(1) unset in that case).
 */
int orc_gpbicg(const korc_opts *o, int64_t n, const zc *K, const int64_t *ia, const int32_t *ja, const zc *b, zc *x,
               double tol, int maxit, double *err_rec) {
    precond_t P;
    divcorr_t D;
    if (o->div_cor) fddc_assemb_iso(o->nx, o->ny, o->nz, o->a, o->b, o->c, o->sig, &D);
    make_precond(o, n, K, ia, ja, &P);
    size_t sz = sizeof(zc) * (size_t)n;
#define ZN() ((zc *)calloc((size_t)n, sizeof(zc)))
    zc *r = ZN(), *rp = ZN(), *y = ZN(), *p = ZN(), *u = ZN(), *w = ZN(), *t = ZN(), *tp = ZN();
    zc *ap = ZN(), *at = ZN(), *z = ZN(), *tmp = ZN(), *r0 = ZN(), *rold = ZN(), *tpold = ZN();
#undef ZN
    for (int i = 0; i < maxit; i++) err_rec[i] = 0;
    zamux(n, x, r, K, ja, ia);
    for (int64_t q = 0; q < n; q++) r[q] = b[q] - r[q];
    memcpy(r0, r, sz);
    psolve(&P, r, rp);
    zc beta = 0, alpha, omega, eta;
    double babs = vnorm(b, n);
    int iters = maxit + 1;
    for (int i = 1; i <= maxit; i++) {
        if (i % o->corr_intv == 0 && o->div_cor) {
            div_correc(&D, x, o->corr_tol);
            zamux(n, x, r, K, ja, ia);
            for (int64_t q = 0; q < n; q++) r[q] = b[q] - r[q];
            memcpy(r0, r, sz);
        }
        memcpy(tpold, tp, sz);
        memcpy(rold, r, sz);
        for (int64_t q = 0; q < n; q++) p[q] = rp[q] + beta * (p[q] - u[q]);
        zamux(n, p, ap, K, ja, ia);
        alpha = dotc(r0, r, n) / dotc(r0, ap, n);
        for (int64_t q = 0; q < n; q++) y[q] = t[q] - r[q] - alpha * w[q] + alpha * ap[q];
        for (int64_t q = 0; q < n; q++) t[q] = r[q] - alpha * ap[q];
        psolve(&P, ap, tmp);
        for (int64_t q = 0; q < n; q++) tp[q] = rp[q] - alpha * tmp[q];
        zamux(n, tp, at, K, ja, ia);
        if (i == 1) {
            omega = dotc(at, t, n) / dotc(at, at, n);
            eta = 0;
        } else {
            zc yy = dotc(y, y, n), att = dotc(at, t, n), yt = dotc(y, t, n), aty = dotc(at, y, n);
            zc atat = dotc(at, at, n), yat = dotc(y, at, n);
            omega = (yy * att - yt * aty) / (atat * yy - yat * aty);
            eta = (atat * yt - yat * att) / (atat * yy - yat * aty);
        }
        for (int64_t q = 0; q < n; q++) u[q] = omega * tmp[q] + eta * (tpold[q] - rp[q] + beta * u[q]);
        for (int64_t q = 0; q < n; q++) z[q] = omega * rp[q] + eta * z[q] - alpha * u[q];
        for (int64_t q = 0; q < n; q++) x[q] = x[q] + alpha * p[q] + z[q];
        for (int64_t q = 0; q < n; q++) r[q] = t[q] - eta * y[q] - omega * at[q];
        double e = vnorm(r, n) / babs;
        err_rec[i - 1] = e;
        if (e <= tol) {
            iters = i;
            break;
        }
        psolve(&P, r, rp);
        beta = alpha / omega * dotc(r0, r, n) / dotc(r0, rold, n);
        for (int64_t q = 0; q < n; q++) w[q] = at[q] + beta * ap[q];
    }
    free(r);
    free(rp);
    free(y);
    free(p);
    free(u);
    free(w);
    free(t);
    free(tp);
    free(ap);
    free(at);
    free(z);
    free(tmp);
    free(r0);
    free(rold);
    free(tpold);
    precond_free(&P);
    if (o->div_cor) divcorr_free(&D);
    return iters;
}

/* Flat-argument wrappers for ctypes. */
int orc_solve(int solver, int nx, int ny, int nz, const double *a, const double *b, const double *c, const double *sig,
              char pre, int div_cor, int corr_intv, double corr_tol, double omega, int64_t n, const zc *K,
              const int64_t *ia, const int32_t *ja, const zc *rhs, zc *x, double eps, int itmax, double *err_rec,
              int64_t ilu_band) {
    korc_opts o = {nx, ny, nz, a, b, c, sig, pre, div_cor, corr_intv, corr_tol, omega, ilu_band};
    if (solver == 3) return orc_gpbicg(&o, n, K, ia, ja, rhs, x, eps, itmax, err_rec);
    return orc_bicgstab(&o, n, K, ia, ja, rhs, x, eps, itmax, err_rec);
}

/* Bounded-time sample for the CPU baseline: run exactly `iters` BiCGStab
 * iterations (no stopping test) and return; used to time the per-iteration
 * cost of the serial SSOR-BiCGStab path on large meshes. */
int orc_bicgstab_fixed(int64_t n, const zc *K, const int64_t *ia, const int32_t *ja, const zc *b, zc *x, int iters) {
    korc_opts o = {0, 0, 0, NULL, NULL, NULL, NULL, 'S', 0, 200, 1e-3, 1.0, 0};
    double *err = (double *)calloc((size_t)iters + 1, sizeof(double));
    int r = orc_bicgstab(&o, n, K, ia, ja, b, x, -1.0, iters, err);
    free(err);
    return r;
}

/* ------------------------------------------------------------------------ */
/* EXCMG prolongation (excmg.f90:9-77 extint_v, :357-512 quad_interp_e,     */
/* :514-660 cubic_interp, :662-752 cal_coef, :754-772 lbf).                 */
/* mid_quirk=1 keeps cal_coef's along-edge nodes at the midpoints of the    */
/* first fine sub-edge of every coarse edge (excmg.f90:685,711,737);        */
/* mid_quirk=0 puts them at the coarse-edge midpoints.                       */
/* ------------------------------------------------------------------------ */
static double lbf(int l_ord, const double *cx, int id, double x) { /* cx 1-based via cx[q-1] */
    double num = 1.0, den = 1.0;
    for (int i = 1; i <= l_ord + 1; i++)
        if (i != id) {
            num = num * (x - cx[i - 1]);
            den = den * (cx[id - 1] - cx[i - 1]);
        }
    return num / den;
}

/* coef[comp][ijk-1][ind-1]; R=(2m+1)^2*2m rows, Cc=(m+1)^2*m cols */
static void cal_coef(const double *aax, const double *bby, const double *ccz, int m, int n1, int n2, int n3,
                     int mid_quirk, double *coef) {
    const int R = (2 * m + 1) * (2 * m + 1) * 2 * m, Cc = (m + 1) * (m + 1) * m;
    double coor[3];
    double cx1[9], cx2[9], cx3[9];
#define AAX(i) aax[(i)-1]
#define BBY(i) bby[(i)-1]
#define CCZ(i) ccz[(i)-1]
    for (int comp = 0; comp < 3; comp++) {
        const double *p1 = comp == 0 ? bby : aax;          /* cx1 axis */
        const double *p2 = comp == 2 ? bby : ccz;          /* cx2 axis */
        const double *pe = comp == 0 ? aax : (comp == 1 ? bby : ccz); /* along-edge axis */
        int b1 = comp == 0 ? n2 : n1, b2 = comp == 2 ? n2 : n3, be = comp == 0 ? n1 : (comp == 1 ? n2 : n3);
        for (int q = 0; q <= m; q++) {
            cx1[q] = p1[(b1 - 1) * m * 2 + 1 + 2 * q - 1];
            cx2[q] = p2[(b2 - 1) * m * 2 + 1 + 2 * q - 1];
        }
        for (int q = 0; q < m; q++) {
            int base = (be - 1) * m * 2;
            if (mid_quirk)
                cx3[q] = (pe[base + 1 + 2 * q - 1] + pe[base + 2 + 2 * q - 1]) / 2;
            else
                cx3[q] = (pe[base + 1 + 2 * q - 1] + pe[base + 3 + 2 * q - 1]) / 2;
        }
        for (int k = 1; k <= 2 * m; k++)
            for (int j = 1; j <= 2 * m + 1; j++)
                for (int i = 1; i <= 2 * m + 1; i++) {
                    int ijk = (k - 1) * (2 * m + 1) * (2 * m + 1) + (j - 1) * (2 * m + 1) + i;
                    double emid = (pe[(be - 1) * m * 2 + k - 1] + pe[(be - 1) * m * 2 + k]) / 2;
                    double t1 = p1[(b1 - 1) * m * 2 + i - 1];
                    double t2 = p2[(b2 - 1) * m * 2 + j - 1];
                    if (comp == 0) { coor[0] = emid; coor[1] = t1; coor[2] = t2; }
                    else if (comp == 1) { coor[0] = t1; coor[1] = emid; coor[2] = t2; }
                    else { coor[0] = t1; coor[1] = t2; coor[2] = emid; }
                    for (int kk = 1; kk <= m; kk++)
                        for (int jj = 1; jj <= m + 1; jj++)
                            for (int ii = 1; ii <= m + 1; ii++) {
                                int ind = (kk - 1) * (m + 1) * (m + 1) + (jj - 1) * (m + 1) + ii;
                                double v;
                                if (comp == 0)
                                    v = lbf(m, cx1, ii, coor[1]) * lbf(m, cx2, jj, coor[2]) * lbf(m - 1, cx3, kk, coor[0]);
                                else if (comp == 1)
                                    v = lbf(m, cx1, ii, coor[0]) * lbf(m, cx2, jj, coor[2]) * lbf(m - 1, cx3, kk, coor[1]);
                                else
                                    v = lbf(m, cx1, ii, coor[0]) * lbf(m, cx2, jj, coor[1]) * lbf(m - 1, cx3, kk, coor[2]);
                                coef[((size_t)comp * R + ijk - 1) * Cc + ind - 1] = v;
                            }
                }
    }
#undef AAX
#undef BBY
#undef CCZ
}

static void node_coords(int n, const double *h, int nair, int is_z, double *out) {
    double s = 0;
    if (is_z) {
        for (int i = 0; i < nair; i++) s += h[i];
        out[0] = -s;
    } else {
        for (int i = 0; i < n; i++) s += h[i];
        out[0] = -s / 2;
    }
    for (int i = 1; i <= n; i++) out[i] = out[i - 1] + h[i - 1];
}

/*
 * Generic block interpolation used by quad_interp_e (m=2) and cubic_interp
 * (m=4).  nx,ny,nz are the FINE sizes of this step; the coarse grid has
 * nx/2.. cells.  Fine blocks of 2m cells per axis; later blocks overwrite the
 * shared faces exactly as the reference loop order does.
 */
static void block_interp(int m, int nx, int ny, int nz, const double *a1, const double *b1, const double *c1, int nair,
                         const zc *u1, zc *u2, int mid_quirk) {
    double *aax = (double *)malloc(sizeof(double) * (nx + 1));
    double *bby = (double *)malloc(sizeof(double) * (ny + 1));
    double *ccz = (double *)malloc(sizeof(double) * (nz + 1));
    node_coords(nx, a1, 0, 0, aax);
    node_coords(ny, b1, 0, 0, bby);
    node_coords(nz, c1, nair, 1, ccz);
    const int R = (2 * m + 1) * (2 * m + 1) * 2 * m, Cc = (m + 1) * (m + 1) * m;
    double *coef = (double *)malloc(sizeof(double) * 3 * R * Cc);
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2; /* coarse sizes */
    const int64_t fxnl = (int64_t)nx * (ny + 1) * (nz + 1), fynl = (int64_t)(nx + 1) * ny * (nz + 1);
    const int64_t cxnl = (int64_t)cx * (cy + 1) * (cz + 1), cynl = (int64_t)(cx + 1) * cy * (cz + 1);
    const int bs = 2 * m; /* fine cells per block */
    for (int k = 1; k <= nz / bs; k++)
        for (int j = 1; j <= ny / bs; j++)
            for (int i = 1; i <= nx / bs; i++) {
                cal_coef(aax, bby, ccz, m, i, j, k, mid_quirk, coef);
                /* fine origin (1-based cell/node indices) and coarse origin */
                int fi0 = (i - 1) * bs, fj0 = (j - 1) * bs, fk0 = (k - 1) * bs;
                int ci0 = (i - 1) * m, cj0 = (j - 1) * m, ck0 = (k - 1) * m;
                for (int comp = 0; comp < 3; comp++) {
                    for (int r = 0; r < R; r++) {
                        /* decode fine row: slow = along-edge e (0..2m-1), mid, fast */
                        int e = r / ((2 * m + 1) * (2 * m + 1));
                        int mid = (r / (2 * m + 1)) % (2 * m + 1);
                        int fast = r % (2 * m + 1);
                        int64_t fidx;
                        if (comp == 0) /* e=x, mid=z, fast=y */
                            fidx = (int64_t)(fk0 + mid) * nx * (ny + 1) + (int64_t)(fj0 + fast) * nx + (fi0 + e);
                        else if (comp == 1) /* e=y, mid=z, fast=x */
                            fidx = fxnl + (int64_t)(fk0 + mid) * (nx + 1) * ny + (int64_t)(fj0 + e) * (nx + 1) + (fi0 + fast);
                        else /* e=z, mid=y, fast=x */
                            fidx = fxnl + fynl + (int64_t)(fk0 + e) * (nx + 1) * (ny + 1) + (int64_t)(fj0 + mid) * (nx + 1) +
                                   (fi0 + fast);
                        zc acc = 0;
                        for (int q = 0; q < Cc; q++) {
                            int ce = q / ((m + 1) * (m + 1));
                            int cmid = (q / (m + 1)) % (m + 1);
                            int cfast = q % (m + 1);
                            int64_t cidx;
                            if (comp == 0)
                                cidx = (int64_t)(ck0 + cmid) * cx * (cy + 1) + (int64_t)(cj0 + cfast) * cx + (ci0 + ce);
                            else if (comp == 1)
                                cidx = cxnl + (int64_t)(ck0 + cmid) * (cx + 1) * cy + (int64_t)(cj0 + ce) * (cx + 1) + (ci0 + cfast);
                            else
                                cidx = cxnl + cynl + (int64_t)(ck0 + ce) * (cx + 1) * (cy + 1) + (int64_t)(cj0 + cmid) * (cx + 1) +
                                       (ci0 + cfast);
                            acc += coef[((size_t)comp * R + r) * Cc + q] * u1[cidx];
                        }
                        u2[fidx] = acc;
                    }
                }
            }
    free(coef);
    free(aax);
    free(bby);
    free(ccz);
}

/* quad_interp_e on its own (4h -> 2h); nx.. are the 2h (output) sizes. */
void orc_quad_interp(int nx, int ny, int nz, const double *a2, const double *b2, const double *c2, int nair, const zc *u0,
                     zc *out, int mid_quirk) {
    int64_t n1 = (int64_t)nx * (ny + 1) * (nz + 1) + (int64_t)(nx + 1) * ny * (nz + 1) + (int64_t)(nx + 1) * (ny + 1) * nz;
    for (int64_t q = 0; q < n1; q++) out[q] = 0;
    block_interp(2, nx, ny, nz, a2, b2, c2, nair, u0, out, mid_quirk);
}

/* cubic_interp on its own (2h -> h); nx.. are the h (output) sizes. */
void orc_cubic_interp(int nx, int ny, int nz, const double *a1, const double *b1, const double *c1, int nair, const zc *u1,
                      zc *out, int mid_quirk) {
    int64_t nl = (int64_t)nx * (ny + 1) * (nz + 1) + (int64_t)(nx + 1) * ny * (nz + 1) + (int64_t)(nx + 1) * (ny + 1) * nz;
    for (int64_t q = 0; q < nl; q++) out[q] = 0;
    block_interp(4, nx, ny, nz, a1, b1, c1, nair, u1, out, mid_quirk);
}

/*
 * extint_v: u = cubic( (1+2^-2) u1 - 2^-2 quad(u0) ).  nx,ny,nz,a1,b1,c1,nair
 * describe the fine (h) level; u1 lives on the 2h level, u0 on the 4h level.
 * Returns the number of NaN entries found (the reference prints them).
 */
int orc_extint_v(int nx, int ny, int nz, const double *a1, const double *b1, const double *c1, int nair, const zc *u0,
                 const zc *u1, zc *u, int mid_quirk) {
    const double order = 2.0;
    double *a2 = (double *)malloc(sizeof(double) * nx / 2), *b2 = (double *)malloc(sizeof(double) * ny / 2);
    double *c2 = (double *)malloc(sizeof(double) * nz / 2);
    for (int i = 1; i <= nx / 2; i++) a2[i - 1] = a1[2 * i - 2] + a1[2 * i - 1];
    for (int i = 1; i <= ny / 2; i++) b2[i - 1] = b1[2 * i - 2] + b1[2 * i - 1];
    for (int i = 1; i <= nz / 2; i++) c2[i - 1] = c1[2 * i - 2] + c1[2 * i - 1];
    int hx = nx / 2, hy = ny / 2, hz = nz / 2;
    int64_t n1 = (int64_t)hx * (hy + 1) * (hz + 1) + (int64_t)(hx + 1) * hy * (hz + 1) + (int64_t)(hx + 1) * (hy + 1) * hz;
    zc *utmp = (zc *)calloc((size_t)n1, sizeof(zc));
    double co1 = 1.0 + 1.0 / pow(2.0, order), co2 = 1.0 / pow(2.0, order);
    block_interp(2, hx, hy, hz, a2, b2, c2, nair / 2, u0, utmp, mid_quirk);
    for (int64_t q = 0; q < n1; q++) utmp[q] = co1 * u1[q] - co2 * utmp[q];
    int64_t nl = (int64_t)nx * (ny + 1) * (nz + 1) + (int64_t)(nx + 1) * ny * (nz + 1) + (int64_t)(nx + 1) * (ny + 1) * nz;
    for (int64_t q = 0; q < nl; q++) u[q] = 0;
    block_interp(4, nx, ny, nz, a1, b1, c1, nair, utmp, u, mid_quirk);
    int nnan = 0;
    for (int64_t q = 0; q < nl; q++)
        if (isnan(cabs(u[q]))) nnan++;
    free(utmp);
    free(a2);
    free(b2);
    free(c2);
    return nnan;
}

/* ------------------------------------------------------------------------ */
/* post_process (fdfe_main.f90:549-716) + arho_interp2 (:718-790).          */
/* x1, x2: the xy and yx solutions (nl each) of one frequency.              */
/* rd=2 reproduces the reference's transposed receiver stencil (quirk 5);   */
/* rd=1 is the un-transposed stencil.                                       */
/* out[nrec*4]: (Re Zxy, Im Zxy, Re Zyx, Im Zyx) (out_type 0/1) or           */
/* (rho_xy, rho_yx, phi_xy, phi_yx) (out_type 2).  tip[nrec*4]: tippers.    */
/* Returns 0, or -(receiver index) for a receiver outside the grid.         */
/* ------------------------------------------------------------------------ */
static double qcoef(double x, const double *x0, int q) {
    if (q == 0) return (x - x0[1]) * (x - x0[2]) / (x0[0] - x0[1]) / (x0[0] - x0[2]);
    if (q == 1) return (x - x0[0]) * (x - x0[2]) / (x0[1] - x0[0]) / (x0[1] - x0[2]);
    return (x - x0[0]) * (x - x0[1]) / (x0[2] - x0[0]) / (x0[2] - x0[1]);
}

static int arho_interp2(int mode, int rd, int nx, int ny, const double *ax, const double *by, const zc *ex, const zc *ey,
                        const zc *hx, const zc *hy, const zc *hz, int nrec, const double *recv, zc *arho) {
    /* field arrays are F(i,j,mode) 1-based, nx*ny*2, column-major */
#define F(arr, i, j) arr[((size_t)(mode - 1) * ny + (j)-1) * nx + (i)-1]
    double *aax = (double *)malloc(sizeof(double) * nx), *bby = (double *)malloc(sizeof(double) * ny);
    double sa = 0, sb = 0;
    for (int i = 0; i < nx; i++) sa += ax[i];
    for (int i = 0; i < ny; i++) sb += by[i];
    aax[0] = (ax[0] - sa) / 2;
    bby[0] = (by[0] - sb) / 2;
    for (int i = 2; i <= nx; i++) {
        double s = 0;
        for (int q = 0; q < i - 1; q++) s += ax[q];
        aax[i - 1] = -sa / 2 + s + ax[i - 1] / 2;
    }
    for (int i = 2; i <= ny; i++) {
        double s = 0;
        for (int q = 0; q < i - 1; q++) s += by[q];
        bby[i - 1] = -sb / 2 + s + by[i - 1] / 2;
    }
    int rc = 0;
    for (int i = 1; i <= nrec; i++) {
        double xr = recv[(size_t)0 * nrec + i - 1], yr = recv[(size_t)1 * nrec + i - 1];
        int irec = -1, jrec = -1;
        for (int j = 1; j <= nx - 1; j++)
            if (xr >= aax[j - 1] && xr <= aax[j]) { irec = j; break; }
        for (int j = 1; j <= ny - 1; j++)
            if (yr >= bby[j - 1] && yr <= bby[j]) { jrec = j; break; }
        if (irec < 2 || jrec < 2 || irec + 1 > nx || jrec + 1 > ny) { rc = -i; break; }
        if (rd == 2 && (jrec + 1 > nx || irec + 1 > ny)) { rc = -i; break; }
        double c1[3], c2[3];
        for (int q = 0; q < 3; q++) c1[q] = qcoef(xr, &aax[irec - 2], q);
        for (int q = 0; q < 3; q++) c2[q] = qcoef(yr, &bby[jrec - 2], q);
        zc e[5] = {0, 0, 0, 0, 0};
        for (int m = 1; m <= 3; m++)
            for (int n = 1; n <= 3; n++) {
                double w = c1[m - 1] * c2[n - 1];
                if (rd == 1) {
                    e[0] += w * F(ex, m + irec - 2, n + jrec - 2);
                    e[1] += w * F(ey, m + irec - 2, n + jrec - 2);
                    e[2] += w * F(hx, m + irec - 2, n + jrec - 2);
                    e[3] += w * F(hy, m + irec - 2, n + jrec - 2);
                    e[4] += w * F(hz, m + irec - 2, n + jrec - 2);
                } else {
                    e[0] += w * F(ex, m + jrec - 2, n + irec - 2);
                    e[1] += w * F(ey, m + jrec - 2, n + irec - 2);
                    e[2] += w * F(hx, m + jrec - 2, n + irec - 2);
                    e[3] += w * F(hy, m + jrec - 2, n + irec - 2);
                    e[4] += w * F(hz, m + irec - 2, n + jrec - 2);
                }
            }
        for (int q = 0; q < 5; q++) arho[(size_t)q * nrec + i - 1] = e[q];
    }
    free(aax);
    free(bby);
    return rc;
#undef F
}

/* post_process with an optional receiver plane per surface column (the
 * topography branch, fdfe_main.f90:604-616): mcol[(j-1)*nx+i-1] is the node
 * plane m of column (i,j) (NULL: nair everywhere) and czcol the vertical step of
 * its H derivatives (NULL: c(nair+1), as the reference uses for every column). */
static int post_process_cols(int nx, int ny, int nz, int nair, const double *a, const double *b, const double *c,
                             double ff, const zc *x1, const zc *x2, int nrec, const double *recv, int out_type, int rd,
                             double *out, double *tip, zc *fields_out, const int *mcol, const double *czcol);
int orc_post_process(int nx, int ny, int nz, int nair, const double *a, const double *b, const double *c, double ff,
                     const zc *x1, const zc *x2, int nrec, const double *recv, int out_type, int rd, double *out,
                     double *tip, zc *fields_out) {
    return post_process_cols(nx, ny, nz, nair, a, b, c, ff, x1, x2, nrec, recv, out_type, rd, out, tip, fields_out,
                             NULL, NULL);
}
int orc_post_process_topo(int nx, int ny, int nz, int nair, const double *a, const double *b, const double *c,
                          double ff, const zc *x1, const zc *x2, int nrec, const double *recv, int out_type, int rd,
                          double *out, double *tip, zc *fields_out, const int *mcol, const double *czcol) {
    return post_process_cols(nx, ny, nz, nair, a, b, c, ff, x1, x2, nrec, recv, out_type, rd, out, tip, fields_out,
                             mcol, czcol);
}
static int post_process_cols(int nx, int ny, int nz, int nair, const double *a, const double *b, const double *c,
                             double ff, const zc *x1, const zc *x2, int nrec, const double *recv, int out_type, int rd,
                             double *out, double *tip, zc *fields_out, const int *mcol, const double *czcol) {
    const int64_t n1 = (int64_t)nx * (ny + 1) * (nz + 1), n2 = (int64_t)ny * (nz + 1) * (nx + 1);
    size_t nxy = (size_t)nx * ny;
    zc *ex = (zc *)calloc(nxy * 2, sizeof(zc)), *ey = (zc *)calloc(nxy * 2, sizeof(zc));
    zc *hx = (zc *)calloc(nxy * 2, sizeof(zc)), *hy = (zc *)calloc(nxy * 2, sizeof(zc)), *hz = (zc *)calloc(nxy * 2, sizeof(zc));
    zc *arho = (zc *)calloc((size_t)nrec * 5, sizeof(zc)), *arho2 = (zc *)calloc((size_t)nrec * 5, sizeof(zc));
    const zc iwm = I * 2.0 * PI * ff * MU;
#define X(v, n) v[(n)-1]
#define FLD(arr, i, j, md) arr[((size_t)((md)-1) * ny + (j)-1) * nx + (i)-1]
    for (int pol = 1; pol <= 2; pol++) {
        const zc *xv = pol == 1 ? x1 : x2;
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                const int m = mcol ? mcol[(size_t)(j - 1) * nx + i - 1] : nair;
                const double cz = czcol ? czcol[(size_t)(j - 1) * nx + i - 1] : c[nair];
                int64_t idx = (int64_t)m * nx * (ny + 1) + (int64_t)(j - 1) * nx + i;
                int64_t idx2 = n1 + (int64_t)m * ny * (nx + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                int64_t idx3 = n1 + n2 + (int64_t)m * (nx + 1) * (ny + 1) + (int64_t)(j - 1) * (nx + 1) + i;
                if (pol == 1) {
                    FLD(ex, i, j, 1) = (X(x1, idx) + X(x1, idx + nx)) / 2.0;
                    FLD(ex, i, j, 2) = (X(x2, idx) + X(x2, idx + nx)) / 2.0;
                    FLD(ey, i, j, 1) = (X(x1, idx2) + X(x1, idx2 + 1)) / 2.0;
                    FLD(ey, i, j, 2) = (X(x2, idx2) + X(x2, idx2 + 1)) / 2.0;
                }
                zc exz = ((X(xv, idx + (int64_t)nx * (ny + 1)) + X(xv, idx + (int64_t)nx * (ny + 1) + nx)) / 2.0 -
                          FLD(ex, i, j, pol)) / cz;
                zc ezx = ((X(xv, idx3 + 1) + X(xv, idx3 + nx + 2)) / 2.0 - (X(xv, idx3 + nx + 1) + X(xv, idx3)) / 2.0) / a[i - 1];
                zc eyz = ((X(xv, idx2 + (int64_t)ny * (nx + 1)) + X(xv, idx2 + (int64_t)ny * (nx + 1) + 1)) / 2.0 -
                          FLD(ey, i, j, pol)) / cz;
                zc ezy = (-(X(xv, idx3) + X(xv, idx3 + 1)) / 2.0 + (X(xv, idx3 + nx + 1) + X(xv, idx3 + nx + 2)) / 2.0) / b[j - 1];
                zc exy = (X(xv, idx + nx) - X(xv, idx)) / b[j - 1];
                zc eyx = (X(xv, idx2 + 1) - X(xv, idx2)) / a[i - 1];
                FLD(hy, i, j, pol) = (exz - ezx) / iwm;
                FLD(hx, i, j, pol) = (ezy - eyz) / iwm;
                FLD(hz, i, j, pol) = (exy - eyx) / iwm;
            }
    }
#undef X
#undef FLD
    int rc = arho_interp2(1, rd, nx, ny, a, b, ex, ey, hx, hy, hz, nrec, recv, arho);
    if (rc == 0) rc = arho_interp2(2, rd, nx, ny, a, b, ex, ey, hx, hy, hz, nrec, recv, arho2);
    if (rc == 0) {
#define AR(arr, i, q) arr[(size_t)((q)-1) * nrec + (i)-1]
        for (int i = 1; i <= nrec; i++) {
            zc tmp = AR(arho, i, 3) * AR(arho2, i, 4) - AR(arho2, i, 3) * AR(arho, i, 4);
            zc z1 = (AR(arho2, i, 1) * AR(arho, i, 3) - AR(arho, i, 1) * AR(arho2, i, 3)) / tmp;
            zc z2 = (AR(arho, i, 2) * AR(arho2, i, 4) - AR(arho2, i, 2) * AR(arho, i, 4)) / tmp;
            double *o = &out[(size_t)(i - 1) * 4];
            if (out_type == 2) {
                o[0] = cabs(z1 * z1 * I) / (2.0 * PI * ff * MU);
                o[1] = cabs(z2 * z2 * I) / (2.0 * PI * ff * MU);
                o[2] = -atan(cimag(z1) / creal(z1)) * 180.0 / PI;
                o[3] = -atan(cimag(z2) / creal(z2)) * 180.0 / PI;
            } else {
                o[0] = creal(z1);
                o[1] = cimag(z1);
                o[2] = creal(z2);
                o[3] = cimag(z2);
            }
            zc tx = (AR(arho2, i, 4) * AR(arho, i, 5) - AR(arho, i, 4) * AR(arho2, i, 5)) / tmp;
            zc ty = (AR(arho, i, 3) * AR(arho2, i, 5) - AR(arho2, i, 3) * AR(arho, i, 5)) / tmp;
            if (tip) {
                double *t = &tip[(size_t)(i - 1) * 4];
                t[0] = creal(tx);
                t[1] = cimag(tx);
                t[2] = creal(ty);
                t[3] = cimag(ty);
            }
            if (fields_out) { /* (Ex,Ey,Hx,Hy,Hz) x 2 polarisations at the receiver */
                for (int q = 1; q <= 5; q++) {
                    fields_out[(size_t)(i - 1) * 10 + q - 1] = AR(arho, i, q);
                    fields_out[(size_t)(i - 1) * 10 + 5 + q - 1] = AR(arho2, i, q);
                }
            }
        }
#undef AR
    }
    free(ex);
    free(ey);
    free(hx);
    free(hy);
    free(hz);
    free(arho);
    free(arho2);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Symmetric Gauss-Seidel sweep on a CSR matrix, in place: one forward pass  */
/* then one backward pass of x_i = (b_i - sum_{j != i} a_ij x_j) / a_ii.     */
/* The smoother of the oracle's converged-solution solver (oracle.py,        */
/* converged_solve); no counterpart in the reference.                        */
/* ------------------------------------------------------------------------ */
void orc_sgs(int64_t n, const zc *a, const int64_t *ia, const int32_t *ja, const zc *b, zc *x) {
    for (int pass = 0; pass < 2; pass++) {
        for (int64_t q = 0; q < n; q++) {
            const int64_t i = pass == 0 ? q : n - 1 - q;
            zc s = b[i], d = 0;
            for (int64_t k = ia[i]; k < ia[i + 1]; k++) {
                const int64_t j = ja[k];
                if (j == i)
                    d = a[k];
                else
                    s -= a[k] * x[j];
            }
            if (d != 0) x[i] = s / d;
        }
    }
}
