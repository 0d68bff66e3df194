// sfdx_device.cuh -- device-side building blocks of the GB300 forward solver.
//
// Layout in HBM (one mesh level):
//   * edge vectors: the reference's edge order (all Ex, then all Ey, then all
//     Ez; x fastest inside each block, fdfe_main.f90:261,310,358), with the
//     systems of a batch interleaved innermost: value(e, s) at [e * ns + s].
//     ns = 1 gives exactly the reference vector.
//   * sigma: [6][ncell] (Fortran sigma(ncell,6)), one copy per precision.
//   * 1-D spacing tables per axis (AxisT below), precomputed on the host in
//     FP64 from a, b, c with the reference's formulas.
//
// Every kernel is matrix-free: the 13-point rows of fd_assemb
// (fdfe_main.f90:226-396) are recomputed from the tables and sigma, and the
// Dirichlet elimination of dcfast (fdfe_main.f90:399-546) is reproduced by
// skipping boundary columns (interior rows) and by identity boundary rows.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sfdx {

// ---------------------------------------------------------------- complex
template <class T> struct CT;
template <> struct CT<float> { typedef float2 type; };
template <> struct CT<double> { typedef double2 type; };
template <class T> using cplx = typename CT<T>::type;

template <class T> __host__ __device__ __forceinline__ cplx<T> mk(T r, T i) { cplx<T> z; z.x = r; z.y = i; return z; }
template <class T> __device__ __forceinline__ cplx<T> zero() { return mk<T>(T(0), T(0)); }
template <class T> __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <class T> __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
template <class T> __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class T> __device__ __forceinline__ cplx<T> rmul(T r, cplx<T> a) { return mk<T>(r * a.x, r * a.y); }
// conj(a) * b  (Fortran dot_product term)
template <class T> __device__ __forceinline__ cplx<T> cdot(cplx<T> a, cplx<T> b) {
    return mk<T>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <class T> __device__ __forceinline__ cplx<T> cdiv(cplx<T> a, cplx<T> b) {
    T d = T(1) / (b.x * b.x + b.y * b.y);
    return mk<T>((a.x * b.x + a.y * b.y) * d, (a.y * b.x - a.x * b.y) * d);
}
template <class T> __device__ __forceinline__ T cabs2(cplx<T> a) { return a.x * a.x + a.y * a.y; }
// multiply by -i*wm (the "- coef * s" of fd_assemb with coef = i*w*mu)
template <class T> __device__ __forceinline__ cplx<T> mul_mi(T wm, cplx<T> a) { return mk<T>(wm * a.y, -wm * a.x); }

template <class T> __device__ __forceinline__ cplx<T> ldc(const cplx<T>* p) { return __ldg(p); }

// ---------------------------------------------------------------- tables
// Per-axis tables, indexed 0-based.  Cell quantities by cell index
// [0, n), node quantities by node index [0, n] (valid for interior nodes
// 1..n-1):  lo = -2/(h(n-1)(h(n-1)+h(n))), hi = -2/(h(n)(h(n-1)+h(n))),
// rs = 1/(h(n-1)+h(n)), wlo = h(n-1)/(h(n-1)+h(n)), whi = h(n)/(..).
template <class T> struct AxisT {
    const T* rh;  // 1/h(cell)
    const T* lo;
    const T* hi;
    const T* rs;
    const T* wlo;
    const T* whi;
};
// number of T values one axis table block occupies for n cells
__host__ __device__ inline int axis_stride(int n) { return n + 2; }

template <class T> struct Lev {
    int nx, ny, nz;
    int64_t xnl, ynl, nl, ncell;
    AxisT<T> ax, ay, az;
    const T* sig;  // [6][ncell]
    int aniso;     // 1 if any off-diagonal conductivity is non-zero
    const T* rc;   // per-row coefficients [nl][12] (sfdx_stencil.cuh row_k_e), or null
};

// ---------------------------------------------------------------- edges
enum { OX = 0, OY = 1, OZ = 2 };

template <class T> __device__ __forceinline__ int64_t eidx(const Lev<T>& L, int o, int i, int j, int k) {
    if (o == OX) return ((int64_t)k * (L.ny + 1) + j) * L.nx + i;
    if (o == OY) return L.xnl + ((int64_t)k * L.ny + j) * (L.nx + 1) + i;
    return L.xnl + L.ynl + ((int64_t)k * (L.ny + 1) + j) * (L.nx + 1) + i;
}
template <class T> __device__ __forceinline__ void edecode(const Lev<T>& L, int64_t e, int& o, int& i, int& j, int& k) {
    if (e < L.xnl) {
        o = OX;
        i = (int)(e % L.nx);
        int64_t r = e / L.nx;
        j = (int)(r % (L.ny + 1));
        k = (int)(r / (L.ny + 1));
    } else if (e < L.xnl + L.ynl) {
        int64_t f = e - L.xnl;
        o = OY;
        i = (int)(f % (L.nx + 1));
        int64_t r = f / (L.nx + 1);
        j = (int)(r % L.ny);
        k = (int)(r / L.ny);
    } else {
        int64_t f = e - L.xnl - L.ynl;
        o = OZ;
        i = (int)(f % (L.nx + 1));
        int64_t r = f / (L.nx + 1);
        j = (int)(r % (L.ny + 1));
        k = (int)(r / (L.ny + 1));
    }
}
// boundary edges (dcfast fdfe_main.f90:439-468)
template <class T> __device__ __forceinline__ bool is_bnd(const Lev<T>& L, int o, int i, int j, int k) {
    if (o == OX) return j == 0 || j == L.ny || k == 0 || k == L.nz;
    if (o == OY) return i == 0 || i == L.nx || k == 0 || k == L.nz;
    return i == 0 || i == L.nx || j == 0 || j == L.ny;
}
template <class T> __device__ __forceinline__ int64_t cidx(const Lev<T>& L, int i, int j, int k) {
    return ((int64_t)k * L.ny + j) * L.nx + i;
}
template <class T> __device__ __forceinline__ T sg(const Lev<T>& L, int comp, int64_t c) {
    return __ldg(L.sig + (int64_t)comp * L.ncell + c);
}

// ---------------------------------------------------------------- stencil
// Values of the neighbouring edges are obtained through a fetch functor
// F(o, i, j, k) that returns the (already masked) neighbour value.  The
// stencil itself only knows the mesh.
//
// Row of orientation O at interior edge (i,j,k).  Groups:
//   SAME  : the four same-orientation neighbours (curl-curl only, real)
//   CA,CB : the two cross-orientation groups (Ex row: Ey, Ez; Ey row: Ex, Ez;
//           Ez row: Ex, Ey), curl + off-diagonal sigma terms.
// diag() returns the complex diagonal of the row.
template <class T> struct RowCoef {
    T dre;   // real part of the diagonal: -(sum of curl neighbours)
    T sbar;  // area-weighted diagonal conductivity of the row
};

template <class T, int O> __device__ __forceinline__ RowCoef<T> row_diag(const Lev<T>& L, int i, int j, int k) {
    RowCoef<T> rc;
    if (O == OX) {
        T loy = __ldg(L.ay.lo + j), hiy = __ldg(L.ay.hi + j), loz = __ldg(L.az.lo + k), hiz = __ldg(L.az.hi + k);
        rc.dre = -(((loz + loy) + hiy) + hiz);
        T wly = __ldg(L.ay.wlo + j), why = __ldg(L.ay.whi + j), wlz = __ldg(L.az.wlo + k), whz = __ldg(L.az.whi + k);
        rc.sbar = sg(L, 0, cidx(L, i, j - 1, k - 1)) * wly * wlz + sg(L, 0, cidx(L, i, j, k - 1)) * why * wlz +
                  sg(L, 0, cidx(L, i, j - 1, k)) * wly * whz + sg(L, 0, cidx(L, i, j, k)) * why * whz;
    } else if (O == OY) {
        T lox = __ldg(L.ax.lo + i), hix = __ldg(L.ax.hi + i), loz = __ldg(L.az.lo + k), hiz = __ldg(L.az.hi + k);
        rc.dre = -(((loz + lox) + hix) + hiz);
        T wlx = __ldg(L.ax.wlo + i), whx = __ldg(L.ax.whi + i), wlz = __ldg(L.az.wlo + k), whz = __ldg(L.az.whi + k);
        rc.sbar = sg(L, 1, cidx(L, i - 1, j, k - 1)) * wlx * wlz + sg(L, 1, cidx(L, i, j, k - 1)) * whx * wlz +
                  sg(L, 1, cidx(L, i - 1, j, k)) * wlx * whz + sg(L, 1, cidx(L, i, j, k)) * whx * whz;
    } else {
        T lox = __ldg(L.ax.lo + i), hix = __ldg(L.ax.hi + i), loy = __ldg(L.ay.lo + j), hiy = __ldg(L.ay.hi + j);
        rc.dre = -(((loy + lox) + hix) + hiy);
        T wlx = __ldg(L.ax.wlo + i), whx = __ldg(L.ax.whi + i), wly = __ldg(L.ay.wlo + j), why = __ldg(L.ay.whi + j);
        rc.sbar = sg(L, 2, cidx(L, i - 1, j - 1, k)) * wly * wlx + sg(L, 2, cidx(L, i - 1, j, k)) * why * wlx +
                  sg(L, 2, cidx(L, i, j - 1, k)) * wly * whx + sg(L, 2, cidx(L, i, j, k)) * why * whx;
    }
    return rc;
}

// Cross term  g*(v1 - v2 - v3 + v4) - i*wm*(s1*(u1a+u1b) + s2*(u2a+u2b))
template <class T>
__device__ __forceinline__ cplx<T> cross4(T g, T wm, T s1, T s2, cplx<T> v1, cplx<T> v2, cplx<T> v3, cplx<T> v4,
                                          cplx<T> m1, cplx<T> m2) {
    cplx<T> cu = (v1 - v2) + (v4 - v3);
    cplx<T> mass = mk<T>(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);
    return rmul<T>(g, cu) + mul_mi<T>(wm, mass);
}

// Off-diagonal part of row (O,i,j,k) restricted to the selected groups.
template <class T, int O, bool SAME, bool CA, bool CB, class F>
__device__ __forceinline__ cplx<T> row_offdiag(const Lev<T>& L, int i, int j, int k, T wm, F fetch) {
    cplx<T> acc = zero<T>();
    const bool an = L.aniso != 0;
    if (O == OX) {
        if (SAME) {
            acc = acc + rmul<T>(__ldg(L.az.lo + k), fetch(OX, i, j, k - 1));
            acc = acc + rmul<T>(__ldg(L.ay.lo + j), fetch(OX, i, j - 1, k));
            acc = acc + rmul<T>(__ldg(L.ay.hi + j), fetch(OX, i, j + 1, k));
            acc = acc + rmul<T>(__ldg(L.az.hi + k), fetch(OX, i, j, k + 1));
        }
        if (CA || CB) {
            T rhx = T(2) * __ldg(L.ax.rh + i);
            T wly = __ldg(L.ay.wlo + j), why = __ldg(L.ay.whi + j), wlz = __ldg(L.az.wlo + k), whz = __ldg(L.az.whi + k);
            int64_t c00 = cidx(L, i, j - 1, k - 1), c10 = cidx(L, i, j, k - 1), c01 = cidx(L, i, j - 1, k), c11 = cidx(L, i, j, k);
            if (CA) {  // Ey
                cplx<T> y1 = fetch(OY, i, j - 1, k), y2 = fetch(OY, i + 1, j - 1, k), y3 = fetch(OY, i, j, k),
                        y4 = fetch(OY, i + 1, j, k);
                T s1 = T(0), s2 = T(0);
                if (an) {
                    s1 = T(0.5) * wly * (sg(L, 3, c00) * wlz + sg(L, 3, c01) * whz);
                    s2 = T(0.5) * why * (sg(L, 3, c10) * wlz + sg(L, 3, c11) * whz);
                }
                acc = acc + cross4<T>(rhx * __ldg(L.ay.rs + j), wm, s1, s2, y1, y2, y3, y4, y1 + y2, y3 + y4);
            }
            if (CB) {  // Ez
                cplx<T> z1 = fetch(OZ, i, j, k - 1), z2 = fetch(OZ, i + 1, j, k - 1), z3 = fetch(OZ, i, j, k),
                        z4 = fetch(OZ, i + 1, j, k);
                T s3 = T(0), s4 = T(0);
                if (an) {
                    s3 = T(0.5) * wlz * (sg(L, 4, c00) * wly + sg(L, 4, c10) * why);
                    s4 = T(0.5) * whz * (sg(L, 4, c01) * wly + sg(L, 4, c11) * why);
                }
                acc = acc + cross4<T>(rhx * __ldg(L.az.rs + k), wm, s3, s4, z1, z2, z3, z4, z1 + z2, z3 + z4);
            }
        }
    } else if (O == OY) {
        if (SAME) {
            acc = acc + rmul<T>(__ldg(L.az.lo + k), fetch(OY, i, j, k - 1));
            acc = acc + rmul<T>(__ldg(L.ax.lo + i), fetch(OY, i - 1, j, k));
            acc = acc + rmul<T>(__ldg(L.ax.hi + i), fetch(OY, i + 1, j, k));
            acc = acc + rmul<T>(__ldg(L.az.hi + k), fetch(OY, i, j, k + 1));
        }
        if (CA || CB) {
            T rhy = T(2) * __ldg(L.ay.rh + j);
            T wlx = __ldg(L.ax.wlo + i), whx = __ldg(L.ax.whi + i), wlz = __ldg(L.az.wlo + k), whz = __ldg(L.az.whi + k);
            int64_t c00 = cidx(L, i - 1, j, k - 1), c10 = cidx(L, i, j, k - 1), c01 = cidx(L, i - 1, j, k), c11 = cidx(L, i, j, k);
            if (CA) {  // Ex
                cplx<T> x1 = fetch(OX, i - 1, j, k), x2 = fetch(OX, i, j, k), x3 = fetch(OX, i - 1, j + 1, k),
                        x4 = fetch(OX, i, j + 1, k);
                T s1 = T(0), s2 = T(0);
                if (an) {
                    s1 = T(0.5) * wlx * (sg(L, 3, c00) * wlz + sg(L, 3, c01) * whz);
                    s2 = T(0.5) * whx * (sg(L, 3, c10) * wlz + sg(L, 3, c11) * whz);
                }
                acc = acc + cross4<T>(rhy * __ldg(L.ax.rs + i), wm, s1, s2, x1, x2, x3, x4, x1 + x3, x2 + x4);
            }
            if (CB) {  // Ez
                cplx<T> z1 = fetch(OZ, i, j, k - 1), z2 = fetch(OZ, i, j + 1, k - 1), z3 = fetch(OZ, i, j, k),
                        z4 = fetch(OZ, i, j + 1, k);
                T s3 = T(0), s4 = T(0);
                if (an) {
                    s3 = T(0.5) * wlz * (sg(L, 5, c00) * wlx + sg(L, 5, c10) * whx);
                    s4 = T(0.5) * whz * (sg(L, 5, c01) * wlx + sg(L, 5, c11) * whx);
                }
                acc = acc + cross4<T>(rhy * __ldg(L.az.rs + k), wm, s3, s4, z1, z2, z3, z4, z1 + z2, z3 + z4);
            }
        }
    } else {
        if (SAME) {
            acc = acc + rmul<T>(__ldg(L.ay.lo + j), fetch(OZ, i, j - 1, k));
            acc = acc + rmul<T>(__ldg(L.ax.lo + i), fetch(OZ, i - 1, j, k));
            acc = acc + rmul<T>(__ldg(L.ax.hi + i), fetch(OZ, i + 1, j, k));
            acc = acc + rmul<T>(__ldg(L.ay.hi + j), fetch(OZ, i, j + 1, k));
        }
        if (CA || CB) {
            T rhz = T(2) * __ldg(L.az.rh + k);
            T wlx = __ldg(L.ax.wlo + i), whx = __ldg(L.ax.whi + i), wly = __ldg(L.ay.wlo + j), why = __ldg(L.ay.whi + j);
            int64_t c00 = cidx(L, i - 1, j - 1, k), c01 = cidx(L, i - 1, j, k), c10 = cidx(L, i, j - 1, k), c11 = cidx(L, i, j, k);
            if (CA) {  // Ex
                cplx<T> x1 = fetch(OX, i - 1, j, k), x2 = fetch(OX, i, j, k), x3 = fetch(OX, i - 1, j, k + 1),
                        x4 = fetch(OX, i, j, k + 1);
                T s1 = T(0), s2 = T(0);
                if (an) {
                    s1 = T(0.5) * wlx * (sg(L, 4, c00) * wly + sg(L, 4, c01) * why);
                    s2 = T(0.5) * whx * (sg(L, 4, c10) * wly + sg(L, 4, c11) * why);
                }
                acc = acc + cross4<T>(rhz * __ldg(L.ax.rs + i), wm, s1, s2, x1, x2, x3, x4, x1 + x3, x2 + x4);
            }
            if (CB) {  // Ey
                cplx<T> y1 = fetch(OY, i, j - 1, k), y2 = fetch(OY, i, j, k), y3 = fetch(OY, i, j - 1, k + 1),
                        y4 = fetch(OY, i, j, k + 1);
                T s3 = T(0), s4 = T(0);
                if (an) {
                    s3 = T(0.5) * wly * (sg(L, 5, c00) * wlx + sg(L, 5, c10) * whx);
                    s4 = T(0.5) * why * (sg(L, 5, c01) * wlx + sg(L, 5, c11) * whx);
                }
                acc = acc + cross4<T>(rhz * __ldg(L.ay.rs + j), wm, s3, s4, y1, y2, y3, y4, y1 + y3, y2 + y4);
            }
        }
    }
    return acc;
}

// Fetch functors ------------------------------------------------------------
// Solution vector with boundary columns removed (interior rows of dcfast).
template <class T> struct FetchInterior {
    const Lev<T>* L;
    const cplx<T>* x;
    int ns, s;
    __device__ __forceinline__ cplx<T> operator()(int o, int i, int j, int k) const {
        if (is_bnd(*L, o, i, j, k)) return zero<T>();
        return ldc<T>(x + eidx(*L, o, i, j, k) * ns + s);
    }
};
// Same, but reading through the plain (coherent) path: used by sweeps that
// read values written by earlier launches of the same vector.
template <class T> struct FetchInteriorRW {
    const Lev<T>* L;
    const cplx<T>* x;
    int ns, s;
    __device__ __forceinline__ cplx<T> operator()(int o, int i, int j, int k) const {
        if (is_bnd(*L, o, i, j, k)) return zero<T>();
        return x[eidx(*L, o, i, j, k) * ns + s];
    }
};

// Dirichlet values of dcfast (fdfe_main.f90:470-494) for one polarisation.
// edc: e_dc(2nz+2) from mt1d_anl, 0-based.
__device__ __forceinline__ double2 dirichlet_value(int nx, int ny, int nz, int pol, const double2* edc, int o, int i,
                                                   int j, int k) {
    if (pol == 0) {
        if (o != OX) return make_double2(0.0, 0.0);
        if (k == 0) return make_double2(1.0, 0.0);
        if (k == nz) return edc[nz];
        if (j == 0 || j == ny) return edc[k];
        return make_double2(0.0, 0.0);
    } else {
        if (o != OY) return make_double2(0.0, 0.0);
        if (k == 0) return make_double2(1.0, 0.0);
        if (k == nz) return edc[2 * nz + 1];
        if (i == 0 || i == nx) return edc[nz + 1 + k];
        return make_double2(0.0, 0.0);
    }
}
struct FetchDirichlet {
    const Lev<double>* L;
    int pol;
    const double2* edc;
    __device__ __forceinline__ double2 operator()(int o, int i, int j, int k) const {
        if (!is_bnd(*L, o, i, j, k)) return make_double2(0.0, 0.0);
        return dirichlet_value(L->nx, L->ny, L->nz, pol, edc, o, i, j, k);
    }
};

}  // namespace sfdx
