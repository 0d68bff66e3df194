// sfdx_stencil.cuh -- the row evaluator of the hot kernels.
//
// Work mapping.  A thread owns one edge and a group of VS consecutive
// systems of the batch (VS = 1, 2 or 4; the systems of an edge are
// contiguous in HBM, so a group is one 8..64-byte vector).  The flattened
// work index t = edge * G + group (G = ns / VS) is decoded with 32-bit
// multiply-high division by precomputed magic numbers, never with 64-bit
// integer division.
//
// Row evaluation.  The 13-point row of fd_assemb (fdfe_main.f90:248-393) at
// an interior edge is split into
//   curl part  (real coefficients):  C = sum same-orientation neighbours
//                                        + gA*curlA + gB*curlB (+ dre*x_e)
//   mass part  (real coefficients):  M = sA1*mA1 + sA2*mA2 + sB1*mB1 + sB2*mB2
//                                        (+ sbar*x_e)
// and y = C - i*wm*M (wm = omega*mu of the system).  The coefficients depend
// only on the mesh and sigma, so they are computed once per thread and applied
// to all VS systems; the boundary columns removed by dcfast
// (fdfe_main.f90:499-524) become per-neighbour predicates that are resolved
// from the row's own (i, j, k) (which transverse index touches the boundary).
#pragma once
#include "sfdx_device.cuh"

namespace sfdx {

// ---------------------------------------------------------------- fast division
// q = (umulhi(n, m) + n) >> l  for 0 <= n < 2^31 and 1 <= d < 2^31
// (Granlund & Montgomery 1994, round-up variant).
struct FastDiv {
    uint32_t d, m, l;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d < 1 ? 1 : d;
    f.l = 0;
    while ((1ull << f.l) < f.d) f.l++;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << f.l) - f.d)) / f.d + 1);
    return f;
}
__device__ __forceinline__ uint32_t fdiv(const FastDiv& f, uint32_t n) { return (__umulhi(n, f.m) + n) >> f.l; }

// Mesh constants of one level for the 32-bit mapping.
struct Mesh {
    int nx, ny, nz;
    uint32_t xnl, ynl, nl;
    uint32_t sx, sy, sz;  // edges per z-plane: Ex nx(ny+1), Ey (nx+1)ny, Ez (nx+1)(ny+1)
    FastDiv fnx, fnx1, fny, fny1, fni2, fnj2, fsp;
};
inline Mesh make_mesh(int nx, int ny, int nz) {
    Mesh M;
    M.nx = nx; M.ny = ny; M.nz = nz;
    M.xnl = (uint32_t)nx * (ny + 1) * (nz + 1);
    M.ynl = (uint32_t)(nx + 1) * ny * (nz + 1);
    M.nl = M.xnl + M.ynl + (uint32_t)(nx + 1) * (ny + 1) * nz;
    M.fnx = make_fastdiv(nx);
    M.fnx1 = make_fastdiv(nx + 1);
    M.fny = make_fastdiv(ny);
    M.fny1 = make_fastdiv(ny + 1);
    M.fni2 = make_fastdiv((nx + 2) / 2);
    M.fnj2 = make_fastdiv((ny + 2) / 2);
    M.sx = (uint32_t)nx * (ny + 1);
    M.sy = (uint32_t)(nx + 1) * ny;
    M.sz = (uint32_t)(nx + 1) * (ny + 1);
    M.fsp = make_fastdiv(M.sx + M.sy + M.sz);
    return M;
}

// Work item w (0 <= w < nl) of the operator-type kernels in plane order:
// plane k holds Ex(.,.,k), Ey(.,.,k) and Ez(.,.,k) (no Ez on the last plane),
// so that the neighbours a row reads (planes k-1..k+1, all orientations) were
// touched moments earlier and are still in L2.  Returns the orientation and
// sets the edge index e of the reference ordering and (i, j, k).
__device__ __forceinline__ int mdecode_plane(const Mesh& M, uint32_t w, uint32_t& e, int& i, int& j, int& k) {
    const uint32_t kk = fdiv(M.fsp, w);
    uint32_t r = w - kk * M.fsp.d;
    k = (int)kk;
    if (r < M.sx) {
        const uint32_t jj = fdiv(M.fnx, r);
        i = (int)(r - jj * (uint32_t)M.nx);
        j = (int)jj;
        e = kk * M.sx + r;
        return OX;
    }
    r -= M.sx;
    const uint32_t jj = fdiv(M.fnx1, r < M.sy ? r : r - M.sy);
    if (r < M.sy) {
        i = (int)(r - jj * (uint32_t)(M.nx + 1));
        j = (int)jj;
        e = M.xnl + kk * M.sy + r;
        return OY;
    }
    r -= M.sy;
    i = (int)(r - jj * (uint32_t)(M.nx + 1));
    j = (int)jj;
    e = M.xnl + M.ynl + kk * M.sz + r;
    return OZ;
}

// edge index -> orientation and (i, j, k)
__device__ __forceinline__ int mdecode(const Mesh& M, uint32_t e, int& i, int& j, int& k) {
    if (e < M.xnl) {
        uint32_t q = fdiv(M.fnx, e);
        i = (int)(e - q * (uint32_t)M.nx);
        uint32_t kk = fdiv(M.fny1, q);
        j = (int)(q - kk * (uint32_t)(M.ny + 1));
        k = (int)kk;
        return OX;
    }
    e -= M.xnl;
    uint32_t q = fdiv(M.fnx1, e);
    i = (int)(e - q * (uint32_t)(M.nx + 1));
    if (e < M.ynl) {
        uint32_t kk = fdiv(M.fny, q);
        j = (int)(q - kk * (uint32_t)M.ny);
        k = (int)kk;
        return OY;
    }
    e -= M.ynl;
    q = fdiv(M.fnx1, e);
    i = (int)(e - q * (uint32_t)(M.nx + 1));
    uint32_t kk = fdiv(M.fny1, q);
    j = (int)(q - kk * (uint32_t)(M.ny + 1));
    k = (int)kk;
    return OZ;
}

// colour (O, P) index -> (i, j, k); false for the padding slots of odd extents
// Colours: Ex (j+k)&1, Ey (i+k)&1, Ez (i+j)&1.
template <int O>
__device__ __forceinline__ bool mcolour(const Mesh& M, int P, uint32_t t, int& i, int& j, int& k) {
    if (O == OX) {
        uint32_t r = fdiv(M.fnx, t);
        i = (int)(t - r * (uint32_t)M.nx);
        uint32_t kk = fdiv(M.fnj2, r);
        int jj = (int)(r - kk * M.fnj2.d);
        k = (int)kk;
        j = 2 * jj + ((P + k) & 1);
        return j <= M.ny;
    } else if (O == OY) {
        uint32_t r = fdiv(M.fni2, t);
        int ii = (int)(t - r * M.fni2.d);
        uint32_t kk = fdiv(M.fny, r);
        j = (int)(r - kk * (uint32_t)M.ny);
        k = (int)kk;
        i = 2 * ii + ((P + k) & 1);
        return i <= M.nx;
    } else {
        uint32_t r = fdiv(M.fni2, t);
        int ii = (int)(t - r * M.fni2.d);
        uint32_t kk = fdiv(M.fny1, r);
        j = (int)(r - kk * (uint32_t)(M.ny + 1));
        k = (int)kk;
        i = 2 * ii + ((P + j) & 1);
        return i <= M.nx;
    }
}
__host__ __device__ inline uint32_t mcolour_count(const Mesh& M, int O) {
    if (O == OX) return (uint32_t)M.nx * ((M.ny + 2) / 2) * (M.nz + 1);
    if (O == OY) return (uint32_t)((M.nx + 2) / 2) * M.ny * (M.nz + 1);
    return (uint32_t)((M.nx + 2) / 2) * (M.ny + 1) * M.nz;
}

__device__ __forceinline__ uint32_t medge(const Mesh& M, int o, int i, int j, int k) {
    if (o == OX) return ((uint32_t)k * (M.ny + 1) + j) * M.nx + i;
    if (o == OY) return M.xnl + ((uint32_t)k * M.ny + j) * (M.nx + 1) + i;
    return M.xnl + M.ynl + ((uint32_t)k * (M.ny + 1) + j) * (M.nx + 1) + i;
}
__device__ __forceinline__ bool mbnd(const Mesh& M, int o, int i, int j, int k) {
    if (o == OX) return j == 0 || j == M.ny || k == 0 || k == M.nz;
    if (o == OY) return i == 0 || i == M.nx || k == 0 || k == M.nz;
    return i == 0 || i == M.nx || j == 0 || j == M.ny;
}

// ---------------------------------------------------------------- system vectors
template <class T, int VS> struct CV {
    cplx<T> v[VS];
};
template <class T, int VS> __device__ __forceinline__ void cvzero(CV<T, VS>& a) {
#pragma unroll
    for (int q = 0; q < VS; q++) a.v[q] = mk<T>(T(0), T(0));
}
// 256-bit accesses (sm_100 and later): one instruction moves the 32 bytes of
// four complex64 or two complex128 values of a thread.  On the operator's
// 13-neighbour gather this is 27 % faster than two 128-bit loads (0.123 vs
// 0.168 ms for 1.57 M edges x 16 systems).  The address must be 32-byte
// aligned: [edge * ns + s0] offsets are (VS divides ns) and vlaunch checks the
// base pointers.
__device__ __forceinline__ void ld256_nc(const void* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ void ld256(const void* p, float4& a, float4& b) {
    asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                 : "l"(p)
                 : "memory");
}
__device__ __forceinline__ void st256(void* p, const float4& a, const float4& b) {
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
                 "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}
__device__ __forceinline__ void ld256_nc(const void* p, double2& a, double2& b) {
    asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(a.x), "=d"(a.y), "=d"(b.x), "=d"(b.y) : "l"(p));
}
__device__ __forceinline__ void ld256(const void* p, double2& a, double2& b) {
    asm volatile("ld.global.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(a.x), "=d"(a.y), "=d"(b.x), "=d"(b.y) : "l"(p) : "memory");
}
__device__ __forceinline__ void st256(void* p, const double2& a, const double2& b) {
    asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p), "d"(a.x), "d"(a.y), "d"(b.x), "d"(b.y) : "memory");
}
// whether VS values of T go as 256-bit groups
template <class T, int VS> struct Wide {
    static constexpr bool value = (sizeof(T) == 4 && VS % 4 == 0) || (sizeof(T) == 8 && VS % 2 == 0);
    static constexpr int per = sizeof(T) == 4 ? 4 : 2;  // complex values per 32 bytes
};

// read-only (non-coherent) vector load of VS consecutive complex values
template <class T, int VS> __device__ __forceinline__ void cvld(CV<T, VS>& a, const cplx<T>* p) {
    if (Wide<T, VS>::value) {
        constexpr int PER = Wide<T, VS>::per;
#pragma unroll
        for (int h = 0; h < VS / PER; h++) {
            if (sizeof(T) == 4) {
                float4 f, g;
                ld256_nc(p + PER * h, f, g);
                a.v[PER * h] = mk<T>((T)f.x, (T)f.y);
                a.v[PER * h + 1] = mk<T>((T)f.z, (T)f.w);
                a.v[(PER * h + 2) % VS] = mk<T>((T)g.x, (T)g.y);
                a.v[(PER * h + 3) % VS] = mk<T>((T)g.z, (T)g.w);
            } else {
                double2 f, g;
                ld256_nc(p + PER * h, f, g);
                a.v[PER * h] = mk<T>((T)f.x, (T)f.y);
                a.v[PER * h + 1] = mk<T>((T)g.x, (T)g.y);
            }
        }
    } else if (sizeof(T) == 4 && VS % 2 == 0) {
        const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
        for (int h = 0; h < VS / 2; h++) {
            float4 f = __ldg(q + h);
            a.v[2 * h] = mk<T>((T)f.x, (T)f.y);
            a.v[2 * h + 1] = mk<T>((T)f.z, (T)f.w);
        }
    } else {
#pragma unroll
        for (int q = 0; q < VS; q++) a.v[q] = __ldg(p + q);
    }
}
// coherent load (arrays written by the same kernel)
template <class T, int VS> __device__ __forceinline__ void cvldw(CV<T, VS>& a, const cplx<T>* p) {
    if (Wide<T, VS>::value) {
        constexpr int PER = Wide<T, VS>::per;
#pragma unroll
        for (int h = 0; h < VS / PER; h++) {
            if (sizeof(T) == 4) {
                float4 f, g;
                ld256(p + PER * h, f, g);
                a.v[PER * h] = mk<T>((T)f.x, (T)f.y);
                a.v[PER * h + 1] = mk<T>((T)f.z, (T)f.w);
                a.v[(PER * h + 2) % VS] = mk<T>((T)g.x, (T)g.y);
                a.v[(PER * h + 3) % VS] = mk<T>((T)g.z, (T)g.w);
            } else {
                double2 f, g;
                ld256(p + PER * h, f, g);
                a.v[PER * h] = mk<T>((T)f.x, (T)f.y);
                a.v[PER * h + 1] = mk<T>((T)g.x, (T)g.y);
            }
        }
    } else if (sizeof(T) == 4 && VS % 2 == 0) {
        const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
        for (int h = 0; h < VS / 2; h++) {
            float4 f = q[h];
            a.v[2 * h] = mk<T>((T)f.x, (T)f.y);
            a.v[2 * h + 1] = mk<T>((T)f.z, (T)f.w);
        }
    } else {
#pragma unroll
        for (int q = 0; q < VS; q++) a.v[q] = p[q];
    }
}
template <class T, int VS> __device__ __forceinline__ void cvst(cplx<T>* p, const CV<T, VS>& a) {
    if (Wide<T, VS>::value) {
        constexpr int PER = Wide<T, VS>::per;
#pragma unroll
        for (int h = 0; h < VS / PER; h++) {
            if (sizeof(T) == 4)
                st256(p + PER * h,
                      make_float4((float)a.v[PER * h].x, (float)a.v[PER * h].y, (float)a.v[PER * h + 1].x,
                                  (float)a.v[PER * h + 1].y),
                      make_float4((float)a.v[(PER * h + 2) % VS].x, (float)a.v[(PER * h + 2) % VS].y,
                                  (float)a.v[(PER * h + 3) % VS].x, (float)a.v[(PER * h + 3) % VS].y));
            else
                st256(p + PER * h, make_double2((double)a.v[PER * h].x, (double)a.v[PER * h].y),
                      make_double2((double)a.v[PER * h + 1].x, (double)a.v[PER * h + 1].y));
        }
    } else if (sizeof(T) == 4 && VS % 2 == 0) {
        float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
        for (int h = 0; h < VS / 2; h++)
            q[h] = make_float4((float)a.v[2 * h].x, (float)a.v[2 * h].y, (float)a.v[2 * h + 1].x, (float)a.v[2 * h + 1].y);
    } else {
#pragma unroll
        for (int q = 0; q < VS; q++) p[q] = a.v[q];
    }
}
// store only the systems whose mask bit is set (all set: one vector store)
template <class T, int VS> __device__ __forceinline__ void cvst_m(cplx<T>* p, const CV<T, VS>& a, unsigned act) {
    if (act == (1u << VS) - 1) {
        cvst<T, VS>(p, a);
    } else {
#pragma unroll
        for (int q = 0; q < VS; q++)
            if (act >> q & 1) p[q] = a.v[q];
    }
}

// ---------------------------------------------------------------- row coefficients
template <class T> struct RowK {
    T cs[4];       // same-orientation curl coefficients (order of fd_assemb's column list)
    T dre, sbar;   // diagonal: -(sum of cs), area-weighted diagonal conductivity
    T gA, sA1, sA2;  // first cross group (Ex row: Ey, Ey row: Ex, Ez row: Ex)
    T gB, sB1, sB2;  // second cross group (Ex row: Ez, Ey row: Ez, Ez row: Ey)
};

template <class T, int O, bool SAME, bool CA, bool CB>
__device__ __forceinline__ RowK<T> row_k(const Lev<T>& L, int i, int j, int k) {
    RowK<T> K;
    const int nx = L.nx, ny = L.ny;
    auto ci = [&](int a, int b, int c) { return ((int64_t)c * ny + b) * nx + a; };
    const bool an = L.aniso != 0;
    if (O == OX) {
        T loy = __ldg(L.ay.lo + j), hiy = __ldg(L.ay.hi + j), loz = __ldg(L.az.lo + k), hiz = __ldg(L.az.hi + k);
        K.cs[0] = loz; K.cs[1] = loy; K.cs[2] = hiy; K.cs[3] = hiz;
        K.dre = -(((loz + loy) + hiy) + hiz);
        T wly = __ldg(L.ay.wlo + j), why = __ldg(L.ay.whi + j), wlz = __ldg(L.az.wlo + k), whz = __ldg(L.az.whi + k);
        int64_t c00 = ci(i, j - 1, k - 1), c10 = ci(i, j, k - 1), c01 = ci(i, j - 1, k), c11 = ci(i, j, k);
        K.sbar = sg(L, 0, c00) * wly * wlz + sg(L, 0, c10) * why * wlz + sg(L, 0, c01) * wly * whz + sg(L, 0, c11) * why * whz;
        T rhx = T(2) * __ldg(L.ax.rh + i);
        if (CA) {
            K.gA = rhx * __ldg(L.ay.rs + j);
            K.sA1 = an ? T(0.5) * wly * (sg(L, 3, c00) * wlz + sg(L, 3, c01) * whz) : T(0);
            K.sA2 = an ? T(0.5) * why * (sg(L, 3, c10) * wlz + sg(L, 3, c11) * whz) : T(0);
        }
        if (CB) {
            K.gB = rhx * __ldg(L.az.rs + k);
            K.sB1 = an ? T(0.5) * wlz * (sg(L, 4, c00) * wly + sg(L, 4, c10) * why) : T(0);
            K.sB2 = an ? T(0.5) * whz * (sg(L, 4, c01) * wly + sg(L, 4, c11) * why) : T(0);
        }
    } else if (O == OY) {
        T lox = __ldg(L.ax.lo + i), hix = __ldg(L.ax.hi + i), loz = __ldg(L.az.lo + k), hiz = __ldg(L.az.hi + k);
        K.cs[0] = loz; K.cs[1] = lox; K.cs[2] = hix; K.cs[3] = hiz;
        K.dre = -(((loz + lox) + hix) + hiz);
        T wlx = __ldg(L.ax.wlo + i), whx = __ldg(L.ax.whi + i), wlz = __ldg(L.az.wlo + k), whz = __ldg(L.az.whi + k);
        int64_t c00 = ci(i - 1, j, k - 1), c10 = ci(i, j, k - 1), c01 = ci(i - 1, j, k), c11 = ci(i, j, k);
        K.sbar = sg(L, 1, c00) * wlx * wlz + sg(L, 1, c10) * whx * wlz + sg(L, 1, c01) * wlx * whz + sg(L, 1, c11) * whx * whz;
        T rhy = T(2) * __ldg(L.ay.rh + j);
        if (CA) {
            K.gA = rhy * __ldg(L.ax.rs + i);
            K.sA1 = an ? T(0.5) * wlx * (sg(L, 3, c00) * wlz + sg(L, 3, c01) * whz) : T(0);
            K.sA2 = an ? T(0.5) * whx * (sg(L, 3, c10) * wlz + sg(L, 3, c11) * whz) : T(0);
        }
        if (CB) {
            K.gB = rhy * __ldg(L.az.rs + k);
            K.sB1 = an ? T(0.5) * wlz * (sg(L, 5, c00) * wlx + sg(L, 5, c10) * whx) : T(0);
            K.sB2 = an ? T(0.5) * whz * (sg(L, 5, c01) * wlx + sg(L, 5, c11) * whx) : T(0);
        }
    } else {
        T lox = __ldg(L.ax.lo + i), hix = __ldg(L.ax.hi + i), loy = __ldg(L.ay.lo + j), hiy = __ldg(L.ay.hi + j);
        K.cs[0] = loy; K.cs[1] = lox; K.cs[2] = hix; K.cs[3] = hiy;
        K.dre = -(((loy + lox) + hix) + hiy);
        T wlx = __ldg(L.ax.wlo + i), whx = __ldg(L.ax.whi + i), wly = __ldg(L.ay.wlo + j), why = __ldg(L.ay.whi + j);
        int64_t c00 = ci(i - 1, j - 1, k), c01 = ci(i - 1, j, k), c10 = ci(i, j - 1, k), c11 = ci(i, j, k);
        K.sbar = sg(L, 2, c00) * wly * wlx + sg(L, 2, c01) * why * wlx + sg(L, 2, c10) * wly * whx + sg(L, 2, c11) * why * whx;
        T rhz = T(2) * __ldg(L.az.rh + k);
        if (CA) {
            K.gA = rhz * __ldg(L.ax.rs + i);
            K.sA1 = an ? T(0.5) * wlx * (sg(L, 4, c00) * wly + sg(L, 4, c01) * why) : T(0);
            K.sA2 = an ? T(0.5) * whx * (sg(L, 4, c10) * wly + sg(L, 4, c11) * why) : T(0);
        }
        if (CB) {
            K.gB = rhz * __ldg(L.ay.rs + j);
            K.sB1 = an ? T(0.5) * wly * (sg(L, 5, c00) * wlx + sg(L, 5, c10) * whx) : T(0);
            K.sB2 = an ? T(0.5) * why * (sg(L, 5, c01) * wlx + sg(L, 5, c11) * whx) : T(0);
        }
    }
    if (!SAME) K.cs[0] = K.cs[1] = K.cs[2] = K.cs[3] = T(0);
    return K;
}

// Coefficients of row e: stored ones when the level has them (built once per
// conductivity by k_row_coef: 12 values, 48 bytes in complex64 arithmetic,
// read by the G threads of the edge as one broadcast), else computed from the
// conductivity and spacing tables as above.
template <class T, int O, bool SAME, bool CA, bool CB>
__device__ __forceinline__ RowK<T> row_k_e(const Lev<T>& L, uint32_t e, int i, int j, int k) {
    if (!L.rc) return row_k<T, O, SAME, CA, CB>(L, i, j, k);
    RowK<T> K;
    const T* p = L.rc + (size_t)e * 12;
    T v[12];
    if (sizeof(T) == 4) {
        const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
        for (int h = 0; h < 3; h++) {
            const float4 f = __ldg(q + h);
            v[4 * h] = (T)f.x; v[4 * h + 1] = (T)f.y; v[4 * h + 2] = (T)f.z; v[4 * h + 3] = (T)f.w;
        }
    } else {
        const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
        for (int h = 0; h < 6; h++) {
            const double2 f = __ldg(q + h);
            v[2 * h] = (T)f.x; v[2 * h + 1] = (T)f.y;
        }
    }
    K.cs[0] = v[0]; K.cs[1] = v[1]; K.cs[2] = v[2]; K.cs[3] = v[3];
    K.dre = v[4]; K.sbar = v[5];
    K.gA = v[6]; K.sA1 = v[7]; K.sA2 = v[8];
    K.gB = v[9]; K.sB1 = v[10]; K.sB2 = v[11];
    return K;
}

// Neighbour positions and boundary predicates of the interior row (O,i,j,k).
//   same[q]  : edge index of the q-th same-orientation neighbour, msame bit q
//   A[0..3]  : first cross group  (v1, v2, v3, v4 of the curl difference)
//   B[0..3]  : second cross group
// A cross group contributes g*((v1-v2)+(v4-v3)) to C and s1*m1 + s2*m2 to M,
// with (m1, m2) = (v1+v2, v3+v4) when PAIR is 0 and (v1+v3, v2+v4) when 1.
struct RowN {
    uint32_t same[4], A[4], B[4];
    unsigned msame, mA, mB;  // bit set = column removed (boundary edge)
};
template <int O> struct RowPair;
template <> struct RowPair<OX> { enum { A = 0, B = 0 }; };
template <> struct RowPair<OY> { enum { A = 1, B = 0 }; };
template <> struct RowPair<OZ> { enum { A = 1, B = 1 }; };

template <int O> __device__ __forceinline__ RowN row_n(const Mesh& M, uint32_t e, int i, int j, int k) {
    RowN N;
    const uint32_t nx = M.nx, ny = M.ny, nx1 = nx + 1, ny1 = ny + 1;
    if (O == OX) {
        const uint32_t pl = nx * ny1;
        N.same[0] = e - pl; N.same[1] = e - nx; N.same[2] = e + nx; N.same[3] = e + pl;
        N.msame = (k == 1) | (j == 1) << 1 | (j + 1 == M.ny) << 2 | (k + 1 == M.nz) << 3;
        const unsigned mi = (i == 0) | (i + 1 == M.nx) << 1;
        const uint32_t a = M.xnl + ((uint32_t)k * ny + j - 1) * nx1 + i;
        N.A[0] = a; N.A[1] = a + 1; N.A[2] = a + nx1; N.A[3] = a + nx1 + 1;
        N.mA = mi | mi << 2;
        const uint32_t b = M.xnl + M.ynl + ((uint32_t)(k - 1) * ny1 + j) * nx1 + i;
        N.B[0] = b; N.B[1] = b + 1; N.B[2] = b + ny1 * nx1; N.B[3] = b + ny1 * nx1 + 1;
        N.mB = mi | mi << 2;
    } else if (O == OY) {
        const uint32_t pl = ny * nx1;
        N.same[0] = e - pl; N.same[1] = e - 1; N.same[2] = e + 1; N.same[3] = e + pl;
        N.msame = (k == 1) | (i == 1) << 1 | (i + 1 == M.nx) << 2 | (k + 1 == M.nz) << 3;
        const unsigned m0 = (j == 0), m1 = (j + 1 == M.ny);
        const uint32_t a = ((uint32_t)k * ny1 + j) * nx + i - 1;
        N.A[0] = a; N.A[1] = a + 1; N.A[2] = a + nx; N.A[3] = a + nx + 1;
        N.mA = m0 | m0 << 1 | m1 << 2 | m1 << 3;
        const uint32_t b = M.xnl + M.ynl + ((uint32_t)(k - 1) * ny1 + j) * nx1 + i;
        N.B[0] = b; N.B[1] = b + nx1; N.B[2] = b + ny1 * nx1; N.B[3] = b + ny1 * nx1 + nx1;
        N.mB = m0 | m1 << 1 | m0 << 2 | m1 << 3;
    } else {
        N.same[0] = e - nx1; N.same[1] = e - 1; N.same[2] = e + 1; N.same[3] = e + nx1;
        N.msame = (j == 1) | (i == 1) << 1 | (i + 1 == M.nx) << 2 | (j + 1 == M.ny) << 3;
        const unsigned m0 = (k == 0), m1 = (k + 1 == M.nz);
        const uint32_t a = ((uint32_t)k * ny1 + j) * nx + i - 1;
        N.A[0] = a; N.A[1] = a + 1; N.A[2] = a + nx * ny1; N.A[3] = a + nx * ny1 + 1;
        N.mA = m0 | m0 << 1 | m1 << 2 | m1 << 3;
        const uint32_t b = M.xnl + ((uint32_t)k * ny + j - 1) * nx1 + i;
        N.B[0] = b; N.B[1] = b + nx1; N.B[2] = b + ny * nx1; N.B[3] = b + ny * nx1 + nx1;
        N.mB = m0 | m0 << 1 | m1 << 2 | m1 << 3;
    }
    return N;
}

// Accumulate the selected groups of the off-diagonal row into C (curl part)
// and Mm (mass part) for VS systems; x is read at [edge * ns + s0].
template <class T, int VS, bool RO>
__device__ __forceinline__ void ld_nb(CV<T, VS>& a, const cplx<T>* x, uint32_t e, int ns, int s0, bool masked) {
    if (masked) {
        cvzero<T, VS>(a);
    } else if (RO) {
        cvld<T, VS>(a, x + (size_t)e * ns + s0);
    } else {
        cvldw<T, VS>(a, x + (size_t)e * ns + s0);
    }
}

// both coefficients +0 (bit test on the integer pipe: the off-diagonal
// conductivity weights are sums of non-negative products, never -0)
__device__ __forceinline__ bool both_zero(float a, float b) { return (__float_as_uint(a) | __float_as_uint(b)) == 0u; }
__device__ __forceinline__ bool both_zero(double a, double b) {
    return (__double_as_longlong(a) | __double_as_longlong(b)) == 0ll;
}

template <class T, int VS, int PAIR, bool RO>
__device__ __forceinline__ void acc_cross(CV<T, VS>& C, CV<T, VS>& Mm, T g, T s1, T s2, const uint32_t (&idx)[4],
                                          unsigned msk, const cplx<T>* x, int ns, int s0) {
    CV<T, VS> v1, v2, v3, v4;
    ld_nb<T, VS, RO>(v1, x, idx[0], ns, s0, msk & 1);
    ld_nb<T, VS, RO>(v2, x, idx[1], ns, s0, msk >> 1 & 1);
    ld_nb<T, VS, RO>(v3, x, idx[2], ns, s0, msk >> 2 & 1);
    ld_nb<T, VS, RO>(v4, x, idx[3], ns, s0, msk >> 3 & 1);
#pragma unroll
    for (int q = 0; q < VS; q++) {
        cplx<T> cu = (v1.v[q] - v2.v[q]) + (v4.v[q] - v3.v[q]);
        C.v[q].x += g * cu.x;
        C.v[q].y += g * cu.y;
    }
    // rows whose cells are all isotropic have no cross-orientation mass terms
    // (adding 0 * m would leave Mm bit-identical): skip the 8 adds and fused
    // multiply-adds per system, a third of the FP64 operator's instructions
    if (both_zero(s1, s2)) return;
#pragma unroll
    for (int q = 0; q < VS; q++) {
        cplx<T> m1 = PAIR == 0 ? v1.v[q] + v2.v[q] : v1.v[q] + v3.v[q];
        cplx<T> m2 = PAIR == 0 ? v3.v[q] + v4.v[q] : v2.v[q] + v4.v[q];
        Mm.v[q].x += s1 * m1.x + s2 * m2.x;
        Mm.v[q].y += s1 * m1.y + s2 * m2.y;
    }
}

template <class T, int VS, int O, bool SAME, bool CA, bool CB, bool RO>
__device__ __forceinline__ void row_off(const RowK<T>& K, const RowN& N, const cplx<T>* x, int ns, int s0, CV<T, VS>& C,
                                        CV<T, VS>& Mm) {
    cvzero<T, VS>(C);
    cvzero<T, VS>(Mm);
    if (SAME) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            CV<T, VS> nb;
            ld_nb<T, VS, RO>(nb, x, N.same[q], ns, s0, N.msame >> q & 1);
#pragma unroll
            for (int v = 0; v < VS; v++) {
                C.v[v].x += K.cs[q] * nb.v[v].x;
                C.v[v].y += K.cs[q] * nb.v[v].y;
            }
        }
    }
    if (CA) acc_cross<T, VS, RowPair<O>::A, RO>(C, Mm, K.gA, K.sA1, K.sA2, N.A, N.mA, x, ns, s0);
    if (CB) acc_cross<T, VS, RowPair<O>::B, RO>(C, Mm, K.gB, K.sB1, K.sB2, N.B, N.mB, x, ns, s0);
}

// y = C - i*wm*M
template <class T> __device__ __forceinline__ cplx<T> cm_combine(cplx<T> C, cplx<T> Mm, T wm) {
    return mk<T>(C.x + wm * Mm.y, C.y - wm * Mm.x);
}
// complex diagonal of the row for frequency wm
template <class T> __device__ __forceinline__ cplx<T> row_dia(const RowK<T>& K, T wm) { return mk<T>(K.dre, -wm * K.sbar); }

// Full row y = A x for VS systems at edge e (boundary rows: identity).
template <class T, int VS, int O>
__device__ __forceinline__ void row_apply_o(const Lev<T>& L, const Mesh& M, uint32_t e, int i, int j, int k,
                                            const cplx<T>* x, int ns, int s0, const T (&wm)[VS], const CV<T, VS>& xe,
                                            CV<T, VS>& y) {
    if (mbnd(M, O, i, j, k)) {
        y = xe;
        return;
    }
    const RowK<T> K = row_k_e<T, O, true, true, true>(L, e, i, j, k);
    const RowN N = row_n<O>(M, e, i, j, k);
    CV<T, VS> C, Mm;
    row_off<T, VS, O, true, true, true, true>(K, N, x, ns, s0, C, Mm);
#pragma unroll
    for (int q = 0; q < VS; q++) {
        C.v[q].x += K.dre * xe.v[q].x;
        C.v[q].y += K.dre * xe.v[q].y;
        Mm.v[q].x += K.sbar * xe.v[q].x;
        Mm.v[q].y += K.sbar * xe.v[q].y;
        y.v[q] = cm_combine<T>(C.v[q], Mm.v[q], wm[q]);
    }
}
template <class T, int VS>
__device__ __forceinline__ void row_apply(const Lev<T>& L, const Mesh& M, int o, uint32_t e, int i, int j, int k,
                                          const cplx<T>* x, int ns, int s0, const T (&wm)[VS], const CV<T, VS>& xe,
                                          CV<T, VS>& y) {
    if (o == OX)
        row_apply_o<T, VS, OX>(L, M, e, i, j, k, x, ns, s0, wm, xe, y);
    else if (o == OY)
        row_apply_o<T, VS, OY>(L, M, e, i, j, k, x, ns, s0, wm, xe, y);
    else
        row_apply_o<T, VS, OZ>(L, M, e, i, j, k, x, ns, s0, wm, xe, y);
}

// Dual volume of edge (o,i,j,k): length x the two transverse half-spacing
// sums -- the row weight that makes the operator complex symmetric (V K = K^T V
// on the interior rows).  Boundary (identity) rows get weight 1.
template <class T>
__device__ __forceinline__ T edge_vol(const Lev<T>& L, const Mesh& M, int o, int i, int j, int k) {
    if (mbnd(M, o, i, j, k)) return T(1);
    if (o == OX) return T(0.25) / (__ldg(L.ax.rh + i) * __ldg(L.ay.rs + j) * __ldg(L.az.rs + k));
    if (o == OY) return T(0.25) / (__ldg(L.ay.rh + j) * __ldg(L.ax.rs + i) * __ldg(L.az.rs + k));
    return T(0.25) / (__ldg(L.az.rh + k) * __ldg(L.ax.rs + i) * __ldg(L.ay.rs + j));
}

// ---------------------------------------------------------------- system groups
// A thread's systems are s0 .. s0+VS-1 with s0 = (threadIdx.x % G) * VS;
// blockDim and the grid stride are multiples of G.
struct SysG {
    int ns, G;
    FastDiv fG;
};
// shared memory of vreduce_last (sfdx_vkern.cuh) for nq partial sums per system
inline size_t vred_smem_bytes(int B, int nq, int ns) {
    size_t a = (size_t)B + (size_t)nq * ns, b = (size_t)(B / 32 + 1) * nq * ns;
    return (a > b ? a : b) * sizeof(double2);
}
inline SysG make_sysg(int ns, int VS) {
    SysG s;
    s.ns = ns;
    s.G = ns / VS;
    s.fG = make_fastdiv(s.G);
    return s;
}

}  // namespace sfdx
