// sfdx_kernels.cuh -- kernels of the matrix-free forward solver (templated on
// the arithmetic type T = float | double).  Host drivers live in
// sfdx_solver.cu.
#pragma once
#include "sfdx_device.cuh"

namespace sfdx {

// ------------------------------------------------------------------ state
// Per-system Krylov state (one entry per system of a batch), FP64 always.
enum { ST_RUN = 0, ST_CONV = 1, ST_MAXIT = 2, ST_NAN = 3, ST_BREAK = 4 };

struct KState {
    double2 rho, rhoold, alpha, omega, beta;
    double2 eta, tau;        // GPBiCG / spare
    double babs, err, tol;
    double wm;               // omega*mu of the system's frequency
    double errv;             // last FP64-verified relative residual (mixed precision)
    int it, itmax, active, status, iters;
    int pad[3];
};

// ------------------------------------------------------------------ reductions
// A reducing kernel keeps NQ complex accumulators per thread (all for the
// thread's system s = threadIdx.x % ns, constant because blockDim and the
// grid stride are multiples of ns).  Block partials go to `part`
// [gridDim][NQ][ns]; the last block to finish sums them in a fixed order
// (deterministic) and hands the totals to the kernel's finaliser.
struct RedBuf {
    double2* part;
    unsigned int* counter;
};

template <int NQ, class Acc>
__device__ __forceinline__ bool block_reduce_and_last(double2 (&acc)[NQ], int ns, RedBuf rb, double2* sm) {
    // sm holds max(NQ,2)*blockDim double2.  On return (last block only) the
    // totals of slot q*ns+s are in sm[blockDim + q*ns + s].
    const int t = threadIdx.x, B = blockDim.x;
    for (int q = 0; q < NQ; q++) sm[q * B + t] = acc[q];
    __syncthreads();
    for (int stride = B >> 1; stride >= ns; stride >>= 1) {
        if (t < stride)
            for (int q = 0; q < NQ; q++) sm[q * B + t] = sm[q * B + t] + sm[q * B + t + stride];
        __syncthreads();
    }
    if (t < ns)
        for (int q = 0; q < NQ; q++) rb.part[((size_t)blockIdx.x * NQ + q) * ns + t] = sm[q * B + t];
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (t == 0) {
        unsigned int prev = atomicAdd(rb.counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    // deterministic final sum: `per` threads share the blocks of each slot
    const int slots = NQ * ns;  // <= B (host guarantees)
    const int per = B / slots;
    const int slot = t / per, lane = t % per;
    double2 a = make_double2(0.0, 0.0);
    if (slot < slots) {
        const int q = slot / ns, s = slot % ns;
        for (int b = lane; b < (int)gridDim.x; b += per) a = a + __ldcg(rb.part + ((size_t)b * NQ + q) * ns + s);
    }
    __syncthreads();
    sm[t] = a;
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (slot < slots && lane == 0)
        for (int l = 0; l < per; l++) r = r + sm[t + l];
    __syncthreads();
    if (slot < slots && lane == 0) sm[B + slot] = r;
    if (t == 0) *rb.counter = 0u;
    __syncthreads();
    return true;
}

template <class T> struct AccOf;
template <> struct AccOf<float> { typedef float type; };
template <> struct AccOf<double> { typedef double type; };

// ------------------------------------------------------------------ operator
// y = A x for edge e of system s (A as assembled by fd_assemb + dcfast).
template <class T>
__device__ __forceinline__ cplx<T> apply_row(const Lev<T>& L, int o, int i, int j, int k, T wm, const cplx<T>* x, int ns,
                                             int s, cplx<T> xe) {
    if (is_bnd(L, o, i, j, k)) return xe;
    FetchInterior<T> f{&L, x, ns, s};
    cplx<T> off;
    RowCoef<T> rc;
    if (o == OX) {
        off = row_offdiag<T, OX, true, true, true>(L, i, j, k, wm, f);
        rc = row_diag<T, OX>(L, i, j, k);
    } else if (o == OY) {
        off = row_offdiag<T, OY, true, true, true>(L, i, j, k, wm, f);
        rc = row_diag<T, OY>(L, i, j, k);
    } else {
        off = row_offdiag<T, OZ, true, true, true>(L, i, j, k, wm, f);
        rc = row_diag<T, OZ>(L, i, j, k);
    }
    return off + cmul<T>(mk<T>(rc.dre, -wm * rc.sbar), xe);
}

// Right-hand side of dcfast: boundary rows carry the Dirichlet value, interior
// rows -sum(K_ij p_j) over boundary columns.  FP64 only; written to b64.
static __global__ void k_build_rhs(Lev<double> L, const double* wms, const int* pols, const double2* edcs, int edc_stride,
                            int ns, double2* __restrict__ b) {
    const int64_t W = L.nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        int s = (int)(g % ns);
        int64_t e = g / ns;
        int o, i, j, k;
        edecode(L, e, o, i, j, k);
        const double2* edc = edcs + (size_t)s * edc_stride;
        int pol = pols[s];
        if (is_bnd(L, o, i, j, k)) {
            b[g] = dirichlet_value(L.nx, L.ny, L.nz, pol, edc, o, i, j, k);
            continue;
        }
        FetchDirichlet f{&L, pol, edc};
        double wm = wms[s];
        double2 off;
        if (o == OX)
            off = row_offdiag<double, OX, true, true, true>(L, i, j, k, wm, f);
        else if (o == OY)
            off = row_offdiag<double, OY, true, true, true>(L, i, j, k, wm, f);
        else
            off = row_offdiag<double, OZ, true, true, true>(L, i, j, k, wm, f);
        b[g] = make_double2(-off.x, -off.y);
    }
}

// Right-hand-side modes of the forward sweep.
enum { RHS_VEC = 0, RHS_PUPD = 1, RHS_SUPD = 2, RHS_COCR = 3 };

// Jacobi preconditioner (pre_type 'J'): y = D^{-1} rhs with the same fused
// right-hand-side modes.
template <class T, int MODE>
__global__ void k_jacobi(Lev<T> L, const KState* st, int ns, cplx<T>* __restrict__ w, cplx<T>* __restrict__ q,
                         const cplx<T>* __restrict__ r, const cplx<T>* __restrict__ v) {
    const int64_t W = L.nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        int s = (int)(g % ns);
        if (!st[s].active) continue;
        int o, i, j, k;
        edecode(L, g / ns, o, i, j, k);
        cplx<T> rhs;
        if (MODE == RHS_PUPD) {
            cplx<T> be = mk<T>((T)st[s].beta.x, (T)st[s].beta.y), om = mk<T>((T)st[s].omega.x, (T)st[s].omega.y);
            rhs = r[g] + cmul<T>(be, q[g] - cmul<T>(om, v[g]));
            q[g] = rhs;
        } else if (MODE == RHS_SUPD) {
            cplx<T> al = mk<T>((T)st[s].alpha.x, (T)st[s].alpha.y);
            rhs = r[g] - cmul<T>(al, v[g]);
            q[g] = rhs;
        } else {
            rhs = q[g];
        }
        if (is_bnd(L, o, i, j, k)) {
            w[g] = rhs;
            continue;
        }
        T wm = (T)st[s].wm;
        RowCoef<T> rc;
        if (o == OX) rc = row_diag<T, OX>(L, i, j, k);
        else if (o == OY) rc = row_diag<T, OY>(L, i, j, k);
        else rc = row_diag<T, OZ>(L, i, j, k);
        w[g] = cdiv<T>(rhs, mk<T>(rc.dre, -wm * rc.sbar));
    }
}

// Residual  r = b - A x  (optionally rhat = r), FP64 operator or mixed.
// MODE 0: initialise a Krylov solve (babs, err, rho, beta, convergence test)
// MODE 1: restart after a divergence correction (rho, beta only)
// MODE 2: refinement residual: stores |r| into st.err * st.babs and scale
template <class T, class XT, int MODE>
__global__ void k_residual(Lev<XT> L, KState* st, int ns, const cplx<XT>* __restrict__ bvec, const cplx<XT>* __restrict__ x,
                           cplx<T>* __restrict__ r, cplx<T>* __restrict__ rhat, RedBuf rb, double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    const int s = threadIdx.x % ns;
    const bool act = st[s].active;
    const XT wm = (XT)st[s].wm;
    double rr = 0, bb = 0;
    const int64_t W = L.nl * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            int o, i, j, k;
            edecode(L, g / ns, o, i, j, k);
            cplx<XT> ax = apply_row<XT>(L, o, i, j, k, wm, x, ns, s, x[g]);
            cplx<XT> bv = bvec[g];
            cplx<XT> rv = bv - ax;
            cplx<T> rt = mk<T>((T)rv.x, (T)rv.y);
            r[g] = rt;
            if (rhat) rhat[g] = rt;
            rr += (double)cabs2<XT>(rv);
            bb += (double)cabs2<XT>(bv);
        }
    double2 acc[1] = {make_double2(rr, bb)};
    if (!block_reduce_and_last<1, double>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = st[ss];
        if (!S.active) continue;
        double2 v = smem[B + ss];
        double nr = sqrt(v.x);
        if (MODE == 0) {
            S.babs = sqrt(v.y);
            S.err = nr / S.babs;
            S.errv = S.err;
            S.rho = make_double2(1.0, 0.0);
            S.alpha = make_double2(1.0, 0.0);
            S.omega = make_double2(1.0, 0.0);
            S.it = 1;
            S.iters = 1;
            if (err_rec) err_rec[(size_t)ss * err_stride] = S.err;
            if (isnan(S.err)) {  // solvers.f90:619
                S.status = ST_NAN;
                S.active = 0;
                S.iters = 0;
                continue;
            }
            if (S.err < S.tol) {
                S.status = ST_CONV;
                S.active = 0;
                continue;
            }
            // rhat == r here, so rho = <rhat, r> = |r|^2 and beta = rho
            S.rhoold = S.rho;
            S.rho = make_double2(v.x, 0.0);
            S.beta = S.rho;
        } else if (MODE == 1) {
            S.rho = make_double2(v.x, 0.0);
            double2 a = S.rho, b = S.rhoold, al2 = S.alpha, om2 = S.omega;
            double bd = b.x * b.x + b.y * b.y, od = om2.x * om2.x + om2.y * om2.y;
            double2 q1 = make_double2((a.x * b.x + a.y * b.y) / bd, (a.y * b.x - a.x * b.y) / bd);
            double2 q2 = make_double2((al2.x * om2.x + al2.y * om2.y) / od, (al2.y * om2.x - al2.x * om2.y) / od);
            S.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        } else if (MODE == 2) {
            S.err = nr;  // absolute residual norm; the host driver scales
            S.babs = sqrt(v.y);
        } else if (MODE == 3) {  // GPBiCG start (solvers.f90:203-221): no stopping test before iteration 1
            S.babs = sqrt(v.y);
            S.err = nr / S.babs;
            S.errv = S.err;
            S.it = 1;
            S.iters = 0;
            S.beta = make_double2(0.0, 0.0);
            if (isnan(S.err)) {
                S.status = ST_NAN;
                S.active = 0;
            }
        }
        // MODE 4: residual restart only (GPBiCG after a divergence correction)
    }
}

// ------------------------------------------------------------------ reliable updates
// Mixed precision: the Krylov iteration runs in complex64 on a partial
// solution x32; every few iterations (and whenever the complex64 recurrence
// claims convergence) the partial solution is folded into the complex128
// solution, the residual is recomputed in FP64 and handed back to the
// complex64 iteration, whose search directions are kept (reliable updated
// residuals, Sleijpen & van der Vorst 1996).  Convergence is decided on the
// FP64 residual only.
enum { ST_VCONV = 5 };
// a system masked out of this solve (already finished, or handed elsewhere):
// never reactivated, never updated
enum { ST_SKIP = 6 };

// systems whose complex64 recurrence converged become active again until the
// FP64 residual confirms it
static __global__ void k_reactivate(KState* st, int ns) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ns && st[s].status == ST_CONV) {
        st[s].status = ST_RUN;
        st[s].active = 1;
    }
}

// x64 = xb for the systems whose last update was rejected (status ST_BREAK)
static __global__ void k_restore(int64_t nl, const KState* st, int ns, double2* __restrict__ x64, const double2* __restrict__ xb) {
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (st[s].status == ST_BREAK && st[s].pad[0] == 1) x64[g] = xb[g];
    }
}

// x64 = xb for the systems selected by sel[s] != 0
static __global__ void k_restore_sel(int64_t nl, const int* __restrict__ sel, int ns, double2* __restrict__ x64,
                                     const double2* __restrict__ xb) {
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (sel[s]) x64[g] = xb[g];
    }
}

// ------------------------------------------------------------------ misc vector kernels
template <class A, class B>
__global__ void k_convert(int64_t n, const cplx<A>* __restrict__ src, cplx<B>* __restrict__ dst) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
        cplx<A> v = src[g];
        dst[g] = mk<B>((B)v.x, (B)v.y);
    }
}

// deterministic smooth input for kernel timing
template <class T>
__global__ void k_pattern(int64_t n, cplx<T>* __restrict__ v) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
        v[g] = mk<T>((T)(1.0 + 1e-3 * (double)(g % 977)), (T)(0.5 - 1e-3 * (double)(g % 613)));
}

template <class T>
__global__ void k_scatter_sys(int64_t nl, int ns, const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst_sys_major) {
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        int s = (int)(g % ns);
        int64_t e = g / ns;
        dst_sys_major[(size_t)s * nl + e] = src[g];
    }
}

}  // namespace sfdx
