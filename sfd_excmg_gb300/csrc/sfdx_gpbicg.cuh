// sfdx_gpbicg.cuh -- GPBiCG (pgpbicg, solvers.f90:137-315; Itoh 2022),
// right-preconditioned, for ns interleaved systems with device-side scalars.
// Per iteration: two operator applications fused with their inner products,
// two multi-colour SSOR applications, three fused vector updates.
#pragma once
#include "sfdx_kernels.cuh"

namespace sfdx {

// Extra per-system scalars live in KState: alpha, omega (as in BiCGStab),
// beta, eta, rho (= <r0, r> of the current r), rhoold (spare).

// ap = A p ; alpha = <r0, r> / <r0, ap>
template <class T>
__global__ void k_gp_ap(Lev<T> L, KState* st, int ns, const cplx<T>* __restrict__ p, cplx<T>* __restrict__ ap,
                        const cplx<T>* __restrict__ r0, const cplx<T>* __restrict__ r, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int s = threadIdx.x % ns;
    const bool act = st[s].active;
    const T wm = (T)st[s].wm;
    A a0r = 0, a0i = 0, a1r = 0, a1i = 0;
    const int64_t W = L.nl * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            int o, i, j, k;
            edecode(L, g / ns, o, i, j, k);
            cplx<T> val = apply_row<T>(L, o, i, j, k, wm, p, ns, s, p[g]);
            ap[g] = val;
            cplx<T> rr0 = r0[g];
            cplx<T> d0 = cdot<T>(rr0, val), d1 = cdot<T>(rr0, r[g]);
            a0r += d0.x; a0i += d0.y; a1r += d1.x; a1i += d1.y;
        }
    double2 acc[2] = {make_double2(a0r, a0i), make_double2(a1r, a1i)};
    if (!block_reduce_and_last<2, A>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = st[ss];
        if (!S.active) continue;
        double2 d = smem[B + ss], n = smem[B + ns + ss];
        double den = d.x * d.x + d.y * d.y;
        S.rho = n;  // <r0, r>, the "rold" inner product of the beta update
        S.alpha = make_double2((n.x * d.x + n.y * d.y) / den, (n.y * d.x - n.x * d.y) / den);
        if (!isfinite(S.alpha.x) || !isfinite(S.alpha.y)) {
            S.active = 0;
            S.status = ST_BREAK;
        }
    }
}

// y = t - r - alpha w + alpha ap ; t = r - alpha ap
template <class T>
__global__ void k_gp_yt(int64_t nl, const KState* st, int ns, cplx<T>* __restrict__ y, cplx<T>* __restrict__ t,
                        const cplx<T>* __restrict__ r, const cplx<T>* __restrict__ w, const cplx<T>* __restrict__ ap) {
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (!st[s].active) continue;
        const cplx<T> al = mk<T>((T)st[s].alpha.x, (T)st[s].alpha.y);
        cplx<T> tt = t[g], rr = r[g], aap = cmul<T>(al, ap[g]);
        y[g] = (tt - rr) - cmul<T>(al, w[g]) + aap;
        t[g] = rr - aap;
    }
}

// tp = rp - alpha tmp
template <class T>
__global__ void k_gp_tp(int64_t nl, const KState* st, int ns, cplx<T>* __restrict__ tp, const cplx<T>* __restrict__ rp,
                        const cplx<T>* __restrict__ tmp) {
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (!st[s].active) continue;
        const cplx<T> al = mk<T>((T)st[s].alpha.x, (T)st[s].alpha.y);
        tp[g] = rp[g] - cmul<T>(al, tmp[g]);
    }
}

// at = A tp ; omega, eta from <at,t>, <at,at>, <y,y>, <y,t>, <at,y>
template <class T>
__global__ void k_gp_at(Lev<T> L, KState* st, int ns, const cplx<T>* __restrict__ tp, cplx<T>* __restrict__ at,
                        const cplx<T>* __restrict__ t, const cplx<T>* __restrict__ y, RedBuf rb) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int s = threadIdx.x % ns;
    const bool act = st[s].active;
    const T wm = (T)st[s].wm;
    A c0r = 0, c0i = 0, c1 = 0, c2 = 0, c3r = 0, c3i = 0, c4r = 0, c4i = 0;
    const int64_t W = L.nl * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            int o, i, j, k;
            edecode(L, g / ns, o, i, j, k);
            cplx<T> val = apply_row<T>(L, o, i, j, k, wm, tp, ns, s, tp[g]);
            at[g] = val;
            cplx<T> tt = t[g], yy = y[g];
            cplx<T> d0 = cdot<T>(val, tt), d3 = cdot<T>(yy, tt), d4 = cdot<T>(val, yy);
            c0r += d0.x; c0i += d0.y;
            c1 += cabs2<T>(val);
            c2 += cabs2<T>(yy);
            c3r += d3.x; c3i += d3.y;
            c4r += d4.x; c4i += d4.y;
        }
    double2 acc[4] = {make_double2(c0r, c0i), make_double2(c1, c2), make_double2(c3r, c3i), make_double2(c4r, c4i)};
    if (!block_reduce_and_last<4, A>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = st[ss];
        if (!S.active) continue;
        typedef double2 Z;
        Z att = smem[B + ss];
        double atat = smem[B + ns + ss].x, yy = smem[B + ns + ss].y;
        Z yt = smem[B + 2 * ns + ss], aty = smem[B + 3 * ns + ss];
        Z yat = make_double2(aty.x, -aty.y);  // <y, at> = conj(<at, y>)
        auto mul = [](Z a, Z b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
        auto sub = [](Z a, Z b) { return make_double2(a.x - b.x, a.y - b.y); };
        auto dv = [](Z a, Z b) {
            double d = b.x * b.x + b.y * b.y;
            return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
        };
        Z om, et;
        if (S.it == 1) {
            om = make_double2(att.x / atat, att.y / atat);
            et = make_double2(0.0, 0.0);
        } else {
            Z Yy = make_double2(yy, 0.0), Atat = make_double2(atat, 0.0);
            Z den = sub(mul(Atat, Yy), mul(yat, aty));
            om = dv(sub(mul(Yy, att), mul(yt, aty)), den);
            et = dv(sub(mul(Atat, yt), mul(yat, att)), den);
        }
        S.omega = om;
        S.eta = et;
        if (!isfinite(om.x) || !isfinite(om.y) || !isfinite(et.x) || !isfinite(et.y) || (om.x == 0.0 && om.y == 0.0)) {
            S.active = 0;
            S.status = ST_BREAK;
        }
    }
}

// u = omega tmp + eta (tpold - rp + beta u) ; z = omega rp + eta z - alpha u ;
// x += alpha p + z ; r = t - eta y - omega at ; err, convergence, beta
template <class T, class XT>
__global__ void k_gp_upd(int64_t nl, KState* st, int ns, cplx<T>* __restrict__ u, cplx<T>* __restrict__ z,
                         cplx<XT>* __restrict__ x, cplx<T>* __restrict__ r, const cplx<T>* __restrict__ tmp,
                         const cplx<T>* __restrict__ tpold, const cplx<T>* __restrict__ rp, const cplx<T>* __restrict__ p,
                         const cplx<T>* __restrict__ t, const cplx<T>* __restrict__ y, const cplx<T>* __restrict__ at,
                         const cplx<T>* __restrict__ r0, RedBuf rb, double* err_rec, int err_stride) {
    extern __shared__ double2 smem[];
    typedef typename AccOf<T>::type A;
    const int s = threadIdx.x % ns;
    const bool act = st[s].active;
    const cplx<T> al = mk<T>((T)st[s].alpha.x, (T)st[s].alpha.y), om = mk<T>((T)st[s].omega.x, (T)st[s].omega.y);
    const cplx<T> et = mk<T>((T)st[s].eta.x, (T)st[s].eta.y), be = mk<T>((T)st[s].beta.x, (T)st[s].beta.y);
    const cplx<XT> alx = mk<XT>((XT)st[s].alpha.x, (XT)st[s].alpha.y);
    A rr = 0, hr = 0, hi = 0;
    const int64_t W = nl * ns;
    if (act)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
            cplx<T> rpg = rp[g];
            cplx<T> un = cmul<T>(om, tmp[g]) + cmul<T>(et, (tpold[g] - rpg) + cmul<T>(be, u[g]));
            u[g] = un;
            cplx<T> zn = cmul<T>(om, rpg) + cmul<T>(et, z[g]) - cmul<T>(al, un);
            z[g] = zn;
            cplx<T> pg = p[g];
            cplx<XT> p2 = mk<XT>((XT)pg.x, (XT)pg.y), z2 = mk<XT>((XT)zn.x, (XT)zn.y);
            x[g] = x[g] + cmul<XT>(alx, p2) + z2;
            cplx<T> rn = (t[g] - cmul<T>(et, y[g])) - cmul<T>(om, at[g]);
            r[g] = rn;
            rr += cabs2<T>(rn);
            cplx<T> d = cdot<T>(r0[g], rn);
            hr += d.x;
            hi += d.y;
        }
    double2 acc[2] = {make_double2(rr, 0.0), make_double2(hr, hi)};
    if (!block_reduce_and_last<2, A>(acc, ns, rb, smem)) return;
    const int B = blockDim.x;
    for (int ss = threadIdx.x; ss < ns; ss += B) {
        KState& S = st[ss];
        if (!S.active) continue;
        double nr = sqrt(smem[B + ss].x);
        double2 rn = smem[B + ns + ss];
        S.err = nr / S.babs;
        if (err_rec && S.it <= S.itmax) err_rec[(size_t)ss * err_stride + S.it - 1] = S.err;
        S.iters = S.it;
        // beta = alpha/omega * <r0, r_new> / <r0, r_old>, computed before the
        // stopping tests so that a resumed system (mixed precision re-check)
        // continues with consistent scalars
        double2 a = S.alpha, o = S.omega, ro = S.rho;
        double od = o.x * o.x + o.y * o.y, rd = ro.x * ro.x + ro.y * ro.y;
        double2 q1 = make_double2((a.x * o.x + a.y * o.y) / od, (a.y * o.x - a.x * o.y) / od);
        double2 q2 = make_double2((rn.x * ro.x + rn.y * ro.y) / rd, (rn.y * ro.x - rn.x * ro.y) / rd);
        S.beta = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        S.it += 1;
        if (isnan(S.err)) {
            S.status = ST_NAN;
            S.active = 0;
            continue;
        }
        if (S.err <= S.tol) {  // solvers.f90:272
            S.status = ST_CONV;
            S.active = 0;
            continue;
        }
        if (S.iters >= S.itmax) {
            S.status = ST_MAXIT;
            S.active = 0;
            continue;
        }
    }
}

// w = at + beta ap ; p = rp + beta (p - u)
template <class T>
__global__ void k_gp_pw(int64_t nl, const KState* st, int ns, cplx<T>* __restrict__ w, cplx<T>* __restrict__ p,
                        const cplx<T>* __restrict__ at, const cplx<T>* __restrict__ ap, const cplx<T>* __restrict__ rp,
                        const cplx<T>* __restrict__ u) {
    const int64_t W = nl * ns;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < W; g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g % ns);
        if (!st[s].active) continue;
        const cplx<T> be = mk<T>((T)st[s].beta.x, (T)st[s].beta.y);
        w[g] = at[g] + cmul<T>(be, ap[g]);
        p[g] = rp[g] + cmul<T>(be, p[g] - u[g]);
    }
}

}  // namespace sfdx
