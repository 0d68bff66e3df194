// sfdx_plan.h -- host-side structures shared by the translation units of the
// solver: device buffers, mesh levels, the plan (one mesh hierarchy + one
// frequency list), launch sizing and the launch counter.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <type_traits>
#include <vector>

#include "sfdx.h"
#include "sfdx_kernels.cuh"
#include "sfdx_nodemg.cuh"
#include "sfdx_stencil.cuh"

namespace sfdx {

static const double kPi = 3.141592653589793238462643;
static const double kMu = 4.0 * 3.141592653589793238462643 * 1e-7;

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) {                                        \
            if (getenv("SFDX_DEBUG"))                                   \
                fprintf(stderr, "sfdx: CUDA %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return SFDX_ERR_CUDA;                                       \
        }                                                               \
    } while (0)
#define RC(call)                       \
    do {                               \
        int r_ = (call);               \
        if (r_ != SFDX_OK) return r_;  \
    } while (0)

// kernel launches issued by this library (process-wide)
extern std::atomic<long long> g_launches;
#define KL(...) (g_launches.fetch_add(1, std::memory_order_relaxed), __VA_ARGS__)

inline int device_sms() {
    static const int nsm = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return nsm;
}

// block size: ns * 2^k in [128, 1024] and >= nq*ns (per-system reductions)
inline int block_for(int ns, int nq = 2) {
    int b = ns;
    while (b < 128 || b < nq * ns) b *= 2;
    return b;
}
inline int grid_for(int64_t work, int B, int per_sm = 8) {
    int64_t g = (work + B - 1) / B;
    int64_t cap = (int64_t)device_sms() * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}
// Grid of a grid-stride kernel: the blocks that can be resident at once (one
// wave), capped by the work.  With one wave every block walks the domain in
// step with the others, so the neighbour data of a plane is fetched from DRAM
// about once; a second wave of blocks would sweep the domain again.
inline int resident_grid(const void* fn, int B, size_t smem, int64_t work) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, size_t>, int> cache;
    int per = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto key = std::make_tuple(fn, B, smem);
        auto it = cache.find(key);
        if (it != cache.end()) {
            per = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, B, smem) != cudaSuccess || per < 1) per = 1;
            cache[key] = per;
        }
    }
    int64_t g = (work + B - 1) / B;
    const int64_t cap = (int64_t)per * device_sms();
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}
// most blocks resident_grid() returns (sizes the per-block partial sums)
inline int64_t max_resident_blocks() { return (int64_t)device_sms() * 32; }

// The system-group kernels move 32-byte groups of a thread's systems with
// 256-bit accesses (sfdx_stencil.cuh).  Their offsets [edge * ns + s0] are
// multiples of 32 bytes (VS divides ns), so alignment rests on the base
// pointers: every pointer argument is checked here, once per launch, and a
// launch with a misaligned one is refused instead of faulting on the device.
// The refusal is recorded per host thread (a plan's work runs on one thread)
// and the next sync_state of that thread reports it as SFDX_ERR_ARG and
// clears it, so it fails the call that hit it and no other.
extern thread_local int g_misaligned;
template <class X> inline bool arg_aligned(const X&) { return true; }
template <class X> inline bool arg_aligned(X* p) { return (reinterpret_cast<uintptr_t>(p) & 31) == 0; }
template <class... KA, class... A>
inline void vlaunch(void (*k)(KA...), int64_t work, int B, size_t smem, cudaStream_t st, A... args) {
    if (!(arg_aligned(args) && ...)) {
        g_misaligned = 1;
        return;
    }
    const int g = resident_grid((const void*)k, B, smem, work);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k<<<g, B, smem, st>>>(args...);
}

// systems per thread of the hot kernels: the largest of 4, 2, 1 that is at
// most `want` and divides ns
inline int vs_pick(int ns, int want) {
    if (want >= 4 && ns % 4 == 0) return 4;
    if (want >= 2 && ns % 2 == 0) return 2;
    return 1;
}
// block of the system-group kernels: G * 2^k >= 128
inline int vblock(int G) {
    int b = G;
    while (b < 128) b *= 2;
    return b;
}

// ------------------------------------------------------------------ device buffers
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
        o.p = nullptr;
        o.bytes = 0;
    }
    ~DBuf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t n) {
        if (n <= bytes) return SFDX_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (cudaMalloc(&p, n) != cudaSuccess) return SFDX_ERR_NOMEM;
        bytes = n;
        return SFDX_OK;
    }
    template <class X> X* as() const { return reinterpret_cast<X*>(p); }
};

// ------------------------------------------------------------------ mesh level
template <class T> AxisT<T> axis_ptrs(const T* base, int stride, int axis) {
    const T* p = base + (size_t)axis * 6 * stride;
    AxisT<T> a;
    a.rh = p;
    a.lo = p + stride;
    a.hi = p + 2 * stride;
    a.rs = p + 3 * stride;
    a.wlo = p + 4 * stride;
    a.whi = p + 5 * stride;
    return a;
}

// One level of the nodal multigrid of the gradient-space correction: the
// 27-point stencil (float) with its inverse diagonal, and the V-cycle work
// vectors (complex64, ns systems) of that grid.
struct NodeMG {
    NGrid g;
    DBuf coef, dinv;
    DBuf x, b, t, r;
    NodeMG() = default;
    NodeMG(NodeMG&&) = default;
};

struct Level {
    int nx = 0, ny = 0, nz = 0, nair = 0;
    int64_t xnl = 0, ynl = 0, nl = 0, ncell = 0;
    Mesh mesh;
    std::vector<double> a, b, c;
    int aniso = 0;
    DBuf tab64, tab32;     // [3 axes][6 arrays][stride]
    DBuf sig64, sig32;     // [6][ncell]
    DBuf rc64, rc32;       // per-row coefficients [nl][12] (k_row_coef), valid if rc_ok
    bool rc_ok = false;
    DBuf spac;             // a, b, c (device, FP64) for coarsening
    DBuf crd_cubic;        // node coordinates used by cubic_interp on this level
    DBuf crd_quad;         // node coordinates used by quad_interp_e (pairwise sums of a,b,c)
    int stride = 0;
    // nodal multigrid hierarchy of the gradient-space correction (mg[0]: this
    // level's node grid); rebuilt after the conductivity of the level changes
    mutable std::vector<NodeMG> mg;
    mutable bool gc_ok = false;
    // work vectors of the edge multigrid preconditioner on this level:
    // residual, smoother output, nodal update, and (below the solve level)
    // the level's right-hand side and solution
    mutable DBuf emg_r, emg_z, emg_phi, emg_b, emg_x;
    mutable DBuf emg_psi, emg_g, emg_t;  // split V-cycle: nodal potential, edge temporaries

    void set_dims(int X, int Y, int Z) {
        nx = X; ny = Y; nz = Z;
        xnl = (int64_t)nx * (ny + 1) * (nz + 1);
        ynl = (int64_t)(nx + 1) * ny * (nz + 1);
        nl = xnl + ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
        ncell = (int64_t)nx * ny * nz;
        mesh = make_mesh(nx, ny, nz);
    }
    template <class T> Lev<T> lev() const {
        Lev<T> L;
        L.nx = nx; L.ny = ny; L.nz = nz;
        L.xnl = xnl; L.ynl = ynl; L.nl = nl; L.ncell = ncell;
        const T* base = std::is_same<T, double>::value ? (const T*)tab64.p : (const T*)tab32.p;
        L.ax = axis_ptrs<T>(base, stride, 0);
        L.ay = axis_ptrs<T>(base, stride, 1);
        L.az = axis_ptrs<T>(base, stride, 2);
        L.sig = std::is_same<T, double>::value ? (const T*)sig64.p : (const T*)sig32.p;
        L.aniso = aniso;
        L.rc = !rc_ok ? nullptr : std::is_same<T, double>::value ? (const T*)rc64.p : (const T*)rc32.p;
        return L;
    }
};

// ------------------------------------------------------------------ CUDA graphs
// Launch sequences that run between two host checks (a check interval of
// Krylov iterations) are captured once per key -- level, batch size,
// buffers, scalar kernel arguments -- and replayed as one graph launch.
struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    long long nodes = 0;
};
struct GraphCache {
    std::map<std::vector<uintptr_t>, GraphEntry> m;
    GraphCache() = default;
    GraphCache(const GraphCache&) = delete;
    ~GraphCache() {
        for (auto& kv : m)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    }
};

// ------------------------------------------------------------------ plan
struct Plan {
    sfdx_opts o;
    int nf = 0, ns = 0, nlev = 0;
    std::vector<double> freq, wm;
    std::vector<Level> lev;  // lev[0] coarsest ... lev[nlev-1] finest
    cudaStream_t st = nullptr;      // stream all work of the plan is issued on
    cudaStream_t own_st = nullptr;  // stream created by the plan (destroyed with it)
    // per-system device data
    DBuf d_state, d_wm, d_pol, d_edc, d_part, d_counter, d_tol, d_mask, d_scale, d_flag;
    // FP64 vectors (finest-level size)
    DBuf x64, b64, r64, u0, u1, ut, ex_out;
    // forward fields of the last solve, interleaved like x64, kept while
    // x64 holds adjoint solutions (xf_valid: xf matches the last solve)
    DBuf xf;
    bool xf_valid = false;
    // fields of the last full (cascade) solve, the initial guess of
    // sfdx_plan_resolve (base_valid: xbase matches that solve)
    DBuf xbase;
    bool base_valid = false;
    // mixed precision: complex64 partial solution and the FP64 iterate saved
    // before each reliable update
    DBuf x32, xb;
    DBuf d_sel;  // per-system selection flags (int) of the complex64 V-cycle fallback
    DBuf d_imp;  // workspace of the device impedance evaluation (sfdx_plan_impedance)
    // Krylov vectors (precision of the active solve)
    DBuf kv[14];
    // divergence correction: t, r, p, v, phi (nodes) and the PCG state
    DBuf dcv[5], d_pst;
    int dc_calls = 0, dc_last_iters = 0;
    // consistent gradient correction: node vectors phi, r, z, p, q of the
    // nodal PCG; edge vectors of the probing that assembles the nodal operator
    DBuf gcn[5], gce[2];
    // FP64 right-hand side and iterate of the running systems packed into a
    // smaller batch (restart cycles), and their indices in the full batch
    DBuf cb64, cx64, d_idx;
    long long gc_calls = 0, gc_iters = 0;
    DBuf errrec;
    int edc_stride = 0;
    double* hist = nullptr;  // optional device residual history [ns][hist_stride]
    int hist_stride = 0;
    std::vector<int> iters;        // [nf][2][nlev]
    std::vector<double> level_ms;  // wall time per level of the last solve
    std::vector<double> relres;    // [nf][2]
    std::vector<KState> hst;
    bool have_solution = false;
    // conductivity generation: advanced by every conductivity load; the
    // solution is current only while sol_gen == sigma_gen (fields of an
    // earlier conductivity must not feed impedances or gradients)
    long long sigma_gen = 0, sol_gen = -1;
    long long cascade_gen = -1;  // sigma_gen of the last EXCMG cascade (u0, u1 hold its two sub-finest levels)
    bool solution_current() const { return have_solution && sol_gen == sigma_gen; }
    // systems per thread of the complex64 / complex128 hot kernels (upper
    // bounds; sfdx_plan_autotune measures and sets them)
    int vs32 = 4, vs64 = 2;
    GraphCache graphs;  // captured check intervals (o.use_graphs)
    // advanced whenever a buffer or nodal operator that the edge multigrid
    // bakes into captured graphs is (re)allocated: part of every graph key
    long long emg_epoch = 0;
    // residual history of the finest-level solves, recorded at every host
    // check (8 iterations): rec_hist[system][iteration] (0: not recorded);
    // rec_map: full-batch index of each system of a packed batch (empty: the
    // identity); rec_off: iterations of earlier restart cycles per system
    bool rec_on = false;
    int rec_len = 0;
    std::vector<double> rec_hist;
    std::vector<int> rec_map, rec_off;
    // complex128 Krylov iteration with the complex64 multigrid V-cycle as its
    // preconditioner (mixed-precision plans with precond 'G', finer levels);
    // emg_q32 / emg_o32: the V-cycle's complex64 input and output
    bool pf32 = false;
    DBuf emg_q32, emg_o32;
    // complex64 Krylov iteration on split vectors y + G psi under the split
    // V-cycle (SFDX_MG_SPLIT): psi_out receives the V-cycle's nodal potential;
    // psi_y, psi_z those of the two preconditioned vectors, psi_x the partial
    // solution's; g_y, g_z = G psi_y, G psi_z on the edges
    bool split = false;
    void* psi_out = nullptr;
    DBuf psi_y, psi_z, psi_x, g_y, g_z;
    Plan() = default;
    Plan(const Plan&) = delete;
    ~Plan() {
        if (own_st) cudaStreamDestroy(own_st);
    }
};

// Run `seq` (kernel launches on P.st only, no host synchronisation) through
// the plan's graph cache under `key`: captured and instantiated on first use,
// replayed afterwards.  The launch counter advances by the graph's node count
// on every replay (the capture itself counted the launches it recorded).
template <class F> int graph_run(Plan& P, const std::vector<uintptr_t>& key, F&& seq) {
    auto it = P.graphs.m.find(key);
    if (it != P.graphs.m.end()) {
        g_launches.fetch_add(it->second.nodes, std::memory_order_relaxed);
        CK(cudaGraphLaunch(it->second.exec, P.st));
        return SFDX_OK;
    }
    cudaGraph_t g = nullptr;
    const int mis0 = g_misaligned;
    CK(cudaStreamBeginCapture(P.st, cudaStreamCaptureModeThreadLocal));
    seq();
    const cudaError_t e = cudaStreamEndCapture(P.st, &g);
    if (e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return SFDX_ERR_CUDA;
    }
    // a launch refused inside the capture (misaligned vector) is missing from
    // the graph: keep no such graph, and fail this call (the flag is cleared
    // here, as sync_state would)
    if (g_misaligned && !mis0) {
        cudaGraphDestroy(g);
        g_misaligned = 0;
        return SFDX_ERR_ARG;
    }
    GraphEntry ge;
    size_t n = 0;
    cudaGraphGetNodes(g, nullptr, &n);
    ge.nodes = (long long)n;
    const cudaError_t ei = cudaGraphInstantiate(&ge.exec, g, 0);
    cudaGraphDestroy(g);
    CK(ei);
    P.graphs.m.emplace(key, ge);
    CK(cudaGraphLaunch(ge.exec, P.st));
    return SFDX_OK;
}

inline int sync_state(Plan& P) {
    if (g_misaligned) {
        g_misaligned = 0;
        return SFDX_ERR_ARG;
    }
    P.hst.resize(P.ns);
    CK(cudaMemcpyAsync(P.hst.data(), P.d_state.p, sizeof(KState) * P.ns, cudaMemcpyDeviceToHost, P.st));
    CK(cudaStreamSynchronize(P.st));
    if (P.rec_on) {
        for (int s = 0; s < P.ns; s++) {
            const KState& Q = P.hst[s];
            if (Q.status == ST_SKIP || !(Q.err > 0)) continue;
            const int full = P.rec_map.empty() ? s : P.rec_map[s];
            const long long gi = (long long)P.rec_off[full] + (Q.it > 0 ? Q.it - 1 : 0);
            if (full < (int)P.rec_off.size() && gi >= 0 && gi < P.rec_len)
                P.rec_hist[(size_t)full * P.rec_len + gi] = Q.err;
        }
    }
    return SFDX_OK;
}

inline RedBuf redbuf(Plan& P) {
    RedBuf r;
    r.part = P.d_part.as<double2>();
    r.counter = P.d_counter.as<unsigned int>();
    return r;
}

// Launch shape of a system-group kernel over the edges of a level (W = nl * G
// work items); `nq` complex partial sums per system for reducing kernels.
struct VCfg {
    int VS, B, grid;
    size_t smem;
    SysG sg;
};
template <class T> inline int plan_vs(const Plan& P) { return vs_pick(P.ns, sizeof(T) == 4 ? P.vs32 : P.vs64); }
inline VCfg vcfg(const Plan& P, int64_t nl, int nq, int VS, int per_sm = 8) {
    VCfg c;
    c.VS = VS;
    c.sg = make_sysg(P.ns, c.VS);
    c.B = vblock(c.sg.G);
    c.grid = grid_for(nl * c.sg.G, c.B, per_sm);
    c.smem = nq > 0 ? vred_smem_bytes(c.B, nq, P.ns) : 0;
    return c;
}

// Reliable-update context of a mixed-precision solve: the FP64 right-hand
// side and solution; the complex64 iteration works on a partial solution.
struct Reliable {
    const double2* b64;
    double2* x64;
    int every;    // iterations between FP64 residual replacements
    double2* xb;  // copy of x64 before the last update (restored on rejection)
};

// ------------------------------------------------------------------ drivers (sfdx_krylov*.cu)
template <class T>
int bicgstab(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
             const int* mask_host, const Reliable* rel = nullptr);
template <class T>
int gpbicg(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
           const int* mask_host, const Reliable* rel = nullptr);
template <class T>
int cocr(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
         const int* mask_host, const Reliable* rel = nullptr);
template <class T>
int tfqmr(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
          const int* mask_host, const Reliable* rel = nullptr);
template <class T>
int bicg(Plan& P, const Level& LV, const cplx<T>* b, cplx<T>* x, const double* tols_host, double tol, int itmax,
         const int* mask_host, const Reliable* rel = nullptr);
// out = M^{-1} q (multi-colour SSOR or Jacobi) for all active systems
template <class T> int precond_vec(Plan& P, const Level& LV, cplx<T>* out, cplx<T>* q);
// y = A x for all systems (per-system frequencies in P.d_wm)
template <class T> int apply_op(Plan& P, const Level& LV, const cplx<T>* x, cplx<T>* y);

// ------------------------------------------------------------------ sfdx_solver.cu
int div_correct(Plan& P, const Level& LV, double2* x);
// FP64 (coarse or FP64 plans) or mixed-precision solve of all systems of level
// LV from the iterate in P.x64 with right-hand side P.b64 (its[], status[]
// per system)
int solve_level(Plan& P, const Level& LV, double tol, int itmax, bool coarse, std::vector<int>& its,
                std::vector<int>& status);
// EXCMG cascade over all levels; rhs(l) writes level l's right-hand side to
// P.b64; the finest solution is left in P.x64 (its[], status[]: finest level)
int excmg_cascade(Plan& P, const std::function<int(int)>& rhs, double eps, bool record, std::vector<int>& its,
                  std::vector<int>& status);
// ||b - A x|| / ||b|| per system in FP64
int true_residual(Plan& P, const Level& LV, const double2* b, const double2* x, double* rel, const int* mask);

// ------------------------------------------------------------------ sfdx_adjoint.cu
// Impedance misfit of the last solution and its gradient with respect to the
// conductivity of every cell and component ([6][ncell], host or device).
int misfit_grad(Plan& P, int nrec, const double* recv, const double* zobs, const double* wts, double tol,
                double* misfit, double* zpred, double* grad, bool grad_on_device, int* adj_iters, double* adj_relres);

// ------------------------------------------------------------------ sfdx_gradcorr.cu
// x += G phi with (G^T V Ms G) phi = G^T V (b - A x) / (-i w mu) for the systems
// with mask[s] != 0 (all when mask is null); nodal PCG to relative tolerance
// `tol`, at most `maxit` iterations (*iters: the most any system took).
int grad_correct(Plan& P, const Level& LV, const double2* b, double2* x, const int* mask, double tol, int maxit,
                 int* iters);
// the nodal operator N = G^T V Ms G of level LV (27-point stencil and its
// inverse diagonal, LV.mg[0]), assembled if the conductivity changed since
int nodal_setup(Plan& P, const Level& LV);

}  // namespace sfdx
