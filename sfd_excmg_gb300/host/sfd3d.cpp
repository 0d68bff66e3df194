// sfd3d.cpp -- drop-in host for `./sfd3d <model> [level eps]`
// (sfd_excmg/src/sfd_excmg.f90:20-58): read <model>.fwd/.dat(/.topo), run the
// forward solve on the GPU through the C ABI, write <model>.res.
//
// Options beyond the reference's argv come from the environment:
//   SFDX_EXCMG=0|1 (fwd_acc, default 0 as in global_para.f90:19),
//   SFDX_PRECISION=fp64|mixed, SFDX_VERBOSE=1, SFDX_TIPPER=1 (output_tipper:
//   the tippers follow the impedances in <model>.res), SFDX_DIV_COR=0|1|2
//   (div_cor, default 1), SFDX_PRECOND=S|J|G (pre_type, default S; G the edge
//   multigrid), SFDX_CCV=1 (output_ccv: the finest-level residual history of
//   every solve in <model>_<freq>_<polar>_<solver|excmg>.ccv).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sfdx.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <model> [level eps]\n", argv[0]);
        return 2;
    }
    const char* name = argv[1];
    int nx, ny, nz, nair, nf, nrec;
    int rc = sfdx_read_sizes(name, &nx, &ny, &nz, &nair, &nf, &nrec);
    if (rc) {
        fprintf(stderr, "sfd3d: %s\n", sfdx_strerror(rc));
        return 1;
    }
    sfdx_opts o;
    sfdx_default_opts(&o);
    const size_t ncell = (size_t)nx * ny * nz;
    std::vector<double> a(nx), b(ny), c(nz), sigma(6 * ncell), freq(nf), recv(3 * (size_t)nrec);
    int level, solver, out_type, abu[6];
    double eps;
    rc = sfdx_read_model(name, &o, &level, &eps, &solver, &out_type, a.data(), b.data(), c.data(), sigma.data(),
                         freq.data(), recv.data(), abu);
    if (rc) {
        fprintf(stderr, "sfd3d: %s\n", sfdx_strerror(rc));
        return 1;
    }
    if (argc > 3) {  // argv override of level and eps (sfd_excmg.f90:45-50)
        level = atoi(argv[2]);
        eps = atof(argv[3]);
    }
    o.level = level;
    o.eps = eps;
    o.solver = solver;
    if (const char* e = getenv("SFDX_EXCMG")) o.excmg = atoi(e);
    if (const char* p = getenv("SFDX_PRECISION")) o.precision = strcmp(p, "mixed") == 0 ? SFDX_MIXED : SFDX_FP64;
    if (getenv("SFDX_VERBOSE")) o.verbose = 1;
    if (const char* d = getenv("SFDX_DIV_COR")) {
        o.div_cor = atoi(d);
        if (o.div_cor == 2) {  // the consistent correction's cycle length and nodal tolerance
            o.corr_intv = 40;
            o.corr_tol = 1e-2;
        }
    }
    if (const char* p = getenv("SFDX_PRECOND")) o.precond = p[0];
    const long long nl = (long long)nx * (ny + 1) * (nz + 1) + (long long)(nx + 1) * ny * (nz + 1) +
                         (long long)(nx + 1) * (ny + 1) * nz;
    std::vector<double> ex((size_t)nf * 2 * nl * 2);
    std::vector<double> relres((size_t)nf * 2);
    const char* ccv = getenv("SFDX_CCV");
    if (ccv && atoi(ccv)) {
        // the plan keeps the histories that the one-shot call discards
        sfdx_plan* plan = nullptr;
        rc = sfdx_plan_create(&plan, &o, nx, ny, nz, nair, a.data(), b.data(), c.data(), nf, freq.data());
        const int nlev = o.excmg ? o.level : 1;
        std::vector<int> its((size_t)nf * 2 * nlev);
        if (rc == SFDX_OK) rc = sfdx_plan_solve(plan, sigma.data(), 0, ex.data(), 0, its.data(), relres.data());
        if (rc == SFDX_OK || rc == SFDX_ERR_NOCONV) {
            const int maxit = o.excmg ? o.maxit_level : o.maxit_plain;
            std::vector<double> hist((size_t)nf * 2 * maxit);
            const int hrc = sfdx_plan_history(plan, hist.data(), maxit);
            static const char* names[7] = {"", "bicgstab", "tfqmr", "gpbicg", "bicg", "", "cocr"};
            const char* tag = o.excmg ? "excmg" : (o.solver >= 0 && o.solver < 7 ? names[o.solver] : "");
            for (int f = 0; f < nf && hrc == SFDX_OK; f++)
                for (int p = 0; p < 2; p++) {
                    const double* h = hist.data() + (size_t)(2 * f + p) * maxit;
                    const int n_it = its[(size_t)(2 * f + p) * nlev + nlev - 1];  // iters(1) of the finest level
                    if (sfdx_write_ccv(name, freq[f], p ? "yx" : "xy", tag, n_it, h, maxit) != SFDX_OK)
                        fprintf(stderr, "sfd3d: cannot write the .ccv file\n");
                }
        }
        sfdx_plan_destroy(plan);
    } else {
        rc = sfdx_fwd_solve(&o, nx, ny, nz, nair, a.data(), b.data(), c.data(), sigma.data(), nf, freq.data(),
                            ex.data(), nullptr, relres.data());
    }
    if (rc && rc != SFDX_ERR_NOCONV) {
        fprintf(stderr, "sfd3d: %s\n", sfdx_strerror(rc));
        return 1;
    }
    if (rc == SFDX_ERR_NOCONV) fprintf(stderr, "sfd3d: warning: %s\n", sfdx_strerror(rc));
    std::vector<double> res((size_t)nf * nrec * 4);
    // output_tipper (global_para.f90:7, off by default): the tipper block follows
    const char* te = getenv("SFDX_TIPPER");
    std::vector<double> tip(te && atoi(te) ? (size_t)nf * nrec * 4 : 0);
    rc = sfdx_impedance(nx, ny, nz, nair, a.data(), b.data(), c.data(), nf, freq.data(), ex.data(), nrec, recv.data(),
                        out_type, o.quirks, res.data(), tip.empty() ? nullptr : tip.data());
    if (rc) {
        fprintf(stderr, "sfd3d: %s\n", sfdx_strerror(rc));
        return 1;
    }
    rc = sfdx_write_res_tipper(name, nf, freq.data(), nrec, recv.data(), res.data(), tip.empty() ? nullptr : tip.data());
    if (rc) {
        fprintf(stderr, "sfd3d: %s\n", sfdx_strerror(rc));
        return 1;
    }
    return 0;
}
