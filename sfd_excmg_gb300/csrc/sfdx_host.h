// sfdx_host.h -- declarations shared by the host-side translation units.
#pragma once
#include <complex>
#include <cstddef>

namespace sfdx {

// mt1d_anl restatement (sfdx_host.cpp); conv is Fortran conv(nz,6).
int mt1d_anl(double ff, int nz, const double* conv, const double* c, std::complex<double>* ex,
             std::complex<double>* hx, std::complex<double>* imp);

// The edge planes the impedance evaluation reads, for both polarisations:
//   ex planes m=nair and m+1 (node planes nair+1, nair+2; [2][ny+1][nx]),
//   ey planes m and m+1 ([2][ny][nx+1]), ez layer m ([ny+1][nx+1]).
struct SurfaceView {
    int nx, ny, nair;
    const std::complex<double>* exs[2];
    const std::complex<double>* eys[2];
    const std::complex<double>* ezs[2];
    std::complex<double> ex(int p, int plane, int i, int j) const {
        return exs[p][((size_t)plane * (ny + 1) + j) * nx + i];
    }
    std::complex<double> ey(int p, int plane, int i, int j) const {
        return eys[p][((size_t)plane * ny + j) * (nx + 1) + i];
    }
    std::complex<double> ez(int p, int i, int j) const { return ezs[p][(size_t)j * (nx + 1) + i]; }
};

// Writable edge planes of the same shape (adjoint sources), both polarisations.
struct SurfaceGrad {
    int nx, ny;
    std::complex<double>* exs[2];
    std::complex<double>* eys[2];
    std::complex<double>* ezs[2];
    std::complex<double>& ex(int p, int plane, int i, int j) { return exs[p][((size_t)plane * (ny + 1) + j) * nx + i]; }
    std::complex<double>& ey(int p, int plane, int i, int j) { return eys[p][((size_t)plane * ny + j) * (nx + 1) + i]; }
    std::complex<double>& ez(int p, int i, int j) { return ezs[p][(size_t)j * (nx + 1) + i]; }
};

// fields (optional): [nrec][2][5] complex, (Ex, Ey, Hx, Hy, Hz) of each
// polarisation interpolated to the receiver (the arho rows of post_process).
// The 3x3 receiver stencils of arho_interp2 (rd=2, fdfe_main.f90:718-790) for
// the device evaluation: per receiver r, id[9r..9r+8] are the surface cells
// [j*nx+i] of E, Hx and Hy (transposed with `transpose`), idz[] those of Hz,
// w[] their weights.  SFDX_ERR_RECEIVER for a receiver outside the
// interpolable area.
int receiver_stencils(int nx, int ny, const double* a, const double* b, int nrec, const double* recv, int transpose,
                      int* id, int* idz, double* w);

int impedance_from_surface(const SurfaceView& sv, const double* a, const double* b, const double* c, double ff,
                           int nrec, const double* recv, int out_type, int transpose, double* out, double* tip,
                           std::complex<double>* fields = nullptr);

// Impedance misfit of one frequency (added to *misfit), the predicted Z
// (optional, [nrec][4]) and its derivative with respect to the receiver fields,
// cf [nrec][2 polarisations][Ex, Ey, Hx, Hy].  zobs [nrec][4] = (Re, Im Zxy,
// Re, Im Zyx); wts [nrec][2] (null: 1).
// receiver plane per surface column with topography and the impedances formed
// there (post_process, fdfe_main.f90:604-616); sfdx_host.cpp
int receiver_planes(int nx, int ny, int nz, int nair, const double* c, const int* abr, const double* topo,
                    int reference, int* mcol, double* czcol);
int impedance_topo(const std::complex<double>* x1, const std::complex<double>* x2, int nx, int ny, int nz,
                   const int* mcol, const double* czcol, const double* a, const double* b, double ff, int nrec,
                   const double* recv, int out_type, int transpose, double* out, double* tip);
int impedance_cotangents(const SurfaceView& sv, const double* a, const double* b, const double* c, double ff,
                         int nrec, const double* recv, int transpose, const double* zobs, const double* wts,
                         double* misfit, double* zpred, std::complex<double>* cf);
// d misfit / d (surface edge values) of a mesh from those cotangents,
// accumulated into g (the adjoint source on that mesh's receiver planes).
int impedance_adjoint_source(SurfaceGrad& g, int nair, const double* a, const double* b, const double* c, double ff,
                             int nrec, const double* recv, int transpose, const std::complex<double>* cf);

}  // namespace sfdx
