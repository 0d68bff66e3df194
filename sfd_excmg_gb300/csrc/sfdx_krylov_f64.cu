// sfdx_krylov_f64.cu -- complex128 instantiation of the Krylov drivers
// (sfdx_krylov.cuh): FP64 solves, coarse levels and FP64 finishes.
#include "sfdx_krylov.cuh"

namespace sfdx {
SFDX_INSTANTIATE_KRYLOV(double)
}  // namespace sfdx
