// sfdx_krylov_f32.cu -- complex64 instantiation of the Krylov drivers
// (sfdx_krylov.cuh): the inner iterations of the mixed-precision solve.
#include "sfdx_krylov.cuh"

namespace sfdx {
SFDX_INSTANTIATE_KRYLOV(float)
}  // namespace sfdx
