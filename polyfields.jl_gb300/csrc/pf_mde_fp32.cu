// float32 instantiation of the propagator kernels (pf_mde_impl.cuh).
#include "pf_mde_impl.cuh"

namespace pf {
PF_INST(float)
}  // namespace pf
