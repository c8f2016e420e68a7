// float64 instantiation of the propagator kernels (pf_mde_impl.cuh) and the dksq grid.
#include "pf_mde_impl.cuh"

namespace pf {
PF_INST(double)

void launch_dksq(double* dk, const CellGeom& g, int nparams, long nk, cudaStream_t st) {
  int blocks = (int)((nk + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  dksq_kernel<<<blocks, 256, 0, st>>>(dk, g, nparams);
  count_launches(1);
}

}  // namespace pf
