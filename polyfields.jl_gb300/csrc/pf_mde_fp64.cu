// float64 instantiation of the propagator kernels (pf_mde_impl.cuh) and the dksq grid.
#include <cmath>

#include "pf_mde_impl.cuh"

namespace pf {
PF_INST(double)

void launch_dksq(double* dk, const CellGeom& g, int nparams, long nk, cudaStream_t st) {
  int blocks = (int)((nk + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  dksq_kernel<<<blocks, 256, 0, st>>>(dk, g, nparams);
  count_launches(1);
}

// Weights of the bond-operator gradient of one block (rows j < nparams: cell parameter j,
// row nparams: the block's ds) on the half spectrum:
//   LD_k = exp(-ds b^2 ksq_k / 6) * scale,  wts[j][k] = LD_k * (-ds b^2 / 6) * dksq_j,k,
//   wts[nparams][k] = LD_k * (-b^2 / 6) * ksq_k.
static __global__ void adj_weights_kernel(double* __restrict__ wts, CellGeom g, int nparams, double ds, double b,
                                          double scale) {
  const long nk = (long)(g.nx / 2 + 1) * g.ny * g.nz;
  const double b2 = b * b;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nk; i += (long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    spectral_index(g, i, ix, iy, iz);
    const double ksq = ksq_at(g, ix, iy, iz);
    const double ld = exp(-ds * b2 * ksq / 6.0) * scale;
    const double j[3] = {(double)ix, fold_index(g, iy, g.ny), fold_index(g, iz, g.nz)};
    for (int p = 0; p < nparams; ++p) {
      double acc = 0.0;
      for (int l = 0; l < g.dim; ++l)
        for (int m = 0; m < g.dim; ++m) acc += j[l] * j[m] * g.dGG[(l * 3 + m) * kMaxParams + p];
      wts[p * nk + i] = ld * (-ds * b2 / 6.0) * acc;
    }
    wts[nparams * nk + i] = ld * (-b2 / 6.0) * ksq;
  }
}

void launch_adj_weights(double* wts, const CellGeom& g, int nparams, double ds, double b, double scale, long nk,
                        cudaStream_t st) {
  int blocks = (int)((nk + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  adj_weights_kernel<<<blocks, 256, 0, st>>>(wts, g, nparams, ds, b, scale);
  count_launches(1);
}

namespace {
template <int N>
int twiddle_table_n(double* re, double* im, int max_entries) {
  int n = 0;
  for (int o = 0; o < 2; ++o) {
    const int P = Plan<N>::P;
    int span = 1;
    for (int p = 0; p < P; ++p) {
      const int R = o == 0 ? Plan<N>::ra(p) : Plan<N>::ra(P - 1 - p);
      const long L = (long)span * R;
      for (int t = 1; t < R; ++t)
        for (int k = 0; k < span; ++k) {
          if (n >= max_entries) return -1;
          const long m = ((long)t * k) % L;
          const long double a = -2.0L * 3.141592653589793238462643383279502884L * (long double)m / (long double)L;
          re[n] = (double)cosl(a);
          im[n] = (double)sinl(a);
          ++n;
        }
      span *= R;
    }
  }
  return n;
}
}  // namespace

int fft_twiddle_table(int n, double* re, double* im, int max_entries) {
  switch (n) {
    case 1: return 0;
#define PF_TW(N) \
  case N:        \
    return twiddle_table_n<N>(re, im, max_entries);
    PF_Z_LENGTHS(PF_TW)
#undef PF_TW
    default:
      return -1;
  }
}

}  // namespace pf
