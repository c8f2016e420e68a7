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
