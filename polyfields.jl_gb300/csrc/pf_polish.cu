// Float64 vector primitives of the Newton-Krylov polish (pf_engine.cu, System::nk_polish): the
// Gram-Schmidt products and updates of a restarted GMRES over field-sized vectors.  Krylov
// vectors are stored back to back, V_i = V + i n.  Every reduction is deterministic: per-block
// partial sums in a fixed grid-stride order, then one fixed-order sum per output.
#include "pf_kernels.h"

namespace pf {
namespace {

constexpr int kPolishBlocks = 304;  // two blocks per SM of a 152-SM GB300
constexpr int kChunk = 8;           // Krylov vectors per pass over z

template <int K>
__global__ void __launch_bounds__(256) multidot_kernel(const double* __restrict__ V, long n,
                                                      const double* __restrict__ z, double* __restrict__ part) {
  __shared__ double red[32];
  double acc[K];
#pragma unroll
  for (int i = 0; i < K; ++i) acc[i] = 0.0;
  for (long x = blockIdx.x * (long)blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x) {
    const double zv = z[x];
#pragma unroll
    for (int i = 0; i < K; ++i) acc[i] += V[(long)i * n + x] * zv;
  }
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const double s = block_sum(acc[i], red);
    if (threadIdx.x == 0) part[(long)blockIdx.x * K + i] = s;
  }
}

// out[i] = sum over the blocks of part[b * K + i], in block order
__global__ void dot_final_kernel(const double* __restrict__ part, int nb, int K, double* __restrict__ out) {
  const int i = threadIdx.x;
  if (i >= K) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[(long)b * K + i];
  out[i] = s;
}

// z = alpha z + beta sum_i c[i] V_i  (c on the device)
template <int K>
__global__ void multiaxpy_kernel(double* __restrict__ z, const double* __restrict__ V, long n,
                                 const double* __restrict__ c, double alpha, double beta) {
  double cc[K];
#pragma unroll
  for (int i = 0; i < K; ++i) cc[i] = c[i];
  for (long x = blockIdx.x * (long)blockDim.x + threadIdx.x; x < n; x += (long)gridDim.x * blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < K; ++i) s += cc[i] * V[(long)i * n + x];
    z[x] = alpha * z[x] + beta * s;
  }
}

// y = a y + b x
__global__ void lincomb_kernel(double* __restrict__ y, const double* __restrict__ x, double a, double b, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = a * y[i] + b * x[i];
}

template <int K>
void multidot_chunk(const double* V, long n, const double* z, double* part, double* out, cudaStream_t st) {
  multidot_kernel<K><<<kPolishBlocks, 256, 0, st>>>(V, n, z, part);
  dot_final_kernel<<<1, 32, 0, st>>>(part, kPolishBlocks, K, out);
  count_launches(2);
}

template <int K>
void multiaxpy_chunk(double* z, const double* V, long n, const double* c, double alpha, double beta,
                     cudaStream_t st) {
  multiaxpy_kernel<K><<<kPolishBlocks * 2, 256, 0, st>>>(z, V, n, c, alpha, beta);
  count_launches(1);
}

}  // namespace

void launch_multidot(const double* V, int k, long n, const double* z, double* part, double* out, cudaStream_t st) {
  for (int i0 = 0; i0 < k; i0 += kChunk) {
    const int c = k - i0 < kChunk ? k - i0 : kChunk;
    const double* v = V + (long)i0 * n;
    switch (c) {
      case 1: multidot_chunk<1>(v, n, z, part, out + i0, st); break;
      case 2: multidot_chunk<2>(v, n, z, part, out + i0, st); break;
      case 3: multidot_chunk<3>(v, n, z, part, out + i0, st); break;
      case 4: multidot_chunk<4>(v, n, z, part, out + i0, st); break;
      case 5: multidot_chunk<5>(v, n, z, part, out + i0, st); break;
      case 6: multidot_chunk<6>(v, n, z, part, out + i0, st); break;
      case 7: multidot_chunk<7>(v, n, z, part, out + i0, st); break;
      default: multidot_chunk<8>(v, n, z, part, out + i0, st); break;
    }
  }
}

void launch_multiaxpy(double* z, const double* V, int k, long n, const double* c, double alpha, double beta,
                      cudaStream_t st) {
  for (int i0 = 0; i0 < k; i0 += kChunk) {
    const int m = k - i0 < kChunk ? k - i0 : kChunk;
    const double* v = V + (long)i0 * n;
    const double a = i0 == 0 ? alpha : 1.0;  // the first chunk scales z, later ones accumulate
    switch (m) {
      case 1: multiaxpy_chunk<1>(z, v, n, c + i0, a, beta, st); break;
      case 2: multiaxpy_chunk<2>(z, v, n, c + i0, a, beta, st); break;
      case 3: multiaxpy_chunk<3>(z, v, n, c + i0, a, beta, st); break;
      case 4: multiaxpy_chunk<4>(z, v, n, c + i0, a, beta, st); break;
      case 5: multiaxpy_chunk<5>(z, v, n, c + i0, a, beta, st); break;
      case 6: multiaxpy_chunk<6>(z, v, n, c + i0, a, beta, st); break;
      case 7: multiaxpy_chunk<7>(z, v, n, c + i0, a, beta, st); break;
      default: multiaxpy_chunk<8>(z, v, n, c + i0, a, beta, st); break;
    }
  }
}

void launch_lincomb(double* y, const double* x, double a, double b, long n, cudaStream_t st) {
  lincomb_kernel<<<kPolishBlocks * 2, 256, 0, st>>>(y, x, a, b, n);
  count_launches(1);
}

int polish_part_doubles() { return kPolishBlocks * kChunk; }

}  // namespace pf
