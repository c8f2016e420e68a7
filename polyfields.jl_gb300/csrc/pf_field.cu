// Density integration, field residuals, reductions and Anderson mixing kernels.
//
// Reference functions: Simpson density (src/species/multiblock.jl:175-228), point species
// (src/species/point.jl:36-53), potentials / incompressibility / residuals with mean
// subtraction (src/system/system.jl:296-340, src/interactions/flory.jl:82-100,
// src/system/compress.jl:37-61), free energy and field error (system.jl:402-486) and the
// Anderson Gram matrix, solve and mixed update (src/updaters/anderson.jl:147-205).
//
// All system-level grids are FP64: fields w, potentials, residuals and densities are
// nmon consecutive grids of Ng.  Sums over the grid are deterministic: each CTA writes a
// partial, a second kernel adds the partials in a fixed order.
#include <atomic>

#include "pf_kernels.h"

namespace pf {

static std::atomic<long> g_launches{0};
void count_launches(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long launch_total() { return g_launches.load(std::memory_order_relaxed); }

static int red_blocks(long n) {
  long b = (n + 255) / 256;
  if (b > kRedBlocks) b = kRedBlocks;
  if (b < 1) b = 1;
  return (int)b;
}

// out[v] = (sum_b part[b * nval + v]) / div
__global__ void reduce_parts_kernel(const double* __restrict__ part, int nblk, int nval, double* __restrict__ out,
                                    double div) {
  __shared__ double red[32];
  const int v = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[(long)b * nval + v];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) out[v] = acc / div;
}

static void reduce_parts(const double* part, int nblk, int nval, double* out, double div, cudaStream_t st) {
  reduce_parts_kernel<<<nval, 256, 0, st>>>(part, nblk, nval, out, div);
  count_launches(1);
}

// ------------------------------------------------------------------ plain sums
template <typename T>
__global__ void sum_kernel(const T* __restrict__ a, long n, double* __restrict__ part) {
  __shared__ double red[32];
  double acc = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    acc += (double)a[i];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

template <typename T>
void launch_sum(const T* a, long n, double* part, double* out, double div, cudaStream_t st) {
  const int nb = red_blocks(n);
  sum_kernel<T><<<nb, 256, 0, st>>>(a, n, part);
  count_launches(1);
  reduce_parts(part, nb, 1, out, div, st);
}
template void launch_sum<float>(const float*, long, double*, double*, double, cudaStream_t);
template void launch_sum<double>(const double*, long, double*, double*, double, cudaStream_t);

// ------------------------------------------------------------------ point species
__global__ void point_q_kernel(const double* __restrict__ w, double vol, long n, double* __restrict__ part) {
  __shared__ double red[32];
  double acc = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    acc += exp(-vol * w[i]);
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

void launch_point_q(const double* w, double vol, long n, double* part, double* Qdev, cudaStream_t st) {
  const int nb = red_blocks(n);
  point_q_kernel<<<nb, 256, 0, st>>>(w, vol, n, part);
  count_launches(1);
  reduce_parts(part, nb, 1, Qdev, (double)n, st);
}

__global__ void point_density_kernel(double* __restrict__ rho, const double* __restrict__ w, double vol, double phi,
                                     const double* __restrict__ Qdev, long n) {
  const double Q = *Qdev;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    rho[i] += phi * (exp(-vol * w[i]) / Q);
}

void launch_point_density(double* rho, const double* w, double vol, double phi, const double* Qdev, long n,
                          cudaStream_t st) {
  point_density_kernel<<<red_blocks(n), 256, 0, st>>>(rho, w, vol, phi, Qdev, n);
  count_launches(1);
}

// ------------------------------------------------------------------ Simpson density
// rho_all[mon*ng + i] += phi * sum_{blocks of mon} (ds/3) * S_blk(i) / (Q * Nref), with
// S_blk = q_b qc_b + q_e qc_e + 4 sum_odd q qc + 2 sum_even q qc in the reference's order.
// Each thread integrates W consecutive grid points (one 16-byte vector of T per contour
// point and chain), keeping the reference's summation order per point; the s loops are
// unrolled so several vector loads are in flight per thread.
template <typename T>
struct Vec;
template <>
struct Vec<float> {
  __device__ static float get(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
};
template <>
struct Vec<double> {
  __device__ static double get(const double2& v, int k) { return k == 0 ? v.x : v.y; }
};

template <typename T>
struct SimpVec;
template <>
struct SimpVec<float> {
  using V = float4;
  static constexpr int W = 4;
  __device__ static void unpack(const V& v, double* o) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
};
template <>
struct SimpVec<double> {
  using V = double2;
  static constexpr int W = 2;
  __device__ static void unpack(const V& v, double* o) {
    o[0] = v.x;
    o[1] = v.y;
  }
};

// Accumulator of one Simpson sum: float64 for float64 histories (the reference's arithmetic);
// for float32 histories a compensated (Kahan) float32 sum, converted to float64 once per
// block -- GB300 runs float64 at 1/57 of the float32 rate, so per-term float64 work would
// dominate this memory-bound pass.
template <typename T>
struct SimpAcc {
  double s;
  __device__ void init(double v) { s = v; }
  __device__ void add(double v) { s += v; }
  __device__ double value() const { return s; }
};
template <>
struct SimpAcc<float> {
  float s, c;
  __device__ void init(float v) {
    s = v;
    c = 0.f;
  }
  __device__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ double value() const { return (double)s - (double)c; }
};

template <typename T>
__global__ void __launch_bounds__(256) simpson_kernel(double* __restrict__ rho_all, const T* __restrict__ q,
                                                      const T* __restrict__ qc, bool rev, int Ns, long ng,
                                                      SimpsonBlocks blk, double phi, double Nref,
                                                      const double* __restrict__ Qdev, const double* __restrict__ fac) {
  using SV = SimpVec<T>;
  using V = typename SV::V;
  constexpr int W = SV::W;
  const double QN = fac ? Nref : (*Qdev) * Nref;
  const long nv = ng / W;
  const V* q4 = reinterpret_cast<const V*>(q);
  const V* qc4 = reinterpret_cast<const V*>(rev ? q : qc);
  const bool sym = rev && blk.nblocks == 1 && blk.bgn[0] == 0 && blk.end[0] == Ns && Ns % 2 == 0 && Ns >= 2;
  for (long iv = blockIdx.x * (long)blockDim.x + threadIdx.x; iv < nv; iv += (long)gridDim.x * blockDim.x) {
    double bval[kMaxMon * 2][W];
    for (int b = 0; b < blk.nblocks; ++b) {
      const int s0 = blk.bgn[b], s1 = blk.end[b];
      SimpAcc<T> acc[W];
      auto term = [&](int s, T wgt, bool first) {
        const long sc = rev ? (long)(Ns - s) : (long)s;
        const V a = q4[(long)s * nv + iv];
        const V c = qc4[sc * nv + iv];
        const T f = fac ? (T)fac[s] : (T)1;
#pragma unroll
        for (int k = 0; k < W; ++k) {
          const T ak = Vec<T>::get(a, k), ck = Vec<T>::get(c, k);
          const T v = wgt == (T)1 ? (ak * f) * ck : wgt * (ak * f) * ck;
          if (first) acc[k].init(v);
          else acc[k].add(v);
        }
      };
      if (sym) {
        // symmetric chain in one block: the integrand at s and Ns - s is the same product
        // (fac is symmetric too), so each mirrored pair is read once and counted twice
        const int h = Ns / 2;
        term(0, (T)2, true);
#pragma unroll 4
        for (int s = 1; s < h; s += 2) term(s, (T)8, false);
#pragma unroll 4
        for (int s = 2; s < h; s += 2) term(s, (T)4, false);
        term(h, (h & 1) ? (T)4 : (T)2, false);
      } else {
        term(s0, (T)1, true);
        term(s1, (T)1, false);
#pragma unroll 4
        for (int s = s0 + 1; s < s1; s += 2) term(s, (T)4, false);
#pragma unroll 4
        for (int s = s0 + 2; s < s1 - 1; s += 2) term(s, (T)2, false);
      }
#pragma unroll
      for (int k = 0; k < W; ++k) bval[b][k] = (acc[k].value() * (blk.ds[b] / 3.0)) / QN;
    }
    // pool blocks by monomer (block order), then add phi * species density
    unsigned done = 0;
    for (int b = 0; b < blk.nblocks; ++b) {
      const int m = blk.mon[b];
      if (done & (1u << m)) continue;
      done |= 1u << m;
#pragma unroll
      for (int k = 0; k < W; ++k) {
        double dens = 0.0;
        for (int c = b; c < blk.nblocks; ++c)
          if (blk.mon[c] == m) dens += bval[c][k];
        rho_all[(long)m * ng + iv * W + k] += phi * dens;
      }
    }
  }
}

template <typename T>
void launch_simpson(double* rho_all, const T* q, const T* qc, bool qc_reversed, int Ns, long ng,
                    const SimpsonBlocks& blk, double phi, double Nref, const double* Qdev, const double* fac,
                    cudaStream_t st) {
  const long nv = ng / SimpVec<T>::W;
  int nb = (int)((nv + 255) / 256);
  if (nb > 8192) nb = 8192;
  simpson_kernel<T><<<nb, 256, 0, st>>>(rho_all, q, qc, qc_reversed, Ns, ng, blk, phi, Nref, Qdev, fac);
  count_launches(1);
}
template void launch_simpson<float>(double*, const float*, const float*, bool, int, long, const SimpsonBlocks&,
                                    double, double, const double*, const double*, cudaStream_t);
template void launch_simpson<double>(double*, const double*, const double*, bool, int, long, const SimpsonBlocks&,
                                     double, double, const double*, const double*, cudaStream_t);

__global__ void scale_finalize_kernel(const double* __restrict__ lf, const double* __restrict__ lb, bool rev, int Ns,
                                      const double* __restrict__ meanq, double* __restrict__ Qdev,
                                      double* __restrict__ fac, double qpow) {
  extern __shared__ double Lsh[];  // forward prefix L_s, s = 0..Ns, then backward L'_s
  double* Lf = Lsh;
  double* Lb = Lsh + (Ns + 1);
  if (threadIdx.x == 0) {
    Lf[0] = 0.0;
    for (int t = 0; t < Ns; ++t) Lf[t + 1] = Lf[t] + lf[t];
    if (rev) {
      for (int s = 0; s <= Ns; ++s) Lb[s] = Lf[Ns - s];
    } else {
      Lb[Ns] = 0.0;
      for (int t = 0; t < Ns; ++t) Lb[Ns - t - 1] = Lb[Ns - t] + lb[t];
    }
    const double logQ = log(*meanq) - Lf[Ns];
    *Qdev = exp(logQ);
    Lsh[2 * (Ns + 1)] = logQ;
  }
  __syncthreads();
  const double logQ = Lsh[2 * (Ns + 1)];
  for (int s = threadIdx.x; s <= Ns; s += blockDim.x) fac[s] = exp(-Lf[s] - Lb[s] - qpow * logQ);
}

void launch_scale_finalize(const double* lsc_fwd, const double* lsc_bwd, bool rev, int Ns, const double* meanq,
                           double* Qdev, double* fac, cudaStream_t st, bool divide_q) {
  const size_t smem = sizeof(double) * (2 * (size_t)(Ns + 1) + 1);
  if (smem > 48 * 1024) cudaFuncSetAttribute(scale_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  scale_finalize_kernel<<<1, 256, smem, st>>>(lsc_fwd, lsc_bwd, rev, Ns, meanq, Qdev, fac, divide_q ? 1.0 : 0.0);
  count_launches(1);
}

// ------------------------------------------------------------------ residuals
// pot_a = sum_b chi_ab rho_b / v_b ; eta = (sum rho - 1 + sum_a (w_a - pot_a)) / nmon ;
// res_a = pot_a + eta - w_a.  Partials: sum w_a (v = a), sum res_a (v = nmon + a).
// NM = the monomer count (compile-time, so the per-point arrays stay in registers).
template <int NM>
__global__ void residual_kernel(const double* __restrict__ w, double* __restrict__ pot, double* __restrict__ res,
                                const double* __restrict__ rho, MonomerSet ms, long ng, double* __restrict__ part) {
  __shared__ double red[2 * kMaxMon][32];
  constexpr int nm = NM;
  double sw[kMaxMon], sr[kMaxMon], ivol[kMaxMon];
  for (int a = 0; a < kMaxMon; ++a) sw[a] = sr[a] = 0.0;
  // per-thread reciprocals: a float64 division is a long FP64 instruction sequence, and the
  // grid loop would otherwise run nm^2 + 1 of them per point (identical results for the
  // usual unit volumes and a power-of-two monomer count)
  for (int a = 0; a < nm; ++a) ivol[a] = 1.0 / ms.vol[a];
  const double inm = 1.0 / (double)nm;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ng; i += (long)gridDim.x * blockDim.x) {
    double r[kMaxMon], wv[kMaxMon], p[kMaxMon];
    double rhosum = 0.0;
    for (int a = 0; a < nm; ++a) {
      r[a] = rho[(long)a * ng + i];
      wv[a] = w[(long)a * ng + i];
      rhosum += r[a];
    }
    double eta = rhosum - 1.0;
    for (int a = 0; a < nm; ++a) {
      double pa = 0.0;
      for (int b = 0; b < nm; ++b) {
        const double c = ms.chi[a * kMaxMon + b];
        if (c != 0.0) pa += c * (r[b] * ivol[b]);
      }
      p[a] = pa;
      eta += wv[a] - pa;
    }
    eta *= inm;
    for (int a = 0; a < nm; ++a) {
      const double ra = p[a] + eta - wv[a];
      pot[(long)a * ng + i] = p[a];
      res[(long)a * ng + i] = ra;
      sw[a] += wv[a];
      sr[a] += ra;
    }
  }
  for (int a = 0; a < nm; ++a) {
    double v1 = block_sum(sw[a], red[a]);
    double v2 = block_sum(sr[a], red[kMaxMon + a]);
    if (threadIdx.x == 0) {
      part[(long)blockIdx.x * 2 * nm + a] = v1;
      part[(long)blockIdx.x * 2 * nm + nm + a] = v2;
    }
  }
}

// w_a -= mean(w_a); res_a -= mean(res_a)  (means[a], means[nm + a])
__global__ void meansub_kernel(double* __restrict__ w, double* __restrict__ res, const double* __restrict__ means,
                               int nm, long ng) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ng; i += (long)gridDim.x * blockDim.x) {
    for (int a = 0; a < nm; ++a) {
      w[(long)a * ng + i] -= means[a];
      res[(long)a * ng + i] -= means[nm + a];
    }
  }
}

int launch_residuals(double* w, double* pot, double* res, const double* rho, const MonomerSet& ms, long ng,
                     bool canonical, double* part, double* sums, cudaStream_t st) {
  const int nb = red_blocks(ng);
  switch (ms.nmon) {
#define PF_RES(N)                                                          \
  case N:                                                                  \
    residual_kernel<N><<<nb, 256, 0, st>>>(w, pot, res, rho, ms, ng, part); \
    break;
    PF_RES(1) PF_RES(2) PF_RES(3) PF_RES(4) PF_RES(5) PF_RES(6) PF_RES(7) PF_RES(8)
#undef PF_RES
    default:
      return E_ARG;
  }
  count_launches(1);
  if (canonical) {
    reduce_parts(part, nb, 2 * ms.nmon, sums, (double)ng, st);
    meansub_kernel<<<nb, 256, 0, st>>>(w, res, sums, ms.nmon, ng);
  count_launches(1);
  }
  return OK;
}

// ------------------------------------------------------------------ field error / energy sums
// out4 = { sum res^2, sum w^2, sum rho*w, sum_pairs chi (rho_a/v_a)(rho_b/v_b) }
__global__ void stats_kernel(const double* __restrict__ w, const double* __restrict__ res,
                             const double* __restrict__ rho, MonomerSet ms, long ng, double* __restrict__ part) {
  __shared__ double red[4][32];
  const int nm = ms.nmon;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ng; i += (long)gridDim.x * blockDim.x) {
    for (int a = 0; a < nm; ++a) {
      const double ra = res[(long)a * ng + i], wa = w[(long)a * ng + i], da = rho[(long)a * ng + i];
      s0 += ra * ra;
      s1 += wa * wa;
      s2 += da * wa;
      for (int b = a + 1; b < nm; ++b) {
        const double c = ms.chi[a * kMaxMon + b];
        if (c != 0.0) s3 += c * (da / ms.vol[a]) * (rho[(long)b * ng + i] / ms.vol[b]);
      }
      const double u = ms.chi[a * kMaxMon + a];  // Edwards: (u/2) (rho_a / v_a)^2
      if (u != 0.0) s3 += 0.5 * u * (da / ms.vol[a]) * (da / ms.vol[a]);
    }
  }
  s0 = block_sum(s0, red[0]);
  s1 = block_sum(s1, red[1]);
  s2 = block_sum(s2, red[2]);
  s3 = block_sum(s3, red[3]);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 4 + 0] = s0;
    part[blockIdx.x * 4 + 1] = s1;
    part[blockIdx.x * 4 + 2] = s2;
    part[blockIdx.x * 4 + 3] = s3;
  }
}

void launch_stats(const double* w, const double* res, const double* rho, const MonomerSet& ms, long ng,
                  double* part, double* out4, cudaStream_t st) {
  const int nb = red_blocks(ng);
  stats_kernel<<<nb, 256, 0, st>>>(w, res, rho, ms, ng, part);
  count_launches(1);
  reduce_parts(part, nb, 4, out4, 1.0, st);
}

// ------------------------------------------------------------------ Anderson mixing
__global__ void axpy_kernel(double* __restrict__ y, const double* __restrict__ x, double a, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = y[i] + a * x[i];
}

void launch_axpy(double* y, const double* x, double a, long n, cudaStream_t st) {
  int nb = (int)((n + 255) / 256);
  if (nb > 8192) nb = 8192;
  axpy_kernel<<<nb, 256, 0, st>>>(y, x, a, n);
  count_launches(1);
}

// Gram sums over all monomer grids (n_all = nmon * Ng): with r = res[ih] and d_m = r - res[ih-m],
// U[m][n] = sum d_m d_n (m <= n, packed row-major upper triangle) and V[m] = sum d_m r.
constexpr int kGramTile = 64;
__global__ void __launch_bounds__(256) gram_kernel(HistPtrs h, int ih, long n, double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* D = reinterpret_cast<double*>(smem_raw);  // [ih][kGramTile]
  double* R = D + ih * kGramTile;                   // [kGramTile]
  const int npair = ih * (ih + 1) / 2;
  const int nout = npair + ih;
  constexpr int kMaxOwn = 8;
  double acc[kMaxOwn];
  int om[kMaxOwn], on[kMaxOwn];
  for (int j = 0; j < kMaxOwn; ++j) {
    acc[j] = 0.0;
    const int o = threadIdx.x + j * blockDim.x;
    om[j] = -1;
    on[j] = -1;
    if (o < npair) {
      int m = 0, rem = o;
      while (rem >= ih - m) {
        rem -= ih - m;
        ++m;
      }
      om[j] = m;
      on[j] = m + rem;
    } else if (o < nout) {
      om[j] = o - npair;
      on[j] = -2;  // V entry
    }
  }
  const double* r = h.res[ih];
  for (long t0 = (long)blockIdx.x * kGramTile; t0 < n; t0 += (long)gridDim.x * kGramTile) {
    for (int idx = threadIdx.x; idx < kGramTile * (ih + 1); idx += blockDim.x) {
      const int p = idx % kGramTile, m = idx / kGramTile;
      const long i = t0 + p;
      const double rv = (i < n) ? r[i] : 0.0;
      if (m == ih) R[p] = rv;
      else D[m * kGramTile + p] = (i < n) ? rv - h.res[ih - 1 - m][i] : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < kMaxOwn; ++j) {
      if (om[j] < 0) continue;
      const double* a = D + om[j] * kGramTile;
      const double* b = (on[j] == -2) ? R : D + on[j] * kGramTile;
      double s = 0.0;
#pragma unroll 8
      for (int p = 0; p < kGramTile; ++p) s += a[p] * b[p];
      acc[j] += s;
    }
    __syncthreads();
  }
  for (int j = 0; j < kMaxOwn; ++j) {
    const int o = threadIdx.x + j * blockDim.x;
    if (o < nout) part[(long)blockIdx.x * nout + o] = acc[j];
  }
}

void launch_gram(const HistPtrs& h, int ih, long n_all, double* part, double* out, cudaStream_t st) {
  const int nout = ih * (ih + 1) / 2 + ih;
  long nb = (n_all + kGramTile - 1) / kGramTile;
  if (nb > 2 * 152) nb = 2 * 152;
  const size_t smem = sizeof(double) * (size_t)(ih + 1) * kGramTile;
  if (smem > 48 * 1024) cudaFuncSetAttribute(gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  gram_kernel<<<(int)nb, 256, smem, st>>>(h, ih, n_all, part);
  count_launches(1);
  reduce_parts(part, (int)nb, nout, out, 1.0, st);
}

// Products of the current residual with the history: t[j] = r . res[j] for logical j = 0..nj-1
// (res[nj-1] is the copy of r).  Blocks write partials part[block * nj + j], in a fixed order.
constexpr int kDotChunk = 8;
__global__ void __launch_bounds__(256) hist_dots_kernel(HistPtrs h, const double* __restrict__ r, int nj, long n,
                                                        double* __restrict__ part) {
  __shared__ double red[kDotChunk][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j0 = 0; j0 < nj; j0 += kDotChunk) {
    const int nc = min(kDotChunk, nj - j0);
    const double* hp[kDotChunk];
    double acc[kDotChunk];
#pragma unroll
    for (int k = 0; k < kDotChunk; ++k) {
      hp[k] = h.res[j0 + (k < nc ? k : 0)];
      acc[k] = 0.0;
    }
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
      const double rv = r[i];
#pragma unroll
      for (int k = 0; k < kDotChunk; ++k)
        if (k < nc) acc[k] = fma(rv, hp[k][i], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < kDotChunk; ++k) {
      const double v = warp_sum(acc[k]);
      if (lane == 0) red[k][wid] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < nc) {
      double v = 0.0;
      for (int q = 0; q < nw; ++q) v += red[threadIdx.x][q];
      part[(long)blockIdx.x * nj + j0 + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

// Gram update from cached products.  P[a * nslot + b] = res(slot a) . res(slot b) for every pair
// of physical slots in the history window (slot of logical j = (base + j) % nslot); t[j] = r . res[j].
// Stores the current slot's row and column of P, then the packed U and V of gram_kernel from
//   U[m][n] = t[ih] - t[ih-1-m] - t[ih-1-n] + P[a_m][a_n],   V[m] = t[ih] - t[ih-1-m]
// (d_m = r - res[ih-1-m]; the same sums expanded).  flag = 1 when a diagonal U[m][m] is not
// positive or is below (|r| + |res[ih-1-m]|)^2 / kGramCancel, where the expansion's rounding could
// exceed ~kGramCancel ulps of U[m][m]: the caller then sums U and V directly (gram_kernel).
constexpr double kGramCancel = 1.0e3;
__global__ void gram_assemble_kernel(double* __restrict__ P, int nslot, int base, const double* __restrict__ t, int ih,
                                     double* __restrict__ packed, int* __restrict__ flag) {
  __shared__ double ts[kMaxHist];
  __shared__ int bad;
  const int c = (base + ih) % nslot;
  for (int j = threadIdx.x; j <= ih; j += blockDim.x) ts[j] = t[j];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = threadIdx.x; j <= ih; j += blockDim.x) {
    const int a = (base + j) % nslot;
    P[(long)c * nslot + a] = ts[j];
    P[(long)a * nslot + c] = ts[j];
  }
  __syncthreads();
  const int npair = ih * (ih + 1) / 2;
  const double rr = ts[ih];
  for (int o = threadIdx.x; o < npair; o += blockDim.x) {
    int m = 0, rem = o;
    while (rem >= ih - m) {
      rem -= ih - m;
      ++m;
    }
    const int n = m + rem;
    const int am = (base + ih - 1 - m) % nslot, an = (base + ih - 1 - n) % nslot;
    const double u = (rr - ts[ih - 1 - m]) - (ts[ih - 1 - n] - P[(long)am * nslot + an]);
    packed[o] = u;
    if (m == n) {
      const double scale = sqrt(rr) + sqrt(P[(long)am * nslot + am]);
      if (!(u > 0.0) || !(scale * scale <= kGramCancel * u)) bad = 1;
    }
  }
  for (int m = threadIdx.x; m < ih; m += blockDim.x) packed[npair + m] = rr - ts[ih - 1 - m];
  __syncthreads();
  if (threadIdx.x == 0) *flag = bad;
}

void launch_gram_cached(const HistPtrs& h, const double* r, int ih, long n_all, double* P, int nslot, int base,
                        double* part, double* t, double* packed, int* flag, cudaStream_t st) {
  const int nb = red_blocks(n_all);
  hist_dots_kernel<<<nb, 256, 0, st>>>(h, r, ih + 1, n_all, part);
  count_launches(1);
  reduce_parts(part, nb, ih + 1, t, 1.0, st);
  gram_assemble_kernel<<<1, 256, 0, st>>>(P, nslot, base, t, ih, packed, flag);
  count_launches(1);
}

// LU with partial pivoting, explicit inverse, Cn = inv(U) V (the inv!(lu!(Umn)) * Vm of
// anderson.jl:184-189).  status = k+1 when pivot k is exactly zero (LAPACK info > 0).
__global__ void solve_kernel(const double* __restrict__ packed, int n, double* __restrict__ Cn, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ld = n + 1;
  double* Af = reinterpret_cast<double*>(smem_raw);
  double* If = Af + n * ld;
#define A(i, j) Af[(i) * ld + (j)]
#define Inv(i, j) If[(i) * ld + (j)]
  __shared__ int perm[kMaxHist];
  __shared__ int piv;
  __shared__ int bad;
  const int npair = n * (n + 1) / 2;
  const double* V = packed + npair;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx % n;
    const int m = i < j ? i : j, c = i < j ? j : i;
    const int o = m * n - m * (m - 1) / 2 + (c - m);
    A(i, j) = packed[o];
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = i;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(A(k, k));
      for (int i = k + 1; i < n; ++i) {
        const double v = fabs(A(i, k));
        if (v > best) {
          best = v;
          p = i;
        }
      }
      piv = p;
      if (A(p, k) == 0.0 && bad == 0) bad = k + 1;
    }
    __syncthreads();
    if (bad) break;
    const int p = piv;
    if (p != k) {
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double t = A(k, j);
        A(k, j) = A(p, j);
        A(p, j) = t;
      }
      if (threadIdx.x == 0) {
        const int t = perm[k];
        perm[k] = perm[p];
        perm[p] = t;
      }
    }
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A(i, k) /= A(k, k);
    __syncthreads();
    for (int idx = threadIdx.x; idx < (n - k - 1) * (n - k - 1); idx += blockDim.x) {
      const int i = k + 1 + idx / (n - k - 1), j = k + 1 + idx % (n - k - 1);
      A(i, j) -= A(i, k) * A(k, j);
    }
    __syncthreads();
  }
  if (bad) {
    if (threadIdx.x == 0) *status = bad;
    return;
  }
  // column col of the inverse: solve L y = P e_col, U x = y
  for (int col = threadIdx.x; col < n; col += blockDim.x) {
    double y[kMaxHist];
    for (int i = 0; i < n; ++i) {
      double s = (perm[i] == col) ? 1.0 : 0.0;
      for (int j = 0; j < i; ++j) s -= A(i, j) * y[j];
      y[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (int j = i + 1; j < n; ++j) s -= A(i, j) * Inv(j, col);
      Inv(i, col) = s / A(i, i);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += Inv(i, j) * V[j];
    Cn[i] = s;
  }
  if (threadIdx.x == 0) *status = 0;
#undef A
#undef Inv
}

void launch_solve(const double* packed, int ih, double* Cn, int* status, cudaStream_t st) {
  const size_t smem = 2 * sizeof(double) * (size_t)ih * (ih + 1);
  if (smem > 48 * 1024) cudaFuncSetAttribute(solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  solve_kernel<<<1, 64, smem, st>>>(packed, ih, Cn, status);
  count_launches(1);
}

// w = W + lam D,  W = w + sum_nn Cn[nn-1] (f[ih-nn] - f[ih]),  D = r + sum_nn Cn[nn-1] (r[ih-nn] - r).
// Evaluated with the coefficients gathered, W = (w - C f[ih]) + sum c f[ih-nn] and
// D = (1 - C) r + sum c r[ih-nn] (C = sum c): two FP64 FMAs per history entry and point instead
// of two subtractions and two FMAs.  With lam = 1 (every iteration after the history has
// filled) w = (w - C f[ih] + (1 - C) r) + sum c s[ih-nn] with s = f + r kept per entry: one
// FMA and one history read per entry and point.  The pass also stores s[ih] = f[ih] + r.
__global__ void mix_kernel(double* __restrict__ w, HistPtrs h, int ih, const double* __restrict__ Cn, double lam,
                           long n) {
  __shared__ double c[kMaxHist];
  __shared__ double csum;
  for (int j = threadIdx.x; j < ih; j += blockDim.x) c[j] = Cn[j];
  __syncthreads();
  if (threadIdx.x == 0) {
    double cs = 0.0;
    for (int j = 0; j < ih; ++j) cs += c[j];
    csum = cs;
  }
  __syncthreads();
  const double C = csum, om = 1.0 - csum;
  const double* r = h.res[ih];
  const double* f = h.field[ih];
  double* s = h.sum[ih];
  if (lam == 1.0) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
      const double fi = f[i], ri = r[i];
      double acc = fma(om, ri, fma(-C, fi, w[i]));
      for (int nn = 1; nn <= ih; ++nn) acc = fma(c[nn - 1], h.sum[ih - nn][i], acc);
      s[i] = fi + ri;
      w[i] = acc;
    }
    return;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double fi = f[i], ri = r[i];
    double W = fma(-C, fi, w[i]), D = om * ri;
    for (int nn = 1; nn <= ih; ++nn) {
      W = fma(c[nn - 1], h.field[ih - nn][i], W);
      D = fma(c[nn - 1], h.res[ih - nn][i], D);
    }
    s[i] = fi + ri;
    w[i] = fma(lam, D, W);
  }
}
void launch_mix(double* w, const HistPtrs& h, int ih, const double* Cn, double lam, long n_all, cudaStream_t st) {
  int nb = (int)((n_all + 255) / 256);
  if (nb > 8192) nb = 8192;
  mix_kernel<<<nb, 256, 0, st>>>(w, h, ih, Cn, lam, n_all);
  count_launches(1);
}

__global__ void add_kernel(double* __restrict__ out, const double* __restrict__ a, const double* __restrict__ b,
                           long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = a[i] + b[i];
}
void launch_add(double* out, const double* a, const double* b, long n, cudaStream_t st) {
  int nb = (int)((n + 255) / 256);
  if (nb > 8192) nb = 8192;
  add_kernel<<<nb, 256, 0, st>>>(out, a, b, n);
  count_launches(1);
}

}  // namespace pf
