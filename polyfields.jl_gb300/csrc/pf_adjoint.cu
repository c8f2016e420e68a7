// Elementwise and reduction pieces of the adjoint (pullback) of density!, and the Euler and
// momentum field updaters (elementwise, at the end of this file).
//
// The reference has no derivative code.  These kernels serve the hand-derived adjoint of
// the chain propagation (src/species/multiblock.jl:125-231): for every application
// y = A x of a block operator A = LW . c2r(LD . r2c(LW . )) (symmetric, so the adjoint
// propagation reuses the forward kernels) with adjoint ybar, the field gradient collects
// ybar*y + x*(A ybar) and the adjoint moves on as lambda = A ybar + (Simpson sources).  With
// float32 histories every quantity is kept in the chain's rescaled variables; the step
// factor c_t of the forward solve multiplies A ybar and the sources carry the Simpson factor
// fac[s] = exp(-L_s - L'_s) / Q, so products of propagators and adjoints are scale-free.
#include "pf_kernels.h"

namespace pf {

static int adj_blocks(long n) {
  long b = (n + 255) / 256;
  if (b > 4096) b = 4096;
  if (b < 1) b = 1;
  return (int)b;
}

template <typename T>
__device__ __forceinline__ double adj_source(const AdjSrc<T>& s, long i) {
  double v = 0.0;
  for (int k = 0; k < s.n; ++k) v += s.coef[k] * s.rb[k][i] * (double)s.qs[k][i];
  return v;
}

template <typename T>
__device__ __forceinline__ double adj_factor(const AdjSrc<T>& s) {
  return s.fac ? *s.fac : 1.0 / *s.Qdev;
}

template <typename T>
__global__ void adj_lw_pair_kernel(T* __restrict__ u1, T* __restrict__ u2, const T* __restrict__ lw,
                                   const T* __restrict__ x, const T* __restrict__ ybar, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T l = lw[i];
    u1[i] = l * x[i];
    u2[i] = l * ybar[i];
  }
}

// lam may alias ybar: each point is read before it is written by the same thread
template <typename T>
__global__ void adj_finish_kernel(T* lam, const T* __restrict__ r, const T* ybar, const T* __restrict__ x,
                                  const T* __restrict__ y, double* __restrict__ G, const float* __restrict__ cfac,
                                  AdjSrc<T> src, long n) {
  const double c = cfac ? (double)*cfac : 1.0;
  const double f = src.n ? adj_factor(src) : 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double rv = c * (double)r[i];
    G[i] += (double)ybar[i] * (double)y[i] + (double)x[i] * rv;
    lam[i] = (T)(rv + f * adj_source(src, i));
  }
}

template <typename T>
__global__ void adj_init_kernel(T* __restrict__ lam, AdjSrc<T> src, double dq, long n) {
  const double f = src.n ? adj_factor(src) : 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    lam[i] = (T)(f * adj_source(src, i) + dq);
}

__global__ void adj_accum_kernel(double* __restrict__ acc, const double* __restrict__ part, int nparts, int nw,
                                 const float* __restrict__ cfac) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += part[(long)i * nw + j];
  v = block_sum(v, red);
  if (threadIdx.x == 0) acc[j] += (cfac ? (double)*cfac : 1.0) * v;
}

__global__ void adj_point_kernel(double* __restrict__ wbar, const double* __restrict__ rho,
                                 const double* __restrict__ rb, const double* __restrict__ w, double vol, double S,
                                 double ngQ, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    wbar[i] += -vol * rho[i] * rb[i] + S * vol * exp(-vol * w[i]) / ngQ;
}

__global__ void daxpy_kernel(double* __restrict__ y, const double* __restrict__ x, double a, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

__global__ void ddot_kernel(const double* __restrict__ a, const double* __restrict__ b, long n,
                            double* __restrict__ part) {
  __shared__ double red[32];
  double v = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    v += a[i] * b[i];
  v = block_sum(v, red);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

__global__ void ddot_final_kernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double red[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += part[i];
  v = block_sum(v, red);
  if (threadIdx.x == 0) *out = v;
}

template <typename T>
void launch_adj_lw_pair(T* u1, T* u2, const T* lw, const T* x, const T* ybar, long n, cudaStream_t st) {
  adj_lw_pair_kernel<T><<<adj_blocks(n), 256, 0, st>>>(u1, u2, lw, x, ybar, n);
  count_launches(1);
}

template <typename T>
void launch_adj_finish(T* lam, const T* r, const T* ybar, const T* x, const T* y, double* G, const float* cfac,
                       const AdjSrc<T>& src, long n, cudaStream_t st) {
  adj_finish_kernel<T><<<adj_blocks(n), 256, 0, st>>>(lam, r, ybar, x, y, G, cfac, src, n);
  count_launches(1);
}

template <typename T>
void launch_adj_init(T* lam, const AdjSrc<T>& src, double dq, long n, cudaStream_t st) {
  adj_init_kernel<T><<<adj_blocks(n), 256, 0, st>>>(lam, src, dq, n);
  count_launches(1);
}

void launch_adj_accum(double* acc, const double* part, int nparts, int nw, const float* cfac, cudaStream_t st) {
  adj_accum_kernel<<<nw, 256, 0, st>>>(acc, part, nparts, nw, cfac);
  count_launches(1);
}

void launch_adj_point(double* wbar, const double* rho, const double* rb, const double* w, double vol, double S,
                      double ngQ, long n, cudaStream_t st) {
  adj_point_kernel<<<adj_blocks(n), 256, 0, st>>>(wbar, rho, rb, w, vol, S, ngQ, n);
  count_launches(1);
}

// dL/drho_a of L = free_energy at fixed fields (system.jl:402-433 with flory.jl:39-59 and
// edwards.jl:34-60): (-w_a + sum_b chi_ab rho_b / (v_a v_b)) / Ng; the diagonal of chi holds
// the Edwards u (energy (u/2) (rho/v)^2, derivative u rho / v^2).
static __global__ void fhelm_cotangent_kernel(double* __restrict__ rbar, const double* __restrict__ w,
                                              const double* __restrict__ rho, MonomerSet ms, long ng) {
  const double inv = 1.0 / (double)ng;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ng; i += (long)gridDim.x * blockDim.x) {
    for (int a = 0; a < ms.nmon; ++a) {
      double s = -w[(long)a * ng + i];
      for (int b = 0; b < ms.nmon; ++b) {
        const double c = ms.chi[a * kMaxMon + b];
        if (c != 0.0) s += c * rho[(long)b * ng + i] / (ms.vol[a] * ms.vol[b]);
      }
      rbar[(long)a * ng + i] = s * inv;
    }
  }
}

void launch_fhelm_cotangent(double* rbar, const double* w, const double* rho, const MonomerSet& ms, long ng,
                            cudaStream_t st) {
  fhelm_cotangent_kernel<<<adj_blocks(ng), 256, 0, st>>>(rbar, w, rho, ms, ng);
  count_launches(1);
}

void launch_daxpy(double* y, const double* x, double a, long n, cudaStream_t st) {
  daxpy_kernel<<<adj_blocks(n), 256, 0, st>>>(y, x, a, n);
  count_launches(1);
}

void launch_ddot(const double* a, const double* b, long n, double* part, double* out, cudaStream_t st) {
  const int nb = std::min(adj_blocks(n), kRedBlocks);
  ddot_kernel<<<nb, 256, 0, st>>>(a, b, n, part);
  ddot_final_kernel<<<1, 256, 0, st>>>(part, nb, out);
  count_launches(2);
}

#define PF_ADJ_INST(T)                                                                                           \
  template void launch_adj_lw_pair<T>(T*, T*, const T*, const T*, const T*, long, cudaStream_t);                \
  template void launch_adj_finish<T>(T*, const T*, const T*, const T*, const T*, double*, const float*,           \
                                     const AdjSrc<T>&, long, cudaStream_t);                                      \
  template void launch_adj_init<T>(T*, const AdjSrc<T>&, double, long, cudaStream_t);
PF_ADJ_INST(float)
PF_ADJ_INST(double)

}  // namespace pf

// ------------------------------------------------------------------ Euler and momentum updaters
// src/updaters/euler.jl:36-65 and src/updaters/momentum.jl:63-165, elementwise over all
// monomer grids (n = nmon * Ng).
namespace pf {

// predictor: w += lam r; temp = w + lam/2 r (on the updated w, as the reference does)
__global__ void euler_predict_kernel(double* __restrict__ w, double* __restrict__ temp, const double* __restrict__ r,
                                     double lam, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = w[i] + lam * r[i];
    w[i] = v;
    temp[i] = v + 0.5 * lam * r[i];
  }
}
// corrector: w = temp + lam/2 r(w_predicted)
__global__ void euler_correct_kernel(double* __restrict__ w, const double* __restrict__ temp,
                                     const double* __restrict__ r, double lam, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    w[i] = temp[i] + 0.5 * lam * r[i];
}
// MOM (0), RMS (1), ADAM (2): moments from the fresh residual, then w += lam * step
__global__ void momentum_kernel(int method, double* __restrict__ w, double* __restrict__ m, double* __restrict__ v,
                                const double* __restrict__ r, double lam, double b1, double b2, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double ri = r[i];
    double step;
    if (method == 0) {
      const double mi = b1 * m[i] + (1.0 - b1) * ri;
      m[i] = mi;
      step = mi;
    } else if (method == 1) {
      const double vi = b2 * v[i] + (1.0 - b2) * ri * ri;
      v[i] = vi;
      step = ri / (sqrt(vi) + 1e-8);
    } else {
      const double mi = b1 * m[i] + (1.0 - b1) * ri;
      const double vi = b2 * v[i] + (1.0 - b2) * ri * ri;
      m[i] = mi;
      v[i] = vi;
      step = mi / (sqrt(vi) + 1e-8);
    }
    w[i] += lam * step;
  }
}
// NAG look-ahead: temp = w; w += lam m
__global__ void nag_ahead_kernel(double* __restrict__ w, double* __restrict__ temp, const double* __restrict__ m,
                                 double lam, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    temp[i] = w[i];
    w[i] += lam * m[i];
  }
}
// NAG update: m = gamma m + (1 - gamma) r(look-ahead); w = temp + lam m
__global__ void nag_update_kernel(double* __restrict__ w, const double* __restrict__ temp, double* __restrict__ m,
                                  const double* __restrict__ r, double lam, double gamma, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double mi = gamma * m[i] + (1.0 - gamma) * r[i];
    m[i] = mi;
    w[i] = temp[i] + lam * mi;
  }
}

void launch_euler_predict(double* w, double* temp, const double* r, double lam, long n, cudaStream_t st) {
  euler_predict_kernel<<<adj_blocks(n), 256, 0, st>>>(w, temp, r, lam, n);
  count_launches(1);
}
void launch_euler_correct(double* w, const double* temp, const double* r, double lam, long n, cudaStream_t st) {
  euler_correct_kernel<<<adj_blocks(n), 256, 0, st>>>(w, temp, r, lam, n);
  count_launches(1);
}
void launch_momentum(int method, double* w, double* m, double* v, const double* r, double lam, double b1, double b2,
                     long n, cudaStream_t st) {
  momentum_kernel<<<adj_blocks(n), 256, 0, st>>>(method, w, m, v, r, lam, b1, b2, n);
  count_launches(1);
}
void launch_nag_ahead(double* w, double* temp, const double* m, double lam, long n, cudaStream_t st) {
  nag_ahead_kernel<<<adj_blocks(n), 256, 0, st>>>(w, temp, m, lam, n);
  count_launches(1);
}
void launch_nag_update(double* w, const double* temp, double* m, const double* r, double lam, double gamma, long n,
                       cudaStream_t st) {
  nag_update_kernel<<<adj_blocks(n), 256, 0, st>>>(w, temp, m, r, lam, gamma, n);
  count_launches(1);
}

}  // namespace pf

// ------------------------------------------------------------------ RQM4 combination
// src/system/mde.jl:83-104: q_{s+1} = (4 q2 - q1) / 3 with q1 one full RK2 step and q2 two
// half steps from q_s.
namespace pf {
template <typename T>
__global__ void rqm4_combine_kernel(T* __restrict__ out, const T* __restrict__ q1, const T* __restrict__ q2, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = (T)((4.0 * (double)q2[i] - (double)q1[i]) / 3.0);
}
template <typename T>
void launch_rqm4_combine(T* out, const T* q1, const T* q2, long n, cudaStream_t st) {
  rqm4_combine_kernel<T><<<adj_blocks(n), 256, 0, st>>>(out, q1, q2, n);
  count_launches(1);
}
template void launch_rqm4_combine<float>(float*, const float*, const float*, long, cudaStream_t);
template void launch_rqm4_combine<double>(double*, const double*, const double*, long, cudaStream_t);
}  // namespace pf
