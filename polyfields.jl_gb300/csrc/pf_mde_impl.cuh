// Pseudo-spectral MDE propagator kernels (reference: src/system/mde.jl:43-104 with the FFTW
// plans of src/system/fft.jl) and the stress transforms (src/species/multiblock.jl:233-295).
//
// One RK2 contour step is  q_{s+1} = LW * irfft( LD * rfft( LW * q_s ) )  with
// LW = exp(-ds vol w / 2) on the real grid and LD = exp(-ds b^2 k^2 / 6) / Ng on the half
// spectrum (the 1/Ng of the normalised irfft folded in).
//
// Layout in HBM: a real grid is Nz planes of Ny rows of Nx values, x fastest (the
// reference's column-major Array{Float64,3}[x,y,z]); the half spectrum is Nz planes of
// Ny rows of Kx = Nx/2+1 complex values.  A propagator history is (Ns+1) consecutive grids.
//
// Grids with Nz == 1 (1D and 2D systems) hold a whole plane in one CTA's shared memory,
// so one persistent CTA runs all contour steps of a chain (chain_plane_kernel).  3D grids
// split each step into a plane pass (x and y transforms, one CTA per z plane:
// xy_step_kernel) and a pencil pass (z transforms and LD, one CTA per tile of pencils:
// z_step_kernel); the plane pass of step t fuses the end of step t-1 (inverse transforms,
// LW, store q) with the start of step t (LW, forward transforms).  Independent chains
// (forward q, backward qc, other species) advance together in the same launches.
//
// Every kernel is specialised on its transform lengths at compile time; the host picks the
// instantiation from the supported plane shapes below.
#pragma once
#include "pf_fft.cuh"
#include "pf_kernels.h"

namespace pf {

// Plane shapes (Nx, Ny) with kernels: 1D rows, square planes and 2:1 rectangles.
#define PF_PLANE_SHAPES(X)                                                                    \
  X(8, 1) X(16, 1) X(32, 1) X(48, 1) X(64, 1) X(96, 1) X(128, 1) X(256, 1) X(16, 16) X(32, 32) \
  X(48, 48) X(64, 64) X(96, 96) X(128, 128) X(32, 16) X(64, 32) X(96, 48) X(128, 64)
#define PF_Z_LENGTHS(X) X(8) X(16) X(32) X(48) X(64) X(96) X(128) X(256)

template <int NX, int NY>
struct PlaneCfg {
  static constexpr int KX = NX / 2 + 1;
  static constexpr int NKP = KX * NY;                 // half-spectrum points of a plane
  static constexpr int NP = NX * NY;                  // real points of a plane
  static constexpr int SLOTS = KX * (NY > 1 ? NY : 2);  // complex slots of the work plane
  static constexpr int THREADS = NY == 1 ? 32 : (NKP >= 4096 ? 512 : (NKP >= 1024 ? 256 : 128));
  // float32 planes of >= 4096 spectral points: two CTAs per SM fit the shared memory, so ask
  // the register allocator for that occupancy
  static constexpr int MINB = NKP >= 4096 ? 2 : 1;
};

// ------------------------------------------------------------------ operator setup
// LW = exp(-coeff * w) evaluated in float64 and rounded once to T: the propagator multiplies
// by LW twice per contour step, so a biased float32 exp would compound over the chain.
template <typename T>
__global__ void lw_kernel(T* __restrict__ lw, const double* __restrict__ w, double coeff, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    lw[i] = (T)exp(-coeff * w[i]);
}

// Folded wavevector index of src/system/cell.jl:273-277 (quirk Q1: |j|, not signed j).
__device__ __forceinline__ double fold_index(int i, int n) { return (double)((i <= n / 2) ? i : n - i); }

__device__ __forceinline__ double ksq_at(const CellGeom& g, int ix, int iy, int iz) {
  const double jx = ix, jy = fold_index(iy, g.ny), jz = fold_index(iz, g.nz);
  // kvec = G * jvec, G columns = reciprocal vectors (row-major storage G[r*3+c])
  const double kx = g.G[0] * jx + g.G[1] * jy + g.G[2] * jz;
  const double ky = g.G[3] * jx + g.G[4] * jy + g.G[5] * jz;
  const double kz = g.G[6] * jx + g.G[7] * jy + g.G[8] * jz;
  return kx * kx + ky * ky + kz * kz;
}

template <typename T>
__global__ void ld_kernel(T* __restrict__ ld, CellGeom g, double coeff, double scale) {
  const int kxn = g.nx / 2 + 1;
  const long nk = (long)kxn * g.ny * g.nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nk; i += (long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % kxn);
    const int iy = (int)((i / kxn) % g.ny);
    const int iz = (int)(i / ((long)kxn * g.ny));
    ld[i] = (T)(exp(-coeff * ksq_at(g, ix, iy, iz)) * scale);
  }
}

// dksq for every cell parameter (src/system/cell.jl:292-320), nparams grids of Nk.
static __global__ void dksq_kernel(double* __restrict__ dk, CellGeom g, int nparams) {
  const int kxn = g.nx / 2 + 1;
  const long nk = (long)kxn * g.ny * g.nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nk; i += (long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % kxn);
    const int iy = (int)((i / kxn) % g.ny);
    const int iz = (int)(i / ((long)kxn * g.ny));
    const double j[3] = {(double)ix, fold_index(iy, g.ny), fold_index(iz, g.nz)};
    for (int p = 0; p < nparams; ++p) {
      double acc = 0.0;
      for (int l = 0; l < g.dim; ++l)
        for (int m = 0; m < g.dim; ++m) acc += j[l] * j[m] * g.dGG[(l * 3 + m) * kMaxParams + p];
      dk[p * nk + i] = acc;
    }
  }
}

template <typename T>
__global__ void fill_kernel(T* __restrict__ a, T v, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) a[i] = v;
}

// Rescale factor of one contour step: 1 / mean(LW * q_t), from the grid sum dc (the k = 0
// coefficient of the forward transform); 1 when that mean is not a positive finite number.
template <typename T>
__device__ __forceinline__ T rescale_factor(T dc, double n) {
  const double m = (double)dc / n;
  return (m > 0.0 && isfinite(m)) ? (T)(1.0 / m) : (T)1;
}

// Copy the twiddle tables of this kernel's transform lengths into shared memory (the FFT
// passes read them every butterfly; shared memory keeps those reads off the L1/L2 path).
template <typename T, int N>
__device__ __forceinline__ void stage_twiddles(Cx<T>* dst, const Cx<T>* __restrict__ src) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) dst[i] = src[i];
}

// 16-byte vector of T (4 floats or 2 doubles).
template <typename T>
struct Vec;
template <>
struct Vec<float> {
  using V = float4;
  static constexpr int W = 4;
  __device__ static float get(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
  __device__ static void set(float4& v, int k, float a) {
    if (k == 0) v.x = a;
    else if (k == 1) v.y = a;
    else if (k == 2) v.z = a;
    else v.w = a;
  }
};
template <>
struct Vec<double> {
  using V = double2;
  static constexpr int W = 2;
  __device__ static double get(const double2& v, int k) { return k == 0 ? v.x : v.y; }
  __device__ static void set(double2& v, int k, double a) {
    if (k == 0) v.x = a;
    else v.y = a;
  }
};

// Copy n complex values global <-> shared with 16-byte accesses when the byte count allows.
template <typename T>
__device__ __forceinline__ void copy_cx(Cx<T>* __restrict__ dst, const Cx<T>* __restrict__ src, int n) {
  if ((n * sizeof(Cx<T>)) % 16 == 0) {
    const int nv = (int)(n * sizeof(Cx<T>) / 16);
    const int4* s4 = reinterpret_cast<const int4*>(src);
    int4* d4 = reinterpret_cast<int4*>(dst);
    for (int i = threadIdx.x; i < nv; i += blockDim.x) d4[i] = s4[i];
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  }
}

// ------------------------------------------------------------------ plane helpers
// Write u = lw * q (or q when lw is null) into the pair layout of S.  Rows are read with
// 16-byte vectors (NX is a multiple of the vector width for every supported shape).
template <typename T, int NX, int NY>
__device__ __forceinline__ void load_plane(Cx<T>* S, const T* __restrict__ lw, const T* __restrict__ q) {
  using C = PlaneCfg<NX, NY>;
  using VT = Vec<T>;
  using V = typename VT::V;
  static_assert(NX % VT::W == 0, "row length must be a multiple of the vector width");
  constexpr int NV = C::NP / VT::W;
  const V* q4 = reinterpret_cast<const V*>(q);
  const V* l4 = reinterpret_cast<const V*>(lw);
  for (int iv = threadIdx.x; iv < NV; iv += blockDim.x) {
    const int i = iv * VT::W;
    const int y = i / NX, x = i - y * NX;
    const V qv = q4[iv];
    V lv;
    if (lw) lv = l4[iv];
#pragma unroll
    for (int k = 0; k < VT::W; ++k) {
      const T u = lw ? VT::get(lv, k) * VT::get(qv, k) : VT::get(qv, k);
      pair_elem(S, C::KX, y, x + k) = u;
      if (NY == 1) S[x + k].y = (T)0;
    }
  }
}

// q_out = lw_cur * cscale * r (r = plane after the inverse transform); store it, and when
// lw_next is given put u = lw_next * q_out back into S for the next step.
template <typename T, int NX, int NY>
__device__ __forceinline__ void finish_plane(Cx<T>* S, const T* __restrict__ lw_cur, const T* __restrict__ lw_next,
                                             T* __restrict__ qout, T cscale) {
  using C = PlaneCfg<NX, NY>;
  using VT = Vec<T>;
  using V = typename VT::V;
  constexpr int NV = C::NP / VT::W;
  const V* lc4 = reinterpret_cast<const V*>(lw_cur);
  const V* ln4 = reinterpret_cast<const V*>(lw_next);
  V* o4 = reinterpret_cast<V*>(qout);
  for (int iv = threadIdx.x; iv < NV; iv += blockDim.x) {
    const int i = iv * VT::W;
    const int y = i / NX, x = i - y * NX;
    const V lc = lc4[iv];
    V ln;
    if (lw_next) ln = ln4[iv];
    V ov;
#pragma unroll
    for (int k = 0; k < VT::W; ++k) {
      T& e = pair_elem(S, C::KX, y, x + k);
      const T qv = VT::get(lc, k) * (e * cscale);
      VT::set(ov, k, qv);
      if (lw_next) {
        e = VT::get(ln, k) * qv;
        if (NY == 1) S[x + k].y = (T)0;
      }
    }
    o4[iv] = ov;
  }
}

// ------------------------------------------------------------------ Nz == 1 chains
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS)
    chain_plane_kernel(const ChainJob<T>* __restrict__ jobs, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  __shared__ Cx<T> twx[NX], twy[NY];
  stage_twiddles<T, NX>(twx, twg.x);
  stage_twiddles<T, NY>(twy, twg.y);
  const Twiddles<T> tw{twx, twy, nullptr};
  const ChainJob<T> job = jobs[blockIdx.x];
#pragma unroll 1
  for (int t = 0; t < job.nsteps; ++t) {
    const StepOp<T> op = job.ops[t];
    if (t == 0) {
      load_plane<T, NX, NY>(S, op.lw, job.hist + (long)job.s0 * C::NP);
    }
    __syncthreads();
    plane_fwd<T, NX, NY>(S, tw.x, tw.y);
    T c = (T)1;
    if (job.csc) {
      c = rescale_factor<T>(S[0].x, (double)C::NP);
      if (threadIdx.x == 0) {
        job.csc[t] = (float)c;
        job.lsc[t] = log((double)c);
      }
      __syncthreads();  // every thread has read S[0] before it is overwritten below
    }
    for (int k = threadIdx.x; k < C::NKP; k += blockDim.x) {
      const T f = op.ld[k] * c;
      S[k] = cx<T>(S[k].x * f, S[k].y * f);
    }
    __syncthreads();
    plane_inv<T, NX, NY>(S, tw.x, tw.y);
    const int s_out = job.s0 + job.dir * (t + 1);
    const T* lw_next = (t + 1 < job.nsteps) ? job.ops[t + 1].lw : nullptr;
    finish_plane<T, NX, NY>(S, op.lw, lw_next, job.hist + (long)s_out * C::NP, (T)1);
    __syncthreads();
  }
}

// ------------------------------------------------------------------ 3D: plane pass
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS, sizeof(T) == 4 ? PlaneCfg<NX, NY>::MINB : 1)
    xy_step_kernel(const ChainJob<T>* __restrict__ jobs, int t, int nz, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  const ChainJob<T> job = jobs[blockIdx.y];
  if (t > job.nsteps) return;
  __shared__ Cx<T> twx[NX], twy[NY];
  stage_twiddles<T, NX>(twx, twg.x);
  stage_twiddles<T, NY>(twy, twg.y);
  const Twiddles<T> tw{twx, twy, nullptr};
  const int z = blockIdx.x;
  const long ng = (long)C::NP * nz;
  const bool finish = t >= 1;
  const bool start = t < job.nsteps;
  if (finish) {
    copy_cx<T>(S, job.kbuf + (long)z * C::NKP, C::NKP);
    __syncthreads();
    plane_inv<T, NX, NY>(S, tw.x, tw.y);
    const StepOp<T> op = job.ops[t - 1];
    const int s_out = job.s0 + job.dir * t;
    const T* lw_next = start ? job.ops[t].lw + (long)z * C::NP : nullptr;
    const T c = job.csc ? (T)job.csc[t - 1] : (T)1;
    finish_plane<T, NX, NY>(S, op.lw + (long)z * C::NP, lw_next, job.hist + (long)s_out * ng + (long)z * C::NP, c);
  } else {
    load_plane<T, NX, NY>(S, job.ops[0].lw + (long)z * C::NP, job.hist + (long)job.s0 * ng + (long)z * C::NP);
  }
  __syncthreads();
  if (start) {
    plane_fwd<T, NX, NY>(S, tw.x, tw.y);
    copy_cx<T>(job.kbuf + (long)z * C::NKP, S, C::NKP);
  }
}

// ------------------------------------------------------------------ 3D: pencil pass
// M consecutive pencils (index m = ky*Kx + kx within a plane) of length NZ per CTA.  The tile
// is pencil-major in shared memory with rows padded by one element, Tl[mm*(NZ+1) + z], so the
// threads of a transform group read consecutive words and the groups of a warp fall on
// different banks.
template <typename T>
struct ZCfg {
  static constexpr int M = sizeof(T) == 4 ? 16 : 8;  // 128-byte rows of the global tile
};

template <typename T, int NZ>
__global__ void __launch_bounds__(512)
    z_step_kernel(const ChainJob<T>* __restrict__ jobs, int t, int nkp, double ng, Twiddles<T> twg) {
  constexpr int M = ZCfg<T>::M;
  constexpr int LDT = NZ + 1;
  constexpr int TOT = NZ * M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* Tl = reinterpret_cast<Cx<T>*>(smem_raw);
  const ChainJob<T> job = jobs[blockIdx.y];
  if (t >= job.nsteps) return;
  __shared__ Cx<T> twz[NZ];
  stage_twiddles<T, NZ>(twz, twg.z);
  const Twiddles<T> tw{nullptr, nullptr, twz};
  const int m0 = blockIdx.x * M;
  const int mc = min(M, nkp - m0);
  Cx<T>* kb = job.kbuf;
  for (int i = threadIdx.x; i < TOT; i += blockDim.x) {
    const int zz = i / M, mm = i - zz * M;
    Tl[mm * LDT + zz] = (mm < mc) ? kb[(long)zz * nkp + m0 + mm] : cx<T>(0, 0);
  }
  __syncthreads();
  fft_batch_n<T, false, NZ>(Tl, 1, LDT, M, tw.z);
  __syncthreads();
  if (job.csc && blockIdx.x == 0 && threadIdx.x == 0) {
    // the (0, 0, 0) coefficient is the grid sum of LW * q_t
    const T c = rescale_factor<T>(Tl[0].x, ng);
    job.csc[t] = (float)c;
    job.lsc[t] = log((double)c);
  }
  const T* ld = job.ops[t].ld;
  for (int i = threadIdx.x; i < TOT; i += blockDim.x) {
    const int zz = i / M, mm = i - zz * M;
    if (mm < mc) {
      const T f = ld[(long)zz * nkp + m0 + mm];
      Cx<T>& e = Tl[mm * LDT + zz];
      e = cx<T>(e.x * f, e.y * f);
    }
  }
  __syncthreads();
  fft_batch_n<T, true, NZ>(Tl, 1, LDT, M, tw.z);
  __syncthreads();
  for (int i = threadIdx.x; i < TOT; i += blockDim.x) {
    const int zz = i / M, mm = i - zz * M;
    if (mm < mc) kb[(long)zz * nkp + m0 + mm] = Tl[mm * LDT + zz];
  }
}

// ------------------------------------------------------------------ stress transforms
// For each item (a contour point s of one block): sum_k c_k Re(qhat_s,k) Re(qchat_s,k) dksq_p,k
// with c_0 = 1 and c_k = 2 otherwise (quirk Q2, multiblock.jl:279-282).  Nz == 1 version:
// one CTA per item transforms both planes.  Output: part[item * nparams + p].
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS)
    stress_plane_kernel(const StressItem<T>* __restrict__ items, const double* __restrict__ dksq, int nparams,
                        double* __restrict__ part, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  __shared__ Cx<T> twx[NX], twy[NY];
  stage_twiddles<T, NX>(twx, twg.x);
  stage_twiddles<T, NY>(twy, twg.y);
  const Twiddles<T> tw{twx, twy, nullptr};
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  T* req = reinterpret_cast<T*>(S + C::SLOTS);
  __shared__ double red[kMaxParams][32];
  const StressItem<T> it = items[blockIdx.x];
  load_plane<T, NX, NY>(S, nullptr, it.q);
  __syncthreads();
  plane_fwd<T, NX, NY>(S, tw.x, tw.y);
  for (int k = threadIdx.x; k < C::NKP; k += blockDim.x) req[k] = S[k].x;
  __syncthreads();
  load_plane<T, NX, NY>(S, nullptr, it.qc);
  __syncthreads();
  plane_fwd<T, NX, NY>(S, tw.x, tw.y);
  double acc[kMaxParams];
  for (int p = 0; p < kMaxParams; ++p) acc[p] = 0.0;
  for (int k = threadIdx.x; k < C::NKP; k += blockDim.x) {
    const double prod = (double)S[k].x * (double)req[k] * (k == 0 ? 1.0 : 2.0);
    for (int p = 0; p < nparams; ++p) acc[p] += prod * dksq[(long)p * C::NKP + k];
  }
  for (int p = 0; p < nparams; ++p) {
    double v = block_sum(acc[p], red[p]);
    if (threadIdx.x == 0) part[(long)blockIdx.x * nparams + p] = v;
  }
}

// 3D stress, plane pass: forward x/y transforms of the real grids src[item] into the
// half-spectrum buffers dst[item] (one CTA per (z, item)).
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS)
    xy_fwd_kernel(const T* const* __restrict__ src, Cx<T>* const* __restrict__ dst, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  __shared__ Cx<T> twx[NX], twy[NY];
  stage_twiddles<T, NX>(twx, twg.x);
  stage_twiddles<T, NY>(twy, twg.y);
  const Twiddles<T> tw{twx, twy, nullptr};
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  const int z = blockIdx.x;
  load_plane<T, NX, NY>(S, nullptr, src[blockIdx.y] + (long)z * C::NP);
  __syncthreads();
  plane_fwd<T, NX, NY>(S, tw.x, tw.y);
  Cx<T>* o = dst[blockIdx.y] + (long)z * C::NKP;
  for (int k = threadIdx.x; k < C::NKP; k += blockDim.x) o[k] = S[k];
}

// 3D stress, pencil pass: z transforms of both spectra of an item and the weighted sum
// over the tile.  Output: part[(item * ntiles + tile) * nparams + p].
template <typename T, int NZ>
__global__ void __launch_bounds__(512)
    z_fwd_stress_kernel(Cx<T>* const* __restrict__ kq, Cx<T>* const* __restrict__ kqc, int nkp,
                        const double* __restrict__ dksq, int nparams, double* __restrict__ part, Twiddles<T> twg) {
  constexpr int M = ZCfg<T>::M;
  constexpr int LDT = NZ + 1;
  __shared__ Cx<T> twz[NZ];
  stage_twiddles<T, NZ>(twz, twg.z);
  const Twiddles<T> tw{nullptr, nullptr, twz};
  constexpr int TOT = NZ * M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* A = reinterpret_cast<Cx<T>*>(smem_raw);
  Cx<T>* B = A + M * LDT;
  __shared__ double red[kMaxParams][32];
  const long nk = (long)nkp * NZ;
  const int m0 = blockIdx.x * M;
  const int mc = min(M, nkp - m0);
  const Cx<T>* a = kq[blockIdx.y];
  const Cx<T>* b = kqc[blockIdx.y];
  for (int i = threadIdx.x; i < TOT; i += blockDim.x) {
    const int zz = i / M, mm = i - zz * M;
    A[mm * LDT + zz] = (mm < mc) ? a[(long)zz * nkp + m0 + mm] : cx<T>(0, 0);
    B[mm * LDT + zz] = (mm < mc) ? b[(long)zz * nkp + m0 + mm] : cx<T>(0, 0);
  }
  __syncthreads();
  fft_batch_n<T, false, NZ>(A, 1, LDT, M, tw.z);
  fft_batch_n<T, false, NZ>(B, 1, LDT, M, tw.z);
  __syncthreads();
  double acc[kMaxParams];
  for (int p = 0; p < kMaxParams; ++p) acc[p] = 0.0;
  for (int i = threadIdx.x; i < TOT; i += blockDim.x) {
    const int zz = i / M, mm = i - zz * M;
    if (mm < mc) {
      const long k = (long)zz * nkp + m0 + mm;
      const double prod = (double)A[mm * LDT + zz].x * (double)B[mm * LDT + zz].x * (k == 0 ? 1.0 : 2.0);
      for (int p = 0; p < nparams; ++p) acc[p] += prod * dksq[p * nk + k];
    }
  }
  for (int p = 0; p < nparams; ++p) {
    double v = block_sum(acc[p], red[p]);
    if (threadIdx.x == 0) part[((long)blockIdx.y * gridDim.x + blockIdx.x) * nparams + p] = v;
  }
}

// ------------------------------------------------------------------ host launchers
template <typename K>
static void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename T, int NX, int NY>
static constexpr size_t plane_smem() {
  return sizeof(Cx<T>) * (size_t)PlaneCfg<NX, NY>::SLOTS;
}

static inline int shape_key(int nx, int ny) { return nx * 1024 + ny; }

template <typename T, int NZ>
static constexpr int z_threads() {
  constexpr int t = ZCfg<T>::M * Plan<NZ>::G;
  return t < 64 ? 64 : t;
}

template <typename T, int NZ>
static void launch_z_step(const ChainJob<T>* jobs, int t, int nkp, double ng, int njobs, const Twiddles<T>& tw,
                          cudaStream_t st) {
  constexpr int M = ZCfg<T>::M;
  const size_t sz = sizeof(Cx<T>) * (size_t)(NZ + 1) * M;
  static bool attr = false;
  if (!attr) {
    set_smem(z_step_kernel<T, NZ>, sz);
    attr = true;
  }
  const int ntiles = (nkp + M - 1) / M;
  z_step_kernel<T, NZ><<<dim3(ntiles, njobs), z_threads<T, NZ>(), sz, st>>>(jobs, t, nkp, ng, tw);
    count_launches(1);
}

template <typename T>
static bool z_step_dispatch(int nz, const ChainJob<T>* jobs, int t, int nkp, double ng, int njobs,
                            const Twiddles<T>& tw,
                            cudaStream_t st) {
  switch (nz) {
#define PF_Z(N)                                           \
  case N:                                                 \
    launch_z_step<T, N>(jobs, t, nkp, ng, njobs, tw, st); \
    return true;
    PF_Z_LENGTHS(PF_Z)
#undef PF_Z
    default:
      return false;
  }
}

template <typename T, int NX, int NY>
static void chains_shape(const ChainJob<T>* jobs, int njobs, int maxsteps, int nz, const Twiddles<T>& tw,
                         cudaStream_t st) {
  using C = PlaneCfg<NX, NY>;
  constexpr size_t sp = plane_smem<T, NX, NY>();
  static bool attr = false;
  if (!attr) {
    set_smem(chain_plane_kernel<T, NX, NY>, sp);
    set_smem(xy_step_kernel<T, NX, NY>, sp);
    attr = true;
  }
  if (nz == 1) {
    chain_plane_kernel<T, NX, NY><<<njobs, C::THREADS, sp, st>>>(jobs, tw);
    count_launches(1);
    return;
  }
  for (int t = 0; t <= maxsteps; ++t) {
    xy_step_kernel<T, NX, NY><<<dim3(nz, njobs), C::THREADS, sp, st>>>(jobs, t, nz, tw);
    count_launches(1);
    if (t < maxsteps) z_step_dispatch<T>(nz, jobs, t, C::NKP, (double)C::NP * nz, njobs, tw, st);
  }
}

template <typename T, int NX, int NY>
static void stress_shape(const StressItem<T>* items, int nitems, const T* const* src_q, const T* const* src_qc,
                         Cx<T>* const* kq, Cx<T>* const* kqc, int nz, const double* dksq, int nparams,
                         double* part, const Twiddles<T>& tw, cudaStream_t st) {
  using C = PlaneCfg<NX, NY>;
  constexpr size_t sp = plane_smem<T, NX, NY>();
  constexpr size_t ss = sp + sizeof(T) * (size_t)C::NKP;
  static bool attr = false;
  if (!attr) {
    set_smem(stress_plane_kernel<T, NX, NY>, ss);
    set_smem(xy_fwd_kernel<T, NX, NY>, sp);
    attr = true;
  }
  if (nz == 1) {
    stress_plane_kernel<T, NX, NY><<<nitems, C::THREADS, ss, st>>>(items, dksq, nparams, part, tw);
    count_launches(1);
    return;
  }
  xy_fwd_kernel<T, NX, NY><<<dim3(nz, nitems), C::THREADS, sp, st>>>(src_q, kq, tw);
    count_launches(1);
  xy_fwd_kernel<T, NX, NY><<<dim3(nz, nitems), C::THREADS, sp, st>>>(src_qc, kqc, tw);
    count_launches(1);
  constexpr int M = ZCfg<T>::M;
  const int ntiles = (C::NKP + M - 1) / M;
  switch (nz) {
#define PF_Z(N)                                                                                              \
  case N: {                                                                                                  \
    const size_t sz = 2 * sizeof(Cx<T>) * (size_t)(N + 1) * M;                                               \
    static bool za = false;                                                                                  \
    if (!za) {                                                                                               \
      set_smem(z_fwd_stress_kernel<T, N>, sz);                                                               \
      za = true;                                                                                             \
    }                                                                                                        \
    z_fwd_stress_kernel<T, N><<<dim3(ntiles, nitems), z_threads<T, N>(), sz, st>>>(kq, kqc, C::NKP, dksq, nparams, part, tw); count_launches(1); \
  } break;
    PF_Z_LENGTHS(PF_Z)
#undef PF_Z
    default:
      break;
  }
}

// Whether kernels exist for this grid (and fit the shared memory of one CTA).
template <typename T>
bool shape_supported(int nx, int ny, int nz) {
  bool plane = false;
  switch (shape_key(nx, ny)) {
#define PF_S(A, B)                                                                        \
  case A * 1024 + B:                                                                      \
    plane = plane_smem<T, A, B>() + sizeof(T) * PlaneCfg<A, B>::NKP <= 227 * 1024;         \
    break;
    PF_PLANE_SHAPES(PF_S)
#undef PF_S
    default:
      plane = false;
  }
  return plane && (nz == 1 || fft_length_supported(nz));
}

template <typename T>
void launch_lw(T* lw, const double* w, double coeff, long n, cudaStream_t st) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  lw_kernel<T><<<blocks, 256, 0, st>>>(lw, w, coeff, n);
    count_launches(1);
}

template <typename T>
void launch_ld(T* ld, const CellGeom& g, double coeff, double scale, long nk, cudaStream_t st) {
  int blocks = (int)((nk + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  ld_kernel<T><<<blocks, 256, 0, st>>>(ld, g, coeff, scale);
    count_launches(1);
}

template <typename T>
void launch_fill(T* a, T v, long n, cudaStream_t st) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  fill_kernel<T><<<blocks, 256, 0, st>>>(a, v, n);
    count_launches(1);
}

template <typename T>
void launch_chains(const ChainJob<T>* jobs_dev, int njobs, int maxsteps, const GridDims& d, const Twiddles<T>& tw,
                   cudaStream_t st) {
  switch (shape_key(d.nx, d.ny)) {
#define PF_S(A, B)                                                   \
  case A * 1024 + B:                                                 \
    chains_shape<T, A, B>(jobs_dev, njobs, maxsteps, d.nz, tw, st);  \
    break;
    PF_PLANE_SHAPES(PF_S)
#undef PF_S
    default:
      break;
  }
}

template <typename T>
void launch_stress(const StressItem<T>* items, int nitems, const T* const* src_q, const T* const* src_qc,
                   Cx<T>* const* kq, Cx<T>* const* kqc, const GridDims& d, const double* dksq, int nparams,
                   double* part, const Twiddles<T>& tw, cudaStream_t st) {
  switch (shape_key(d.nx, d.ny)) {
#define PF_S(A, B)                                                                                   \
  case A * 1024 + B:                                                                                 \
    stress_shape<T, A, B>(items, nitems, src_q, src_qc, kq, kqc, d.nz, dksq, nparams, part, tw, st); \
    break;
    PF_PLANE_SHAPES(PF_S)
#undef PF_S
    default:
      break;
  }
}

#define PF_INST(T)                                                                                         \
  template bool shape_supported<T>(int, int, int);                                                         \
  template void launch_lw<T>(T*, const double*, double, long, cudaStream_t);                              \
  template void launch_ld<T>(T*, const CellGeom&, double, double, long, cudaStream_t);                    \
  template void launch_fill<T>(T*, T, long, cudaStream_t);                                                \
  template void launch_chains<T>(const ChainJob<T>*, int, int, const GridDims&, const Twiddles<T>&,       \
                                 cudaStream_t);                                                            \
  template void launch_stress<T>(const StressItem<T>*, int, const T* const*, const T* const*, Cx<T>* const*, \
                                 Cx<T>* const*, const GridDims&, const double*, int, double*,              \
                                 const Twiddles<T>&, cudaStream_t);

}  // namespace pf
