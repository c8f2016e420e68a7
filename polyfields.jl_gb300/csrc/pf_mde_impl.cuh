// Pseudo-spectral MDE propagator kernels (reference: src/system/mde.jl:43-104 with the FFTW
// plans of src/system/fft.jl) and the stress transforms (src/species/multiblock.jl:233-295).
//
// One RK2 contour step is  q_{s+1} = LW * irfft( LD * rfft( LW * q_s ) )  with
// LW = exp(-ds vol w / 2) on the real grid and LD = exp(-ds b^2 k^2 / 6) / Ng on the half
// spectrum (the 1/Ng of the normalised irfft folded in).
//
// Layout in HBM: a real grid is Nz planes of Ny rows of Nx values, x fastest (the
// reference's column-major Array{Float64,3}[x,y,z]).  Half-spectrum arrays of the engine
// (LD, dksq, the 3D scratch) are Nz planes of Kx = Nx/2+1 columns of Ny values, ky fastest:
// [kz][kx][ky].  A propagator history is (Ns+1) consecutive grids.
//
// A plane (one z slice) is transformed by one CTA: the real rows 2p, 2p+1 ride one complex
// FFT along x (two-for-one), the Kx columns are transformed along y.  Row pairs and columns
// share one shared-memory buffer S of Kx * max(Ny, 2) complex values: pair p owns the span
// S[2p Kx, 2p Kx + 2 Kx) and column kx the strided elements S[y Kx + kx].  Transform passes
// read and write global memory directly where they can (first y-inverse pass, last
// y-forward pass, first and last z pass), and the x-inverse -> LW -> store q -> LW ->
// x-forward sequence and the LD multiplies happen in registers between two passes.
//
// Grids with Nz == 1 (1D and 2D systems): one persistent CTA per chain runs all contour
// steps (chain_plane_kernel).  3D grids: each step is a plane pass (xy_step_kernel, one CTA
// per z plane) and a pencil pass (z_pipe_kernel, tiles of 16 or 8 pencils staged by TMA); the
// plane pass of step t fuses the end of step t-1 with the start of step t.  Independent
// chains (forward q, backward qc, other species) run on their own streams and overlap.
//
// Every kernel is specialised on its transform lengths at compile time; the host picks the
// instantiation from the supported plane shapes below.
#pragma once
#include "pf_fft.cuh"
#include "pf_kernels.h"
#include "pf_tma.cuh"
#include <cudaTypedefs.h>
#include <map>
#include <mutex>
#include <stdexcept>
#include <utility>

namespace pf {

// Plane shapes (Nx, Ny) with kernels: 1D rows, square planes and 2:1 rectangles.
#define PF_PLANE_SHAPES(X)                                                                    \
  X(8, 1) X(16, 1) X(32, 1) X(48, 1) X(64, 1) X(96, 1) X(128, 1) X(256, 1) X(16, 16) X(32, 32) \
  X(48, 48) X(64, 64) X(96, 96) X(128, 128) X(32, 16) X(64, 32) X(96, 48) X(128, 64)
#define PF_Z_LENGTHS(X) X(8) X(16) X(32) X(48) X(64) X(96) X(128) X(256)

__host__ __device__ constexpr int round32(int n) { return (n + 31) / 32 * 32; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

// twiddle entries of both orders of a length (1 for a length-1 axis, which has no transform)
template <int N>
__host__ __device__ constexpr int tw_total() {
  if constexpr (N > 1) return Order<N, 0>::TW_SIZE + Order<N, 1>::TW_SIZE;
  else return 1;
}
template <int N>
__host__ __device__ constexpr int plan_group() {
  if constexpr (N > 1) return Plan<N>::G;
  else return 1;
}

template <int NX, int NY>
struct PlaneCfg {
  static constexpr int KX = NX / 2 + 1;
  static constexpr int NKP = KX * NY;                    // half-spectrum points of a plane
  static constexpr int NP = NX * NY;                     // real points of a plane
  static constexpr int SLOTS = KX * (NY > 1 ? NY : 2);   // complex slots of S
  static constexpr int NPAIR = NY > 1 ? NY / 2 : 1;
  static constexpr int GX = Plan<NX>::G;
  static constexpr int GY = plan_group<NY>();
  static constexpr int SP = pair_stride<NX>();
  static constexpr int SC = NY > 1 ? col_stride<NY>() : 1;
  // one group per row pair and one per column, all in one round
  static constexpr int THREADS =
      32 * cmax(warps_for<GX, SP>(NPAIR), NY > 1 ? warps_for<(NY > 1 ? plan_group<NY>() : 32), SC>(KX) : 1);
  static constexpr int TWX = tw_total<NX>();
  static constexpr int TWY = tw_total<NY>();
  // the whole register file for one CTA (persistent chain kernels run one CTA per SM): each of
  // the SM's four sub-partitions holds 16384 registers for ceil(warps / 4) of the CTA's warps
  static constexpr int WPS = (THREADS / 32 + 3) / 4;
  static constexpr int MAXREG = (16384 / (WPS * 32) / 8 * 8) > 255 ? 255 : (16384 / (WPS * 32) / 8 * 8);
};

template <typename T>
struct ZCfg {
  static constexpr int M = sizeof(T) == 4 ? 16 : 8;  // pencils per tile (128-byte rows)
};

// ------------------------------------------------------------------ operator setup
// LW = exp(-coeff * w) evaluated in float64 and rounded once to T: the propagator multiplies
// by LW twice per contour step, so a biased float32 exp would compound over the chain.
template <typename T>
__global__ void lw_kernel(T* __restrict__ lw, const double* __restrict__ w, double coeff, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    lw[i] = (T)exp(-coeff * w[i]);
}

// Wavevector index along y or z: the reference's fold of src/system/cell.jl:273-277 (quirk Q1:
// |j|, not signed j), or with g.signed_k the signed frequency j - n above n/2 (the Nyquist
// index stays +n/2).  The two give the same |k|^2 in orthogonal cells.
__device__ __forceinline__ double fold_index(const CellGeom& g, int i, int n) {
  return (double)((i <= n / 2) ? i : (g.signed_k ? i - n : n - i));
}

__device__ __forceinline__ double ksq_at(const CellGeom& g, int ix, int iy, int iz) {
  const double jx = ix, jy = fold_index(g, iy, g.ny), jz = fold_index(g, iz, g.nz);
  // kvec = G * jvec, G columns = reciprocal vectors (row-major storage G[r*3+c])
  const double kx = g.G[0] * jx + g.G[1] * jy + g.G[2] * jz;
  const double ky = g.G[3] * jx + g.G[4] * jy + g.G[5] * jz;
  const double kz = g.G[6] * jx + g.G[7] * jy + g.G[8] * jz;
  return kx * kx + ky * ky + kz * kz;
}

// (ix, iy, iz) of half-spectrum index i in the [kz][kx][ky] layout
__device__ __forceinline__ void spectral_index(const CellGeom& g, long i, int& ix, int& iy, int& iz) {
  const long nkp = (long)(g.nx / 2 + 1) * g.ny;
  iz = (int)(i / nkp);
  const long r = i - (long)iz * nkp;
  ix = (int)(r / g.ny);
  iy = (int)(r - (long)ix * g.ny);
}

template <typename T>
__global__ void ld_kernel(T* __restrict__ ld, CellGeom g, double coeff, double scale) {
  const long nk = (long)(g.nx / 2 + 1) * g.ny * g.nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nk; i += (long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    spectral_index(g, i, ix, iy, iz);
    ld[i] = (T)(exp(-coeff * ksq_at(g, ix, iy, iz)) * scale);
  }
}

// dksq for every cell parameter (src/system/cell.jl:292-320), nparams grids of Nk.
static __global__ void dksq_kernel(double* __restrict__ dk, CellGeom g, int nparams) {
  const long nk = (long)(g.nx / 2 + 1) * g.ny * g.nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nk; i += (long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    spectral_index(g, i, ix, iy, iz);
    const double j[3] = {(double)ix, fold_index(g, iy, g.ny), fold_index(g, iz, g.nz)};
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

template <typename T>
__device__ __forceinline__ void stage(Cx<T>* dst, const Cx<T>* __restrict__ src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// ------------------------------------------------------------------ plane pipeline pieces
// Registers at the x join: z(x) = (row 2p, row 2p+1) at positions Join<NX>::pos.
template <typename T, int NX>
struct XRegs {
  Cx<T> v[Join<NX>::BPT][Join<NX>::R];
};
// Registers at the y (or z) forward -> inverse join: positions JoinBA<N>::pos.
template <typename T, int N>
struct BARegs {
  Cx<T> v[JoinBA<N>::BPT][JoinBA<N>::R];
};

// Inputs of the first column pass (inverse, order A) of one group: column c of the [kx][ky]
// global plane.
template <typename T, int NY>
struct ColIn {
  using P0 = PassOf<T, true, NY, 0, 0>;
  Cx<T> v[P0::BPT][Order<NY, 0>::radix(0)];
};

template <typename T>
__device__ __forceinline__ Cx<T> ld_l2(const Cx<T>* p) {
  if constexpr (sizeof(T) == 4) {
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return cx<T>(v.x, v.y);
  } else {
    const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
    return cx<T>(v.x, v.y);
  }
}

// Issue the loads of the first column pass from the global plane kin (cached in L2 only: the
// plane is read once).  Independent of shared memory, so it can run before the twiddles are
// staged.
template <typename T, int NX, int NY>
__device__ __forceinline__ void y_inverse_load(ColIn<T, NY>& in, const Cx<T>* __restrict__ kin) {
  using C = PlaneCfg<NX, NY>;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), g = threadIdx.x % C::GY;
  if (c < C::KX) ColIn<T, NY>::P0::load(in.v, g, [&](int i) { return ld_l2<T>(kin + c * NY + i); });
}

// Column transforms, inverse, order A, from the loaded inputs into S[y Kx + kx].  Group c < Kx
// handles column c.  The caller syncs the CTA afterwards.
template <typename T, int NX, int NY>
__device__ __forceinline__ void y_inverse_from_loaded(Cx<T>* S, ColIn<T, NY>& in, const Cx<T>* twy) {
  using C = PlaneCfg<NX, NY>;
  constexpr int P = Order<NY, 0>::P;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), g = threadIdx.x % C::GY;
  const bool active = c < C::KX;
  Cx<T>* col = S + (active ? c : 0);
  using P0 = typename ColIn<T, NY>::P0;
  if (active) {
    P0::compute(in.v, g, twy);
    P0::store(in.v, g, [&](int i, const Cx<T>& x) { col[(P > 1 ? pswz<NY>(i) : i) * C::KX] = x; });
  }
  __syncwarp();
  smem_passes<T, true, NY, 0, 1, P, true, false>(col, C::KX, g, twy, active);
}

// Column transforms, inverse, order A, starting from registers at the forward -> inverse join
// (after the LD multiply) and ending in S[y Kx + c].  The caller syncs the CTA afterwards.
template <typename T, int NX, int NY>
__device__ __forceinline__ void y_inverse_from_regs(Cx<T>* S, const Cx<T>* twy, BARegs<T, NY>& w, int c, int g,
                                                    bool active) {
  using C = PlaneCfg<NX, NY>;
  constexpr int P = Order<NY, 0>::P;
  Cx<T>* col = S + (active ? c : 0);
  using P0 = PassOf<T, true, NY, 0, 0>;
  if (active) {
    P0::compute(w.v, g, twy);
    P0::store(w.v, g, [&](int i, const Cx<T>& x) { col[(P > 1 ? pswz<NY>(i) : i) * C::KX] = x; });
  }
  __syncwarp();
  smem_passes<T, true, NY, 0, 1, P, true, false>(col, C::KX, g, twy, active);
}

// Row-pair transforms, inverse, order A: the half spectra of rows 2p, 2p+1 in S -> registers at
// the x join.  The first pass builds z(x) = A(x) + i B(x) from the Hermitian halves.  Needs the
// CTA synced before (S written by the column transforms).
template <typename T, int NX, int NY>
__device__ __forceinline__ void x_inverse_to_regs(Cx<T>* S, const Cx<T>* twx, XRegs<T, NX>& out, int p, int g,
                                                  bool active) {
  using C = PlaneCfg<NX, NY>;
  constexpr int P = Order<NX, 0>::P;
  Cx<T>* z = S + (active ? p : 0) * 2 * C::KX;
  auto build = [&](int x) {
    Cx<T> A, B;
    if (x <= NX / 2) {
      A = z[x];
      B = NY > 1 ? z[C::KX + x] : cx<T>(0, 0);
    } else {
      A = conj(z[NX - x]);
      B = NY > 1 ? conj(z[C::KX + NX - x]) : cx<T>(0, 0);
    }
    return cx<T>(A.x - B.y, A.y + B.x);
  };
  using P0 = PassOf<T, true, NX, 0, 0>;
  if constexpr (P == 1) {
    if (active) {
      P0::load(out.v, g, build);
      P0::compute(out.v, g, twx);
    }
    __syncwarp();
  } else {
    Cx<T> v[P0::BPT][Order<NX, 0>::radix(0)];
    if (active) {
      P0::load(v, g, build);
      P0::compute(v, g, twx);
    }
    __syncwarp();
    if (active) P0::store(v, g, [&](int i, const Cx<T>& x) { z[pswz<NX>(i)] = x; });
    __syncwarp();
    smem_passes<T, true, NX, 0, 1, P - 1, true, true>(z, 1, g, twx, active);
    using PL = PassOf<T, true, NX, 0, P - 1>;
    if (active) {
      PL::load(out.v, g, [&](int i) { return z[pswz<NX>(i)]; });
      PL::compute(out.v, g, twx + Order<NX, 0>::tw_offset(P - 1));
    }
    __syncwarp();
  }
}

// Row-pair transforms, forward, order B: registers at the x join -> z(x) in the pair's span of S
// (natural order).  The caller syncs the CTA afterwards.
template <typename T, int NX, int NY>
__device__ __forceinline__ void x_forward_from_regs(Cx<T>* S, const Cx<T>* twx, XRegs<T, NX>& in, int p, int g,
                                                    bool active) {
  using C = PlaneCfg<NX, NY>;
  constexpr int P = Order<NX, 1>::P;
  Cx<T>* z = S + (active ? p : 0) * 2 * C::KX;
  const Cx<T>* twb = twx + Order<NX, 0>::TW_SIZE;
  using P0 = PassOf<T, false, NX, 1, 0>;
  if (active) {
    P0::compute(in.v, g, twb);
    P0::store(in.v, g, [&](int i, const Cx<T>& x) { z[P > 1 ? pswz<NX>(i) : i] = x; });
  }
  __syncwarp();
  smem_passes<T, false, NX, 1, 1, P, true, false>(z, 1, g, twb, active);
}

// Column transforms, forward, order B, ending in registers (positions JoinBA<NY>::pos of column
// c).  The first pass unpacks the row pairs' spectra, A = (Z_k + conj Z_{N-k})/2 (row 2p) and
// B = (Z_k - conj Z_{N-k})/(2i) (row 2p+1); a CTA-wide barrier separates its reads of every
// pair span from its writes (all columns are handled in one round).  Needs the CTA synced
// before (S written by the row transforms).
template <typename T, int NX, int NY>
__device__ __forceinline__ void y_forward_to_regs(Cx<T>* S, const Cx<T>* twy, BARegs<T, NY>& out, int c, int g,
                                                  bool active) {
  using C = PlaneCfg<NX, NY>;
  constexpr int P = Order<NY, 1>::P;
  const Cx<T>* twb = twy + Order<NY, 0>::TW_SIZE;
  auto unpack = [&](int y) {
    const Cx<T>* z = S + (y >> 1) * 2 * C::KX;
    const Cx<T> zk = z[c];
    const Cx<T> zn = z[(NX - c) % NX];
    return (y & 1) ? cx<T>((T)0.5 * (zk.y + zn.y), (T)0.5 * (zn.x - zk.x))
                   : cx<T>((T)0.5 * (zk.x + zn.x), (T)0.5 * (zk.y - zn.y));
  };
  using P0 = PassOf<T, false, NY, 1, 0>;
  if constexpr (P == 1) {
    if (active) {
      P0::load(out.v, g, unpack);
      P0::compute(out.v, g, twb);
    }
    __syncthreads();
  } else {
    Cx<T> v[P0::BPT][Order<NY, 1>::radix(0)];
    if (active) {
      P0::load(v, g, unpack);
      P0::compute(v, g, twb);
    }
    __syncthreads();
    Cx<T>* col = S + (active ? c : 0);
    if (active) P0::store(v, g, [&](int i, const Cx<T>& x) { col[pswz<NY>(i) * C::KX] = x; });
    __syncwarp();
    smem_passes<T, false, NY, 1, 1, P - 1, true, true>(col, C::KX, g, twb, active);
    using PL = PassOf<T, false, NY, 1, P - 1>;
    if (active) {
      PL::load(out.v, g, [&](int i) { return col[pswz<NY>(i) * C::KX]; });
      PL::compute(out.v, g, twb + Order<NY, 1>::tw_offset(P - 1));
    }
    __syncwarp();
  }
}

// Finish step t-1 and start step t on the registers of one row pair:
// q = lw_cur * (cs * r) is stored; u = lw_next * q goes back into the registers.  Inside a
// block lw_next is lw_cur (the same array), which is then read once.
template <typename T, int NX, int NY>
__device__ __forceinline__ void finish_regs(XRegs<T, NX>& r, int p, int g, const T* __restrict__ lw_cur,
                                            const T* __restrict__ lw_next, T* __restrict__ qout, T cs) {
  using J = Join<NX>;
  const int y0 = 2 * p, y1 = 2 * p + 1;
  const bool same = lw_next == lw_cur;
#pragma unroll
  for (int b = 0; b < J::BPT; ++b)
#pragma unroll
    for (int t = 0; t < J::R; ++t) {
      const int x = J::pos(g, b, t);
      const int i0 = y0 * NX + x, i1 = y1 * NX + x;
      const T l0 = __ldg(lw_cur + i0);
      const T q0 = l0 * (r.v[b][t].x * cs);
      __stcs(qout + i0, q0);  // history: streamed past L2, which keeps LW and the spectra
      T l1 = (T)0, q1 = (T)0;
      if constexpr (NY > 1) {
        l1 = __ldg(lw_cur + i1);
        q1 = l1 * (r.v[b][t].y * cs);
        __stcs(qout + i1, q1);
      }
      if (lw_next) {
        const T n0 = same ? l0 : __ldg(lw_next + i0);
        const T n1 = NY > 1 ? (same ? l1 : __ldg(lw_next + i1)) : (T)0;
        r.v[b][t] = cx<T>(n0 * q0, n1 * q1);
      }
    }
}

// u = lw * q (q alone when lw is null) into the registers of one row pair at the x join.
template <typename T, int NX, int NY>
__device__ __forceinline__ void load_regs(XRegs<T, NX>& r, int p, int g, const T* __restrict__ lw,
                                          const T* __restrict__ q) {
  using J = Join<NX>;
  const int y0 = 2 * p, y1 = 2 * p + 1;
#pragma unroll
  for (int b = 0; b < J::BPT; ++b)
#pragma unroll
    for (int t = 0; t < J::R; ++t) {
      const int x = J::pos(g, b, t);
      const int i0 = y0 * NX + x, i1 = y1 * NX + x;
      const T a = lw ? lw[i0] * q[i0] : q[i0];
      T b1 = (T)0;
      if constexpr (NY > 1) b1 = lw ? lw[i1] * q[i1] : q[i1];
      r.v[b][t] = cx<T>(a, b1);
    }
}

// 1D rows: forward transform (order B) of the registers at the x join into registers at the
// B -> A join (full complex spectrum of the real row, natural positions).
template <typename T, int NX>
__device__ __forceinline__ void row_forward_1d(Cx<T>* z, const Cx<T>* twx, XRegs<T, NX>& r, BARegs<T, NX>& w, int g,
                                               bool active) {
  constexpr int P = Order<NX, 1>::P;
  const Cx<T>* twb = twx + Order<NX, 0>::TW_SIZE;
  using P0 = PassOf<T, false, NX, 1, 0>;
  if constexpr (P == 1) {
    if (active) {
      P0::compute(r.v, g, twb);
#pragma unroll
      for (int b = 0; b < JoinBA<NX>::BPT; ++b)
#pragma unroll
        for (int t = 0; t < JoinBA<NX>::R; ++t) w.v[b][t] = r.v[b][t];
    }
  } else {
    if (active) {
      P0::compute(r.v, g, twb);
      P0::store(r.v, g, [&](int i, const Cx<T>& x) { z[pswz<NX>(i)] = x; });
    }
    __syncwarp();
    smem_passes<T, false, NX, 1, 1, P - 1, true, true>(z, 1, g, twb, active);
    using PL = PassOf<T, false, NX, 1, P - 1>;
    if (active) {
      PL::load(w.v, g, [&](int i) { return z[pswz<NX>(i)]; });
      PL::compute(w.v, g, twb + Order<NX, 1>::tw_offset(P - 1));
    }
    __syncwarp();
  }
}

// 1D rows: inverse transform (order A) from registers at the B -> A join into registers at the
// x join.
template <typename T, int NX>
__device__ __forceinline__ void row_inverse_1d(Cx<T>* z, const Cx<T>* twx, BARegs<T, NX>& w, XRegs<T, NX>& r, int g,
                                               bool active) {
  constexpr int P = Order<NX, 0>::P;
  using P0 = PassOf<T, true, NX, 0, 0>;
  if constexpr (P == 1) {
    if (active) {
      P0::compute(w.v, g, twx);
#pragma unroll
      for (int b = 0; b < Join<NX>::BPT; ++b)
#pragma unroll
        for (int t = 0; t < Join<NX>::R; ++t) r.v[b][t] = w.v[b][t];
    }
  } else {
    if (active) {
      P0::compute(w.v, g, twx);
      P0::store(w.v, g, [&](int i, const Cx<T>& x) { z[pswz<NX>(i)] = x; });
    }
    __syncwarp();
    smem_passes<T, true, NX, 0, 1, P - 1, true, true>(z, 1, g, twx, active);
    using PL = PassOf<T, true, NX, 0, P - 1>;
    if (active) {
      PL::load(r.v, g, [&](int i) { return z[pswz<NX>(i)]; });
      PL::compute(r.v, g, twx + Order<NX, 0>::tw_offset(P - 1));
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ Nz == 1 chains
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS) __maxnreg__((PlaneCfg<NX, NY>::MAXREG))
    chain_plane_kernel(const ChainJob<T>* __restrict__ jobs, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  __shared__ Cx<T> twx[C::TWX], twy[C::TWY];
  __shared__ T cshare;
  stage<T>(twx, twg.x, C::TWX);
  if (NY > 1) stage<T>(twy, twg.y, C::TWY);
  const ChainJob<T> job = jobs[blockIdx.x];
  const int p = group_index<C::GX, C::SP>(threadIdx.x / C::GX), gx = threadIdx.x % C::GX;
  const bool xact = p < C::NPAIR;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), gy = threadIdx.x % C::GY;
  const bool yact = NY > 1 && c < C::KX;
  XRegs<T, NX> r;
  __syncthreads();
  if (xact) load_regs<T, NX, NY>(r, p, gx, job.ops[0].lw, job.hist + (long)job.s0 * C::NP);
#pragma unroll 1
  for (int t = 0; t < job.nsteps; ++t) {
    const StepOp<T> op = job.ops[t];
    if constexpr (NY == 1) {
      // forward row transform -> LD (and rescale) in registers -> inverse row transform
      BARegs<T, NX> w;
      row_forward_1d<T, NX>(S, twx, r, w, gx, xact);
      T cs = (T)1;
      if (job.csc) {
        T c0 = (T)0;
        if (xact && gx == 0) c0 = rescale_factor<T>(w.v[0][0].x, (double)C::NP);  // DC at position 0
        cs = __shfl_sync(0xffffffffu, c0, 0);
        if (threadIdx.x == 0) {
          job.csc[t] = (float)cs;
          job.lsc[t] = log((double)cs);
        }
      }
      if (xact) {
#pragma unroll
        for (int b = 0; b < JoinBA<NX>::BPT; ++b)
#pragma unroll
          for (int tt = 0; tt < JoinBA<NX>::R; ++tt) {
            const int x = JoinBA<NX>::pos(gx, b, tt);
            const T f = op.ld[x <= NX / 2 ? x : NX - x] * cs;
            w.v[b][tt] = cx<T>(w.v[b][tt].x * f, w.v[b][tt].y * f);
          }
      }
      row_inverse_1d<T, NX>(S, twx, w, r, gx, xact);
    } else {
      // forward x -> forward y -> LD (and rescale) in registers -> inverse y -> inverse x
      x_forward_from_regs<T, NX, NY>(S, twx, r, p, gx, xact);
      __syncthreads();
      BARegs<T, NY> w;
      y_forward_to_regs<T, NX, NY>(S, twy, w, c, gy, yact);
      T cs = (T)1;
      if (job.csc) {
        if (yact && c == 0 && gy == 0) cshare = rescale_factor<T>(w.v[0][0].x, (double)C::NP);
        __syncthreads();
        cs = cshare;
        if (threadIdx.x == 0) {
          job.csc[t] = (float)cs;
          job.lsc[t] = log((double)cs);
        }
      }
      if (yact) {
#pragma unroll
        for (int b = 0; b < JoinBA<NY>::BPT; ++b)
#pragma unroll
          for (int tt = 0; tt < JoinBA<NY>::R; ++tt) {
            const int ky = JoinBA<NY>::pos(gy, b, tt);
            const T f = op.ld[c * NY + ky] * cs;
            w.v[b][tt] = cx<T>(w.v[b][tt].x * f, w.v[b][tt].y * f);
          }
      }
      y_inverse_from_regs<T, NX, NY>(S, twy, w, c, gy, yact);
      __syncthreads();
      x_inverse_to_regs<T, NX, NY>(S, twx, r, p, gx, xact);
    }
    const int s_out = job.s0 + job.dir * (t + 1);
    const T* lw_next = (t + 1 < job.nsteps) ? job.ops[t + 1].lw : nullptr;
    if (xact) finish_regs<T, NX, NY>(r, p, gx, op.lw, lw_next, job.hist + (long)s_out * C::NP, (T)1);
    if (NY > 1) __syncthreads();  // the next step's row transforms overwrite S
  }
}

// ------------------------------------------------------------------ 3D: plane pass
#ifndef PF_XY_MINB
#define PF_XY_MINB 2
#endif



// Two CTAs per SM for float planes.  Float64 instantiations take the registers of a whole SM:
// a 128 x 65 half-spectrum plane (133 KB of shared memory) fits once per SM anyway, and a
// two-CTA bound (56 registers) made the float64 transforms spill.
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS, sizeof(T) == 8 ? 1 : PF_XY_MINB)
    xy_step_kernel(const ChainJob<T>* __restrict__ jobs, int t, int nz, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  static_assert(NY > 1, "3D grids have Ny > 1");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  const ChainJob<T> job = jobs[blockIdx.y];
  if (t > job.nsteps) return;
  __shared__ Cx<T> twx[C::TWX], twy[C::TWY];
  const int z = blockIdx.x;
  const long ng = (long)C::NP * nz;
  const bool finish = t >= 1;
  const bool start = t < job.nsteps;
  const int p = group_index<C::GX, C::SP>(threadIdx.x / C::GX), gx = threadIdx.x % C::GX;
  const bool xact = p < C::NPAIR;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), gy = threadIdx.x % C::GY;
  const bool yact = c < C::KX;
  // Launched as a programmatic dependent of the previous pencil pass: what does not depend on
  // that pass (the step operators, the twiddles) is read before grid_dep_wait, overlapping the
  // pencil pass's tail; the spectra and the rescale factor after it.
  const T* lw_cur = nullptr;
  const T* lw_next = nullptr;
  T cs = (T)1;
  ColIn<T, NY> in;
  if (finish) lw_cur = job.ops[t - 1].lw + (long)z * C::NP;
  if (start) lw_next = job.ops[t].lw + (long)z * C::NP;
  stage<T>(twx, twg.x, C::TWX);
  stage<T>(twy, twg.y, C::TWY);
  grid_dep_wait();  // the pencil pass of step t-1 (spectra, rescale factor) has completed
  if (finish) {
    if (job.csc) cs = (T)job.csc[t - 1];
    y_inverse_load<T, NX, NY>(in, job.kbuf + (long)z * C::NKP);
  }
  __syncthreads();
  XRegs<T, NX> r;
  if (finish) {
    y_inverse_from_loaded<T, NX, NY>(S, in, twy);
    __syncthreads();
    x_inverse_to_regs<T, NX, NY>(S, twx, r, p, gx, xact);
    const int s_out = job.s0 + job.dir * t;
    if (xact) finish_regs<T, NX, NY>(r, p, gx, lw_cur, lw_next, job.hist + (long)s_out * ng + (long)z * C::NP, cs);
  } else if (xact) {
    load_regs<T, NX, NY>(r, p, gx, job.ops[0].lw + (long)z * C::NP, job.hist + (long)job.s0 * ng + (long)z * C::NP);
  }
  if (start) {
    x_forward_from_regs<T, NX, NY>(S, twx, r, p, gx, xact);
    __syncthreads();
    BARegs<T, NY> w;
    y_forward_to_regs<T, NX, NY>(S, twy, w, c, gy, yact);
    grid_dep_launch();  // the pencil pass may be scheduled; it waits for these stores
    if (yact) {
      Cx<T>* dst = job.kbuf + (long)z * C::NKP + c * NY;
#pragma unroll
      for (int b = 0; b < JoinBA<NY>::BPT; ++b)
#pragma unroll
        for (int tt = 0; tt < JoinBA<NY>::R; ++tt) dst[JoinBA<NY>::pos(gy, b, tt)] = w.v[b][tt];
    }
  }
}

// ------------------------------------------------------------------ 3D: pencil pass through TMA
// The pencil pass as a pipeline: a tile is M pencils (M * sizeof(Cx<T>) = 128 bytes, one row
// per z) brought into shared memory by one 2D TMA copy, together with the matching LD tile (M
// values of T per row).  Lanes are assigned pencil-major: thread lt of a tile works on pencil
// m = lt % M as member g = lt / M of that pencil's G-thread group, so a warp touches whole
// 128-byte rows (M lanes per row) and every shared-memory access is conflict-free without a
// swizzle; an element's address is the thread's base plus a compile-time offset.  The G
// threads of a pencil sit in different warps, so the transform passes, which work in place on
// the tile, separate their loads from their stores with block barriers.  Each CTA runs several
// tiles through STAGES buffers; the copies of round k + STAGES - 1 are issued when round k
// starts, so they overlap its transforms.
// When a bounded wait gives up, the launch writes 1 to its owner's status word (a per-handle
// device int, read and cleared by the host) and its output is invalid.

template <typename T, int NZ, int STAGES_ = 3>
struct ZPipe {
  static constexpr int E = (int)sizeof(Cx<T>);
  static constexpr int M = 128 / E;              // pencils per tile
  static constexpr int G = Plan<NZ>::G;
  static constexpr int TT = M * G;               // threads per tile
  static constexpr int TPC = TT >= 128 ? 1 : 128 / TT;  // tiles per stage
  static constexpr int THREADS = TPC * TT;
  static constexpr int KB = NZ * 128;            // bytes of a spectrum tile
  static constexpr int LB = NZ * M * (int)sizeof(T);  // bytes of an LD tile
  static constexpr int STAGES = STAGES_;
  static constexpr int SMEM = STAGES * TPC * (KB + LB) + 1024;  // + alignment of the buffers
  // CTAs per SM that the shared memory allows (at most PF_ZMINB): the register budget follows
#ifndef PF_ZMINB
#define PF_ZMINB 4
#endif
  static constexpr int MINB =
      (200 * 1024 / SMEM) < 1 ? 1 : ((200 * 1024 / SMEM) > PF_ZMINB ? PF_ZMINB : (200 * 1024 / SMEM));
};

// Passes p in [P0, P1) of the transform of one pencil, in place on its tile column (element z
// at kt[z * M]), between block barriers.
template <typename T, bool INV, int N, int O, int P0, int P1>
__device__ __forceinline__ void ztile_passes(Cx<T>* kt, int g, const Cx<T>* tw, bool active) {
  constexpr int M = ZPipe<T, N>::M;
  if constexpr (P0 < P1) {
    using PS = PassOf<T, INV, N, O, P0>;
    Cx<T> v[PS::BPT][Order<N, O>::radix(P0)];
    if (active) {
      PS::load(v, g, [&](int i) { return kt[i * M]; });
      PS::compute(v, g, tw + Order<N, O>::tw_offset(P0));
    }
    __syncthreads();
    if (active) PS::store(v, g, [&](int i, const Cx<T>& x) { kt[i * M] = x; });
    __syncthreads();
    ztile_passes<T, INV, N, O, P0 + 1, P1>(kt, g, tw, active);
  }
}

// Forward z transform (order B) of one pencil (kt = tile + m), ending in registers at the
// B -> A join.
template <typename T, int NZ>
__device__ __forceinline__ void ztile_forward(Cx<T>* kt, int g, const Cx<T>* twb, BARegs<T, NZ>& w, bool active) {
  constexpr int P = Order<NZ, 1>::P;
  constexpr int M = ZPipe<T, NZ>::M;
  using F0 = PassOf<T, false, NZ, 1, 0>;
  if constexpr (P == 1) {
    if (active) {
      F0::load(w.v, g, [&](int i) { return kt[i * M]; });
      F0::compute(w.v, g, twb);
    }
  } else {
    Cx<T> v[F0::BPT][Order<NZ, 1>::radix(0)];
    if (active) {
      F0::load(v, g, [&](int i) { return kt[i * M]; });
      F0::compute(v, g, twb);
    }
    __syncthreads();
    if (active) F0::store(v, g, [&](int i, const Cx<T>& x) { kt[i * M] = x; });
    __syncthreads();
    ztile_passes<T, false, NZ, 1, 1, P - 1>(kt, g, twb, active);
    using FL = PassOf<T, false, NZ, 1, P - 1>;
    if (active) {
      FL::load(w.v, g, [&](int i) { return kt[i * M]; });
      FL::compute(w.v, g, twb + Order<NZ, 1>::tw_offset(P - 1));
    }
  }
  __syncthreads();
}

// Inverse z transform (order A) from registers at the join back into the tile, natural rows.
template <typename T, int NZ>
__device__ __forceinline__ void ztile_inverse(Cx<T>* kt, int g, const Cx<T>* twa, BARegs<T, NZ>& w, bool active) {
  constexpr int P = Order<NZ, 0>::P;
  constexpr int M = ZPipe<T, NZ>::M;
  using I0 = PassOf<T, true, NZ, 0, 0>;
  if constexpr (P == 1) {
    if (active) {
      I0::compute(w.v, g, twa);
      I0::store(w.v, g, [&](int i, const Cx<T>& x) { kt[i * M] = x; });
    }
  } else {
    if (active) {
      I0::compute(w.v, g, twa);
      I0::store(w.v, g, [&](int i, const Cx<T>& x) { kt[i * M] = x; });
    }
    __syncthreads();
    ztile_passes<T, true, NZ, 0, 1, P - 1>(kt, g, twa, active);
    using IL = PassOf<T, true, NZ, 0, P - 1>;
    Cx<T> v[IL::BPT][Order<NZ, 0>::radix(P - 1)];
    if (active) {
      IL::load(v, g, [&](int i) { return kt[i * M]; });
      IL::compute(v, g, twa + Order<NZ, 0>::tw_offset(P - 1));
    }
    __syncthreads();
    if (active) IL::store(v, g, [&](int i, const Cx<T>& x) { kt[i * M] = x; });
  }
}

// One contour step's pencil pass of one chain: forward z, LD (and, for tile 0, the rescale
// factor of the step from the (0,0,0) coefficient), inverse z.  kmap views the chain's
// half-spectrum scratch as rows of Nkp elements (8-byte units), lmap the step's LD.  A wait
// for a tile that gives up after wait_ns sets *status (when not null); the copies already
// issued are then drained with the default limit before the CTA exits.
template <typename T, int NZ, int STAGES>
__global__ void __launch_bounds__(ZPipe<T, NZ, STAGES>::THREADS, ZPipe<T, NZ, STAGES>::MINB)
    z_pipe_kernel(const __grid_constant__ CUtensorMap kmap, const __grid_constant__ CUtensorMap lmap,
                  float* __restrict__ csc, double* __restrict__ lsc, int t, int ntiles, double ng, Twiddles<T> twg,
                  int* __restrict__ status, unsigned long long wait_ns) {
  using Z = ZPipe<T, NZ, STAGES>;
  constexpr int S = Z::STAGES, TPC = Z::TPC, G = Z::G;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sbase = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  Cx<T>* ktiles = reinterpret_cast<Cx<T>*>(sbase);                    // [S][TPC] tiles of KB bytes
  T* ltiles = reinterpret_cast<T*>(sbase + (size_t)S * TPC * Z::KB);  // [S][TPC] tiles of LB bytes
  __shared__ __align__(8) uint64_t full[S];
  __shared__ __align__(16) Cx<T> twz[tw_total<NZ>()];
  const int nrounds = (ntiles + TPC - 1) / TPC;
  const int nk = (int)blockIdx.x < nrounds ? (nrounds - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  // twiddles ride on the first stage's bulk copies when the table is 16-byte aligned
  constexpr unsigned TWB = (unsigned)(sizeof(Cx<T>) * tw_total<NZ>());
  const bool tw_bulk = (TWB % 16 == 0) && ((reinterpret_cast<uintptr_t>(twg.z) & 15) == 0);
  if (!tw_bulk) stage<T>(twz, twg.z, tw_total<NZ>());
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  grid_dep_wait();  // the plane pass that wrote this step's spectra has completed
  const uint64_t keep = l2_evict_last();  // LD is read by every step of the chain's block
  auto issue = [&](int k) {  // thread 0: fill stage k % S with round k of this CTA
    const int s = k % S, r = (int)blockIdx.x + k * (int)gridDim.x;
    const int nt = min(TPC, ntiles - r * TPC);
    const bool tw = k == 0 && tw_bulk;
    mbar_expect_tx(&full[s], (unsigned)(nt * (Z::KB + Z::LB)) + (tw ? TWB : 0u));
    if (tw) bulk_load(twz, twg.z, TWB, &full[s]);
    for (int j = 0; j < nt; ++j) {
      const int tile = r * TPC + j;
      tma_load_2d(ktiles + (size_t)(s * TPC + j) * (Z::KB / Z::E), &kmap, tile * 16, 0, &full[s]);
      tma_load_2d_hint(ltiles + (size_t)(s * TPC + j) * (Z::LB / sizeof(T)), &lmap, tile * Z::M, 0, &full[s],
                       keep);
    }
  };
  if (threadIdx.x == 0)
    for (int k = 0; k < S - 1 && k < nk; ++k) issue(k);
  const int slot = threadIdx.x / Z::TT, lt = threadIdx.x % Z::TT;
  const int m = lt % Z::M, g = lt / Z::M;  // pencil-major lanes
  const Cx<T>* twb = twz + Order<NZ, 0>::TW_SIZE;
  int waited = 0;  // rounds whose stage completed
  bool ok = true;
#pragma unroll 1
  for (int k = 0; k < nk; ++k) {
    const int s = k % S, r = (int)blockIdx.x + k * (int)gridDim.x;
    const bool good = mbar_wait(&full[s], (unsigned)((k / S) & 1), wait_ns);
    if (__syncthreads_or(!good)) {
      ok = false;
      break;
    }
    waited = k + 1;
    // refill the stage that round k-1 used with round k + S - 1 now, so that its copies overlap
    // this round's transforms (the store of round k-1 must have finished reading that stage)
    if (threadIdx.x == 0 && k + S - 1 < nk) {
      bulk_wait_read<0>();
      issue(k + S - 1);
    }
    const int tile = r * TPC + slot;
    const bool active = tile < ntiles;
    Cx<T>* kt = ktiles + (size_t)(s * TPC + slot) * (Z::KB / Z::E) + m;
    const T* ltl = ltiles + (size_t)(s * TPC + slot) * (Z::LB / sizeof(T)) + m;
    BARegs<T, NZ> w;
    ztile_forward<T, NZ>(kt, g, twb, w, active);
    if (csc && r == 0 && threadIdx.x == 0) {
      // tile 0, pencil 0, position 0: the (0, 0, 0) coefficient = grid sum of LW * q_t
      const T c = rescale_factor<T>(w.v[0][0].x, ng);
      csc[t] = (float)c;
      lsc[t] = log((double)c);
    }
    if (active) {
#pragma unroll
      for (int b = 0; b < JoinBA<NZ>::BPT; ++b)
#pragma unroll
        for (int tt = 0; tt < JoinBA<NZ>::R; ++tt) {
          const T f = ltl[JoinBA<NZ>::pos(g, b, tt) * Z::M];
          w.v[b][tt] = cx<T>(w.v[b][tt].x * f, w.v[b][tt].y * f);
        }
    }
    if (k == nk - 1) grid_dep_launch();  // last round: the next plane pass may be scheduled
    ztile_inverse<T, NZ>(kt, g, twz, w, active);
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      const int nt = min(TPC, ntiles - r * TPC);
      for (int j = 0; j < nt; ++j)
        tma_store_2d(&kmap, (r * TPC + j) * 16, 0, ktiles + (size_t)(s * TPC + j) * (Z::KB / Z::E));
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) {
    bulk_wait<0>();
    if (!ok) {
      if (status) *status = 1;
      // drain the copies still in flight into this CTA's stages (bounded waits, default limit)
      const int issued = min(nk, waited + S - 1);
      for (int k = waited; k < issued; ++k) mbar_wait(&full[k % S], (unsigned)((k / S) & 1));
    }
  }
}

// ------------------------------------------------------------------ stress transforms
// Sum over the half spectrum of c_k Re(qhat_k) Re(qchat_k) dksq_p,k with c_0 = 1 and c_k = 2
// otherwise (quirk Q2, multiblock.jl:279-282), for every item (a contour point of a block).
// Nz == 1: one CTA per item transforms both planes.  Output part[item * nparams + p].
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS)
    stress_plane_kernel(const StressItem<T>* __restrict__ items, const double* __restrict__ dksq, int nparams,
                        double* __restrict__ part, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  T* req = reinterpret_cast<T*>(S + C::SLOTS);  // Re(qhat) in [kx][ky] order
  __shared__ Cx<T> twx[C::TWX], twy[C::TWY];
  __shared__ double red[kMaxParams][32];
  stage<T>(twx, twg.x, C::TWX);
  if (NY > 1) stage<T>(twy, twg.y, C::TWY);
  const StressItem<T> it = items[blockIdx.x];
  const int p = group_index<C::GX, C::SP>(threadIdx.x / C::GX), gx = threadIdx.x % C::GX;
  const bool xact = p < C::NPAIR;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), gy = threadIdx.x % C::GY;
  const bool yact = NY > 1 && c < C::KX;
  double acc[kMaxParams];
  for (int k = 0; k < kMaxParams; ++k) acc[k] = 0.0;
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    XRegs<T, NX> r;
    if (xact) load_regs<T, NX, NY>(r, p, gx, nullptr, pass == 0 ? it.q : it.qc);
    if constexpr (NY == 1) {
      BARegs<T, NX> w;
      row_forward_1d<T, NX>(S, twx, r, w, gx, xact);
      if (xact) {
#pragma unroll
        for (int b = 0; b < JoinBA<NX>::BPT; ++b)
#pragma unroll
          for (int tt = 0; tt < JoinBA<NX>::R; ++tt) {
            const int x = JoinBA<NX>::pos(gx, b, tt);
            if (x > NX / 2) continue;
            if (pass == 0) {
              req[x] = w.v[b][tt].x;
            } else {
              const double prod = (double)w.v[b][tt].x * (double)req[x] * (x == 0 ? 1.0 : 2.0);
              for (int k = 0; k < nparams; ++k) acc[k] += prod * dksq[(long)k * C::NKP + x];
            }
          }
      }
      __syncwarp();
    } else {
      x_forward_from_regs<T, NX, NY>(S, twx, r, p, gx, xact);
      __syncthreads();
      BARegs<T, NY> w;
      y_forward_to_regs<T, NX, NY>(S, twy, w, c, gy, yact);
      if (yact) {
#pragma unroll
        for (int b = 0; b < JoinBA<NY>::BPT; ++b)
#pragma unroll
          for (int tt = 0; tt < JoinBA<NY>::R; ++tt) {
            const int ky = JoinBA<NY>::pos(gy, b, tt);
            const int kk = c * NY + ky;
            if (pass == 0) {
              req[kk] = w.v[b][tt].x;
            } else {
              const double prod = (double)w.v[b][tt].x * (double)req[kk] * (kk == 0 ? 1.0 : 2.0);
              for (int k = 0; k < nparams; ++k) acc[k] += prod * dksq[(long)k * C::NKP + kk];
            }
          }
      }
    }
    __syncthreads();
  }
  for (int k = 0; k < nparams; ++k) {
    const double v = block_sum(acc[k], red[k]);
    if (threadIdx.x == 0) part[(long)blockIdx.x * nparams + k] = v;
  }
}

// 3D stress, plane pass: forward x/y transforms of the real grids src[item] into the
// half-spectrum buffers dst[item] ([kz][kx][ky]), one CTA per (z, item).
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS)
    xy_fwd_kernel(const T* const* __restrict__ src, Cx<T>* const* __restrict__ dst, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  static_assert(NY > 1, "3D grids have Ny > 1");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  __shared__ Cx<T> twx[C::TWX], twy[C::TWY];
  stage<T>(twx, twg.x, C::TWX);
  stage<T>(twy, twg.y, C::TWY);
  const int z = blockIdx.x;
  const int p = group_index<C::GX, C::SP>(threadIdx.x / C::GX), gx = threadIdx.x % C::GX;
  const bool xact = p < C::NPAIR;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), gy = threadIdx.x % C::GY;
  const bool yact = c < C::KX;
  __syncthreads();
  XRegs<T, NX> r;
  if (xact) load_regs<T, NX, NY>(r, p, gx, nullptr, src[blockIdx.y] + (long)z * C::NP);
  x_forward_from_regs<T, NX, NY>(S, twx, r, p, gx, xact);
  __syncthreads();
  BARegs<T, NY> w;
  y_forward_to_regs<T, NX, NY>(S, twy, w, c, gy, yact);
  if (yact) {
    Cx<T>* o = dst[blockIdx.y] + (long)z * C::NKP + c * NY;
#pragma unroll
    for (int b = 0; b < JoinBA<NY>::BPT; ++b)
#pragma unroll
      for (int tt = 0; tt < JoinBA<NY>::R; ++tt) o[JoinBA<NY>::pos(gy, b, tt)] = w.v[b][tt];
  }
}

// Forward z transform (order B) of one pencil from global into registers (JoinBA positions).
template <typename T, int NZ>
__device__ __forceinline__ void z_forward_to_regs(const Cx<T>* __restrict__ kb, long nkp, long col, Cx<T>* pen,
                                                  const Cx<T>* twz, BARegs<T, NZ>& w, int g, bool active) {
  constexpr int P = Order<NZ, 0>::P;
  const Cx<T>* twb = twz + Order<NZ, 0>::TW_SIZE;
  using F0 = PassOf<T, false, NZ, 1, 0>;
  if constexpr (P == 1) {
    if (active) {
      F0::load(w.v, g, [&](int i) { return kb[(long)i * nkp + col]; });
      F0::compute(w.v, g, twb);
    }
  } else {
    Cx<T> v[F0::BPT][Order<NZ, 1>::radix(0)];
    if (active) {
      F0::load(v, g, [&](int i) { return kb[(long)i * nkp + col]; });
      F0::compute(v, g, twb);
      F0::store(v, g, [&](int i, const Cx<T>& x) { pen[pswz<NZ>(i)] = x; });
    }
    __syncwarp();
    smem_passes<T, false, NZ, 1, 1, P - 1, true, true>(pen, 1, g, twb, active);
    using FL = PassOf<T, false, NZ, 1, P - 1>;
    if (active) {
      FL::load(w.v, g, [&](int i) { return pen[pswz<NZ>(i)]; });
      FL::compute(w.v, g, twb + Order<NZ, 1>::tw_offset(P - 1));
    }
    __syncwarp();
  }
}

// 3D stress, pencil pass: z transforms of both spectra of an item and the weighted sum over
// the tile.  Output part[(item * ntiles + tile) * nparams + p].
template <typename T, int NZ>
__global__ void __launch_bounds__(512)
    z_fwd_stress_kernel(Cx<T>* const* __restrict__ kq, Cx<T>* const* __restrict__ kqc, int nkp,
                        const double* __restrict__ dksq, int nparams, double* __restrict__ part, Twiddles<T> twg) {
  constexpr int M = ZCfg<T>::M;
  constexpr int LDT = NZ + pencil_pad<NZ>();
  constexpr int G = Plan<NZ>::G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* A = reinterpret_cast<Cx<T>*>(smem_raw);
  Cx<T>* B = A + M * LDT;
  __shared__ Cx<T> twz[tw_total<NZ>()];
  __shared__ double red[kMaxParams][32];
  stage<T>(twz, twg.z, tw_total<NZ>());
  __syncthreads();
  const long nk = (long)nkp * NZ;
  const int m0 = blockIdx.x * M;
  const int mm = threadIdx.x / G, g = threadIdx.x % G;
  const bool active = mm < M && m0 + mm < nkp;
  const long col = m0 + (active ? mm : 0);
  BARegs<T, NZ> wa, wb;
  z_forward_to_regs<T, NZ>(kq[blockIdx.y], nkp, col, A + (active ? mm : 0) * LDT, twz, wa, g, active);
  z_forward_to_regs<T, NZ>(kqc[blockIdx.y], nkp, col, B + (active ? mm : 0) * LDT, twz, wb, g, active);
  double acc[kMaxParams];
  for (int k = 0; k < kMaxParams; ++k) acc[k] = 0.0;
  if (active) {
#pragma unroll
    for (int b = 0; b < JoinBA<NZ>::BPT; ++b)
#pragma unroll
      for (int tt = 0; tt < JoinBA<NZ>::R; ++tt) {
        const long kk = (long)JoinBA<NZ>::pos(g, b, tt) * nkp + col;
        const double prod = (double)wa.v[b][tt].x * (double)wb.v[b][tt].x * (kk == 0 ? 1.0 : 2.0);
        for (int k = 0; k < nparams; ++k) acc[k] += prod * dksq[k * nk + kk];
      }
  }
  for (int k = 0; k < nparams; ++k) {
    const double v = block_sum(acc[k], red[k]);
    if (threadIdx.x == 0) part[((long)blockIdx.y * gridDim.x + blockIdx.x) * nparams + k] = v;
  }
}

// ------------------------------------------------------------------ adjoint transforms
// Gradient sums of the bond operator: for real grids u1, u2 with half spectra U1 = rfft(u1),
// U2 = rfft(u2), part[.. * nw + j] = sum_k mult_k Re(U1_k conj U2_k) wts[j * Nk + k], where
// mult_k is the Hermitian multiplicity of the half spectrum (1 on the kx = 0 and kx = Nx/2
// planes, 2 elsewhere).  Nz == 1: one CTA transforms u1 (its spectrum parked in k1, same
// thread -> element mapping in both passes) and then u2.
template <typename T, int NX, int NY>
__global__ void __launch_bounds__(PlaneCfg<NX, NY>::THREADS)
    grad_plane_kernel(const T* __restrict__ u1, const T* __restrict__ u2, Cx<T>* __restrict__ k1,
                      const double* __restrict__ wts, int nw, double* __restrict__ part, Twiddles<T> twg) {
  using C = PlaneCfg<NX, NY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* S = reinterpret_cast<Cx<T>*>(smem_raw);
  __shared__ Cx<T> twx[C::TWX], twy[C::TWY];
  __shared__ double red[kMaxParams + 1][32];
  stage<T>(twx, twg.x, C::TWX);
  if (NY > 1) stage<T>(twy, twg.y, C::TWY);
  const int p = group_index<C::GX, C::SP>(threadIdx.x / C::GX), gx = threadIdx.x % C::GX;
  const bool xact = p < C::NPAIR;
  const int c = group_index<C::GY, C::SC>(threadIdx.x / C::GY), gy = threadIdx.x % C::GY;
  const bool yact = NY > 1 && c < C::KX;
  double acc[kMaxParams + 1];
  for (int j = 0; j <= kMaxParams; ++j) acc[j] = 0.0;
  auto visit = [&](int pass, int kk, int kx, const Cx<T>& v) {
    if (pass == 0) {
      k1[kk] = v;
    } else {
      const Cx<T> a = k1[kk];
      const double m = (kx == 0 || 2 * kx == NX) ? 1.0 : 2.0;
      const double prod = m * ((double)a.x * (double)v.x + (double)a.y * (double)v.y);
      for (int j = 0; j < nw; ++j) acc[j] += prod * wts[(long)j * C::NKP + kk];
    }
  };
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    XRegs<T, NX> r;
    if (xact) load_regs<T, NX, NY>(r, p, gx, nullptr, pass == 0 ? u1 : u2);
    if constexpr (NY == 1) {
      BARegs<T, NX> w;
      row_forward_1d<T, NX>(S, twx, r, w, gx, xact);
      if (xact) {
#pragma unroll
        for (int b = 0; b < JoinBA<NX>::BPT; ++b)
#pragma unroll
          for (int tt = 0; tt < JoinBA<NX>::R; ++tt) {
            const int x = JoinBA<NX>::pos(gx, b, tt);
            if (x <= NX / 2) visit(pass, x, x, w.v[b][tt]);
          }
      }
      __syncwarp();
    } else {
      x_forward_from_regs<T, NX, NY>(S, twx, r, p, gx, xact);
      __syncthreads();
      BARegs<T, NY> w;
      y_forward_to_regs<T, NX, NY>(S, twy, w, c, gy, yact);
      if (yact) {
#pragma unroll
        for (int b = 0; b < JoinBA<NY>::BPT; ++b)
#pragma unroll
          for (int tt = 0; tt < JoinBA<NY>::R; ++tt) {
            const int ky = JoinBA<NY>::pos(gy, b, tt);
            visit(pass, c * NY + ky, c, w.v[b][tt]);
          }
      }
    }
    __syncthreads();
  }
  for (int j = 0; j < nw; ++j) {
    const double v = block_sum(acc[j], red[j]);
    if (threadIdx.x == 0) part[j] = v;
  }
}

// 3D, pencil pass: z transforms of the two plane-transformed spectra k1, k2 ([kz][kx][ky])
// and the weighted sums over the tile.  Output part[tile * nw + j].
template <typename T, int NZ>
__global__ void __launch_bounds__(512)
    z_fwd_grad_kernel(const Cx<T>* __restrict__ k1, const Cx<T>* __restrict__ k2, int nkp, int nx, int ny,
                      const double* __restrict__ wts, int nw, double* __restrict__ part, Twiddles<T> twg) {
  constexpr int M = ZCfg<T>::M;
  constexpr int LDT = NZ + pencil_pad<NZ>();
  constexpr int G = Plan<NZ>::G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* A = reinterpret_cast<Cx<T>*>(smem_raw);
  Cx<T>* B = A + M * LDT;
  __shared__ Cx<T> twz[tw_total<NZ>()];
  __shared__ double red[kMaxParams + 1][32];
  stage<T>(twz, twg.z, tw_total<NZ>());
  __syncthreads();
  const long nk = (long)nkp * NZ;
  const int m0 = blockIdx.x * M;
  const int mm = threadIdx.x / G, g = threadIdx.x % G;
  const bool active = mm < M && m0 + mm < nkp;
  const long col = m0 + (active ? mm : 0);
  BARegs<T, NZ> wa, wb;
  z_forward_to_regs<T, NZ>(k1, nkp, col, A + (active ? mm : 0) * LDT, twz, wa, g, active);
  z_forward_to_regs<T, NZ>(k2, nkp, col, B + (active ? mm : 0) * LDT, twz, wb, g, active);
  double acc[kMaxParams + 1];
  for (int j = 0; j <= kMaxParams; ++j) acc[j] = 0.0;
  if (active) {
    const int kx = (int)(col / ny);
    const double m = (kx == 0 || 2 * kx == nx) ? 1.0 : 2.0;
#pragma unroll
    for (int b = 0; b < JoinBA<NZ>::BPT; ++b)
#pragma unroll
      for (int tt = 0; tt < JoinBA<NZ>::R; ++tt) {
        const long kk = (long)JoinBA<NZ>::pos(g, b, tt) * nkp + col;
        const double prod =
            m * ((double)wa.v[b][tt].x * (double)wb.v[b][tt].x + (double)wa.v[b][tt].y * (double)wb.v[b][tt].y);
        for (int j = 0; j < nw; ++j) acc[j] += prod * wts[j * nk + kk];
      }
  }
  for (int j = 0; j < nw; ++j) {
    const double v = block_sum(acc[j], red[j]);
    if (threadIdx.x == 0) part[(long)blockIdx.x * nw + j] = v;
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
  return round32(ZCfg<T>::M * Plan<NZ>::G);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime.
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// TMA views of a chain's half-spectrum scratch (rows of Nkp complex values, one per kz, as
// 8-byte units; boxes of 128 bytes x Nz rows) and of an LD array (rows of Nkp values of T;
// boxes of M values x Nz rows), both unswizzled: the pencil pass reads whole rows per half warp.
template <typename T>
static void make_zmaps(CUtensorMap* km, CUtensorMap* lm, const Cx<T>* kbuf, const T* ld, int nkp, int nz) {
  auto enc = tmap_encoder();
  if (!enc) throw DeviceError("cuTensorMapEncodeTiled is not available from the driver");
  // box starts are multiples of 128 (scratch) and 64 (LD) bytes; rows must be 16-byte strided
  if (nkp % 4 != 0 || nz > 256 || (reinterpret_cast<uintptr_t>(kbuf) & 15) || (reinterpret_cast<uintptr_t>(ld) & 15))
    throw std::runtime_error("pencil pass: spectrum rows or buffers not 16-byte aligned");
  const cuuint32_t es[2] = {1, 1};
  {
    const cuuint64_t dim[2] = {(cuuint64_t)nkp * (sizeof(Cx<T>) / 8), (cuuint64_t)nz};
    const cuuint64_t str[1] = {(cuuint64_t)nkp * sizeof(Cx<T>)};
    const cuuint32_t box[2] = {16, (cuuint32_t)nz};
    if (enc(km, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<Cx<T>*>(kbuf), dim, str, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      throw DeviceError("cuTensorMapEncodeTiled failed for a half-spectrum scratch");
  }
  {
    const cuuint64_t dim[2] = {(cuuint64_t)nkp, (cuuint64_t)nz};
    const cuuint64_t str[1] = {(cuuint64_t)nkp * sizeof(T)};
    const cuuint32_t box[2] = {(cuuint32_t)z_tile_pencils<T>(), (cuuint32_t)nz};
    if (enc(lm, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2,
            const_cast<T*>(ld), dim, str, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      throw DeviceError("cuTensorMapEncodeTiled failed for a bond operator");
  }
}

// Launch on st; with pdl the launch may begin while the previous kernel on st finishes (its
// reads of that kernel's results wait in grid_dep_wait).
template <typename... KArgs, typename... Args>
static void launch_on(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                      Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
  if (e != cudaSuccess) throw DeviceError(std::string("kernel launch failed: ") + cudaGetErrorString(e));
}

// Pencil-pass schedules: pipeline stages (2 or 3 tile buffers per CTA) and rounds (tiles per
// CTA, which sets the grid).  The choice per (precision, Nz, plane size) comes from the
// autotuner (System::autotune_pencil: real chain steps timed per candidate when a handle first
// builds its 3D chains) or, before tuning, the default below; a chain may also force one.
constexpr int kZDefaultStages = 3, kZDefaultRounds = 2;
struct ZSchedule {
  int stages = kZDefaultStages, rounds = kZDefaultRounds;
};
template <typename T>
struct ZScheduleTable {
  std::mutex mu;
  std::map<std::pair<int, int>, ZSchedule> tuned;  // (Nz, Nkp) -> schedule
  static ZScheduleTable& get() {
    static ZScheduleTable t;
    return t;
  }
};

template <typename T, int NZ, int S>
static void launch_z_pipe_s(const ChainHost<T>& h, int t, int nkp, double ng, const Twiddles<T>& tw, int rounds,
                            cudaStream_t st) {
  using Z = ZPipe<T, NZ, S>;
  static const int grid_cap = [] {  // thread-safe one-time setup
    set_smem(z_pipe_kernel<T, NZ, S>, Z::SMEM);
    int occ = 0, dev = 0, nsm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, z_pipe_kernel<T, NZ, S>, Z::THREADS, Z::SMEM);
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return (occ > 0 ? occ : 1) * (nsm > 0 ? nsm : 1);
  }();
  CUtensorMap km, lm;
  make_zmaps<T>(&km, &lm, h.kbuf, h.ld[t], nkp, NZ);
  const int ntiles = (nkp + Z::M - 1) / Z::M;
  const int nrounds = (ntiles + Z::TPC - 1) / Z::TPC;
  int grid = (nrounds + rounds - 1) / rounds;
  if (grid > grid_cap) grid = grid_cap;
  if (grid < 1) grid = 1;
  launch_on(z_pipe_kernel<T, NZ, S>, dim3(grid), dim3(Z::THREADS), Z::SMEM, st, true, km, lm, h.csc, h.lsc, t,
            ntiles, ng, tw, h.status, h.wait_ns);
  count_launches(1);
}

template <typename T, int NZ>
static void launch_z_pipe(const ChainHost<T>& h, int t, int nkp, double ng, const Twiddles<T>& tw,
                          cudaStream_t st) {
  ZSchedule z;
  if (h.zstages > 0) {
    z.stages = h.zstages;
    z.rounds = h.zrounds > 0 ? h.zrounds : kZDefaultRounds;
  } else {
    auto& tab = ZScheduleTable<T>::get();
    std::lock_guard<std::mutex> lock(tab.mu);
    auto it = tab.tuned.find({NZ, nkp});
    if (it != tab.tuned.end()) z = it->second;
  }
  if (z.stages == 2) launch_z_pipe_s<T, NZ, 2>(h, t, nkp, ng, tw, z.rounds, st);
  else launch_z_pipe_s<T, NZ, 3>(h, t, nkp, ng, tw, z.rounds, st);
}

template <typename T>
static void z_pipe_dispatch(int nz, const ChainHost<T>& h, int t, int nkp, double ng, const Twiddles<T>& tw,
                            cudaStream_t st) {
  switch (nz) {
#define PF_Z(N)                                        \
  case N:                                              \
    launch_z_pipe<T, N>(h, t, nkp, ng, tw, st);        \
    return;
    PF_Z_LENGTHS(PF_Z)
#undef PF_Z
    default:
      return;
  }
}

template <typename T>
void set_pencil_schedule(int nz, int nkp, int stages, int rounds) {
  auto& tab = ZScheduleTable<T>::get();
  std::lock_guard<std::mutex> lock(tab.mu);
  tab.tuned[{nz, nkp}] = ZSchedule{stages, rounds};
}
template <typename T>
bool get_pencil_schedule(int nz, int nkp, int* stages, int* rounds) {
  auto& tab = ZScheduleTable<T>::get();
  std::lock_guard<std::mutex> lock(tab.mu);
  auto it = tab.tuned.find({nz, nkp});
  const ZSchedule z = it != tab.tuned.end() ? it->second : ZSchedule{};
  if (stages) *stages = z.stages;
  if (rounds) *rounds = z.rounds;
  return it != tab.tuned.end();
}

template <typename T, int NX, int NY>
static void chains_shape(const ChainJob<T>* jobs, int njobs, int maxsteps, int nz, const Twiddles<T>& tw,
                         cudaStream_t st, const ChainHost<T>* hosts, const Branches* br) {
  using C = PlaneCfg<NX, NY>;
  constexpr size_t sp = plane_smem<T, NX, NY>();
  static const bool attr = [] {  // thread-safe one-time setup
    set_smem(chain_plane_kernel<T, NX, NY>, sp);
    if constexpr (NY > 1) set_smem(xy_step_kernel<T, NX, NY>, sp);
    return true;
  }();
  (void)attr;
  if (nz == 1) {
    chain_plane_kernel<T, NX, NY><<<njobs, C::THREADS, sp, st>>>(jobs, tw);
    count_launches(1);
    return;
  }
  if constexpr (NY > 1) {
    if (!hosts) throw std::runtime_error("3D chains need the jobs' host descriptions");
    const double ng = (double)C::NP * nz;
    // job j's steps on stream sj: plane pass t (finishing t-1, starting t), pencil pass t
    auto run_job = [&](int j, cudaStream_t sj) {
      const int ns = hosts[j].nsteps;
      for (int t = 0; t <= ns; ++t) {
        launch_on(xy_step_kernel<T, NX, NY>, dim3(nz, 1), dim3(C::THREADS), sp, sj, t > 0, jobs + j,
                  t, nz, tw);
        count_launches(1);
        if (t < ns) z_pipe_dispatch<T>(nz, hosts[j], t, C::NKP, ng, tw, sj);
      }
    };
    if (br && br->n > 0 && njobs > 1) {
      // one branch stream per job: chains of different lengths and phases overlap
      cudaEventRecord(br->fork, st);
      const int nb = br->n < njobs ? br->n : njobs;
      for (int b = 0; b < nb; ++b) cudaStreamWaitEvent(br->s[b], br->fork, 0);
      for (int j = 0; j < njobs; ++j) run_job(j, br->s[j % nb]);
      for (int b = 0; b < nb; ++b) {
        cudaEventRecord(br->join[b], br->s[b]);
        cudaStreamWaitEvent(st, br->join[b], 0);
      }
      return;
    }
    for (int j = 0; j < njobs; ++j) run_job(j, st);
  }
}

template <typename T, int NX, int NY>
static void stress_shape(const StressItem<T>* items, int nitems, const T* const* src_q, const T* const* src_qc,
                         Cx<T>* const* kq, Cx<T>* const* kqc, int nz, const double* dksq, int nparams,
                         double* part, const Twiddles<T>& tw, cudaStream_t st) {
  using C = PlaneCfg<NX, NY>;
  constexpr size_t sp = plane_smem<T, NX, NY>();
  constexpr size_t ss = sp + sizeof(T) * (size_t)C::NKP;
  static const bool attr = [] {  // thread-safe one-time setup
    set_smem(stress_plane_kernel<T, NX, NY>, ss);
    if constexpr (NY > 1) set_smem(xy_fwd_kernel<T, NX, NY>, sp);
    return true;
  }();
  (void)attr;
  if (nz == 1) {
    stress_plane_kernel<T, NX, NY><<<nitems, C::THREADS, ss, st>>>(items, dksq, nparams, part, tw);
    count_launches(1);
    return;
  }
  if constexpr (NY > 1) {
    xy_fwd_kernel<T, NX, NY><<<dim3(nz, nitems), C::THREADS, sp, st>>>(src_q, kq, tw);
    count_launches(1);
    xy_fwd_kernel<T, NX, NY><<<dim3(nz, nitems), C::THREADS, sp, st>>>(src_qc, kqc, tw);
    count_launches(1);
    constexpr int M = ZCfg<T>::M;
    const int ntiles = (C::NKP + M - 1) / M;
    switch (nz) {
#define PF_Z(N)                                                                                                    \
  case N: {                                                                                                        \
    const size_t sz = 2 * sizeof(Cx<T>) * (size_t)(N + pencil_pad<N>()) * M;                                       \
    static const bool za = (set_smem(z_fwd_stress_kernel<T, N>, sz), true);                                       \
    (void)za;                                                                                                      \
    z_fwd_stress_kernel<T, N><<<dim3(ntiles, nitems), z_threads<T, N>(), sz, st>>>(kq, kqc, C::NKP, dksq, nparams, \
                                                                                  part, tw);                      \
    count_launches(1);                                                                                             \
  } break;
      PF_Z_LENGTHS(PF_Z)
#undef PF_Z
      default:
        break;
    }
  }
}

template <typename T, int NX, int NY>
static int grad_shape(const T* u1, const T* u2, Cx<T>* k1, Cx<T>* k2, const T* const* src, Cx<T>* const* dst, int nz,
                      const double* wts, int nw, double* part, const Twiddles<T>& tw, cudaStream_t st) {
  using C = PlaneCfg<NX, NY>;
  constexpr size_t sp = plane_smem<T, NX, NY>();
  static const bool attr = [] {
    set_smem(grad_plane_kernel<T, NX, NY>, sp);
    if constexpr (NY > 1) set_smem(xy_fwd_kernel<T, NX, NY>, sp);
    return true;
  }();
  (void)attr;
  if (nz == 1) {
    grad_plane_kernel<T, NX, NY><<<1, C::THREADS, sp, st>>>(u1, u2, k1, wts, nw, part, tw);
    count_launches(1);
    return 1;
  }
  if constexpr (NY > 1) {
    xy_fwd_kernel<T, NX, NY><<<dim3(nz, 2), C::THREADS, sp, st>>>(src, dst, tw);
    count_launches(1);
    constexpr int M = ZCfg<T>::M;
    const int ntiles = (C::NKP + M - 1) / M;
    switch (nz) {
#define PF_Z(N)                                                                                         \
  case N: {                                                                                             \
    const size_t sz = 2 * sizeof(Cx<T>) * (size_t)(N + pencil_pad<N>()) * M;                            \
    static const bool za = (set_smem(z_fwd_grad_kernel<T, N>, sz), true);                               \
    (void)za;                                                                                           \
    z_fwd_grad_kernel<T, N><<<ntiles, z_threads<T, N>(), sz, st>>>(k1, k2, C::NKP, NX, NY, wts, nw, part, \
                                                                  tw);                                 \
    count_launches(1);                                                                                  \
  } break;
      PF_Z_LENGTHS(PF_Z)
#undef PF_Z
      default:
        break;
    }
    return ntiles;
  }
  return 0;
}

template <typename T>
int launch_grad_transform(const T* u1, const T* u2, Cx<T>* k1, Cx<T>* k2, const T* const* src_dev,
                          Cx<T>* const* dst_dev, const GridDims& d, const double* wts, int nw, double* part,
                          const Twiddles<T>& tw, cudaStream_t st) {
  switch (shape_key(d.nx, d.ny)) {
#define PF_S(A, B)                                                                                  \
  case A * 1024 + B:                                                                                \
    return grad_shape<T, A, B>(u1, u2, k1, k2, src_dev, dst_dev, d.nz, wts, nw, part, tw, st);
    PF_PLANE_SHAPES(PF_S)
#undef PF_S
    default:
      return 0;
  }
}

// Whether kernels exist for this grid (and fit the shared memory of one CTA).
template <typename T>
bool shape_supported(int nx, int ny, int nz) {
  bool plane = false;
  switch (shape_key(nx, ny)) {
#define PF_S(A, B)                                                                       \
  case A * 1024 + B:                                                                     \
    plane = plane_smem<T, A, B>() + sizeof(T) * PlaneCfg<A, B>::NKP <= 200 * 1024;       \
    break;
    PF_PLANE_SHAPES(PF_S)
#undef PF_S
    default:
      plane = false;
  }
  return plane && (nz == 1 || (ny > 1 && fft_length_supported(nz)));
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
                   cudaStream_t st, const ChainHost<T>* hosts, const Branches* br) {
  switch (shape_key(d.nx, d.ny)) {
#define PF_S(A, B)                                                              \
  case A * 1024 + B:                                                            \
    chains_shape<T, A, B>(jobs_dev, njobs, maxsteps, d.nz, tw, st, hosts, br);  \
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
  template void set_pencil_schedule<T>(int, int, int, int);                                                \
  template bool get_pencil_schedule<T>(int, int, int*, int*);                                              \
  template void launch_ld<T>(T*, const CellGeom&, double, double, long, cudaStream_t);                    \
  template void launch_fill<T>(T*, T, long, cudaStream_t);                                                \
  template void launch_chains<T>(const ChainJob<T>*, int, int, const GridDims&, const Twiddles<T>&,       \
                                 cudaStream_t, const ChainHost<T>*, const Branches*);                     \
  template int launch_grad_transform<T>(const T*, const T*, Cx<T>*, Cx<T>*, const T* const*, Cx<T>* const*,   \
                                        const GridDims&, const double*, int, double*, const Twiddles<T>&,     \
                                        cudaStream_t);                                                          \
  template void launch_stress<T>(const StressItem<T>*, int, const T* const*, const T* const*, Cx<T>* const*, \
                                 Cx<T>* const*, const GridDims&, const double*, int, double*,              \
                                 const Twiddles<T>&, cudaStream_t);

}  // namespace pf
