// Declarations shared by the kernel translation units and the host engine.
#pragma once
#include "pf_common.cuh"
#include <stdexcept>

namespace pf {

// A CUDA call inside a kernel launcher failed (tensor-map encoding, launch configuration);
// the C ABI reports it as PF_ECUDA.
struct DeviceError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

constexpr int kMaxParams = 6;   // triclinic cells have 6 parameters
constexpr int kMaxMon = 8;      // monomer types per system
constexpr int kMaxHist = 64;    // Anderson history slots (nhist + 1)

struct GridDims {
  int nx, ny, nz;
};

// Reciprocal basis and its parameter derivatives, row-major G[r*3+c] (column c is the
// reciprocal vector b_c), dGG[(l*3+m)*kMaxParams + p].
struct CellGeom {
  int nx, ny, nz, dim;
  int signed_k;  // 0: the reference's folded |j| along y and z (quirk Q1); 1: signed frequencies
  double G[9];
  double dGG[9 * kMaxParams];
};

// Operators of one contour step.
template <typename T>
struct StepOp {
  const T* lw;  // exp(-ds vol w / 2), Ng
  const T* ld;  // exp(-ds b^2 k^2 / 6) / Ng, Nk
};

// One chain propagation: hist[s] for s = s0, s0+dir, ..., s0+dir*nsteps.
// With csc/lsc set, step t is rescaled by the factor c_t = Ng / sum(LW * q_t) (the k = 0
// term of the forward transform), so the stored histories stay O(1) in float32; csc[t] is
// the float factor applied and lsc[t] = log(c_t) in float64.  The stored q_s is then the
// true propagator times exp(sum_{t<s} lsc[t]).
template <typename T>
struct ChainJob {
  T* hist;
  const StepOp<T>* ops;  // nsteps entries
  Cx<T>* kbuf;           // 3D grids: half-spectrum scratch of Nk complex
  float* csc;            // nsteps rescale factors, or null (no rescaling)
  double* lsc;           // nsteps log factors
  int s0, dir, nsteps, pad;
};

template <typename T>
struct StressItem {
  const T* q;
  const T* qc;
};

// Block-wide deterministic double sum; the result is valid in thread 0.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Number of kernels this library has launched (all handles), for launch accounting.
void count_launches(long n);
long launch_total();

// ---- propagator launchers (pf_mde_impl.cuh, instantiated in pf_mde_fp32.cu / pf_mde_fp64.cu)
// Pencils per tile of the z pass (128-byte rows): 16 for float32, 8 for float64.
template <typename T>
constexpr int z_tile_pencils() { return sizeof(T) == 4 ? 16 : 8; }
template <typename T> bool shape_supported(int nx, int ny, int nz);
// Twiddle tables of one transform length for the in-kernel FFTs: the per-pass tables of the
// plan in A order followed by those in B order, forward sign, written as (re[i], im[i]).
// Returns the number of entries (0 for n = 1, -1 for an unsupported length or short buffers).
int fft_twiddle_table(int n, double* re, double* im, int max_entries);
template <typename T> void launch_lw(T* lw, const double* w, double coeff, long n, cudaStream_t st);
template <typename T> void launch_ld(T* ld, const CellGeom& g, double coeff, double scale, long nk, cudaStream_t st);
void launch_dksq(double* dk, const CellGeom& g, int nparams, long nk, cudaStream_t st);
template <typename T> void launch_fill(T* a, T v, long n, cudaStream_t st);
// Branch streams for 3D chains: with n > 0 each job advances on its own stream (job j on
// s[j % n]), forked from the main stream by `fork` and joined back by join[], so that the plane
// and pencil passes of independent chains overlap on the GPU.  steps[j] = job j's step count.
constexpr int kMaxBranches = 8;
struct Branches {
  int n = 0;
  cudaStream_t s[kMaxBranches] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[kMaxBranches] = {};
  const int* steps = nullptr;
};
// Host-side view of a chain job, for launchers that build TMA descriptors of its buffers.
template <typename T>
struct ChainHost {
  Cx<T>* kbuf = nullptr;         // half-spectrum scratch, [kz][kx][ky]
  float* csc = nullptr;          // per-step rescale factors (float32 chains), or null
  double* lsc = nullptr;
  int nsteps = 0;
  const T* const* ld = nullptr;  // bond operator of each step (host array of nsteps pointers)
  // Device status word of the chain's owner (a handle, or the allocation-free entry point's
  // scratch array): the pencil pass sets it nonzero when one of its bounded waits on a TMA copy
  // gave up (that launch's output is invalid).  Null: not reported.
  int* status = nullptr;
  // Time limit (ns of GPU time) of the pencil pass's waits for its tiles; 0 makes them give up
  // at once (failure tests).  The drain of copies in flight keeps the default limit.
  unsigned long long wait_ns = 1000000000ull;
  // Pencil-pass schedule forced for this chain (stages 2 or 3, rounds = tiles per CTA); 0: the
  // autotuned schedule of the transform length, else the default.
  int zstages = 0, zrounds = 0;
};
// Autotuned pencil-pass schedules per (precision T, Nz, half-spectrum plane size Nkp).
template <typename T> void set_pencil_schedule(int nz, int nkp, int stages, int rounds);
template <typename T> bool get_pencil_schedule(int nz, int nkp, int* stages, int* rounds);
// 3D grids need hosts (njobs entries); 1D/2D grids ignore it.
template <typename T>
void launch_chains(const ChainJob<T>* jobs_dev, int njobs, int maxsteps, const GridDims& d, const Twiddles<T>& tw,
                   cudaStream_t st, const ChainHost<T>* hosts, const Branches* br = nullptr);
// Adjoint of the bond operator: rfft of the real grids u1, u2 and, for j < nw, the sums
// sum_k mult_k Re(U1_k conj U2_k) wts[j * Nk + k] (mult_k: Hermitian multiplicity) into
// part[i * nw + j] for i < the returned number of partial blocks.  3D grids use the
// half-spectrum scratch k1, k2 and the device pointer arrays src_dev = {u1, u2},
// dst_dev = {k1, k2}; Nz == 1 uses k1 only.  nw <= kMaxParams + 1.
template <typename T>
int launch_grad_transform(const T* u1, const T* u2, Cx<T>* k1, Cx<T>* k2, const T* const* src_dev,
                          Cx<T>* const* dst_dev, const GridDims& d, const double* wts, int nw, double* part,
                          const Twiddles<T>& tw, cudaStream_t st);
// Gradient weights of a block's bond operator (pf_mde_fp64.cu): nparams + 1 rows of Nk.
void launch_adj_weights(double* wts, const CellGeom& g, int nparams, double ds, double b, double scale, long nk,
                        cudaStream_t st);
// ---- adjoint elementwise pieces (pf_adjoint.cu)
// Source terms of the adjoint at one contour point: sum_i coef[i] * rb[i] * qs[i], times
// f = fac ? *fac : 1 / *Qdev.
template <typename T>
struct AdjSrc {
  int n = 0;
  const double* rb[3] = {};
  const T* qs[3] = {};
  double coef[3] = {};
  const double* fac = nullptr;
  const double* Qdev = nullptr;
};
// u1 = lw * x, u2 = lw * ybar
template <typename T>
void launch_adj_lw_pair(T* u1, T* u2, const T* lw, const T* x, const T* ybar, long n, cudaStream_t st);
// G += ybar * y + c * x * r; lam = c * r + sources (c = cfac ? *cfac : 1); lam may alias ybar
template <typename T>
void launch_adj_finish(T* lam, const T* r, const T* ybar, const T* x, const T* y, double* G, const float* cfac,
                       const AdjSrc<T>& src, long n, cudaStream_t st);
// lam = sources + dq (dq added to every point)
template <typename T>
void launch_adj_init(T* lam, const AdjSrc<T>& src, double dq, long n, cudaStream_t st);
// acc[j] += c * sum_i part[i * nw + j]  (c = cfac ? *cfac : 1; one block, fixed order)
void launch_adj_accum(double* acc, const double* part, int nparts, int nw, const float* cfac, cudaStream_t st);
// Point species: wbar += -vol * rho * rb + S * vol * exp(-vol * w) / (Ng * Q)
void launch_adj_point(double* wbar, const double* rho, const double* rb, const double* w, double vol, double S,
                      double ngQ, long n, cudaStream_t st);
// dL/drho of L = free_energy at fixed fields, every monomer: (-w_a + sum_b chi_ab rho_b / (v_a v_b)) / Ng
struct MonomerSet;
void launch_fhelm_cotangent(double* rbar, const double* w, const double* rho, const MonomerSet& ms, long ng,
                            cudaStream_t st);
// y += a * x (float64 grids)
void launch_daxpy(double* y, const double* x, double a, long n, cudaStream_t st);
// sum_x a_x * b_x into *out (device), float64, deterministic
void launch_ddot(const double* a, const double* b, long n, double* part, double* out, cudaStream_t st);
// ---- Euler and momentum field updaters (pf_adjoint.cu), n = nmon * Ng
void launch_euler_predict(double* w, double* temp, const double* r, double lam, long n, cudaStream_t st);
void launch_euler_correct(double* w, const double* temp, const double* r, double lam, long n, cudaStream_t st);
// method 0 MOM, 1 RMS, 2 ADAM
void launch_momentum(int method, double* w, double* m, double* v, const double* r, double lam, double b1, double b2,
                     long n, cudaStream_t st);
void launch_nag_ahead(double* w, double* temp, const double* m, double lam, long n, cudaStream_t st);
void launch_nag_update(double* w, const double* temp, double* m, const double* r, double lam, double gamma, long n,
                       cudaStream_t st);
// RQM4: out = (4 q2 - q1) / 3 (pf_adjoint.cu)
template <typename T>
void launch_rqm4_combine(T* out, const T* q1, const T* q2, long n, cudaStream_t st);
// Stress sums: Nz == 1 uses items (device array of nitems); 3D grids use the pointer arrays
// src_q/src_qc (real grids) and kq/kqc (half-spectrum scratch), each nitems long.
template <typename T>
void launch_stress(const StressItem<T>* items, int nitems, const T* const* src_q, const T* const* src_qc,
                   Cx<T>* const* kq, Cx<T>* const* kqc, const GridDims& d, const double* dksq, int nparams,
                   double* part, const Twiddles<T>& tw, cudaStream_t st);

// ---- field / density / updater launchers (pf_field.cu)
struct MonomerSet {
  int nmon;
  double vol[kMaxMon];
  double chi[kMaxMon * kMaxMon];  // symmetric; off-diagonal Flory chi, diagonal Edwards u
};

// Simpson block description for one species (reference multiblock.jl:182-228).
struct SimpsonBlocks {
  int nblocks;
  int mon[kMaxMon * 2];       // monomer index of each block
  int bgn[kMaxMon * 2];       // 0-based contour index of the block start
  int end[kMaxMon * 2];       // 0-based contour index of the block end
  double ds[kMaxMon * 2];
};

constexpr int kRedBlocks = 1024;  // partial-sum blocks of the grid reductions

template <typename T>
void launch_sum(const T* a, long n, double* part, double* out, double div, cudaStream_t st);
void launch_point_q(const double* w, double vol, long n, double* part, double* Qdev, cudaStream_t st);
void launch_point_density(double* rho, const double* w, double vol, double phi, const double* Qdev, long n,
                          cudaStream_t st);
// fac (optional, Ns+1 entries) multiplies each contour term: rescaled histories pass
// fac[s] = exp(-L_s - L'_s - log Q) and the kernel then skips the division by Q.
template <typename T>
void launch_simpson(double* rho_all, const T* q, const T* qc, bool qc_reversed, int Ns, long ng,
                    const SimpsonBlocks& blk, double phi, double Nref, const double* Qdev, const double* fac,
                    cudaStream_t st);
// Q and the Simpson factors of a rescaled chain: L_s = sum_{t<s} lsc_fwd[t],
// L'_s = sum_{t<Ns-s} lsc_bwd[t] (or L_{Ns-s} when rev), log Q = log(meanq) - L_Ns,
// fac[s] = exp(-L_s - L'_s - log Q) (without the log Q term when !divide_q: grand-canonical
// densities carry exp(mu) instead of 1/Q).  One block.
void launch_scale_finalize(const double* lsc_fwd, const double* lsc_bwd, bool rev, int Ns, const double* meanq,
                           double* Qdev, double* fac, cudaStream_t st,
                           bool divide_q = true);
int launch_residuals(double* w, double* pot, double* res, const double* rho, const MonomerSet& ms, long ng,
                     bool canonical, double* part, double* sums, cudaStream_t st);
void launch_stats(const double* w, const double* res, const double* rho, const MonomerSet& ms, long ng,
                  double* part, double* out4, cudaStream_t st);
void launch_axpy(double* y, const double* x, double a, long n, cudaStream_t st);
struct HistPtrs {
  const double* res[kMaxHist];    // logical order 0..ih
  const double* field[kMaxHist];
  double* sum[kMaxHist];          // field + residual of each entry (entry ih written by the step)
};
void launch_gram(const HistPtrs& h, int ih, long n_all, double* part, double* out, cudaStream_t st);
// The packed U, V of launch_gram from the cached history products P (nslot x nslot, physical
// slots, updated here with the current residual's row); flag = 1 asks for launch_gram instead.
void launch_gram_cached(const HistPtrs& h, const double* r, int ih, long n_all, double* P, int nslot, int base,
                        double* part, double* t, double* packed, int* flag, cudaStream_t st);
void launch_solve(const double* packed, int ih, double* Cn, int* status, cudaStream_t st);
void launch_mix(double* w, const HistPtrs& h, int ih, const double* Cn, double lam, long n_all, cudaStream_t st);
// out = a + b (the history sum of an entry in iterations without a mix)
void launch_add(double* out, const double* a, const double* b, long n, cudaStream_t st);

// ---- Newton-Krylov polish vector primitives (pf_polish.cu); V_i = V + i n, float64
// out[i] = V_i . z for i < k (device; part needs polish_part_doubles() doubles)
void launch_multidot(const double* V, int k, long n, const double* z, double* part, double* out, cudaStream_t st);
// z = alpha z + beta sum_{i<k} c[i] V_i (c on the device)
void launch_multiaxpy(double* z, const double* V, int k, long n, const double* c, double alpha, double beta,
                      cudaStream_t st);
// y = a y + b x
void launch_lincomb(double* y, const double* x, double a, double b, long n, cudaStream_t st);
int polish_part_doubles();

}  // namespace pf
