// Host engine and C ABI of libpolyfields_gpu.so.
//
// A pf_system is the GPU counterpart of the reference's FieldSystem
// (src/system/system.jl:22-49): grid, unit cell, monomers, species, Flory interactions and
// the device state (fields, potentials, residuals, densities, propagators, operators),
// plus the Anderson and Domain updaters (src/updaters/anderson.jl, domain.jl) and the
// scft! driver loop (src/simulate.jl:60-148).  The orchestration runs on the host; every
// grid-sized operation runs on the device, on the handle's own stream.
#include <cmath>
#include <atomic>
#include <thread>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>
#include <algorithm>
#include <array>
#include <chrono>
#include <ctime>

#include "pf_kernels.h"
#include "polyfields_gpu.h"

namespace pf {

// ------------------------------------------------------------------ errors
struct PFError : std::runtime_error {
  int code;
  PFError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define PF_CU(call)                                                                                  \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      throw pf::PFError(e_ == cudaErrorMemoryAllocation ? pf::E_NOMEM : pf::E_CUDA,                  \
                        std::string("CUDA error ") + cudaGetErrorString(e_) + " at " #call);         \
  } while (0)

// A launch error (or, with synchronous launches, a kernel fault) names the source line of
// the check that saw it.
#define check_launch() check_launch_at(__LINE__)
static void check_launch_at(int line) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    throw PFError(E_CUDA, std::string("kernel launch failed (pf_engine.cu:") + std::to_string(line) +
                              "): " + cudaGetErrorString(e));
}

// Host -> device copy ordered on stream st and complete on return.  A plain cudaMemcpy runs
// on the legacy default stream, which does not order with the non-blocking streams the engine
// launches on, and returns for pageable sources before its DMA has landed: a kernel on st could
// read the destination before the data arrives.
#define PF_H2D(dst, src, bytes, st)                                                   \
  do {                                                                                \
    PF_CU(cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyHostToDevice, (st)));       \
    PF_CU(cudaStreamSynchronize(st));                                                 \
  } while (0)

// Owning device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t n) {
    if (n == bytes && p) return;
    release();
    if (n == 0) return;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      throw PFError(E_NOMEM, std::string("cudaMalloc of ") + std::to_string(n) + " bytes failed: " + cudaGetErrorString(e));
    }
    bytes = n;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// ------------------------------------------------------------------ cell geometry (host)
// src/system/basis.jl and src/system/cell.jl.  Matrices are row-major 3x3, the Bravais
// vectors a_c are the columns of R and the reciprocal vectors b_c the columns of G.
using Mat3 = std::array<double, 9>;

static bool isapprox(double a, double b) {
  const double rtol = std::sqrt(2.220446049250313e-16);
  return std::fabs(a - b) <= rtol * std::max(std::fabs(a), std::fabs(b));
}

static Mat3 basis_matrix(double a, double b, double c, double alpha, double beta, double gamma) {
  const double p2 = M_PI / 2;
  Mat3 R{};
  if (isapprox(alpha, p2) && isapprox(beta, p2) && isapprox(gamma, p2)) {
    R = {a, 0, 0, 0, b, 0, 0, 0, c};
    return R;
  }
  const double ca = isapprox(alpha, p2) ? 0.0 : std::cos(alpha);
  const double cb = isapprox(beta, p2) ? 0.0 : std::cos(beta);
  double cg, sg;
  if (isapprox(gamma, p2)) {
    cg = 0.0;
    sg = 1.0;
  } else {
    cg = std::cos(gamma);
    sg = std::sin(gamma);
  }
  const double ax = a, bx = b * cg, by = b * sg, cx = c * cb, cy = c * (ca - cb * cg) / sg;
  const double cz = std::sqrt(c * c - cx * cx - cy * cy);
  R = {ax, bx, cx, 0.0, by, cy, 0.0, 0.0, cz};
  return R;
}

static int crystal_nparams(int dim, const std::string& c) {
  if (dim == 1 && c == "lamellar") return 1;
  if (dim == 2) {
    if (c == "square" || c == "hexagonal") return 1;
    if (c == "rectangular") return 2;
    if (c == "oblique") return 3;
  }
  if (dim == 3) {
    if (c == "cubic" || c == "pnna" || c == "fddd1") return 1;
    if (c == "tetragonal" || c == "hexagonal") return 2;
    if (c == "orthorhombic") return 3;
    if (c == "monoclinic") return 4;
    if (c == "triclinic") return 6;
  }
  return -1;
}

static Mat3 make_basis(int dim, const std::string& c, const std::vector<double>& p) {
  const double pi = M_PI;
  if (dim == 1) return basis_matrix(p[0], 1.0, 1.0, pi / 2, pi / 2, pi / 2);
  if (dim == 2) {
    if (c == "square") return basis_matrix(p[0], p[0], 1.0, pi / 2, pi / 2, pi / 2);
    if (c == "rectangular") return basis_matrix(p[0], p[1], 1.0, pi / 2, pi / 2, pi / 2);
    if (c == "hexagonal") return basis_matrix(p[0], p[0], 1.0, pi / 2, pi / 2, pi / 3);
    return basis_matrix(p[0], p[1], 1.0, pi / 2, pi / 2, p[2]);  // oblique
  }
  if (c == "cubic") return basis_matrix(p[0], p[0], p[0], pi / 2, pi / 2, pi / 2);
  if (c == "tetragonal") return basis_matrix(p[0], p[0], p[1], pi / 2, pi / 2, pi / 2);
  if (c == "orthorhombic") return basis_matrix(p[0], p[1], p[2], pi / 2, pi / 2, pi / 2);
  if (c == "hexagonal") return basis_matrix(p[0], p[0], p[1], pi / 2, pi / 2, pi / 3);
  if (c == "monoclinic") return basis_matrix(p[0], p[1], p[2], pi / 2, p[3], pi / 2);
  if (c == "triclinic") return basis_matrix(p[0], p[1], p[2], p[3], p[4], p[5]);
  if (c == "pnna") return basis_matrix(2.0 * p[0], std::sqrt(3.0) * p[0], p[0], pi / 2, pi / 2, pi / 2);
  return basis_matrix(p[0], std::sqrt(3.0) * p[0], 2.0 * std::sqrt(3.0) * p[0], pi / 2, pi / 2, pi / 2);  // fddd1
}

static double det3(const Mat3& m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

static Mat3 inv3(const Mat3& m) {
  const double d = det3(m);
  Mat3 r;
  r[0] = (m[4] * m[8] - m[5] * m[7]) / d;
  r[1] = (m[2] * m[7] - m[1] * m[8]) / d;
  r[2] = (m[1] * m[5] - m[2] * m[4]) / d;
  r[3] = (m[5] * m[6] - m[3] * m[8]) / d;
  r[4] = (m[0] * m[8] - m[2] * m[6]) / d;
  r[5] = (m[2] * m[3] - m[0] * m[5]) / d;
  r[6] = (m[3] * m[7] - m[4] * m[6]) / d;
  r[7] = (m[1] * m[6] - m[0] * m[7]) / d;
  r[8] = (m[0] * m[4] - m[1] * m[3]) / d;
  return r;
}

struct Cell {
  int dim = 0;
  std::string crystal;
  std::vector<double> params;
  double volume = 0.0;
  Mat3 R{}, G{};
  // dR[(i*3+j)*kMaxParams+k] etc.
  std::vector<double> dR, dG, dRR, dGG;
  int np() const { return (int)params.size(); }

  // update!(cell) (cell.jl:96-109) without the grids (they are device-side).
  void update() {
    R = make_basis(dim, crystal, params);
    Mat3 Ri = inv3(R);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) G[r * 3 + c] = 2 * M_PI * Ri[c * 3 + r];
    volume = det3(R);
    dbasis();
    ddbasis();
  }
  double& at(std::vector<double>& a, int i, int j, int k) { return a[(i * 3 + j) * kMaxParams + k]; }
  void dbasis() {  // cell.jl:120-231
    dR.assign(9 * kMaxParams, 0.0);
    dG.assign(9 * kMaxParams, 0.0);
    const auto& p = params;
    const std::string& c = crystal;
    if (dim == 1) {
      if (c == "lamellar") at(dR, 0, 0, 0) = 1.0;
    } else if (dim == 2) {
      if (c == "square") {
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 1, 1, 0) = 1.0;
      } else if (c == "rectangular") {
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 1, 1, 1) = 1.0;
      } else if (c == "hexagonal") {
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 0, 1, 0) = 0.5;
        at(dR, 1, 1, 0) = std::sqrt(0.75);
      } else if (c == "oblique") {
        const double b = p[1], gamma = p[2];
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 0, 1, 1) = std::cos(gamma);
        at(dR, 1, 1, 1) = std::sin(gamma);
        at(dR, 0, 1, 2) = -b * std::sin(gamma);
        at(dR, 1, 1, 2) = b * std::cos(gamma);
      }
    } else if (dim == 3) {
      if (c == "cubic") {
        at(dR, 0, 0, 0) = at(dR, 1, 1, 0) = at(dR, 2, 2, 0) = 1.0;
      } else if (c == "tetragonal") {
        at(dR, 0, 0, 0) = at(dR, 1, 1, 0) = 1.0;
        at(dR, 2, 2, 1) = 1.0;
      } else if (c == "orthorhombic") {
        at(dR, 0, 0, 0) = at(dR, 1, 1, 1) = at(dR, 2, 2, 2) = 1.0;
      } else if (c == "hexagonal") {
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 0, 1, 0) = 0.5;
        at(dR, 1, 1, 0) = std::sqrt(0.75);
        at(dR, 2, 2, 1) = 1.0;
      } else if (c == "monoclinic") {
        const double cc = p[2], beta = p[3];
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 1, 1, 1) = 1.0;
        at(dR, 0, 2, 2) = std::cos(beta);
        at(dR, 2, 2, 2) = std::sin(beta);
        at(dR, 0, 2, 3) = -cc * std::sin(beta);
        at(dR, 2, 2, 3) = cc * std::cos(beta);
      } else if (c == "triclinic") {
        const double b = p[1], cc = p[2], alpha = p[3], beta = p[4], gamma = p[5];
        const double cy = R[1 * 3 + 2], cz = R[2 * 3 + 2];
        const double sa = std::sin(alpha), ca = std::cos(alpha), sb = std::sin(beta), cb = std::cos(beta);
        const double sg = std::sin(gamma), cg = std::cos(gamma), tg = std::tan(gamma);
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 0, 1, 1) = cg;
        at(dR, 1, 1, 1) = sg;
        at(dR, 0, 2, 2) = cb;
        at(dR, 1, 2, 2) = cy / cc;
        at(dR, 2, 2, 2) = cz / cc;
        at(dR, 1, 2, 3) = -cc * sa / sg;
        at(dR, 2, 2, 3) = cc * cc * (ca - cb * cg) * sa / (sg * sg) / cz;
        at(dR, 0, 2, 4) = -cc * sb;
        at(dR, 1, 2, 4) = cc * sb / tg;
        at(dR, 2, 2, 4) = cc * cc * (-ca / tg + cb / sg) * sb / sg / cz;
        at(dR, 0, 1, 5) = -b * sg;
        at(dR, 1, 1, 5) = b * cg;
        at(dR, 1, 2, 5) = cc * (-ca / tg + cb / sg) / sg;
        at(dR, 2, 2, 5) = cc * cc * ((2 + std::cos(2 * alpha) + std::cos(2 * beta)) / tg -
                                     ca * cb * (3 + std::cos(2 * gamma)) / sg) / (sg * sg) / cz / 2;
      } else if (c == "pnna") {
        at(dR, 0, 0, 0) = 2.0;
        at(dR, 1, 1, 0) = std::sqrt(3.0);
        at(dR, 2, 2, 0) = 1.0;
      } else if (c == "fddd1") {
        at(dR, 0, 0, 0) = 1.0;
        at(dR, 1, 1, 0) = std::sqrt(3.0);
        at(dR, 2, 2, 0) = 2.0 * std::sqrt(3.0);
      }
    }
    for (int k = 0; k < np(); ++k)
      for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
          for (int l = 0; l < dim; ++l)
            for (int m = 0; m < dim; ++m) at(dG, i, j, k) -= G[i * 3 + l] * at(dR, m, l, k) * G[m * 3 + j];
    for (auto& v : dG) v /= 2 * M_PI;
  }
  void ddbasis() {  // cell.jl:233-258 (R transposed as in the reference)
    dRR.assign(9 * kMaxParams, 0.0);
    dGG.assign(9 * kMaxParams, 0.0);
    for (int k = 0; k < np(); ++k)
      for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
          for (int l = 0; l < dim; ++l) {
            at(dRR, i, j, k) += R[l * 3 + i] * at(dR, l, j, k) + R[l * 3 + j] * at(dR, l, i, k);
            at(dGG, i, j, k) += G[l * 3 + i] * at(dG, l, j, k) + G[l * 3 + j] * at(dG, l, i, k);
          }
  }
};

// Host LU with partial pivoting + explicit inverse (the reference's inv()).
static bool lu_inverse(std::vector<double> a, int n, std::vector<double>& inv) {
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(a[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[i * n + k]) > best) {
        best = std::fabs(a[i * n + k]);
        p = i;
      }
    if (a[p * n + k] == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
      std::swap(perm[k], perm[p]);
    }
    for (int i = k + 1; i < n; ++i) a[i * n + k] /= a[k * n + k];
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j) a[i * n + j] -= a[i * n + k] * a[k * n + j];
  }
  inv.assign(n * n, 0.0);
  std::vector<double> y(n);
  for (int col = 0; col < n; ++col) {
    for (int i = 0; i < n; ++i) {
      double s = (perm[i] == col) ? 1.0 : 0.0;
      for (int j = 0; j < i; ++j) s -= a[i * n + j] * y[j];
      y[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (int j = i + 1; j < n; ++j) s -= a[i * n + j] * inv[j * n + col];
      inv[i * n + col] = s / a[i * n + i];
    }
  }
  return true;
}

// ------------------------------------------------------------------ species
struct Species {
  int kind = 0;  // 0 multiblock, 1 point
  double phi = 0.0, mu = 0.0, Q = 0.0, Nref = 0.0;
  double mu_in = 0.0;  // grand ensemble: the chemical potential given to add_species!
  std::vector<int> mids;  // sorted monomer ids
  // multiblock (src/species/multiblock.jl:5-60)
  int Ns = 0, N = 0;
  std::vector<int> mid_block, N_block, begin_block;  // begin_block 1-based
  std::vector<double> b_block, ds_block, Nref_block, f_block;
  // device, per precision (0 = FP64, 1 = FP32)
  DevBuf q[2], qc[2];
  std::vector<std::unique_ptr<DevBuf>> lw[2], ld[2];
  DevBuf ops[2];  // StepOp<T> of the forward then backward job
  DevBuf kbuf[2][2];
  // float32 histories are rescaled per contour step (ChainJob::csc/lsc): factors of the
  // forward and backward jobs, the Simpson factors fac[s] and the mean of the last q
  DevBuf csc[2], lsc[2], fac, meanq;
  int ld_version[2] = {-1, -1};
  // RQM4 (float64): half-step operators per block, one-step and two-half-step jobs per block
  std::vector<std::unique_ptr<DevBuf>> lw2, ld2;
  DevBuf rq_ops, rq_jobs;
  std::vector<const double*> rq_ld1, rq_ld2;  // host: LD of the full and the half steps
  int ld2_version = -1;
  DevBuf Qdev;
  bool Q_valid = false;
  int nblocks() const { return (int)N_block.size(); }
  double monomer_fraction(int mid) const {
    if (kind == 1) return (mids[0] == mid) ? 1.0 : 0.0;
    double f = 0.0;
    for (int b = 0; b < nblocks(); ++b)
      if (mid_block[b] == mid) f += f_block[b];
    return f;
  }
};

// chain_grid (src/species/base.jl:27-56)
static void chain_grid(const std::vector<double>& Nb, int Ns, double& N, std::vector<int>& begin_block,
                       std::vector<double>& ds_block) {
  N = 0.0;
  for (double v : Nb) N += v;
  const int nb = (int)Nb.size();
  const double ds = N / Ns;
  begin_block.assign(nb + 1, 0);
  ds_block.assign(nb, 0.0);
  int bgn = 1;
  begin_block[0] = bgn;
  for (int i = 0; i < nb; ++i) {
    int Ns_half = (int)std::floor(Nb[i] / ds / 2.0 + 0.5);
    if (Ns_half == 0) {
      Ns_half = 1;
      ds_block[i] = Nb[i] / 2.0;
    } else {
      ds_block[i] = Nb[i] / Ns_half / 2.0;
    }
    bgn = bgn + Ns_half * 2;
    begin_block[i + 1] = bgn;
  }
}

// ------------------------------------------------------------------ the system
// Handles run on their own streams, batched ones from their own host threads (pf_scft_batch).
// The CUDA runtime maps the streams of a process onto CUDA_DEVICE_MAX_CONNECTIONS hardware work
// queues (8 unless set), and streams that share a queue wait on one another's work.  When the
// library is loaded it asks for the maximum, 32, unless the caller has set the variable; this
// takes effect only if the process has not created its CUDA context yet.
__attribute__((constructor)) static void pf_request_connections() {
  setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

struct System {
  int nx, ny, nz;
  long ng, nk;
  int prec;         // current precision of the propagators
  int last_prec = -1;  // precision of the last density solve
  cudaStream_t st = nullptr;
  std::string err;

  Cell cell;
  bool has_cell = false;
  int cell_version = 0;
  bool signed_k = false;  // ksq/dksq with signed frequencies instead of the reference's fold
  int dksq_version = -1;

  std::map<int, std::pair<double, double>> monomers;  // id -> (vol, charge)
  std::vector<int> mon_ids;                            // sorted ids; index = position
  std::map<std::pair<int, int>, double> chis;          // ordered pair -> chi
  std::map<int, double> edwards;                       // monomer id -> u (EdwardsInteraction)
  std::vector<std::unique_ptr<Species>> species;

  DevBuf w, pot, res, rho;   // nmon * ng doubles
  DevBuf rbar, wbar;         // adjoint: dL/drho (set by the caller) and dL/dw, nmon * ng doubles
  DevBuf part, sums, stats4, packed, cn, status;
  // Pencil-pass status word of this handle: set nonzero on the device when a bounded wait of a
  // pencil pass gave up (check_pipe reads and clears it); and the limit of those waits.
  DevBuf pipe_st;
  unsigned long long wait_ns = 1000000000ull;
  DevBuf twid[2];
  int tw_off[2][3] = {};  // offsets of the x, y, z tables in twid
  DevBuf dksq;
  DevBuf jobs[2];
  int njobs = 0, maxsteps = 0;
  // 3D chains run one branch stream per job (PF_NO_BRANCHES=1: all jobs in shared launches)
  bool use_branches = true;
  Branches br;
  std::vector<int> job_steps;
  // host views of the jobs (TMA descriptors of the pencil pass): per precision
  std::vector<ChainHost<float>> hosts_f;
  std::vector<ChainHost<double>> hosts_d;
  std::vector<std::vector<const float*>> lds_f;
  std::vector<std::vector<const double*>> lds_d;
  template <typename T>
  std::vector<ChainHost<T>>& hosts_of() {
    if constexpr (sizeof(T) == 4) return hosts_f;
    else return hosts_d;
  }
  template <typename T>
  std::vector<std::vector<const T*>>& lds_of() {
    if constexpr (sizeof(T) == 4) return lds_f;
    else return lds_d;
  }
  bool jobs_dirty[2] = {true, true};
  bool timing = false;
  int mde = 0;     // 0 RK2 (mde.jl:65-81), 1 RQM4 (mde.jl:83-104, float64 chains)
  std::string savepath;  // SCFTOptions.savepath (simulate.jl:12-19), written every nsave steps
  int adj_ckpt = 0;  // pullback: 0 = read the stored histories, K > 0 = recompute between checkpoints
  int ensemble = 0;  // 0 Canonical, 1 Grand (system.jl:6-13)
  DevBuf one;        // a device 1.0 (grand-canonical densities are not divided by Q)
  DevBuf rq_scratch;  // RQM4: [x, q1] and [x, h, q2]
  // density solves replay a captured CUDA graph per precision (PF_NO_GRAPHS=1 disables)
  bool use_graphs = true;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  bool graph_warm[2] = {false, false};
  long graph_kernels[2] = {0, 0};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t uev[8] = {};  // user events (pf_record_event)
  double t_prop_ms = 0.0, t_dens_ms = 0.0;
  int mde_steps = 0;
  // Small device-to-host reads (status words, Q, reduction results) land in this handle's pinned
  // staging buffer.  A read into pageable memory is staged by the driver through buffers shared
  // by the whole process, and with many handles stepping on their own threads (pf_scft_batch)
  // those reads queued behind one another: 32 identical 2D systems on 32 threads advanced about
  // three at a time.  With this buffer and 32 hardware queues (pf_request_connections) they run
  // side by side.
  static constexpr size_t kPinBytes = 64 * 1024;
  unsigned char* hpin = nullptr;
  // Queue a read of `bytes` from device address src into the staging buffer at byte offset off;
  // the data is valid after the next sync_st().
  void d2h_pin(size_t off, const void* src, size_t bytes) {
    if (off + bytes > kPinBytes) throw PFError(E_ARG, "pinned staging buffer too small");
    PF_CU(cudaMemcpyAsync(hpin + off, src, bytes, cudaMemcpyDeviceToHost, st));
  }
  // Read `bytes` from device address src into dst and wait for it.
  void d2h_now(void* dst, const void* src, size_t bytes) {
    if (bytes <= kPinBytes) {
      d2h_pin(0, src, bytes);
      sync_st();
      std::memcpy(dst, hpin, bytes);
    } else {
      PF_CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
      sync_st();
    }
  }
  // Host wait on the handle's stream.
  void sync_st() { PF_CU(cudaStreamSynchronize(st)); }

  // Anderson updater (src/updaters/anderson.jl:13-47)
  struct Anderson {
    bool exists = false, is_setup = false;
    int nhist = 50, iter = 0, iter_hist = 0, iter_euler = 1, base = 0;
    double lam = 0.0, lam_euler = 0.01;
    DevBuf res_hist, field_hist;
    // gram_p[a * nslot + b] = res(slot a) . res(slot b) for the slots of the window, gram_t
    // the current residual's products with the window (launch_gram_cached)
    DevBuf gram_p, gram_t;
    DevBuf sum_hist;  // field + residual of each entry (the mix's single history once lam = 1)
    void reset() {
      exists = is_setup = false;
      nhist = 50;
      iter = iter_hist = 0;
      iter_euler = 1;
      base = 0;
      lam = 0.0;
      lam_euler = 0.01;
      res_hist.release();
      field_hist.release();
      gram_p.release();
      gram_t.release();
      sum_hist.release();
    }
  } and_;
  // EulerUpdater (kind 1, method 0 PEC / 1 PECE) and MomentumUpdater (kind 2, method 0 MOM,
  // 1 RMS, 2 ADAM, 3 NAG).  A system can carry several of them, each with its own state, as
  // the reference's updater objects do (test/test_updaters.jl:16-30 sets up an Euler, a NAG
  // and an Anderson updater on one system and steps each in turn).  `su` is the current one;
  // `active` is the kind of the current updater (0 = the Anderson updater).
  struct SimpleUpdater {
    int kind = 0, method = 0;
    bool is_setup = false;
    double lam = 0.05, gamma = 0.9, beta1 = 0.9, beta2 = 0.999;
    DevBuf temp, mt, vt;
    void reset(int k, int m, double l) {
      kind = k;
      method = m;
      lam = l;
      is_setup = false;
      gamma = beta1 = 0.9;
      beta2 = 0.999;
      temp.release();
      mt.release();
      vt.release();
    }
  };
  std::vector<std::unique_ptr<SimpleUpdater>> simple;
  SimpleUpdater* su = nullptr;
  int active = 0;
  // Domain updater (src/updaters/domain.jl:7-24)
  struct Domain {
    bool exists = false, is_setup = false;
    int nper = 10, nskip = 200;
    double lam = 0.1, pmax = 1.0, rlxn = 0.5;
    std::vector<double> oldparams, step, stress, dstress;
  } dom;

  System(int x, int y, int z, int p) : nx(x), ny(y), nz(z), prec(p) {
    ng = (long)nx * ny * nz;
    nk = (long)(nx / 2 + 1) * ny * nz;
    PF_CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    PF_CU(cudaHostAlloc(reinterpret_cast<void**>(&hpin), kPinBytes, cudaHostAllocDefault));
    part.alloc(sizeof(double) * (size_t)kRedBlocks * 4 * (kMaxMon + 1) + sizeof(double) * 2048 * 2 * 152);
    sums.alloc(sizeof(double) * 4 * kMaxMon);
    stats4.alloc(sizeof(double) * 8);
    packed.alloc(sizeof(double) * 4096);
    cn.alloc(sizeof(double) * kMaxHist);
    status.alloc(sizeof(int) * 4);
    pipe_st.alloc(sizeof(int));
    PF_CU(cudaMemsetAsync(pipe_st.p, 0, sizeof(int), st));
    {
      const double v1 = 1.0;
      one.alloc(sizeof(double));
      PF_H2D(one.p, &v1, sizeof(double), st);
    }
    build_twiddles<double>(0);
    build_twiddles<float>(1);
    for (auto& e : ev) PF_CU(cudaEventCreate(&e));
    for (auto& e : uev) PF_CU(cudaEventCreate(&e));
    const char* ng_env = getenv("PF_NO_GRAPHS");
    if (ng_env && ng_env[0] == '1') use_graphs = false;
    const char* nb_env = getenv("PF_NO_BRANCHES");
    if (nb_env && nb_env[0] == '1') use_branches = false;
    const char* na_env = getenv("PF_NO_AUTOTUNE");
    if (na_env && na_env[0] == '1') autotune = false;
  }
  ~System() {
    if (st) cudaStreamSynchronize(st);
    invalidate_graphs();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : uev)
      if (e) cudaEventDestroy(e);
    for (auto& e : tev)
      if (e) cudaEventDestroy(e);
    if (hpin) cudaFreeHost(hpin);
    for (int b = 0; b < kMaxBranches; ++b) {
      if (br.s[b]) cudaStreamDestroy(br.s[b]);
      if (br.join[b]) cudaEventDestroy(br.join[b]);
    }
    if (br.fork) cudaEventDestroy(br.fork);
    if (st) cudaStreamDestroy(st);
  }
  // branch streams for njobs chains (created once, kept for the handle's lifetime)
  const Branches* branches() {
    if (!use_branches || nz == 1 || njobs < 2) return nullptr;
    const int want = std::min(njobs, kMaxBranches);
    if (!br.fork) PF_CU(cudaEventCreateWithFlags(&br.fork, cudaEventDisableTiming));
    for (int b = 0; b < want; ++b) {
      if (!br.s[b]) PF_CU(cudaStreamCreateWithFlags(&br.s[b], cudaStreamNonBlocking));
      if (!br.join[b]) PF_CU(cudaEventCreateWithFlags(&br.join[b], cudaEventDisableTiming));
    }
    br.n = want;
    br.steps = job_steps.data();
    return &br;
  }

  int nmon() const { return (int)mon_ids.size(); }
  int mon_index(int id) const {
    auto it = std::find(mon_ids.begin(), mon_ids.end(), id);
    if (it == mon_ids.end()) throw PFError(E_ARG, "monomer with id = " + std::to_string(id) + " not present in system");
    return (int)(it - mon_ids.begin());
  }
  // pencils per tile of the z pass
  static int zM(int p) { return p == 1 ? z_tile_pencils<float>() : z_tile_pencils<double>(); }

  template <typename T>
  void build_twiddles(int p) {
    const int lens[3] = {nx, ny, nz};
    std::vector<Cx<T>> h;
    for (int a = 0; a < 3; ++a) {
      tw_off[p][a] = (int)h.size();
      std::vector<double> re(2048), im(2048);
      const int cnt = fft_twiddle_table(lens[a], re.data(), im.data(), 2048);
      if (cnt < 0) throw PFError(E_UNSUPPORTED, "no FFT plan for length " + std::to_string(lens[a]));
      for (int i = 0; i < cnt; ++i) h.push_back(cx<T>((T)re[i], (T)im[i]));
    }
    if (h.empty()) h.push_back(cx<T>(1, 0));
    twid[p].alloc(sizeof(Cx<T>) * h.size());
    PF_H2D(twid[p].p, h.data(), sizeof(Cx<T>) * h.size(), st);
  }
  template <typename T>
  Twiddles<T> tw(int p) const {
    const Cx<T>* b = twid[p].as<Cx<T>>();
    return Twiddles<T>{b + tw_off[p][0], b + tw_off[p][1], b + tw_off[p][2]};
  }

  CellGeom geom() const {
    CellGeom g{};
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.dim = cell.dim;
    g.signed_k = signed_k ? 1 : 0;
    for (int i = 0; i < 9; ++i) g.G[i] = cell.G[i];
    for (int i = 0; i < 9 * kMaxParams; ++i) g.dGG[i] = cell.dGG[i];
    return g;
  }

  MonomerSet monomer_set() const {
    MonomerSet ms{};
    ms.nmon = nmon();
    for (int a = 0; a < nmon(); ++a) ms.vol[a] = monomers.at(mon_ids[a]).first;
    for (auto& kv : chis) {
      const int a = mon_index(kv.first.first), b = mon_index(kv.first.second);
      ms.chi[a * kMaxMon + b] = kv.second;
      ms.chi[b * kMaxMon + a] = kv.second;
    }
    // Edwards excluded volume (edwards.jl:66-87) as the diagonal: pot_a += u_a rho_a / v_a,
    // energy (u_a / 2) (rho_a / v_a)^2
    for (auto& kv : edwards) ms.chi[mon_index(kv.first) * kMaxMon + mon_index(kv.first)] = kv.second;
    return ms;
  }

  double* grid_ptr(DevBuf& b, int mid) { return b.as<double>() + (long)mon_index(mid) * ng; }

  // ---------------------------------------------------------------- composition
  void add_monomer(int id, double vol, double charge) {
    if (nmon() >= kMaxMon && !monomers.count(id)) throw PFError(E_ARG, "too many monomer types (max 8)");
    std::vector<int> old_ids = mon_ids;
    monomers[id] = {vol, charge};
    mon_ids.clear();
    for (auto& kv : monomers) mon_ids.push_back(kv.first);
    // re-layout the per-monomer grids (add_monomer! zero-initialises the new monomer)
    DevBuf* bufs[6] = {&w, &pot, &res, &rho, &rbar, &wbar};
    for (DevBuf* b : bufs) {
      DevBuf nb;
      nb.alloc(sizeof(double) * ng * nmon());
      PF_CU(cudaMemsetAsync(nb.p, 0, nb.bytes, st));
      if (b->p) {
        for (size_t i = 0; i < old_ids.size(); ++i) {
          if (old_ids[i] == id) continue;
          const int ni = mon_index(old_ids[i]);
          PF_CU(cudaMemcpyAsync(nb.as<double>() + ni * ng, b->as<double>() + i * ng, sizeof(double) * ng,
                                cudaMemcpyDeviceToDevice, st));
        }
      }
      sync_st();
      std::swap(b->p, nb.p);
      std::swap(b->bytes, nb.bytes);
    }
    and_.reset();
    jobs_dirty[0] = jobs_dirty[1] = true;
    invalidate_graphs();
  }

  void add_multiblock(int nb, const int* bm, const int* Nb, const double* bb, int Ns, double phi) {
    if (nb < 1 || nb > 2 * kMaxMon) throw PFError(E_ARG, "number of blocks must be in [1, 16]");
    if (Ns < 1) throw PFError(E_ARG, "Ns must be positive");
    auto sp = std::make_unique<Species>();
    sp->kind = 0;
    std::set<int> ids;
    for (int i = 0; i < nb; ++i) {
      if (!monomers.count(bm[i]))
        throw PFError(E_ARG, "Species contains monomer with id = " + std::to_string(bm[i]) + " not present in system.");
      ids.insert(bm[i]);
      sp->mid_block.push_back(bm[i]);
      sp->N_block.push_back(Nb[i]);
      sp->b_block.push_back(bb[i]);
      sp->N += Nb[i];
      sp->Nref_block.push_back(monomers[bm[i]].first * Nb[i]);
    }
    sp->mids.assign(ids.begin(), ids.end());
    chain_grid(sp->Nref_block, Ns, sp->Nref, sp->begin_block, sp->ds_block);
    for (double v : sp->Nref_block) sp->f_block.push_back(v / sp->Nref);
    sp->Ns = sp->begin_block.back() - 1;  // multiblock.jl:56-59
    if (ensemble == 0 && phi <= 0.0) throw PFError(E_ARG, "Bulk volume fraction must be 0 < phi <= 1.");
    sp->phi = ensemble == 0 ? phi : 0.0;  // system.jl:148-157
    sp->mu_in = ensemble == 0 ? 0.0 : phi;
    sp->Qdev.alloc(sizeof(double));
    species.push_back(std::move(sp));
    jobs_dirty[0] = jobs_dirty[1] = true;
    invalidate_graphs();
  }

  void add_point(int mid, double phi) {
    if (!monomers.count(mid))
      throw PFError(E_ARG, "Species contains monomer with id = " + std::to_string(mid) + " not present in system.");
    if (ensemble == 0 && phi <= 0.0) throw PFError(E_ARG, "Bulk volume fraction must be 0 < phi <= 1.");
    auto sp = std::make_unique<Species>();
    sp->kind = 1;
    sp->mids = {mid};
    sp->Nref = monomers[mid].first;
    sp->phi = ensemble == 0 ? phi : 0.0;
    sp->mu_in = ensemble == 0 ? 0.0 : phi;
    sp->Qdev.alloc(sizeof(double));
    species.push_back(std::move(sp));
    invalidate_graphs();
  }

  void set_flory(int a, int b, double chi) {
    if (a == b) throw PFError(E_ARG, "AssertionError: alpha != beta");
    if (!monomers.count(a) || !monomers.count(b))
      throw PFError(E_ARG, "Interaction contains monomer not present in system.");
    chis[{std::min(a, b), std::max(a, b)}] = chi;
  }

  void set_edwards(int mid, double u) {  // set_interaction!(::EdwardsInteraction, mid, u)
    if (!monomers.count(mid)) throw PFError(E_ARG, "Interaction contains monomer not present in system.");
    edwards[mid] = u;
  }

  void set_cell(int dim, const std::string& crystal, const std::vector<double>& params) {
    const int nd = (nx > 1) + (ny > 1) + (nz > 1);
    if (dim != nd) throw PFError(E_ARG, "Number of non-singleton dimensions in System and Cell do not match!");
    const int npr = crystal_nparams(dim, crystal);
    if (npr < 0) throw PFError(E_ARG, "Unrecognized crystal system `" + crystal + "` for dim = " + std::to_string(dim) + ".");
    if ((int)params.size() != npr) throw PFError(E_ARG, "AssertionError: wrong number of cell parameters");
    cell.dim = dim;
    cell.crystal = crystal;
    cell.params = params;
    cell.update();
    has_cell = true;
    ++cell_version;
  }

  void cell_update() {
    cell.update();
    ++cell_version;
  }

  void require_ready() {
    if (!has_cell) throw PFError(E_STATE, "no unit cell set");
    if (species.empty()) throw PFError(E_STATE, "no species added");
  }

  // float32 propagators are rescaled per contour step; float64 ones follow the reference as is
  static bool scaled(int p) { return p == 1; }

  // a chain launched by this handle reports its pencil-pass timeouts to the handle's word
  template <typename T>
  void own(ChainHost<T>& h) const {
    h.status = pipe_st.as<int>();
    h.wait_ns = wait_ns;
  }

  // ---------------------------------------------------------------- propagator setup
  template <typename T>
  void ensure_prop(int p) {
    if (!jobs_dirty[p]) return;
    if (gexec[p]) cudaGraphExecDestroy(gexec[p]);
    gexec[p] = nullptr;
    graph_warm[p] = false;
    std::vector<ChainJob<T>> hjobs;
    auto& hosts = hosts_of<T>();
    auto& lds = lds_of<T>();
    hosts.clear();
    lds.clear();
    maxsteps = 0;
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind != 0) continue;
      const int nb = sp.nblocks();
      sp.q[p].alloc(sizeof(T) * (size_t)(sp.Ns + 1) * ng);
      if (nb > 1) sp.qc[p].alloc(sizeof(T) * (size_t)(sp.Ns + 1) * ng);
      sp.lw[p].clear();
      sp.ld[p].clear();
      for (int b = 0; b < nb; ++b) {
        sp.lw[p].emplace_back(new DevBuf());
        sp.lw[p].back()->alloc(sizeof(T) * ng);
        sp.ld[p].emplace_back(new DevBuf());
        sp.ld[p].back()->alloc(sizeof(T) * nk);
      }
      sp.ld_version[p] = -1;
      // step operators: forward step t (s = t -> t+1) in block b with bgn0 <= t < end0,
      // backward step t (s = Ns-t -> Ns-t-1) in block b with bgn0 < Ns-t <= end0
      std::vector<StepOp<T>> hops(2 * (size_t)sp.Ns);
      for (int t = 0; t < sp.Ns; ++t) {
        for (int b = 0; b < nb; ++b) {
          const int b0 = sp.begin_block[b] - 1, b1 = sp.begin_block[b + 1] - 1;
          if (b0 <= t && t < b1) hops[t] = StepOp<T>{sp.lw[p][b]->as<T>(), sp.ld[p][b]->as<T>()};
          const int s = sp.Ns - t;
          if (b0 < s && s <= b1) hops[sp.Ns + t] = StepOp<T>{sp.lw[p][b]->as<T>(), sp.ld[p][b]->as<T>()};
        }
      }
      sp.ops[p].alloc(sizeof(StepOp<T>) * hops.size());
      PF_H2D(sp.ops[p].p, hops.data(), sizeof(StepOp<T>) * hops.size(), st);
      const StepOp<T>* ops = sp.ops[p].as<StepOp<T>>();
      Cx<T>* kb0 = nullptr;
      Cx<T>* kb1 = nullptr;
      if (nz > 1) {
        sp.kbuf[p][0].alloc(sizeof(Cx<T>) * nk);
        kb0 = sp.kbuf[p][0].as<Cx<T>>();
        if (nb > 1) {
          sp.kbuf[p][1].alloc(sizeof(Cx<T>) * nk);
          kb1 = sp.kbuf[p][1].as<Cx<T>>();
        }
      }
      float* c0 = nullptr;
      float* c1 = nullptr;
      double* l0 = nullptr;
      double* l1 = nullptr;
      if (scaled(p)) {
        for (int j = 0; j < 2; ++j) {
          sp.csc[j].alloc(sizeof(float) * sp.Ns);
          sp.lsc[j].alloc(sizeof(double) * sp.Ns);
        }
        sp.fac.alloc(sizeof(double) * (sp.Ns + 1));
        sp.meanq.alloc(sizeof(double));
        c0 = sp.csc[0].as<float>();
        l0 = sp.lsc[0].as<double>();
        if (nb > 1) {
          c1 = sp.csc[1].as<float>();
          l1 = sp.lsc[1].as<double>();
        }
      }
      hjobs.push_back(ChainJob<T>{sp.q[p].as<T>(), ops, kb0, c0, l0, 0, +1, sp.Ns, 0});
      if (nb > 1) hjobs.push_back(ChainJob<T>{sp.qc[p].as<T>(), ops + sp.Ns, kb1, c1, l1, sp.Ns, -1, sp.Ns, 0});
      for (int dir = 0; dir < (nb > 1 ? 2 : 1); ++dir) {
        std::vector<const T*> l(sp.Ns);
        for (int t = 0; t < sp.Ns; ++t) l[t] = hops[(size_t)dir * sp.Ns + t].ld;
        lds.push_back(std::move(l));
        ChainHost<T> h;
        h.kbuf = dir ? kb1 : kb0;
        h.csc = dir ? c1 : c0;
        h.lsc = dir ? l1 : l0;
        h.nsteps = sp.Ns;
        own(h);
        hosts.push_back(h);
      }
      maxsteps = std::max(maxsteps, sp.Ns);
    }
    njobs = (int)hjobs.size();
    for (size_t j = 0; j < hosts.size(); ++j) hosts[j].ld = lds[j].data();
    job_steps.clear();
    for (const auto& j : hjobs) job_steps.push_back(j.nsteps);
    jobs[p].alloc(sizeof(ChainJob<T>) * std::max(1, njobs));
    if (njobs) PF_H2D(jobs[p].p, hjobs.data(), sizeof(ChainJob<T>) * njobs, st);
    jobs_dirty[p] = false;
  }

  // ---------------------------------------------------------------- RQM4 chains (float64)
  void ensure_rqm4() {
    rq_scratch.alloc(sizeof(double) * 5 * ng);
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind != 0) continue;
      const int nb = sp.nblocks();
      if ((int)sp.lw2.size() != nb) {
        sp.lw2.clear();
        sp.ld2.clear();
        for (int b = 0; b < nb; ++b) {
          sp.lw2.emplace_back(new DevBuf());
          sp.lw2.back()->alloc(sizeof(double) * ng);
          sp.ld2.emplace_back(new DevBuf());
          sp.ld2.back()->alloc(sizeof(double) * nk);
        }
        sp.ld2_version = -1;
      }
      // per block: ops {LW, LD} then 2 x {LW2, LD2}; jobs: one full step on [x, q1], two half
      // steps on [x, h, q2]
      std::vector<StepOp<double>> hops;
      std::vector<ChainJob<double>> hj;
      double* X = rq_scratch.as<double>();
      double* Y = X + 2 * ng;
      Cx<double>* kb = nz > 1 ? sp.kbuf[0][0].as<Cx<double>>() : nullptr;
      sp.rq_ld1.clear();
      sp.rq_ld2.clear();
      for (int b = 0; b < nb; ++b) {
        hops.push_back(StepOp<double>{sp.lw[0][b]->as<double>(), sp.ld[0][b]->as<double>()});
        hops.push_back(StepOp<double>{sp.lw2[b]->as<double>(), sp.ld2[b]->as<double>()});
        hops.push_back(StepOp<double>{sp.lw2[b]->as<double>(), sp.ld2[b]->as<double>()});
        sp.rq_ld1.push_back(sp.ld[0][b]->as<double>());
        sp.rq_ld2.push_back(sp.ld2[b]->as<double>());
      }
      sp.rq_ops.alloc(sizeof(StepOp<double>) * hops.size());
      PF_H2D(sp.rq_ops.p, hops.data(), sp.rq_ops.bytes, st);
      const StepOp<double>* ops = sp.rq_ops.as<StepOp<double>>();
      for (int b = 0; b < nb; ++b) {
        hj.push_back(ChainJob<double>{X, ops + 3 * b, kb, nullptr, nullptr, 0, +1, 1, 0});
        hj.push_back(ChainJob<double>{Y, ops + 3 * b + 1, kb, nullptr, nullptr, 0, +1, 2, 0});
      }
      sp.rq_jobs.alloc(sizeof(ChainJob<double>) * hj.size());
      PF_H2D(sp.rq_jobs.p, hj.data(), sp.rq_jobs.bytes, st);
    }
  }
  // x -> y by one RQM4 step of block b: y = (4 q2 - q1) / 3
  void rqm4_step(Species& sp, int b, const double* x, double* y) {
    double* X = rq_scratch.as<double>();
    double* Y = X + 2 * ng;
    PF_CU(cudaMemcpyAsync(X, x, sizeof(double) * ng, cudaMemcpyDeviceToDevice, st));
    PF_CU(cudaMemcpyAsync(Y, x, sizeof(double) * ng, cudaMemcpyDeviceToDevice, st));
    const ChainJob<double>* jd = sp.rq_jobs.as<ChainJob<double>>() + 2 * b;
    const GridDims dims{nx, ny, nz};
    const double* ld1[1] = {sp.rq_ld1[b]};
    const double* ld2[2] = {sp.rq_ld2[b], sp.rq_ld2[b]};
    ChainHost<double> h1, h2;
    h1.kbuf = h2.kbuf = nz > 1 ? sp.kbuf[0][0].as<Cx<double>>() : nullptr;
    h1.nsteps = 1;
    h1.ld = ld1;
    h2.nsteps = 2;
    h2.ld = ld2;
    own(h1);
    own(h2);
    launch_chains<double>(jd, 1, 1, dims, tw<double>(0), st, &h1);
    launch_chains<double>(jd + 1, 1, 2, dims, tw<double>(0), st, &h2);
    launch_rqm4_combine<double>(y, X + ng, Y + 2 * ng, ng, st);
    check_launch();
  }
  void rqm4_chains() {
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind != 0) continue;
      const int nb = sp.nblocks(), Ns = sp.Ns;
      double* q = sp.q[0].as<double>();
      for (int t = 0; t < Ns; ++t) {
        int b = 0;
        while (!(sp.begin_block[b] - 1 <= t && t < sp.begin_block[b + 1] - 1)) ++b;
        rqm4_step(sp, b, q + (long)t * ng, q + (long)(t + 1) * ng);
      }
      if (nb > 1) {
        double* qc = sp.qc[0].as<double>();
        for (int s = Ns; s >= 1; --s) {
          int b = 0;
          while (!(sp.begin_block[b] - 1 < s && s <= sp.begin_block[b + 1] - 1)) ++b;
          rqm4_step(sp, b, qc + (long)s * ng, qc + (long)(s - 1) * ng);
        }
      }
    }
  }

  // ---------------------------------------------------------------- density solve body
  bool capturing = false;
  void record_ev(int i) {
    if (capturing) PF_CU(cudaEventRecordWithFlags(ev[i], st, cudaEventRecordExternal));
    else PF_CU(cudaEventRecord(ev[i], st));
  }
  // Everything of one density solve that depends only on device pointers fixed at setup:
  // captured once per precision into a CUDA graph and replayed on later solves.  The timing
  // events are recorded as external-event nodes so that replays record them too.
  template <typename T>
  void density_enqueue(int p) {
    PF_CU(cudaMemsetAsync(rho.p, 0, sizeof(double) * ng * nmon(), st));
    record_ev(0);
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind != 0) continue;
      for (int b = 0; b < sp.nblocks(); ++b) {
        const auto& m = monomers.at(sp.mid_block[b]);
        launch_lw<T>(sp.lw[p][b]->as<T>(), grid_ptr(w, sp.mid_block[b]), sp.ds_block[b] / 2.0 * m.first, ng, st);
        if (mde == 1)  // half-step factor exp(-ds vol w / 4)
          launch_lw<double>(sp.lw2[b]->as<double>(), grid_ptr(w, sp.mid_block[b]), sp.ds_block[b] / 4.0 * m.first,
                            ng, st);
      }
      launch_fill<T>(sp.q[p].as<T>(), (T)1, ng, st);
      if (sp.nblocks() > 1) launch_fill<T>(sp.qc[p].as<T>() + (long)sp.Ns * ng, (T)1, ng, st);
    }
    record_ev(1);
    if (mde == 1) rqm4_chains();
    else if (njobs)
      launch_chains<T>(jobs[p].as<ChainJob<T>>(), njobs, maxsteps, GridDims{nx, ny, nz}, tw<T>(p), st,
                       hosts_of<T>().data(), branches());
    record_ev(2);
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind == 0) {
        const double* fac = nullptr;
        const bool grand = ensemble == 1;
        if (scaled(p)) {
          launch_sum<T>(sp.q[p].as<T>() + (long)sp.Ns * ng, ng, part.as<double>(), sp.meanq.as<double>(), (double)ng,
                        st);
          launch_scale_finalize(sp.lsc[0].as<double>(), sp.lsc[1].as<double>(), sp.nblocks() == 1, sp.Ns,
                                sp.meanq.as<double>(), sp.Qdev.as<double>(), sp.fac.as<double>(), st, !grand);
          fac = sp.fac.as<double>();
        } else {
          launch_sum<T>(sp.q[p].as<T>() + (long)sp.Ns * ng, ng, part.as<double>(), sp.Qdev.as<double>(), (double)ng,
                        st);
        }
        SimpsonBlocks sb{};
        sb.nblocks = sp.nblocks();
        for (int b = 0; b < sb.nblocks; ++b) {
          sb.mon[b] = mon_index(sp.mid_block[b]);
          sb.bgn[b] = sp.begin_block[b] - 1;
          sb.end[b] = sp.begin_block[b + 1] - 1;
          sb.ds[b] = sp.ds_block[b];
        }
        const T* qc = sp.nblocks() > 1 ? sp.qc[p].as<T>() : nullptr;
        // pooled density: phi / Q (canonical) or exp(mu) (grand: phi = Q exp(mu), system.jl:248-289)
        launch_simpson<T>(rho.as<double>(), sp.q[p].as<T>(), qc, sp.nblocks() == 1, sp.Ns, ng, sb,
                          grand ? std::exp(sp.mu_in) : sp.phi, sp.Nref,
                          grand ? one.as<double>() : sp.Qdev.as<double>(), fac, st);
      } else {
        const int mid = sp.mids[0];
        const double vol = monomers.at(mid).first;
        const bool grand = ensemble == 1;
        launch_point_q(grid_ptr(w, mid), vol, ng, part.as<double>(), sp.Qdev.as<double>(), st);
        launch_point_density(grid_ptr(rho, mid), grid_ptr(w, mid), vol, grand ? std::exp(sp.mu_in) : sp.phi,
                             grand ? one.as<double>() : sp.Qdev.as<double>(), ng, st);
      }
    }
    record_ev(3);
  }

  // ---------------------------------------------------------------- density!(sys)
  template <typename T>
  void density_t(int p) {
    require_ready();
    ensure_prop<T>(p);
    if (mde == 1) {
      if (p != 0) throw PFError(E_UNSUPPORTED, "the RQM4 propagator runs with float64 chains");
      ensure_rqm4();
    }
    // bond operators: regenerated (outside the graph) when the cell changed
    const CellGeom g = geom();
    mde_steps = 0;
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind != 0) continue;
      if (sp.ld_version[p] != cell_version)
        for (int b = 0; b < sp.nblocks(); ++b)
          launch_ld<T>(sp.ld[p][b]->as<T>(), g, sp.ds_block[b] * sp.b_block[b] * sp.b_block[b] / 6.0,
                       1.0 / (double)ng, nk, st);
      sp.ld_version[p] = cell_version;
      if (mde == 1 && sp.ld2_version != cell_version) {
        for (int b = 0; b < sp.nblocks(); ++b)
          launch_ld<double>(sp.ld2[b]->as<double>(), g, sp.ds_block[b] * sp.b_block[b] * sp.b_block[b] / 12.0,
                            1.0 / (double)ng, nk, st);
        sp.ld2_version = cell_version;
      }
      mde_steps += sp.Ns * (sp.nblocks() > 1 ? 2 : 1);
    }
    check_launch();
    if (!use_graphs || mde == 1) {
      density_enqueue<T>(p);
    } else if (gexec[p]) {
      PF_CU(cudaGraphLaunch(gexec[p], st));
      count_launches(graph_kernels[p]);
    } else if (!graph_warm[p]) {
      // first solve runs directly (it also sets the kernels' shared-memory attributes); the
      // pencil-pass schedule is tuned after it, before any capture
      density_enqueue<T>(p);
      autotune_pencil<T>(p);
      graph_warm[p] = true;
    } else {
      const long l0 = launch_total();
      PF_CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      capturing = true;
      try {
        density_enqueue<T>(p);
      } catch (...) {
        capturing = false;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      capturing = false;
      cudaGraph_t graph = nullptr;
      PF_CU(cudaStreamEndCapture(st, &graph));
      graph_kernels[p] = launch_total() - l0;
      cudaError_t e = cudaGraphInstantiate(&gexec[p], graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) throw PFError(E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      PF_CU(cudaGraphLaunch(gexec[p], st));
    }
    check_launch();
    for (auto& sp : species) sp->Q_valid = false;
    if (timing) {
      PF_CU(cudaEventSynchronize(ev[3]));
      float a = 0, b = 0;
      PF_CU(cudaEventElapsedTime(&a, ev[1], ev[2]));
      PF_CU(cudaEventElapsedTime(&b, ev[0], ev[3]));
      t_prop_ms = a;
      t_dens_ms = b;
    }
    last_prec = p;
  }
  // Pencil-pass autotuner.  The first time a 3D handle has solved a density for a transform
  // length and plane size that no handle of this process has tuned, each candidate schedule
  // (pipeline stages x tiles per CTA) reruns the first kTuneSteps contour steps of every chain
  // on the chains' branch streams, as a density solve runs them (the rerun rewrites the same
  // values), three times; the fastest of the last two timings (CUDA events) counts, and the
  // fastest candidate is kept for every later launch.  Schedules differ only in how tiles are
  // distributed, not in arithmetic, so results do not depend on the choice.  PF_NO_AUTOTUNE=1
  // keeps the default schedule.
  bool autotune = true;
  cudaEvent_t tev[2] = {nullptr, nullptr};
  template <typename T>
  void autotune_pencil(int p) {
    if (nz == 1 || njobs == 0 || mde != 0 || !autotune || capturing) return;
    const int nkp = (nx / 2 + 1) * ny;
    if (get_pencil_schedule<T>(nz, nkp, nullptr, nullptr)) return;
    static const int cands[][2] = {{2, 1}, {2, 2}, {3, 1}, {3, 2}, {3, 4}};
    constexpr int kTuneSteps = 16;
    std::vector<ChainHost<T>> hs = hosts_of<T>();
    int tsteps = 0;
    for (auto& h : hs) {
      h.nsteps = std::min(kTuneSteps, h.nsteps);
      tsteps = std::max(tsteps, h.nsteps);
    }
    const Branches* brs = branches();
    for (auto& e : tev)
      if (!e) PF_CU(cudaEventCreate(&e));
    float best = 1e30f;
    int bs = 0, brd = 0;
    for (const auto& c : cands) {
      for (auto& h : hs) {
        h.zstages = c[0];
        h.zrounds = c[1];
      }
      float tmin = 1e30f;
      for (int rep = 0; rep < 3; ++rep) {
        PF_CU(cudaEventRecord(tev[0], st));
        launch_chains<T>(jobs[p].as<ChainJob<T>>(), njobs, tsteps, GridDims{nx, ny, nz}, tw<T>(p), st, hs.data(),
                         brs);
        PF_CU(cudaEventRecord(tev[1], st));
        check_launch();
        PF_CU(cudaEventSynchronize(tev[1]));
        float ms = 0.0f;
        PF_CU(cudaEventElapsedTime(&ms, tev[0], tev[1]));
        if (rep > 0) tmin = std::min(tmin, ms);
      }
      if (tmin < best) {
        best = tmin;
        bs = c[0];
        brd = c[1];
      }
    }
    check_pipe(p);
    set_pencil_schedule<T>(nz, nkp, bs, brd);
  }
  void invalidate_graphs() {
    for (int p = 0; p < 2; ++p) {
      if (gexec[p]) cudaGraphExecDestroy(gexec[p]);
      gexec[p] = nullptr;
      graph_warm[p] = false;
    }
  }
  void density() {
    if (prec == 0) density_t<double>(0);
    else density_t<float>(1);
  }

  // relative cost of one density solve: grid points x contour steps of all chains
  double solve_cost() const {
    double steps = 0.0;
    for (const auto& sp : species)
      if (sp->kind == 0) steps += (double)sp->Ns * (sp->nblocks() > 1 ? 2 : 1);
    return (double)ng * std::max(1.0, steps);
  }
  // A pencil pass that gave up waiting on a TMA copy sets this handle's status word; read and
  // clear it (synchronises the handle's stream) and report PF_ETIMEOUT.
  void check_pipe(int = 0) {
    int v = 0;
    if (nz > 1) {  // 1D/2D chains have no pencil pass
      d2h_pin(kPinBytes - sizeof(int), pipe_st.p, sizeof(int));
      PF_CU(cudaMemsetAsync(pipe_st.p, 0, sizeof(int), st));
    }
    sync_st();
    if (nz > 1) std::memcpy(&v, hpin + kPinBytes - sizeof(int), sizeof(int));
    if (v)
      throw PFError(E_TIMEOUT, "pencil pass: a TMA copy did not complete within its time limit; the last density "
                               "solve is invalid");
  }
  void fetch_Q() {
    size_t k = 0;
    for (auto& sp : species) {
      if (!sp->Q_valid) d2h_pin(sizeof(double) * k, sp->Qdev.p, sizeof(double));
      ++k;
    }
    sync_st();
    check_pipe(last_prec);
    k = 0;
    for (auto& sp : species) {
      if (!sp->Q_valid) std::memcpy(&sp->Q, hpin + sizeof(double) * k, sizeof(double));
      ++k;
    }
    for (auto& sp : species) {
      sp->Q_valid = true;
      if (ensemble == 0) {
        sp->mu = std::log(sp->phi / sp->Q);  // muphi! canonical (system.jl:248-259)
      } else {
        sp->mu = sp->mu_in;  // muphi! grand: phi = Q exp(mu)
        sp->phi = sp->Q * std::exp(sp->mu_in);
      }
    }
  }

  // ---------------------------------------------------------------- residuals!(sys)
  void residuals() {
    density();
    launch_residuals(w.as<double>(), pot.as<double>(), res.as<double>(), rho.as<double>(), monomer_set(), ng,
                     ensemble == 0, part.as<double>(), sums.as<double>(), st);  // mean-subtract: canonical only
    check_launch();
  }

  // field_error and free_energy from one reduction pass
  void stats(double& ferr, double& fhelm) {
    if (ensemble == 1) fetch_Q();  // phi = Q exp(mu) enters the translational term
    launch_stats(w.as<double>(), res.as<double>(), rho.as<double>(), monomer_set(), ng, part.as<double>(),
                 stats4.as<double>(), st);
    check_launch();
    double s[4];
    d2h_pin(0, stats4.p, sizeof(s));
    check_pipe();  // also synchronises: a timed-out pencil pass invalidates these sums
    std::memcpy(s, hpin, sizeof(s));
    ferr = std::sqrt(s[0]) / std::sqrt(2.220446049250313e-16 + s[1]);
    double ftrans = 0.0;
    for (auto& sp : species) {
      const double phi = sp->phi, mu = sp->phi;  // quirk Q3 (system.jl:407)
      if (phi > 1e-8) ftrans += phi * (mu - 1.0) / sp->Nref;
    }
    double ffield = -s[2];
    ffield /= (double)ng;
    fhelm = ftrans + ffield + s[3] / (double)ng;
  }

  double free_energy_bulk() {
    std::map<int, double> fr;
    for (int id : mon_ids) fr[id] = 0.0;
    double f = 0.0;
    for (auto& sp : species) {
      if (sp->phi > 1e-8) f += sp->phi * (std::log(sp->phi) - 1.0) / sp->Nref;
      for (int mid : sp->mids) fr[mid] += sp->phi * sp->monomer_fraction(mid);
    }
    double e = 0.0;
    for (auto& kv : chis) {
      const double va = monomers.at(kv.first.first).first, vb = monomers.at(kv.first.second).first;
      e += kv.second * (fr[kv.first.first] / va) * (fr[kv.first.second] / vb);
    }
    for (auto& kv : edwards) {  // edwards.jl:49-64
      const double v = monomers.at(kv.first).first;
      e += kv.second / 2.0 * (fr[kv.first] / v) * (fr[kv.first] / v);
    }
    return f + e;
  }

  void validate() {  // system.jl:192-237
    require_ready();
    // fields initialised: some field with nonzero mean or std
    launch_stats(w.as<double>(), w.as<double>(), w.as<double>(), monomer_set(), ng, part.as<double>(),
                 stats4.as<double>(), st);
    check_launch();
    double s[4];
    d2h_now(s, stats4.p, sizeof(s));
    if (s[1] == 0.0) throw PFError(E_ARG, "Fields must be initialized before SCFT simulation.");
    double phisum = 0.0;
    for (auto& sp : species) phisum += sp->phi;
    if (ensemble == 0 && !isapprox(phisum, 1.0))
      throw PFError(E_ARG, "Species volume fractions do not sum to unity.");
    double charge = 0.0;
    for (int id : mon_ids) {
      double fr = 0.0;
      for (auto& sp : species) fr += sp->phi * sp->monomer_fraction(id);
      charge += fr * monomers.at(id).second / monomers.at(id).first;
    }
    if (!(charge == 0.0)) throw PFError(E_ARG, "Bulk system not charge neutral.");
    for (int id : mon_ids) {
      bool found = false;
      for (auto& sp : species)
        if (std::find(sp->mids.begin(), sp->mids.end(), id) != sp->mids.end()) found = true;
      if (!found) throw PFError(E_ARG, "Monomer with ID = " + std::to_string(id) + " not found in any species.");
    }
  }

  // ---------------------------------------------------------------- scfstress(sys)
  template <typename T>
  std::vector<double> chain_dQ(Species& sp, int p) {
    const int npr = cell.np();
    std::vector<double> dQ(npr, 0.0);
    struct It { const T* q; const T* qc; double w; double b; };
    std::vector<It> items;
    for (int b = 0; b < sp.nblocks(); ++b) {
      const int bgn = sp.begin_block[b], end = sp.begin_block[b + 1];
      for (int s = bgn; s <= end; ++s) {
        double ds = sp.ds_block[b];
        if (s != bgn && s != end) ds *= (s % 2 == 0) ? 4.0 : 2.0;
        const long s0 = s - 1;
        const T* q = sp.q[p].as<T>() + s0 * ng;
        const T* qc = sp.nblocks() > 1 ? sp.qc[p].as<T>() + s0 * ng : sp.q[p].as<T>() + (sp.Ns - s0) * ng;
        items.push_back(It{q, qc, ds, sp.b_block[b]});
      }
    }
    const int nit = (int)items.size();
    std::vector<double> qint(nit * (size_t)npr, 0.0);
    // rescaled histories: each term carries fac[s] = exp(-L_s - L'_s - log Q), so Q is
    // already divided out
    std::vector<double> hfac;
    std::vector<int> item_s;
    if (scaled(p)) {
      hfac.resize(sp.Ns + 1);
      d2h_now(hfac.data(), sp.fac.p, sizeof(double) * (sp.Ns + 1));
      for (int b = 0; b < sp.nblocks(); ++b)
        for (int s = sp.begin_block[b]; s <= sp.begin_block[b + 1]; ++s) item_s.push_back(s - 1);
    }
    const GridDims d{nx, ny, nz};
    if (nz == 1) {
      std::vector<StressItem<T>> h(nit);
      for (int i = 0; i < nit; ++i) h[i] = StressItem<T>{items[i].q, items[i].qc};
      DevBuf di, dp;
      di.alloc(sizeof(StressItem<T>) * nit);
      dp.alloc(sizeof(double) * nit * npr);
      PF_CU(cudaMemcpyAsync(di.p, h.data(), di.bytes, cudaMemcpyHostToDevice, st));
      launch_stress<T>(di.as<StressItem<T>>(), nit, nullptr, nullptr, nullptr, nullptr, d, dksq.as<double>(), npr,
                       dp.as<double>(), tw<T>(p), st);
      check_launch();
      d2h_now(qint.data(), dp.p, dp.bytes);
    } else {
      const int M = zM(p);
      const int nkp = (nx / 2 + 1) * ny;
      const int ntiles = (nkp + M - 1) / M;
      const int chunk = 16;
      DevBuf kq, kqc, ptrs, dp;
      kq.alloc(sizeof(Cx<T>) * nk * chunk);
      kqc.alloc(sizeof(Cx<T>) * nk * chunk);
      ptrs.alloc(sizeof(void*) * 4 * chunk);
      dp.alloc(sizeof(double) * (size_t)chunk * ntiles * npr);
      std::vector<double> hp((size_t)chunk * ntiles * npr);
      for (int c0 = 0; c0 < nit; c0 += chunk) {
        const int cn_ = std::min(chunk, nit - c0);
        std::vector<void*> hptr(4 * chunk);
        for (int i = 0; i < cn_; ++i) {
          hptr[i] = (void*)items[c0 + i].q;
          hptr[chunk + i] = (void*)items[c0 + i].qc;
          hptr[2 * chunk + i] = (void*)(kq.as<Cx<T>>() + (long)i * nk);
          hptr[3 * chunk + i] = (void*)(kqc.as<Cx<T>>() + (long)i * nk);
        }
        PF_CU(cudaMemcpyAsync(ptrs.p, hptr.data(), sizeof(void*) * 4 * chunk, cudaMemcpyHostToDevice, st));
        void** pp = ptrs.as<void*>();
        launch_stress<T>(nullptr, cn_, (const T* const*)pp, (const T* const*)(pp + chunk),
                         (Cx<T>* const*)(pp + 2 * chunk), (Cx<T>* const*)(pp + 3 * chunk), d, dksq.as<double>(), npr,
                         dp.as<double>(), tw<T>(p), st);
        check_launch();
        d2h_now(hp.data(), dp.p, sizeof(double) * (size_t)cn_ * ntiles * npr);
        for (int i = 0; i < cn_; ++i)
          for (int k = 0; k < npr; ++k) {
            double s = 0.0;
            for (int t = 0; t < ntiles; ++t) s += hp[((size_t)i * ntiles + t) * npr + k];
            qint[(size_t)(c0 + i) * npr + k] = s;
          }
      }
    }
    const double ng2 = (double)ng * (double)ng;
    for (int i = 0; i < nit; ++i) {
      const double f = scaled(p) ? hfac[item_s[i]] : 1.0;
      for (int k = 0; k < npr; ++k)
        dQ[k] -= items[i].b * items[i].b * items[i].w * (qint[(size_t)i * npr + k] * f) / 6.0 / ng2;
    }
    for (int k = 0; k < npr; ++k) {
      dQ[k] /= 3.0;
      // rescaled canonical chains carry 1/Q in fac[s]; grand-canonical fac[s] does not
      dQ[k] /= (scaled(p) && ensemble == 0) ? sp.Nref : sp.Q * sp.Nref;
    }
    return dQ;
  }

  std::vector<double> scfstress() {
    require_ready();
    if (last_prec < 0) throw PFError(E_STATE, "scfstress needs a density solve first");
    const int npr = cell.np();
    if (dksq_version != cell_version) {
      dksq.alloc(sizeof(double) * nk * std::max(1, npr));
      launch_dksq(dksq.as<double>(), geom(), npr, nk, st);
      check_launch();
      dksq_version = cell_version;
    }
    fetch_Q();
    std::vector<double> stress(npr, 0.0);
    for (auto& sp : species) {
      if (sp->kind != 0) continue;
      std::vector<double> dQ = last_prec == 0 ? chain_dQ<double>(*sp, 0) : chain_dQ<float>(*sp, 1);
      for (int k = 0; k < npr; ++k) stress[k] -= sp->phi * dQ[k];
    }
    return stress;
  }

  // ---------------------------------------------------------------- Anderson (anderson.jl)
  double* hist_slot(DevBuf& b, int logical) {
    const int nslot = and_.nhist + 1;
    const int phys = (and_.base + logical) % nslot;
    return b.as<double>() + (long)phys * nmon() * ng;
  }

  void anderson_setup() {  // anderson.jl:54-92
    if (!and_.exists) throw PFError(E_STATE, "no AndersonUpdater created");
    if (and_.is_setup) {
      fprintf(stderr, "Warning: Using previous iterations in AndersonUpdater history.\n");
      return;
    }
    if (ensemble != 0)  // anderson.jl:61-63
      throw PFError(E_STATE, "Anderson mixing can only be used for systems in the canonical ensemble.");
    const size_t slot = sizeof(double) * nmon() * ng;
    and_.res_hist.alloc(slot * (and_.nhist + 1));
    and_.field_hist.alloc(slot * (and_.nhist + 1));
    and_.sum_hist.alloc(slot * (and_.nhist + 1));
    and_.gram_p.alloc(sizeof(double) * kMaxHist * kMaxHist);
    and_.gram_t.alloc(sizeof(double) * kMaxHist);
    PF_CU(cudaMemsetAsync(and_.res_hist.p, 0, and_.res_hist.bytes, st));
    PF_CU(cudaMemsetAsync(and_.field_hist.p, 0, and_.field_hist.bytes, st));
    and_.base = 0;
    PF_CU(cudaMemcpyAsync(hist_slot(and_.field_hist, 0), w.p, slot, cudaMemcpyDeviceToDevice, st));
    and_.iter = 0;
    and_.iter_hist = 0;
    and_.lam = 0.0;
    and_.is_setup = true;
  }

  // ---------------------------------------------------------------- Euler / Momentum
  void simple_setup() {  // euler.jl:31-35, momentum.jl:49-61
    if (!su) throw PFError(E_STATE, "no field updater created");
    const long nall = (long)nmon() * ng;
    su->temp.alloc(sizeof(double) * nall);
    PF_CU(cudaMemcpyAsync(su->temp.p, w.p, sizeof(double) * nall, cudaMemcpyDeviceToDevice, st));
    if (su->kind == 2) {
      su->mt.alloc(sizeof(double) * nall);
      su->vt.alloc(sizeof(double) * nall);
      PF_CU(cudaMemsetAsync(su->mt.p, 0, su->mt.bytes, st));
      PF_CU(cudaMemsetAsync(su->vt.p, 0, su->vt.bytes, st));
    }
    su->is_setup = true;
  }
  void simple_step() {  // euler.jl:37-65, momentum.jl:63-165
    if (!su || !su->is_setup) throw PFError(E_STATE, "field updater not set up");
    const long nall = (long)nmon() * ng;
    double* wp = w.as<double>();
    double* rp = res.as<double>();
    double* tp = su->temp.as<double>();
    if (su->kind == 1) {
      launch_euler_predict(wp, tp, rp, su->lam, nall, st);
      residuals();
      launch_euler_correct(wp, tp, rp, su->lam, nall, st);
      if (su->method == 1) residuals();
    } else if (su->method == 3) {
      launch_nag_ahead(wp, tp, su->mt.as<double>(), su->lam, nall, st);
      residuals();
      launch_nag_update(wp, tp, su->mt.as<double>(), rp, su->lam, su->gamma, nall, st);
    } else {
      residuals();
      launch_momentum(su->method, wp, su->mt.as<double>(), su->vt.as<double>(), rp, su->lam, su->beta1, su->beta2, nall,
                      st);
    }
    check_launch();
  }
  void updater_setup() {
    if (active == 0) anderson_setup();
    else simple_setup();
  }
  void updater_step() {
    if (active == 0) anderson_step();
    else simple_step();
  }

  // Mixed precision: at the float32 -> float64 switch the history holds residuals with
  // float32 rounding (~1e-7 relative), as large as the differences the float64 phase has to
  // resolve; the history restarts from the current field exactly as setup! starts it
  // (anderson.jl:54-92: iteration count 0, the field as the only history entry).
  void anderson_restart() {
    if (!and_.is_setup) return;
    const size_t slot = sizeof(double) * nmon() * ng;
    and_.base = 0;
    PF_CU(cudaMemcpyAsync(hist_slot(and_.field_hist, 0), w.p, slot, cudaMemcpyDeviceToDevice, st));
    and_.iter = 0;
    and_.iter_hist = 0;
    and_.lam = 0.0;
  }

  // ---------------------------------------------------------------- Newton-Krylov polish
  // The float64 phase of a mixed run, as inexact Newton steps on F64(w) = 0 (F = residuals!
  // with float64 propagators): w <- w + delta with J delta = -F64(w) solved by restarted GMRES
  // whose Jacobian-vector products are finite differences of float32 residuals about w,
  //   J v ~ (F32(w + e v) - F32(w)) / e,   e |v| = kNKStep |w|.
  // A perturbation of 0.1% of the field balances the two errors of a product: float32 rounding
  // (~1e-7 of |w| in the residual, ~1e-4 of the product) and the one-sided difference's
  // truncation (~1e-3 of it; at 1% the truncation limited each Newton step to shrinking ferr
  // 6-10x and the GMRES solves to 1e-2 were largely wasted).  Only the acceptance test and the
  // right-hand side are float64 solves.  The forcing term (the GMRES tolerance relative to
  // |F64|) is 0.3 far from the answer and no tighter than kNKEtaMin: tighter solves buy no more
  // per Newton step than the finite-difference Jacobian allows (at 0.1 a 128^3 run stalled and
  // fell back to float64 updater steps).  Measured on the 128^3 blend from a switch at ferr
  // 3e-3: 221 float32 products and 5 float64 residuals (4.5 s) against 290 and 6 (5.4 s) with a
  // 1% step and a floor of 1e-2.  The fixed point is the reference's: a run ends only when the
  // float64 ferr < ftol.
  static constexpr int kNKRestart = 30;      // GMRES restart length
  static constexpr int kNKMaxMatvec = 240;   // float32 products per Newton step at most
  static constexpr double kNKStep = 1e-3;
  static constexpr double kNKEtaMin = 3e-2;
  struct NKBufs {
    DevBuf V, wk, r64, r32, z, delta, h, part;
  } nkb;
  int nk_fp32 = 0, nk_fp64 = 0;

  double nk_dot(const double* a, const double* b, long n) {
    double* hd = nkb.h.as<double>() + 3 * (kNKRestart + 2);
    launch_multidot(a, 1, n, b, nkb.part.as<double>(), hd, st);
    double v = 0.0;
    d2h_now(&v, hd, sizeof(double));
    return v;
  }
  // z = (F32(wk + e v) - F32(wk)) / e with e = kNKStep |wk| / vnorm
  void nk_jvp(const double* v, double vnorm, double wnorm, long n) {
    const double e = kNKStep * wnorm / vnorm;
    double* wp = w.as<double>();
    PF_CU(cudaMemcpyAsync(wp, nkb.wk.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    launch_lincomb(wp, v, 1.0, e, n, st);
    prec = 1;
    residuals();
    double* z = nkb.z.as<double>();
    PF_CU(cudaMemcpyAsync(z, res.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    launch_lincomb(z, nkb.r32.as<double>(), 1.0 / e, -1.0 / e, n, st);
    check_launch();
    ++nk_fp32;
  }
  // Returns true once the float64 ferr < ftol; false when a Newton step did not shrink ferr
  // (the fields are then the last accepted ones and the caller goes on with float64 steps of
  // its field updater).  Each Newton step counts as one scft! step.
  bool nk_polish(const pf_scft_options& o, int& step, double& ferr, double& fhelm) {
    const long n = (long)nmon() * ng;
    const int m = kNKRestart;
    nkb.V.alloc(sizeof(double) * n * (m + 1));
    for (DevBuf* b : {&nkb.wk, &nkb.r64, &nkb.r32, &nkb.z, &nkb.delta}) b->alloc(sizeof(double) * n);
    nkb.h.alloc(sizeof(double) * 4 * (m + 2));
    nkb.part.alloc(sizeof(double) * polish_part_doubles());
    double* V = nkb.V.as<double>();
    double* hd = nkb.h.as<double>();
    double* wk = nkb.wk.as<double>();
    double* r64 = nkb.r64.as<double>();
    double* z = nkb.z.as<double>();
    double* delta = nkb.delta.as<double>();
    prec = 0;
    residuals();
    stats(ferr, fhelm);
    ++nk_fp64;
    int poor = 0;
    std::vector<double> H((size_t)(m + 1) * m), g(m + 1), cs(m), sn(m), y(m), hh(2 * (m + 1) + 1);
    while (ferr >= o.ftol && step < o.nsteps) {
      PF_CU(cudaMemcpyAsync(wk, w.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      PF_CU(cudaMemcpyAsync(r64, res.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      const double beta = std::sqrt(nk_dot(r64, r64, n));
      const double wnorm = std::sqrt(nk_dot(wk, wk, n));
      // float32 residual at the linearisation point
      prec = 1;
      residuals();
      PF_CU(cudaMemcpyAsync(nkb.r32.p, res.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      ++nk_fp32;
      const double eta = std::min(0.3, std::max(kNKEtaMin, 0.3 * o.ftol / ferr));  // forcing term
      PF_CU(cudaMemsetAsync(delta, 0, sizeof(double) * n, st));
      // first cycle: V_0 = -r64 / beta
      PF_CU(cudaMemcpyAsync(V, r64, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      launch_lincomb(V, V, -1.0 / beta, 0.0, n, st);
      double rcur = beta;
      int matvecs = 0;
      for (;;) {
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = rcur;
        int jl = -1;
        double resid = rcur;
        for (int j = 0; j < m; ++j) {
          nk_jvp(V + (long)j * n, 1.0, wnorm, n);
          ++matvecs;
          // classical Gram-Schmidt, twice
          launch_multidot(V, j + 1, n, z, nkb.part.as<double>(), hd, st);
          launch_multiaxpy(z, V, j + 1, n, hd, 1.0, -1.0, st);
          launch_multidot(V, j + 1, n, z, nkb.part.as<double>(), hd + (m + 1), st);
          launch_multiaxpy(z, V, j + 1, n, hd + (m + 1), 1.0, -1.0, st);
          launch_multidot(z, 1, n, z, nkb.part.as<double>(), hd + 2 * (m + 1), st);
          check_launch();
          d2h_now(hh.data(), hd, sizeof(double) * (2 * (m + 1) + 1));
          for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hh[i] + hh[m + 1 + i];
          const double hn = std::sqrt(std::max(0.0, hh[2 * (m + 1)]));
          H[(size_t)(j + 1) * m + j] = hn;
          if (hn > 0.0) {
            PF_CU(cudaMemcpyAsync(V + (long)(j + 1) * n, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            launch_lincomb(V + (long)(j + 1) * n, z, 1.0 / hn, 0.0, n, st);
          }
          for (int i = 0; i < j; ++i) {  // earlier Givens rotations on column j
            const double a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
            H[(size_t)i * m + j] = cs[i] * a + sn[i] * b;
            H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
          }
          const double a = H[(size_t)j * m + j], b = H[(size_t)(j + 1) * m + j];
          const double rr = std::hypot(a, b);
          cs[j] = rr > 0.0 ? a / rr : 1.0;
          sn[j] = rr > 0.0 ? b / rr : 0.0;
          H[(size_t)j * m + j] = rr;
          H[(size_t)(j + 1) * m + j] = 0.0;
          g[j + 1] = -sn[j] * g[j];
          g[j] = cs[j] * g[j];
          jl = j;
          resid = std::fabs(g[j + 1]);
          if (resid <= eta * beta || matvecs >= kNKMaxMatvec || hn == 0.0) break;
        }
        // delta += V y with H y = g (upper triangular, jl + 1 columns)
        for (int i = jl; i >= 0; --i) {
          double s = g[i];
          for (int k = i + 1; k <= jl; ++k) s -= H[(size_t)i * m + k] * y[k];
          y[i] = H[(size_t)i * m + i] != 0.0 ? s / H[(size_t)i * m + i] : 0.0;
        }
        PF_H2D(hd + 3 * (m + 1), y.data(), sizeof(double) * (jl + 1), st);
        launch_multiaxpy(delta, V, jl + 1, n, hd + 3 * (m + 1), 1.0, 1.0, st);
        if (resid <= eta * beta || matvecs >= kNKMaxMatvec) break;
        // restart from the true linear residual -r64 - J delta
        const double dn = std::sqrt(nk_dot(delta, delta, n));
        nk_jvp(delta, dn, wnorm, n);
        ++matvecs;
        PF_CU(cudaMemcpyAsync(V, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        launch_lincomb(V, r64, -1.0, -1.0, n, st);
        rcur = std::sqrt(nk_dot(V, V, n));
        if (!(rcur > 0.0)) break;
        launch_lincomb(V, V, 1.0 / rcur, 0.0, n, st);
      }
      // Newton step, accepted on a float64 residual
      double* wp = w.as<double>();
      PF_CU(cudaMemcpyAsync(wp, wk, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      launch_lincomb(wp, delta, 1.0, 1.0, n, st);
      prec = 0;
      residuals();
      double fe = 0.0, fh = 0.0;
      stats(fe, fh);
      ++nk_fp64;
      step += 1;
      if (o.nsout > 0)
        printf("Newton-Krylov step %d: ferr = %8e, fhelm = %.5e (%d float32 products)\n", step, fe, fh, matvecs);
      if (!(fe < ferr)) {  // no progress: back to the last accepted fields
        PF_CU(cudaMemcpyAsync(wp, wk, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        residuals();
        stats(ferr, fhelm);
        ++nk_fp64;
        return false;
      }
      const bool slow = !(fe < 0.5 * ferr);
      ferr = fe;
      fhelm = fh;
      if (slow && ++poor >= 2) return ferr < o.ftol;
    }
    return ferr < o.ftol;
  }

  void anderson_step() {  // anderson.jl:98-228
    if (!and_.is_setup) throw PFError(E_STATE, "AndersonUpdater not set up");
    auto& A = and_;
    A.iter += 1;
    if (A.iter < A.nhist + 1) {
      A.iter_hist = A.iter - 1;
      A.lam = 1.0 - std::pow(0.9, A.iter);
    } else {
      A.iter_hist = A.nhist;
      A.lam = 1.0;
    }
    const int it = A.iter, ih = A.iter_hist;
    const long nall = (long)nmon() * ng;
    residuals();
    PF_CU(cudaMemcpyAsync(hist_slot(A.res_hist, ih), res.p, sizeof(double) * nall, cudaMemcpyDeviceToDevice, st));
    HistPtrs h{};
    for (int j = 0; j <= ih; ++j) {
      h.res[j] = hist_slot(A.res_hist, j);
      h.field[j] = hist_slot(A.field_hist, j);
      h.sum[j] = hist_slot(A.sum_hist, j);
    }
    // U and V from the current residual's products with the window and the cached pair
    // products of the older entries; every iteration (Euler warm-up included) adds its row, so
    // the cache covers every pair of the window
    int* flag = status.as<int>() + 1;
    launch_gram_cached(h, res.as<double>(), ih, nall, A.gram_p.as<double>(), A.nhist + 1, A.base, part.as<double>(),
                       A.gram_t.as<double>(), packed.as<double>(), flag, st);
    if (it <= A.iter_euler) {
      launch_add(h.sum[ih], h.field[ih], h.res[ih], nall, st);
      launch_axpy(w.as<double>(), res.as<double>(), A.lam_euler, nall, st);
    } else {
      launch_solve(packed.as<double>(), ih, cn.as<double>(), status.as<int>(), st);
      check_launch();
      int sv[2] = {0, 0};
      d2h_now(sv, status.p, sizeof(int) * 2);
      if (sv[1] != 0) {
        // cancellation guard of the expanded sums: sum U and V directly
        launch_gram(h, ih, nall, part.as<double>(), packed.as<double>(), st);
        launch_solve(packed.as<double>(), ih, cn.as<double>(), status.as<int>(), st);
        check_launch();
        d2h_now(sv, status.p, sizeof(int));
      }
      if (sv[0] != 0)
        throw PFError(E_SINGULAR, "Error inverting Umn matrix on iteration " + std::to_string(it) +
                                      ": SingularException(" + std::to_string(sv[0]) + ")");
      launch_mix(w.as<double>(), h, ih, cn.as<double>(), A.lam, nall, st);
    }
    check_launch();
    if (it < A.nhist + 1) {
      PF_CU(cudaMemcpyAsync(hist_slot(A.field_hist, it), w.p, sizeof(double) * nall, cudaMemcpyDeviceToDevice, st));
    } else {
      A.base = (A.base + 1) % (A.nhist + 1);
      PF_CU(cudaMemcpyAsync(hist_slot(A.field_hist, A.nhist), w.p, sizeof(double) * nall, cudaMemcpyDeviceToDevice, st));
    }
  }

  // ---------------------------------------------------------------- Domain (domain.jl)
  double stress_error() const {
    double s = 0.0;
    for (double v : dom.stress) s += v * v;
    return std::sqrt(s);
  }
  void domain_setup() {
    if (!dom.exists) throw PFError(E_STATE, "no DomainUpdater created");
    const int npr = cell.np();
    dom.stress = scfstress();
    dom.oldparams.assign(npr, 0.0);
    dom.step.assign(npr, 0.0);
    dom.dstress.assign(npr * npr, 0.0);
    dom.is_setup = true;
  }
  // FD step of the Jacobian: the reference's 1e-8 (domain.jl:101) for FP64 propagators; in
  // FP32 the stress carries ~1e-7 relative noise, so the FP32 phase of a mixed run uses 1e-4.
  double fd_dx() const { return prec == 0 ? 1e-8 : 1e-4; }
  void dstress_update() {  // domain.jl:94-121
    const int npr = cell.np();
    dom.oldparams = cell.params;
    const double dx = fd_dx();
    const double x = 1.0 / dx;
    for (int k = 0; k < npr; ++k) {
      cell.params = dom.oldparams;
      cell.params[k] += dx;
      cell_update();
      density();
      std::vector<double> ps = scfstress();
      for (int i = 0; i < npr; ++i) dom.dstress[i * npr + k] = x * (ps[i] - dom.stress[i]);
    }
    cell.params = dom.oldparams;
    // The reference re-runs density! here with the stale perturbed cell (quirk Q4).  Its
    // result is overwritten by the residuals! that follows the Newton step before anything
    // reads it, so the solve is skipped.
  }
  void domain_step(int nsteps, bool stress_current) {  // domain.jl:50-92
    if (!dom.is_setup) throw PFError(E_STATE, "DomainUpdater not set up");
    const int npr = cell.np();
    if (!stress_current) dom.stress = scfstress();
    for (int iter = 0; iter < nsteps; ++iter) {
      dstress_update();
      if (cell.dim == 1) {
        for (int k = 0; k < npr; ++k) dom.step[k] = -1.0 * dom.stress[0] / dom.dstress[0];
      } else {
        std::vector<double> inv;
        if (!lu_inverse(dom.dstress, npr, inv)) throw PFError(E_SINGULAR, "SingularException in DomainUpdater");
        for (int i = 0; i < npr; ++i) {
          double s = 0.0;
          for (int j = 0; j < npr; ++j) s += inv[i * npr + j] * dom.stress[j];
          dom.step[i] = -1.0 * s;
        }
      }
      double ss = 0.0;
      for (double v : dom.step) ss += v * v;
      const double step_size = std::sqrt(ss);
      if (step_size > dom.pmax)
        for (double& v : dom.step) v *= dom.pmax / step_size;
      for (int k = 0; k < npr; ++k) {
        cell.params[k] += dom.lam * dom.step[k];
        cell.params[k] = dom.rlxn * cell.params[k] + (1 - dom.rlxn) * dom.oldparams[k];
      }
      cell_update();
      // density!(sys) directly followed by residuals!(sys) recomputes the same density
      // twice in the reference; one solve gives the identical state.
      residuals();
      dom.stress = scfstress();
    }
  }

  // ---------------------------------------------------------------- pullback of density!
  // Simpson weight of offset i in a block of n intervals (multiblock.jl:209-222)
  static double simpson_w(int i, int n) {
    if (i == 0 || i == n) return (n == 0) ? 2.0 : 1.0;
    return (i % 2 == 1) ? 4.0 : 2.0;
  }

  // dL/dw (into wbar), dL/dtheta of the cell and dL/dNref_b of every Multiblock block for a
  // loss with dL/drho = rbar, at the current fields and cell.  Runs density!(sys) first so
  // that the histories it differentiates are those of the current state.  Adjoint walks:
  // forward chain t = Ns-1 .. 0 and backward chain s = 1 .. Ns, one contour step at a time
  // through the forward kernels (the block operator is symmetric).
  template <typename T>
  void pullback_t(int p, std::vector<double>& cell_bar, std::vector<double>& nref_bar, bool recompute = true) {
    require_ready();
    if (mde != 0) throw PFError(E_UNSUPPORTED, "the pullback differentiates the RK2 propagator");
    if (ensemble != 0) throw PFError(E_UNSUPPORTED, "the pullback differentiates the canonical ensemble");
    if (recompute || last_prec != p) density_t<T>(p);
    fetch_Q();
    const int npr = cell.np(), nw = npr + 1;
    const CellGeom g = geom();
    const GridDims dims{nx, ny, nz};
    cell_bar.assign(npr, 0.0);
    nref_bar.clear();
    PF_CU(cudaMemsetAsync(wbar.p, 0, wbar.bytes, st));
    int nbmax = 1;
    for (auto& sp : species) nbmax = std::max(nbmax, sp->kind == 0 ? sp->nblocks() : 1);
    DevBuf lamh, u, G, acc, part, wts, kq, ptrs, dpart, dots, rsp, jobsd;
    lamh.alloc(sizeof(T) * 2 * ng);
    u.alloc(sizeof(T) * 2 * ng);
    G.alloc(sizeof(double) * nbmax * ng);
    acc.alloc(sizeof(double) * nbmax * nw);
    const int M = zM(p);
    const long ntiles = ((nx / 2 + 1) * (long)ny + M - 1) / M;
    part.alloc(sizeof(double) * (size_t)std::max<long>(1, ntiles) * nw);
    wts.alloc(sizeof(double) * (size_t)nbmax * nw * nk);
    kq.alloc(sizeof(Cx<T>) * 2 * nk);
    dpart.alloc(sizeof(double) * kRedBlocks);
    dots.alloc(sizeof(double) * 4 * kMaxMon);
    rsp.alloc(sizeof(double) * nmon() * ng);
    T* lam = lamh.as<T>();
    T* rr = lam + ng;
    T* u1 = u.as<T>();
    T* u2 = u1 + ng;
    Cx<T>* k1 = kq.as<Cx<T>>();
    Cx<T>* k2 = k1 + nk;
    {
      const void* hp[4] = {u1, u2, k1, k2};
      ptrs.alloc(sizeof(hp));
      PF_CU(cudaMemcpyAsync(ptrs.p, hp, sizeof(hp), cudaMemcpyHostToDevice, st));
    }
    const T* const* src_dev = reinterpret_cast<const T* const*>(ptrs.as<void*>());
    Cx<T>* const* dst_dev = reinterpret_cast<Cx<T>* const*>(ptrs.as<void*>() + 2);
    const double* rb = rbar.as<double>();
    // checkpointed walks: each chain's propagators are recomputed segment by segment (K steps
    // from the stored checkpoint q_{cK}) into a (K+1)-grid buffer, with scratch rescale factors
    const int K = adj_ckpt;
    DevBuf segb, segcsc, seglsc, segjobs;
    if (K > 0) {
      segb.alloc(sizeof(T) * (size_t)(K + 1) * ng);
      segcsc.alloc(sizeof(float) * K);
      seglsc.alloc(sizeof(double) * K);
    }
    int jobidx = 0;  // index of the species' forward job in the host views
    auto dot_host = [&](const double* a, const double* b) {
      launch_ddot(a, b, ng, dpart.as<double>(), dots.as<double>(), st);
      double v = 0.0;
      d2h_now(&v, dots.p, sizeof(double));
      return v;
    };
    for (auto& spp : species) {
      Species& sp = *spp;
      if (sp.kind == 1) {  // point species (point.jl:36-58)
        const int mid = sp.mids[0];
        const double vol = monomers.at(mid).first;
        PF_CU(cudaMemsetAsync(rsp.p, 0, rsp.bytes, st));
        launch_point_density(grid_ptr(rsp, mid), grid_ptr(w, mid), vol, sp.phi, sp.Qdev.as<double>(), ng, st);
        const double S = dot_host(rb + (long)mon_index(mid) * ng, grid_ptr(rsp, mid));
        launch_adj_point(grid_ptr(wbar, mid), grid_ptr(rsp, mid), rb + (long)mon_index(mid) * ng, grid_ptr(w, mid),
                         vol, S, (double)ng * sp.Q, ng, st);
        continue;
      }
      const int nb = sp.nblocks(), Ns = sp.Ns;
      const bool homo = nb == 1;
      const T* q = sp.q[p].as<T>();
      const T* qc = homo ? nullptr : sp.qc[p].as<T>();
      auto b0 = [&](int b) { return sp.begin_block[b] - 1; };
      auto b1 = [&](int b) { return sp.begin_block[b + 1] - 1; };
      // Simpson contribution of each block: <rbar_m, phi rho_block>
      std::vector<double> contrib(nb);
      double S = 0.0;
      for (int b = 0; b < nb; ++b) {
        PF_CU(cudaMemsetAsync(rsp.p, 0, rsp.bytes, st));
        SimpsonBlocks sb{};
        sb.nblocks = 1;
        sb.mon[0] = mon_index(sp.mid_block[b]);
        sb.bgn[0] = b0(b);
        sb.end[0] = b1(b);
        sb.ds[0] = sp.ds_block[b];
        launch_simpson<T>(rsp.as<double>(), q, homo ? nullptr : qc, homo, Ns, ng, sb, sp.phi, sp.Nref,
                          sp.Qdev.as<double>(), scaled(p) ? sp.fac.as<double>() : nullptr, st);
        contrib[b] = dot_host(rb + (long)sb.mon[0] * ng, rsp.as<double>() + (long)sb.mon[0] * ng);
        S += contrib[b];
      }
      double meanq = sp.Q;
      if (scaled(p)) {
        d2h_now(&meanq, sp.meanq.p, sizeof(double));
      }
      const double dq = -S / (meanq * (double)ng);  // through Q = mean(q_Ns), rescaled
      for (int b = 0; b < nb; ++b)
        launch_adj_weights(wts.as<double>() + (size_t)b * nw * nk, g, npr, sp.ds_block[b], sp.b_block[b],
                           1.0 / (double)ng, nk, st);
      PF_CU(cudaMemsetAsync(G.p, 0, G.bytes, st));
      PF_CU(cudaMemsetAsync(acc.p, 0, acc.bytes, st));
      // one-step jobs: forward step t at ops[t], backward step t' = Ns - s at ops[Ns + t']
      const StepOp<T>* ops = sp.ops[p].as<StepOp<T>>();
      std::vector<ChainJob<T>> hj(2 * (size_t)Ns);
      for (int t = 0; t < 2 * Ns; ++t)
        hj[t] = ChainJob<T>{lam, ops + t, nz > 1 ? k1 : nullptr, nullptr, nullptr, 0, +1, 1, 0};
      jobsd.alloc(sizeof(ChainJob<T>) * hj.size());
      PF_CU(cudaMemcpyAsync(jobsd.p, hj.data(), jobsd.bytes, cudaMemcpyHostToDevice, st));
      const ChainJob<T>* jd = jobsd.as<ChainJob<T>>();
      // adjoint sources at contour point s: chain q (qs = qc_s) or chain qc (qs = q_s)
      auto src_at = [&](int s, bool chain_q) {
        AdjSrc<T> a;
        for (int b = 0; b < nb && a.n < 3; ++b) {
          if (s < b0(b) || s > b1(b)) continue;
          const int n = b1(b) - b0(b);
          double wsum = simpson_w(s - b0(b), n);
          if (homo) wsum += simpson_w(Ns - s - b0(b), n);  // qc_s = q_{Ns-s}
          a.coef[a.n] = sp.phi * sp.ds_block[b] / 3.0 * wsum / sp.Nref;
          a.rb[a.n] = rb + (long)mon_index(sp.mid_block[b]) * ng;
          a.qs[a.n] = chain_q ? (homo ? q + (long)(Ns - s) * ng : qc + (long)s * ng) : q + (long)s * ng;
          ++a.n;
        }
        a.fac = scaled(p) ? sp.fac.as<double>() + s : nullptr;
        a.Qdev = sp.Qdev.as<double>();
        return a;
      };
      // one adjoint step: ybar in lam, x -> y the primal step, block b, factor cfac
      auto step = [&](int job, int b, const T* x, const T* y, const float* cfac, const AdjSrc<T>& src) {
        const T* lwb = sp.lw[p][b]->as<T>();
        const T* ldb = sp.ld[p][b]->as<T>();
        launch_adj_lw_pair<T>(u1, u2, lwb, x, lam, ng, st);
        const int nparts = launch_grad_transform<T>(u1, u2, k1, k2, src_dev, dst_dev, dims,
                                                    wts.as<double>() + (size_t)b * nw * nk, nw, part.as<double>(),
                                                    tw<T>(p), st);
        launch_adj_accum(acc.as<double>() + (size_t)b * nw, part.as<double>(), nparts, nw, cfac, st);
        ChainHost<T> h;
        h.kbuf = nz > 1 ? k1 : nullptr;
        h.nsteps = 1;
        h.ld = &ldb;
        own(h);
        launch_chains<T>(jd + job, 1, 1, dims, tw<T>(p), st, &h);
        launch_adj_finish<T>(lam, rr, lam, x, y, G.as<double>() + (size_t)b * ng, cfac, src, ng, st);
        check_launch();
      };
      // segment jobs: chain 0 (forward, ops[t]) and chain 1 (backward, ops[Ns + t'])
      const int nseg = K > 0 ? (Ns + K - 1) / K : 0;
      if (K > 0) {
        std::vector<ChainJob<T>> sj;
        for (int ch = 0; ch < 2; ++ch)
          for (int c = 0; c < nseg; ++c)
            sj.push_back(ChainJob<T>{segb.as<T>(), ops + (ch ? Ns : 0) + c * K, nz > 1 ? k1 : nullptr,
                                     scaled(p) ? segcsc.as<float>() : nullptr,
                                     scaled(p) ? seglsc.as<double>() : nullptr, 0, +1, std::min(K, Ns - c * K), 0});
        segjobs.alloc(sizeof(ChainJob<T>) * sj.size());
        PF_H2D(segjobs.p, sj.data(), segjobs.bytes, st);
      }
      // propagators of segment c of chain ch: B[j] = step c*K + j of that chain, from its checkpoint
      auto recompute = [&](int ch, int c, const T* start) {
        T* B = segb.as<T>();
        PF_CU(cudaMemcpyAsync(B, start, sizeof(T) * ng, cudaMemcpyDeviceToDevice, st));
        ChainHost<T> h;
        h.kbuf = nz > 1 ? k1 : nullptr;
        h.csc = scaled(p) ? segcsc.as<float>() : nullptr;
        h.lsc = scaled(p) ? seglsc.as<double>() : nullptr;
        h.nsteps = std::min(K, Ns - c * K);
        h.ld = lds_of<T>()[jobidx + ch].data() + c * K;
        own(h);
        launch_chains<T>(segjobs.as<ChainJob<T>>() + ch * nseg + c, 1, h.nsteps, dims, tw<T>(p), st, &h);
        check_launch();
        return static_cast<const T*>(B);
      };
      // forward chain q_{t+1} = A q_t: adjoint from t = Ns down to 0
      launch_adj_init<T>(lam, src_at(Ns, true), dq, ng, st);
      int cur = -1;
      const T* B = nullptr;
      for (int t = Ns - 1; t >= 0; --t) {
        int b = 0;
        while (!(b0(b) <= t && t < b1(b))) ++b;
        const float* cf = scaled(p) ? sp.csc[0].as<float>() + t : nullptr;
        const T* x = q + (long)t * ng;
        if (K > 0) {
          const int c = t / K;
          if (c != cur) {
            B = recompute(0, c, q + (long)c * K * ng);
            cur = c;
          }
          x = B + (long)(t - c * K) * ng;
        }
        step(t, b, x, x + ng, cf, src_at(t, true));
      }
      if (!homo) {
        // backward chain qc_{s-1} = A qc_s: adjoint from s = 0 up to Ns
        launch_adj_init<T>(lam, src_at(0, false), 0.0, ng, st);
        cur = -1;
        for (int s = 1; s <= Ns; ++s) {
          int b = 0;
          while (!(b0(b) < s && s <= b1(b))) ++b;
          const int tp = Ns - s;
          const float* cf = scaled(p) ? sp.csc[1].as<float>() + tp : nullptr;
          const T* x = qc + (long)s * ng;
          const T* y = qc + (long)(s - 1) * ng;
          if (K > 0) {
            const int c = tp / K;
            if (c != cur) {
              B = recompute(1, c, qc + (long)(Ns - c * K) * ng);
              cur = c;
            }
            x = B + (long)(tp - c * K) * ng;
            y = x + ng;
          }
          step(Ns + tp, b, x, y, cf, src_at(s, false));
        }
      }
      // w gradients and the ds / Nref terms of every block
      std::vector<double> hacc((size_t)nb * nw);
      PF_CU(cudaMemcpyAsync(hacc.data(), acc.p, sizeof(double) * hacc.size(), cudaMemcpyDeviceToHost, st));
      for (int b = 0; b < nb; ++b) {
        const int mid = sp.mid_block[b];
        const double vol = monomers.at(mid).first;
        const double* Gb = G.as<double>() + (size_t)b * ng;
        launch_daxpy(grid_ptr(wbar, mid), Gb, -sp.ds_block[b] * vol / 2.0, ng, st);
        const double wg = dot_host(grid_ptr(w, mid), Gb);
        for (int j = 0; j < npr; ++j) cell_bar[j] += hacc[(size_t)b * nw + j];
        const double dds = hacc[(size_t)b * nw + npr] - vol / 2.0 * wg + contrib[b] / sp.ds_block[b];
        nref_bar.push_back(dds / (double)(b1(b) - b0(b)) - S / sp.Nref);
      }
      jobidx += homo ? 1 : 2;
    }
    sync_st();
    check_pipe(p);
  }
  void pullback(std::vector<double>& cell_bar, std::vector<double>& nref_bar, bool recompute = true) {
    if (prec == 0) pullback_t<double>(0, cell_bar, nref_bar, recompute);
    else pullback_t<float>(1, cell_bar, nref_bar, recompute);
  }

  // Gradient of free_energy (system.jl:402-433) at the current fields and cell: density! is
  // solved, dL/drho = (-w + sum chi rho / (v v)) / Ng is set as the density cotangent (it
  // replaces one set by pf_set_density_cotangent), the density pullback gives the chain
  // dependence, and the direct terms are added: -rho / Ng to dL/dw, <rho_a rho_b> / (v_a v_b)
  // to dL/dchi_ab (Flory pairs in ascending id order), <(rho/v)^2> / 2 to dL/du (Edwards
  // monomers in ascending id order), and -phi (phi - 1) / Nref^2 (the translational term with
  // mu = phi, as the reference computes it) to dL/dNref of every block.  Returns free_energy.
  double fhelm_pullback(std::vector<double>& cell_bar, std::vector<double>& nref_bar, std::vector<double>& chi_bar,
                        std::vector<double>& u_bar) {
    require_ready();
    if (ensemble != 0) throw PFError(E_UNSUPPORTED, "the pullback differentiates the canonical ensemble");
    density();
    fetch_Q();
    double ferr = 0.0, fhelm = 0.0;
    stats(ferr, fhelm);
    launch_fhelm_cotangent(rbar.as<double>(), w.as<double>(), rho.as<double>(), monomer_set(), ng, st);
    check_launch();
    pullback(cell_bar, nref_bar, false);
    launch_daxpy(wbar.as<double>(), rho.as<double>(), -1.0 / (double)ng, (long)nmon() * ng, st);
    DevBuf dp, dd;
    dp.alloc(sizeof(double) * kRedBlocks);
    dd.alloc(sizeof(double));
    auto dot = [&](const double* a, const double* b) {
      launch_ddot(a, b, ng, dp.as<double>(), dd.as<double>(), st);
      double v = 0.0;
      d2h_now(&v, dd.p, sizeof(double));
      return v;
    };
    chi_bar.clear();
    for (auto& kv : chis) {
      const int a = kv.first.first, b = kv.first.second;
      const double va = monomers.at(a).first, vb = monomers.at(b).first;
      chi_bar.push_back(dot(grid_ptr(rho, a), grid_ptr(rho, b)) / (va * vb * (double)ng));
    }
    u_bar.clear();
    for (auto& kv : edwards) {
      const double v = monomers.at(kv.first).first;
      const double* r = grid_ptr(rho, kv.first);
      u_bar.push_back(0.5 * dot(r, r) / (v * v * (double)ng));
    }
    size_t k = 0;
    for (auto& sp : species) {
      if (sp->kind != 0) continue;
      const double phi = sp->phi, t = phi > 1e-8 ? -phi * (phi - 1.0) / (sp->Nref * sp->Nref) : 0.0;
      for (int b = 0; b < sp->nblocks() && k < nref_bar.size(); ++b) nref_bar[k++] += t;
    }
    check_launch();
    sync_st();
    return fhelm;
  }

  // ---------------------------------------------------------------- scft! (simulate.jl:60-148)
  static bool isconverged(double ferr, double ftol, double serr, double stol, bool vcell) {
    bool fc = false, sc = true;
    if (ferr < ftol) {
      fc = true;
      if (vcell && serr > stol) sc = false;
    }
    return fc && sc;
  }

  // savefields(sys, path) (fileio.jl:77-97) for the omega fields: dim, grid, mids, date,
  // crystal, cell_params, field_type and the fields as nested [z][y][x] lists, one per monomer id.
  void save_fields(const std::string& path) {
    std::vector<double> h((size_t)ng * nmon());
    d2h_now(h.data(), w.p, sizeof(double) * h.size());
    FILE* f = fopen(path.c_str(), "w");
    if (!f) throw PFError(E_ARG, "cannot open " + path + " for writing");
    char date[32] = "";
    const std::time_t now = std::time(nullptr);
    std::tm tmv{};
    if (localtime_r(&now, &tmv)) std::strftime(date, sizeof date, "%Y-%m-%d %H:%M:%S", &tmv);
    fprintf(f, "{\n    \"dim\": %d,\n    \"grid\": [%d, %d, %d],\n    \"mids\": [", cell.dim, nx, ny, nz);
    for (int a = 0; a < nmon(); ++a) fprintf(f, "%s%d", a ? ", " : "", mon_ids[a]);
    fprintf(f, "],\n    \"date\": \"%s\",\n    \"crystal\": \"%s\",\n    \"cell_params\": [", date,
            cell.crystal.c_str());
    for (int i = 0; i < cell.np(); ++i) fprintf(f, "%s%.17g", i ? ", " : "", cell.params[i]);
    fprintf(f, "],\n    \"field_type\": \"omega\",\n    \"fields\": {");
    for (int a = 0; a < nmon(); ++a) {
      fprintf(f, "%s\n        \"%d\": [", a ? "," : "", mon_ids[a]);
      const double* g = h.data() + (size_t)a * ng;
      for (int z = 0; z < nz; ++z) {
        fprintf(f, "%s[", z ? ", " : "");
        for (int y = 0; y < ny; ++y) {
          fprintf(f, "%s[", y ? ", " : "");
          const double* row = g + ((size_t)z * ny + y) * nx;
          for (int x = 0; x < nx; ++x) fprintf(f, "%s%.17g", x ? ", " : "", row[x]);
          fprintf(f, "]");
        }
        fprintf(f, "]");
      }
      fprintf(f, "]");
    }
    fprintf(f, "\n    }\n}\n");
    const bool bad = ferror(f) != 0;
    if (fclose(f) != 0 || bad) throw PFError(E_ARG, "writing " + path + " failed");
  }

  pf_scft_results scft(const pf_scft_options& o, bool vcell) {
    auto t0 = std::chrono::steady_clock::now();
    pf_scft_results r{};
    r.switch_step = -1;
    nk_fp32 = nk_fp64 = 0;
    if (active == 0 && !and_.exists) throw PFError(E_STATE, "no field updater created");
    if (vcell && !dom.exists) throw PFError(E_STATE, "no DomainUpdater created");
    validate();
    residuals();
    updater_setup();
    int step = 0;
    double ferr, fhelm;
    stats(ferr, fhelm);
    double serr = 0.0;
    if (vcell) {
      domain_setup();
      serr = stress_error();
    }
    bool converged = isconverged(ferr, o.ftol, serr, o.stol, vcell);
    const bool mixed = o.mixed_switch_ferr > 0.0 && prec == 1;
    if (mixed && ferr < o.mixed_switch_ferr) {
      prec = 0;
      r.switch_step = 0;
    }
    // a float32 phase that stops improving (no new minimum of ferr for kStall iterations: its
    // rounding floor lies above mixed_switch_ferr) switches to float64 as well
    constexpr int kStall = 200;
    double best = ferr;
    int best_step = 0;
    if (!converged && o.nsout > 0) printf("--------------------------------------------------------------\n");
    while (step < o.nsteps && !converged) {
      if (o.nsout > 0 && step % o.nsout == 0)
        printf("Step (%-5d / %5d): ferr = %8e, fhelm = %.5e\n", step, o.nsteps, ferr, fhelm);
      updater_step();
      if (vcell && step % dom.nskip == 0) {
        dom.stress = scfstress();
        serr = stress_error();
        if (serr > o.stol) {
          domain_step(dom.nper, true);
          serr = stress_error();
          if (o.nsout > 0) printf("Updating cell dimensions: serr = %.5e\n", serr);
        }
      }
      stats(ferr, fhelm);
      if (std::isnan(ferr)) throw PFError(E_NAN, "Diverging field updater -- breaking.");
      converged = isconverged(ferr, o.ftol, serr, o.stol, vcell);
      if (converged) {
        if (o.nsout > 0) {
          printf("Converged @ step = %d: ferr = %8e, fhelm = %.5e\n", step, ferr, fhelm);
          if (vcell) {  // simulate.jl:115-117
            printf("Converged cell parameters: [");
            for (int i = 0; i < cell.np(); ++i) printf("%s%.17g", i ? ", " : "", cell.params[i]);
            printf("]\n");
          }
        }
        break;
      }
      if (o.nsave > 0 && step % o.nsave == 0 && !savepath.empty()) save_fields(savepath);  // simulate.jl:124-128
      if (mixed && prec == 1) {
        if (ferr < 0.99 * best) {
          best = ferr;
          best_step = step;
        }
        if (ferr < o.mixed_switch_ferr || step - best_step >= kStall) {
          prec = 0;
          r.switch_step = step;
          if (active == 0) anderson_restart();
          // polish 0 (automatic): Newton-Krylov on 3D grids, where a float64 density solve costs
          // ~20 float32 ones; on 1D/2D grids a solve is short enough that the field updater's own
          // float64 steps finish sooner than GMRES cycles with their host round trips
          const bool newton = o.polish == 2 || (o.polish == 0 && nz > 1);
          if (newton && !vcell) {
            // float64 polish by Newton-Krylov steps with float32 Jacobian products
            step += 1;
            converged = nk_polish(o, step, ferr, fhelm);
            if (std::isnan(ferr)) throw PFError(E_NAN, "Diverging field updater -- breaking.");
            if (converged) {
              if (o.nsout > 0) printf("Converged @ step = %d: ferr = %8e, fhelm = %.5e\n", step, ferr, fhelm);
              break;
            }
            // a Newton step stalled: float64 iterations of the field updater from here
            if (active == 0) anderson_restart();
            continue;
          }
        }
      }
      step += 1;
    }
    residuals();
    stats(ferr, fhelm);
    if (vcell) serr = stress_error();
    r.time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r.polish_fp64_solves = nk_fp64;
    r.polish_fp32_solves = nk_fp32;
    r.nsteps = step;
    r.converged = converged ? 1 : 0;
    r.ferr = ferr;
    r.serr = serr;
    r.fhelm = fhelm;
    return r;
  }

  // ---------------------------------------------------------------- low-level propagate
  template <typename T>
  void propagate_t(int p, const double* omega, double vol, double b, double ds, const double* qin, double* qout,
                   int nsteps) {
    if (!has_cell) throw PFError(E_STATE, "no unit cell set");
    if (nsteps < 1) throw PFError(E_ARG, "nsteps must be positive");
    DevBuf dw, lw, ld, hist, ops, job, kb;
    dw.alloc(sizeof(double) * ng);
    lw.alloc(sizeof(T) * ng);
    ld.alloc(sizeof(T) * nk);
    hist.alloc(sizeof(T) * ng * (nsteps + 1));
    PF_CU(cudaMemcpyAsync(dw.p, omega, sizeof(double) * ng, cudaMemcpyHostToDevice, st));
    launch_lw<T>(lw.as<T>(), dw.as<double>(), ds / 2.0 * vol, ng, st);
    launch_ld<T>(ld.as<T>(), geom(), ds * b * b / 6.0, 1.0 / (double)ng, nk, st);
    std::vector<T> h0(ng);
    for (long i = 0; i < ng; ++i) h0[i] = (T)qin[i];
    PF_CU(cudaMemcpyAsync(hist.p, h0.data(), sizeof(T) * ng, cudaMemcpyHostToDevice, st));
    std::vector<StepOp<T>> hops(nsteps, StepOp<T>{lw.as<T>(), ld.as<T>()});
    ops.alloc(sizeof(StepOp<T>) * nsteps);
    PF_CU(cudaMemcpyAsync(ops.p, hops.data(), ops.bytes, cudaMemcpyHostToDevice, st));
    Cx<T>* kp = nullptr;
    if (nz > 1) {
      kb.alloc(sizeof(Cx<T>) * nk);
      kp = kb.as<Cx<T>>();
    }
    ChainJob<T> hj{hist.as<T>(), ops.as<StepOp<T>>(), kp, nullptr, nullptr, 0, +1, nsteps, 0};
    job.alloc(sizeof(hj));
    PF_CU(cudaMemcpyAsync(job.p, &hj, sizeof(hj), cudaMemcpyHostToDevice, st));
    std::vector<const T*> ld_steps(nsteps, ld.as<T>());
    ChainHost<T> host;
    host.kbuf = kp;
    host.nsteps = nsteps;
    own(host);
    host.ld = ld_steps.data();
    launch_chains<T>(job.as<ChainJob<T>>(), 1, nsteps, GridDims{nx, ny, nz}, tw<T>(p), st, &host);
    check_launch();
    std::vector<T> ho(ng);
    d2h_now(ho.data(), hist.as<T>() + (long)nsteps * ng, sizeof(T) * ng);
    check_pipe(p);
    for (long i = 0; i < ng; ++i) qout[i] = (double)ho[i];
  }
};

// Grids with kernels: planes (Nx, Ny) of 1D rows Nx in {8, 16, 32, 48, 64, 96, 128, 256},
// squares Nx = Ny in {16, ..., 128} and 2:1 rectangles; Nz = 1 or a supported length.
static bool dims_supported(int nx, int ny, int nz, std::string& why) {
  if (!shape_supported<double>(nx, ny, nz) || !shape_supported<float>(nx, ny, nz)) {
    why = "grid " + std::to_string(nx) + "x" + std::to_string(ny) + "x" + std::to_string(nz) + " has no kernels";
    return false;
  }
  return true;
}

}  // namespace pf

// ====================================================================== C ABI
struct pf_system {
  std::unique_ptr<pf::System> s;
  std::string err;
};

namespace {
template <typename F>
int guard(pf_system* h, F&& f) {
  if (!h || !h->s) return PF_EARG;
  try {
    f(*h->s);
    h->err.clear();
    return PF_OK;
  } catch (const pf::PFError& e) {
    h->err = e.what();
    return e.code;
  } catch (const pf::DeviceError& e) {
    h->err = e.what();
    return PF_ECUDA;
  } catch (const std::exception& e) {
    h->err = e.what();
    return PF_EARG;
  }
}
}  // namespace

extern "C" {

int pf_version(void) { return 100; }

const char* pf_status_string(int status) {
  switch (status) {
    case PF_OK: return "ok";
    case PF_EARG: return "invalid argument";
    case PF_ECUDA: return "CUDA error";
    case PF_ENAN: return "Diverging field updater -- breaking.";
    case PF_ESINGULAR: return "Error inverting Umn matrix";
    case PF_ETIMEOUT: return "device wait timed out";
    case PF_ESTATE: return "call out of order";
    case PF_ENOMEM: return "device allocation failed";
    case PF_EUNSUPPORTED: return "unsupported grid size";
    default: return "unknown status";
  }
}

int pf_system_create(pf_system** out, int nx, int ny, int nz, int precision) {
  if (!out) return PF_EARG;
  *out = nullptr;
  if (!(nx >= ny && ny >= nz && nz >= 1)) return PF_EARG;  // descending dims (system.jl:58)
  if (precision != PF_FP64 && precision != PF_FP32) return PF_EARG;
  std::string why;
  if (!pf::dims_supported(nx, ny, nz, why)) return PF_EUNSUPPORTED;
  auto* h = new pf_system();
  try {
    h->s.reset(new pf::System(nx, ny, nz, precision));
  } catch (const pf::PFError& e) {
    delete h;
    return e.code;
  } catch (const std::exception&) {  // no exception crosses the C ABI
    delete h;
    return PF_ECUDA;
  }
  *out = h;
  return PF_OK;
}

int pf_system_destroy(pf_system* sys) {
  delete sys;
  return PF_OK;
}

const char* pf_last_error(const pf_system* sys) { return sys ? sys->err.c_str() : "null handle"; }

int pf_set_precision(pf_system* sys, int precision) {
  return guard(sys, [&](pf::System& s) {
    if (precision != PF_FP64 && precision != PF_FP32) throw pf::PFError(PF_EARG, "precision must be PF_FP64 or PF_FP32");
    s.prec = precision;
  });
}

int pf_set_adjoint_checkpoints(pf_system* sys, int every) {
  return guard(sys, [&](pf::System& s) {
    if (every < 0) throw pf::PFError(PF_EARG, "checkpoint interval must be >= 0");
    s.adj_ckpt = every;
  });
}

int pf_set_ensemble(pf_system* sys, int ensemble) {
  return guard(sys, [&](pf::System& s) {
    if (ensemble != 0 && ensemble != 1) throw pf::PFError(PF_EARG, "ensemble must be 0 (Canonical) or 1 (Grand)");
    if (!s.species.empty()) throw pf::PFError(PF_ESTATE, "set the ensemble before adding species");
    s.ensemble = ensemble;
  });
}

int pf_set_edwards(pf_system* sys, int mid, double u) {
  return guard(sys, [&](pf::System& s) { s.set_edwards(mid, u); });
}

int pf_set_savepath(pf_system* sys, const char* path) {
  return guard(sys, [&](pf::System& s) { s.savepath = path ? std::string(path) : std::string(); });
}

int pf_set_mde(pf_system* sys, int method) {
  return guard(sys, [&](pf::System& s) {
    if (method != 0 && method != 1)
      throw pf::PFError(PF_EARG, "Invalid propagator method for PseudoSpectralSolver: 0 = :RK2, 1 = :RQM4");
    s.mde = method;
    s.invalidate_graphs();
  });
}

int pf_get_precision(const pf_system* sys, int* precision) {
  if (!sys || !precision) return PF_EARG;
  *precision = sys->s->prec;
  return PF_OK;
}

int pf_set_cell(pf_system* sys, int dim, const char* crystal, const double* params, int nparams) {
  return guard(sys, [&](pf::System& s) {
    if (!crystal || (nparams > 0 && !params) || nparams < 0 || nparams > pf::kMaxParams)
      throw pf::PFError(PF_EARG, "bad cell arguments");
    std::string c(crystal);
    if (!c.empty() && c[0] == ':') c = c.substr(1);
    s.set_cell(dim, c, std::vector<double>(params, params + nparams));
  });
}

int pf_set_signed_k(pf_system* sys, int on) {
  return guard(sys, [&](pf::System& s) {
    if ((on != 0) != s.signed_k) {
      s.signed_k = on != 0;
      ++s.cell_version;  // LD and dksq are rebuilt before their next use
    }
  });
}

int pf_get_cell(const pf_system* sys, double* params, int nparams, double* volume) {
  if (!sys || !sys->s->has_cell) return PF_ESTATE;
  const auto& c = sys->s->cell;
  if (params)
    for (int i = 0; i < std::min(nparams, c.np()); ++i) params[i] = c.params[i];
  if (volume) *volume = c.volume;
  return PF_OK;
}

int pf_get_basis(const pf_system* sys, double* R, double* G) {
  if (!sys || !sys->s->has_cell) return PF_ESTATE;
  for (int i = 0; i < 9; ++i) {
    if (R) R[i] = sys->s->cell.R[i];
    if (G) G[i] = sys->s->cell.G[i];
  }
  return PF_OK;
}

int pf_add_monomer(pf_system* sys, int id, double vol, double charge) {
  return guard(sys, [&](pf::System& s) { s.add_monomer(id, vol, charge); });
}

int pf_add_multiblock(pf_system* sys, int nblocks, const int* block_mids, const int* N_block, const double* b_block,
                      int Ns, double phi) {
  return guard(sys, [&](pf::System& s) {
    if (!block_mids || !N_block || !b_block) throw pf::PFError(PF_EARG, "null block arrays");
    s.add_multiblock(nblocks, block_mids, N_block, b_block, Ns, phi);
  });
}

int pf_add_point(pf_system* sys, int mid, double phi) {
  return guard(sys, [&](pf::System& s) { s.add_point(mid, phi); });
}

int pf_set_flory(pf_system* sys, int a, int b, double chi) {
  return guard(sys, [&](pf::System& s) { s.set_flory(a, b, chi); });
}

int pf_species_info(const pf_system* sys, int isp, int* Ns, double* Nref, int* begin_block, double* ds_block,
                    int max_blocks) {
  if (!sys || isp < 0 || isp >= (int)sys->s->species.size()) return PF_EARG;
  const auto& sp = *sys->s->species[isp];
  if (Ns) *Ns = sp.Ns;
  if (Nref) *Nref = sp.Nref;
  for (int i = 0; i < std::min(max_blocks + 1, (int)sp.begin_block.size()); ++i)
    if (begin_block) begin_block[i] = sp.begin_block[i];
  for (int i = 0; i < std::min(max_blocks, (int)sp.ds_block.size()); ++i)
    if (ds_block) ds_block[i] = sp.ds_block[i];
  return PF_OK;
}

int pf_set_field(pf_system* sys, int mid, const double* w) {
  return guard(sys, [&](pf::System& s) {
    if (!w) throw pf::PFError(PF_EARG, "null field");
    PF_CU(cudaMemcpyAsync(s.grid_ptr(s.w, mid), w, sizeof(double) * s.ng, cudaMemcpyHostToDevice, s.st));
    PF_CU(cudaStreamSynchronize(s.st));
  });
}

int pf_get_grid(pf_system* sys, int kind, int mid, double* out) {
  return guard(sys, [&](pf::System& s) {
    if (!out) throw pf::PFError(PF_EARG, "null output");
    if (kind < PF_FIELD || kind > PF_FIELD_COTANGENT) throw pf::PFError(PF_EARG, "unknown grid kind");
    pf::DevBuf* b = kind == PF_FIELD      ? &s.w
                    : kind == PF_DENSITY  ? &s.rho
                    : kind == PF_RESIDUAL ? &s.res
                    : kind == PF_POTENTIAL ? &s.pot
                                           : &s.wbar;
    PF_CU(cudaMemcpyAsync(out, s.grid_ptr(*b, mid), sizeof(double) * s.ng, cudaMemcpyDeviceToHost, s.st));
    PF_CU(cudaStreamSynchronize(s.st));
  });
}

int pf_get_propagator(pf_system* sys, int isp, int conjugate, int s_idx, double* out) {
  return guard(sys, [&](pf::System& s) {
    if (isp < 0 || isp >= (int)s.species.size() || s.species[isp]->kind != 0) throw pf::PFError(PF_EARG, "bad species");
    auto& sp = *s.species[isp];
    if (s_idx < 0 || s_idx > sp.Ns || s.last_prec < 0) throw pf::PFError(PF_EARG, "bad contour index / no density");
    const int p = s.last_prec;
    long off = (long)s_idx * s.ng;
    pf::DevBuf* src = &sp.q[p];
    if (conjugate) {
      if (sp.nblocks() > 1) src = &sp.qc[p];
      else off = (long)(sp.Ns - s_idx) * s.ng;
    }
    if (p == 0) {
      PF_CU(cudaMemcpyAsync(out, src->as<double>() + off, sizeof(double) * s.ng, cudaMemcpyDeviceToHost, s.st));
      PF_CU(cudaStreamSynchronize(s.st));
    } else {
      std::vector<float> t(s.ng);
      PF_CU(cudaMemcpyAsync(t.data(), src->as<float>() + off, sizeof(float) * s.ng, cudaMemcpyDeviceToHost, s.st));
      // undo the per-step rescaling: stored = true * exp(L), L the sum of the applied logs
      const int job = (conjugate && sp.nblocks() > 1) ? 1 : 0;
      const int idx = (int)(off / s.ng);
      const int nlog = job == 0 ? idx : sp.Ns - idx;
      std::vector<double> l(sp.Ns);
      PF_CU(cudaMemcpyAsync(l.data(), sp.lsc[job].p, sizeof(double) * sp.Ns, cudaMemcpyDeviceToHost, s.st));
      PF_CU(cudaStreamSynchronize(s.st));
      double L = 0.0;
      for (int k = 0; k < nlog; ++k) L += l[k];
      const double f = std::exp(-L);
      for (long i = 0; i < s.ng; ++i) out[i] = (double)t[i] * f;
    }
  });
}

int pf_validate(pf_system* sys) { return guard(sys, [&](pf::System& s) { s.validate(); }); }
int pf_density(pf_system* sys) {
  return guard(sys, [&](pf::System& s) {
    s.density();
    PF_CU(cudaStreamSynchronize(s.st));
  });
}
int pf_residuals(pf_system* sys) {
  return guard(sys, [&](pf::System& s) {
    s.residuals();
    PF_CU(cudaStreamSynchronize(s.st));
  });
}
int pf_free_energy(pf_system* sys, double* out) {
  return guard(sys, [&](pf::System& s) {
    double fe, fh;
    s.stats(fe, fh);
    if (out) *out = fh;
  });
}
int pf_free_energy_bulk(pf_system* sys, double* out) {
  return guard(sys, [&](pf::System& s) {
    if (out) *out = s.free_energy_bulk();
  });
}
int pf_field_error(pf_system* sys, double* out) {
  return guard(sys, [&](pf::System& s) {
    double fe, fh;
    s.stats(fe, fh);
    if (out) *out = fe;
  });
}
int pf_scfstress(pf_system* sys, double* out, int nparams) {
  return guard(sys, [&](pf::System& s) {
    std::vector<double> st = s.scfstress();
    for (int i = 0; i < std::min(nparams, (int)st.size()); ++i) out[i] = st[i];
  });
}
int pf_species_q(pf_system* sys, int isp, double* Q) {
  return guard(sys, [&](pf::System& s) {
    if (isp < 0 || isp >= (int)s.species.size()) throw pf::PFError(PF_EARG, "bad species index");
    s.fetch_Q();
    if (Q) *Q = s.species[isp]->Q;
  });
}

int pf_anderson_create(pf_system* sys, int nhist, int iter_euler, double lam_euler) {
  return guard(sys, [&](pf::System& s) {
    if (nhist < 1 || nhist > 60) throw pf::PFError(PF_EARG, "nhist must be in [1, 60]");
    s.and_.reset();
    s.and_.exists = true;
    s.active = 0;
    s.and_.nhist = nhist;
    s.and_.iter_euler = iter_euler <= 1 ? 1 : iter_euler;
    s.and_.lam_euler = lam_euler;
  });
}
int pf_anderson_setup(pf_system* sys) { return guard(sys, [&](pf::System& s) { s.anderson_setup(); }); }

int pf_euler_create(pf_system* sys, int method, double lam) {
  return guard(sys, [&](pf::System& s) {
    if (method != 0 && method != 1)
      throw pf::PFError(PF_EARG, "Invalid `method` parameter for EulerUpdater. Options include: (:PEC, :PECE)");
    s.simple.push_back(std::make_unique<pf::System::SimpleUpdater>());
    s.su = s.simple.back().get();
    s.su->reset(1, method, lam);
    s.active = 1;
  });
}
int pf_momentum_create(pf_system* sys, int method, double lam, double gamma, double beta1, double beta2) {
  return guard(sys, [&](pf::System& s) {
    if (method < 0 || method > 3)
      throw pf::PFError(PF_EARG,
                        "Invalid `method` parameter for MomentumUpdater. Options include: (:MOM, :RMS, :ADAM, :NAG)");
    if (!(gamma > 0.0 && gamma < 1.0) || !(beta1 > 0.0 && beta1 < 1.0) || !(beta2 > 0.0 && beta2 < 1.0))
      throw pf::PFError(PF_EARG, "AssertionError: 0 < gamma, beta1, beta2 < 1");
    s.simple.push_back(std::make_unique<pf::System::SimpleUpdater>());
    s.su = s.simple.back().get();
    s.su->reset(2, method, lam);
    s.su->gamma = gamma;
    s.su->beta1 = beta1;
    s.su->beta2 = beta2;
    s.active = 2;
  });
}
int pf_updater_current(pf_system* sys, int* id) {
  return guard(sys, [&](pf::System& s) {
    if (!id) throw pf::PFError(PF_EARG, "null output pointer");
    *id = -1;
    if (s.active != 0)
      for (size_t i = 0; i < s.simple.size(); ++i)
        if (s.simple[i].get() == s.su) *id = (int)i;
  });
}
int pf_updater_select(pf_system* sys, int id) {
  return guard(sys, [&](pf::System& s) {
    if (id == -1) {
      if (!s.and_.exists) throw pf::PFError(PF_ESTATE, "no AndersonUpdater created");
      s.active = 0;
      return;
    }
    if (id < 0 || id >= (int)s.simple.size()) throw pf::PFError(PF_EARG, "no field updater with this id");
    s.su = s.simple[id].get();
    s.active = s.su->kind;
  });
}
int pf_updater_setup(pf_system* sys) { return guard(sys, [&](pf::System& s) { s.updater_setup(); }); }
int pf_updater_step(pf_system* sys) {
  return guard(sys, [&](pf::System& s) {
    s.updater_step();
    PF_CU(cudaStreamSynchronize(s.st));
  });
}
int pf_anderson_step(pf_system* sys) {
  return guard(sys, [&](pf::System& s) {
    s.anderson_step();
    PF_CU(cudaStreamSynchronize(s.st));
  });
}
int pf_domain_create(pf_system* sys, int nper, int nskip, double lam, double pmax, double rlxn) {
  return guard(sys, [&](pf::System& s) {
    s.dom = pf::System::Domain();
    s.dom.exists = true;
    s.dom.nper = nper;
    s.dom.nskip = nskip;
    s.dom.lam = lam;
    s.dom.pmax = pmax;
    s.dom.rlxn = rlxn;
  });
}
int pf_domain_setup(pf_system* sys) { return guard(sys, [&](pf::System& s) { s.domain_setup(); }); }
int pf_domain_step(pf_system* sys, int nsteps) {
  return guard(sys, [&](pf::System& s) { s.domain_step(nsteps, false); });
}
int pf_domain_stress_error(pf_system* sys, double* out) {
  return guard(sys, [&](pf::System& s) {
    if (out) *out = s.stress_error();
  });
}

int pf_scft(pf_system* sys, const pf_scft_options* opts, int use_domain, pf_scft_results* out) {
  return guard(sys, [&](pf::System& s) {
    if (!opts || !out) throw pf::PFError(PF_EARG, "null options/results");
    *out = s.scft(*opts, use_domain != 0);
  });
}

int pf_set_density_cotangent(pf_system* sys, int mid, const double* rho_bar) {
  return guard(sys, [&](pf::System& s) {
    double* dst = s.grid_ptr(s.rbar, mid);
    if (rho_bar) PF_CU(cudaMemcpyAsync(dst, rho_bar, sizeof(double) * s.ng, cudaMemcpyHostToDevice, s.st));
    else PF_CU(cudaMemsetAsync(dst, 0, sizeof(double) * s.ng, s.st));
    PF_CU(cudaStreamSynchronize(s.st));
  });
}

int pf_density_pullback(pf_system* sys, double* cell_bar, int ncell, double* nref_bar, int nnref) {
  return guard(sys, [&](pf::System& s) {
    std::vector<double> cb, nb;
    s.pullback(cb, nb);
    if (cell_bar)
      for (int i = 0; i < std::min(ncell, (int)cb.size()); ++i) cell_bar[i] = cb[i];
    if (nref_bar)
      for (int i = 0; i < std::min(nnref, (int)nb.size()); ++i) nref_bar[i] = nb[i];
  });
}

int pf_free_energy_pullback(pf_system* sys, double* cell_bar, int ncell, double* nref_bar, int nnref, double* chi_bar,
                            int nchi, double* u_bar, int nu, double* fhelm) {
  return guard(sys, [&](pf::System& s) {
    std::vector<double> cb, nb, xb, ub;
    const double f = s.fhelm_pullback(cb, nb, xb, ub);
    if (fhelm) *fhelm = f;
    if (cell_bar)
      for (int i = 0; i < std::min(ncell, (int)cb.size()); ++i) cell_bar[i] = cb[i];
    if (nref_bar)
      for (int i = 0; i < std::min(nnref, (int)nb.size()); ++i) nref_bar[i] = nb[i];
    if (chi_bar)
      for (int i = 0; i < std::min(nchi, (int)xb.size()); ++i) chi_bar[i] = xb[i];
    if (u_bar)
      for (int i = 0; i < std::min(nu, (int)ub.size()); ++i) u_bar[i] = ub[i];
  });
}

int pf_scft_batch(pf_system* const* systems, int n, const pf_scft_options* opts, int use_domain,
                  pf_scft_results* results, int* status, int nthreads) {
  if (!systems || n < 0 || !opts || !results || !status) return PF_EARG;
  for (int i = 0; i < n; ++i)
    if (!systems[i] || !systems[i]->s) return PF_EARG;
  // longest runs first (grid points x contour steps per density solve), so the tail is short
  std::vector<int> order(n);
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    order[i] = i;
    cost[i] = systems[i]->s->solve_cost();
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  const int nt = std::max(1, std::min(n, nthreads > 0 ? nthreads : 32));
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int> next{0};
  // Batched systems replay their captured density-solve graphs like single runs.  (Under the
  // process-wide staging of pageable reads this was 15% slower than direct launches; with
  // pinned reads and 32 hardware queues the two take the same time.)
  auto worker = [&]() {
    cudaSetDevice(dev);
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= n) break;
      const int i = order[k];
      status[i] = pf_scft(systems[i], opts, use_domain, &results[i]);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  for (int i = 0; i < n; ++i)
    if (status[i] != PF_OK) return status[i];
  return PF_OK;
}

int pf_propagate(pf_system* sys, const double* omega, double vol, double b, double ds, const double* qin, double* qout,
                 int nsteps) {
  return guard(sys, [&](pf::System& s) {
    if (!omega || !qin || !qout) throw pf::PFError(PF_EARG, "null array");
    if (s.prec == 0) s.propagate_t<double>(0, omega, vol, b, ds, qin, qout, nsteps);
    else s.propagate_t<float>(1, omega, vol, b, ds, qin, qout, nsteps);
  });
}

int pf_set_wait_limit(pf_system* sys, double seconds) {
  return guard(sys, [&](pf::System& s) {
    if (!(seconds >= 0.0) || seconds > 10.0) throw pf::PFError(pf::E_ARG, "wait limit must be in [0, 10] seconds");
    s.wait_ns = (unsigned long long)(seconds * 1e9);
    for (auto& h : s.hosts_f) h.wait_ns = s.wait_ns;
    for (auto& h : s.hosts_d) h.wait_ns = s.wait_ns;
    s.invalidate_graphs();  // captured launches hold the old limit
  });
}

int pf_get_pencil_schedule(pf_system* sys, int* stages, int* rounds, int* tuned) {
  return guard(sys, [&](pf::System& s) {
    const int nkp = (s.nx / 2 + 1) * s.ny;
    const bool t = s.prec == 0 ? pf::get_pencil_schedule<double>(s.nz, nkp, stages, rounds)
                               : pf::get_pencil_schedule<float>(s.nz, nkp, stages, rounds);
    if (tuned) *tuned = t ? 1 : 0;
  });
}

int pf_set_timing(pf_system* sys, int enable) {
  return guard(sys, [&](pf::System& s) { s.timing = enable != 0; });
}
int pf_last_timing(const pf_system* sys, double* propagate_ms, double* density_ms, int* mde_steps) {
  if (!sys) return PF_EARG;
  if (propagate_ms) *propagate_ms = sys->s->t_prop_ms;
  if (density_ms) *density_ms = sys->s->t_dens_ms;
  if (mde_steps) *mde_steps = sys->s->mde_steps;
  return PF_OK;
}
int pf_record_event(pf_system* sys, int slot) {
  return guard(sys, [&](pf::System& s) {
    if (slot < 0 || slot >= 8) throw pf::PFError(PF_EARG, "event slot must be in [0, 8)");
    PF_CU(cudaEventRecord(s.uev[slot], s.st));
  });
}

int pf_elapsed_ms(pf_system* sys, int a, int b, double* ms) {
  return guard(sys, [&](pf::System& s) {
    if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) throw pf::PFError(PF_EARG, "bad event slots");
    PF_CU(cudaEventSynchronize(s.uev[b]));
    float v = 0.f;
    PF_CU(cudaEventElapsedTime(&v, s.uev[a], s.uev[b]));
    *ms = v;
  });
}

long pf_launch_count(void) { return pf::launch_total(); }

int pf_synchronize(pf_system* sys) {
  return guard(sys, [&](pf::System& s) { PF_CU(cudaStreamSynchronize(s.st)); });
}

}  // extern "C"
