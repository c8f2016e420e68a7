// Allocation-free propagation entry point: pf_propagate_noalloc.
//
// Some callers cannot allocate device memory at the moment they need a propagation: code
// that runs inside another framework's memory pool (whose buffers it receives but may not
// grow), code on a real-time path where allocation is forbidden, or a host language binding
// that owns all device buffers itself.  This entry point takes the caller's device buffers
// for inputs and outputs and keeps everything else it needs -- the chain descriptor, the
// per-step operator table, the twiddle tables and the 3D half-spectrum buffer -- in one
// file-scope __device__ array of fixed size, so it never calls cudaMalloc or cudaFree.
//
// The array (16 MiB) exists on every GPU that loads this library until the process exits.
// Every call uses the same array: two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on it and must be serialised by the caller.
// Nothing in the array needs clearing between calls: each call writes every byte it later
// reads (descriptors and twiddles by copy, the half spectrum by the first plane pass).  The
// one exception is the status word: a 3D pencil pass whose bounded wait for a TMA copy gave
// up sets it (the call's output is then invalid); it starts at zero when the library loads,
// stays set across calls, and pf_propagate_noalloc_status reads and clears it.
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "pf_kernels.h"
#include "polyfields_gpu.h"

namespace pf {
namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;  // 16 MiB
constexpr size_t kJobOffset = 0;                     // one ChainJob
constexpr size_t kStatusOffset = 1024;               // the pencil passes' status word (int)
constexpr size_t kOpsOffset = 4096;                  // StepOp table
constexpr size_t kTwOffset = 64 * 1024;              // twiddle tables for x, y, z
constexpr size_t kKbufOffset = 96 * 1024;            // half-spectrum buffer (3D)
constexpr int kMaxNoallocSteps = (int)((kTwOffset - kOpsOffset) / sizeof(StepOp<double>));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of g_noalloc_scratch on the current device, looked up once per device with
// that device current (a host-side reference to the symbol is not a device address).
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return E_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return E_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "pf_propagate_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return E_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return OK;
}

template <typename T>
int propagate_noalloc(int nx, int ny, int nz, T* hist, const T* lw, const T* ld, int nsteps, cudaStream_t st) {
  const long nk = (long)(nx / 2 + 1) * ny * nz;
  const size_t kbytes = nz > 1 ? sizeof(Cx<T>) * (size_t)nk : 0;
  if (kbytes > kScratchBytes - kKbufOffset) {
    fprintf(stderr,
            "pf_propagate_noalloc: grid %dx%dx%d needs %zu bytes of half-spectrum scratch, more than the %zu "
            "bytes available; use pf_propagate\n",
            nx, ny, nz, kbytes, kScratchBytes - kKbufOffset);
    return E_TOOLARGE;
  }
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc != OK) return rc;
  unsigned char* b = static_cast<unsigned char*>(base);
  ChainJob<T>* job_dev = reinterpret_cast<ChainJob<T>*>(b + kJobOffset);
  StepOp<T>* ops_dev = reinterpret_cast<StepOp<T>*>(b + kOpsOffset);
  Cx<T>* tw_dev = reinterpret_cast<Cx<T>*>(b + kTwOffset);
  Cx<T>* kbuf = nz > 1 ? reinterpret_cast<Cx<T>*>(b + kKbufOffset) : nullptr;

  // descriptors and twiddles from host memory (copied into the scratch array, no allocation)
  std::vector<StepOp<T>> hops(nsteps, StepOp<T>{lw, ld});
  const ChainJob<T> hjob{hist, ops_dev, kbuf, nullptr, nullptr, 0, +1, nsteps, 0};
  std::vector<Cx<T>> htw;
  int off[3];
  for (int a = 0; a < 3; ++a) {
    const int n = a == 0 ? nx : a == 1 ? ny : nz;
    double re[1024], im[1024];
    const int cnt = fft_twiddle_table(n, re, im, 1024);
    if (cnt < 0) return E_UNSUPPORTED;
    off[a] = (int)htw.size();
    for (int i = 0; i < cnt; ++i) htw.push_back(cx<T>((T)re[i], (T)im[i]));
  }
  if (sizeof(Cx<T>) * htw.size() > kKbufOffset - kTwOffset) return E_UNSUPPORTED;
  if (cudaMemcpyAsync(ops_dev, hops.data(), sizeof(StepOp<T>) * nsteps, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(job_dev, &hjob, sizeof(hjob), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(tw_dev, htw.data(), sizeof(Cx<T>) * htw.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return E_CUDA;
  const Twiddles<T> tw{tw_dev + off[0], tw_dev + off[1], tw_dev + off[2]};
  // host view for the TMA descriptors of the pencil pass (host memory only)
  std::vector<const T*> ld_steps(nsteps, ld);
  ChainHost<T> host;
  host.kbuf = kbuf;
  host.nsteps = nsteps;
  host.ld = ld_steps.data();
  host.status = reinterpret_cast<int*>(b + kStatusOffset);
  try {
    launch_chains<T>(job_dev, 1, nsteps, GridDims{nx, ny, nz}, tw, st, &host);
  } catch (const DeviceError& e) {
    fprintf(stderr, "pf_propagate_noalloc: %s\n", e.what());
    return E_CUDA;
  } catch (const std::exception& e) {
    fprintf(stderr, "pf_propagate_noalloc: %s\n", e.what());
    return E_ARG;
  }
  return cudaGetLastError() == cudaSuccess ? OK : E_CUDA;
}

// Reads the status word on stream st, waits for st, clears the word.
int take_status(cudaStream_t st, int* out) {
  void* base = nullptr;
  const int rc = scratch_address(&base);
  if (rc != OK) return rc;
  int* word = reinterpret_cast<int*>(static_cast<unsigned char*>(base) + kStatusOffset);
  int v = 0;
  if (cudaMemcpyAsync(&v, word, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemsetAsync(word, 0, sizeof(int), st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
    return E_CUDA;
  *out = v;
  return OK;
}

}  // namespace
}  // namespace pf

extern "C" int pf_propagate_noalloc(int nx, int ny, int nz, int precision, void* hist, const void* lw, const void* ld,
                                    int nsteps, void* stream) {
  if (!hist || !lw || !ld) return PF_EARG;
  if (!(nx >= ny && ny >= nz && nz >= 1)) return PF_EARG;
  if (nsteps < 1 || nsteps > pf::kMaxNoallocSteps) {
    fprintf(stderr, "pf_propagate_noalloc: nsteps must be in [1, %d]\n", pf::kMaxNoallocSteps);
    return PF_EARG;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == PF_FP64) {
    if (!pf::shape_supported<double>(nx, ny, nz)) return PF_EUNSUPPORTED;
    return pf::propagate_noalloc<double>(nx, ny, nz, static_cast<double*>(hist), static_cast<const double*>(lw),
                                         static_cast<const double*>(ld), nsteps, st);
  }
  if (precision == PF_FP32) {
    if (!pf::shape_supported<float>(nx, ny, nz)) return PF_EUNSUPPORTED;
    return pf::propagate_noalloc<float>(nx, ny, nz, static_cast<float*>(hist), static_cast<const float*>(lw),
                                        static_cast<const float*>(ld), nsteps, st);
  }
  return PF_EARG;
}

extern "C" int pf_propagate_noalloc_status(void* stream) {
  int v = 0;
  const int rc = pf::take_status(static_cast<cudaStream_t>(stream), &v);
  if (rc != pf::OK) return rc;
  return v ? PF_ETIMEOUT : PF_OK;
}
