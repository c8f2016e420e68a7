// In-shared-memory FFTs for the pseudo-spectral MDE step.
//
// A transform of length N is run by a group of G threads (G divides 32, so groups never
// straddle a warp).  Each pass of radix R is one Stockham autosort step: every thread
// loads all of its butterflies into registers, the group synchronises (__syncwarp), and
// the results are written back in place.  Lengths are 8, 16, 32, 48, 64, 96, 128, 256, covering the
// grids of the reference's examples and benchmark cases (32 ... 128 per axis).
//
// Forward transforms use exp(-2 pi i k n / N) and are unnormalised, as FFTW's r2c in the
// reference (src/system/fft.jl:31); inverse transforms use exp(+2 pi i k n / N) and are also
// unnormalised here: the 1/Ng factor of the reference's normalised irfft (fft.jl:32) is folded
// into the bond operator LD by the caller.
#pragma once
#include "pf_common.cuh"

namespace pf {

// ---------------------------------------------------------------- small DFTs in registers
template <typename T, bool INV>
__device__ __forceinline__ void dft2(Cx<T>& a0, Cx<T>& a1) {
  Cx<T> t = a0 - a1;
  a0 = a0 + a1;
  a1 = t;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft3(Cx<T>& a0, Cx<T>& a1, Cx<T>& a2) {
  const T s3 = (T)0.866025403784438646763723170752936183;  // sqrt(3)/2
  Cx<T> t1 = a1 + a2;
  Cx<T> t2 = cx<T>(a0.x - (T)0.5 * t1.x, a0.y - (T)0.5 * t1.y);
  Cx<T> d = a1 - a2;
  // forward: y1 = t2 - i s3 d, y2 = t2 + i s3 d ; inverse swaps the sign of i
  Cx<T> t3 = mul_mi<T, INV>(cscale(d, s3));
  a0 = a0 + t1;
  a1 = t2 + t3;
  a2 = t2 - t3;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4(Cx<T>& a0, Cx<T>& a1, Cx<T>& a2, Cx<T>& a3) {
  Cx<T> s02 = a0 + a2, d02 = a0 - a2;
  Cx<T> s13 = a1 + a3, d13 = mul_mi<T, INV>(a1 - a3);
  a0 = s02 + s13;
  a2 = s02 - s13;
  a1 = d02 + d13;
  a3 = d02 - d13;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(Cx<T>* a) {
  const T r = (T)0.707106781186547524400844362104849039;  // 1/sqrt(2)
  Cx<T> e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  Cx<T> o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<T, INV>(e0, e1, e2, e3);
  dft4<T, INV>(o0, o1, o2, o3);
  // twiddles w8^k, w8 = exp(-+ i pi/4)
  Cx<T> w1o = INV ? cx<T>(r * (o1.x - o1.y), r * (o1.x + o1.y)) : cx<T>(r * (o1.x + o1.y), r * (o1.y - o1.x));
  Cx<T> w2o = mul_mi<T, INV>(o2);
  Cx<T> w3o = INV ? cx<T>(-r * (o3.x + o3.y), r * (o3.x - o3.y)) : cx<T>(r * (o3.y - o3.x), -r * (o3.x + o3.y));
  a[0] = e0 + o0;
  a[4] = e0 - o0;
  a[1] = e1 + w1o;
  a[5] = e1 - w1o;
  a[2] = e2 + w2o;
  a[6] = e2 - w2o;
  a[3] = e3 + w3o;
  a[7] = e3 - w3o;
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void dftR(Cx<T>* v) {
  if constexpr (R == 2) dft2<T, INV>(v[0], v[1]);
  else if constexpr (R == 3) dft3<T, INV>(v[0], v[1], v[2]);
  else if constexpr (R == 4) dft4<T, INV>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 8) dft8<T, INV>(v);
  else static_assert(R == 2, "unsupported radix");
}

// ---------------------------------------------------------------- one Stockham pass
// Sequence of length N at buf[0], buf[es], ..., buf[(N-1) es], processed by the G threads
// of one group (g = rank in the group).  LS = product of the radices already applied.
template <typename T, bool INV, int N, int G, int LS, int R>
__device__ __forceinline__ void stockham_pass(Cx<T>* buf, int es, int g, const Cx<T>* tw,
                                              bool active) {
  constexpr int NB = N / R;
  static_assert(NB % G == 0, "butterflies must divide evenly over the group");
  constexpr int BPT = NB / G;
  Cx<T> v[BPT][R];
  if (active) {
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = g + b * G;
#pragma unroll
      for (int t = 0; t < R; ++t) v[b][t] = buf[(j + t * NB) * es];
      if constexpr (LS > 1) {
        const int k = j % LS;
#pragma unroll
        for (int t = 1; t < R; ++t) {
          Cx<T> w = tw[t * k * (N / (LS * R))];
          if (INV) w.y = -w.y;
          v[b][t] = cmul(v[b][t], w);
        }
      }
      dftR<T, INV, R>(v[b]);
    }
  }
  __syncwarp();
  if (active) {
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = g + b * G;
      const int k = j % LS;
      const int base = (j / LS) * LS * R + k;
#pragma unroll
      for (int t = 0; t < R; ++t) buf[(base + t * LS) * es] = v[b][t];
    }
  }
  __syncwarp();
}

template <typename T, bool INV, int N, int G, int LS, int R, int... Rest>
__device__ __forceinline__ void stockham(Cx<T>* buf, int es, int g, const Cx<T>* tw, bool active) {
  stockham_pass<T, INV, N, G, LS, R>(buf, es, g, tw, active);
  if constexpr (sizeof...(Rest) > 0) stockham<T, INV, N, G, LS * R, Rest...>(buf, es, g, tw, active);
}

// ---------------------------------------------------------------- per-length plans
// G threads per transform; radix sequences chosen so every pass divides evenly over G.
template <int N>
struct Plan;
#define PF_PLAN(NN, GG, ...)                                                                 \
  template <>                                                                                \
  struct Plan<NN> {                                                                          \
    static constexpr int G = GG;                                                             \
    template <typename T, bool INV>                                                          \
    __device__ __forceinline__ static void run(Cx<T>* b, int es, int g, const Cx<T>* tw, bool a) { \
      stockham<T, INV, NN, GG, 1, __VA_ARGS__>(b, es, g, tw, a);                             \
    }                                                                                        \
  };
PF_PLAN(8, 1, 8)
PF_PLAN(16, 4, 4, 4)
PF_PLAN(32, 4, 8, 4)
PF_PLAN(48, 4, 3, 4, 4)
PF_PLAN(64, 8, 8, 8)
PF_PLAN(96, 8, 2, 3, 4, 4)
PF_PLAN(128, 16, 4, 4, 8)
PF_PLAN(256, 32, 4, 8, 8)
#undef PF_PLAN

// ---------------------------------------------------------------- batched complex FFTs
// nseq sequences of length N; sequence q starts at base[q*bs], elements at stride es.
// Every thread of the CTA must call this (uniform trip counts keep __syncwarp legal).
template <typename T, bool INV, int N>
__device__ __forceinline__ void fft_batch_n(Cx<T>* base, int es, int bs, int nseq, const Cx<T>* tw) {
  constexpr int G = Plan<N>::G;
  const int g = threadIdx.x % G;
  const int grp = threadIdx.x / G;
  const int ngrp = blockDim.x / G;
#pragma unroll 1
  for (int q0 = 0; q0 < nseq; q0 += ngrp) {
    const int q = q0 + grp;
    const bool active = q < nseq;
    Plan<N>::template run<T, INV>(base + (active ? q : 0) * bs, es, g, tw, active);
  }
}


// ---------------------------------------------------------------- real transforms along x
// Shared-memory plane layout S[y*Kx + kx], Kx = Nx/2+1 (the reference's half spectrum on x).
// Rows are processed in pairs (2p, 2p+1) that occupy the span S[2p*Kx, 2p*Kx + 2Kx): the
// real rows enter as the complex sequence z[x] = row_2p[x] + i row_2p+1[x] in the first Nx
// slots of that span, one complex FFT gives both half spectra (two-for-one), and they are
// unpacked in place to rows 2p and 2p+1.  A 1-row plane (Ny = 1) uses a zero second row.

// Forward: z (spans, Nx complex each) -> half spectra A (row 2p) and B (row 2p+1).
template <typename T, int N>
__device__ __forceinline__ void rfft_pairs_fwd_n(Cx<T>* S, int kxn, int npairs, bool two_rows, const Cx<T>* tw) {
  constexpr int G = Plan<N>::G;
  constexpr int KX = N / 2 + 1;
  constexpr int PER = (KX + G - 1) / G;
  const int g = threadIdx.x % G;
  const int grp = threadIdx.x / G;
  const int ngrp = blockDim.x / G;
#pragma unroll 1
  for (int p0 = 0; p0 < npairs; p0 += ngrp) {
    const int p = p0 + grp;
    const bool active = p < npairs;
    Cx<T>* z = S + (active ? p : 0) * 2 * kxn;
    Plan<N>::template run<T, false>(z, 1, g, tw, active);
    Cx<T> a[PER], b[PER];
    if (active) {
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int k = g + i * G;
        if (k < KX) {
          const Cx<T> zk = z[k];
          const Cx<T> zn = z[(N - k) % N];
          // A = (Z_k + conj Z_{N-k}) / 2 ; B = (Z_k - conj Z_{N-k}) / (2i)
          a[i] = cx<T>((T)0.5 * (zk.x + zn.x), (T)0.5 * (zk.y - zn.y));
          b[i] = cx<T>((T)0.5 * (zk.y + zn.y), (T)0.5 * (zn.x - zk.x));
        }
      }
    }
    __syncwarp();
    if (active) {
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int k = g + i * G;
        if (k < KX) {
          z[k] = a[i];
          if (two_rows) z[kxn + k] = b[i];
        }
      }
    }
    __syncwarp();
  }
}

// Inverse: half spectra A (row 2p), B (row 2p+1) -> z[x] = a[x] + i b[x], x in [0, Nx).
template <typename T, int N>
__device__ __forceinline__ void rfft_pairs_inv_n(Cx<T>* S, int kxn, int npairs, bool two_rows, const Cx<T>* tw) {
  constexpr int G = Plan<N>::G;
  constexpr int PER = N / G;
  const int g = threadIdx.x % G;
  const int grp = threadIdx.x / G;
  const int ngrp = blockDim.x / G;
#pragma unroll 1
  for (int p0 = 0; p0 < npairs; p0 += ngrp) {
    const int p = p0 + grp;
    const bool active = p < npairs;
    Cx<T>* z = S + (active ? p : 0) * 2 * kxn;
    Cx<T> v[PER];
    if (active) {
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int x = g + i * G;
        Cx<T> A, B;
        if (x <= N / 2) {
          A = z[x];
          B = two_rows ? z[kxn + x] : cx<T>(0, 0);
        } else {
          A = conj(z[N - x]);
          B = two_rows ? conj(z[kxn + N - x]) : cx<T>(0, 0);
        }
        v[i] = cx<T>(A.x - B.y, A.y + B.x);  // A + i B
      }
    }
    __syncwarp();
    if (active) {
#pragma unroll
      for (int i = 0; i < PER; ++i) z[g + i * G] = v[i];
    }
    __syncwarp();
    Plan<N>::template run<T, true>(z, 1, g, tw, active);
  }
}


// Forward 2D real transform of the NX x NY plane held in S as row pairs (see above);
// afterwards S holds the half spectrum S[ky*Kx + kx].  Ends with __syncthreads.
template <typename T, int NX, int NY>
__device__ __forceinline__ void plane_fwd(Cx<T>* S, const Cx<T>* twx, const Cx<T>* twy) {
  constexpr int KX = NX / 2 + 1;
  constexpr int NP = NY > 1 ? NY / 2 : 1;
  rfft_pairs_fwd_n<T, NX>(S, KX, NP, NY > 1, twx);
  __syncthreads();
  if constexpr (NY > 1) {
    fft_batch_n<T, false, NY>(S, KX, 1, KX, twy);
    __syncthreads();
  }
}

// Inverse of plane_fwd (unnormalised).  Afterwards S[p*2Kx + x] = (row_2p[x], row_2p+1[x]).
template <typename T, int NX, int NY>
__device__ __forceinline__ void plane_inv(Cx<T>* S, const Cx<T>* twx, const Cx<T>* twy) {
  constexpr int KX = NX / 2 + 1;
  constexpr int NP = NY > 1 ? NY / 2 : 1;
  if constexpr (NY > 1) {
    fft_batch_n<T, true, NY>(S, KX, 1, KX, twy);
    __syncthreads();
  }
  rfft_pairs_inv_n<T, NX>(S, KX, NP, NY > 1, twx);
  __syncthreads();
}

// Element (y, x) of a real plane held in pair layout.
template <typename T>
__device__ __forceinline__ T& pair_elem(Cx<T>* S, int kxn, int y, int x) {
  Cx<T>& c = S[(y >> 1) * 2 * kxn + x];
  return (y & 1) ? c.y : c.x;
}

}  // namespace pf
