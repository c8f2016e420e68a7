// In-register / shared-memory FFT building blocks for the pseudo-spectral MDE step.
//
// A transform of length N is run by a group of G threads (G divides 32, so a group never
// straddles a warp).  It is a sequence of Stockham autosort passes of radices R_1..R_P; in
// pass p every thread owns BPT = N/(R_p G) butterflies, loads their R_p inputs (from wherever
// the caller's accessor reads: global memory, shared memory, or its own registers), applies
// the twiddles and a register DFT, and hands the outputs to the caller's store accessor.
//
// Plans list the radices in "A" order; a transform can run in A order or in the reversed "B"
// order.  Running the inverse in A order and the forward in B order makes the last inverse
// pass and the first forward pass the same radix with the same per-thread element set
// ({j + t N/R}), so a caller can finish one transform and start the next without a
// shared-memory round trip; likewise forward-B then inverse-A around a pointwise multiply.
//
// Twiddles of a pass with span LS and radix R are read from a per-pass table laid out
// [(t-1) LS + k] = exp(-2 pi i t k / (LS R)): lanes with consecutive k read consecutive
// words (no bank conflicts).  Forward transforms use exp(-2 pi i ...), inverse ones the
// conjugate; both are unnormalised (the 1/Ng of the reference's irfft is folded into LD).
#pragma once
#include "pf_common.cuh"

namespace pf {

// ---------------------------------------------------------------- small DFTs in registers
template <typename T, bool INV>
__device__ __forceinline__ void dft2(Cx<T>& a0, Cx<T>& a1) {
  const Cx<T> t = a0 - a1;
  a0 = a0 + a1;
  a1 = t;
}

// d +- (-i) t for the forward transform, d +- (+i) t for the inverse, written per component so
// that no lane swap is needed (the complex sums elsewhere are packed two-lane instructions)
template <typename T, bool INV>
__device__ __forceinline__ void rot_pair(const Cx<T>& d, const Cx<T>& t, Cx<T>& plus, Cx<T>& minus) {
  if (INV) {
    plus = cx<T>(d.x - t.y, d.y + t.x);
    minus = cx<T>(d.x + t.y, d.y - t.x);
  } else {
    plus = cx<T>(d.x + t.y, d.y - t.x);
    minus = cx<T>(d.x - t.y, d.y + t.x);
  }
}

template <typename T, bool INV>
__device__ __forceinline__ void dft3(Cx<T>& a0, Cx<T>& a1, Cx<T>& a2) {
  const T s3 = (T)0.866025403784438646763723170752936183;  // sqrt(3)/2
  const Cx<T> t1 = a1 + a2;
  const Cx<T> t2 = cx<T>(a0.x - (T)0.5 * t1.x, a0.y - (T)0.5 * t1.y);
  const Cx<T> t3 = cscale(a1 - a2, s3);
  a0 = a0 + t1;
  rot_pair<T, INV>(t2, t3, a1, a2);  // t2 +- (-i or +i) t3
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4(Cx<T>& a0, Cx<T>& a1, Cx<T>& a2, Cx<T>& a3) {
  const Cx<T> s02 = a0 + a2, d02 = a0 - a2;
  const Cx<T> s13 = a1 + a3, t13 = a1 - a3;
  a0 = s02 + s13;
  a2 = s02 - s13;
  rot_pair<T, INV>(d02, t13, a1, a3);
}

// a * (c - i s) for forward transforms, a * (c + i s) for inverse ones
template <typename T, bool INV>
__device__ __forceinline__ Cx<T> wmul(Cx<T> a, T c, T s) {
  return INV ? cx<T>(a.x * c - a.y * s, a.x * s + a.y * c) : cx<T>(a.x * c + a.y * s, a.y * c - a.x * s);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft6(Cx<T>* a) {
  // n = n1 + 3 n2, k = 2 k1 + k2: radix 2 over n2, twiddle w6^(n1 k2), radix 3 over n1
  const T h = (T)0.5, s3 = (T)0.866025403784438646763723170752936183;
  Cx<T> b0 = a[0] + a[3], c0 = a[0] - a[3];
  Cx<T> b1 = a[1] + a[4], c1 = a[1] - a[4];
  Cx<T> b2 = a[2] + a[5], c2 = a[2] - a[5];
  c1 = wmul<T, INV>(c1, h, s3);   // w6^1
  c2 = wmul<T, INV>(c2, -h, s3);  // w6^2
  dft3<T, INV>(b0, b1, b2);
  dft3<T, INV>(c0, c1, c2);
  a[0] = b0;
  a[2] = b1;
  a[4] = b2;
  a[1] = c0;
  a[3] = c1;
  a[5] = c2;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(Cx<T>* a) {
  const T r = (T)0.707106781186547524400844362104849039;  // 1/sqrt(2)
  Cx<T> e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  Cx<T> o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<T, INV>(e0, e1, e2, e3);
  dft4<T, INV>(o0, o1, o2, o3);
  const Cx<T> w1o = wmul<T, INV>(o1, r, r);
  const Cx<T> w3o = wmul<T, INV>(o3, -r, r);
  a[0] = e0 + o0;
  a[4] = e0 - o0;
  a[1] = e1 + w1o;
  a[5] = e1 - w1o;
  rot_pair<T, INV>(e2, o2, a[2], a[6]);  // o2 times -i (forward) / +i (inverse)
  a[3] = e3 + w3o;
  a[7] = e3 - w3o;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft16(Cx<T>* a) {
  // n = n1 + 4 n2, k = 4 k1 + k2: inner DFT4 over n2, twiddle w16^(n1 k2), outer DFT4 over n1
  const T c1 = (T)0.923879532511286756128183189396788933;  // cos(pi/8)
  const T s1 = (T)0.382683432365089771728459984030398866;  // sin(pi/8)
  const T r = (T)0.707106781186547524400844362104849039;
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) dft4<T, INV>(a[n1], a[n1 + 4], a[n1 + 8], a[n1 + 12]);
  // a[n1 + 4 k2] now holds b[n1][k2]
  a[5] = wmul<T, INV>(a[5], c1, s1);      // w^1
  a[9] = wmul<T, INV>(a[9], r, r);        // w^2
  a[13] = wmul<T, INV>(a[13], s1, c1);    // w^3
  a[6] = wmul<T, INV>(a[6], r, r);        // w^2
  a[10] = mul_mi<T, INV>(a[10]);          // w^4
  a[14] = wmul<T, INV>(a[14], -r, r);     // w^6
  a[7] = wmul<T, INV>(a[7], s1, c1);      // w^3
  a[11] = wmul<T, INV>(a[11], -r, r);     // w^6
  a[15] = wmul<T, INV>(a[15], -c1, -s1);  // w^9
  Cx<T> y[16];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    Cx<T> b0 = a[4 * k2 + 0], b1 = a[4 * k2 + 1], b2 = a[4 * k2 + 2], b3 = a[4 * k2 + 3];
    dft4<T, INV>(b0, b1, b2, b3);
    y[k2] = b0;
    y[4 + k2] = b1;
    y[8 + k2] = b2;
    y[12 + k2] = b3;
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = y[k];
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void dftR(Cx<T>* v) {
  if constexpr (R == 2) dft2<T, INV>(v[0], v[1]);
  else if constexpr (R == 3) dft3<T, INV>(v[0], v[1], v[2]);
  else if constexpr (R == 4) dft4<T, INV>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 6) dft6<T, INV>(v);
  else if constexpr (R == 8) dft8<T, INV>(v);
  else if constexpr (R == 16) dft16<T, INV>(v);
  else static_assert(R == 2, "unsupported radix");
}

// ---------------------------------------------------------------- plans
// Radices in A order and the group size G (G divides N / R for every R).
template <int N>
struct Plan;
#define PF_PLAN(NN, GG, NP, R0, R1, R2)                                                   \
  template <>                                                                             \
  struct Plan<NN> {                                                                       \
    static constexpr int G = GG;                                                          \
    static constexpr int P = NP;                                                          \
    __host__ __device__ static constexpr int ra(int p) { return p == 0 ? R0 : p == 1 ? R1 : R2; } \
  };
PF_PLAN(8, 1, 1, 8, 1, 1)
PF_PLAN(16, 4, 2, 4, 4, 1)
PF_PLAN(32, 4, 2, 4, 8, 1)
PF_PLAN(48, 4, 3, 3, 4, 4)
PF_PLAN(64, 8, 2, 8, 8, 1)
PF_PLAN(96, 8, 3, 6, 4, 4)
PF_PLAN(128, 8, 2, 16, 8, 1)
PF_PLAN(256, 16, 2, 16, 16, 1)
#undef PF_PLAN

// Radix of pass p (0-based) in order O (0 = A, 1 = B, reversed), the span before it and the
// offset of its twiddle table.
template <int N, int O>
struct Order {
  static constexpr int P = Plan<N>::P;
  __host__ __device__ static constexpr int radix(int p) { return O == 0 ? Plan<N>::ra(p) : Plan<N>::ra(P - 1 - p); }
  __host__ __device__ static constexpr int span(int p) { return p == 0 ? 1 : span(p - 1) * radix(p - 1); }
  __host__ __device__ static constexpr int tw_offset(int p) {
    return p == 0 ? 0 : tw_offset(p - 1) + (radix(p - 1) - 1) * span(p - 1);
  }
  static constexpr int TW_SIZE = tw_offset(P);
};

// ---------------------------------------------------------------- one pass
// Thread g's butterfly b has j = g + b G; inputs j + t NB, outputs (j / LS) LS R + j % LS + t LS.
template <typename T, bool INV, int N, int G, int LS, int R>
struct Pass {
  static constexpr int NB = N / R;
  static_assert(NB % G == 0, "butterflies must divide evenly over the group");
  static constexpr int BPT = NB / G;

  template <class Ld>
  __device__ __forceinline__ static void load(Cx<T> (&v)[BPT][R], int g, Ld&& ld) {
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = g + b * G;
#pragma unroll
      for (int t = 0; t < R; ++t) v[b][t] = ld(j + t * NB);
    }
  }
  // tw: this pass's table [(t-1) LS + k]
  __device__ __forceinline__ static void compute(Cx<T> (&v)[BPT][R], int g, const Cx<T>* tw) {
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      if constexpr (LS > 1) {
        const int k = (g + b * G) % LS;
#pragma unroll
        for (int t = 1; t < R; ++t) {
          Cx<T> w = tw[(t - 1) * LS + k];
          if (INV) w.y = -w.y;
          v[b][t] = cmul(v[b][t], w);
        }
      }
      dftR<T, INV, R>(v[b]);
    }
  }
  template <class St>
  __device__ __forceinline__ static void store(const Cx<T> (&v)[BPT][R], int g, St&& st) {
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = g + b * G;
      const int base = (j / LS) * LS * R + j % LS;
#pragma unroll
      for (int t = 0; t < R; ++t) st(base + t * LS, v[b][t]);
    }
  }
};

template <typename T, bool INV, int N, int O, int p>
using PassOf = Pass<T, INV, N, Plan<N>::G, Order<N, O>::span(p), Order<N, O>::radix(p)>;

// Element positions held by a thread at the join of two transforms: the outputs of the last
// pass of order A (= inputs of the first pass of order B): position j + t N/R.
template <int N>
struct Join {
  static constexpr int G = Plan<N>::G;
  static constexpr int R = Plan<N>::ra(Plan<N>::P - 1);  // last radix of A = first radix of B
  static constexpr int NB = N / R;
  static constexpr int BPT = NB / G;
  __device__ __forceinline__ static int pos(int g, int b, int t) { return g + b * G + t * NB; }
};
// ... and at the join forward-B -> inverse-A: the last radix of B = the first radix of A.
template <int N>
struct JoinBA {
  static constexpr int G = Plan<N>::G;
  static constexpr int R = Plan<N>::ra(0);
  static constexpr int NB = N / R;
  static constexpr int BPT = NB / G;
  __device__ __forceinline__ static int pos(int g, int b, int t) { return g + b * G + t * NB; }
};

// Scratch index between passes: XOR of the low four bits with the next four, a bijection on
// every 256 consecutive indices.  A Stockham pass with LS = 1 writes j R + t (stride R over
// the lanes), which would put the lanes of a group on one bank; swizzled they spread out.
// Data that leaves a transform (its final store) stays in natural order.
__device__ __forceinline__ int swz(int i) { return i ^ ((i >> 4) & 15); }

// Per-length scratch index of the plane and pencil transforms: each XORs the low bits with
// higher ones (a bijection on every aligned block of 4 or 8 indices), chosen with the group
// strides below from a wavefront count of every shared-memory access of the plane pass under
// the hardware's rule for 8-byte accesses (each half warp of 16 lanes must cover 16 distinct
// 8-byte bank pairs to take one wavefront).
template <int N>
__device__ __forceinline__ int pswz(int i) {
  if constexpr (N == 16) return i ^ ((i >> 2) & 3);
  else if constexpr (N == 32 || N == 48) return i ^ (((i >> 2) ^ (i >> 4)) & 3);
  else if constexpr (N == 64) return i ^ ((i >> 3) & 7);
  else if constexpr (N == 96 || N == 128) return i ^ (((i >> 3) ^ (i >> 6)) & 7);
  else return swz(i);
}

// Passes p in [P0, P1) of a transform held in shared memory at buf[m(i) * es], in place and
// group-synchronised (load all, __syncwarp, store all).  Loads of pass P0 use the swizzled
// index pswz<N> when SWZ_IN, stores of pass P1-1 when SWZ_OUT; everything in between is
// swizzled.
template <typename T, bool INV, int N, int O, int P0, int P1, bool SWZ_IN, bool SWZ_OUT>
__device__ __forceinline__ void smem_passes(Cx<T>* buf, int es, int g, const Cx<T>* twtab, bool active) {
  if constexpr (P0 < P1) {
    using PS = PassOf<T, INV, N, O, P0>;
    Cx<T> v[PS::BPT][Order<N, O>::radix(P0)];
    if (active) {
      PS::load(v, g, [&](int i) { return buf[(SWZ_IN ? pswz<N>(i) : i) * es]; });
      PS::compute(v, g, twtab + Order<N, O>::tw_offset(P0));
    }
    __syncwarp();
    constexpr bool last = P0 + 1 == P1;
    if (active)
      PS::store(v, g, [&](int i, const Cx<T>& x) { buf[((!last || SWZ_OUT) ? pswz<N>(i) : i) * es] = x; });
    __syncwarp();
    smem_passes<T, INV, N, O, P0 + 1, P1, true, SWZ_OUT>(buf, es, g, twtab, active);
  }
}

// Group -> row pair / column assignment.  The GPW = 32/G groups of a warp get indices S apart
// (then the next warp), so that their shared-memory windows fall on different banks; S is
// chosen per length with pswz from the same wavefront count (the x transforms of a row pair
// use pair_stride<Nx>, the y transforms of a column col_stride<Ny>).
template <int N>
__host__ __device__ constexpr int pair_stride() {
  return (N == 16 || N == 32 || N == 48) ? 2 : (N == 64 || N == 96 || N == 128) ? 4 : 1;
}
template <int N>
__host__ __device__ constexpr int col_stride() {
  return (N == 16 || N == 32 || N == 48) ? 4 : (N == 64 || N == 96 || N == 128) ? 8 : 1;
}
// padding (complex elements) after each z pencil of a tile
template <int N>
__host__ __device__ constexpr int pencil_pad() {
  return (N == 16 || N == 32 || N == 48) ? 2 : (N == 64 || N == 96 || N == 128) ? 4 : 1;
}
// index of group grp (of groups of G threads) under stride S
template <int G, int S>
__host__ __device__ constexpr int group_index(int grp) {
  constexpr int GPW = 32 / G;
  const int w = grp / GPW, lg = grp % GPW;
  return (w / S) * (GPW * S) + lg * S + (w % S);
}
// warps needed so that every index below count has a group
template <int G, int S>
__host__ __device__ constexpr int warps_for(int count) {
  constexpr int GPW = 32 / G;
  int wmax = 0;
  for (int idx = 0; idx < count; ++idx) {
    const int w = (idx / (GPW * S)) * S + (idx % S);
    if (w > wmax) wmax = w;
  }
  return wmax + 1;
}

}  // namespace pf
