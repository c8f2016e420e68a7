// pf_cpu.cpp -- FP64 CPU restatement of PolyFields.jl's scft! iteration in C++17 + OpenMP.
//
// TEST INFRASTRUCTURE, not the product: the timed CPU baseline of bench.py (its cpu_baseline
// leg and its --impl reference arm) and a second CPU restatement that the tests pin to the
// NumPy oracle (oracle/pf_oracle.py) at 1e-12.  Nothing in the GPU engine links or calls it.
//
// It follows the reference function by function (file:line within PolyFields.jl):
//   PseudoSpectralSolver update! / propagate! (:RK2)   src/system/mde.jl:43-57, 65-81
//   FFTHolder rfft / irfft (normalised by 1/Ng)        src/system/fft.jl:17-36
//   density!(::Multiblock): forward and backward chains, Q, Simpson, normalisation
//                                                      src/species/multiblock.jl:125-231
//   density!(::Point)                                  src/species/point.jl:36-53
//   muphi! (canonical), density!(sys)                  src/system/system.jl:248-289
//   potentials! / potential!(::FloryInteraction)       src/system/system.jl:296-310, src/interactions/flory.jl:82-100
//   update!(::Compressibility) (strict)                src/system/compress.jl:37-54
//   residuals! with mean subtraction                   src/system/system.jl:317-340
//   free_energy (quirk: mu = phi), field_error         src/system/system.jl:402-433, 470-486
//   energy(::FloryInteraction)                         src/interactions/flory.jl:39-59
//   AndersonUpdater setup! / step!                     src/updaters/anderson.jl:54-228
// The FFT is this file's own mixed-radix Stockham transform (radices 8, 4, 2, 3), standing in for
// FFTW; a DFT is unique, so any correct FFT agrees with FFTW to rounding.  Threads: OpenMP over
// transform rows / columns / pencils and grid points (the reference lets FFTW thread,
// src/utils.jl:16-18).  Grids are [z][y][x] with x fastest (the reference's column-major
// Array{Float64,3}[x, y, z]); the half spectrum is [kz][ky][kx], kx in [0, Nx/2].
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

namespace {

using cplx = std::complex<double>;

// ---------------------------------------------------------------- batched complex FFT (Stockham)
// A transform of length n over "elements" that are vectors of B contiguous complex values
// (interleaved re, im): element t of the input sits at x[t * B].  Pass with radix R and span L
// (product of the radices before it): butterfly j (0 <= j < n/R) reads elements j + t n/R,
// multiplies element t by w^(t k) with k = j mod L, w = exp(sign 2 pi i / (L R)), applies a
// length-R DFT and writes elements (j / L) L R + k + s L.  The last pass leaves natural order.
// Every butterfly works on B-long vectors, so the inner loops are contiguous.
struct Plan1D {
  int n = 1;
  std::vector<int> radix;
  std::vector<std::vector<double>> tw;  // per pass: [(t - 1) L + k] -> (cos, sin) of -2 pi t k / (L R)
  explicit Plan1D(int n_ = 1) : n(n_) {
    int m = n;
    while (m % 8 == 0) {
      radix.push_back(8);
      m /= 8;
    }
    while (m % 4 == 0 && m > 1) {
      radix.push_back(4);
      m /= 4;
    }
    while (m % 2 == 0) {
      radix.push_back(2);
      m /= 2;
    }
    while (m % 3 == 0) {
      radix.push_back(3);
      m /= 3;
    }
    if (m != 1) throw std::runtime_error("FFT length must be 2^a 3^b");
    int L = 1;
    for (int R : radix) {
      std::vector<double> t(2 * (size_t)(R - 1) * L);
      for (int a = 1; a < R; ++a)
        for (int k = 0; k < L; ++k) {
          const long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)(a * k) /
                                  (long double)(L * R);
          t[2 * ((size_t)(a - 1) * L + k)] = (double)cosl(ang);
          t[2 * ((size_t)(a - 1) * L + k) + 1] = (double)sinl(ang);
        }
      tw.push_back(std::move(t));
      L *= R;
    }
  }
};

struct C2 {
  double r, i;
};
static inline C2 add(C2 a, C2 b) { return {a.r + b.r, a.i + b.i}; }
static inline C2 sub(C2 a, C2 b) { return {a.r - b.r, a.i - b.i}; }
static inline C2 mul(C2 a, double c, double s) { return {a.r * c - a.i * s, a.r * s + a.i * c}; }
// multiply by -i (forward, sign < 0) or +i (inverse)
static inline C2 rot(C2 a, int sign) { return sign < 0 ? C2{a.i, -a.r} : C2{-a.i, a.r}; }

template <int R>
static inline void dft(C2* v, int sign) {
  if constexpr (R == 2) {
    const C2 a = v[0], b = v[1];
    v[0] = add(a, b);
    v[1] = sub(a, b);
  } else if constexpr (R == 3) {
    const double s3 = 0.866025403784438646763723170752936183;
    const C2 t1 = add(v[1], v[2]);
    const C2 t2 = {v[0].r - 0.5 * t1.r, v[0].i - 0.5 * t1.i};
    const C2 d = sub(v[1], v[2]);
    const C2 t3 = rot(C2{d.r * s3, d.i * s3}, sign);
    v[0] = add(v[0], t1);
    v[1] = add(t2, t3);
    v[2] = sub(t2, t3);
  } else if constexpr (R == 4) {
    const C2 s02 = add(v[0], v[2]), d02 = sub(v[0], v[2]), s13 = add(v[1], v[3]), d13 = rot(sub(v[1], v[3]), sign);
    v[0] = add(s02, s13);
    v[2] = sub(s02, s13);
    v[1] = add(d02, d13);
    v[3] = sub(d02, d13);
  } else {  // R == 8: two length-4 DFTs of the even and odd inputs, twiddles w8^k, combine
    const double h = 0.707106781186547524400844362104849039;
    C2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft<4>(e, sign);
    dft<4>(o, sign);
    const double sg = sign < 0 ? -1.0 : 1.0;
    o[1] = mul(o[1], h, sg * h);
    o[2] = rot(o[2], sign);
    o[3] = mul(o[3], -h, sg * h);
    for (int k = 0; k < 4; ++k) {
      v[k] = add(e[k], o[k]);
      v[k + 4] = sub(e[k], o[k]);
    }
  }
}

template <int R>
static void stockham_pass(const C2* in, C2* out, int n, int L, long B, const double* tw, int sign) {
  const int nb = n / R;
  C2 v[8];
  for (int j = 0; j < nb; ++j) {
    const int k = j % L;
    double c[8], sn[8];
    for (int t = 1; t < R; ++t) {
      c[t] = tw[2 * ((t - 1) * L + k)];
      sn[t] = sign < 0 ? tw[2 * ((t - 1) * L + k) + 1] : -tw[2 * ((t - 1) * L + k) + 1];
    }
    const long base = (long)(j / L) * L * R + k;
    for (long b = 0; b < B; ++b) {
      for (int t = 0; t < R; ++t) v[t] = in[((long)j + (long)t * nb) * B + b];
      if (k > 0)
        for (int t = 1; t < R; ++t) v[t] = mul(v[t], c[t], sn[t]);
      dft<R>(v, sign);
      for (int s2 = 0; s2 < R; ++s2) out[(base + (long)s2 * L) * B + b] = v[s2];
    }
  }
}

// x: n elements of B complex values; work: the same size.  Result in x.
static void fft_batch(const Plan1D& p, C2* x, C2* work, long B, int sign) {
  if (p.n == 1) return;
  C2* in = x;
  C2* out = work;
  int L = 1;
  for (size_t q = 0; q < p.radix.size(); ++q) {
    const int R = p.radix[q];
    const double* tw = p.tw[q].data();
    switch (R) {
      case 2: stockham_pass<2>(in, out, p.n, L, B, tw, sign); break;
      case 3: stockham_pass<3>(in, out, p.n, L, B, tw, sign); break;
      case 4: stockham_pass<4>(in, out, p.n, L, B, tw, sign); break;
      default: stockham_pass<8>(in, out, p.n, L, B, tw, sign); break;
    }
    std::swap(in, out);
    L *= R;
  }
  if (in != x) std::memcpy(x, in, sizeof(C2) * (size_t)p.n * B);
}

// ---------------------------------------------------------------- 3D real FFT
// Real grids [z][y][x]; half spectra [z][y][kx].  x: two real rows per complex transform; y:
// batched over the kx columns of a plane; z: batched over chunks of the (y, kx) plane.
struct FFT3 {
  int nx, ny, nz, kx;
  Plan1D px, py, pz;
  static constexpr long kChunk = 64;  // complex values per z-transform chunk
  static constexpr int kPairs = 8;    // row pairs per batched x transform
  FFT3(int x, int y, int z) : nx(x), ny(y), nz(z), kx(x / 2 + 1), px(x), py(y), pz(z) {}

  void zpass(cplx* k, int sign) const {
    const long plane = (long)ny * kx;
    const long nchunk = (plane + kChunk - 1) / kChunk;
#pragma omp parallel
    {
      std::vector<C2> a((size_t)nz * kChunk), b(a.size());
#pragma omp for schedule(static)
      for (long c = 0; c < nchunk; ++c) {
        const long c0 = c * kChunk, B = std::min(kChunk, plane - c0);
        C2* src = reinterpret_cast<C2*>(k);
        for (int z = 0; z < nz; ++z) std::memcpy(&a[(size_t)z * B], src + (long)z * plane + c0, sizeof(C2) * B);
        fft_batch(pz, a.data(), b.data(), B, sign);
        for (int z = 0; z < nz; ++z) std::memcpy(src + (long)z * plane + c0, &a[(size_t)z * B], sizeof(C2) * B);
      }
    }
  }

  // forward z transform, multiply by ld, inverse z transform, chunk by chunk (the spectrum
  // between the two transforms never leaves the chunk buffer)
  void zfilter(cplx* k, const double* ld) const {
    const long plane = (long)ny * kx;
    const long nchunk = (plane + kChunk - 1) / kChunk;
#pragma omp parallel
    {
      std::vector<C2> a((size_t)nz * kChunk), b(a.size());
#pragma omp for schedule(static)
      for (long c = 0; c < nchunk; ++c) {
        const long c0 = c * kChunk, B = std::min(kChunk, plane - c0);
        C2* src = reinterpret_cast<C2*>(k);
        for (int z = 0; z < nz; ++z) std::memcpy(&a[(size_t)z * B], src + (long)z * plane + c0, sizeof(C2) * B);
        fft_batch(pz, a.data(), b.data(), B, -1);
        for (int z = 0; z < nz; ++z) {
          const double* l = ld + (long)z * plane + c0;
          C2* v = &a[(size_t)z * B];
          for (long j = 0; j < B; ++j) v[j] = C2{v[j].r * l[j], v[j].i * l[j]};
        }
        fft_batch(pz, a.data(), b.data(), B, +1);
        for (int z = 0; z < nz; ++z) std::memcpy(src + (long)z * plane + c0, &a[(size_t)z * B], sizeof(C2) * B);
      }
    }
  }

  // real r[z][y][x] -> half spectrum k[z][y][kx] (unnormalised); with lw, transforms lw * r
  // (one multiply per point, as the load into the x transform), and leaves out the z pass
  // (xy_only, for zfilter)
  void forward(const double* r, cplx* k, const double* lw = nullptr, bool xy_only = false) const {
#pragma omp parallel
    {
      std::vector<C2> a(std::max((long)nx * kPairs, (long)ny * kx)), b(a.size());
#pragma omp for schedule(static)
      for (int z = 0; z < nz; ++z) {
        C2* kp = reinterpret_cast<C2*>(k) + (long)z * ny * kx;
        // rows y, y+1 as the real and imaginary parts of one complex row; P such row pairs
        // side by side (element x of pair p at a[x P + p]) in one batched transform
        for (int y0 = 0; y0 < ny; y0 += 2 * kPairs) {
          const int P = std::min(kPairs, (ny - y0 + 1) / 2);
          for (int p = 0; p < P; ++p) {
            const int y = y0 + 2 * p;
            const double* r0 = r + ((long)z * ny + y) * nx;
            const double* r1 = (y + 1 < ny) ? r0 + nx : nullptr;
            if (lw) {
              const double* l0 = lw + ((long)z * ny + y) * nx;
              for (int x = 0; x < nx; ++x) a[(long)x * P + p] = C2{l0[x] * r0[x], r1 ? l0[nx + x] * r1[x] : 0.0};
            } else {
              for (int x = 0; x < nx; ++x) a[(long)x * P + p] = C2{r0[x], r1 ? r1[x] : 0.0};
            }
          }
          fft_batch(px, a.data(), b.data(), P, -1);
          for (int p = 0; p < P; ++p) {
            const int y = y0 + 2 * p;
            const bool two = y + 1 < ny;
            C2* k0 = kp + (long)y * kx;
            for (int i = 0; i < kx; ++i) {
              const C2 zk = a[(long)i * P + p], zn = a[(long)((nx - i) % nx) * P + p];
              k0[i] = C2{0.5 * (zk.r + zn.r), 0.5 * (zk.i - zn.i)};
              if (two) k0[kx + i] = C2{0.5 * (zk.i + zn.i), 0.5 * (zn.r - zk.r)};
            }
          }
        }
        if (ny > 1) fft_batch(py, kp, b.data(), kx, -1);
      }
    }
    if (nz > 1 && !xy_only) zpass(k, -1);
  }

  // half spectrum k (overwritten) -> real r, unnormalised inverse (the caller folds 1/Ng in);
  // with lw, writes lw * r; xy_only leaves out the z pass (done by zfilter)
  void inverse(cplx* k, double* r, const double* lw = nullptr, bool xy_only = false) const {
    if (nz > 1 && !xy_only) zpass(k, +1);
#pragma omp parallel
    {
      std::vector<C2> a(std::max((long)nx * kPairs, (long)ny * kx)), b(a.size());
#pragma omp for schedule(static)
      for (int z = 0; z < nz; ++z) {
        C2* kp = reinterpret_cast<C2*>(k) + (long)z * ny * kx;
        if (ny > 1) fft_batch(py, kp, b.data(), kx, +1);
        // Hermitian halves of rows y, y+1 -> one complex row; P row pairs per batched transform
        for (int y0 = 0; y0 < ny; y0 += 2 * kPairs) {
          const int P = std::min(kPairs, (ny - y0 + 1) / 2);
          for (int p = 0; p < P; ++p) {
            const int y = y0 + 2 * p;
            const bool two = y + 1 < ny;
            const C2* k0 = kp + (long)y * kx;
            const C2* k1 = two ? k0 + kx : nullptr;
            for (int x = 0; x < nx; ++x) {
              C2 A, Bv = {0.0, 0.0};
              if (x < kx) {
                A = k0[x];
                if (two) Bv = k1[x];
              } else {
                A = C2{k0[nx - x].r, -k0[nx - x].i};
                if (two) Bv = C2{k1[nx - x].r, -k1[nx - x].i};
              }
              a[(long)x * P + p] = C2{A.r - Bv.i, A.i + Bv.r};  // A + i B
            }
          }
          fft_batch(px, a.data(), b.data(), P, +1);
          for (int p = 0; p < P; ++p) {
            const int y = y0 + 2 * p;
            const bool two = y + 1 < ny;
            double* r0 = r + ((long)z * ny + y) * nx;
            if (lw) {
              const double* l0 = lw + ((long)z * ny + y) * nx;
              for (int x = 0; x < nx; ++x) r0[x] = l0[x] * a[(long)x * P + p].r;
              if (two)
                for (int x = 0; x < nx; ++x) r0[nx + x] = l0[nx + x] * a[(long)x * P + p].i;
            } else {
              for (int x = 0; x < nx; ++x) r0[x] = a[(long)x * P + p].r;
              if (two)
                for (int x = 0; x < nx; ++x) r0[nx + x] = a[(long)x * P + p].i;
            }
          }
        }
      }
    }
  }
};

// ---------------------------------------------------------------- system
struct Species {
  int kind = 0;  // 0 Multiblock, 1 Point
  std::vector<int> mon;     // monomer index of each block (Point: one entry)
  std::vector<double> b, ds;
  std::vector<int> begin;   // 1-based block boundaries, nblocks + 1 entries
  int Ns = 0;
  double Nref = 1.0, phi = 1.0, Q = 0.0;
  std::vector<double> q, qc;  // (Ns+1) x Ng
};

struct Anderson {
  int nhist = 20, iter = 0, iter_hist = 0, iter_euler = 1;
  double lam = 0.0, lam_euler = 0.01;
  std::vector<std::vector<double>> res_hist, field_hist;  // (nhist+1) x (nmon Ng)
  bool setup = false;
};

struct System {
  int nx, ny, nz;
  long ng, nk;
  FFT3 fft;
  std::vector<double> ksq;     // [kz][ky][kx]
  std::vector<double> vol;     // per monomer
  std::vector<double> chi;     // nmon x nmon, symmetric, 0 on the diagonal
  std::vector<std::vector<double>> w, rho, pot, res;
  std::vector<Species> species;
  Anderson A;
  // propagator scratch
  std::vector<double> lw, ld, qr;
  std::vector<cplx> qk;

  System(int x, int y, int z) : nx(x), ny(y), nz(z), ng((long)x * y * z), nk((long)(x / 2 + 1) * y * z), fft(x, y, z) {
    ksq.assign(nk, 0.0);
    lw.resize(ng);
    ld.resize(nk);
    qr.resize(ng);
    qk.resize(nk);
  }
  int nmon() const { return (int)vol.size(); }

  // update!(solver, omega, ksq, vol, b, ds) (mde.jl:43-57): LW1 and LD1, with irfft's 1/Ng folded into LD
  void update(const std::vector<double>& omega, double v, double b, double ds) {
    const double cw = ds / 2.0 * v, cd = ds * b * b / 6.0, inv = 1.0 / (double)ng;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ng; ++i) lw[i] = std::exp(-cw * omega[i]);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nk; ++i) ld[i] = std::exp(-cd * ksq[i]) * inv;
  }
  // propagate! :RK2 (mde.jl:76-81): qout = LW1 * irfft(LD1 * rfft(LW1 * qin))
  // The LW multiplies ride the x transforms' loads and stores; on 3D grids the LD multiply
  // sits between the forward and inverse z transforms of each chunk (FFT3::zfilter).
  void propagate(const double* qin, double* qout) {
    fft.forward(qin, qk.data(), lw.data(), true);
    if (nz > 1) {
      fft.zfilter(qk.data(), ld.data());
    } else {
#pragma omp parallel for schedule(static)
      for (long i = 0; i < nk; ++i) qk[i] = cplx(qk[i].real() * ld[i], qk[i].imag() * ld[i]);
    }
    fft.inverse(qk.data(), qout, lw.data(), true);
  }

  // density!(::Multiblock) (multiblock.jl:125-231); block densities added to rho with phi / (Q Nref)
  void chain_density(Species& sp) {
    const int nb = (int)sp.mon.size(), Ns = sp.Ns;
    sp.q.resize((size_t)(Ns + 1) * ng);
    double* q = sp.q.data();
    std::fill(q, q + ng, 1.0);
    for (int ib = 0; ib < nb; ++ib) {
      update(w[sp.mon[ib]], vol[sp.mon[ib]], sp.b[ib], sp.ds[ib]);
      for (int s = sp.begin[ib]; s < sp.begin[ib + 1]; ++s) propagate(q + (long)(s - 1) * ng, q + (long)s * ng);
    }
    // one block: qc_s = q_{Ns - s} (the chain reads the same from both ends), used in place
    double* qc = nullptr;
    if (nb > 1) {
      sp.qc.resize((size_t)(Ns + 1) * ng);
      qc = sp.qc.data();
      std::fill(qc + (long)Ns * ng, qc + (long)(Ns + 1) * ng, 1.0);
      for (int ib = nb - 1; ib >= 0; --ib) {
        update(w[sp.mon[ib]], vol[sp.mon[ib]], sp.b[ib], sp.ds[ib]);
        for (int s = sp.begin[ib + 1]; s > sp.begin[ib]; --s)
          propagate(qc + (long)(s - 1) * ng, qc + (long)(s - 2) * ng);
      }
    }
    double qsum = 0.0;
#pragma omp parallel for reduction(+ : qsum) schedule(static)
    for (long i = 0; i < ng; ++i) qsum += q[(long)Ns * ng + i];
    sp.Q = qsum / (double)ng;
    const double scale = sp.phi / (sp.Q * sp.Nref);  // muphi! canonical: phi_sp rho_sp
    auto qplane = [&](int s) { return q + (long)s * ng; };
    auto qcplane = [&](int s) { return qc ? qc + (long)s * ng : q + (long)(Ns - s) * ng; };
    // Simpson over the block's contour points, a chunk of grid points at a time: each chunk
    // streams the planes in order (per point the sums run in ascending s, as a point-by-point
    // loop would)
    constexpr long kCh = 2048;
    for (int ib = 0; ib < nb; ++ib) {
      const int bgn = sp.begin[ib], end = sp.begin[ib + 1];
      const double f = sp.ds[ib] / 3.0;
      double* out = rho[sp.mon[ib]].data();
#pragma omp parallel
      {
        std::vector<double> r(kCh), r4(kCh), r2(kCh);
#pragma omp for schedule(static)
        for (long c0 = 0; c0 < ng; c0 += kCh) {
          const long m = std::min(kCh, ng - c0);
          const double *qa = qplane(bgn - 1) + c0, *ca = qcplane(bgn - 1) + c0;
          const double *qb = qplane(end - 1) + c0, *cb = qcplane(end - 1) + c0;
          for (long i = 0; i < m; ++i) {
            r[i] = qa[i] * ca[i];
            r[i] += qb[i] * cb[i];
            r4[i] = 0.0;
            r2[i] = 0.0;
          }
          for (int s = bgn + 1; s < end; s += 2) {
            const double *qs = qplane(s - 1) + c0, *cs = qcplane(s - 1) + c0;
            for (long i = 0; i < m; ++i) r4[i] += qs[i] * cs[i];
          }
          for (int s = bgn + 2; s < end - 1; s += 2) {
            const double *qs = qplane(s - 1) + c0, *cs = qcplane(s - 1) + c0;
            for (long i = 0; i < m; ++i) r2[i] += qs[i] * cs[i];
          }
          for (long i = 0; i < m; ++i) out[c0 + i] += (r[i] + 4.0 * r4[i] + 2.0 * r2[i]) * f * scale;
        }
      }
    }
  }

  // density!(::Point) (point.jl:36-53)
  void point_density(Species& sp) {
    const int m = sp.mon[0];
    const double v = vol[m];
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < ng; ++i) s += std::exp(-v * w[m][i]);
    sp.Q = s / (double)ng;
    const double scale = sp.phi / sp.Q;
    double* out = rho[m].data();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ng; ++i) out[i] += scale * std::exp(-v * w[m][i]);
  }

  // residuals!(sys) (system.jl:317-340): density!, potentials!, compress, residual, mean subtraction
  void residuals() {
    const int M = nmon();
    for (auto& r : rho) std::fill(r.begin(), r.end(), 0.0);
    for (auto& sp : species) {
      if (sp.kind == 0) chain_density(sp);
      else point_density(sp);
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < ng; ++i) {
      double rs = 0.0, f = 0.0;
      for (int a = 0; a < M; ++a) {
        double p = 0.0;
        for (int b = 0; b < M; ++b)
          if (chi[a * M + b] != 0.0) p += chi[a * M + b] * (rho[b][i] / vol[b]);
        pot[a][i] = p;
        rs += rho[a][i];
      }
      f = rs - 1.0;
      for (int a = 0; a < M; ++a) f += w[a][i] - pot[a][i];
      const double eta = f / (double)M;
      for (int a = 0; a < M; ++a) res[a][i] = pot[a][i] + eta - w[a][i];
    }
    for (int a = 0; a < M; ++a) {
      double sw = 0.0, sr = 0.0;
#pragma omp parallel for reduction(+ : sw, sr) schedule(static)
      for (long i = 0; i < ng; ++i) {
        sw += w[a][i];
        sr += res[a][i];
      }
      sw /= (double)ng;
      sr /= (double)ng;
#pragma omp parallel for schedule(static)
      for (long i = 0; i < ng; ++i) {
        w[a][i] -= sw;
        res[a][i] -= sr;
      }
    }
  }

  double field_error() const {  // system.jl:470-486
    double rs = 0.0, ws = 2.220446049250313e-16;
    for (int a = 0; a < nmon(); ++a) {
      double r = 0.0, x = 0.0;
#pragma omp parallel for reduction(+ : r, x) schedule(static)
      for (long i = 0; i < ng; ++i) {
        r += res[a][i] * res[a][i];
        x += w[a][i] * w[a][i];
      }
      rs += r;
      ws += x;
    }
    return std::sqrt(rs) / std::sqrt(ws);
  }

  double free_energy() const {  // system.jl:402-433 (mu = phi, as the reference writes it)
    double ftrans = 0.0;
    for (const auto& sp : species)
      if (sp.phi > 1e-8) ftrans += sp.phi * (sp.phi - 1.0) / sp.Nref;
    double ffield = 0.0;
    for (int a = 0; a < nmon(); ++a) {
      double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
      for (long i = 0; i < ng; ++i) s += rho[a][i] * w[a][i];
      ffield -= s;
    }
    ffield /= (double)ng;
    const int M = nmon();
    double fexc = 0.0;  // energy(::FloryInteraction), flory.jl:39-59
    for (int a = 0; a < M; ++a)
      for (int b = a + 1; b < M; ++b) {
        const double c = chi[a * M + b];
        if (c == 0.0) continue;
        double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (long i = 0; i < ng; ++i) s += c * (rho[a][i] / vol[a]) * (rho[b][i] / vol[b]);
        fexc += s;
      }
    return ftrans + ffield + fexc / (double)ng;
  }

  // flat (monomer-major) copies of w and res
  void flat(const std::vector<std::vector<double>>& g, std::vector<double>& out) const {
    out.resize((size_t)nmon() * ng);
    for (int a = 0; a < nmon(); ++a) std::memcpy(out.data() + (size_t)a * ng, g[a].data(), sizeof(double) * ng);
  }

  void anderson_setup(int nhist) {  // anderson.jl:54-92
    A = Anderson();
    A.nhist = nhist;
    A.res_hist.assign(nhist + 1, std::vector<double>((size_t)nmon() * ng, 0.0));
    A.field_hist.assign(nhist + 1, std::vector<double>((size_t)nmon() * ng, 0.0));
    flat(w, A.field_hist[0]);
    A.setup = true;
  }

  static double dot(const double* a, const double* b, long n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
  }

  // step!(::AndersonUpdater) (anderson.jl:98-228); returns 0, or the 1-based zero pivot
  int anderson_step() {
    A.iter += 1;
    if (A.iter < A.nhist + 1) {
      A.iter_hist = A.iter - 1;
      A.lam = 1.0 - std::pow(0.9, A.iter);
    } else {
      A.iter_hist = A.nhist;
      A.lam = 1.0;
    }
    const int it = A.iter, ih = A.iter_hist;
    const long n = (long)nmon() * ng;
    residuals();
    flat(res, A.res_hist[ih]);
    std::vector<double> W;
    flat(w, W);
    if (it <= A.iter_euler) {
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) W[i] += A.lam_euler * A.res_hist[ih][i];
    } else {
      const double* r = A.res_hist[ih].data();
      std::vector<double> U((size_t)ih * ih, 0.0), V(ih, 0.0), d((size_t)ih * n);
      for (int m = 1; m <= ih; ++m) {
        const double* rm = A.res_hist[ih - m].data();
        double* dm = d.data() + (size_t)(m - 1) * n;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) dm[i] = r[i] - rm[i];
      }
      for (int m = 1; m <= ih; ++m) {
        const double* dm = d.data() + (size_t)(m - 1) * n;
        for (int k = m; k <= ih; ++k) {
          const double u = dot(dm, d.data() + (size_t)(k - 1) * n, n);
          U[(m - 1) * ih + (k - 1)] = u;
          U[(k - 1) * ih + (m - 1)] = u;
        }
        V[m - 1] = dot(dm, r, n);
      }
      // inv!(lu!(Umn)) * Vm (anderson.jl:184-189): LU with partial pivoting
      std::vector<double> a = U;
      std::vector<int> perm(ih);
      for (int i = 0; i < ih; ++i) perm[i] = i;
      for (int k = 0; k < ih; ++k) {
        int p = k;
        for (int i = k + 1; i < ih; ++i)
          if (std::fabs(a[i * ih + k]) > std::fabs(a[p * ih + k])) p = i;
        if (a[p * ih + k] == 0.0) return k + 1;
        if (p != k) {
          for (int j = 0; j < ih; ++j) std::swap(a[k * ih + j], a[p * ih + j]);
          std::swap(perm[k], perm[p]);
        }
        for (int i = k + 1; i < ih; ++i) {
          a[i * ih + k] /= a[k * ih + k];
          for (int j = k + 1; j < ih; ++j) a[i * ih + j] -= a[i * ih + k] * a[k * ih + j];
        }
      }
      std::vector<double> y(ih), C(ih);
      for (int i = 0; i < ih; ++i) {
        double s = V[perm[i]];
        for (int j = 0; j < i; ++j) s -= a[i * ih + j] * y[j];
        y[i] = s;
      }
      for (int i = ih - 1; i >= 0; --i) {
        double s = y[i];
        for (int j = i + 1; j < ih; ++j) s -= a[i * ih + j] * C[j];
        C[i] = s / a[i * ih + i];
      }
      const double* fi = A.field_hist[ih].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) {
        double WW = W[i], DD = r[i];
        for (int m = 1; m <= ih; ++m) {
          WW += C[m - 1] * (A.field_hist[ih - m][i] - fi[i]);
          DD += C[m - 1] * (A.res_hist[ih - m][i] - r[i]);
        }
        W[i] = WW + A.lam * DD;
      }
    }
    for (int a2 = 0; a2 < nmon(); ++a2) std::memcpy(w[a2].data(), W.data() + (size_t)a2 * ng, sizeof(double) * ng);
    if (it < A.nhist + 1) {
      A.field_hist[it] = W;
    } else {
      std::rotate(A.res_hist.begin(), A.res_hist.begin() + 1, A.res_hist.end());
      std::rotate(A.field_hist.begin(), A.field_hist.begin() + 1, A.field_hist.end());
      A.field_hist[A.nhist] = W;
    }
    return 0;
  }
};

}  // namespace

// ---------------------------------------------------------------- C ABI (ctypes)
extern "C" {

void* pfc_create(int nx, int ny, int nz, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  try {
    return new System(nx, ny, nz);
  } catch (...) {
    return nullptr;
  }
}
void pfc_destroy(void* h) { delete static_cast<System*>(h); }
int pfc_threads(void) { return omp_get_max_threads(); }

// |k|^2 on the half spectrum, [kz][ky][kx] (the oracle's UnitCell.ksq, quirk Q1 fold included)
void pfc_set_ksq(void* h, const double* ksq) {
  auto* s = static_cast<System*>(h);
  std::memcpy(s->ksq.data(), ksq, sizeof(double) * s->nk);
}
int pfc_add_monomer(void* h, double vol) {
  auto* s = static_cast<System*>(h);
  const int M = s->nmon() + 1;
  std::vector<double> c((size_t)M * M, 0.0);
  for (int a = 0; a < M - 1; ++a)
    for (int b = 0; b < M - 1; ++b) c[a * M + b] = s->chi[a * (M - 1) + b];
  s->chi = c;
  s->vol.push_back(vol);
  for (auto* g : {&s->w, &s->rho, &s->pot, &s->res}) g->emplace_back(s->ng, 0.0);
  return M - 1;
}
void pfc_set_chi(void* h, int a, int b, double chi) {
  auto* s = static_cast<System*>(h);
  const int M = s->nmon();
  s->chi[a * M + b] = chi;
  s->chi[b * M + a] = chi;
}
// Multiblock with chain_grid already applied: begin (nblocks + 1, 1-based), ds and b per block
int pfc_add_multiblock(void* h, int nblocks, const int* mon, const double* b, const double* ds, const int* begin,
                       double Nref, double phi) {
  auto* s = static_cast<System*>(h);
  Species sp;
  sp.kind = 0;
  sp.mon.assign(mon, mon + nblocks);
  sp.b.assign(b, b + nblocks);
  sp.ds.assign(ds, ds + nblocks);
  sp.begin.assign(begin, begin + nblocks + 1);
  sp.Ns = begin[nblocks] - 1;
  sp.Nref = Nref;
  sp.phi = phi;
  s->species.push_back(std::move(sp));
  return (int)s->species.size() - 1;
}
int pfc_add_point(void* h, int mon, double phi) {
  auto* s = static_cast<System*>(h);
  Species sp;
  sp.kind = 1;
  sp.mon = {mon};
  sp.Nref = s->vol[mon];
  sp.phi = phi;
  s->species.push_back(std::move(sp));
  return (int)s->species.size() - 1;
}
void pfc_set_field(void* h, int mon, const double* w) {
  auto* s = static_cast<System*>(h);
  std::memcpy(s->w[mon].data(), w, sizeof(double) * s->ng);
}
// kind: 0 field, 1 density, 2 residual, 3 potential
void pfc_get_grid(void* h, int kind, int mon, double* out) {
  auto* s = static_cast<System*>(h);
  const auto& g = kind == 0 ? s->w : kind == 1 ? s->rho : kind == 2 ? s->res : s->pot;
  std::memcpy(out, g[mon].data(), sizeof(double) * s->ng);
}
void pfc_residuals(void* h) { static_cast<System*>(h)->residuals(); }
double pfc_field_error(void* h) { return static_cast<System*>(h)->field_error(); }
double pfc_free_energy(void* h) { return static_cast<System*>(h)->free_energy(); }
double pfc_species_q(void* h, int isp) { return static_cast<System*>(h)->species[isp].Q; }
// propagate! nsteps RK2 steps of (w, vol, b, ds) from qin
void pfc_propagate(void* h, const double* w, double vol, double b, double ds, const double* qin, double* qout,
                   int nsteps) {
  auto* s = static_cast<System*>(h);
  std::vector<double> om(w, w + s->ng), a(qin, qin + s->ng), c(s->ng);
  s->update(om, vol, b, ds);
  for (int t = 0; t < nsteps; ++t) {
    s->propagate(a.data(), c.data());
    std::swap(a, c);
  }
  std::memcpy(qout, a.data(), sizeof(double) * s->ng);
}
void pfc_anderson_setup(void* h, int nhist) { static_cast<System*>(h)->anderson_setup(nhist); }
int pfc_anderson_step(void* h) { return static_cast<System*>(h)->anderson_step(); }

}  // extern "C"
