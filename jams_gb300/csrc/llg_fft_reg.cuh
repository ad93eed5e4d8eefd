// Register FFT passes for power-of-two lines, 16 <= N <= 1024, single
// precision (llg_dipole.cu takes them for every such axis of an FP32 grid;
// other lengths and the FP64 form use the shared-memory Stockham passes of
// llg_fft.cuh).
//
// A line of N = E T points is held by T threads, E points each.  With
// n = t + T e and k = k1 + E k2 (t, k2 < T; e, k1 < E):
//   X[k1 + E k2] = sum_t W_T^{t k2} W_N^{t k1} sum_e x[t + T e] W_E^{e k1}
// (the two-factor Cooley-Tukey split): thread t loads x[t + T e] for every e
// straight from global memory into registers, transforms them over e (an
// E-point radix-2 Stockham FFT in registers, every index and twiddle
// position a compile-time constant), multiplies by W_N^{t k1}, and writes the E results
// to shared memory; after one barrier each thread takes E / T of the k1 and
// transforms over t (a T-point FFT in registers), holding X[k1 + E k2] for
// every k2.  One shared-memory round trip per point instead of two per
// Stockham stage, and no run-time index division.
//
// Thread layouts: the strided complex pass keeps the G = 256 / T lines of a
// CTA fastest across threads (consecutive lines are consecutive in global
// memory); the real passes keep the T threads of a line fastest (a line's
// points are consecutive).  The real passes are "two for one" as in
// llg_fft.cuh.  Twiddles come from the pass's table W_N^j in shared memory.
#pragma once

#include "llg_fft.cuh"

namespace jams_llg {

constexpr int kFftRegMin = 16, kFftRegMax = 1024;

template <int N>
struct RegShape;
template <>
struct RegShape<16> {
  static constexpr int E = 4, T = 4;
};
template <>
struct RegShape<32> {
  static constexpr int E = 8, T = 4;
};
template <>
struct RegShape<64> {
  static constexpr int E = 8, T = 8;
};
template <>
struct RegShape<128> {
  static constexpr int E = 16, T = 8;
};
template <>
struct RegShape<256> {
  static constexpr int E = 16, T = 16;
};
template <>
struct RegShape<512> {
  static constexpr int E = 32, T = 16;
};
template <>
struct RegShape<1024> {
  static constexpr int E = 32, T = 32;
};


__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// W_N^t from the table, conjugated for the inverse transform (INV is a
// compile-time direction, so the sign folds into the arithmetic)
template <bool INV>
__device__ __forceinline__ float2 reg_twiddle(const float2* tws, int t) {
  const float2 w = tws[t];
  return INV ? make_float2(w.x, -w.y) : w;
}

// D-point DFT of v in registers, natural order in and out: self-sorting
// (Stockham) radix-2 stages, one template instance per stage so that every
// register index and twiddle position is a compile-time constant.  Stage
// Ns (1, 2, 4, .. D/2) maps butterfly j < D/2, k = j mod Ns, as
//   b[(j / Ns) 2 Ns + k]      = a[j] + W_{2Ns}^k a[j + D/2]
//   b[(j / Ns) 2 Ns + k + Ns] = a[j] - W_{2Ns}^k a[j + D/2]
// with W_{2Ns}^k = W_N^{k N / 2Ns} from the table (-i forward, +i inverse
// at k = Ns / 2, needing no table).
template <int D, int N, bool INV, int NS>
struct RegStage {
  __device__ __forceinline__ static void run(float2 (&a)[D], const float2* tws) {
    if constexpr (NS < D) {
      float2 b[D];
#pragma unroll
      for (int j = 0; j < D / 2; ++j) {
        const int k = j % NS, o = (j / NS) * 2 * NS + k;
        const float2 v0 = a[j];
        float2 v1 = a[j + D / 2];
        if (k != 0) {
          if (2 * k == NS)
            v1 = INV ? make_float2(-v1.y, v1.x) : make_float2(v1.y, -v1.x);
          else
            v1 = cmul(v1, reg_twiddle<INV>(tws, k * (N / (2 * NS))));
        }
        b[o] = c_add(v0, v1);
        b[o + NS] = c_sub(v0, v1);
      }
      RegStage<D, N, INV, 2 * NS>::run(b, tws);
#pragma unroll
      for (int i = 0; i < D; ++i) a[i] = b[i];
    }
  }
};

template <int D, int N, bool INV>
__device__ __forceinline__ void reg_dft(float2 (&v)[D], const float2* tws) {
  RegStage<D, N, INV, 1>::run(v, tws);
}

// the first factor: v[e] = x[t + T e] -> W_N^{t k1} sum_e x[t + T e] W_E^{e k1}
template <int N, bool INV>
__device__ __forceinline__ void reg_first(float2 (&v)[RegShape<N>::E], int t, const float2* tws) {
  constexpr int E = RegShape<N>::E;
  reg_dft<E, N, INV>(v, tws);
#pragma unroll
  for (int k1 = 1; k1 < E; ++k1) v[k1] = cmul(v[k1], reg_twiddle<INV>(tws, t * k1));
}

// shared-memory bytes of a register pass (twiddle table + exchange)
template <int N>
constexpr size_t reg_pass_smem() {
  return (size_t)(N + 256 * RegShape<N>::E) * sizeof(float2);
}
template <int N>
constexpr size_t reg_real_smem() {
  constexpr int E = RegShape<N>::E, T = RegShape<N>::T, G = 256 / T;
  constexpr int LS = T * (E + 1) > N + 1 ? T * (E + 1) : N + 1;
  return (size_t)(N + G * LS) * sizeof(float2);
}

// complex pass along an axis whose elements are `stride` apart: CTA b takes
// lines i0 .. i0 + G - 1 of outer block o (b = o * chunks + i0 / G,
// dchunks.d = chunks); in place.  At 128 and 256 points three CTAs per SM
// (80 registers, a 20-32 B spill) beat two without the spill: 1.11 against
// 1.21 ms per bcc 256^3 dipole evaluation.  Other lengths take no minimum
// (0): at 64 points a minimum raised the registers from 48 to 61 and made
// the pass slower.
template <int N, bool INV>
__global__ void __launch_bounds__(256, (N == 128 || N == 256) ? 3 : 0) fft_pass_reg(float2* __restrict__ g, int stride, const FastDiv dchunks,
                                                   const float2* __restrict__ tw) {
  constexpr int E = RegShape<N>::E, T = RegShape<N>::T, G = 256 / T;
  extern __shared__ unsigned char fft_smem[];
  float2* tws = reinterpret_cast<float2*>(fft_smem);
  float2* ex = tws + N;   // [k1][t][l]
  fft_prologue(tws, tw, N);
  const int l = threadIdx.x % G, t = threadIdx.x / G;
  const int o = (int)fdiv(blockIdx.x, dchunks);
  const int i0 = (int)(blockIdx.x - (uint32_t)o * dchunks.d) * G;
  const bool valid = i0 + l < stride;
  float2* line = g + (int64_t)o * N * stride + i0 + l;
  const int64_t st = stride;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = valid ? line[(t + T * e) * st] : make_float2(0.f, 0.f);
  __syncthreads();
  reg_first<N, INV>(v, t, tws);
#pragma unroll
  for (int k1 = 0; k1 < E; ++k1) ex[(k1 * T + t) * G + l] = v[k1];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E / T; ++i) {
    const int k1 = t + T * i;
    float2 u[T];
#pragma unroll
    for (int tt = 0; tt < T; ++tt) u[tt] = ex[(k1 * T + tt) * G + l];
    reg_dft<T, N, INV>(u, tws);
    if (valid) {
#pragma unroll
      for (int k2 = 0; k2 < T; ++k2) line[(k1 + E * k2) * st] = u[k2];
    }
  }
}

// The real passes reach their lines through the source's and sink's line
// accessors: line(f, o) is a pointer to point 0 of the line (null for a
// line in the padding), point p sits at line[p * step()] for p < length(),
// and the rest of the line is zero padding.  They pair their lines in one of
// two ways.  Consecutive lines (SITES false): pair c is lines 2c and 2c + 1.
// Basis-site pairs (SITES true, an even number of fields): pair c = fp * O
// + o is position o of fields 2 fp and 2 fp + 1, which the spin planes hold
// side by side (two basis sites of one component), so that one aligned
// 8-byte access moves both.
struct RealPair {
  int fa, fb, o;      // fields and position before the axis
  int64_t la, lb;     // line indices into the half spectrum
  bool va, vb;
};

template <bool SITES>
__device__ __forceinline__ RealPair real_pair(int c, int nlines, const FastDiv& dO) {
  RealPair r;
  const int O = (int)dO.d;
  if constexpr (SITES) {
    const int fp = (int)fdiv((uint32_t)c, dO);
    r.o = c - fp * O;
    r.fa = 2 * fp;
    r.fb = 2 * fp + 1;
    r.la = (int64_t)r.fa * O + r.o;
    r.lb = r.la + O;
    r.va = r.vb = r.la < nlines;
  } else {
    const int la = 2 * c;
    r.va = la < nlines;
    r.vb = la + 1 < nlines;
    const LinePair q = line_pair(r.va ? la : 0, dO);
    r.fa = q.fa;
    r.fb = q.fb;
    r.o = q.oa;   // line la + 1 is (fb, ob): ob = oa + 1 unless it wraps to the next field
    r.la = la;
    r.lb = la + 1;
  }
  return r;
}

// forward real pass ("two for one", see llg_fft.cuh): CTA b takes pairs
// 256 / T * b ..; outputs 0 .. N/2 of real line l go to k[l (N/2+1) + q]
template <int N, bool SITES, class Src>
__global__ void __launch_bounds__(256) fft_real_forward_reg(const __grid_constant__ Src src, int nlines, int npairs,
                                                           const FastDiv dO, const float2* __restrict__ tw,
                                                           float2* __restrict__ k) {
  constexpr int E = RegShape<N>::E, T = RegShape<N>::T, G = 256 / T, NH = N / 2 + 1;
  constexpr int LS = T * (E + 1) > N + 1 ? T * (E + 1) : N + 1;
  extern __shared__ unsigned char fft_smem[];
  float2* tws = reinterpret_cast<float2*>(fft_smem);
  const int t = threadIdx.x % T, l = threadIdx.x / T;
  float2* ex = tws + N + l * LS;   // this line: [t][k1] rows of E + 1, then the spectrum
  fft_prologue(tws, tw, N);
  const int c = blockIdx.x * G + l;
  const RealPair q = real_pair<SITES>(c < npairs ? c : 0, nlines, dO);
  const bool va = c < npairs && q.va, vb = c < npairs && q.vb;
  const int len = src.length(), sp = src.step();
  const float* pa = va ? src.line(q.fa, q.o) : nullptr;
  const float* pb = vb && !SITES ? src.line(q.fb, q.fb == q.fa ? q.o + 1 : 0) : nullptr;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int p = t + T * e;
    const bool in = p < len;
    if constexpr (SITES) {
      v[e] = pa && in ? __ldg(reinterpret_cast<const float2*>(pa + p * sp)) : make_float2(0.f, 0.f);
    } else {
      v[e] = make_float2(pa && in ? __ldg(pa + p * sp) : 0.f, pb && in ? __ldg(pb + p * sp) : 0.f);
    }
  }
  __syncthreads();
  reg_first<N, false>(v, t, tws);
#pragma unroll
  for (int k1 = 0; k1 < E; ++k1) ex[t * (E + 1) + k1] = v[k1];
  __syncthreads();
  float2 z[E / T][T];
#pragma unroll
  for (int i = 0; i < E / T; ++i) {
    const int k1 = t + T * i;
#pragma unroll
    for (int tt = 0; tt < T; ++tt) z[i][tt] = ex[tt * (E + 1) + k1];
    reg_dft<T, N, false>(z[i], tws);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E / T; ++i)
#pragma unroll
    for (int k2 = 0; k2 < T; ++k2) ex[t + T * i + E * k2] = z[i][k2];
  __syncthreads();
  if (!va) return;
  for (int qq = t; qq < NH; qq += T) {
    const float2 a = ex[qq], b = ex[qq == 0 ? 0 : N - qq];
    k[q.la * NH + qq] = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
    if (vb) k[q.lb * NH + qq] = make_float2(0.5f * (a.y + b.y), 0.5f * (b.x - a.x));
  }
}

// inverse real pass ("two for one"): the half spectra of the pair's lines
// completed by Hermitian symmetry, transformed as A + i B, the real part to
// the first line and the imaginary part to the second through sink
template <int N, bool SITES, class Sink>
__global__ void __launch_bounds__(256) fft_real_inverse_reg(const float2* __restrict__ k, int nlines, int npairs,
                                                           const FastDiv dO, const float2* __restrict__ tw,
                                                           const __grid_constant__ Sink sink) {
  constexpr int E = RegShape<N>::E, T = RegShape<N>::T, G = 256 / T, NH = N / 2 + 1;
  constexpr int LS = T * (E + 1) > N + 1 ? T * (E + 1) : N + 1;
  extern __shared__ unsigned char fft_smem[];
  float2* tws = reinterpret_cast<float2*>(fft_smem);
  const int t = threadIdx.x % T, l = threadIdx.x / T;
  float2* ex = tws + N + l * LS;
  fft_prologue(tws, tw, N);
  const int c = blockIdx.x * G + l;
  const RealPair q = real_pair<SITES>(c < npairs ? c : 0, nlines, dO);
  const bool va = c < npairs && q.va, vb = c < npairs && q.vb;
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int p = t + T * e;
    const bool mirror = p >= NH;
    const int off = mirror ? N - p : p;
    float2 xa = va ? k[q.la * NH + off] : make_float2(0.f, 0.f);
    float2 xb = vb ? k[q.lb * NH + off] : make_float2(0.f, 0.f);
    if (mirror) {
      xa.y = -xa.y;
      xb.y = -xb.y;
    }
    if (p == 0 || 2 * p == N) xa.y = xb.y = 0.f;   // X[0], X[N/2]: real
    v[e] = make_float2(xa.x - xb.y, xa.y + xb.x);   // A + i B
  }
  __syncthreads();
  reg_first<N, true>(v, t, tws);
#pragma unroll
  for (int k1 = 0; k1 < E; ++k1) ex[t * (E + 1) + k1] = v[k1];
  __syncthreads();
  const int len = sink.length(), sp = sink.step();
  float* pa = va ? sink.line(q.fa, q.o) : nullptr;
  float* pb = vb ? (SITES ? (pa ? pa + 1 : nullptr) : sink.line(q.fb, q.fb == q.fa ? q.o + 1 : 0)) : nullptr;
  const float ma = va ? sink.moment(q.fa) : 0.f, mb = vb ? sink.moment(q.fb) : 0.f;
#pragma unroll
  for (int i = 0; i < E / T; ++i) {
    const int k1 = t + T * i;
    float2 u[T];
#pragma unroll
    for (int tt = 0; tt < T; ++tt) u[tt] = ex[tt * (E + 1) + k1];
    reg_dft<T, N, true>(u, tws);
#pragma unroll
    for (int k2 = 0; k2 < T; ++k2) {
      const int p = k1 + E * k2;
      if (p >= len) continue;
      if constexpr (SITES) {
        if (pa) *reinterpret_cast<float2*>(pa + p * sp) = make_float2(ma * u[k2].x, mb * u[k2].y);
      } else {
        if (pa) pa[p * sp] = ma * u[k2].x;
        if (pb) pb[p * sp] = mb * u[k2].y;
      }
    }
  }
}

}  // namespace jams_llg
