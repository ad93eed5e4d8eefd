// Hand-written FFTs for the dipole-dipole convolution (llg_dipole.cu): the
// transforms of a 3-D grid of M0 x M1 x M2 cells, several real fields, with
// the half spectrum kept along the last axis longer than one cell (axis h),
// the layout a batched real-to-complex transform produces (row-major over the
// M axes with M_h replaced by M_h / 2 + 1).
//
// Each axis is one kernel pass over lines of the grid: a CTA loads a batch of
// lines into shared memory, transforms them there and writes them back.  A
// line of length N is transformed by the self-sorting (Stockham) mixed-radix
// algorithm: N = R_1 R_2 ... R_s (radix 4 first, then 2, 3, 5, 7 and any
// other prime), and stage s maps butterfly j (of N / R) with Ns = R_1 ...
// R_{s-1} as
//   v_r = in[j + r N / R] W_N^{(j mod Ns) r N / (Ns R)},  r < R
//   out[(j / Ns) Ns R + (j mod Ns) + k Ns] = sum_r v_r W_R^{r k},  k < R
// (Govindaraju et al., "High performance discrete Fourier transforms on
// graphics processors", SC 2008), ping-ponging between two shared-memory
// buffers.  W_N^t = exp(-2 pi i t / N) comes from a table computed on the host
// in double precision; the inverse transform uses its conjugate.  Neither
// transform is normalised.
//
// The real axis h is contiguous in both the real grid and the half spectrum
// (every later axis has one cell).  The real passes take two real lines a, b
// as one complex line z = a + i b ("two for one"): the forward pass reads
// them through a source functor (the spin planes, fusing the scatter onto
// the grid, or a real grid), transforms z and separates
//   A[q] = (Z[q] + conj Z[N-q]) / 2,  B[q] = (Z[q] - conj Z[N-q]) / 2i,
// keeping q = 0 .. N/2.  The inverse pass completes each half spectrum by
// Hermitian symmetry (X[N-q] = conj X[q], the imaginary parts of X[0] and
// X[N/2] dropped as a complex-to-real transform does), transforms A + i B
// and hands the real part (line a) and the imaginary part (line b) to a sink
// functor (the field planes, fusing the gather).
//
// Every pass keeps its twiddle table in shared memory, and is launched with
// programmatic stream serialisation where the caller asks: it loads the
// table, then waits for the previous kernel in the stream to complete before
// it touches the grid.
//
// Index arithmetic is 32-bit (the host keeps every grid below 2^31 values)
// and divides by run-time constants through multiply-high reciprocals
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): for 1 <= d < 2^31, l = ceil(log2 d),
// mul = floor(2^32 (2^l - d) / d) + 1, and x / d = (umulhi(x, mul) + x) >> l
// for every x < 2^31.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace jams_llg {

constexpr int kFftMaxStages = 16;
constexpr int kFftThreads = 256;

struct FastDiv {
  uint32_t d = 1, mul = 1;
  int shift = 0;
};

inline FastDiv fast_div(uint32_t d) {
  FastDiv f;
  f.d = d;
  int l = 0;
  while ((1ull << l) < d) ++l;
  f.shift = l;
  f.mul = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t x, const FastDiv& f) { return (__umulhi(x, f.mul) + x) >> f.shift; }

// one Stockham stage: radix R, m = n / R butterflies, Ns = product of the
// earlier radices, st = n / (Ns R) the twiddle step
struct FftStage {
  int R, m, Ns, st;
  FastDiv dm, dNs;
};

struct FftPlan1D {
  int n = 1;
  int nstages = 0;
  FastDiv dn, dnh;   // n and n / 2 + 1
  FftStage stage[kFftMaxStages];
};

// radices of n: 4 while more than 4 remains, then 4, 2, 3, 5, 7 and the
// remaining primes (n <= 4842 needs at most 12 stages)
inline FftPlan1D fft_plan(int n) {
  FftPlan1D p;
  p.n = n;
  p.dn = fast_div((uint32_t)n);
  p.dnh = fast_div((uint32_t)(n / 2 + 1));
  int rad[kFftMaxStages], ns = 0;
  int m = n;
  while (m % 4 == 0 && m > 4 && ns < kFftMaxStages) {
    rad[ns++] = 4;
    m /= 4;
  }
  for (int r : {4, 2, 3, 5, 7})
    while (m % r == 0 && ns < kFftMaxStages) {
      rad[ns++] = r;
      m /= r;
    }
  for (int r = 11; m > 1 && ns < kFftMaxStages; r += 2)
    while (m % r == 0 && ns < kFftMaxStages) {
      rad[ns++] = r;
      m /= r;
    }
  int Ns = 1;
  for (int s = 0; s < ns; ++s) {
    FftStage& S = p.stage[s];
    S.R = rad[s];
    S.m = n / S.R;
    S.Ns = Ns;
    S.st = n / (Ns * S.R);
    S.dm = fast_div((uint32_t)S.m);
    S.dNs = fast_div((uint32_t)Ns);
    Ns *= S.R;
  }
  p.nstages = ns;
  return p;
}

template <class C>
struct CT;
template <>
struct CT<float2> {
  using Real = float;
  __device__ static float2 make(float x, float y) { return make_float2(x, y); }
};
template <>
struct CT<double2> {
  using Real = double;
  __device__ static double2 make(double x, double y) { return make_double2(x, y); }
};

template <class C>
__device__ __forceinline__ C cmul(C a, C b) {
  return CT<C>::make(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// W_N^t (inverse: its conjugate) from the table of exp(-2 pi i t / N)
template <class C>
__device__ __forceinline__ C twiddle(const C* tw, int t, bool inverse) {
  const C w = tw[t];
  return inverse ? CT<C>::make(w.x, -w.y) : w;
}

// the twiddle table into shared memory; then, under programmatic dependent
// launch, let the next kernel be scheduled and wait for the previous one to
// complete (without the launch attribute both return at once)
template <class C>
__device__ __forceinline__ void fft_prologue(C* tws, const C* __restrict__ tw, int n) {
  for (int t = threadIdx.x; t < n; t += blockDim.x) tws[t] = __ldg(tw + t);
  asm volatile("griddepcontrol.launch_dependents;");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// transforms `nl` lines of length P.n held in shared memory at a, b the same
// size; every thread of the CTA takes part.  Element e of line l sits at
// l * P.n + e (INTER false: consecutive threads take consecutive butterflies
// of one line) or at e * nl + l (INTER true: the lines interleaved,
// consecutive threads take the same butterfly of consecutive lines, so that
// neither the strided global loads nor the butterflies conflict on
// shared-memory banks; dnl divides by nl).  Returns the buffer that holds the
// result.
template <class C, bool INTER>
__device__ C* fft_lines(C* a, C* b, int nl, const FastDiv& dnl, const FftPlan1D& P, const C* tw, bool inverse) {
  const int n = P.n;
  const int es = INTER ? nl : 1;   // element stride within a line
  for (int s = 0; s < P.nstages; ++s) {
    const FftStage& S = P.stage[s];
    const int R = S.R, m = S.m, Ns = S.Ns, st = S.st;
    const int items = nl * m;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      int line, j;
      if (INTER) {
        j = (int)fdiv((uint32_t)it, dnl);
        line = it - j * nl;
      } else {
        line = (int)fdiv((uint32_t)it, S.dm);
        j = it - line * m;
      }
      const C* in = a + (INTER ? line : line * n);
      C* out = b + (INTER ? line : line * n);
      const int jq = (int)fdiv((uint32_t)j, S.dNs);
      const int k = j - jq * Ns;
      const int dst = jq * Ns * R + k;
      if (R == 2) {
        const C v0 = in[j * es];
        const C v1 = k ? cmul(in[(j + m) * es], twiddle(tw, k * st, inverse)) : in[(j + m) * es];
        out[dst * es] = CT<C>::make(v0.x + v1.x, v0.y + v1.y);
        out[(dst + Ns) * es] = CT<C>::make(v0.x - v1.x, v0.y - v1.y);
      } else if (R == 4) {
        const C v0 = in[j * es];
        C v1 = in[(j + m) * es], v2 = in[(j + 2 * m) * es], v3 = in[(j + 3 * m) * es];
        if (k) {
          v1 = cmul(v1, twiddle(tw, k * st, inverse));
          v2 = cmul(v2, twiddle(tw, 2 * k * st, inverse));
          v3 = cmul(v3, twiddle(tw, 3 * k * st, inverse));
        }
        const C s02 = CT<C>::make(v0.x + v2.x, v0.y + v2.y), d02 = CT<C>::make(v0.x - v2.x, v0.y - v2.y);
        const C s13 = CT<C>::make(v1.x + v3.x, v1.y + v3.y), d13 = CT<C>::make(v1.x - v3.x, v1.y - v3.y);
        // W_4 = -i forward, +i inverse: y1 = d02 -+ i d13, y3 = d02 +- i d13
        const C id13 = inverse ? CT<C>::make(-d13.y, d13.x) : CT<C>::make(d13.y, -d13.x);
        out[dst * es] = CT<C>::make(s02.x + s13.x, s02.y + s13.y);
        out[(dst + Ns) * es] = CT<C>::make(d02.x + id13.x, d02.y + id13.y);
        out[(dst + 2 * Ns) * es] = CT<C>::make(s02.x - s13.x, s02.y - s13.y);
        out[(dst + 3 * Ns) * es] = CT<C>::make(d02.x - id13.x, d02.y - id13.y);
      } else {
        // any other radix: output q from all R inputs, the twiddle and the
        // R-point DFT factor together as W_N^{r (k st + q m)} (R m = n)
        for (int q = 0; q < R; ++q) {
          typename CT<C>::Real ax = 0, ay = 0;
          const int step = k * st + q * m;   // < 2 n
          int t = 0;
          for (int r = 0; r < R; ++r) {
            const C w = twiddle(tw, t, inverse);
            const C v = in[(j + r * m) * es];
            ax += v.x * w.x - v.y * w.y;
            ay += v.x * w.y + v.y * w.x;
            t += step;
            while (t >= n) t -= n;
          }
          out[(dst + q * Ns) * es] = CT<C>::make(ax, ay);
        }
      }
    }
    __syncthreads();
    C* t = a;
    a = b;
    b = t;
  }
  return a;
}

// complex pass along an axis whose elements are `stride` (> 1) apart: the
// lines of one outer block are its `stride` consecutive inner offsets, a CTA
// takes G consecutive ones (dchunks.d = ceil(stride / G) CTAs per outer
// block), and element el of its lines is one contiguous run of global
// memory.  In place.
template <class C>
__global__ void __launch_bounds__(kFftThreads) fft_pass(C* __restrict__ g, int stride, int G, const FastDiv dG,
                                                        const FastDiv dchunks, const __grid_constant__ FftPlan1D P,
                                                        const C* __restrict__ tw, bool inverse) {
  extern __shared__ unsigned char fft_smem[];
  C* tws = reinterpret_cast<C*>(fft_smem);
  C* a = tws + P.n;
  C* b = a + G * P.n;
  const int n = P.n;
  fft_prologue(tws, tw, n);
  const int o = (int)fdiv(blockIdx.x, dchunks);
  const int i0 = (int)(blockIdx.x - (uint32_t)o * dchunks.d) * G;
  const int lines = min(G, stride - i0);
  const int64_t base = (int64_t)o * n * stride + i0;
  for (int e = threadIdx.x; e < G * n; e += blockDim.x) {
    const int el = (int)fdiv((uint32_t)e, dG), l = e - el * G;
    a[e] = l < lines ? g[base + (int64_t)el * stride + l] : CT<C>::make(0, 0);
  }
  __syncthreads();
  const C* r = fft_lines<C, true>(a, b, G, dG, P, tws, inverse);
  for (int e = threadIdx.x; e < G * n; e += blockDim.x) {
    const int el = (int)fdiv((uint32_t)e, dG), l = e - el * G;
    if (l < lines) g[base + (int64_t)el * stride + l] = r[e];
  }
}

// (field, position before the axis) of real line l = f * O + o, and of l + 1
struct LinePair {
  int fa, oa, fb, ob;
};
__device__ __forceinline__ LinePair line_pair(int la, const FastDiv& dO) {
  LinePair q;
  q.fa = (int)fdiv((uint32_t)la, dO);
  q.oa = la - q.fa * (int)dO.d;
  const bool wrap = q.oa + 1 == (int)dO.d;
  q.fb = wrap ? q.fa + 1 : q.fa;
  q.ob = wrap ? 0 : q.oa + 1;
  return q;
}

// forward pass along the real axis over nlines real lines, l = f * O + o
// (field f, position o before the axis, dO.d = O); src(f, o, p) gives the
// real value at position p of a line.  A CTA takes G line pairs (2 c, 2 c + 1)
// and writes outputs 0 .. N/2 of every line to k[l * (N/2 + 1) + q].
template <class C, class Src>
__global__ void __launch_bounds__(kFftThreads) fft_real_forward(const __grid_constant__ Src src, int nlines,
                                                                const FastDiv dO, int G,
                                                                const __grid_constant__ FftPlan1D P,
                                                                const C* __restrict__ tw, C* __restrict__ k) {
  extern __shared__ unsigned char fft_smem[];
  C* tws = reinterpret_cast<C*>(fft_smem);
  C* a = tws + P.n;
  C* b = a + G * P.n;
  const int n = P.n, nh = n / 2 + 1;
  fft_prologue(tws, tw, n);
  const int c0 = blockIdx.x * G;
  const int npairs = (nlines + 1) / 2;
  const int lines = min(G, npairs - c0);
  for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
    const int c = (int)fdiv((uint32_t)e, P.dn), p = e - c * n;
    const int la = 2 * (c0 + c);
    const LinePair q = line_pair(la, dO);
    const auto va = src(q.fa, q.oa, p);
    const auto vb = la + 1 < nlines ? src(q.fb, q.ob, p) : decltype(va)(0);
    a[e] = CT<C>::make(va, vb);
  }
  __syncthreads();
  const C* r = fft_lines<C, false>(a, b, lines, P.dn, P, tws, false);
  for (int e = threadIdx.x; e < lines * nh; e += blockDim.x) {
    const int c = (int)fdiv((uint32_t)e, P.dnh), q = e - c * nh;
    const C z = r[c * n + q], w = r[c * n + (q == 0 ? 0 : n - q)];
    const typename CT<C>::Real half = 0.5;
    const int64_t la = 2 * (int64_t)(c0 + c);
    k[la * nh + q] = CT<C>::make(half * (z.x + w.x), half * (z.y - w.y));
    if (la + 1 < nlines) k[(la + 1) * nh + q] = CT<C>::make(half * (z.y + w.y), half * (w.x - z.x));
  }
}

// inverse pass along the real axis: the half spectrum of real line l at
// k[l * (N/2 + 1) ..]; sink(f, o, p, x) receives output p of line l = f * O +
// o.  A CTA takes G line pairs.
template <class C, class Sink>
__global__ void __launch_bounds__(kFftThreads) fft_real_inverse(const C* __restrict__ k, int nlines,
                                                                const FastDiv dO, int G,
                                                                const __grid_constant__ FftPlan1D P,
                                                                const C* __restrict__ tw,
                                                                const __grid_constant__ Sink sink) {
  extern __shared__ unsigned char fft_smem[];
  C* tws = reinterpret_cast<C*>(fft_smem);
  C* a = tws + P.n;
  C* b = a + G * P.n;
  const int n = P.n, nh = n / 2 + 1;
  fft_prologue(tws, tw, n);
  const int c0 = blockIdx.x * G;
  const int npairs = (nlines + 1) / 2;
  const int lines = min(G, npairs - c0);
  for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
    const int c = (int)fdiv((uint32_t)e, P.dn), p = e - c * n;
    const int64_t la = 2 * (int64_t)(c0 + c);
    const bool mirror = p >= nh;
    const int64_t off = mirror ? n - p : p;
    const bool edge = p == 0 || 2 * p == n;   // X[0], X[N/2]: real
    C xa = k[la * nh + off];
    C xb = la + 1 < nlines ? k[(la + 1) * nh + off] : CT<C>::make(0, 0);
    if (mirror) {
      xa.y = -xa.y;
      xb.y = -xb.y;
    }
    if (edge) xa.y = xb.y = 0;
    a[e] = CT<C>::make(xa.x - xb.y, xa.y + xb.x);   // A + i B
  }
  __syncthreads();
  const C* r = fft_lines<C, false>(a, b, lines, P.dn, P, tws, true);
  for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
    const int c = (int)fdiv((uint32_t)e, P.dn), p = e - c * n;
    const int la = 2 * (c0 + c);
    const LinePair q = line_pair(la, dO);
    sink(q.fa, q.oa, p, r[e].x);
    if (la + 1 < nlines) sink(q.fb, q.ob, p, r[e].y);
  }
}

}  // namespace jams_llg
