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
// (every later axis has one cell).  The forward real pass reads its line
// through a source functor (the spin planes, fusing the scatter onto the
// grid, or a real grid), transforms it as a complex line with zero imaginary
// part and keeps outputs 0 .. N/2.  The inverse real pass rebuilds the full
// spectrum by Hermitian symmetry, transforms it and hands the real parts to
// a sink functor (the field planes, fusing the gather).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace jams_llg {

constexpr int kFftMaxStages = 30;
constexpr int kFftThreads = 256;

struct FftPlan1D {
  int n;
  int nstages;
  int radix[kFftMaxStages];
};

// radices of n: 4 while more than 4 remains, then 4, 2, 3, 5, 7 and the
// remaining primes
inline FftPlan1D fft_plan(int n) {
  FftPlan1D p{};
  p.n = n;
  int m = n;
  while (m % 4 == 0 && m > 4) {
    p.radix[p.nstages++] = 4;
    m /= 4;
  }
  for (int r : {4, 2, 3, 5, 7})
    while (m % r == 0) {
      p.radix[p.nstages++] = r;
      m /= r;
    }
  for (int r = 11; m > 1; r += 2)
    while (m % r == 0) {
      p.radix[p.nstages++] = r;
      m /= r;
    }
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
__device__ __forceinline__ C twiddle(const C* __restrict__ tw, int t, bool inverse) {
  const C w = tw[t];
  return inverse ? CT<C>::make(w.x, -w.y) : w;
}

// transforms `nlines` lines of length P.n held in shared memory at a, b the
// same size; every thread of the CTA takes part.  Element e of line l sits at
// l * P.n + e (INTER false: consecutive threads take consecutive butterflies
// of one line) or at e * nlines + l (INTER true: the lines interleaved,
// consecutive threads take the same butterfly of consecutive lines, so that
// neither the strided loads nor the butterflies conflict on shared-memory
// banks).  Returns the buffer that holds the result.
template <class C, bool INTER>
__device__ C* fft_lines(C* a, C* b, int nlines, const FftPlan1D& P, const C* __restrict__ tw, bool inverse) {
  const int n = P.n;
  const int tid = threadIdx.x;
  const int es = INTER ? nlines : 1;     // element stride within a line
  int Ns = 1;
  for (int s = 0; s < P.nstages; ++s) {
    const int R = P.radix[s];
    const int m = n / R;
    const int st = n / (Ns * R);
    const int items = nlines * m;
    for (int it = tid; it < items; it += blockDim.x) {
      int line, j;
      if (INTER) {
        j = it / nlines;
        line = it - j * nlines;
      } else {
        line = it / m;
        j = it - line * m;
      }
      const C* in = a + (INTER ? line : line * n);
      C* out = b + (INTER ? line : line * n);
      const int k = j % Ns;
      const int dst = (j / Ns) * Ns * R + k;
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
        // any other radix: each output from all R inputs, the twiddle and
        // the R-point DFT factor as one power of W_N
        for (int q = 0; q < R; ++q) {
          typename CT<C>::Real ax = 0, ay = 0;
          for (int r = 0; r < R; ++r) {
            const int t = (k * r * st + ((r * q) % R) * m) % n;
            const C w = twiddle(tw, t, inverse);
            const C v = in[(j + r * m) * es];
            ax += v.x * w.x - v.y * w.y;
            ay += v.x * w.y + v.y * w.x;
          }
          out[(dst + q * Ns) * es] = CT<C>::make(ax, ay);
        }
      }
    }
    __syncthreads();
    C* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// lines per CTA for length n: at most `elems` complex values per buffer
__host__ __device__ inline int fft_batch(int n, int elems) {
  const int g = elems / n;
  return g < 1 ? 1 : (g > 256 ? 256 : g);
}

// complex pass along an axis whose elements are `stride` apart (stride > 1:
// the lines of one outer block are its `stride` consecutive inner offsets;
// a CTA takes `G` consecutive ones) or contiguous (stride == 1: a CTA takes
// G consecutive lines).  In place.
template <class C>
__global__ void __launch_bounds__(kFftThreads) fft_pass(C* __restrict__ g, int64_t outer, int stride, int G,
                                                        const __grid_constant__ FftPlan1D P, const C* __restrict__ tw,
                                                        bool inverse) {
  extern __shared__ unsigned char fft_smem[];
  C* a = reinterpret_cast<C*>(fft_smem);
  C* b = a + (size_t)G * P.n;
  const int n = P.n;
  int64_t base;
  int lines;
  if (stride == 1) {
    const int64_t l0 = (int64_t)blockIdx.x * G;
    lines = (int)min((int64_t)G, outer - l0);
    base = l0 * n;
    for (int e = threadIdx.x; e < lines * n; e += blockDim.x) a[e] = g[base + e];
  } else {
    const int64_t chunks = (stride + G - 1) / G;
    const int64_t o = blockIdx.x / chunks;
    const int i0 = (int)(blockIdx.x % chunks) * G;
    lines = min(G, stride - i0);
    base = o * (int64_t)n * stride + i0;
    // element el of the `lines` inner offsets: one contiguous run of global
    // memory, stored interleaved (a[el * lines + l])
    for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
      const int el = e / lines, l = e - el * lines;
      a[e] = g[base + (int64_t)el * stride + l];
    }
  }
  __syncthreads();
  if (stride == 1) {
    const C* r = fft_lines<C, false>(a, b, lines, P, tw, inverse);
    for (int e = threadIdx.x; e < lines * n; e += blockDim.x) g[base + e] = r[e];
  } else {
    const C* r = fft_lines<C, true>(a, b, lines, P, tw, inverse);
    for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
      const int el = e / lines, l = e - el * lines;
      g[base + (int64_t)el * stride + l] = r[e];
    }
  }
}

// forward pass along the real axis: line l = (field f, position o before the
// axis); src(f, o, p) gives the real value at position p of the line.  Writes
// outputs 0 .. N/2 of every line to k[(f * O + o) * (N/2 + 1) + q].
template <class C, class Src>
__global__ void __launch_bounds__(kFftThreads) fft_real_forward(const __grid_constant__ Src src, int64_t nlines,
                                                                int64_t O, int G, const __grid_constant__ FftPlan1D P,
                                                                const C* __restrict__ tw, C* __restrict__ k) {
  extern __shared__ unsigned char fft_smem[];
  C* a = reinterpret_cast<C*>(fft_smem);
  C* b = a + (size_t)G * P.n;
  const int n = P.n, nh = n / 2 + 1;
  const int64_t l0 = (int64_t)blockIdx.x * G;
  const int lines = (int)min((int64_t)G, nlines - l0);
  for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
    const int l = e / n, p = e - l * n;
    const int64_t line = l0 + l;
    a[e] = CT<C>::make(src(line / O, line % O, p), 0);
  }
  __syncthreads();
  const C* r = fft_lines<C, false>(a, b, lines, P, tw, false);
  for (int e = threadIdx.x; e < lines * nh; e += blockDim.x) {
    const int l = e / nh, q = e - l * nh;
    k[(l0 + l) * nh + q] = r[l * n + q];
  }
}

// inverse pass along the real axis: the half spectrum of line l at
// k[l * (N/2 + 1) ..], completed by X[N - q] = conj(X[q]); sink(f, o, p, x)
// receives the real part of output p
template <class C, class Sink>
__global__ void __launch_bounds__(kFftThreads) fft_real_inverse(const C* __restrict__ k, int64_t nlines, int64_t O,
                                                                int G, const __grid_constant__ FftPlan1D P,
                                                                const C* __restrict__ tw, const __grid_constant__ Sink sink) {
  extern __shared__ unsigned char fft_smem[];
  C* a = reinterpret_cast<C*>(fft_smem);
  C* b = a + (size_t)G * P.n;
  const int n = P.n, nh = n / 2 + 1;
  const int64_t l0 = (int64_t)blockIdx.x * G;
  const int lines = (int)min((int64_t)G, nlines - l0);
  for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
    const int l = e / n, p = e - l * n;
    const int64_t row = (l0 + l) * nh;
    if (p < nh) {
      a[e] = k[row + p];
    } else {
      const C v = k[row + (n - p)];
      a[e] = CT<C>::make(v.x, -v.y);
    }
  }
  __syncthreads();
  const C* r = fft_lines<C, false>(a, b, lines, P, tw, true);
  for (int e = threadIdx.x; e < lines * n; e += blockDim.x) {
    const int l = e / n, p = e - l * n;
    const int64_t line = l0 + l;
    sink(line / O, line % O, p, r[e].x);
  }
}

}  // namespace jams_llg
