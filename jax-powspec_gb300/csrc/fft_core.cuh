// Batched radix-8 Stockham FFTs on data resident in shared memory.
//
// Layout: element i of column c (one transform per column) sits at
// s[i * CP + c]; CP >= C is the row pitch.  A CTA transforms its C columns
// of length N together, one butterfly of 8 values per thread and stage.
// Lengths N = 8^a * {1, 2, 4} (64 .. 4096) use radix-8 stages and at most one
// radix-2 or radix-4 stage; the output is in natural order (Stockham).
//
// Stage with radix R, p = product of the previous radices: butterfly
// i in [0, N/R) with k = i mod p reads x[i + r N/R] (r < R), multiplies by
// exp(-2 pi i r k / (p R)), takes the R-point DFT and writes it to
// y[(i - k) R + k + r p].  Forward transform: exp(-2 pi i j k / N), as cuFFT
// and numpy.
#pragma once

#include <cuda_runtime.h>

namespace gbp {
namespace fft {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmi(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)

__device__ __forceinline__ void dft2(float2& a, float2& b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

__device__ __forceinline__ void dft4(float2* u) {
  const float2 a0 = cadd(u[0], u[2]), a1 = csub(u[0], u[2]);
  const float2 a2 = cadd(u[1], u[3]), a3 = cmi(csub(u[1], u[3]));
  u[0] = cadd(a0, a2);
  u[2] = csub(a0, a2);
  u[1] = cadd(a1, a3);
  u[3] = csub(a1, a3);
}

__device__ __forceinline__ void dft8(float2* u) {
  const float s = 0.70710678118654752440f;
  const float2 a0 = cadd(u[0], u[4]), a1 = csub(u[0], u[4]);
  const float2 a2 = cadd(u[2], u[6]), a3 = cmi(csub(u[2], u[6]));
  const float2 a4 = cadd(u[1], u[5]), a5 = csub(u[1], u[5]);
  const float2 a6 = cadd(u[3], u[7]), a7 = cmi(csub(u[3], u[7]));
  const float2 b0 = cadd(a0, a2), b2 = csub(a0, a2);
  const float2 b1 = cadd(a1, a3), b3 = csub(a1, a3);
  const float2 b4 = cadd(a4, a6), b6 = cmi(csub(a4, a6));
  const float2 t5 = cadd(a5, a7), t7 = csub(a5, a7);
  const float2 b5 = make_float2(s * (t5.x + t5.y), s * (t5.y - t5.x));    // * exp(-i pi/4)
  const float2 b7 = make_float2(s * (t7.y - t7.x), -s * (t7.x + t7.y));   // * exp(-3 i pi/4)
  u[0] = cadd(b0, b4);
  u[4] = csub(b0, b4);
  u[1] = cadd(b1, b5);
  u[5] = csub(b1, b5);
  u[2] = cadd(b2, b6);
  u[6] = csub(b2, b6);
  u[3] = cadd(b3, b7);
  u[7] = csub(b3, b7);
}

template <int N>
struct Radices {
  static constexpr int log2n = (N == 64) ? 6 : (N == 128) ? 7 : (N == 256) ? 8 : (N == 512) ? 9
                               : (N == 1024) ? 10 : (N == 2048) ? 11 : 12;
  static constexpr int n8 = log2n / 3;      // radix-8 stages
  static constexpr int tail = log2n % 3;    // 0, 1 (radix 2) or 2 (radix 4)
  static constexpr int stages = n8 + (tail ? 1 : 0);
};

// One Stockham stage over C columns.  nthreads threads, each owning
// butterflies b = tid, tid + nthreads, ... of the C * N / R in the stage.
// Every thread loads all its inputs before the barrier and stores after it.
template <int N, int R, int C, int CP, int NT>
__device__ __forceinline__ void stage(float2* s, const float2* __restrict__ tw, int p, int tid) {
  constexpr int NB = C * (N / R);          // butterflies in the stage
  constexpr int PER = (NB + NT - 1) / NT;  // per thread
  float2 u[PER][R];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int b = tid + q * NT;
    if (PER * NT == NB || b < NB) {
      const int col = b % C, i = b / C;
      const int k = i & (p - 1);
#pragma unroll
      for (int r = 0; r < R; ++r) u[q][r] = s[(i + r * (N / R)) * CP + col];
      if (p > 1) {
        const int step = N / (p * R);
#pragma unroll
        for (int r = 1; r < R; ++r) u[q][r] = cmul(u[q][r], __ldg(tw + ((r * k * step) & (N - 1))));
      }
      if constexpr (R == 8) dft8(u[q]);
      else if constexpr (R == 4) dft4(u[q]);
      else dft2(u[q][0], u[q][1]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int b = tid + q * NT;
    if (PER * NT == NB || b < NB) {
      const int col = b % C, i = b / C;
      const int k = i & (p - 1);
      const int j = (i - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) s[(j + r * p) * CP + col] = u[q][r];
    }
  }
  __syncthreads();
}

// Full forward FFT of the C columns (natural-order output, in place).
template <int N, int C, int CP, int NT>
__device__ __forceinline__ void fft_columns(float2* s, const float2* __restrict__ tw, int tid) {
  using RD = Radices<N>;
  int p = 1;
#pragma unroll
  for (int st = 0; st < RD::n8; ++st) {
    stage<N, 8, C, CP, NT>(s, tw, p, tid);
    p *= 8;
  }
  if constexpr (RD::tail == 1) stage<N, 2, C, CP, NT>(s, tw, p, tid);
  if constexpr (RD::tail == 2) stage<N, 4, C, CP, NT>(s, tw, p, tid);
}

}  // namespace fft
}  // namespace gbp
