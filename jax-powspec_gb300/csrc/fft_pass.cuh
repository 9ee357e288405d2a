// Column-FFT engine shared by every pass of the library transform: radix-8
// Stockham stages (fft_core.cuh) over blocks of columns, where
//
//   * each thread transforms the same butterfly of two adjacent columns at
//     once: every shared or global access moves 16 bytes (two complex
//     values), and the two butterflies share one set of twiddle factors;
//   * the twiddles come from per-stage tables, w_r(k) = exp(-2 pi i r k /
//     (R p)) for r < 8 stored contiguously per k (four 16-byte loads);
//   * the first stage reads its inputs from wherever they are (HBM, or
//     integer accumulators) and the last stage writes its outputs to
//     wherever they go (HBM, or a transposed shared buffer); only the
//     exchanges between stages go through shared memory.
//
// Two shared layouts, both free of bank conflicts for every stage's access
// pattern (checked by enumeration):
//
//   ColBlock (thread b owns column pair b % CP, butterfly b / CP): row j of a
//     block of 8 columns is 64 bytes, stored at physical row j ^ bit3(j), so
//     the two rows of a quarter-warp fall on the two halves of a 128-byte
//     bank line; two slabs (two grids) are offset by 64 bytes.
//   Column-major pairs (IFAST: consecutive lanes on consecutive rows): the
//     16-byte slot of rows j of two adjacent columns is at j ^ ((j >> 3) & 7),
//     so 8 consecutive rows of any stage (the stride-8 writes of the first
//     stage included) hit 8 distinct slots.
//
// Forward transform exp(-2 pi i j k / N) (cuFFT, numpy), natural-order output.
#pragma once

#include "fft_core.cuh"

namespace gbp {
namespace fft {

// Offset (in float2) of the twiddle table of the stage with span p > 1; the
// first N entries of the table buffer are exp(-2 pi i e / N).
template <int N>
__host__ __device__ constexpr int tw_off(int p) { return N + 8 * (p - 8) / 7; }

// Size (in float2) of the whole twiddle buffer for N.
template <int N>
constexpr int tw_size() {
  int p = 1;
  for (int s = 0; s < Radices<N>::n8; ++s) p *= 8;   // span of the last radix-8 stage's successor
  return tw_off<N>(p) + 8 * p;
}

__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 pack2(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }

// Barrier of the GS consecutive threads that share data (a named barrier,
// id 1 + tid / GS), or of the whole CTA when GS == 0.
template <int GS>
__device__ __forceinline__ void group_sync(int tid) {
  if constexpr (GS == 0) {
    __syncthreads();
  } else {
    static_assert(GS % 32 == 0, "named barriers count whole warps");
    asm volatile("bar.sync %0, %1;" ::"r"(1 + tid / GS), "n"(GS) : "memory");
  }
}

// One stage over CP column pairs.  In(row, cp) -> float4, Out(row, cp, float4).
// MID_SYNC separates the reads from the writes (in-place shared stages);
// END_SYNC publishes the writes.  IFAST: thread b owns butterfly b % (N/R) of
// column pair b / (N/R) (consecutive lanes, consecutive rows); otherwise
// column pair b % CP, butterfly b / CP.  GS > 0 (IFAST, N/R == GS threads per
// column pair, one butterfly each): the barriers cover only the threads of
// one column pair, whose data no other thread touches.
template <int N, int R, int CP, int NT, bool MID_SYNC, bool END_SYNC, bool IFAST, class In, class Out,
          int GS = 0>
__device__ __forceinline__ void stage2(In in, Out out, const float2* __restrict__ tw, int p, int tid) {
  constexpr int NB = CP * (N / R);
  constexpr int PER = (NB + NT - 1) / NT;
  float4 u[PER][R];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int b = tid + q * NT;
    if (PER * NT != NB && b >= NB) continue;
    const int cp = IFAST ? b / (N / R) : b % CP, i = IFAST ? b % (N / R) : b / CP;
#pragma unroll
    for (int r = 0; r < R; ++r) u[q][r] = in(i + r * (N / R), cp);
    float2 a[R], c[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      a[r] = lo2(u[q][r]);
      c[r] = hi2(u[q][r]);
    }
    if (p > 1) {
      const int k = i & (p - 1);
      const float4* t4 = reinterpret_cast<const float4*>(tw + tw_off<N>(p) + k * 8);
#pragma unroll
      for (int rr = 0; rr < R / 2; ++rr) {
        const float4 w = __ldg(t4 + rr);
        if (rr > 0) {
          a[2 * rr] = cmul(a[2 * rr], lo2(w));
          c[2 * rr] = cmul(c[2 * rr], lo2(w));
        }
        a[2 * rr + 1] = cmul(a[2 * rr + 1], hi2(w));
        c[2 * rr + 1] = cmul(c[2 * rr + 1], hi2(w));
      }
    }
    if constexpr (R == 8) {
      dft8(a);
      dft8(c);
    } else if constexpr (R == 4) {
      dft4(a);
      dft4(c);
    } else {
      dft2(a[0], a[1]);
      dft2(c[0], c[1]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) u[q][r] = pack2(a[r], c[r]);
  }
  static_assert(GS == 0 || (IFAST && N / R == GS && NB == NT), "group barriers need one column pair per group");
  if (MID_SYNC) group_sync<GS>(tid);
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int b = tid + q * NT;
    if (PER * NT != NB && b >= NB) continue;
    const int cp = IFAST ? b / (N / R) : b % CP, i = IFAST ? b % (N / R) : b / CP;
    const int k = i & (p - 1);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out(j + r * p, cp, u[q][r]);
  }
  if (END_SYNC) group_sync<GS>(tid);
}

// Full transform: the first stage reads `gin`, the stages in between go
// through shared memory (`sin` / `sout`), the last stage writes `gout`.
// Starts without a barrier (the caller orders earlier uses of shared
// memory).  IN_SHARED: `gin` reads shared memory that the first stage's
// writes alias; OUT_SHARED: `gout` writes the shared memory the last stage
// reads (each then reads everything before it writes; OUT_SHARED also ends
// with a barrier).
template <int N, int CP, int NT, bool IFAST, bool IN_SHARED, bool OUT_SHARED, class GIn, class SIn, class SOut,
          class GOut, int GS = 0>
__device__ __forceinline__ void run_stages2(GIn gin, SIn sin_, SOut sout, GOut gout, const float2* __restrict__ tw,
                                            int tid) {
  using RD = Radices<N>;
  static_assert(RD::stages >= 2, "at least two stages");
  static_assert(GS == 0 || RD::tail == 0, "group barriers need radix-8 stages only");
  stage2<N, 8, CP, NT, IN_SHARED, true, IFAST, GIn, SOut, GS>(gin, sout, tw, 1, tid);
  int p = 8;
  if constexpr (RD::tail == 0) {
#pragma unroll
    for (int st = 1; st < RD::n8 - 1; ++st) {
      stage2<N, 8, CP, NT, true, true, IFAST, SIn, SOut, GS>(sin_, sout, tw, p, tid);
      p *= 8;
    }
    // the last stage's outputs may be read by any thread: a CTA barrier ends it
    stage2<N, 8, CP, NT, OUT_SHARED, false, IFAST, SIn, GOut, GS>(sin_, gout, tw, p, tid);
    if (OUT_SHARED) __syncthreads();
  } else {
#pragma unroll
    for (int st = 1; st < RD::n8; ++st) {
      stage2<N, 8, CP, NT, true, true, IFAST>(sin_, sout, tw, p, tid);
      p *= 8;
    }
    if constexpr (RD::tail == 1) stage2<N, 2, CP, NT, OUT_SHARED, OUT_SHARED, IFAST>(sin_, gout, tw, p, tid);
    else stage2<N, 4, CP, NT, OUT_SHARED, OUT_SHARED, IFAST>(sin_, gout, tw, p, tid);
  }
}

// Blocks of 8 columns (x SLABS); a float4 holds two adjacent columns.
template <int N, int SLABS>
struct ColBlock {
  static constexpr int COLS = 8 * SLABS;
  static constexpr int CP = COLS / 2;
  static constexpr int SLAB = N * 8 + 8;    // complex per slab (+8: the 64-byte shift of slab 1)
  __device__ static __forceinline__ int row(int j) { return SLABS == 1 ? (j ^ ((j >> 3) & 1)) : j; }
  // float4 index of column pair cp (columns 2cp, 2cp+1) in row j
  __device__ static __forceinline__ int at(int j, int cp) { return (cp >> 2) * (SLAB / 2) + row(j) * 4 + (cp & 3); }
};

// IN_SHARED: the first stage's shared-memory writes must wait for earlier
// readers of `s` (a barrier between its loads and its writes), so a caller
// can start the loads of the next block while other warps still read the
// previous one.
template <int N, int SLABS, int NT, bool OUT_SHARED, class In, class Out, bool IN_SHARED = false>
__device__ __forceinline__ void col_fft(float2* s, In gin, Out gout, const float2* __restrict__ tw, int tid) {
  using L = ColBlock<N, SLABS>;
  float4* s4 = reinterpret_cast<float4*>(s);
  auto sin_ = [s4](int j, int cp) { return s4[L::at(j, cp)]; };
  auto sout = [s4](int j, int cp, float4 v) { s4[L::at(j, cp)] = v; };
  run_stages2<N, L::CP, NT, false, IN_SHARED, OUT_SHARED>(gin, sin_, sout, gout, tw, tid);
}

// Slot of row j in a column-major block of column pairs (IFAST stages).
__device__ __forceinline__ int zsw(int j) { return j ^ ((j >> 3) & 7); }

}  // namespace fft
}  // namespace gbp
