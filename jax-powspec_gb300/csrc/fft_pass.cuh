// Column-FFT engine for the y and x passes: C columns x N rows per CTA,
// radix-8 Stockham stages (fft_core.cuh) whose first stage reads its inputs
// straight from global memory and whose last stage writes its outputs
// straight to their destination (global memory, or a transposed shared
// buffer).  Only the exchanges between stages go through shared memory, so
// each element costs 4 shared-memory accesses per pass instead of 8 (a
// staged load, three in-place stages and a staged store).
//
// Shared layout of a block of 8 columns: row j holds the 8 complex values of
// the columns (64 bytes).  Row j is stored at physical row j ^ bit3(j): a
// warp touches 4 aligned rows per access, which then fall on alternating
// halves of the 128-byte bank line (the minimum of 2 wavefronts for 32 x 8
// bytes) both in the stride-8 writes of the first stage and in the
// consecutive-row accesses of the others.  Two slabs of 8 columns (two
// grids) are offset by 64 bytes, so a half-warp's 16 columns of one row
// cover one whole bank line.
//
// Thread b of a stage owns butterfly (col = b % COLS, i = b / COLS).  The
// forward transform is exp(-2 pi i j k / N) (cuFFT, numpy), natural-order
// output.
#pragma once

#include "fft_core.cuh"

namespace gbp {
namespace fft {

// Row position of element j in a column-major block walked with consecutive
// lanes on consecutive rows (IFAST stages): bits 4-6 of j are XORed into bits
// 0-3, which puts the 16 lanes of a half-warp on 16 distinct 8-byte bank slots
// in every stage (the stride-8 writes of the first stage, the two
// interleaved runs of the second, the consecutive rows of the others).
__device__ __forceinline__ int zsw(int j) { return j ^ ((j >> 4) & 7) ^ (((j >> 6) & 1) << 3); }

template <int N, int SLABS>
struct ColBlock {
  static constexpr int COLS = 8 * SLABS;
  static constexpr int SLAB = N * 8 + 8;    // complex per slab (+8: the 64-byte shift of slab 1)
  __device__ static __forceinline__ int row(int j) { return SLABS == 1 ? (j ^ ((j >> 3) & 1)) : j; }
  __device__ static __forceinline__ int at(int j, int col) { return (col >> 3) * SLAB + row(j) * 8 + (col & 7); }
};

// One stage.  In(row, col) -> float2 gives the inputs, Out(row, col, v)
// takes the outputs; MID_SYNC separates the reads from the writes (in-place
// shared stages), END_SYNC publishes the writes to the next stage.  Thread
// b owns butterfly (col = b % COLS, i = b / COLS), or with IFAST (i = b %
// (N/R), col = b / (N/R)): consecutive lanes on consecutive rows.
template <int N, int R, int COLS, int NT, bool MID_SYNC, bool END_SYNC, bool IFAST = false, class In, class Out>
__device__ __forceinline__ void stage_io(In in, Out out, const float2* __restrict__ tw, int p, int tid) {
  constexpr int NB = COLS * (N / R);
  constexpr int PER = (NB + NT - 1) / NT;
  float2 u[PER][R];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int b = tid + q * NT;
    if (PER * NT != NB && b >= NB) continue;
    const int col = IFAST ? b / (N / R) : b % COLS, i = IFAST ? b % (N / R) : b / COLS;
    const int k = i & (p - 1);
#pragma unroll
    for (int r = 0; r < R; ++r) u[q][r] = in(i + r * (N / R), col);
    if (p > 1) {
      const int step = N / (p * R);
#pragma unroll
      for (int r = 1; r < R; ++r) u[q][r] = cmul(u[q][r], __ldg(tw + ((r * k * step) & (N - 1))));
    }
    if constexpr (R == 8) dft8(u[q]);
    else if constexpr (R == 4) dft4(u[q]);
    else dft2(u[q][0], u[q][1]);
  }
  if (MID_SYNC) __syncthreads();
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int b = tid + q * NT;
    if (PER * NT != NB && b >= NB) continue;
    const int col = IFAST ? b / (N / R) : b % COLS, i = IFAST ? b % (N / R) : b / COLS;
    const int k = i & (p - 1);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out(j + r * p, col, u[q][r]);
  }
  if (END_SYNC) __syncthreads();
}

// Full transform: the first stage reads `gin`, the stages in between go
// through shared memory (`sin` / `sout`), the last stage writes `gout`.
// Starts without a barrier (the caller orders earlier uses of shared
// memory).  OUT_SHARED: `gout` writes the shared buffer the last stage
// reads, so it reads everything first and ends with a barrier.  IN_SHARED:
// `gin` reads shared memory that the first stage's writes alias, so the
// first stage, too, reads everything before it writes.
template <int N, int COLS, int NT, bool IFAST, bool OUT_SHARED, bool IN_SHARED = false, class GIn, class SIn,
          class SOut, class GOut>
__device__ __forceinline__ void run_stages(GIn gin, SIn sin_, SOut sout, GOut gout, const float2* __restrict__ tw,
                                           int tid) {
  using RD = Radices<N>;
  static_assert(RD::stages >= 2, "at least two stages");
  if constexpr (RD::tail == 0) {
    stage_io<N, 8, COLS, NT, IN_SHARED, true, IFAST>(gin, sout, tw, 1, tid);
    int p = 8;
#pragma unroll
    for (int st = 1; st < RD::n8 - 1; ++st) {
      stage_io<N, 8, COLS, NT, true, true, IFAST>(sin_, sout, tw, p, tid);
      p *= 8;
    }
    stage_io<N, 8, COLS, NT, OUT_SHARED, OUT_SHARED, IFAST>(sin_, gout, tw, p, tid);
  } else {
    stage_io<N, 8, COLS, NT, IN_SHARED, true, IFAST>(gin, sout, tw, 1, tid);
    int p = 8;
#pragma unroll
    for (int st = 1; st < RD::n8; ++st) {
      stage_io<N, 8, COLS, NT, true, true, IFAST>(sin_, sout, tw, p, tid);
      p *= 8;
    }
    if constexpr (RD::tail == 1) stage_io<N, 2, COLS, NT, OUT_SHARED, OUT_SHARED, IFAST>(sin_, gout, tw, p, tid);
    else stage_io<N, 4, COLS, NT, OUT_SHARED, OUT_SHARED, IFAST>(sin_, gout, tw, p, tid);
  }
}

// Column blocks of 8 (x SLABS) columns in the ColBlock layout.
template <int N, int SLABS, int NT, bool OUT_SHARED, class In, class Out>
__device__ __forceinline__ void col_fft(float2* s, In gin, Out gout, const float2* __restrict__ tw, int tid) {
  using L = ColBlock<N, SLABS>;
  auto sin_ = [s](int j, int col) { return s[L::at(j, col)]; };
  auto sout = [s](int j, int col, float2 v) { s[L::at(j, col)] = v; };
  run_stages<N, L::COLS, NT, false, OUT_SHARED>(gin, sin_, sout, gout, tw, tid);
}

}  // namespace fft
}  // namespace gbp
