// Particles -> multipole sums with the deposit fused into the z pass of the
// FFT (library transform sizes: power-of-two meshes 64..1024, B-spline
// deposits).  Included by one translation unit per mesh size
// (depfft_n<N>.cu); depfft.cu holds the C ABI and picks the unit by N.
//
// The mesh is never written.  Particles are bucketed (deposit_core.cuh) by
// column tile: TX x TY pencils spanning the whole z axis (the tile shape is
// a plan option: 4x4, 8x4 or 8x8, see column_tile_variants), so a stencil is
// replicated across x and y tile faces only.  One CTA per column tile:
//
//   1. accumulates its bucket in shared memory as 32-bit fixed point.  Each
//      4x4-pencil block of the tile has a scale of its own, 2^s with
//      s = s_g - ceil(log2(c)) (+1 for TSC and PCS, whose node weights stay
//      below 1/2), where c is the largest number of entries that cover the
//      block in one z plane (counted first) and 2^s_g puts the largest
//      particle weight just below 2^30.  No cell can then exceed 2^30 +
//      rounding in magnitude, whatever the order of the adds, so the integer
//      sums are exact, order-independent and overflow-free (fire-and-forget
//      shared reductions, no carries).  The scales belong to the 4x4 blocks,
//      not to the tile, so every tile shape gives the same cells, the same
//      floats and the same P_l, bit for bit;
//   2. transforms its pencils along z: the first radix-8 stage reads the
//      integer cells of two pencils (packed as one complex pencil), converts
//      them to float and writes the complex buffer that aliases the
//      accumulators; the remaining stages run in place (fft_pass.cuh),
//   3. splits each packed spectrum into its two real-input half spectra and
//      writes the pencils' rows of the z-transformed spectrum (P = N/2 + 8
//      complex per row, as the library's own transform),
//   4. adds up the tile's exact integer total at the common scale 2^s_g
//      (the mean density; stats_kernel folds the tiles).
//
// A block whose densest plane would cost more than SH_MAX bits (a dense
// clump) sends its whole tile to deposit_fftz_wide_kernel: 64-bit cells, the
// clumped blocks at the common scale, the others at their own.
//
// Then the y pass (fft.cu) and the x pass fused with the binning (xbin.cu)
// finish the transform and the P_l sums.  HBM traffic per grid: the
// spectrum is written once here, read and written by the y pass, and read
// once by the binning; no mesh goes through HBM.
#pragma once

#include <algorithm>
#include <type_traits>

#include "deposit_core.cuh"
#include "fft_pass.cuh"
#include "gbp_bins.h"
#include "gbp_fft.h"

namespace gbp {
namespace {

template <int N, int TX_, int TY_>
struct ColTile {
  static constexpr int TX = TX_, TY = TY_;
  static constexpr int NPEN = TX * TY;            // pencils per tile; pencil f = lx * TY + ly
  static constexpr int PAIRS = NPEN / 2;          // complex transforms (pencils 2q, 2q+1)
  static constexpr int NFFT = PAIRS * N / 16;     // butterfly pairs (two columns) per radix-8 stage
  static constexpr int NT = NFFT < 256 ? 256 : NFFT;
  static constexpr int MINB = NT >= 1024 ? 1 : (NT >= 512 ? 2 : 3);   // CTAs per SM the registers are sized for
  static constexpr int SBX = TX / 4, SBY = TY / 4, NSB = SBX * SBY;    // 4x4-pencil scale blocks
  static constexpr size_t SMEM = (size_t)(NPEN + NSB) * N * sizeof(int);   // cells + per-block plane counts
  static constexpr size_t SMEM_WIDE = (size_t)NPEN * N * sizeof(long long);
  static_assert(TX % 4 == 0 && TY % 4 == 0, "tiles are whole 4x4 scale blocks");
};

// Scale block of local pencil column (lx, ly).
template <class CT>
__device__ __forceinline__ int scale_block(int lx, int ly) { return (lx >> 2) * CT::SBY + (ly >> 2); }

// v[b] for a block index known only at run time, by selects (no local memory).
template <int NSB, class T>
__device__ __forceinline__ T pick_block(int b, const T (&v)[NSB]) {
  T r = v[0];
#pragma unroll
  for (int k = 1; k < NSB; ++k) r = b == k ? v[k] : r;
  return r;
}

// Bits of resolution a block may give up to its 32-bit cells.  A block whose
// densest z plane is covered by more than 2^(SH_MAX + WBIT) entries (a dense
// clump: a halo, a point mass) is deposited with 64-bit cells at the common
// scale instead, by deposit_fftz_wide_kernel: with the coarse quantum the
// rounding of many identical contributions adds up instead of averaging out.
constexpr int SH_MAX = 10;
constexpr long long WIDE_MARK = (-0x7fffffffffffffffLL - 1);   // tile_mass entry of a tile left to the wide kernel

// Deposit, z transform, split and row stores of one column tile and grid
// (steps 1-4 above).  WIDE: 64-bit cells.  sh[b]: bits given up by scale
// block b (its scale 2^(sg - sh[b]), sh[b] <= SH_MAX).  Returns the tile's
// exact total at the common scale 2^sg (valid in thread 0).
template <int N, int MAS, int G, class CT, bool WIDE>
__device__ __forceinline__ long long tile_grid(const DepGeom& g, const float4* __restrict__ entries, unsigned beg,
                                               unsigned end, int sg, const int (&sh)[CT::NSB], int grid, int x0,
                                               int y0, const float2* __restrict__ tw, float2* __restrict__ spec,
                                               unsigned char* smem, long long* s_part) {
  using Cell = typename std::conditional<WIDE, unsigned long long, int>::type;
  constexpr int R = MAS, TX = CT::TX, TY = CT::TY, NPEN = CT::NPEN, PAIRS = CT::PAIRS, NT = CT::NT;
  constexpr int NSB = CT::NSB;
  constexpr int P = N / 2 + 8, H = N / 2;
  Cell* acc = reinterpret_cast<Cell*>(smem);                   // [NPEN][N] fixed-point cells
  float4* cs4 = reinterpret_cast<float4*>(smem);               // [PAIRS/2][N] slots of two columns, alias the cells
  const int tid = threadIdx.x;
  // 2^s and 2^-s of each block: s = sg - sh in [-110, 100], one normal float each
  float up[NSB], dn[NSB];
#pragma unroll
  for (int b = 0; b < NSB; ++b) {
    up[b] = ldexpf(1.0f, sg - sh[b]);
    dn[b] = ldexpf(1.0f, sh[b] - sg);
  }
  const long long gstride = (long long)N * N * P;

  {
    uint4* a4 = reinterpret_cast<uint4*>(acc);
    for (int k = tid; k < (int)(NPEN * N * sizeof(Cell) / 16); k += NT) a4[k] = make_uint4(0u, 0u, 0u, 0u);
  }
  __syncthreads();
  for (unsigned i = beg + tid; i < end; i += NT) {
    const float4 e = entries[i];
    Axis<R> ax, ay, az;
    make_axis<MAS, 0, N>(g, e.x, grid, ax);
    make_axis<MAS, 0, N>(g, e.y, grid, ay);
    make_axis<MAS, 0, N>(g, e.z, grid, az);
    int lx[R], ly[R], zz[R];
    local_nodes<R>(ax, N, x0, TX, lx);
    local_nodes<R>(ay, N, y0, TY, ly);
    // z weight times the particle weight at each block's scale (exact: powers of two)
    float wz[NSB][R];
#pragma unroll
    for (int r = 0; r < R; ++r) zz[r] = wrapn(az.first + r, N);
#pragma unroll
    for (int b = 0; b < NSB; ++b) {
      const float wsc = __fmul_rn(e.w, up[b]);
#pragma unroll
      for (int r = 0; r < R; ++r) wz[b][r] = __fmul_rn(az.w[r], wsc);
    }
#pragma unroll
    for (int rx = 0; rx < R; ++rx) {
      if (lx[rx] < 0) continue;
      // with one block row (TY = 4) the block depends on x only: select the z weights once per x node
      float wzx[R];
      if constexpr (CT::SBY == 1) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          float wzb[NSB];
#pragma unroll
          for (int k = 0; k < NSB; ++k) wzb[k] = wz[k][r];
          wzx[r] = pick_block<NSB>(lx[rx] >> 2, wzb);
        }
      }
#pragma unroll
      for (int ry = 0; ry < R; ++ry) {
        if (ly[ry] < 0) continue;
        const float wxy = __fmul_rn(ax.w[rx], ay.w[ry]);
        const int row = (lx[rx] * TY + ly[ry]) * N;
#pragma unroll
        for (int rz = 0; rz < R; ++rz) {
          float wzr;
          if constexpr (CT::SBY == 1) {
            wzr = wzx[rz];
          } else {
            float wzb[NSB];
#pragma unroll
            for (int k = 0; k < NSB; ++k) wzb[k] = wz[k][rz];
            wzr = pick_block<NSB>(scale_block<CT>(lx[rx], ly[ry]), wzb);
          }
          const int v = __float2int_rn(__fmul_rn(wxy, wzr));
          if constexpr (WIDE) atomicAdd(&acc[row + zz[rz]], (unsigned long long)(long long)v);
          else atomicAdd(&acc[row + zz[rz]], v);
        }
      }
    }
  }
  __syncthreads();

  // z transform: pencils 2q and 2q+1 are the real and imaginary parts of
  // column q; a thread transforms columns 2cp and 2cp+1 (pencils 4cp..4cp+3,
  // one scale block), the same column pair in every stage of the first
  // (and only) butterfly per thread: cp = tid / (N/8)
  long long part = 0;
  auto gin = [&part, &dn, acc](int j, int cp) {
    const int f = 4 * cp;
    const float d = pick_block<NSB>(scale_block<CT>(f / TY, f % TY), dn);
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const long long q = (long long)acc[(f + k) * N + j];
      part += q;
      v[k] = __fmul_rn(WIDE ? __ll2float_rn(q) : __int2float_rn((int)q), d);   // exact: a power of two
    }
    return make_float4(v[0], v[1], v[2], v[3]);
  };
  auto sin_ = [cs4](int j, int cp) { return cs4[cp * N + fft::zsw(j)]; };
  auto sout = [cs4](int j, int cp, float4 v) { cs4[cp * N + fft::zsw(j)] = v; };
  // N = 512, 32-bit cells: every stage is radix 8 and the 64 threads of a column pair own its data
  // (the first stage's writes alias the pair's own pencils), so the stages synchronise 64-thread
  // groups only.  64-bit cells span twice the bytes of the complex slots: whole-CTA barriers.
  constexpr int GS = (!WIDE && N == 512 && NT == PAIRS / 2 * (N / 8)) ? N / 8 : 0;
  static_assert(CT::NFFT <= NT, "one first-stage butterfly per thread");
  fft::run_stages2<N, PAIRS / 2, NT, true, true, true, decltype(gin), decltype(sin_), decltype(sout),
                   decltype(sout), GS>(gin, sin_, sout, sout, tw, tid);
  {
    // this thread's cells belong to one scale block: shift its total to the common scale
    const int cp = tid / (N / 8);
    if (cp < PAIRS / 2) {
      int shb[NSB];
#pragma unroll
      for (int b = 0; b < NSB; ++b) shb[b] = sh[b];
      part *= (1LL << pick_block<NSB>(scale_block<CT>(4 * cp / TY, 4 * cp % TY), shb));
    }
  }

  // split the packed spectra; write all pencils' rows (row padding -> 0), two k per thread and
  // 16-byte stores
  const float2* cs = reinterpret_cast<const float2*>(cs4);
  float2* out = spec + grid * gstride;
  constexpr int P2 = P / 2;
  for (int idx = tid; idx < PAIRS * P2; idx += NT) {
    const int q = idx / P2, k0 = 2 * (idx - q * P2);
    const float2* col = cs + (q >> 1) * N * 2 + (q & 1);
    float2 a[2], b[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = k0 + h;
      a[h] = b[h] = make_float2(0.f, 0.f);
      if (k <= H) {
        const float2 c = col[fft::zsw(k) * 2];
        const float2 m = col[fft::zsw((N - k) & (N - 1)) * 2];
        const float2 cm = make_float2(m.x, -m.y);
        const float2 sum = fft::cadd(c, cm), dif = fft::cmi(fft::csub(c, cm));
        a[h] = make_float2(0.5f * sum.x, 0.5f * sum.y);
        b[h] = make_float2(0.5f * dif.x, 0.5f * dif.y);
      }
    }
    const int f0 = 2 * q, f1 = 2 * q + 1;
    const long long r0 = (long long)(x0 + f0 / TY) * N + (y0 + f0 % TY);
    const long long r1 = (long long)(x0 + f1 / TY) * N + (y0 + f1 % TY);
    __stcs(reinterpret_cast<float4*>(out + r0 * P + k0), make_float4(a[0].x, a[0].y, a[1].x, a[1].y));
    __stcs(reinterpret_cast<float4*>(out + r1 * P + k0), make_float4(b[0].x, b[0].y, b[1].x, b[1].y));
  }

  // the tile's exact total
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((tid & 31) == 0) s_part[tid >> 5] = part;
  __syncthreads();                                     // also: the next grid reuses the accumulators
  long long tm = 0;
  if (tid == 0)
    for (int k = 0; k < NT / 32; ++k) tm += s_part[k];
  return tm;
}

// Per-block plane counts of a tile (zc [NSB][N], zeroed on entry) and the
// bits each block gives up; returns true when some block is a dense clump
// (then sh[] holds SH_MAX + 1 for those blocks).  An entry covers block b in
// plane z when its nodes (any grid) reach b's 4 x-columns, its 4 y-columns
// and z.
template <int N, int MAS, int G, class CT>
__device__ __forceinline__ bool block_scales(const DepGeom& g, const float4* __restrict__ entries, unsigned beg,
                                             unsigned end, int x0, int y0, int* zc, int* s_max, int (&sh)[CT::NSB]) {
  constexpr int R = MAS, NT = CT::NT, NSB = CT::NSB, W = R + G - 1;
  const int tid = threadIdx.x;
  // this pass is the tile's first touch of its bucket: a thread issues EB entry loads at once
  constexpr int EB = 4;
  for (unsigned i0 = beg + tid; i0 < end; i0 += EB * NT) {
    float4 ev[EB];
#pragma unroll
    for (int k = 0; k < EB; ++k) {
      const unsigned i = i0 + k * NT;
      ev[k] = i < end ? entries[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < EB; ++k) {
      if (i0 + k * NT >= end) break;
      const float4 e = ev[k];
      // the union of the grids' nodes along each axis: first .. last (the second grid's first node
      // is the first grid's or the next one), as the bucketing counts them.  Every entry of the
      // bucket reaches the tile, so an axis with one block row needs no test
      int first[3], last[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if ((a == 0 && CT::SBX == 1) || (a == 1 && CT::SBY == 1)) {
          first[a] = last[a] = 0;
          continue;
        }
        Axis<R> a0;
        make_axis<MAS, 0, N>(g, a == 0 ? e.x : (a == 1 ? e.y : e.z), 0, a0);
        first[a] = a0.first;
        last[a] = a0.first + R - 1;
        if constexpr (G == 2) {
          Axis<R> a1;
          make_axis<MAS, 0, N>(g, a == 0 ? e.x : (a == 1 ? e.y : e.z), 1, a1);
          last[a] = a1.first + R - 1;
        }
      }
      // scale blocks reached along x and y
      unsigned mx = CT::SBX == 1 ? 1u : 0u, my = CT::SBY == 1 ? 1u : 0u;
#pragma unroll
      for (int r = 0; r < W; ++r) {
        if constexpr (CT::SBX > 1) {
          const int cx = wrapn(first[0] + r, N) - x0;
          if (first[0] + r <= last[0] && cx >= 0 && cx < CT::TX) mx |= 1u << (cx >> 2);
        }
        if constexpr (CT::SBY > 1) {
          const int cy = wrapn(first[1] + r, N) - y0;
          if (first[1] + r <= last[1] && cy >= 0 && cy < CT::TY) my |= 1u << (cy >> 2);
        }
      }
#pragma unroll
      for (int bx = 0; bx < CT::SBX; ++bx)
#pragma unroll
        for (int by = 0; by < CT::SBY; ++by)
          if (((mx >> bx) & 1u) && ((my >> by) & 1u))
            for (int zn = first[2]; zn <= last[2]; ++zn) atomicAdd(&zc[(bx * CT::SBY + by) * N + wrapn(zn, N)], 1);
    }
  }
  __syncthreads();
  // a node weight of TSC (<= 0.75^3) or PCS (<= (2/3)^3) is below 1/2: one more bit
  constexpr int WBIT = (MAS == GBP_TSC || MAS == GBP_PCS) ? 1 : 0;
  bool heavy = false;
#pragma unroll
  for (int b = 0; b < NSB; ++b) {
    int cmax = 0;
    for (int k = tid; k < N; k += NT) cmax = max(cmax, zc[b * N + k]);
    cmax = __reduce_max_sync(0xffffffffu, cmax);
    if ((tid & 31) == 0) s_max[tid >> 5] = cmax;
    __syncthreads();
    cmax = 0;
    for (int k = 0; k < NT / 32; ++k) cmax = max(cmax, s_max[k]);
    __syncthreads();                                   // s_max is reused by the next block
    const unsigned cnt = (unsigned)cmax;
    const int lg = cnt > 1u ? 32 - __clz(cnt - 1u) : 0;  // ceil(log2(entries per plane))
    sh[b] = lg > WBIT ? lg - WBIT : 0;                 // block scale 2^(sg - sh), never finer than 2^sg
    if (sh[b] > SH_MAX) heavy = true;
  }
  return heavy;
}

template <int N, int MAS, int G, class CT>
__global__ void __launch_bounds__(CT::NT, CT::MINB)
deposit_fftz_kernel(DepGeom g, const float4* __restrict__ entries, const unsigned* __restrict__ counts,
                    const unsigned* __restrict__ offsets, const DepCounters* ctr, const float2* __restrict__ tw,
                    float2* __restrict__ spec, long long* __restrict__ tile_mass) {
  pdl_wait();
  constexpr int NPEN = CT::NPEN, NT = CT::NT, NSB = CT::NSB;
  extern __shared__ __align__(16) int acc_smem[];
  int* zc = acc_smem + NPEN * N;                       // [NSB][N] entries covering each block's planes
  __shared__ long long s_part[NT / 32];
  __shared__ int s_max[NT / 32];
  const int tid = threadIdx.x;
  const int t = blockIdx.x;
  const int ty = t % g.nt[1], tx = t / g.nt[1];
  const int x0 = tx * CT::TX, y0 = ty * CT::TY;
  unsigned beg, end;
  tile_range(g, t, counts, offsets, ctr, beg, end);
  const int sg = fixed_scale_exp(ctr->maxw_bits, 0);
  for (int k = tid; k < NSB * N; k += NT) zc[k] = 0;
  __syncthreads();
  int sh[NSB];
  if (block_scales<N, MAS, G, CT>(g, entries, beg, end, x0, y0, zc, s_max, sh)) {
    // a dense clump: the wide kernel takes this tile (the clumped blocks at the common scale)
    if (tid == 0) {
      long long packed = 0;
      for (int b = 0; b < NSB; ++b) packed |= (long long)(sh[b] > SH_MAX ? 0 : sh[b]) << (8 * b);
      tile_mass[t] = WIDE_MARK;
      tile_mass[(long long)gridDim.x + t] = packed;    // the second grid's slot is free until the wide kernel
    }
    return;
  }
  for (int grid = 0; grid < G; ++grid) {
    const long long tm = tile_grid<N, MAS, G, CT, false>(g, entries, beg, end, sg, sh, grid, x0, y0, tw, spec,
                                                         reinterpret_cast<unsigned char*>(acc_smem), s_part);
    if (tid == 0) tile_mass[(long long)grid * gridDim.x + t] = tm;   // exact, at the common scale 2^sg
  }
}

// The tiles deposit_fftz_kernel left (tile_mass entry WIDE_MARK, the
// blocks' shifts packed in the second slot): 64-bit cells.  Persistent:
// CTA b owns a contiguous range of tiles, finds its marked ones with one
// parallel scan (such tiles are rare; with none, that scan is all a CTA
// does) and processes them in turn.
constexpr int WIDE_LIST = 64;                          // marked tiles listed per scan round

template <int N, int MAS, int G, class CT>
__global__ void __launch_bounds__(CT::NT, CT::MINB)
deposit_fftz_wide_kernel(DepGeom g, const float4* __restrict__ entries, const unsigned* __restrict__ counts,
                         const unsigned* __restrict__ offsets, const DepCounters* ctr, const float2* __restrict__ tw,
                         float2* __restrict__ spec, long long* __restrict__ tile_mass, int ntiles) {
  pdl_wait();
  constexpr int NT = CT::NT, NSB = CT::NSB;
  extern __shared__ __align__(16) unsigned long long wide_smem[];
  __shared__ long long s_part[NT / 32];
  __shared__ int s_list[WIDE_LIST];
  __shared__ int s_n;
  const int sg = fixed_scale_exp(ctr->maxw_bits, 0);
  const int per = (ntiles + gridDim.x - 1) / gridDim.x;
  const int t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
  for (int base = t0; base < t1; base += NT) {
    for (;;) {                                         // list the marked tiles of [base, base + NT), 64 at a time
      if (threadIdx.x == 0) s_n = 0;
      __syncthreads();
      const int t = base + (int)threadIdx.x;
      if (t < t1 && tile_mass[t] == WIDE_MARK) {
        const int k = atomicAdd(&s_n, 1);
        if (k < WIDE_LIST) s_list[k] = t;
      }
      __syncthreads();
      const int n = min(s_n, WIDE_LIST);
      if (n == 0) break;                               // uniform over the CTA
      for (int k = 0; k < n; ++k) {
        const int tt = s_list[k];
        const int ty = tt % g.nt[1], tx = tt / g.nt[1];
        unsigned beg, end;
        tile_range(g, tt, counts, offsets, ctr, beg, end);
        const long long packed = tile_mass[(long long)ntiles + tt];
        int sh[NSB];
#pragma unroll
        for (int b = 0; b < NSB; ++b) sh[b] = (int)((packed >> (8 * b)) & 0xff);
        __syncthreads();                               // every thread has read the shifts before they are replaced
        for (int grid = 0; grid < G; ++grid) {
          const long long tm = tile_grid<N, MAS, G, CT, true>(g, entries, beg, end, sg, sh, grid, tx * CT::TX,
                                                              ty * CT::TY, tw, spec,
                                                              reinterpret_cast<unsigned char*>(wide_smem), s_part);
          if (threadIdx.x == 0) tile_mass[(long long)grid * ntiles + tt] = tm;   // clears the mark
        }
        if (G == 1 && threadIdx.x == 0) tile_mass[(long long)ntiles + tt] = 0;
      }
      __syncthreads();                                 // the marks are replaced before the next scan
    }
  }
}

struct PartLayout {
  DepLayout dep;
  size_t xbin, total;
};

int particles_layout(int64_t n, gbp_fft_plan plan, gbp_bins B, int mas, int ells, int tx, int ty, PartLayout& L) {
  if (!plan || !B || plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own || (plan->grids != 1 && plan->grids != 2)) return GBP_ERR_UNSUPPORTED;
  const int tile[3] = {tx, ty, B->N};
  int st = deposit_layout(n, B->N, mas, plan->grids == 2, GBP_COMPAT_NONE, tile, L.dep, true);
  if (st) return st;
  st = xbin_power_workspace(plan, B, ells, &L.xbin);
  if (st) return st;
  L.total = align256(L.dep.total) + L.xbin;
  return GBP_OK;
}

template <int N, int MAS, int G, class CT>
int run_fused(const DepGeom& g, const DepLayout& L, const DepBuffers& b, const float2* tw, float2* spec,
              cudaStream_t st) {
  int r = bucket_particles<MAS, G, 0>(g, L, b, st);
  if (r) return r;
  auto k = deposit_fftz_kernel<N, MAS, G, CT>;
  GBP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CT::SMEM));
  {
    GBP_TRACE("deposit_fft_z", st);
    GBP_CUDA_TRY(launch_pdl(k, dim3(L.ntiles), dim3(CT::NT), CT::SMEM, st, g, b.entries, b.counts, b.offsets, b.ctr,
                            tw, spec, b.tile_mass));
  }
  // tiles of dense clumps, if any, with 64-bit cells (as many CTAs as fit at once scan the marks: a
  // dense small mesh can send most of its tiles here)
  auto kw = deposit_fftz_wide_kernel<N, MAS, G, CT>;
  GBP_CUDA_TRY(cudaFuncSetAttribute(kw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CT::SMEM_WIDE));
  int dev = 0, sms = 0, per_sm = 0;
  GBP_CUDA_TRY(cudaGetDevice(&dev));
  GBP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GBP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kw, CT::NT, CT::SMEM_WIDE));
  GBP_TRACE("deposit_fft_z_wide", st);
  GBP_CUDA_TRY(launch_pdl(kw, dim3(std::max(1, std::min(sms * std::max(per_sm, 1), L.ntiles))), dim3(CT::NT),
                          CT::SMEM_WIDE, st, g, b.entries, b.counts, b.offsets, b.ctr, tw, spec, b.tile_mass,
                          L.ntiles));
  return GBP_OK;
}

template <int N, class CT>
int dispatch_mas(int mas, int G, const DepGeom& g, const DepLayout& L, const DepBuffers& b, const float2* tw,
                 float2* spec, cudaStream_t st) {
  if (G == 2) {
    switch (mas) {
      case GBP_NGP: return run_fused<N, GBP_NGP, 2, CT>(g, L, b, tw, spec, st);
      case GBP_CIC: return run_fused<N, GBP_CIC, 2, CT>(g, L, b, tw, spec, st);
      case GBP_TSC: return run_fused<N, GBP_TSC, 2, CT>(g, L, b, tw, spec, st);
      default: return run_fused<N, GBP_PCS, 2, CT>(g, L, b, tw, spec, st);
    }
  }
  switch (mas) {
    case GBP_NGP: return run_fused<N, GBP_NGP, 1, CT>(g, L, b, tw, spec, st);
    case GBP_CIC: return run_fused<N, GBP_CIC, 1, CT>(g, L, b, tw, spec, st);
    case GBP_TSC: return run_fused<N, GBP_TSC, 1, CT>(g, L, b, tw, spec, st);
    default: return run_fused<N, GBP_PCS, 1, CT>(g, L, b, tw, spec, st);
  }
}

// The whole fused path for mesh side N: bucketing, deposit + z pass, y pass,
// x pass + binning.  (tx, ty) is a supported tile shape for N (checked by
// the caller).
template <int N>
int particles_power_n(DepGeom g, int64_t n_launch, gbp_fft_plan plan, gbp_bins B, int mas, int ells, int tx, int ty,
                      void* spectrum, double* sums_out, long long* nmodes_out, double* ksum_out,
                      gbp_deposit_stats* stats_out, void* workspace, size_t ws_bytes, cudaStream_t st) {
  if (!spectrum || !sums_out || !nmodes_out || !stats_out) return GBP_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(spectrum) & 15u) != 0) return GBP_ERR_INVALID;
  PartLayout L;
  int r = particles_layout(n_launch, plan, B, mas, ells, tx, ty, L);
  if (r) return r;
  if (!workspace || ws_bytes < L.total) return GBP_ERR_WORKSPACE;
  const DepBuffers b = carve_deposit(workspace, L.dep);
  void* xws = static_cast<char*>(workspace) + align256(L.dep.total);
  for (int a = 0; a < 3; ++a) { g.td[a] = L.dep.td[a]; g.ts[a] = L.dep.ts[a]; g.nt[a] = L.dep.nt[a]; }
  g.vec_ok = 0;
  g.tcap = L.dep.tcap;
  const int G = plan->grids;
  float2* spec = static_cast<float2*>(spectrum);
  GBP_CUDA_TRY(cudaMemsetAsync(b.ctr, 0, zeroed_bytes(L.dep), st));
  r = GBP_ERR_UNSUPPORTED;
  if (tx == 4 && ty == 4) {
    r = dispatch_mas<N, ColTile<N, 4, 4>>(mas, G, g, L.dep, b, plan->tw, spec, st);
  } else if (tx == 8 && ty == 4) {
    if constexpr (N <= 512) r = dispatch_mas<N, ColTile<N, 8, 4>>(mas, G, g, L.dep, b, plan->tw, spec, st);
  } else if (tx == 8 && ty == 8) {
    if constexpr (N == 128 || N == 256) r = dispatch_mas<N, ColTile<N, 8, 8>>(mas, G, g, L.dep, b, plan->tw, spec, st);
  }
  if (r) return r;
  r = deposit_stats(b, L.dep, GBP_COMPAT_NONE, G, stats_out, st);
  if (r) return r;
  r = own_fft_y(N, G, spec, plan->tw, st);
  if (r) return r;
  const double* mass = reinterpret_cast<const double*>(stats_out);   // gbp_deposit_stats starts with mass[2]
  return xbin_power(plan, spec, B, mas, ells, mass, sums_out, nmodes_out, ksum_out, xws, L.xbin, st);
}

}  // namespace
}  // namespace gbp

// One translation unit per mesh side defines these (no reference
// counterpart; depfft.cu's C ABI calls them).  The job pointer, when
// non-null, replaces x, y, z, w, n and the box geometry (capacity = n).
#define GBP_DEPFFT_INSTANCE(NN)                                                                                    \
  namespace gbp {                                                                                                  \
  int particles_ws_n##NN(int64_t n, gbp_fft_plan plan, gbp_bins bins, int mas, int ells, int tx, int ty,           \
                         size_t* bytes) {                                                                          \
    PartLayout L;                                                                                                  \
    const int st = particles_layout(n, plan, bins, mas, ells, tx, ty, L);                                          \
    if (st) return st;                                                                                             \
    *bytes = L.total;                                                                                              \
    return GBP_OK;                                                                                                 \
  }                                                                                                                \
  int particles_power_n##NN(const float* x, const float* y, const float* z, const float* w, int64_t n, float xmin, \
                            float ymin, float zmin, float inv_cell, const gbp_job* job, gbp_fft_plan plan,        \
                            gbp_bins bins, int mas, int ells, int tx, int ty, void* spectrum, double* sums_out,    \
                            long long* nmodes_out, double* ksum_out, gbp_deposit_stats* stats_out,                 \
                            void* workspace, size_t ws_bytes, cudaStream_t st) {                                   \
    DepGeom g{};                                                                                                   \
    g.x = x; g.y = y; g.z = z; g.w = w; g.n = n;                                                                   \
    g.ox = xmin; g.oy = ymin; g.oz = zmin; g.inv_cell = inv_cell;                                                  \
    g.N = NN;                                                                                                      \
    g.job = job;                                                                                                   \
    g.cap = n;                                                                                                     \
    return particles_power_n<NN>(g, n, plan, bins, mas, ells, tx, ty, spectrum, sums_out, nmodes_out, ksum_out,   \
                                 stats_out, workspace, ws_bytes, st);                                              \
  }                                                                                                                \
  }
