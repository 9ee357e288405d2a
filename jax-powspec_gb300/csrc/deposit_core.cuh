// Deposit internals shared by the mesh deposit (deposit.cu) and the deposit
// fused with the z pass of the FFT (depfft.cu): geometry, B-spline and
// reference-compatible stencils, tile bucketing (count / scan / scatter),
// int64 fixed-point helpers, statistics and workspace layout.
#pragma once

#include <algorithm>
#include <cmath>

#include <cub/device/device_scan.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/transform_iterator.h>

#include "gbp_internal.cuh"

namespace gbp {
namespace {

constexpr int TILE = 16;              // tile edge (cells); >= widest stencil (5)
constexpr int TILE3 = TILE * TILE * TILE;
constexpr int DEP_THREADS = 256;
constexpr int CNT_THREADS = 256;
constexpr int CNT_ITEMS = 2;          // particles per thread in count/scatter
constexpr float MAX_ABS_U = 1073741824.0f;  // |u| < 2^30 cells, else dropped
constexpr int kCubeTiles[3] = {TILE, TILE, TILE};   // mesh deposit: 16^3-cell tiles
// Per-tile counters sit one 128-byte line apart: the bucketing's global
// atomics on different tiles never contend for one L2 line.
constexpr int CSTRIDE = 32;

struct DepGeom {
  const float* x;
  const float* y;
  const float* z;
  const float* w;
  long long n;
  float ox, oy, oz, inv_cell;
  int N;
  int wrap;         // compat modes only
  int td[3];        // tile edge per axis (x, y, z)
  int ts[3];        // log2(td) when td is a power of two, else -1
  int nt[3];        // tiles per axis
  int vec_ok;       // mesh pointers are 16-byte aligned (float4 tile stores allowed)
  const gbp_job* job;  // non-null: particles, n and box geometry are read from here
  long long cap;       // job mode: the capacity the launches were sized for
  unsigned tcap;       // > 0: buckets of a fixed capacity, tile t's at entry t * tcap (fill path)
};

// Job mode: the particle pointers, count and box geometry come from a
// gbp_job in device memory (one broadcast load per thread), so the launch
// parameters do not depend on the mock.
__device__ __forceinline__ void resolve_job(DepGeom& g) {
  if (!g.job) return;
  const gbp_job j = *g.job;
  g.x = j.x; g.y = j.y; g.z = j.z; g.w = j.w;
  g.n = j.n < 0 ? 0 : (j.n > g.cap ? g.cap : j.n);   // the buckets hold `cap` particles at most
  g.ox = j.xmin; g.oy = j.ymin; g.oz = j.zmin; g.inv_cell = j.inv_cell;
}

// Node index reduced into [0, N).  Stencil nodes lie within a few cells of
// [0, N); tiny meshes fall back to the general modulo.
__device__ __forceinline__ int wrapn(int n, int N) {
  if (N < 8) return pmod(n, N);
  return n < 0 ? n + N : (n >= N ? n - N : n);
}

__device__ __forceinline__ int tile_of(const DepGeom& g, int ax, int node) {
  return g.ts[ax] >= 0 ? (node >> g.ts[ax]) : node / g.td[ax];
}

template <int MAS, int CM>
struct Scheme {
  static constexpr int R = CM ? 2 : MAS;    // nodes per axis
};

// One axis of one particle: nodes first .. first+R-1 (not yet wrapped), their
// weights, and a mask of nodes that are valid scatter indices (only the
// reference-compat variants ever drop nodes).
template <int R>
struct Axis {
  int first;
  unsigned vmask;
  float w[R];
};

// B-spline of order MAS with nodes at integer grid coordinates (the
// reference's node convention: node i sits at xmin + i*H).  `half` shifts
// the particle by +half a cell (the second, interlaced grid).  NC > 0: the
// mesh side as a power-of-two constant (the cell index wraps with a mask,
// the same value as pmod for every int).
template <int MAS, int NC = 0>
__device__ __forceinline__ void axis_bspline(float u, int N, int half, Axis<MAS>& a) {
  static_assert(NC == 0 || (NC & (NC - 1)) == 0, "NC is a power of two");
  const float fu = floorf(u);
  float d = __fsub_rn(u, fu);                 // exact, in [0, 1)
  const int i0 = __float2int_rz(fu);
  int i = NC ? (i0 & (NC - 1)) : wrap_index(i0, N);
  if (half) {
    d = __fadd_rn(d, 0.5f);
    if (d >= 1.0f) { d = __fsub_rn(d, 1.0f); i += 1; }
  }
  a.vmask = (1u << MAS) - 1u;
  if constexpr (MAS == GBP_NGP) {
    a.first = i + (d >= 0.5f ? 1 : 0);
    a.w[0] = 1.0f;
  } else if constexpr (MAS == GBP_CIC) {
    a.first = i;
    a.w[0] = __fsub_rn(1.0f, d);
    a.w[1] = d;
  } else if constexpr (MAS == GBP_TSC) {
    const int up = d >= 0.5f ? 1 : 0;           // nearest node is i+up
    const float s = up ? __fsub_rn(d, 1.0f) : d;  // offset from it, [-0.5, 0.5)
    a.first = i + up - 1;
    const float l = 0.5f - s, r = 0.5f + s;
    a.w[0] = 0.5f * l * l;
    a.w[1] = 0.75f - s * s;
    a.w[2] = 0.5f * r * r;
  } else {                                      // PCS (cubic B-spline)
    const float t = d, m = 1.0f - d;
    const float c6 = 1.0f / 6.0f;
    a.first = i - 1;
    a.w[0] = m * m * m * c6;
    a.w[1] = (4.0f - 6.0f * t * t + 3.0f * t * t * t) * c6;
    a.w[2] = (4.0f - 6.0f * m * m + 3.0f * m * m * m) * c6;
    a.w[3] = t * t * t * c6;
  }
}

// The reference CIC along one axis, bit for bit.
//   CM == GBP_COMPAT_VEC follows src/mas.py:103-140 (cic_mas_vec): truncating
//     int32 cast (:107), fraction (:111), wrap = floor-mod of ix+1 (:121);
//     no-wrap zeroes ixp but tests the zeroed value, so the fraction is kept
//     (:125-126).
//   CM == GBP_COMPAT_SCAN follows src/mas.py:44-67 (cic_mas): mdx is computed
//     before the wrap branch (:56); wrap subtracts n once (:24); no-wrap sets
//     both ixp and the fraction to zero (:34).
// Then the scatter's index rule: -N <= idx < 0 maps to idx+N, anything else
// outside [0, N) drops the update (jax .at[].add default mode).
template <int CM>
__device__ __forceinline__ void axis_compat(float u, int N, int wrap, Axis<2>& a) {
  const int ix = __float2int_rz(u);
  const float d = __fsub_rn(u, __int2float_rn(ix));
  const float m = __fsub_rn(1.0f, d);
  int ixp = ix + 1;
  float dh = d;
  if (CM == GBP_COMPAT_VEC) {
    if (wrap) ixp = wrap_index(ixp, N);         // = pmod(ixp + N, N): |ixp| < 2^30 + 1
    else if (ixp >= N) ixp = 0;
  } else {
    if (wrap) { if (ixp >= N) ixp -= N; }
    else if (ixp >= N) { ixp = 0; dh = 0.0f; }
  }
  const bool lo_ok = ix >= -N && ix < N;
  const bool hi_ok = ixp >= -N && ixp < N;
  const int lo = ix < 0 ? ix + N : ix;
  const int hi = ixp < 0 ? ixp + N : ixp;
  // When both are valid, hi == lo + 1 (mod N) in every branch above.
  a.first = lo_ok ? lo : hi - 1;
  a.vmask = (lo_ok ? 1u : 0u) | (hi_ok ? 2u : 0u);
  a.w[0] = m;
  a.w[1] = dh;
}

template <int MAS, int CM, int NC = 0>
__device__ __forceinline__ void make_axis(const DepGeom& g, float u, int grid, Axis<Scheme<MAS, CM>::R>& a) {
  if constexpr (CM != 0) axis_compat<CM>(u, g.N, g.wrap, a);
  else axis_bspline<MAS, NC>(u, g.N, grid, a);
}

// The particles of one thread in count/scatter: loads issued together.
struct Batch {
  float x[CNT_ITEMS], y[CNT_ITEMS], z[CNT_ITEMS], w[CNT_ITEMS];
  bool in[CNT_ITEMS];
};

__device__ __forceinline__ void load_batch(const DepGeom& g, Batch& b, long long blk) {
  const long long base = blk * CNT_THREADS * CNT_ITEMS + threadIdx.x;
#pragma unroll
  for (int k = 0; k < CNT_ITEMS; ++k) {
    const long long i = base + (long long)k * CNT_THREADS;
    b.in[k] = i < g.n;
    if (b.in[k]) {
      b.x[k] = __ldcs(g.x + i);
      b.y[k] = __ldcs(g.y + i);
      b.z[k] = __ldcs(g.z + i);
      b.w[k] = g.w ? __ldcs(g.w + i) : 1.0f;
    }
  }
}

// Grid coordinate of a particle; false if it must be dropped (non-finite, or
// so far outside the box that int32 cells would overflow).
__device__ __forceinline__ bool grid_coords(const DepGeom& g, float x, float y, float z, float u[3]) {
  u[0] = __fmul_rn(__fsub_rn(x, g.ox), g.inv_cell);
  u[1] = __fmul_rn(__fsub_rn(y, g.oy), g.inv_cell);
  u[2] = __fmul_rn(__fsub_rn(z, g.oz), g.inv_cell);
  return fabsf(u[0]) < MAX_ABS_U && fabsf(u[1]) < MAX_ABS_U && fabsf(u[2]) < MAX_ABS_U;  // false for NaN
}

// Distinct tiles touched along one axis by the valid nodes of all grids
// (at most 3 because a stencil spans at most 5 nodes and tiles are wider).
template <int MAS, int G, int CM>
__device__ __forceinline__ int axis_tiles(const DepGeom& g, int ax, float u, int& t0, int& t1, int& t2) {
  constexpr int R = Scheme<MAS, CM>::R;
  constexpr int W = R + (G - 1);
  Axis<R> a;
  make_axis<MAS, CM>(g, u, 0, a);
  int lo = a.first, hi = a.first + R - 1;
  if constexpr (CM != 0) {
    if (a.vmask == 0u) return 0;
    if (!(a.vmask & 1u)) lo += 1;
    if (!(a.vmask & 2u)) hi -= 1;
  }
  if constexpr (G == 2) {
    Axis<R> b;
    make_axis<MAS, CM>(g, u, 1, b);
    hi = b.first + R - 1;                        // b.first is a.first or a.first + 1
  }
  int nt = 0;
  t0 = t1 = t2 = -1;
#pragma unroll
  for (int k = 0; k < W; ++k) {
    if (lo + k > hi) break;
    const int t = tile_of(g, ax, wrapn(lo + k, g.N));
    if (t == t0 || t == t1 || t == t2) continue;
    if (nt == 0) t0 = t; else if (nt == 1) t1 = t; else t2 = t;
    ++nt;
  }
  return nt;
}

__device__ __forceinline__ int pick3(int k, int a, int b, int c) { return k == 0 ? a : (k == 1 ? b : c); }

__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ ff warp_ff_sum(ff v) {
  for (int o = 16; o > 0; o >>= 1) {
    ff t{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = ff_add(v, t);
  }
  return v;
}

struct DepCounters {           // zeroed by one memset per call
  unsigned int maxw_bits;
  unsigned int overflow;       // fill path: some tile has more entries than its bucket holds
  unsigned int pad_[2];
};

// Block reductions of the weight statistics in a fixed order (deterministic
// partials per particle block), and the global max |w|.
__device__ __forceinline__ void flush_block_stats(float maxw, ff sw, ff sw2, unsigned kept, unsigned bad,
                                                  DepCounters* ctr, float4* block_stats, uint2* block_counts) {
  __shared__ float s_max[CNT_THREADS / 32];
  __shared__ ff s_sw[CNT_THREADS / 32], s_sw2[CNT_THREADS / 32];
  __shared__ unsigned s_kept, s_bad;
  if (threadIdx.x == 0) { s_kept = 0; s_bad = 0; }
  __syncthreads();
  maxw = warp_max(maxw);
  sw = warp_ff_sum(sw);
  sw2 = warp_ff_sum(sw2);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s_max[wid] = maxw; s_sw[wid] = sw; s_sw2[wid] = sw2; }
  if (kept) atomicAdd(&s_kept, kept);
  if (bad) atomicAdd(&s_bad, bad);
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    ff a{0.f, 0.f}, b{0.f, 0.f};
    for (int k = 0; k < CNT_THREADS / 32; ++k) {
      m = fmaxf(m, s_max[k]);
      a = ff_add(a, s_sw[k]);
      b = ff_add(b, s_sw2[k]);
    }
    block_stats[blockIdx.x] = make_float4(a.hi, a.lo, b.hi, b.lo);
    block_counts[blockIdx.x] = make_uint2(s_kept, s_bad);
    if (m > 0.f) atomicMax(&ctr->maxw_bits, __float_as_uint(m));
  }
}

// Pass 1: tile occupancy counts + weight statistics.
template <int MAS, int G, int CM>
__global__ void __launch_bounds__(CNT_THREADS)
count_kernel(DepGeom gp, unsigned* __restrict__ counts, DepCounters* ctr, float4* block_stats,
             uint2* block_counts) {
  pdl_wait();
  DepGeom g = gp;
  resolve_job(g);
  float maxw = 0.0f;
  ff sw{0.f, 0.f}, sw2{0.f, 0.f};
  unsigned kept = 0, bad = 0;
  Batch bt;
  load_batch(g, bt, blockIdx.x);
#pragma unroll
  for (int k = 0; k < CNT_ITEMS; ++k) {
    if (!bt.in[k]) continue;
    float u[3];
    const float w = bt.w[k];
    if (!grid_coords(g, bt.x[k], bt.y[k], bt.z[k], u)) { ++bad; continue; }
    int x0, x1, x2, y0, y1, y2, z0, z1, z2;
    const int nx = axis_tiles<MAS, G, CM>(g, 0, u[0], x0, x1, x2);
    const int ny = axis_tiles<MAS, G, CM>(g, 1, u[1], y0, y1, y2);
    const int nz = axis_tiles<MAS, G, CM>(g, 2, u[2], z0, z1, z2);
    if (nx * ny * nz == 0) continue;
    ++kept;
    for (int a = 0; a < nx; ++a)
      for (int b = 0; b < ny; ++b)
        for (int c = 0; c < nz; ++c)
          atomicAdd(&counts[((pick3(a, x0, x1, x2) * g.nt[1] + pick3(b, y0, y1, y2)) * g.nt[2] +
                             pick3(c, z0, z1, z2)) * CSTRIDE], 1u);
    maxw = fmaxf(maxw, fabsf(w));
    sw = ff_add_f(sw, w);
    sw2 = ff_add_f(sw2, __fmul_rn(w, w));
  }
  flush_block_stats(maxw, sw, sw2, kept, bad, ctr, block_stats, block_counts);
}

// Passes 1 and 3 at once (fill path: buckets of a fixed capacity g.tcap, tile
// t's at entry t * tcap).  The count of tile t that a particle's atomic
// returns is also its slot in t's bucket, so the entry is written right away;
// a slot beyond the capacity is not written and raises ctr->overflow, after
// which the scan and scatter passes (they run only then) rebuild all buckets
// packed, from these counts: every attempt was counted.  The statistics are
// those of count_kernel, over the same particle blocks.  Registers for 5
// CTAs per SM: its returning atomics want warps in flight (0.151 -> 0.142 ms
// for 4 Mi particles at 512^3 against 4 CTAs per SM).
template <int MAS, int G, int CM>
__global__ void __launch_bounds__(CNT_THREADS, 5)
fill_kernel(DepGeom gp, unsigned* __restrict__ counts, float4* __restrict__ entries, DepCounters* ctr,
            float4* block_stats, uint2* block_counts) {
  pdl_wait();
  DepGeom g = gp;
  resolve_job(g);
  const unsigned tcap = g.tcap;
  float maxw = 0.0f;
  ff sw{0.f, 0.f}, sw2{0.f, 0.f};
  unsigned kept = 0, bad = 0;
  bool over = false;
  Batch bt;
  load_batch(g, bt, blockIdx.x);
#pragma unroll
  for (int k = 0; k < CNT_ITEMS; ++k) {
    if (!bt.in[k]) continue;
    float u[3];
    const float w = bt.w[k];
    if (!grid_coords(g, bt.x[k], bt.y[k], bt.z[k], u)) { ++bad; continue; }
    int x0, x1, x2, y0, y1, y2, z0, z1, z2;
    const int nx = axis_tiles<MAS, G, CM>(g, 0, u[0], x0, x1, x2);
    const int ny = axis_tiles<MAS, G, CM>(g, 1, u[1], y0, y1, y2);
    const int nz = axis_tiles<MAS, G, CM>(g, 2, u[2], z0, z1, z2);
    if (nx * ny * nz == 0) continue;
    ++kept;
    const float4 e = make_float4(u[0], u[1], u[2], w);
    if (nx <= 2 && ny <= 2 && nz <= 2) {
      // at most 2 x 2 x 2 tiles: all slots claimed at once (the returning atomics overlap)
      int tt[8];
      unsigned slot[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int a = q >> 2, b = (q >> 1) & 1, c = q & 1;
        tt[q] = (a < nx && b < ny && c < nz)
                    ? ((a ? x1 : x0) * g.nt[1] + (b ? y1 : y0)) * g.nt[2] + (c ? z1 : z0) : -1;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (tt[q] >= 0) slot[q] = atomicAdd(&counts[tt[q] * CSTRIDE], 1u);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (tt[q] >= 0) {
          if (slot[q] < tcap) entries[(unsigned)tt[q] * tcap + slot[q]] = e;
          else over = true;
        }
    } else {
      for (int a = 0; a < nx; ++a)
        for (int b = 0; b < ny; ++b)
          for (int c = 0; c < nz; ++c) {
            const int t = (pick3(a, x0, x1, x2) * g.nt[1] + pick3(b, y0, y1, y2)) * g.nt[2] + pick3(c, z0, z1, z2);
            const unsigned slot = atomicAdd(&counts[t * CSTRIDE], 1u);
            if (slot < tcap) entries[(unsigned)t * tcap + slot] = e;
            else over = true;
          }
    }
    maxw = fmaxf(maxw, fabsf(w));
    sw = ff_add_f(sw, w);
    sw2 = ff_add_f(sw2, __fmul_rn(w, w));
  }
  if (over) atomicOr(&ctr->overflow, 1u);
  flush_block_stats(maxw, sw, sw2, kept, bad, ctr, block_stats, block_counts);
}

// Pass 2 of the fill path, run only when a bucket overflowed (one CTA:
// otherwise it returns at once): exclusive scan of the tile counts.
constexpr int FSCAN_THREADS = 1024;
__global__ void __launch_bounds__(FSCAN_THREADS)
gated_scan_kernel(const unsigned* __restrict__ counts, unsigned* __restrict__ offsets, int ntiles,
                  const DepCounters* ctr) {
  pdl_wait();
  if (ctr->overflow == 0u) return;
  __shared__ unsigned s_warp[FSCAN_THREADS / 32];
  const int per = (ntiles + FSCAN_THREADS - 1) / FSCAN_THREADS;
  const int a = min(ntiles, (int)threadIdx.x * per), b = min(ntiles, a + per);
  unsigned sum = 0;
  for (int i = a; i < b; ++i) sum += counts[(long long)i * CSTRIDE];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned inc = sum;                                  // inclusive scan within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    unsigned v = s_warp[lane], w = v;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    s_warp[lane] = w - v;                              // exclusive prefix of the warp totals
  }
  __syncthreads();
  unsigned run = s_warp[wid] + inc - sum;
  for (int i = a; i < b; ++i) {
    offsets[i] = run;
    run += counts[(long long)i * CSTRIDE];
  }
}

// First entry and end of tile t's bucket: fixed-capacity buckets unless the
// fill path overflowed (then, as on the count path, packed at the scanned
// offsets); the counts are the same on both paths.
__device__ __forceinline__ void tile_range(const DepGeom& g, int t, const unsigned* counts, const unsigned* offsets,
                                           const DepCounters* ctr, unsigned& beg, unsigned& end) {
  const unsigned c = counts[(long long)t * CSTRIDE];
  beg = (g.tcap && ctr->overflow == 0u) ? (unsigned)t * g.tcap : offsets[t];
  end = beg + c;
}

// Pass 3: append (u_x, u_y, u_z, w) to every touched tile's bucket.
template <int MAS, int G, int CM>
__global__ void __launch_bounds__(CNT_THREADS, 4)
scatter_kernel(DepGeom gp, const unsigned* __restrict__ offsets, unsigned* __restrict__ fills,
               float4* __restrict__ entries, const DepCounters* gate) {
  pdl_wait();
  if (gate && gate->overflow == 0u) return;            // fill path: the buckets are complete
  DepGeom g = gp;
  resolve_job(g);
  for (long long blk = blockIdx.x; blk * (CNT_THREADS * CNT_ITEMS) < g.n; blk += gridDim.x) {
    Batch bt;
    load_batch(g, bt, blk);
#pragma unroll
    for (int k = 0; k < CNT_ITEMS; ++k) {
      if (!bt.in[k]) continue;
      float u[3];
      const float w = bt.w[k];
      if (!grid_coords(g, bt.x[k], bt.y[k], bt.z[k], u)) continue;
      int x0, x1, x2, y0, y1, y2, z0, z1, z2;
      const int nx = axis_tiles<MAS, G, CM>(g, 0, u[0], x0, x1, x2);
      const int ny = axis_tiles<MAS, G, CM>(g, 1, u[1], y0, y1, y2);
      const int nz = axis_tiles<MAS, G, CM>(g, 2, u[2], z0, z1, z2);
      if (nx * ny * nz == 0) continue;
      const float4 e = make_float4(u[0], u[1], u[2], w);
      if (nx <= 2 && ny <= 2 && nz <= 2) {
        // at most 2 x 2 x 2 tiles (every tile at least as wide as the stencil): all slots claimed at
        // once, so the returning atomics of one particle overlap instead of forming a chain
        int tt[8];
        unsigned base[8], slot[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int a = q >> 2, b = (q >> 1) & 1, c = q & 1;
          tt[q] = (a < nx && b < ny && c < nz)
                      ? ((a ? x1 : x0) * g.nt[1] + (b ? y1 : y0)) * g.nt[2] + (c ? z1 : z0) : -1;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (tt[q] >= 0) {
            base[q] = offsets[tt[q]];
            slot[q] = atomicAdd(&fills[tt[q] * CSTRIDE], 1u);
          }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (tt[q] >= 0) entries[base[q] + slot[q]] = e;
      } else {
        for (int a = 0; a < nx; ++a)
          for (int b = 0; b < ny; ++b)
            for (int c = 0; c < nz; ++c) {
              const int t = (pick3(a, x0, x1, x2) * g.nt[1] + pick3(b, y0, y1, y2)) * g.nt[2] + pick3(c, z0, z1, z2);
              entries[offsets[t] + atomicAdd(&fills[t * CSTRIDE], 1u)] = e;
            }
      }
    }
  }
}

// Fixed-point exponent s: one contribution w * W (|W| <= 1, or <= 8 for the
// reference CIC, whose fractions can leave [0,1) off the box) is an integer
// below 2^30 in magnitude, so it fits one 32-bit atomic on the low word; the
// 64-bit cell sums hold n * 2^30 without overflow for any n < 2^32.
// Float32 and integer operations only (GB300's FP64 rate is tiny).
__device__ __forceinline__ int fixed_scale_exp(unsigned maxw_bits, int compat) {
  const float maxw = __uint_as_float(maxw_bits);
  if (!(maxw > 0.0f) || !(maxw < 3.0e38f)) return 0;
  int ew;
  frexpf(maxw, &ew);                            // maxw < 2^ew
  const int s = 30 - ew - (compat ? 3 : 0);
  return s < -100 ? -100 : (s > 100 ? 100 : s);
}

// int64 fixed-point value -> float32 (two exact 32-bit halves, one rounding in the FMA).
__device__ __forceinline__ float fixed_to_float(long long q, float inv_sc) {
  const int hi = (int)(q >> 32);
  const unsigned lo = (unsigned)(q & 0xffffffffull);
  const float v = __fmaf_rn(__int2float_rn(hi), 4294967296.0f, __uint2float_rn(lo));
  return __fmul_rn(v, inv_sc);
}

// Local (in-tile) coordinate of stencil node r of an axis, or -1.
template <int R>
__device__ __forceinline__ void local_nodes(const Axis<R>& a, int N, int t0, int ext, int (&l)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int c = wrapn(a.first + r, N) - t0;
    l[r] = (((a.vmask >> r) & 1u) && c >= 0 && c < ext) ? c : -1;
  }
}

// Pass 5: fold the per-block statistics and the per-tile mass totals into
// gbp_deposit_stats.  Float partials are folded in a fixed order; integer
// totals are exact in any order.
constexpr int STATS_THREADS = 1024;
__global__ void __launch_bounds__(STATS_THREADS)
stats_kernel(const DepCounters* ctr, const float4* block_stats, const uint2* block_counts, int nblocks,
             const long long* tile_mass, int ntiles, int compat, int G, gbp_deposit_stats* out) {
  pdl_wait();
  __shared__ ff s_a[32], s_b[32];
  __shared__ long long s_m[2][32], s_c[2][32];
  ff a{0.f, 0.f}, b{0.f, 0.f};
  long long kept = 0, bad = 0, m0 = 0, m1 = 0;
  // a thread adds blocks k = tid, tid + blockDim, ... in that order; the loads of SU of them are issued
  // before the adds
  constexpr int SU = 4;
  const int nt = blockDim.x;
  for (int k0 = threadIdx.x; k0 < nblocks; k0 += SU * nt) {
    float4 v[SU];
    uint2 c[SU];
#pragma unroll
    for (int u = 0; u < SU; ++u) {
      const int k = k0 + u * nt;
      v[u] = k < nblocks ? block_stats[k] : make_float4(0.f, 0.f, 0.f, 0.f);
      c[u] = k < nblocks ? block_counts[k] : make_uint2(0u, 0u);
    }
#pragma unroll
    for (int u = 0; u < SU; ++u) {
      if (k0 + u * nt >= nblocks) break;
      a = ff_add(a, ff{v[u].x, v[u].y});
      b = ff_add(b, ff{v[u].z, v[u].w});
      kept += c[u].x;
      bad += c[u].y;
    }
  }
  for (int k0 = threadIdx.x; k0 < ntiles; k0 += SU * nt) {       // integers: any order
#pragma unroll
    for (int u = 0; u < SU; ++u) {
      const int k = k0 + u * nt;
      if (k < ntiles) {
        m0 += tile_mass[k];
        if (G == 2) m1 += tile_mass[ntiles + k];
      }
    }
  }
  a = warp_ff_sum(a);
  b = warp_ff_sum(b);
  for (int o = 16; o > 0; o >>= 1) {
    kept += __shfl_xor_sync(0xffffffffu, kept, o);
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
    m0 += __shfl_xor_sync(0xffffffffu, m0, o);
    m1 += __shfl_xor_sync(0xffffffffu, m1, o);
  }
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_a[wid] = a; s_b[wid] = b;
    s_c[0][wid] = kept; s_c[1][wid] = bad;
    s_m[0][wid] = m0; s_m[1][wid] = m1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ff ta{0.f, 0.f}, tb{0.f, 0.f};
    long long tk = 0, tbad = 0, tm[2] = {0, 0};
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      ta = ff_add(ta, s_a[k]);
      tb = ff_add(tb, s_b[k]);
      tk += s_c[0][k]; tbad += s_c[1][k];
      tm[0] += s_m[0][k]; tm[1] += s_m[1][k];
    }
    const int s = fixed_scale_exp(ctr->maxw_bits, compat);
    const double inv = ldexp(1.0, -s);
    for (int grid = 0; grid < 2; ++grid) out->mass[grid] = grid < G ? (double)tm[grid] * inv : 0.0;
    out->sum_w = (double)ta.hi + (double)ta.lo;
    out->sum_w2 = (double)tb.hi + (double)tb.lo;
    out->n_kept = tk;
    out->n_nonfinite = tbad;
    out->scale_exp = s;
    out->flags = ctr->overflow ? GBP_STATS_REFILLED : 0;
  }
}

struct DepLayout {
  int td[3], ts[3], nt[3], ntiles, maxrep, nblocks;
  unsigned tcap;        // fill path: entries per bucket (0: count path)
  size_t nentries;      // entries the bucket buffer holds
  size_t scan_bytes;
  size_t total;
};

// Blocks of the fill path's fallback scatter (a grid-stride loop; when no
// bucket overflowed they return at once).
constexpr int FILL_SCATTER_BLOCKS = 1216;

// Bytes at the start of the workspace that one memset clears per call: the
// counters, the tiles' entry counts and their fill counters (adjacent).
inline size_t zeroed_bytes(const DepLayout& L) {
  return align256(sizeof(DepCounters)) + 2 * align256((size_t)L.ntiles * CSTRIDE * sizeof(unsigned));
}

struct StrideLoad {
  const unsigned* p;
  __host__ __device__ unsigned operator()(int i) const { return p[(long long)i * CSTRIDE]; }
};

inline thrust::transform_iterator<StrideLoad, thrust::counting_iterator<int>> strided_counts(const unsigned* p) {
  return thrust::make_transform_iterator(thrust::counting_iterator<int>(0), StrideLoad{p});
}

// Largest number of distinct tiles a run of `width` consecutive nodes can
// touch along one periodic axis (exact, by enumeration).
int max_tiles_axis(int N, int tdim, int width) {
  int best = 0;
  for (int s = 0; s < N; ++s) {
    int seen[8], ns = 0;
    for (int r = 0; r < width; ++r) {
      const int t = ((s + r) % N) / tdim;
      bool dup = false;
      for (int k = 0; k < ns; ++k) dup = dup || seen[k] == t;
      if (!dup && ns < 8) seen[ns++] = t;
    }
    best = ns > best ? ns : best;
  }
  return best;
}

// Tiles of td[0] x td[1] x td[2] cells (each at most N); every particle goes
// to the bucket of each tile its stencil (all grids) touches.  fill: buckets
// of a fixed capacity, twice the mean fill m of a uniform catalogue of n
// particles plus 64 (a span of `width` nodes reaches the next tile along an
// axis with probability (width - 1) / td), so that one pass fills them
// unless the catalogue is strongly clustered; the count path when m < 32
// (few particles per tile: small buffers matter more than the pass).  Wider
// buckets cost the one pass time: the same entries written over a larger
// range (3 m + 64 instead of 2 m + 64: 0.169 against 0.147 ms for 4 Mi
// particles at 512^3).
int deposit_layout(int64_t n, int N, int mas, int interlace, int compat, const int (&tile)[3], DepLayout& L,
                   bool fill = false) {
  if (N < 1 || N > 4096) return GBP_ERR_INVALID;
  if (n < 0) return GBP_ERR_INVALID;
  if (mas < GBP_NGP || mas > GBP_PCS) return GBP_ERR_INVALID;
  if (compat < 0 || compat > GBP_COMPAT_SCAN) return GBP_ERR_INVALID;
  if (compat && (mas != GBP_CIC || interlace)) return GBP_ERR_INVALID;
  const int R = compat ? 2 : mas;
  const int width = R + (interlace ? 1 : 0);
  L.ntiles = 1;
  L.maxrep = 1;
  for (int a = 0; a < 3; ++a) {
    L.td[a] = N < tile[a] ? N : tile[a];
    L.ts[a] = (L.td[a] & (L.td[a] - 1)) == 0 ? __builtin_ctz(L.td[a]) : -1;
    L.nt[a] = (N + L.td[a] - 1) / L.td[a];
    const int m = max_tiles_axis(N, L.td[a], width);
    if (m > 3) return GBP_ERR_UNSUPPORTED;
    L.ntiles *= L.nt[a];
    L.maxrep *= m;
  }
  if ((double)n * L.maxrep >= 4294967295.0) return GBP_ERR_UNSUPPORTED;
  L.nblocks = (int)((n + (long long)CNT_THREADS * CNT_ITEMS - 1) / ((long long)CNT_THREADS * CNT_ITEMS));
  L.tcap = 0;
  L.nentries = (size_t)n * L.maxrep + 1;
  if (fill && n > 0) {
    double rep = 1.0;
    for (int a = 0; a < 3; ++a)
      if (L.td[a] < N) rep *= 1.0 + (double)(width - 1) / (double)L.td[a];
    const double mean = (double)n * rep / (double)L.ntiles;
    const double cap = 4.0 * std::ceil((2.0 * mean + 64.0) / 4.0);
    if (mean >= 32.0 && cap * (double)L.ntiles < 4294967295.0) {
      L.tcap = (unsigned)cap;
      L.nentries = std::max(L.nentries, (size_t)L.tcap * (size_t)L.ntiles + 1);
    }
  }
  L.scan_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, L.scan_bytes, strided_counts(nullptr), (unsigned*)nullptr, L.ntiles);
  const size_t nbl = (size_t)(L.nblocks > 0 ? L.nblocks : 1);
  L.total = zeroed_bytes(L) + align256((size_t)L.ntiles * 4) + align256(nbl * sizeof(float4)) +
            align256(nbl * sizeof(uint2)) + align256((size_t)L.ntiles * 2 * sizeof(long long)) +
            align256(L.nentries * sizeof(float4)) + align256(L.scan_bytes);
  return GBP_OK;
}

// Workspace slices shared by both deposit paths.
struct DepBuffers {
  DepCounters* ctr;
  unsigned* counts;      // [ntiles * CSTRIDE] entries per tile (count pass)
  unsigned* fills;       // [ntiles * CSTRIDE] entries written so far (scatter pass)
  unsigned* offsets;     // [ntiles] first entry of each tile (exclusive scan of the counts)
  float4* block_stats;
  uint2* block_counts;
  long long* tile_mass;
  float4* entries;
  void* scan_tmp;
};

inline DepBuffers carve_deposit(void* workspace, const DepLayout& L) {
  Carver cv(workspace);
  DepBuffers b;
  const int nbl = L.nblocks > 0 ? L.nblocks : 1;
  b.ctr = cv.take<DepCounters>(1);
  b.counts = cv.take<unsigned>((size_t)L.ntiles * CSTRIDE);
  b.fills = cv.take<unsigned>((size_t)L.ntiles * CSTRIDE);
  b.offsets = cv.take<unsigned>(L.ntiles);
  b.block_stats = cv.take<float4>(nbl);
  b.block_counts = cv.take<uint2>(nbl);
  b.tile_mass = cv.take<long long>((size_t)L.ntiles * 2);
  b.entries = cv.take<float4>(L.nentries);
  b.scan_tmp = cv.take<char>(L.scan_bytes);
  return b;
}

// Passes 1-3: bucket the particles by tile (the first zeroed_bytes(L) of the
// workspace must be zero on entry).
template <int MAS, int G, int CM>
int bucket_particles(const DepGeom& g, const DepLayout& L, const DepBuffers& b, cudaStream_t st) {
  if (L.tcap) {
    // fill path: one pass; the scan and the scatter return at once unless a bucket overflowed
    if (L.nblocks > 0) {
      GBP_TRACE("deposit_fill", st);
      GBP_CUDA_TRY(launch_pdl(fill_kernel<MAS, G, CM>, dim3(L.nblocks), dim3(CNT_THREADS), 0, st, g, b.counts,
                              b.entries, b.ctr, b.block_stats, b.block_counts));
    }
    {
      GBP_TRACE("deposit_scan", st);
      GBP_CUDA_TRY(launch_pdl(gated_scan_kernel, dim3(1), dim3(FSCAN_THREADS), 0, st, b.counts, b.offsets,
                              L.ntiles, b.ctr));
    }
    if (L.nblocks > 0) {
      GBP_TRACE("deposit_scatter", st);
      GBP_CUDA_TRY(launch_pdl(scatter_kernel<MAS, G, CM>, dim3(std::min(L.nblocks, FILL_SCATTER_BLOCKS)),
                              dim3(CNT_THREADS), 0, st, g, b.offsets, b.fills, b.entries,
                              static_cast<const DepCounters*>(b.ctr)));
    }
    return GBP_OK;
  }
  if (L.nblocks > 0) {
    GBP_TRACE("deposit_count", st);
    GBP_CUDA_TRY(launch_pdl(count_kernel<MAS, G, CM>, dim3(L.nblocks), dim3(CNT_THREADS), 0, st, g, b.counts, b.ctr,
                            b.block_stats, b.block_counts));
  }
  {
    GBP_TRACE("deposit_scan", st);
    size_t scan_bytes = L.scan_bytes;
    GBP_CUDA_TRY(cub::DeviceScan::ExclusiveSum(b.scan_tmp, scan_bytes, strided_counts(b.counts), b.offsets,
                                               L.ntiles, st));
  }
  if (L.nblocks > 0) {
    GBP_TRACE("deposit_scatter", st);
    GBP_CUDA_TRY(launch_pdl(scatter_kernel<MAS, G, CM>, dim3(L.nblocks), dim3(CNT_THREADS), 0, st, g, b.offsets,
                            b.fills, b.entries, static_cast<const DepCounters*>(nullptr)));
  }
  return GBP_OK;
}

inline int deposit_stats(const DepBuffers& b, const DepLayout& L, int compat, int G, gbp_deposit_stats* out,
                         cudaStream_t st) {
  GBP_TRACE("deposit_stats", st);
  GBP_CUDA_TRY(launch_pdl(stats_kernel, dim3(1), dim3(STATS_THREADS), 0, st, static_cast<const DepCounters*>(b.ctr),
                          static_cast<const float4*>(b.block_stats), static_cast<const uint2*>(b.block_counts),
                          L.nblocks, static_cast<const long long*>(b.tile_mass), L.ntiles, compat, G, out));
  return GBP_OK;
}

}  // namespace
}  // namespace gbp
