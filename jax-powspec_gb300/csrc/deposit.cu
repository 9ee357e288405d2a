// Particle -> mesh deposit (NGP / CIC / TSC / PCS, optional interlacing, and
// the two reference-compatible CIC variants of src/mas.py).
//
// Pipeline (all on one stream, deterministic):
//   1. count_kernel    every particle adds 1 to each mesh tile (16^3 cells)
//                      that its stencil touches (integer atomics: the counts
//                      do not depend on order), and reduces max|w|, sum w and
//                      sum w^2 per block.
//   2. cub scan        exclusive prefix sum of the tile counts -> offsets.
//   3. scatter_kernel  every particle appends (u_x, u_y, u_z, w) to each
//                      touched tile's bucket: a one-digit radix sort of the
//                      particles by tile, replicated across tile faces.
//                      (Per-tile counters sit one L2 line apart.)
//   4. deposit_kernel  one CTA per tile accumulates its bucket in shared
//                      memory in int64 fixed point (scale 2^s fixed by max|w|;
//                      each add is a native 32-bit atomic on the low word plus
//                      a carry into the high word), then writes its cells of
//                      the mesh exactly once.
//   5. stats_kernel    folds the per-block partial sums in a fixed order.
//
// With enough particles per tile, passes 1-3 are one: fill_kernel gives
// each tile a bucket of fixed capacity and writes every entry at the slot
// its count atomic returns; scan and scatter (from those counts) run only if
// a bucket overflowed (deposit_core.cuh, deposit_layout).
//
// Integer accumulation makes each cell's sum independent of particle order
// and scheduling, so the mesh is bitwise reproducible; no float atomics are
// used.  Every cell is written once (zeros included): no clearing pass.
// The scheme (MAS order, number of grids, reference-compat variant) is a
// template parameter so every stencil lives in registers.
#include "deposit_core.cuh"

namespace gbp {
namespace {

// Pass 4: one CTA per tile; the grids go one after the other through the
// same shared memory (more CTAs per SM), re-reading the bucket from L2.
//
// Each cell is an int64 kept as separate low and high 32-bit words
// (consecutive cells hit consecutive banks).  A contribution is one native
// 32-bit atomic on the low word, whose return value tells whether it carried
// into the high word, which then gets the (rare) second atomic.  The integer
// sums are exact whatever the order of the adds.
template <int MAS, int G, int CM>
__global__ void __launch_bounds__(DEP_THREADS)
deposit_kernel(DepGeom g, const float4* __restrict__ entries, const unsigned* __restrict__ counts,
               const unsigned* __restrict__ offsets, const DepCounters* ctr, const float* __restrict__ mesh_in,
               float* __restrict__ mesh_out, long long* __restrict__ tile_mass) {
  pdl_wait();
  constexpr int R = Scheme<MAS, CM>::R;
  extern __shared__ __align__(16) unsigned acc32[];
  __shared__ long long s_part[DEP_THREADS / 32];
  unsigned* lo = acc32;
  unsigned* hi = acc32 + TILE3;
  const int t = blockIdx.x;
  const int tz = t % g.nt[2], ty = (t / g.nt[2]) % g.nt[1], tx = t / (g.nt[2] * g.nt[1]);
  const int x0 = tx * g.td[0], y0 = ty * g.td[1], z0 = tz * g.td[2];
  const int ex = min(g.td[0], g.N - x0), ey = min(g.td[1], g.N - y0), ez = min(g.td[2], g.N - z0);

  unsigned beg, end;
  tile_range(g, t, counts, offsets, ctr, beg, end);
  const int s = fixed_scale_exp(ctr->maxw_bits, CM);
  const float sc = ldexpf(1.0f, s);
  const float inv_sc = ldexpf(1.0f, -s);
  const long long N = g.N;
  const long long M = N * N * N;
  const bool vec4 = g.vec_ok && (ez == TILE) && ((g.N & 3) == 0);

  for (int grid = 0; grid < G; ++grid) {
    {
      uint4* a4 = reinterpret_cast<uint4*>(acc32);
      for (int k = threadIdx.x; k < 2 * TILE3 / 4; k += DEP_THREADS) a4[k] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
    for (unsigned i = beg + threadIdx.x; i < end; i += DEP_THREADS) {
      const float4 e = entries[i];
      Axis<R> ax, ay, az;
      make_axis<MAS, CM>(g, e.x, grid, ax);
      make_axis<MAS, CM>(g, e.y, grid, ay);
      make_axis<MAS, CM>(g, e.z, grid, az);
      int lx[R], ly[R], lz[R];
      local_nodes<R>(ax, g.N, x0, ex, lx);
      local_nodes<R>(ay, g.N, y0, ey, ly);
      local_nodes<R>(az, g.N, z0, ez, lz);
#pragma unroll
      for (int rx = 0; rx < R; ++rx) {
        if (lx[rx] < 0) continue;
#pragma unroll
        for (int ry = 0; ry < R; ++ry) {
          if (ly[ry] < 0) continue;
          // src/mas.py:149 (and :76) weights corner (ix, iyp, izp) with
          // mdx*mdy*ddz; the compat variants keep that (wxy_bug).  The
          // product order ((wx*wy)*wz)*w is the reference's.
          const float wxy = __fmul_rn(ax.w[rx], ay.w[ry]);
          const float wxy_bug = __fmul_rn(ax.w[rx], ay.w[0]);
          const int row = (lx[rx] * TILE + ly[ry]) * TILE;
          int q[R];
          unsigned old[R];
#pragma unroll
          for (int rz = 0; rz < R; ++rz) {         // issue the row's low-word adds together
            if (lz[rz] < 0) continue;
            const bool bug = CM != 0 && rx == 0 && ry == 1 && rz == 1;
            const float c = __fmul_rn(__fmul_rn(bug ? wxy_bug : wxy, az.w[rz]), e.w);
            q[rz] = __float2int_rn(__fmul_rn(c, sc));
            old[rz] = atomicAdd(&lo[row + lz[rz]], static_cast<unsigned>(q[rz]));
          }
#pragma unroll
          for (int rz = 0; rz < R; ++rz) {         // then the carries into the high words
            if (lz[rz] < 0) continue;
            const unsigned add = static_cast<unsigned>(q[rz]);
            const int dh = (q[rz] < 0 ? -1 : 0) + (old[rz] + add < old[rz] ? 1 : 0);
            if (dh) atomicAdd(&hi[row + lz[rz]], static_cast<unsigned>(dh));
          }
        }
      }
    }
    __syncthreads();

    // Write this grid's tile once; sum it exactly for the mean density.
    long long part = 0;
    if (vec4) {
      for (int k = threadIdx.x; k < TILE3 / 4; k += DEP_THREADS) {
        const int lz = (k % (TILE / 4)) * 4, ly = (k / (TILE / 4)) % TILE, lx = k / (TILE * TILE / 4);
        if (lx >= ex || ly >= ey) continue;
        const int c0 = (lx * TILE + ly) * TILE + lz;
        const uint4 l4 = *reinterpret_cast<const uint4*>(lo + c0);
        const uint4 h4 = *reinterpret_cast<const uint4*>(hi + c0);
        const long long q0 = (long long)(((unsigned long long)h4.x << 32) | l4.x);
        const long long q1 = (long long)(((unsigned long long)h4.y << 32) | l4.y);
        const long long q2 = (long long)(((unsigned long long)h4.z << 32) | l4.z);
        const long long q3 = (long long)(((unsigned long long)h4.w << 32) | l4.w);
        part += q0 + q1 + q2 + q3;
        float4 v = make_float4(fixed_to_float(q0, inv_sc), fixed_to_float(q1, inv_sc), fixed_to_float(q2, inv_sc),
                               fixed_to_float(q3, inv_sc));
        const long long gi = grid * M + ((x0 + lx) * N + (y0 + ly)) * N + (z0 + lz);
        if (mesh_in) {
          const float4 b = *reinterpret_cast<const float4*>(mesh_in + gi);
          v = make_float4(__fadd_rn(b.x, v.x), __fadd_rn(b.y, v.y), __fadd_rn(b.z, v.z), __fadd_rn(b.w, v.w));
        }
        *reinterpret_cast<float4*>(mesh_out + gi) = v;
      }
    } else {
      for (int k = threadIdx.x; k < TILE3; k += DEP_THREADS) {
        const int lz = k % TILE, ly = (k / TILE) % TILE, lx = k / (TILE * TILE);
        if (lx >= ex || ly >= ey || lz >= ez) continue;
        const long long q = (long long)(((unsigned long long)hi[k] << 32) | lo[k]);
        part += q;
        const long long gi = grid * M + ((x0 + lx) * N + (y0 + ly)) * N + (z0 + lz);
        float v = fixed_to_float(q, inv_sc);
        if (mesh_in) v = __fadd_rn(mesh_in[gi], v);
        mesh_out[gi] = v;
      }
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = part;
    __syncthreads();                            // the next grid reuses the accumulators
    if (threadIdx.x == 0) {                     // this tile's exact total (read by stats_kernel)
      long long tm = 0;
      for (int k = 0; k < DEP_THREADS / 32; ++k) tm += s_part[k];
      tile_mass[(long long)grid * gridDim.x + t] = tm;
    }
  }
}

// Buckets of a fixed capacity filled in one pass (count, scan and scatter
// only when one overflows), as on the fused path.
constexpr bool kMeshFill = true;

template <int MAS, int G, int CM>
int run_scheme(const DepGeom& g, const DepLayout& L, const DepBuffers& b, const float* mesh_in, float* mesh_out,
               cudaStream_t st) {
  int r = bucket_particles<MAS, G, CM>(g, L, b, st);
  if (r) return r;
  const size_t smem = (size_t)2 * TILE3 * sizeof(unsigned);   // lo + hi words, one grid
  // more than 48 KB of dynamic shared memory needs the opt-in (cheap, per call)
  GBP_CUDA_TRY(cudaFuncSetAttribute(deposit_kernel<MAS, G, CM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  GBP_TRACE("deposit_tiles", st);
  GBP_CUDA_TRY(launch_pdl(deposit_kernel<MAS, G, CM>, dim3(L.ntiles), dim3(DEP_THREADS), smem, st, g, b.entries,
                          b.counts, b.offsets, b.ctr, mesh_in, mesh_out, b.tile_mass));
  return GBP_OK;
}

// Carve the workspace, launch the scheme's kernels, fold the statistics.
// `n` sizes the launches (the particle count, or a job's capacity).
int deposit_launch(DepGeom g, const DepLayout& L, int64_t n, int mas, int G, int compat, const float* mesh_in,
                   float* mesh_out, gbp_deposit_stats* stats_out, void* workspace, cudaStream_t stream) {
  const DepBuffers b = carve_deposit(workspace, L);
  for (int a = 0; a < 3; ++a) { g.td[a] = L.td[a]; g.ts[a] = L.ts[a]; g.nt[a] = L.nt[a]; }
  g.tcap = L.tcap;
  g.vec_ok = ((reinterpret_cast<uintptr_t>(mesh_out) | reinterpret_cast<uintptr_t>(mesh_in)) & 15u) == 0;
  GBP_CUDA_TRY(cudaMemsetAsync(b.ctr, 0, zeroed_bytes(L), stream));
  int st;
  if (compat == GBP_COMPAT_VEC) st = run_scheme<GBP_CIC, 1, GBP_COMPAT_VEC>(g, L, b, mesh_in, mesh_out, stream);
  else if (compat == GBP_COMPAT_SCAN) st = run_scheme<GBP_CIC, 1, GBP_COMPAT_SCAN>(g, L, b, mesh_in, mesh_out, stream);
  else if (G == 1) {
    switch (mas) {
      case GBP_NGP: st = run_scheme<GBP_NGP, 1, 0>(g, L, b, mesh_in, mesh_out, stream); break;
      case GBP_CIC: st = run_scheme<GBP_CIC, 1, 0>(g, L, b, mesh_in, mesh_out, stream); break;
      case GBP_TSC: st = run_scheme<GBP_TSC, 1, 0>(g, L, b, mesh_in, mesh_out, stream); break;
      default: st = run_scheme<GBP_PCS, 1, 0>(g, L, b, mesh_in, mesh_out, stream); break;
    }
  } else {
    switch (mas) {
      case GBP_NGP: st = run_scheme<GBP_NGP, 2, 0>(g, L, b, mesh_in, mesh_out, stream); break;
      case GBP_CIC: st = run_scheme<GBP_CIC, 2, 0>(g, L, b, mesh_in, mesh_out, stream); break;
      case GBP_TSC: st = run_scheme<GBP_TSC, 2, 0>(g, L, b, mesh_in, mesh_out, stream); break;
      default: st = run_scheme<GBP_PCS, 2, 0>(g, L, b, mesh_in, mesh_out, stream); break;
    }
  }
  if (st) return st;
  if (stats_out) return deposit_stats(b, L, compat, G, stats_out, stream);
  return GBP_OK;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_deposit_workspace_size(int64_t n, int N, int mas, int interlace, int compat,
                                          size_t* bytes) {
  if (!bytes) return GBP_ERR_INVALID;
  DepLayout L;
  const int st = deposit_layout(n, N, mas, interlace, compat, kCubeTiles, L, kMeshFill);
  if (st) return st;
  *bytes = L.total;
  return GBP_OK;
}

extern "C" int gbp_deposit(const float* x, const float* y, const float* z, const float* w, int64_t n,
                           float xmin, float ymin, float zmin, float inv_cell, int N, int mas,
                           int interlace, int compat, int wrap, const float* mesh_in, float* mesh_out,
                           gbp_deposit_stats* stats_out, void* workspace, size_t ws_bytes,
                           gbp_stream_t stream_) {
  DepLayout L;
  const int st = deposit_layout(n, N, mas, interlace, compat, kCubeTiles, L, kMeshFill);
  if (st) return st;
  if (!mesh_out) return GBP_ERR_INVALID;
  if (n > 0 && (!x || !y || !z)) return GBP_ERR_INVALID;
  if (!workspace || ws_bytes < L.total) return GBP_ERR_WORKSPACE;
  DepGeom g{};
  g.x = x; g.y = y; g.z = z; g.w = w; g.n = n;
  g.ox = xmin; g.oy = ymin; g.oz = zmin; g.inv_cell = inv_cell;
  g.N = N; g.wrap = wrap ? 1 : 0;
  g.job = nullptr;
  return deposit_launch(g, L, n, mas, interlace ? 2 : 1, compat, mesh_in, mesh_out, stats_out, workspace,
                        reinterpret_cast<cudaStream_t>(stream_));
}

extern "C" int gbp_deposit_job(const gbp_job* job, int64_t capacity, int N, int mas, int interlace,
                               float* mesh_out, gbp_deposit_stats* stats_out, void* workspace, size_t ws_bytes,
                               gbp_stream_t stream_) {
  DepLayout L;
  const int st = deposit_layout(capacity, N, mas, interlace, GBP_COMPAT_NONE, kCubeTiles, L, kMeshFill);
  if (st) return st;
  if (!job || !mesh_out) return GBP_ERR_INVALID;
  if (!workspace || ws_bytes < L.total) return GBP_ERR_WORKSPACE;
  DepGeom g{};
  g.N = N;
  g.job = job;
  g.cap = capacity;
  return deposit_launch(g, L, capacity, mas, interlace ? 2 : 1, GBP_COMPAT_NONE, nullptr, mesh_out, stats_out,
                        workspace, reinterpret_cast<cudaStream_t>(stream_));
}
