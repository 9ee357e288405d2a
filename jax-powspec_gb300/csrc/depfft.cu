// Particles -> multipole sums with the deposit fused into the z pass of the
// FFT (library transform sizes: power-of-two meshes 64..1024, B-spline
// deposits).
//
// The mesh is never written.  Particles are bucketed (deposit_core.cuh) by
// column tile: TX x TY pencils (8 x 4 at 256^3 and 512^3, 4 x 4 otherwise)
// spanning the whole z axis, so a stencil is replicated across x and y tile
// faces only.  One CTA per column tile and grid:
//
//   1. accumulates its bucket in shared memory as 32-bit fixed point with a
//      scale of its own: 2^s, s = s_g - ceil(log2(c)) (+1 for TSC and PCS,
//      whose node weights stay below 1/2), where c is the largest number of
//      the tile's entries covering one z plane (counted first) and 2^s_g
//      puts the largest particle weight just below 2^30.  No cell can then
//      exceed 2^30 + rounding in magnitude, whatever the order of the adds,
//      so the integer sums are exact, order-independent and overflow-free
//      (fire-and-forget shared reductions, no carries);
//   2. transforms its pencils along z: the first radix-8 stage reads the
//      integer cells of two pencils (packed as one complex pencil), converts
//      them to float and writes the complex buffer that aliases the
//      accumulators; the remaining stages run in place (fft_pass.cuh),
//   3. splits each packed spectrum into its two real-input half spectra and
//      writes the pencils' rows of the z-transformed spectrum (P = N/2 + 8
//      complex per row, as the library's own transform),
//   4. adds up the tile's exact integer total, shifted to the common scale
//      2^s_g (the mean density; stats_kernel folds the tiles).
//
// Then the y pass (fft.cu) and the x pass fused with the binning (xbin.cu)
// finish the transform and the P_l sums.  HBM traffic per grid: the
// spectrum is written once here, read and written by the y pass, and read
// once by the binning; no mesh goes through HBM.
#include <algorithm>
#include <type_traits>

#include "deposit_core.cuh"
#include "fft_pass.cuh"
#include "gbp_bins.h"
#include "gbp_fft.h"

namespace gbp {
namespace {

template <int N>
struct ColTile {
  static constexpr int TX = (N == 256 || N == 512) ? 8 : 4;
  static constexpr int TY = 4;
  static constexpr int NPEN = TX * TY;            // pencils per tile; pencil f = lx * TY + ly
  static constexpr int PAIRS = NPEN / 2;          // complex transforms (pencils 2q, 2q+1)
  static constexpr int NFFT = PAIRS * N / 16;     // butterfly pairs (two columns) per radix-8 stage
  static constexpr int NT = NFFT < 256 ? 256 : NFFT;
  static constexpr int MINB = NT >= 512 ? 2 : 3;  // CTAs per SM the registers are sized for
  static constexpr size_t SMEM = (size_t)(NPEN + 1) * N * sizeof(int);   // cells + per-plane entry counts
  static constexpr size_t SMEM_WIDE = (size_t)NPEN * N * sizeof(long long);
};

// Bits of resolution a tile may give up to its 32-bit cells.  A tile whose
// densest z plane is covered by more than 2^(SH_MAX + WBIT) entries (a dense
// clump: a halo, a point mass) is deposited with 64-bit cells at the common
// scale instead, by deposit_fftz_wide_kernel: with the coarse quantum the
// rounding of many identical contributions adds up instead of averaging out.
constexpr int SH_MAX = 10;
constexpr long long WIDE_MARK = (-0x7fffffffffffffffLL - 1);   // tile_mass entry of a tile left to the wide kernel

// Deposit, z transform, split and row stores of one column tile and grid
// (steps 1-4 above).  WIDE: 64-bit cells at the common scale 2^sg (sh = 0);
// otherwise 32-bit cells at 2^(sg - sh).  Returns the tile's exact total at
// the scale 2^(sg - sh) (valid in thread 0).
template <int N, int MAS, int G, bool WIDE>
__device__ __forceinline__ long long tile_grid(const DepGeom& g, const float4* __restrict__ entries, unsigned beg,
                                               unsigned end, int sg, int sh, int grid, int x0, int y0,
                                               const float2* __restrict__ tw, float2* __restrict__ spec,
                                               unsigned char* smem, long long* s_part) {
  using CT = ColTile<N>;
  using Cell = typename std::conditional<WIDE, unsigned long long, int>::type;
  constexpr int R = MAS, TX = CT::TX, TY = CT::TY, NPEN = CT::NPEN, PAIRS = CT::PAIRS, NT = CT::NT;
  constexpr int P = N / 2 + 8, H = N / 2;
  Cell* acc = reinterpret_cast<Cell*>(smem);                   // [NPEN][N] fixed-point cells
  float4* cs4 = reinterpret_cast<float4*>(smem);               // [PAIRS/2][N] slots of two columns, alias the cells
  const int tid = threadIdx.x;
  const int s = sg - sh;
  // 2^s and 2^-s as two exact power-of-two factors each (s may reach -130); 2^-s is one normal
  // float unless s < -126 (weights beyond 2^150)
  const float up1 = ldexpf(1.0f, s / 2), up2 = ldexpf(1.0f, s - s / 2);
  const bool one_dn = s >= -126;
  const float dn1 = one_dn ? ldexpf(1.0f, -s) : ldexpf(1.0f, -(s / 2));
  const float dn2 = one_dn ? 1.0f : ldexpf(1.0f, -(s - s / 2));
  const long long gstride = (long long)N * N * P;

  {
    uint4* a4 = reinterpret_cast<uint4*>(acc);
    for (int k = tid; k < (int)(NPEN * N * sizeof(Cell) / 16); k += NT) a4[k] = make_uint4(0u, 0u, 0u, 0u);
  }
  __syncthreads();
  for (unsigned i = beg + tid; i < end; i += NT) {
    const float4 e = entries[i];
    Axis<R> ax, ay, az;
    make_axis<MAS, 0>(g, e.x, grid, ax);
    make_axis<MAS, 0>(g, e.y, grid, ay);
    make_axis<MAS, 0>(g, e.z, grid, az);
    int lx[R], ly[R], zz[R];
    local_nodes<R>(ax, N, x0, TX, lx);
    local_nodes<R>(ay, N, y0, TY, ly);
    const float wsc = __fmul_rn(__fmul_rn(e.w, up1), up2);   // exact: powers of two
    float wz[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      zz[r] = wrapn(az.first + r, N);
      wz[r] = __fmul_rn(az.w[r], wsc);
    }
#pragma unroll
    for (int rx = 0; rx < R; ++rx) {
      if (lx[rx] < 0) continue;
#pragma unroll
      for (int ry = 0; ry < R; ++ry) {
        if (ly[ry] < 0) continue;
        const float wxy = __fmul_rn(ax.w[rx], ay.w[ry]);
        const int row = (lx[rx] * TY + ly[ry]) * N;
#pragma unroll
        for (int rz = 0; rz < R; ++rz) {
          const int v = __float2int_rn(__fmul_rn(wxy, wz[rz]));
          if constexpr (WIDE) atomicAdd(&acc[row + zz[rz]], (unsigned long long)(long long)v);
          else atomicAdd(&acc[row + zz[rz]], v);
        }
      }
    }
  }
  __syncthreads();

  // z transform: pencils 2q and 2q+1 are the real and imaginary parts of
  // column q; a thread transforms columns 2cp and 2cp+1 (pencils 4cp..4cp+3)
  long long part = 0;
  auto gin = [&part, one_dn, dn1, dn2, acc](int j, int cp) {
    float v[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const long long q = (long long)acc[(4 * cp + f) * N + j];
      part += q;
      v[f] = __fmul_rn(WIDE ? __ll2float_rn(q) : __int2float_rn((int)q), dn1);   // exact: a power of two
      if (!one_dn) v[f] = __fmul_rn(v[f], dn2);
    }
    return make_float4(v[0], v[1], v[2], v[3]);
  };
  auto sin_ = [cs4](int j, int cp) { return cs4[cp * N + fft::zsw(j)]; };
  auto sout = [cs4](int j, int cp, float4 v) { cs4[cp * N + fft::zsw(j)] = v; };
  // N = 512, 32-bit cells: every stage is radix 8 and the 64 threads of a column pair own its data
  // (the first stage's writes alias the pair's own pencils), so the stages synchronise 64-thread
  // groups only.  64-bit cells span twice the bytes of the complex slots: whole-CTA barriers.
  constexpr int GS = (!WIDE && N == 512 && NT == PAIRS / 2 * (N / 8)) ? N / 8 : 0;
  fft::run_stages2<N, PAIRS / 2, NT, true, true, true, decltype(gin), decltype(sin_), decltype(sout),
                   decltype(sout), GS>(gin, sin_, sout, sout, tw, tid);

  // split the packed spectra; write all pencils' rows (row padding -> 0)
  const float2* cs = reinterpret_cast<const float2*>(cs4);
  float2* out = spec + grid * gstride;
  for (int idx = tid; idx < PAIRS * P; idx += NT) {
    const int q = idx / P, k = idx - (idx / P) * P;
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (k <= H) {
      const float2 c = cs[((q >> 1) * N + fft::zsw(k)) * 2 + (q & 1)];
      const float2 m = cs[((q >> 1) * N + fft::zsw((N - k) & (N - 1))) * 2 + (q & 1)];
      const float2 cm = make_float2(m.x, -m.y);
      const float2 sum = fft::cadd(c, cm), dif = fft::cmi(fft::csub(c, cm));
      a = make_float2(0.5f * sum.x, 0.5f * sum.y);
      b = make_float2(0.5f * dif.x, 0.5f * dif.y);
    }
    const int f0 = 2 * q, f1 = 2 * q + 1;
    const long long r0 = (long long)(x0 + f0 / TY) * N + (y0 + f0 % TY);
    const long long r1 = (long long)(x0 + f1 / TY) * N + (y0 + f1 % TY);
    __stcs(out + r0 * P + k, a);
    __stcs(out + r1 * P + k, b);
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

template <int N, int MAS, int G>
__global__ void __launch_bounds__(ColTile<N>::NT, ColTile<N>::MINB)
deposit_fftz_kernel(DepGeom g, const float4* __restrict__ entries, const unsigned* __restrict__ counts,
                    const unsigned* __restrict__ offsets, const DepCounters* ctr, const float2* __restrict__ tw,
                    float2* __restrict__ spec, long long* __restrict__ tile_mass) {
  using CT = ColTile<N>;
  constexpr int R = MAS, TX = CT::TX, TY = CT::TY, NPEN = CT::NPEN, NT = CT::NT;
  extern __shared__ __align__(16) int acc_smem[];
  int* zc = acc_smem + NPEN * N;                       // [N] entries whose stencil (any grid) covers plane z
  __shared__ long long s_part[NT / 32];
  __shared__ int s_max[NT / 32];
  const int tid = threadIdx.x;
  const int t = blockIdx.x;
  const int ty = t % g.nt[1], tx = t / g.nt[1];
  const int x0 = tx * TX, y0 = ty * TY;
  const unsigned beg = offsets[t];
  const unsigned end = beg + counts[t * CSTRIDE];
  const int sg = fixed_scale_exp(ctr->maxw_bits, 0);
  // A cell of plane z only receives entries covering z: the largest such
  // count bounds every cell of the tile.
  for (int k = tid; k < N; k += NT) zc[k] = 0;
  __syncthreads();
  for (unsigned i = beg + tid; i < end; i += NT) {
    const float z = entries[i].z;
    Axis<R> a0;
    make_axis<MAS, 0>(g, z, 0, a0);
    int last = a0.first + R - 1;
    if constexpr (G == 2) {
      Axis<R> a1;
      make_axis<MAS, 0>(g, z, 1, a1);
      last = a1.first + R - 1;                         // a1.first is a0.first or a0.first + 1
    }
    for (int zn = a0.first; zn <= last; ++zn) atomicAdd(&zc[wrapn(zn, N)], 1);
  }
  __syncthreads();
  int cmax = 0;
  for (int k = tid; k < N; k += NT) cmax = max(cmax, zc[k]);
  cmax = __reduce_max_sync(0xffffffffu, cmax);
  if ((tid & 31) == 0) s_max[tid >> 5] = cmax;
  __syncthreads();
  cmax = 0;
  for (int k = 0; k < NT / 32; ++k) cmax = max(cmax, s_max[k]);
  const unsigned cnt = (unsigned)cmax;
  const int lg = cnt > 1u ? 32 - __clz(cnt - 1u) : 0;  // ceil(log2(entries per plane))
  // a node weight of TSC (<= 0.75^3) or PCS (<= (2/3)^3) is below 1/2: one more bit
  constexpr int WBIT = (MAS == GBP_TSC || MAS == GBP_PCS) ? 1 : 0;
  const int sh = lg > WBIT ? lg - WBIT : 0;            // tile scale 2^s = 2^(sg - sh), never finer than 2^sg
  if (sh > SH_MAX) {                                   // a dense clump: the wide kernel takes this tile
    if (tid == 0) tile_mass[t] = WIDE_MARK;
    return;
  }
  for (int grid = 0; grid < G; ++grid) {
    const long long tm = tile_grid<N, MAS, G, false>(g, entries, beg, end, sg, sh, grid, x0, y0, tw, spec,
                                                     reinterpret_cast<unsigned char*>(acc_smem), s_part);
    if (tid == 0) tile_mass[(long long)grid * gridDim.x + t] = tm * (1LL << sh);   // exact, at the common scale 2^sg
  }
}

// The tiles deposit_fftz_kernel left (tile_mass entry WIDE_MARK): 64-bit
// cells at the common scale.  Persistent: CTA b owns a contiguous range of
// tiles, finds its marked ones with one parallel scan (such tiles are rare;
// with none, that scan is all a CTA does) and processes them in turn.
constexpr int WIDE_LIST = 64;                          // marked tiles listed per scan round

template <int N, int MAS, int G>
__global__ void __launch_bounds__(ColTile<N>::NT, 1)
deposit_fftz_wide_kernel(DepGeom g, const float4* __restrict__ entries, const unsigned* __restrict__ counts,
                         const unsigned* __restrict__ offsets, const DepCounters* ctr, const float2* __restrict__ tw,
                         float2* __restrict__ spec, long long* __restrict__ tile_mass, int ntiles) {
  using CT = ColTile<N>;
  constexpr int NT = CT::NT;
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
        const unsigned beg = offsets[tt];
        const unsigned end = beg + counts[tt * CSTRIDE];
        for (int grid = 0; grid < G; ++grid) {
          const long long tm = tile_grid<N, MAS, G, true>(g, entries, beg, end, sg, 0, grid, tx * CT::TX,
                                                          ty * CT::TY, tw, spec,
                                                          reinterpret_cast<unsigned char*>(wide_smem), s_part);
          if (threadIdx.x == 0) tile_mass[(long long)grid * ntiles + tt] = tm;   // clears the mark
        }
      }
      __syncthreads();                                 // the marks are replaced before the next scan
    }
  }
}

template <int N>
void tile_shape(int (&tile)[3]) {
  tile[0] = ColTile<N>::TX;
  tile[1] = ColTile<N>::TY;
  tile[2] = N;
}

int column_tiles(int N, int (&tile)[3]) {
  switch (N) {
    case 64: tile_shape<64>(tile); return GBP_OK;
    case 128: tile_shape<128>(tile); return GBP_OK;
    case 256: tile_shape<256>(tile); return GBP_OK;
    case 512: tile_shape<512>(tile); return GBP_OK;
    case 1024: tile_shape<1024>(tile); return GBP_OK;
    default: return GBP_ERR_UNSUPPORTED;
  }
}

struct PartLayout {
  DepLayout dep;
  size_t xbin, total;
};

int particles_layout(int64_t n, gbp_fft_plan plan, gbp_bins B, int mas, int ells, PartLayout& L) {
  if (!plan || !B || plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own || (plan->grids != 1 && plan->grids != 2)) return GBP_ERR_UNSUPPORTED;
  int tile[3];
  int st = column_tiles(B->N, tile);
  if (st) return st;
  st = deposit_layout(n, B->N, mas, plan->grids == 2, GBP_COMPAT_NONE, tile, L.dep);
  if (st) return st;
  st = xbin_power_workspace(plan, B, ells, &L.xbin);
  if (st) return st;
  L.total = align256(L.dep.total) + L.xbin;
  return GBP_OK;
}

template <int N, int MAS, int G>
int run_fused(const DepGeom& g, const DepLayout& L, const DepBuffers& b, const float2* tw, float2* spec,
              cudaStream_t st) {
  int r = bucket_particles<MAS, G, 0>(g, L, b, st);
  if (r) return r;
  auto k = deposit_fftz_kernel<N, MAS, G>;
  const size_t smem = ColTile<N>::SMEM;
  GBP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  {
    GBP_TRACE("deposit_fft_z", st);
    k<<<L.ntiles, ColTile<N>::NT, smem, st>>>(g, b.entries, b.counts, b.offsets, b.ctr, tw, spec, b.tile_mass);
    GBP_LAUNCH_CHECK();
  }
  // tiles of dense clumps, if any, with 64-bit cells (one CTA per SM scans the marks)
  auto kw = deposit_fftz_wide_kernel<N, MAS, G>;
  const size_t smem_w = ColTile<N>::SMEM_WIDE;
  GBP_CUDA_TRY(cudaFuncSetAttribute(kw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_w));
  int dev = 0, sms = 0;
  GBP_CUDA_TRY(cudaGetDevice(&dev));
  GBP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GBP_TRACE("deposit_fft_z_wide", st);
  kw<<<std::max(1, std::min(sms, L.ntiles)), ColTile<N>::NT, smem_w, st>>>(g, b.entries, b.counts, b.offsets, b.ctr,
                                                                          tw, spec, b.tile_mass, L.ntiles);
  GBP_LAUNCH_CHECK();
  return GBP_OK;
}

template <int N>
int dispatch_fused(int mas, int G, const DepGeom& g, const DepLayout& L, const DepBuffers& b, const float2* tw,
                   float2* spec, cudaStream_t st) {
  if (G == 2) {
    switch (mas) {
      case GBP_NGP: return run_fused<N, GBP_NGP, 2>(g, L, b, tw, spec, st);
      case GBP_CIC: return run_fused<N, GBP_CIC, 2>(g, L, b, tw, spec, st);
      case GBP_TSC: return run_fused<N, GBP_TSC, 2>(g, L, b, tw, spec, st);
      default: return run_fused<N, GBP_PCS, 2>(g, L, b, tw, spec, st);
    }
  }
  switch (mas) {
    case GBP_NGP: return run_fused<N, GBP_NGP, 1>(g, L, b, tw, spec, st);
    case GBP_CIC: return run_fused<N, GBP_CIC, 1>(g, L, b, tw, spec, st);
    case GBP_TSC: return run_fused<N, GBP_TSC, 1>(g, L, b, tw, spec, st);
    default: return run_fused<N, GBP_PCS, 1>(g, L, b, tw, spec, st);
  }
}

int particles_power(DepGeom g, int64_t n_launch, gbp_fft_plan plan, gbp_bins B, int mas, int ells, void* spectrum,
                    double* sums_out, long long* nmodes_out, double* ksum_out, gbp_deposit_stats* stats_out,
                    void* workspace, size_t ws_bytes, cudaStream_t st) {
  if (!spectrum || !sums_out || !nmodes_out || !stats_out) return GBP_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(spectrum) & 15u) != 0) return GBP_ERR_INVALID;
  PartLayout L;
  int r = particles_layout(n_launch, plan, B, mas, ells, L);
  if (r) return r;
  if (!workspace || ws_bytes < L.total) return GBP_ERR_WORKSPACE;
  const DepBuffers b = carve_deposit(workspace, L.dep, n_launch);
  void* xws = static_cast<char*>(workspace) + align256(L.dep.total);
  for (int a = 0; a < 3; ++a) { g.td[a] = L.dep.td[a]; g.ts[a] = L.dep.ts[a]; g.nt[a] = L.dep.nt[a]; }
  g.vec_ok = 0;
  const int N = B->N, G = plan->grids;
  float2* spec = static_cast<float2*>(spectrum);
  GBP_CUDA_TRY(cudaMemsetAsync(b.ctr, 0, zeroed_bytes(L.dep), st));
  switch (N) {
    case 64: r = dispatch_fused<64>(mas, G, g, L.dep, b, plan->tw, spec, st); break;
    case 128: r = dispatch_fused<128>(mas, G, g, L.dep, b, plan->tw, spec, st); break;
    case 256: r = dispatch_fused<256>(mas, G, g, L.dep, b, plan->tw, spec, st); break;
    case 512: r = dispatch_fused<512>(mas, G, g, L.dep, b, plan->tw, spec, st); break;
    default: r = dispatch_fused<1024>(mas, G, g, L.dep, b, plan->tw, spec, st); break;
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

using namespace gbp;

extern "C" int gbp_particles_power_workspace_size(int64_t n, gbp_fft_plan plan, gbp_bins bins, int mas, int ells,
                                                  size_t* bytes) {
  if (!bytes) return GBP_ERR_INVALID;
  PartLayout L;
  const int st = particles_layout(n, plan, bins, mas, ells, L);
  if (st) return st;
  *bytes = L.total;
  return GBP_OK;
}

extern "C" int gbp_particles_power(const float* x, const float* y, const float* z, const float* w, int64_t n,
                                   float xmin, float ymin, float zmin, float inv_cell, gbp_fft_plan plan,
                                   gbp_bins bins, int mas, int ells, void* spectrum, double* sums_out,
                                   long long* nmodes_out, double* ksum_out, gbp_deposit_stats* stats_out,
                                   void* workspace, size_t ws_bytes, gbp_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y || !z))) return GBP_ERR_INVALID;
  if (!plan || !bins) return GBP_ERR_INVALID;
  DepGeom g{};
  g.x = x; g.y = y; g.z = z; g.w = w; g.n = n;
  g.ox = xmin; g.oy = ymin; g.oz = zmin; g.inv_cell = inv_cell;
  g.N = bins->N;
  g.job = nullptr;
  return particles_power(g, n, plan, bins, mas, ells, spectrum, sums_out, nmodes_out, ksum_out, stats_out, workspace,
                         ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int gbp_particles_power_job(const gbp_job* job, int64_t capacity, gbp_fft_plan plan, gbp_bins bins,
                                       int mas, int ells, void* spectrum, double* sums_out, long long* nmodes_out,
                                       double* ksum_out, gbp_deposit_stats* stats_out, void* workspace,
                                       size_t ws_bytes, gbp_stream_t stream) {
  if (!job || capacity < 0 || !plan || !bins) return GBP_ERR_INVALID;
  DepGeom g{};
  g.N = bins->N;
  g.job = job;
  g.cap = capacity;
  return particles_power(g, capacity, plan, bins, mas, ells, spectrum, sums_out, nmodes_out, ksum_out, stats_out,
                         workspace, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}
