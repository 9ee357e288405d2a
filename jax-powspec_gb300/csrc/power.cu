// Fused post-FFT kernel: window deconvolution, interlacing combination,
// |delta_k|^2 x Legendre L_l(mu) (line of sight z) and k-shell binning.
//
// Layout: a spectrum is complex64 [N][N][Lz] with Lz = N/2+1 (cuFFT R2C).
// Each warp walks a contiguous run of that flat array.  Along a z pencil |k|
// grows with kz, so consecutive modes form sorted runs of equal bin:
//
//  * main kernel (even N >= 64): a lane owns 4 consecutive modes per step
//    (two 16-byte loads per grid, next step prefetched).  It sums its own
//    runs, then one warp-shuffle segmented scan joins runs that continue
//    across lanes.  Every maximal run is added exactly once, by the lane
//    where it ends, to the warp's private float32 bins in shared memory.
//  * simple kernel (odd or small N): one mode per lane and step, same scan.
//
// Runs of different pencils in one step can share a bin, so the adds are
// issued pencil by pencil with __syncwarp() between them: no shared-memory
// atomics, a fixed order, bitwise reproducible results.  At the end each CTA
// folds its warps' bins into a float-float (hi, lo) partial, and
// power_reduce_kernel folds the CTAs' partials in a fixed order into
// doubles.  (GB300 runs FP64 at a small fraction of its FP32 rate, so
// doubles appear only in the final per-bin totals.)
//
// The kernels accumulate the moments sum p, sum p mu^2, sum p mu^4 with
// p = |delta|^2 W^2; the reduction turns them into the Legendre sums
// L_0 = 1, L_2 = (3 mu^2 - 1)/2, L_4 = (35 mu^4 - 30 mu^2 + 3)/8
// (src/correlations.py:45-47).  Mode counts and sum |k| per bin depend only
// on the grid and come from the bin plan.
//
// Bin membership uses integer thresholds on k2 = kx^2+ky^2+kz^2 computed on
// the host (gbp_bin_thresholds), which reproduces jnp.histogram applied to
// k = sqrtf((float)k2) exactly (src/correlations.py:34,42,45-48).
#include <math.h>

#include <algorithm>
#include <mutex>

#include "gbp_bins.h"
#include "gbp_internal.cuh"
#include "power_core.cuh"

namespace gbp {
namespace {

// ---------------------------------------------------------------------------
// Main kernel: 4 modes per lane, 128 per warp step.  Requires even N (so that
// both grids' arrays are 16-byte aligned and every lane's 4 modes are either
// all in range or all out) and a chunk that is a multiple of 128.
template <int NV, bool INTER>
__device__ __forceinline__ void chunk4(const PowGeom& g, const Smem& s, float* wb, int lane, long long beg,
                                       long long end) {
  if (beg < end) {
    // first mode of this lane in the current step, and its pencil / kz
    long long f = beg + 4 * lane;
    long long pen = f / g.Lzs;
    int kz = (int)(f - pen * g.Lzs);
    int iy = (int)(pen % g.N);
    int ix = (int)(pen / g.N);
    const float4* s0 = reinterpret_cast<const float4*>(g.s0);
    const float4* s1 = reinterpret_cast<const float4*>(g.s1);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 a01 = z4, a23 = z4, b01 = z4, b23 = z4;
    if (f < end) {
      a01 = __ldcs(s0 + f / 2);
      a23 = __ldcs(s0 + f / 2 + 1);
      if (INTER) { b01 = __ldcs(s1 + f / 2); b23 = __ldcs(s1 + f / 2 + 1); }
    }
    for (long long fb = beg; fb < end; fb += 128) {
      const bool valid = f < end;
      // prefetch the next step
      const long long fn = f + 128;
      float4 na01 = z4, na23 = z4, nb01 = z4, nb23 = z4;
      if (fn < end) {
        na01 = __ldcs(s0 + fn / 2);
        na23 = __ldcs(s0 + fn / 2 + 1);
        if (INTER) { nb01 = __ldcs(s1 + fn / 2); nb23 = __ldcs(s1 + fn / 2 + 1); }
      }
      const float2 A[4] = {make_float2(a01.x, a01.y), make_float2(a01.z, a01.w), make_float2(a23.x, a23.y),
                           make_float2(a23.z, a23.w)};
      const float2 Bv[4] = {make_float2(b01.x, b01.y), make_float2(b01.z, b01.w), make_float2(b23.x, b23.y),
                            make_float2(b23.z, b23.w)};
      // per-mode moments, bins and pencil ids (4 consecutive modes)
      float P[4][NV];          // running in-lane run sums
      int bin[4], pid[4];
      {
        int cix = ix, ciy = iy, ckz = kz;
        Pencil pc = pencil_of<INTER>(g, s, cix, ciy);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (j > 0 && ++ckz == g.Lzs) {
            ckz = 0;
            if (++ciy == g.N) { ciy = 0; ++cix; }
            pc = pencil_of<INTER>(g, s, cix, ciy);
          }
          pid[j] = cix * g.N + ciy;
          int k2;
          const bool zero = g.zero_dc && (f + j == 0);
          const bool real_mode = ckz < g.Lz;     // not row padding
          mode_moments<NV, INTER>(s, pc, real_mode ? ckz : 0, A[j], Bv[j], zero || !real_mode, P[j], k2);
          bin[j] = (valid && real_mode) ? bin_of(g, s, k2) : -1;
        }
      }
      // in-lane runs: P[j] becomes the sum of the run up to mode j
      bool start[4];
      start[0] = true;
#pragma unroll
      for (int j = 1; j < 4; ++j) {
        start[j] = (bin[j] != bin[j - 1]) || (pid[j] != pid[j - 1]);
        if (!start[j]) {
#pragma unroll
          for (int q = 0; q < NV; ++q) P[j][q] += P[j - 1][q];
        }
      }
      const bool multi = start[1] || start[2] || start[3];
      // run keys: pencil relative to lane 0's first mode, and bin
      const int p0 = __shfl_sync(0xffffffffu, pid[0], 0);
      const int key_first = ((pid[0] - p0) << 20) | (bin[0] + 1);
      const int key_last = ((pid[3] - p0) << 20) | (bin[3] + 1);
      const int prev_last = __shfl_up_sync(0xffffffffu, key_last, 1);
      const bool cont = lane > 0 && key_first == prev_last;       // first run continues the previous lane's last
      const unsigned heads = __ballot_sync(0xffffffffu, multi || !cont);
      float T[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) T[q] = P[3][q];
      seg_scan<NV>(T, heads, lane);
      float Tprev[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) Tprev[q] = __shfl_up_sync(0xffffffffu, T[q], 1);
      const bool next_cont = __shfl_down_sync(0xffffffffu, cont, 1) && lane < 31;
      // run ends inside the lane (j < 3); the first one absorbs the carry
      bool endin[3];
      int firstend = 3;
#pragma unroll
      for (int j = 2; j >= 0; --j) {
        endin[j] = start[j + 1];
        if (endin[j]) firstend = j;
      }
      if (cont && multi) {
#pragma unroll
        for (int j = 0; j < 3; ++j)
          if (j == firstend) {
#pragma unroll
            for (int q = 0; q < NV; ++q) P[j][q] += Tprev[q];
          }
      }
      const bool flush_last = !next_cont;
      // flush pencil by pencil
      const int rel0 = pid[0] - p0, rel3 = pid[3] - p0;
      const int nph = __reduce_max_sync(0xffffffffu, valid ? rel3 : 0) + 1;   // pencils in this step
      for (int ph = 0; ph < nph; ++ph) {
        if (rel0 <= ph && ph <= rel3) {
#pragma unroll
          for (int j = 0; j < 3; ++j)
            if (endin[j] && bin[j] >= 0 && pid[j] - p0 == ph) bin_add<NV>(wb, g.nbe, bin[j], P[j]);
          if (flush_last && bin[3] >= 0 && rel3 == ph) bin_add<NV>(wb, g.nbe, bin[3], T);
        }
        __syncwarp();
      }
      // advance
      a01 = na01; a23 = na23; b01 = nb01; b23 = nb23;
      f += 128;
      kz += 128;
      while (kz >= g.Lzs) {
        kz -= g.Lzs;
        if (++iy == g.N) { iy = 0; ++ix; }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Simple path: one mode per lane per step (any N, any alignment).
template <int NV, bool INTER>
__device__ __forceinline__ void chunk1(const PowGeom& g, const Smem& s, float* wb, int lane, long long beg,
                                       long long end) {
  if (beg < end) {
    long long f = beg + lane;
    long long pen = f / g.Lzs;
    int kz = (int)(f - pen * g.Lzs);
    int iy = (int)(pen % g.N);
    int ix = (int)(pen / g.N);
    for (long long fb = beg; fb < end; fb += 32) {
      const bool valid = f < end;
      float v[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) v[q] = 0.0f;
      int bin = -1;
      if (valid && kz < g.Lz) {
        const Pencil pc = pencil_of<INTER>(g, s, ix, iy);
        const float2 a = g.s0[f];
        const float2 b = INTER ? g.s1[f] : make_float2(0.f, 0.f);
        int k2;
        mode_moments<NV, INTER>(s, pc, kz, a, b, g.zero_dc && f == 0, v, k2);
        bin = bin_of(g, s, k2);
      }
      const int bprev = __shfl_up_sync(0xffffffffu, bin, 1);
      const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || bin != bprev);
      seg_scan<NV>(v, heads, lane);
      const bool segend = (lane == 31) || ((heads >> (lane + 1)) & 1u);
      const int pid = ix * g.N + iy;
      const int rel = pid - __shfl_sync(0xffffffffu, pid, 0);
      const int nph = __reduce_max_sync(0xffffffffu, valid ? rel : 0) + 1;   // pencils in this step
      for (int ph = 0; ph < nph; ++ph) {
        if (segend && bin >= 0 && rel == ph) bin_add<NV>(wb, g.nbe, bin, v);
        __syncwarp();
      }
      f += 32;
      kz += 32;
      while (kz >= g.Lzs) {
        kz -= g.Lzs;
        if (++iy == g.N) { iy = 0; ++ix; }
      }
    }
  }
}

// Persistent CTAs walk the fixed work groups (g.warps warp chunks each); a
// group's sums go to its own partial, so the result does not depend on how
// many CTAs run.
template <int NV, bool INTER, bool WIDE>
__global__ void __launch_bounds__(POW_WARPS * 32, 4)
power_kernel(PowGeom g) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem[];
  const Smem s = load_tables<NV, INTER>(g, smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* wb = s.wbase + warp * NV * g.nbe;
  for (int grp = blockIdx.x; grp < g.groups; grp += gridDim.x) {
    const long long beg = ((long long)grp * g.warps + warp) * g.chunk;
    const long long end = min(beg + g.chunk, g.total);
    if (WIDE) chunk4<NV, INTER>(g, s, wb, lane, beg, end);
    else chunk1<NV, INTER>(g, s, wb, lane, beg, end);
    cta_fold<NV>(g, s, grp);
  }
}

__global__ void power_normalize_kernel(const double* sums, const long long* nmodes, const double* ksum, int nb,
                                       double norm_delta, double box3, double kf, const double* mass,
                                       const gbp_deposit_stats* stats, int subtract_shot, double* pk_out,
                                       double* kmean_out, const gbp_job* job, int N) {
  pdl_wait();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  if (job) {                      // box size from the device job descriptor
    const double box = job->box_size;
    const double n2 = (double)N * (double)N;
    norm_delta = (box / n2) * (box / n2) * (box / n2);
    box3 = box * box * box;
    kf = 2.0 * M_PI / box;
  }
  double norm = norm_delta, shot = 0.0;
  if (mass) {
    const double m = mass[0];
    norm = box3 / (m * m);
    if (subtract_shot && stats) shot = box3 * stats->sum_w2 / (m * m);
  }
  const double n = (double)nmodes[b];
  for (int l = 0; l < 3; ++l) {
    double p = (4.0 * l + 1.0) * sums[b * 3 + l] / n * norm;  // (2 ell + 1); 0/0 -> NaN like the reference
    if (l == 0) p -= shot;
    pk_out[b * 3 + l] = p;
  }
  if (kmean_out) kmean_out[b] = ksum ? ksum[b] / n * kf : 0.0;
}

struct PowLayout {
  int NV, warps, C;
  bool wide;                // the 4-modes-per-lane kernel
  long long total, chunk;
  size_t smem, ws_total;
};

// A pure function of (N, bins, ells): the summation order, and therefore the
// result, is the same on every device.
int power_layout(const gbp_bins_s* B, int G, int ells, int Lzs, PowLayout& L) {
  if (Lzs < B->N / 2 + 1) return GBP_ERR_INVALID;
  L.NV = (ells & GBP_ELL4) ? 3 : ((ells & GBP_ELL2) ? 2 : 1);
  const size_t budget = 200 * 1024;
  int w = POW_WARPS;
  while (w > 1 && smem_plan(B->N, B->nbe, B->lut_n, w, L.NV).total > budget) --w;
  L.smem = smem_plan(B->N, B->nbe, B->lut_n, w, L.NV).total;
  if (L.smem > budget) return GBP_ERR_UNSUPPORTED;
  L.warps = w;
  L.total = (long long)B->N * B->N * Lzs;
  L.wide = (B->N % 2 == 0) && B->N >= 64;   // N*N*Lzs stays a multiple of 4 modes
  long long target = L.total / (8LL * 152 * 8);   // ~8 groups per SM on a GB300
  target = std::max(1024LL, std::min(16384LL, target));
  L.chunk = (target + 127) & ~127LL;
  const long long nw = (L.total + L.chunk - 1) / L.chunk;
  L.C = (int)((nw + w - 1) / w);
  L.ws_total = align256((size_t)L.C * L.NV * B->nbe * sizeof(float2));
  (void)G;
  return GBP_OK;
}

// Argument checks shared by gbp_power and gbp_power_noalloc.
int power_args(const void* spectrum, int G, gbp_bins B, int mas_order, int ells, double* sums_out,
               long long* nmodes_out, double* ksum_out) {
  if (!spectrum || !B || !sums_out || !nmodes_out) return GBP_ERR_INVALID;
  if (G != 1 && G != 2) return GBP_ERR_INVALID;
  if (mas_order < 0 || mas_order > 8) return GBP_ERR_INVALID;
  if ((ells & (GBP_ELL0 | GBP_ELL2 | GBP_ELL4)) == 0 || (ells & ~15)) return GBP_ERR_INVALID;
  if ((ells & GBP_KSUM) && !ksum_out) return GBP_ERR_INVALID;
  return GBP_OK;
}

// The binning launches of gbp_power and gbp_power_noalloc: the persistent
// binning kernel writes the per-group float-float partials to part_ff
// (L.C * L.NV * nbe float2), then one block per bin folds them.
int launch_power(const void* spectrum, int G, int Lzs, gbp_bins B, int mas_order, int ells, const double* mass,
                 double* sums_out, long long* nmodes_out, double* ksum_out, const PowLayout& L, float2* part_ff,
                 cudaStream_t stream) {
  PowGeom g;
  g.s0 = static_cast<const float2*>(spectrum);
  g.s1 = G == 2 ? g.s0 + L.total : nullptr;
  g.N = B->N;
  g.Lz = B->N / 2 + 1;
  g.Lzs = Lzs;
  g.total = L.total;
  g.chunk = L.chunk;
  g.nb = B->nb;
  g.nbe = B->nbe;
  g.tu = B->last_closed;
  g.lut_shift = B->lut_shift;
  g.lut_n = B->lut_n;
  g.mas_order = mas_order;
  g.thr = B->d_thr;
  g.lut = B->d_lut;
  g.inv_sinc2 = B->d_inv_sinc2;
  g.eph = B->d_eph;
  g.zero_dc = mass != nullptr;
  g.part_ff = part_ff;
  g.warps = L.warps;
  // the wide kernel reads float4s: both grids must start 16-byte aligned
  const bool aligned = ((reinterpret_cast<uintptr_t>(g.s0) | reinterpret_cast<uintptr_t>(g.s1)) & 15u) == 0;
  const bool wide = L.wide && aligned;

  void (*kern)(PowGeom) = nullptr;
  const bool inter = G == 2;
#define GBP_PICK(NVv)                                                                                   \
  kern = wide ? (inter ? power_kernel<NVv, true, true> : power_kernel<NVv, false, true>)               \
              : (inter ? power_kernel<NVv, true, false> : power_kernel<NVv, false, false>);
  if (L.NV == 1) { GBP_PICK(1) } else if (L.NV == 2) { GBP_PICK(2) } else { GBP_PICK(3) }
#undef GBP_PICK
  GBP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  // persistent grid: as many CTAs as fit on the device at once (never more than the groups)
  int dev = 0, sms = 0, per_sm = 0;
  GBP_CUDA_TRY(cudaGetDevice(&dev));
  GBP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GBP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, L.warps * 32, L.smem));
  g.groups = L.C;
  const int grid = std::max(1, std::min(L.C, sms * std::max(per_sm, 1)));
  {
    GBP_TRACE("power_bins", stream);
    GBP_CUDA_TRY(launch_pdl(kern, dim3(grid), dim3(L.warps * 32), L.smem, stream, g));
  }
  GBP_TRACE("power_reduce", stream);
  GBP_CUDA_TRY(launch_pdl(power_reduce_kernel, dim3(B->nb), dim3(FOLD_THREADS), 0, stream,
                          static_cast<const float2*>(part_ff), L.C, L.NV, B->nb, B->nbe,
                          static_cast<const long long*>(B->d_nmodes), static_cast<const double*>(B->d_ksum), sums_out,
                          nmodes_out, (ells & GBP_KSUM) ? ksum_out : nullptr));
  return GBP_OK;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_power_workspace_size(gbp_bins bins, int G, int z_pitch, int ells, size_t* bytes) {
  if (!bins || !bytes || (G != 1 && G != 2)) return GBP_ERR_INVALID;
  PowLayout L;
  const int st = power_layout(bins, G, ells, z_pitch > 0 ? z_pitch : bins->N / 2 + 1, L);
  if (st) return st;
  *bytes = L.ws_total;
  return GBP_OK;
}

extern "C" int gbp_power(const void* spectrum, int G, int z_pitch, gbp_bins B, int mas_order, int ells,
                         const double* mass, double* sums_out, long long* nmodes_out, double* ksum_out,
                         void* workspace, size_t ws_bytes, gbp_stream_t stream_) {
  int st = power_args(spectrum, G, B, mas_order, ells, sums_out, nmodes_out, ksum_out);
  if (st) return st;
  const int Lzs = z_pitch > 0 ? z_pitch : B->N / 2 + 1;
  PowLayout L;
  st = power_layout(B, G, ells, Lzs, L);
  if (st) return st;
  if (!workspace || ws_bytes < L.ws_total) return GBP_ERR_WORKSPACE;
  Carver cv(workspace);
  float2* part_ff = cv.take<float2>((size_t)L.C * L.NV * B->nbe);
  return launch_power(spectrum, G, Lzs, B, mas_order, ells, mass, sums_out, nmodes_out, ksum_out, L, part_ff,
                      reinterpret_cast<cudaStream_t>(stream_));
}

extern "C" int gbp_power_normalize(const double* sums, const long long* nmodes, const double* ksum, int nb, int N,
                                   double box, const double* mass, const gbp_deposit_stats* stats,
                                   int subtract_shot, double* pk_out, double* kmean_out, gbp_stream_t stream_) {
  cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
  if (!sums || !nmodes || !pk_out || nb < 1 || N < 1 || !(box > 0.0)) return GBP_ERR_INVALID;
  const double n2 = (double)N * (double)N;
  const double norm_delta = (box / n2) * (box / n2) * (box / n2);
  const double box3 = box * box * box;
  const double kf = 2.0 * M_PI / box;
  GBP_TRACE("power_normalize", stream);
  GBP_CUDA_TRY(launch_pdl(power_normalize_kernel, dim3((nb + 127) / 128), dim3(128), 0, stream, sums, nmodes, ksum,
                          nb, norm_delta, box3, kf, mass, stats, subtract_shot, pk_out, kmean_out,
                          static_cast<const gbp_job*>(nullptr), N));
  return GBP_OK;
}

extern "C" int gbp_power_normalize_job(const double* sums, const long long* nmodes, const double* ksum, int nb,
                                       int N, const gbp_job* job, const double* mass,
                                       const gbp_deposit_stats* stats, int subtract_shot, double* pk_out,
                                       double* kmean_out, gbp_stream_t stream_) {
  cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
  if (!sums || !nmodes || !pk_out || !job || nb < 1 || N < 1) return GBP_ERR_INVALID;
  GBP_TRACE("power_normalize", stream);
  GBP_CUDA_TRY(launch_pdl(power_normalize_kernel, dim3((nb + 127) / 128), dim3(128), 0, stream, sums, nmodes, ksum,
                          nb, 0.0, 0.0, 0.0, mass, stats, subtract_shot, pk_out, kmean_out, job, N));
  return GBP_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free binning.  Some callers cannot allocate device memory when
// they call in: a JAX/XLA custom call (the way a JAX program would reach
// this path) is handed only its operand and result buffers, and its device
// memory belongs to JAX's allocator, which reserves most of the GPU up front,
// so a cudaMalloc of the library's own can fail or compete with it.
// gbp_power_noalloc is gbp_power with its scratch (the per-group float-float
// partial sums) in a fixed device array owned by the library, so the caller
// passes only inputs and outputs.
//
// Limit: groups * moments * bins <= GBP_NOALLOC_PARTIALS float2 (16 MiB), e.g.
// every 512^3 mesh with up to ~560 bins and l = 0,2,4.  Larger requests are
// rejected with GBP_ERR_UNSUPPORTED before anything is launched.
//
// The array lives in every GPU that loads the library, until the process
// exits.  Its device address is looked up once per device, with that device
// current, the first time the entry point runs there; make that first call
// before any stream capture.  All calls share the one array: calls whose
// kernels overlap on the GPU (different streams, no ordering between them)
// race on it.  Nothing needs clearing between calls: every partial the
// reduce kernel reads is written earlier in the same call.
namespace gbp {
namespace {
constexpr size_t GBP_NOALLOC_PARTIALS = (size_t)2 << 20;   // float2 entries (16 MiB)
__device__ __align__(256) float2 g_noalloc_partials[GBP_NOALLOC_PARTIALS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
float2* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the array on the current device (looked up once).
int noalloc_partials(float2** out) {
  int dev = 0;
  GBP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return GBP_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      return GBP_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = static_cast<float2*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return GBP_OK;
}
}  // namespace
}  // namespace gbp

extern "C" int gbp_power_noalloc(const void* spectrum, int G, int z_pitch, gbp_bins B, int mas_order, int ells,
                                 const double* mass, double* sums_out, long long* nmodes_out, double* ksum_out,
                                 gbp_stream_t stream_) {
  int st = power_args(spectrum, G, B, mas_order, ells, sums_out, nmodes_out, ksum_out);
  if (st) return st;
  const int Lzs = z_pitch > 0 ? z_pitch : B->N / 2 + 1;
  PowLayout L;
  st = power_layout(B, G, ells, Lzs, L);
  if (st) return st;
  if ((size_t)L.C * L.NV * B->nbe > GBP_NOALLOC_PARTIALS) return GBP_ERR_UNSUPPORTED;
  float2* part_ff = nullptr;
  st = noalloc_partials(&part_ff);
  if (st) return st;
  return launch_power(spectrum, G, Lzs, B, mas_order, ells, mass, sums_out, nmodes_out, ksum_out, L, part_ff,
                      reinterpret_cast<cudaStream_t>(stream_));
}
