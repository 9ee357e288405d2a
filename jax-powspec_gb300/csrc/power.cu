// Fused post-FFT kernel: window deconvolution, interlacing combination,
// |delta_k|^2 x Legendre L_l(mu) (line of sight z) and k-shell binning.
//
// Layout: a spectrum is complex64 [N][N][Lz] with Lz = N/2+1 (cuFFT R2C).
// Each warp walks a contiguous run of that flat array, 32 modes per step
// (coalesced 8-byte loads).  Along a z pencil |k| grows with kz, so the
// 32 bins of a step form sorted runs; a warp-shuffle segmented scan sums
// each run and its last lane adds the run total to the warp's private
// float32 bins in shared memory.  Runs of different pencils in one step can
// share a bin, so the adds are issued pencil by pencil with __syncwarp()
// between them: no shared-memory atomics, a fixed order, bitwise
// reproducible results.  At the end each CTA folds its warps' bins into a
// float-float (hi, lo) partial, and power_reduce_kernel folds the CTAs'
// partials in a fixed order into double totals.  (GB300 runs FP64 at a
// small fraction of FP32 throughput, so doubles appear only in the totals.)
//
// Bin membership uses integer thresholds on k2 = kx^2+ky^2+kz^2 computed on
// the host (gbp_bin_thresholds), which reproduces jnp.histogram applied to
// k = sqrtf((float)k2) exactly, so mode counts match the reference bit for
// bit (src/correlations.py:34,42,45-48).
#include <math.h>

#include <algorithm>

#include "gbp_bins.h"
#include "gbp_internal.cuh"

namespace gbp {
namespace {

constexpr int POW_MAX_WARPS = 8;

struct PowGeom {
  const float2* s0;
  const float2* s1;
  int N, Lz;
  long long total;          // N*N*Lz modes per grid
  long long chunk;          // modes per warp
  int nb, nbe;              // bins, bins some mode can reach
  int tu;                   // closed upper k2 limit of the last bin
  int lut_shift, lut_n;
  int mas_order;
  const int* thr;           // [nbe+1]
  const int* lut;           // [lut_n]
  const float* inv_sinc2;   // [N/2+1] 1/sinc(pi k/N)^2
  const float2* eph;        // [N/2+1] exp(i pi k / N)
  const double* mass;       // nullable
  float2* part_ff;          // [C][NVT][nbe]
  long long* part_cnt;      // [C][nbe]
  int warps;
};

struct SmemPlan {
  size_t c2, eph, thr, lut, bins, total;
};

__host__ __device__ inline size_t a16(size_t b) { return (b + 15) & ~size_t(15); }

__host__ __device__ inline SmemPlan smem_plan(int N, int nbe, int lut_n, int warps, int NVT) {
  SmemPlan p;
  const int h = N / 2;
  p.c2 = 0;
  p.eph = p.c2 + a16((size_t)(h + 1) * 4);
  p.thr = p.eph + a16((size_t)(h + 1) * 8);
  p.lut = p.thr + a16((size_t)(nbe + 1) * 4);
  p.bins = p.lut + a16((size_t)lut_n * 4);
  p.total = p.bins + (size_t)warps * (NVT + 1) * nbe * 4;
  return p;
}

template <int NV, bool KS, bool INTER>
__global__ void __launch_bounds__(POW_MAX_WARPS * 32)
power_kernel(PowGeom g) {
  constexpr int NVT = NV + (KS ? 1 : 0);
  extern __shared__ __align__(16) unsigned char smem[];
  const SmemPlan sp = smem_plan(g.N, g.nbe, g.lut_n, g.warps, NVT);
  const int h = g.N / 2;
  float* c2 = reinterpret_cast<float*>(smem + sp.c2);
  float2* eph = reinterpret_cast<float2*>(smem + sp.eph);
  int* thr = reinterpret_cast<int*>(smem + sp.thr);
  int* lut = reinterpret_cast<int*>(smem + sp.lut);
  float* wbase = reinterpret_cast<float*>(smem + sp.bins);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int stride_w = (NVT + 1) * g.nbe;
  float* wb = wbase + warp * stride_w;                          // [NVT][nbe]
  int* wc = reinterpret_cast<int*>(wb + NVT * g.nbe);           // [nbe]

  for (int k = threadIdx.x; k <= h; k += blockDim.x) {
    float r = g.inv_sinc2[k], c = 1.0f;
    for (int p = 0; p < g.mas_order; ++p) c *= r;               // sinc^(-2 p)
    c2[k] = c;
    if (INTER) eph[k] = g.eph[k];
  }
  for (int k = threadIdx.x; k <= g.nbe; k += blockDim.x) thr[k] = g.thr[k];
  for (int k = threadIdx.x; k < g.lut_n; k += blockDim.x) lut[k] = g.lut[k];
  for (int k = threadIdx.x; k < g.warps * stride_w; k += blockDim.x) wbase[k] = 0.0f;  // int 0 == float 0 bits
  __syncthreads();

  const long long wglob = (long long)blockIdx.x * g.warps + warp;
  const long long beg = wglob * g.chunk;
  const long long end = min(beg + g.chunk, g.total);
  if (beg < end) {
    long long f = beg + lane;
    long long pen = f / g.Lz;
    int kz = (int)(f - pen * g.Lz);
    int iy = (int)(pen % g.N);
    int ix = (int)(pen / g.N);
    const double m0 = g.mass ? g.mass[0] : 0.0;
    const double m1 = (g.mass && INTER) ? g.mass[1] : 0.0;

    for (long long fb = beg; fb < end; fb += 32) {
      const bool valid = f < end;
      float v[NVT];
#pragma unroll
      for (int q = 0; q < NVT; ++q) v[q] = 0.0f;
      int bin = -1;
      if (valid) {
        const int kx = signed_k(ix, g.N), ky = signed_k(iy, g.N);
        const int ax = kx < 0 ? -kx : kx, ay = ky < 0 ? -ky : ky;
        const int k2 = kx * kx + ky * ky + kz * kz;
        float2 a = g.s0[f];
        float re, im;
        if (INTER) {
          float2 b = g.s1[f];
          if (f == 0 && g.mass) {
            a.x = (float)((double)a.x - m0);
            b.x = (float)((double)b.x - m1);
          }
          // exp(i pi (kx+ky+kz)/N) from the |k| table (conjugate for k < 0)
          float2 ex = eph[ax], ey = eph[ay], ez = eph[kz];
          if (kx < 0) ex.y = -ex.y;
          if (ky < 0) ey.y = -ey.y;
          const float pr = ex.x * ey.x - ex.y * ey.y;
          const float pi = ex.x * ey.y + ex.y * ey.x;
          const float qr = pr * ez.x - pi * ez.y;
          const float qi = pr * ez.y + pi * ez.x;
          re = 0.5f * (a.x + (b.x * qr - b.y * qi));
          im = 0.5f * (a.y + (b.x * qi + b.y * qr));
        } else {
          if (f == 0 && g.mass) a.x = (float)((double)a.x - m0);
          re = a.x;
          im = a.y;
        }
        const float p = (re * re + im * im) * (c2[ax] * c2[ay] * c2[kz]);
        v[0] = p;
        if (NV > 1) {
          const float mu2 = k2 > 0 ? __fdividef((float)(kz * kz), (float)k2) : 0.0f;
          v[1] = p * (1.5f * mu2 - 0.5f);
          if (NV > 2) v[2] = p * ((4.375f * mu2 - 3.75f) * mu2 + 0.375f);
        }
        if (KS) v[NV] = sqrtf((float)k2);
        if (k2 <= g.tu) {
          int r = lut[k2 >> g.lut_shift];
          while (r <= g.nbe && thr[r] <= k2) ++r;
          bin = min(min(r, g.nb), g.nbe) - 1;   // r <= nbe whenever nbe < nb; the clamp only guards
        }
      }
      // segmented inclusive scan over runs of equal bin
      const int bprev = __shfl_up_sync(0xffffffffu, bin, 1);
      const bool head = (lane == 0) || (bin != bprev);
      const unsigned hm = __ballot_sync(0xffffffffu, head);
      const int segstart = 31 - __clz(hm & (0xffffffffu >> (31 - lane)));
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const bool take = lane - d >= segstart;
#pragma unroll
        for (int q = 0; q < NVT; ++q) {
          const float t = __shfl_up_sync(0xffffffffu, v[q], d);
          if (take) v[q] += t;
        }
      }
      const bool segend = (lane == 31) || ((hm >> (lane + 1)) & 1u);
      // flush pencil by pencil (a bin can repeat only across pencils)
      const int pid = ix * g.N + iy;
      const int rel = pid - __shfl_sync(0xffffffffu, pid, 0);
      const int nph = __shfl_sync(0xffffffffu, rel, 31) + 1;
      for (int ph = 0; ph < nph; ++ph) {
        if (segend && bin >= 0 && rel == ph) {
#pragma unroll
          for (int q = 0; q < NVT; ++q) wb[q * g.nbe + bin] += v[q];
          wc[bin] += lane - segstart + 1;
        }
        __syncwarp();
      }
      f += 32;
      kz += 32;
      while (kz >= g.Lz) {
        kz -= g.Lz;
        if (++iy == g.N) { iy = 0; ++ix; }
      }
    }
  }
  __syncthreads();

  // CTA fold: warps in order, float-float; counts in int64.
  float2* pf = g.part_ff + (long long)blockIdx.x * NVT * g.nbe;
  long long* pc = g.part_cnt + (long long)blockIdx.x * g.nbe;
  for (int b = threadIdx.x; b < g.nbe; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NVT; ++q) {
      ff s{0.f, 0.f};
      for (int w = 0; w < g.warps; ++w) s = ff_add_f(s, wbase[w * stride_w + q * g.nbe + b]);
      pf[q * g.nbe + b] = make_float2(s.hi, s.lo);
    }
    long long c = 0;
    for (int w = 0; w < g.warps; ++w) c += reinterpret_cast<const int*>(wbase + w * stride_w + NVT * g.nbe)[b];
    pc[b] = c;
  }
}

// One warp per bin: fold the CTA partials (fixed order) into doubles.
__global__ void power_reduce_kernel(const float2* __restrict__ part_ff, const long long* __restrict__ part_cnt,
                                    int C, int NV, int KS, int nb, int nbe, double* sums_out,
                                    long long* nmodes_out, double* ksum_out) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nb) return;
  const int NVT = NV + KS;
  double tot[4] = {0.0, 0.0, 0.0, 0.0};
  long long cnt = 0;
  if (b < nbe) {
    for (int q = 0; q < NVT; ++q) {
      ff s{0.f, 0.f};
      for (int c = lane; c < C; c += 32) {
        const float2 v = part_ff[((long long)c * NVT + q) * nbe + b];
        s = ff_add(s, ff{v.x, v.y});
      }
      for (int o = 16; o > 0; o >>= 1) {
        ff t{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
        s = ff_add(s, t);
      }
      tot[q] = (double)s.hi + (double)s.lo;
    }
    for (int c = lane; c < C; c += 32) cnt += part_cnt[(long long)c * nbe + b];
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if (lane == 0) {
    for (int l = 0; l < 3; ++l) sums_out[b * 3 + l] = l < NV ? tot[l] : 0.0;
    nmodes_out[b] = cnt;
    if (ksum_out) ksum_out[b] = KS ? tot[NV] : 0.0;
  }
}

__global__ void power_normalize_kernel(const double* sums, const long long* nmodes, const double* ksum, int nb,
                                       double norm_delta, double box3, double kf, const double* mass,
                                       const gbp_deposit_stats* stats, int subtract_shot, double* pk_out,
                                       double* kmean_out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  double norm = norm_delta, shot = 0.0;
  if (mass) {
    const double m = mass[0];
    norm = box3 / (m * m);
    if (subtract_shot && stats) shot = box3 * stats->sum_w2 / (m * m);
  }
  const double n = (double)nmodes[b];
  for (int l = 0; l < 3; ++l) {
    double p = (4.0 * l + 1.0) * sums[b * 3 + l] / n * norm;  // 0/0 -> NaN, as the reference
    if (l == 0) p -= shot;
    pk_out[b * 3 + l] = p;
  }
  if (kmean_out) kmean_out[b] = ksum ? ksum[b] / n * kf : 0.0;
}

struct PowLayout {
  int NV, KS, warps, C;
  long long total, chunk;
  size_t smem, ws_total;
};

// A pure function of (N, bins, ells): the summation order, and therefore the
// result, is the same on every device.
int power_layout(const gbp_bins_s* B, int ells, PowLayout& L) {
  L.NV = (ells & GBP_ELL4) ? 3 : ((ells & GBP_ELL2) ? 2 : 1);
  L.KS = (ells & GBP_KSUM) ? 1 : 0;
  const int NVT = L.NV + L.KS;
  const size_t budget = 200 * 1024;
  int w = POW_MAX_WARPS;
  while (w > 1 && smem_plan(B->N, B->nbe, B->lut_n, w, NVT).total > budget) --w;
  L.smem = smem_plan(B->N, B->nbe, B->lut_n, w, NVT).total;
  if (L.smem > budget) return GBP_ERR_UNSUPPORTED;
  L.warps = w;
  L.total = (long long)B->N * B->N * (B->N / 2 + 1);
  long long target = L.total / (8LL * 152 * 4);
  target = std::max(1024LL, std::min(8192LL, target));
  L.chunk = (target + 31) & ~31LL;
  const long long nw = (L.total + L.chunk - 1) / L.chunk;
  L.C = (int)((nw + w - 1) / w);
  L.ws_total = align256((size_t)L.C * NVT * B->nbe * sizeof(float2)) + align256((size_t)L.C * B->nbe * 8);
  return GBP_OK;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_power_workspace_size(gbp_bins bins, int G, int ells, size_t* bytes) {
  if (!bins || !bytes || (G != 1 && G != 2)) return GBP_ERR_INVALID;
  PowLayout L;
  int st = power_layout(bins, ells, L);
  if (st) return st;
  *bytes = L.ws_total;
  return GBP_OK;
}

extern "C" int gbp_power(const void* spectrum, int G, gbp_bins B, int mas_order, int ells, const double* mass,
                         double* sums_out, long long* nmodes_out, double* ksum_out, void* workspace,
                         size_t ws_bytes, gbp_stream_t stream_) {
  cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
  if (!spectrum || !B || !sums_out || !nmodes_out) return GBP_ERR_INVALID;
  if (G != 1 && G != 2) return GBP_ERR_INVALID;
  if (mas_order < 0 || mas_order > 8) return GBP_ERR_INVALID;
  if ((ells & (GBP_ELL0 | GBP_ELL2 | GBP_ELL4)) == 0 || (ells & ~15)) return GBP_ERR_INVALID;
  if ((ells & GBP_KSUM) && !ksum_out) return GBP_ERR_INVALID;
  PowLayout L;
  int st = power_layout(B, ells, L);
  if (st) return st;
  if (!workspace || ws_bytes < L.ws_total) return GBP_ERR_WORKSPACE;

  Carver cv(workspace);
  float2* part_ff = cv.take<float2>((size_t)L.C * (L.NV + L.KS) * B->nbe);
  long long* part_cnt = cv.take<long long>((size_t)L.C * B->nbe);

  PowGeom g;
  g.s0 = static_cast<const float2*>(spectrum);
  g.s1 = G == 2 ? g.s0 + L.total : nullptr;
  g.N = B->N;
  g.Lz = B->N / 2 + 1;
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
  g.mass = mass;
  g.part_ff = part_ff;
  g.part_cnt = part_cnt;
  g.warps = L.warps;

  void (*kern)(PowGeom) = nullptr;
  const bool inter = G == 2;
#define GBP_PICK(NVv, KSv) kern = inter ? power_kernel<NVv, KSv, true> : power_kernel<NVv, KSv, false>;
  if (L.KS) {
    if (L.NV == 1) { GBP_PICK(1, true) } else if (L.NV == 2) { GBP_PICK(2, true) } else { GBP_PICK(3, true) }
  } else {
    if (L.NV == 1) { GBP_PICK(1, false) } else if (L.NV == 2) { GBP_PICK(2, false) } else { GBP_PICK(3, false) }
  }
#undef GBP_PICK
  GBP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  kern<<<L.C, L.warps * 32, L.smem, stream>>>(g);
  GBP_LAUNCH_CHECK();
  const int wpb = 8;
  power_reduce_kernel<<<(B->nb + wpb - 1) / wpb, wpb * 32, 0, stream>>>(
      part_ff, part_cnt, L.C, L.NV, L.KS, B->nb, B->nbe, sums_out, nmodes_out, ksum_out);
  GBP_LAUNCH_CHECK();
  return GBP_OK;
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
  power_normalize_kernel<<<(nb + 127) / 128, 128, 0, stream>>>(sums, nmodes, ksum, nb, norm_delta, box3, kf, mass,
                                                               stats, subtract_shot, pk_out, kmean_out);
  GBP_LAUNCH_CHECK();
  return GBP_OK;
}
