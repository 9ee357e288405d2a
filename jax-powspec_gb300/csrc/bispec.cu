// The FFT bispectrum estimator of src/correlations.py:334-462 (`bispec`):
// for shells |k| in [k_i - kF, k_i + kF) around k_1, k_2 and k_3(theta),
//
//   delta_i(x) = irfftn(mask_i W delta_k),   I_i(x) = irfftn(mask_i),
//   P_i = sum_x delta_i^2 / sum_x I_i^2 (L / N^2)^3,
//   B   = sum_x delta_1 delta_2 delta_3 / sum_x I_1 I_2 I_3 (L^2 / N^3)^3,
//   Q   = B / (P_1 P_2 + P_1 P_3 + P_2 P_3).
//
// The reference transforms two fields back per shell (2 (n_theta + 2)
// inverse FFTs).  Here Parseval's theorem moves every sum but the first two
// shells' fields to Fourier space:
//
//   sum_x delta_i^2        = N^-3 sum_k |mask_i W delta_k|^2
//   sum_x I_i^2            = N^-3 n_i                   (modes in shell i)
//   sum_x delta_1 delta_2 delta_3 = N^-3 sum_k mask_3 W delta_k conj(FFT(delta_1 delta_2))
//   sum_x I_1 I_2 I_3      = N^-3 sum_k mask_3 conj(FFT(I_1 I_2))
//
// so a whole theta scan costs four inverse transforms (delta_1, delta_2,
// I_1, I_2), two forward transforms (of the products delta_1 delta_2 and
// I_1 I_2) and one pass over the spectrum that bins every mode once:
//
//   1. R2C of the contrast (the plan's transform) into the caller's spectrum,
//   2. bispec_fill_kernel: mask_1 W delta_k, mask_2 W delta_k, mask_1, mask_2
//      as four half spectra,
//   3. one batched cuFFT C2R of the four (unnormalised; the common factor
//      N^3 cancels in every ratio),
//   4. bispec_products_kernel: delta_1 delta_2 and I_1 I_2, in place,
//   5. the plan's R2C of the two products,
//   6. bispec_bin_kernel: every half-spectrum mode with its Hermitian weight
//      (2, or 1 on the kz = 0 and Nyquist planes) into elementary bins --
//      the intervals between consecutive shell limits, so that every shell
//      is a run of them -- with four sums: w |W delta|^2, w W Re(delta
//      conj D), w Re J, w; per-warp float32 bins, float-float partials,
//   7. bispec_reduce_kernel: the partials in double, in a fixed order,
//   8. bispec_finish_kernel: shell sums from their elementary bins, P, B, Q.
//
// Shell membership is the reference's float32 rule, k = sqrtf(k^2) >=
// (k_i - kF) / kF and < (k_i + kF) / kF, through the bin plan's integer k^2
// thresholds.  Deterministic: no float atomics.
#include <cufft.h>
#include <limits.h>
#include <math.h>

#include "gbp_bins.h"
#include "gbp_fft.h"
#include "gbp_internal.cuh"
#include "power_core.cuh"

namespace gbp {
namespace {

constexpr int BK_NV = 4;   // w |W delta|^2, w W Re(delta conj D), w Re J, w

// Amplitude window of one axis, sinc^(-p) = (1/sinc^2)^(p/2).
__device__ __forceinline__ float amp_axis(float inv_sinc2, int p) {
  float a = 1.0f;
  for (int i = 0; i < (p >> 1); ++i) a *= inv_sinc2;
  if (p & 1) a *= sqrtf(inv_sinc2);
  return a;
}

// k^2 threshold of elementary edge e: modes with k^2 >= it are at or above the edge.
__device__ __forceinline__ int edge_q(const int* __restrict__ thr, int nbe, int e) {
  if (e <= 0) return e < 0 ? 0 : __ldg(thr);
  return e <= nbe ? __ldg(thr + e) : INT_MAX;      // edges past nbe are beyond every mode
}

__global__ void bispec_fill_kernel(const float2* __restrict__ spec, int P, float2* __restrict__ A, int Pc, int N,
                                   const int* __restrict__ thr, int nbe, const int* __restrict__ shell_bins,
                                   const float* __restrict__ inv_sinc2, int p) {
  const long long T = (long long)N * N * Pc;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T) return;
  const int kz = (int)(i % Pc);
  const long long row = i / Pc;
  const int iy = (int)(row % N), ix = (int)(row / N);
  const int kx = signed_k(ix, N), ky = signed_k(iy, N);
  const int k2 = kx * kx + ky * ky + kz * kz;
  const bool m1 = k2 >= edge_q(thr, nbe, __ldg(shell_bins + 0)) && k2 < edge_q(thr, nbe, __ldg(shell_bins + 1));
  const bool m2 = k2 >= edge_q(thr, nbe, __ldg(shell_bins + 2)) && k2 < edge_q(thr, nbe, __ldg(shell_bins + 3));
  float2 v1 = make_float2(0.f, 0.f), v2 = v1;
  if (m1 || m2) {
    const float c = amp_axis(__ldg(inv_sinc2 + abs(kx)), p) * amp_axis(__ldg(inv_sinc2 + abs(ky)), p) *
                    amp_axis(__ldg(inv_sinc2 + kz), p);
    const float2 d = spec[row * P + kz];
    const float2 cd = make_float2(d.x * c, d.y * c);
    if (m1) v1 = cd;
    if (m2) v2 = cd;
  }
  A[i] = v1;
  A[T + i] = v2;
  A[2 * T + i] = make_float2(m1 ? 1.f : 0.f, 0.f);
  A[3 * T + i] = make_float2(m2 ? 1.f : 0.f, 0.f);
}

// R[0] <- R[0] R[1], R[1] <- R[2] R[3] (fields of M cells each).
__global__ void bispec_products_kernel(float* R, long long M) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  if ((M & 3) == 0) {
    float4* r4 = reinterpret_cast<float4*>(R);
    const long long M4 = M >> 2;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M4; i += stride) {
      const float4 a = r4[i], b = r4[M4 + i], c = r4[2 * M4 + i], d = r4[3 * M4 + i];
      r4[i] = make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w);
      r4[M4 + i] = make_float4(c.x * d.x, c.y * d.y, c.z * d.z, c.w * d.w);
    }
  } else {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += stride) {
      const float a = R[i], b = R[M + i], c = R[2 * M + i], d = R[3 * M + i];
      R[i] = a * b;
      R[M + i] = c * d;
    }
  }
}

// One warp step over 32 consecutive entries of the [N][N][P] spectra.
__device__ __forceinline__ void bk_step(const PowGeom& g, const Smem& t, const float2* __restrict__ sd,
                                        const float2* __restrict__ sD, const float2* __restrict__ sJ, float* wb,
                                        int lane, long long f, long long end) {
  const int N = g.N, P = g.Lzs, h = N / 2;
  const int kz = (int)(f % P);
  const long long row = f / P;
  float v[BK_NV] = {0.f, 0.f, 0.f, 0.f};
  int bin = -1;
  if (f < end && kz <= h) {
    const int iy = (int)(row % N), ix = (int)(row / N);
    const int kx = signed_k(ix, N), ky = signed_k(iy, N);
    bin = bin_of(g, t, kx * kx + ky * ky + kz * kz);
    if (bin >= 0) {
      const float c = t.c2[kx < 0 ? -kx : kx] * t.c2[ky < 0 ? -ky : ky] * t.c2[kz];
      const float w = (kz == 0 || ((N & 1) == 0 && kz == h)) ? 1.0f : 2.0f;
      const float2 d = sd[f], D = sD[f], J = sJ[f];
      const float dr = d.x * c, di = d.y * c;
      v[0] = w * (dr * dr + di * di);
      v[1] = w * (dr * D.x + di * D.y);
      v[2] = w * J.x;
      v[3] = w;
    }
  }
  const long long rprev = __shfl_up_sync(0xffffffffu, row, 1);
  const int bprev = __shfl_up_sync(0xffffffffu, bin, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || bin != bprev || row != rprev);
  seg_scan<BK_NV>(v, heads, lane);
  const bool segend = (lane == 31) || ((heads >> (lane + 1)) & 1u);
  // runs of different z rows in one step may share a bin: flush row by row
  const int rel = (int)(row - __shfl_sync(0xffffffffu, row, 0));
  const int nph = __reduce_max_sync(0xffffffffu, f < end ? rel : 0) + 1;
  for (int ph = 0; ph < nph; ++ph) {
    if (segend && bin >= 0 && rel == ph) bin_add<BK_NV>(wb, g.nbe, bin, v);
    __syncwarp();
  }
}

__global__ void __launch_bounds__(POW_WARPS * 32, 4)
bispec_bin_kernel(PowGeom g, const float2* __restrict__ sD, const float2* __restrict__ sJ, int p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Smem s = load_tables<BK_NV, false>(g, smem);          // g.mas_order = 0: c2 is rewritten below
  for (int k = threadIdx.x; k <= g.N / 2; k += blockDim.x) s.c2[k] = amp_axis(g.inv_sinc2[k], p);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* wb = s.wbase + warp * BK_NV * g.nbe;
  for (int grp = blockIdx.x; grp < g.groups; grp += gridDim.x) {
    const long long beg = ((long long)grp * g.warps + warp) * g.chunk;
    const long long end = min(beg + g.chunk, g.total);
    for (long long f = beg + lane; f - lane < end; f += 32) bk_step(g, s, g.s0, sD, sJ, wb, lane, f, end);
    cta_fold<BK_NV>(g, s, grp);
  }
}

// One block per elementary bin: the C group partials folded in a fixed order (fold_bin).
__global__ void __launch_bounds__(FOLD_THREADS)
bispec_reduce_kernel(const float2* __restrict__ part_ff, int C, int nbe, double* E) {
  const int b = blockIdx.x;
  if (b >= nbe) return;                        // uniform over the block
  double m[BK_NV] = {0.0, 0.0, 0.0, 0.0};
  fold_bin<BK_NV>(part_ff, C, BK_NV, nbe, b, m);
  if (threadIdx.x == 0)
    for (int q = 0; q < BK_NV; ++q) E[b * BK_NV + q] = m[q];
}

struct ShellSums {
  double p, b, t, n;
};

__device__ ShellSums shell_sums(const double* __restrict__ E, int nbe, const int* __restrict__ shell_bins, int s) {
  const int lo = max(0, shell_bins[2 * s]), hi = min(nbe, shell_bins[2 * s + 1]);
  ShellSums r{0.0, 0.0, 0.0, 0.0};
  for (int e = lo; e < hi; ++e) {
    r.p += E[e * BK_NV + 0];
    r.b += E[e * BK_NV + 1];
    r.t += E[e * BK_NV + 2];
    r.n += E[e * BK_NV + 3];
  }
  return r;
}

__global__ void bispec_finish_kernel(const double* __restrict__ E, int nbe, const int* __restrict__ shell_bins,
                                     int S, int N, double box, double* pk_out, double* bk_out, double* qk_out,
                                     long long* nmodes_out) {
  const double n3 = (double)N * N * N;
  const double pnorm = (box / ((double)N * N)) * (box / ((double)N * N)) * (box / ((double)N * N));
  const double l2n3 = box * box / n3;
  const double bnorm = l2n3 * l2n3 * l2n3;
  const ShellSums a = shell_sums(E, nbe, shell_bins, 0), b = shell_sums(E, nbe, shell_bins, 1);
  const double p1 = a.p / a.n * pnorm, p2 = b.p / b.n * pnorm;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const ShellSums r = s == 0 ? a : (s == 1 ? b : shell_sums(E, nbe, shell_bins, s));
    const double p3 = r.p / r.n * pnorm;
    pk_out[s] = p3;
    if (nmodes_out) nmodes_out[s] = (long long)llrint(r.n);
    if (s >= 2) {
      const double bk = r.b / r.t * bnorm;
      bk_out[s - 2] = bk;
      qk_out[s - 2] = bk / (p1 * p2 + p1 * p3 + p2 * p3);
    }
  }
}

struct BkLayout {
  int warps, C, Pc;
  long long total, chunk;
  size_t smem, A, R, part, E, cws, total_ws;
};

int bk_layout(const gbp_fft_plan_s* plan, const gbp_bins_s* B, BkLayout& L) {
  const int N = plan->n;
  int w = POW_WARPS;
  while (w > 1 && smem_plan(N, B->nbe, B->lut_n, w, BK_NV).total > 200 * 1024) --w;
  L.smem = smem_plan(N, B->nbe, B->lut_n, w, BK_NV).total;
  if (L.smem > 200 * 1024) return GBP_ERR_UNSUPPORTED;
  L.warps = w;
  L.Pc = N / 2 + 1;
  L.total = (long long)N * N * plan->pitch;
  long long target = L.total / (8LL * 152 * 8);
  target = std::max(1024LL, std::min(16384LL, target));
  L.chunk = (target + 31) & ~31LL;
  const long long nw = (L.total + L.chunk - 1) / L.chunk;
  L.C = (int)((nw + w - 1) / w);
  const size_t M = (size_t)N * N * N;
  // the four half spectra; the two product spectra later reuse the same bytes
  L.A = align256(std::max((size_t)4 * N * N * L.Pc, (size_t)2 * N * N * plan->pitch) * sizeof(float2));
  L.R = align256(4 * M * sizeof(float));
  L.part = align256((size_t)L.C * BK_NV * B->nbe * sizeof(float2));
  L.E = align256((size_t)B->nbe * BK_NV * sizeof(double));
  cufftHandle h;
  size_t cw = 0;
  const int st = c2r_plan(N, L.Pc, 4, &h, &cw);
  if (st) return st;
  L.cws = align256(std::max(std::max(cw, plan->ws), (size_t)1));
  L.total_ws = L.A + L.R + L.part + L.E + L.cws;
  return GBP_OK;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_bispec_workspace_size(gbp_fft_plan plan, gbp_bins B, size_t* bytes) {
  if (!plan || !B || !bytes || plan->n != B->N || plan->grids != 1) return GBP_ERR_INVALID;
  BkLayout L;
  const int st = bk_layout(plan, B, L);
  if (st) return st;
  *bytes = L.total_ws;
  return GBP_OK;
}

extern "C" int gbp_bispec(gbp_fft_plan plan, const float* delta, void* spectrum, gbp_bins B, int mas_order,
                          const int32_t* shell_bins, int n_shells, double box_size, double* pk_out, double* bk_out,
                          double* qk_out, long long* nmodes_out, void* workspace, size_t ws_bytes,
                          gbp_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!plan || !delta || !spectrum || !B || !shell_bins || !pk_out || !(box_size > 0.0)) return GBP_ERR_INVALID;
  if (plan->n != B->N || plan->grids != 1 || mas_order < 0 || mas_order > 8 || n_shells < 2) return GBP_ERR_INVALID;
  if (n_shells > 2 && (!bk_out || !qk_out)) return GBP_ERR_INVALID;
  BkLayout L;
  int r = bk_layout(plan, B, L);
  if (r) return r;
  if (!workspace || ws_bytes < L.total_ws) return GBP_ERR_WORKSPACE;
  const int N = plan->n, P = plan->pitch;
  const long long M = (long long)N * N * N, T = (long long)N * N * L.Pc;
  Carver cv(workspace);
  float2* A = cv.take<float2>(L.A / sizeof(float2));
  float* R = cv.take<float>(L.R / sizeof(float));
  float2* part = cv.take<float2>(L.part / sizeof(float2));
  double* E = cv.take<double>(L.E / sizeof(double));
  void* cws = cv.take<char>(L.cws);
  // 1. forward transform of the contrast
  r = gbp_fft_r2c(plan, delta, spectrum, cws, L.cws, stream_);
  if (r) return r;
  // 2. the first two shells' masked spectra and masks
  {
    GBP_TRACE("bispec_fill", st);
    bispec_fill_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(static_cast<const float2*>(spectrum), P, A,
                                                                     L.Pc, N, B->d_thr, B->nbe, shell_bins,
                                                                     B->d_inv_sinc2, mas_order);
    GBP_LAUNCH_CHECK();
  }
  // 3. their fields
  {
    GBP_TRACE("bispec_c2r", st);
    r = c2r_exec(N, L.Pc, 4, A, R, cws, st);
    if (r) return r;
  }
  // 4. delta_1 delta_2 and I_1 I_2
  int dev = 0, sms = 0;
  GBP_CUDA_TRY(cudaGetDevice(&dev));
  GBP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  {
    GBP_TRACE("bispec_products", st);
    const long long work = (M & 3) == 0 ? M / 4 : M;
    const int grid = (int)std::max(1LL, std::min((long long)sms * 8, (work + 255) / 256));
    bispec_products_kernel<<<grid, 256, 0, st>>>(R, M);
    GBP_LAUNCH_CHECK();
  }
  // 5. their spectra (the plan's transform), over the consumed half spectra
  float2* sD = A;
  float2* sJ = A + (long long)N * N * P;
  r = gbp_fft_r2c(plan, R, sD, cws, L.cws, stream_);
  if (r) return r;
  r = gbp_fft_r2c(plan, R + M, sJ, cws, L.cws, stream_);
  if (r) return r;
  // 6. one pass over the spectrum into elementary bins
  PowGeom g{};
  g.s0 = static_cast<const float2*>(spectrum);
  g.N = N;
  g.Lz = N / 2 + 1;
  g.Lzs = P;
  g.total = L.total;
  g.chunk = L.chunk;
  g.nb = B->nb;
  g.nbe = B->nbe;
  g.tu = B->last_closed;
  g.lut_shift = B->lut_shift;
  g.lut_n = B->lut_n;
  g.mas_order = 0;
  g.thr = B->d_thr;
  g.lut = B->d_lut;
  g.inv_sinc2 = B->d_inv_sinc2;
  g.eph = B->d_eph;
  g.part_ff = part;
  g.warps = L.warps;
  g.groups = L.C;
  int per_sm = 0;
  GBP_CUDA_TRY(cudaFuncSetAttribute(bispec_bin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  GBP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bispec_bin_kernel, L.warps * 32, L.smem));
  {
    GBP_TRACE("bispec_bins", st);
    const int grid = std::max(1, std::min(L.C, sms * std::max(per_sm, 1)));
    bispec_bin_kernel<<<grid, L.warps * 32, L.smem, st>>>(g, sD, sJ, mas_order);
    GBP_LAUNCH_CHECK();
  }
  {
    GBP_TRACE("bispec_reduce", st);
    bispec_reduce_kernel<<<B->nbe, FOLD_THREADS, 0, st>>>(part, L.C, B->nbe, E);
    GBP_LAUNCH_CHECK();
  }
  {
    GBP_TRACE("bispec_finish", st);
    bispec_finish_kernel<<<1, 256, 0, st>>>(E, B->nbe, shell_bins, n_shells, N, box_size, pk_out, bk_out, qk_out,
                                            nmodes_out);
    GBP_LAUNCH_CHECK();
  }
  return GBP_OK;
}
