// Two-point correlation multipoles xi_l(r) from the same |delta_k|^2 as P_l(k)
// (src/correlations.py:120-187 xi_vec, :641-712 compute_2pt_correlations):
//
//   1. forward R2C of the density contrast (the plan's transform),
//   2. pk_field_kernel: |delta_k|^2 (sinc)^(-2p) per axis, in place, as a
//      complex field with zero imaginary part,
//   3. inverse C2R (cuFFT, unnormalised: the field holds N^3 xi(r)),
//   4. xi_bin_kernel: separation shells on the full grid (signed offsets on
//      all three axes; integer r^2 against the bin plan's thresholds, the
//      jnp.histogram rule), moments sum xi, xi mu^2, xi mu^4 and the cell
//      count; runs along z are summed by warp segmented scans and flushed
//      half-pencil by half-pencil into per-warp float32 bins, folded in
//      float-float per work group and in double at the end (deterministic),
//   5. xi_reduce_kernel: Legendre sums and counts.
//
// mu = r_z / r; at r = 0 it is NaN (xi_vec divides 0 by 0) or 0
// (compute_2pt_correlations guards it), selected by the caller.
#include <cufft.h>
#include <math.h>

#include "gbp_bins.h"
#include "gbp_fft.h"
#include "gbp_internal.cuh"
#include "power_core.cuh"

namespace gbp {
namespace {

constexpr int XI_NV = 4;      // sum xi, xi mu^2, xi mu^4, count

__global__ void pk_field_kernel(float2* spec, int N, int P, const float* __restrict__ inv_sinc2, int mas_order) {
  const long long total = (long long)N * N * P;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int kz = (int)(i % P);
  if (kz > N / 2) return;                         // row padding: never read by the C2R
  const int iy = (int)((i / P) % N), ix = (int)(i / ((long long)P * N));
  const int ax = abs(signed_k(ix, N)), ay = abs(signed_k(iy, N));
  float w = 1.0f;
  for (int p = 0; p < mas_order; ++p) w *= inv_sinc2[ax] * inv_sinc2[ay] * inv_sinc2[kz];
  const float2 v = spec[i];
  spec[i] = make_float2((v.x * v.x + v.y * v.y) * w, 0.0f);
}

// One warp step over 32 consecutive cells of the flat [N][N][N] field.
__device__ __forceinline__ void xi_step(const PowGeom& g, const Smem& t, const float* __restrict__ field, float* wb,
                                        int lane, long long f, long long end, int nan_origin) {
  const int N = g.N;
  const bool valid = f < end;
  float v[XI_NV] = {0.f, 0.f, 0.f, 0.f};
  int bin = -1;
  const int z = (int)(f % N);
  const long long pen = f / N;
  const int hp = (int)(pen * 2 + (z > N / 2 ? 1 : 0));       // half-pencil: |r_z| is monotone inside it
  if (valid) {
    const int y = (int)(pen % N), x = (int)(pen / N);
    const int rx = signed_k(x, N), ry = signed_k(y, N), rz = signed_k(z, N);
    const int r2 = rx * rx + ry * ry + rz * rz;
    bin = bin_of(g, t, r2);
    const float xi = field[f];
    float mu2;
    if (r2 > 0) mu2 = __fdividef((float)(rz * rz), (float)r2);
    else mu2 = nan_origin ? __int_as_float(0x7fc00000) : 0.0f;
    v[0] = xi;
    v[1] = xi * mu2;
    v[2] = v[1] * mu2;
    v[3] = 1.0f;
  }
  const int bprev = __shfl_up_sync(0xffffffffu, bin, 1);
  const int hprev = __shfl_up_sync(0xffffffffu, hp, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || bin != bprev || hp != hprev);
  seg_scan<XI_NV>(v, heads, lane);
  const bool segend = (lane == 31) || ((heads >> (lane + 1)) & 1u);
  // runs of different half-pencils in one step may share a bin: flush phase by phase
  const int rel = hp - __shfl_sync(0xffffffffu, hp, 0);
  const int nph = __reduce_max_sync(0xffffffffu, valid ? rel : 0) + 1;
  for (int ph = 0; ph < nph; ++ph) {
    if (segend && bin >= 0 && rel == ph) bin_add<XI_NV>(wb, g.nbe, bin, v);
    __syncwarp();
  }
}

__global__ void __launch_bounds__(POW_WARPS * 32, 4)
xi_bin_kernel(PowGeom g, const float* __restrict__ field, int nan_origin) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Smem s = load_tables<XI_NV, false>(g, smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* wb = s.wbase + warp * XI_NV * g.nbe;
  for (int grp = blockIdx.x; grp < g.groups; grp += gridDim.x) {
    const long long beg = ((long long)grp * g.warps + warp) * g.chunk;
    const long long end = min(beg + g.chunk, g.total);
    for (long long f = beg + lane; f - lane < end; f += 32) xi_step(g, s, field, wb, lane, f, end, nan_origin);
    cta_fold<XI_NV>(g, s, grp);
  }
}

// One block per bin: the group partials folded in a fixed order (fold_bin),
// then the Legendre sums and the cell count.
__global__ void __launch_bounds__(FOLD_THREADS)
xi_reduce_kernel(const float2* __restrict__ part_ff, int C, int nb, int nbe, double* sums_out,
                 long long* counts_out) {
  const int b = blockIdx.x;
  if (b >= nb) return;                         // uniform over the block
  double m[XI_NV] = {0.0, 0.0, 0.0, 0.0};
  if (b < nbe) fold_bin<XI_NV>(part_ff, C, XI_NV, nbe, b, m);
  if (threadIdx.x == 0) {
    sums_out[b * 3 + 0] = m[0];
    sums_out[b * 3 + 1] = 1.5 * m[1] - 0.5 * m[0];
    sums_out[b * 3 + 2] = (35.0 * m[2] - 30.0 * m[1] + 3.0 * m[0]) * 0.125;
    counts_out[b] = (long long)llrint(m[3]);
  }
}

struct XiLayout {
  int warps, C;
  long long total, chunk;
  size_t smem, part, c2r_ws, total_ws;
};

int xi_layout(const gbp_bins_s* B, int P, size_t r2c_ws, XiLayout& L) {
  const int N = B->N;
  int w = POW_WARPS;
  while (w > 1 && smem_plan(N, B->nbe, B->lut_n, w, XI_NV).total > 200 * 1024) --w;
  L.smem = smem_plan(N, B->nbe, B->lut_n, w, XI_NV).total;
  if (L.smem > 200 * 1024) return GBP_ERR_UNSUPPORTED;
  L.warps = w;
  L.total = (long long)N * N * N;
  long long target = L.total / (8LL * 152 * 8);
  target = std::max(1024LL, std::min(16384LL, target));
  L.chunk = (target + 31) & ~31LL;
  const long long nw = (L.total + L.chunk - 1) / L.chunk;
  L.C = (int)((nw + w - 1) / w);
  L.part = align256((size_t)L.C * XI_NV * B->nbe * sizeof(float2));
  cufftHandle h;
  int st = c2r_plan(N, P, 1, &h, &L.c2r_ws);
  if (st) return st;
  if (r2c_ws > L.c2r_ws) L.c2r_ws = r2c_ws;          // one work area serves both transforms
  L.total_ws = L.part + align256(L.c2r_ws);
  return GBP_OK;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_xi_workspace_size(gbp_fft_plan plan, gbp_bins B, size_t* bytes) {
  if (!plan || !B || !bytes || plan->n != B->N || plan->grids != 1) return GBP_ERR_INVALID;
  XiLayout L;
  const int st = xi_layout(B, plan->pitch, plan->ws, L);
  if (st) return st;
  *bytes = L.total_ws;
  return GBP_OK;
}

extern "C" int gbp_xi(gbp_fft_plan plan, const float* delta, void* spectrum, float* field, gbp_bins B, int mas_order,
                      int nan_mu_at_origin, double* sums_out, long long* counts_out, void* workspace,
                      size_t ws_bytes, gbp_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!plan || !delta || !spectrum || !field || !B || !sums_out || !counts_out) return GBP_ERR_INVALID;
  if (plan->n != B->N || plan->grids != 1 || mas_order < 0 || mas_order > 8) return GBP_ERR_INVALID;
  XiLayout L;
  int r = xi_layout(B, plan->pitch, plan->ws, L);
  if (r) return r;
  if (!workspace || ws_bytes < L.total_ws) return GBP_ERR_WORKSPACE;
  const int N = B->N, P = plan->pitch;
  Carver cv(workspace);
  float2* part = cv.take<float2>(L.part / sizeof(float2));
  void* cws = cv.take<char>(L.c2r_ws);
  // 1. forward transform (library or cuFFT, as the plan says)
  r = gbp_fft_r2c(plan, delta, spectrum, cws, L.c2r_ws, stream_);
  if (r) return r;
  // 2. |delta_k|^2 W(k)^2
  float2* spec = static_cast<float2*>(spectrum);
  const long long total = (long long)N * N * P;
  {
    GBP_TRACE("xi_pk_field", st);
    pk_field_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(spec, N, P, B->d_inv_sinc2, mas_order);
    GBP_LAUNCH_CHECK();
  }
  // 3. inverse real transform (unnormalised)
  {
    GBP_TRACE("xi_c2r", st);
    r = c2r_exec(N, P, 1, spec, field, cws, st);
    if (r) return r;
  }
  // 4. separation shells
  PowGeom g{};
  g.N = N;
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
  int dev = 0, sms = 0, per_sm = 0;
  GBP_CUDA_TRY(cudaGetDevice(&dev));
  GBP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GBP_CUDA_TRY(cudaFuncSetAttribute(xi_bin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  GBP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, xi_bin_kernel, L.warps * 32, L.smem));
  const int grid = std::max(1, std::min(L.C, sms * std::max(per_sm, 1)));
  {
    GBP_TRACE("xi_bins", st);
    xi_bin_kernel<<<grid, L.warps * 32, L.smem, st>>>(g, field, nan_mu_at_origin ? 1 : 0);
    GBP_LAUNCH_CHECK();
  }
  {
    GBP_TRACE("xi_reduce", st);
    xi_reduce_kernel<<<B->nb, FOLD_THREADS, 0, st>>>(part, L.C, B->nb, B->nbe, sums_out, counts_out);
    GBP_LAUNCH_CHECK();
  }
  return GBP_OK;
}
