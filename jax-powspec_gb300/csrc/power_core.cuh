// Binning helpers shared by the binning kernels (power.cu, xbin.cu): work
// geometry, shared-memory tables, bin lookup on integer k^2, warp segmented
// scans, per-warp bins and their deterministic folds.
#pragma once

#include <math.h>

#include "gbp_bins.h"
#include "gbp_internal.cuh"

namespace gbp {
namespace {

constexpr int POW_WARPS = 8;

struct PowGeom {
  const float2* s0;
  const float2* s1;
  int N, Lz;                // Lz = N/2+1 modes per z row
  int Lzs;                  // z row pitch (>= Lz); entries kz >= Lz are padding
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
  int zero_dc;              // density mesh: delta(k=0) = 0 exactly
  float2* part_ff;          // [C][NV][nbe]
  int warps;
  int groups;               // work groups (g.warps chunks each), one partial per group
  // fused x-pass + binning (xbin.cu) only
  const float2* tw;         // [N] exp(-2 pi i e / N)
  int items, nkb;           // (y, kz block) work items; kz blocks per row
};

struct SmemPlan {
  size_t c2, eph, thr, lut, bins, total;
};

__host__ __device__ inline size_t a16(size_t b) { return (b + 15) & ~size_t(15); }

__host__ __device__ inline SmemPlan smem_plan(int N, int nbe, int lut_n, int warps, int NV) {
  SmemPlan p;
  const int h = N / 2;
  p.c2 = 0;
  p.eph = p.c2 + a16((size_t)(h + 1) * 4);
  p.thr = p.eph + a16((size_t)(h + 1) * 8);
  p.lut = p.thr + a16((size_t)(nbe + 1) * 4);
  p.bins = p.lut + a16((size_t)lut_n * 4);
  p.total = p.bins + (size_t)warps * NV * nbe * 4;
  return p;
}

struct Smem {
  float* c2;
  float2* eph;
  int* thr;
  int* lut;
  float* wbase;
};

template <int NV, bool INTER>
__device__ __forceinline__ Smem load_tables(const PowGeom& g, unsigned char* smem) {
  const SmemPlan sp = smem_plan(g.N, g.nbe, g.lut_n, g.warps, NV);
  Smem s;
  s.c2 = reinterpret_cast<float*>(smem + sp.c2);
  s.eph = reinterpret_cast<float2*>(smem + sp.eph);
  s.thr = reinterpret_cast<int*>(smem + sp.thr);
  s.lut = reinterpret_cast<int*>(smem + sp.lut);
  s.wbase = reinterpret_cast<float*>(smem + sp.bins);
  const int h = g.N / 2;
  for (int k = threadIdx.x; k <= h; k += blockDim.x) {
    const float r = g.inv_sinc2[k];
    float c = 1.0f;
    for (int p = 0; p < g.mas_order; ++p) c *= r;  // sinc^(-2 mas_order)
    s.c2[k] = c;
    if (INTER) s.eph[k] = g.eph[k];
  }
  for (int k = threadIdx.x; k <= g.nbe; k += blockDim.x) s.thr[k] = g.thr[k];
  for (int k = threadIdx.x; k < g.lut_n; k += blockDim.x) s.lut[k] = g.lut[k];
  for (int k = threadIdx.x; k < g.warps * NV * g.nbe; k += blockDim.x) s.wbase[k] = 0.0f;
  __syncthreads();
  return s;
}

// Bin of k2 (>= 0), or -1 when outside the edges.
__device__ __forceinline__ int bin_of(const PowGeom& g, const Smem& s, int k2) {
  if (k2 > g.tu) return -1;
  int r = s.lut[k2 >> g.lut_shift];
  while (r <= g.nbe && s.thr[r] <= k2) ++r;
  return min(min(r, g.nb), g.nbe) - 1;          // r <= nbe whenever nbe < nb; the clamp only guards
}

// Per-pencil constants: signed (kx, ky), window of x and y, interlacing phase.
struct Pencil {
  int kp2;
  float cxy;
  float pr, pi;
};

template <bool INTER>
__device__ __forceinline__ Pencil pencil_of(const PowGeom& g, const Smem& s, int ix, int iy) {
  const int kx = signed_k(ix, g.N), ky = signed_k(iy, g.N);
  const int ax = kx < 0 ? -kx : kx, ay = ky < 0 ? -ky : ky;
  Pencil p;
  p.kp2 = kx * kx + ky * ky;
  // an interlaced pair is averaged, |(a + b)/2|^2: the 1/4 rides on the pencil constant
  p.cxy = s.c2[ax] * s.c2[ay] * (INTER ? 0.25f : 1.0f);
  p.pr = 1.0f;
  p.pi = 0.0f;
  if (INTER) {  // exp(i pi (kx+ky)/N) from the |k| table (conjugate for k < 0)
    float2 ex = s.eph[ax], ey = s.eph[ay];
    if (kx < 0) ex.y = -ex.y;
    if (ky < 0) ey.y = -ey.y;
    p.pr = ex.x * ey.x - ex.y * ey.y;
    p.pi = ex.x * ey.y + ex.y * ey.x;
  }
  return p;
}

// One mode: its moments (p, p mu^2, p mu^4) and its k2.  The window of z,
// the factor 1/4 of the interlaced average and the pencil's x,y window are
// folded into c2 / cxy.
template <int NV, bool INTER>
__device__ __forceinline__ void mode_moments(const Smem& s, const Pencil& pc, int kz, float2 a, float2 b,
                                             bool zero, float (&v)[NV], int& k2) {
  float re = a.x, im = a.y;
  if (INTER) {
    const float2 ez = s.eph[kz];
    const float qr = pc.pr * ez.x - pc.pi * ez.y;
    const float qi = pc.pr * ez.y + pc.pi * ez.x;
    re = a.x + (b.x * qr - b.y * qi);
    im = a.y + (b.x * qi + b.y * qr);
  }
  if (zero) re = im = 0.0f;
  k2 = pc.kp2 + kz * kz;
  const float p = (re * re + im * im) * (pc.cxy * s.c2[kz]);
  v[0] = p;
  if (NV > 1) {
    const float mu2 = k2 > 0 ? __fdividef((float)(kz * kz), (float)k2) : 0.0f;
    v[1] = p * mu2;
    if (NV > 2) v[2] = v[1] * mu2;
  }
}

// Warp-inclusive segmented scan (segments start at lanes whose head flag is set).
template <int NV>
__device__ __forceinline__ void seg_scan(float (&v)[NV], unsigned heads, int lane) {
  const int segstart = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const bool take = lane - d >= segstart;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const float t = __shfl_up_sync(0xffffffffu, v[q], d);
      if (take) v[q] += t;
    }
  }
}

template <int NV>
__device__ __forceinline__ void bin_add(float* wb, int nbe, int bin, const float (&v)[NV]) {
#pragma unroll
  for (int q = 0; q < NV; ++q) wb[q * nbe + bin] += v[q];
}

// Fold the warps' bins (in warp order, float-float) into the group's partial
// and clear them for the next group.
template <int NV>
__device__ __forceinline__ void cta_fold(const PowGeom& g, const Smem& s, int grp) {
  __syncthreads();
  float2* pf = g.part_ff + (long long)grp * NV * g.nbe;
  for (int b = threadIdx.x; b < g.nbe; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      ff acc{0.f, 0.f};
      for (int w = 0; w < g.warps; ++w) {
        float* p = &s.wbase[(w * NV + q) * g.nbe + b];
        acc = ff_add_f(acc, *p);
        *p = 0.0f;
      }
      pf[q * g.nbe + b] = make_float2(acc.hi, acc.lo);
    }
  }
  __syncthreads();
}

// Fold of one bin's group partials (float-float, [C][NV][nbe] layout) into
// doubles, by a whole block of FOLD_THREADS: thread t takes groups t, t +
// FOLD_THREADS, ...; each warp folds its lanes by a fixed xor tree; thread 0
// folds the warps in order.  Fixed order throughout: bitwise reproducible.
// Only thread 0 receives the results; every thread of the block must call.
constexpr int FOLD_THREADS = 256;

template <int MAXV>
__device__ __forceinline__ void fold_bin(const float2* __restrict__ part_ff, int C, int NV, int nbe, int b,
                                         double (&m)[MAXV]) {
  __shared__ ff s_w[MAXV][FOLD_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // a thread adds partials c = tid, tid + FOLD_THREADS, ... in that order; the loads of FU of them
  // (every moment) are issued before the adds
  constexpr int FU = 4;
  ff acc[MAXV];
#pragma unroll
  for (int q = 0; q < MAXV; ++q) acc[q] = ff{0.f, 0.f};
  for (int c0 = threadIdx.x; c0 < C; c0 += FU * FOLD_THREADS) {
    float2 v[MAXV][FU];
#pragma unroll
    for (int q = 0; q < MAXV; ++q)
#pragma unroll
      for (int u = 0; u < FU; ++u) {
        const int c = c0 + u * FOLD_THREADS;
        v[q][u] = (q < NV && c < C) ? part_ff[((long long)c * NV + q) * nbe + b] : make_float2(0.f, 0.f);
      }
#pragma unroll
    for (int q = 0; q < MAXV; ++q)
#pragma unroll
      for (int u = 0; u < FU; ++u)
        if (q < NV && c0 + u * FOLD_THREADS < C) acc[q] = ff_add(acc[q], ff{v[q][u].x, v[q][u].y});
  }
#pragma unroll
  for (int q = 0; q < MAXV; ++q) {
    if (q >= NV) break;
    for (int o = 16; o > 0; o >>= 1) {
      ff t{__shfl_xor_sync(0xffffffffu, acc[q].hi, o), __shfl_xor_sync(0xffffffffu, acc[q].lo, o)};
      acc[q] = ff_add(acc[q], t);
    }
    if (lane == 0) s_w[q][warp] = acc[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < NV; ++q) {
      ff t = s_w[q][0];
      for (int w = 1; w < FOLD_THREADS / 32; ++w) t = ff_add(t, s_w[q][w]);
      m[q] = (double)t.hi + (double)t.lo;
    }
  }
}

// One block per bin (FOLD_THREADS threads): fold the CTA partials into double
// moment totals and form the Legendre sums; copy the plan's geometry per bin.
__global__ void __launch_bounds__(FOLD_THREADS)
power_reduce_kernel(const float2* __restrict__ part_ff, int C, int NV, int nb, int nbe,
                    const long long* __restrict__ plan_nmodes, const double* __restrict__ plan_ksum,
                    double* sums_out, long long* nmodes_out, double* ksum_out) {
  pdl_wait();
  const int b = blockIdx.x;
  if (b >= nb) return;                         // uniform over the block
  double m[3] = {0.0, 0.0, 0.0};
  if (b < nbe) fold_bin<3>(part_ff, C, NV, nbe, b, m);
  if (threadIdx.x == 0) {
    sums_out[b * 3 + 0] = m[0];
    sums_out[b * 3 + 1] = NV > 1 ? 1.5 * m[1] - 0.5 * m[0] : 0.0;
    sums_out[b * 3 + 2] = NV > 2 ? (35.0 * m[2] - 30.0 * m[1] + 3.0 * m[0]) * 0.125 : 0.0;
    nmodes_out[b] = plan_nmodes[b];
    if (ksum_out) ksum_out[b] = plan_ksum[b];
  }
}

}  // namespace
}  // namespace gbp
