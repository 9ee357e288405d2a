// The x pass of the 3-D FFT fused with the binning.
//
// After the z and y passes (fft.cu) the spectrum buffer holds, for every
// grid, the transform over z and y; the remaining 1-D transforms run along
// x, whose rows lie N*P complex apart.  Instead of writing them back and
// reading them again for the binning, one CTA takes a work item = one ky row
// and a block of 8 adjacent kz columns, for all grids:
//
//   1. loads the item's N x 8 complex values of each grid (16-byte loads,
//      64 contiguous bytes per x row) into shared memory,
//   2. transforms the 8 (or 16, two grids) columns along x with radix-8
//      Stockham stages (fft_core.cuh); the last stage writes the result
//      column-major with an XOR swizzle, so the binning reads it without
//      bank conflicts,
//   3. bins the 8 x N modes: from 128^3 up the modes x and N - x of a
//      column (kx and -kx) share |k|, mu, the window and the bin, so they
//      are summed first and looked up once; a warp walks one column over
//      half of the |kx| range (pairs p = 0..N/4-1 or N/4..N/2-1; x = N/2
//      alone is added after the upper half), so bins are monotone along the
//      walk (at 64^3: single modes over half of the x axis).  A lane owns
//      consecutive pairs; runs of equal bin are summed in-lane, joined
//      across lanes by one warp segmented scan, and each run is added once
//      to the warp's float32 bins (distinct bins within a step: no atomics).
//
// The mode arithmetic (window deconvolution, interlacing average, |delta|^2,
// mu^2 and mu^4 moments, DC removal) and the bin lookup are those of
// power.cu.  CTA g walks work group g (items g, g + groups, ...); each
// group folds its warps' bins in a fixed order into
// a float-float partial, and power_reduce_kernel folds the partials into
// doubles, so results are bitwise reproducible on every device.  The full
// spectrum never returns to HBM: the pipeline reads 8 bytes per mode here
// instead of writing and reading them three more times.
#include <algorithm>

#include "fft_core.cuh"
#include "fft_pass.cuh"
#include "gbp_bins.h"
#include "gbp_fft.h"
#include "gbp_internal.cuh"
#include "power_core.cuh"

namespace gbp {
namespace {

constexpr int XB_THREADS = 512;
constexpr int XB_BINS = 8;                   // per-warp bin arrays; warps w and w + 8 share one
constexpr int XB_C = 8;                      // kz columns per work item
// The next item's HBM loads start before the barrier that ends the binning (512^3 and up)
template <int N>
constexpr bool XB_EARLY = N >= 512;

template <int N>
struct XLayout {
  static constexpr int TST = N + 1;          // complex per column (transposed layout); odd: no store conflicts
  static constexpr int M = N / 64;           // modes per lane in a half axis
  static constexpr int MS = M < 8 ? M : 8;   // modes per lane and warp step
  // N >= 128: the modes x and N - x of a column (kx and -kx: the same |k|, mu, window and bin) are
  // binned together, M2 such pairs per lane in half of the |kx| range
  static constexpr bool PAIRED = N >= 128;
  static constexpr int M2 = N / 128;
  static constexpr int MS2 = M2 < 8 ? M2 : 8;
  static_assert(!PAIRED || (MS2 > 0 && M2 % MS2 == 0), "whole warp steps of mode pairs");
  static __host__ __device__ constexpr size_t data_bytes(int G) {
    const size_t rows = (size_t)G * fft::ColBlock<N, 2>::SLAB, cols = (size_t)G * XB_C * TST;
    return ((rows > cols ? rows : cols) * 8 + 127) & ~size_t(127);
  }
  // per-x tables (swizzled like the columns): window c2(|kx|) and exp(i pi kx / N)
  static __host__ __device__ constexpr size_t xtab_bytes() { return (size_t)N * 12; }
};

// Swizzled position of x in a transposed column: lane l reads x = base + L l
// (L = the modes or mode pairs a lane takes per half axis), and so does it
// read the mirror N - x; with x's low bits XORed by bits 4.. of x, the 16
// lanes of a half-warp hit 16 distinct 8-byte slots in both reads, and the
// last FFT stage's stores stay conflict-free (checked by enumeration of
// every stage and mesh size).
template <int N>
__device__ __forceinline__ int xswz(int x) {
  constexpr int L = XLayout<N>::PAIRED ? XLayout<N>::M2 : XLayout<N>::M;
  if constexpr (L <= 1) return x;
  else return x ^ ((x >> 4) & (L - 1));
}

// One warp step: lane modes x0 + j (j < MS) of one column, bins monotone in
// lane order; sums runs and adds each once to the warp's bins.
template <int MS, int NV>
__device__ __forceinline__ void flush_runs(float (&P)[MS][NV], const int (&bin)[MS], int lane, float* wb, int nbe) {
  bool start[MS];
  start[0] = true;
#pragma unroll
  for (int j = 1; j < MS; ++j) {
    start[j] = bin[j] != bin[j - 1];
    if (!start[j]) {
#pragma unroll
      for (int q = 0; q < NV; ++q) P[j][q] += P[j - 1][q];
    }
  }
  bool multi = false;
#pragma unroll
  for (int j = 1; j < MS; ++j) multi = multi || start[j];
  const int prev_last = __shfl_up_sync(0xffffffffu, bin[MS - 1], 1);
  const bool cont = lane > 0 && bin[0] == prev_last;       // the lane's first run continues the previous lane's last
  const unsigned heads = __ballot_sync(0xffffffffu, multi || !cont);
  float T[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) T[q] = P[MS - 1][q];
  seg_scan<NV>(T, heads, lane);
  float Tprev[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) Tprev[q] = __shfl_up_sync(0xffffffffu, T[q], 1);
  const bool next_cont = __shfl_down_sync(0xffffffffu, cont, 1) && lane < 31;
  // runs that end inside the lane: the first of them absorbs the carry from earlier lanes
  bool carry = cont && multi;
#pragma unroll
  for (int j = 0; j < MS - 1; ++j) {
    if (start[j + 1]) {
      if (carry) {
#pragma unroll
        for (int q = 0; q < NV; ++q) P[j][q] += Tprev[q];
        carry = false;
      }
      if (bin[j] >= 0) bin_add<NV>(wb, nbe, bin[j], P[j]);
    }
  }
  if (!next_cont && bin[MS - 1] >= 0) bin_add<NV>(wb, nbe, bin[MS - 1], T);
  __syncwarp();
}

// Moments and bins of one warp step (lane modes x0 .. x0 + MS - 1 of column c).
template <int N, int NV, bool INTER, int MS>
__device__ __forceinline__ void xbin_modes(const PowGeom& g, const Smem& t, const float* c2x, const float2* ephx,
                                           const float2* a_col, const float2* b_col, int x0, int kyz2, float cyz,
                                           float fz2, float2 eyz, float (&P)[MS][NV], int (&bin)[MS]) {
#pragma unroll
  for (int j = 0; j < MS; ++j) {
    const int x = x0 + j;
    const int kx = signed_k(x, N);
    const int sx = xswz<N>(x);
    const float2 a = a_col[sx];
    float re = a.x, im = a.y;
    if (INTER) {
      const float2 b = b_col[sx];
      const float2 ex = ephx[sx];
      const float qr = ex.x * eyz.x - ex.y * eyz.y;
      const float qi = ex.x * eyz.y + ex.y * eyz.x;
      re = a.x + (b.x * qr - b.y * qi);
      im = a.y + (b.x * qi + b.y * qr);
    }
    const int k2 = kx * kx + kyz2;
    if (g.zero_dc && k2 == 0) re = im = 0.0f;
    const float p = (re * re + im * im) * (cyz * c2x[sx]);
    P[j][0] = p;
    if (NV > 1) {
      const float mu2 = k2 > 0 ? __fdividef(fz2, (float)k2) : 0.0f;
      P[j][1] = p * mu2;
      if (NV > 2) P[j][2] = P[j][1] * mu2;
    }
    bin[j] = bin_of(g, t, k2);
  }
}

// Moments and bins of one warp step of mode pairs: lane pairs p0 .. p0 + MS - 1
// of column (a_col, b_col), pair p = the columns x = p and x = N - p
// (kx = p and -p), whose |k|, mu, window and bin agree; p = 0 is x = 0 alone.
template <int N, int NV, bool INTER, int MS>
__device__ __forceinline__ void xbin_pairs(const PowGeom& g, const Smem& t, const float* c2x, const float2* ephx,
                                           const float2* a_col, const float2* b_col, int p0, int kyz2, float cyz,
                                           float fz2, float2 eyz, float (&P)[MS][NV], int (&bin)[MS]) {
#pragma unroll
  for (int j = 0; j < MS; ++j) {
    const int p = p0 + j;
    const int sp = xswz<N>(p), sm = xswz<N>((N - p) & (N - 1));
    const float2 a = a_col[sp], am = a_col[sm];
    float re = a.x, im = a.y, rem = am.x, imm = am.y;
    if (INTER) {
      const float2 b = b_col[sp], bm = b_col[sm];
      const float2 ex = ephx[sp];                            // exp(i pi p / N); kx = -p takes its conjugate
      const float ar = ex.x * eyz.x, ai = ex.x * eyz.y, br = ex.y * eyz.y, bi = ex.y * eyz.x;
      const float qr = ar - br, qi = ai + bi;                // exp(i pi p / N) eyz
      const float mr = ar + br, mi = ai - bi;                // exp(-i pi p / N) eyz
      re = a.x + (b.x * qr - b.y * qi);
      im = a.y + (b.x * qi + b.y * qr);
      rem = am.x + (bm.x * mr - bm.y * mi);
      imm = am.y + (bm.x * mi + bm.y * mr);
    }
    const int k2 = p * p + kyz2;
    float pw = re * re + im * im;
    if (g.zero_dc && k2 == 0) pw = 0.0f;
    if (p > 0) pw += rem * rem + imm * imm;
    const float v = pw * (cyz * c2x[sp]);
    P[j][0] = v;
    if (NV > 1) {
      const float mu2 = k2 > 0 ? __fdividef(fz2, (float)k2) : 0.0f;
      P[j][1] = v * mu2;
      if (NV > 2) P[j][2] = P[j][1] * mu2;
    }
    bin[j] = bin_of(g, t, k2);
  }
}

// The column x = N/2 (kx = N/2, its own mirror) of one column, added to the
// warp's bins by one lane.  Out of line: it runs once per column and only
// for bins beyond k_Nyq, and inlined it would cost the binning registers.
template <int N, int NV, bool INTER>
__device__ __noinline__ void add_nyquist_x(const PowGeom& g, const Smem& t, const float* c2x, const float2* ephx,
                                           const float2* a_col, const float2* b_col, int kyz2, float cyz, float fz2,
                                           float2 eyz, float* wb) {
  float P[1][NV];
  int bin[1];
  xbin_modes<N, NV, INTER, 1>(g, t, c2x, ephx, a_col, b_col, N / 2, kyz2, cyz, fz2, eyz, P, bin);
  if (bin[0] >= 0) bin_add<NV>(wb, g.nbe, bin[0], P[0]);
}

// Bin the 8 columns of one item (transposed layout in s).  Warp w takes
// column w / 2 and half w % 2 of the x axis (of the |kx| range, in mode
// pairs x, N - x from 128^3 up); warps w and w + 8 share bin
// array w % 8 and flush in two phases separated by barriers.  No barrier
// follows the last step: the caller's next barrier (the next item's first
// FFT stage, or the fold) orders the last flushes and reads of s.
template <int N, int NV, bool INTER>
__device__ __forceinline__ void xbin_item(const PowGeom& g, const Smem& t, const float* c2x, const float2* ephx,
                                          const float2* s, int warp, int lane, int y, int kb) {
  constexpr int H = N / 2, M = XLayout<N>::M, MS = XLayout<N>::MS, TST = XLayout<N>::TST;
  const int c = warp >> 1, h = warp & 1;
  const int kz = kb * XB_C + c;
  const bool active = kz <= H;                              // else row padding
  const int kzc = active ? kz : 0;
  const int ky = signed_k(y, N);
  const int ay = ky < 0 ? -ky : ky;
  float2 eyz = make_float2(1.f, 0.f);
  if (INTER) {
    float2 ey = t.eph[ay];
    if (ky < 0) ey.y = -ey.y;
    const float2 ez = t.eph[kzc];
    eyz = make_float2(ey.x * ez.x - ey.y * ez.y, ey.x * ez.y + ey.y * ez.x);
  }
  // |(a + b)/2|^2: the 1/4 of the interlaced average rides on the constant
  const float cyz = t.c2[ay] * t.c2[kzc] * (INTER ? 0.25f : 1.0f);
  const int kyz2 = ky * ky + kzc * kzc;
  const float fz2 = (float)(kzc * kzc);
  const float2* a_col = s + c * TST;
  const float2* b_col = s + (XB_C + c) * TST;
  float* wb = t.wbase + (warp & (XB_BINS - 1)) * NV * g.nbe;
  if constexpr (XLayout<N>::PAIRED) {
    // warp half h walks pairs h N/4 .. (h+1) N/4 - 1 (|kx| ascending); the column x = N/2, its own
    // mirror, is added by lane 0 of the upper half after its last flush
    constexpr int M2 = XLayout<N>::M2, MS2 = XLayout<N>::MS2;
#pragma unroll 1
    for (int s0 = 0; s0 < M2; s0 += MS2) {
      float P[MS2][NV];
      int bin[MS2];
      if (active)
        xbin_pairs<N, NV, INTER, MS2>(g, t, c2x, ephx, a_col, b_col, h * (H / 2) + lane * M2 + s0, kyz2, cyz, fz2,
                                      eyz, P, bin);
      auto flush = [&]() {
        flush_runs<MS2, NV>(P, bin, lane, wb, g.nbe);
        // |kx| = N/2 reaches a bin only when the last edge lies beyond k_Nyq
        if (h == 1 && s0 + MS2 >= M2 && (H * H + kyz2 <= g.tu)) {
          if (lane == 0) add_nyquist_x<N, NV, INTER>(g, t, c2x, ephx, a_col, b_col, kyz2, cyz, fz2, eyz, wb);
          __syncwarp();
        }
      };
      if (warp < XB_BINS && active) flush();
      __syncthreads();
      if (warp >= XB_BINS && active) flush();
      if (s0 + MS2 < M2) __syncthreads();   // after the last step, the next item's (or the fold's) barrier follows
    }
  } else {
#pragma unroll 1
    for (int s0 = 0; s0 < M; s0 += MS) {
      float P[MS][NV];
      int bin[MS];
      if (active) {
        xbin_modes<N, NV, INTER, MS>(g, t, c2x, ephx, a_col, b_col, h * H + lane * M + s0, kyz2, cyz, fz2, eyz, P,
                                     bin);
      }
      if (warp < XB_BINS && active) flush_runs<MS, NV>(P, bin, lane, wb, g.nbe);
      __syncthreads();
      if (warp >= XB_BINS && active) flush_runs<MS, NV>(P, bin, lane, wb, g.nbe);
      if (s0 + MS < M) __syncthreads();     // after the last step, the next item's (or the fold's) barrier follows
    }
  }
}

template <int N, int NV, bool INTER>
__global__ void __launch_bounds__(XB_THREADS, N >= 1024 ? 1 : 2)
xbin_kernel(PowGeom g) {
  pdl_wait();
  constexpr int G = INTER ? 2 : 1;
  constexpr int P = N / 2 + 8;                              // z row pitch of the own transform
  constexpr int TST = XLayout<N>::TST;
  extern __shared__ __align__(16) unsigned char smem[];
  float2* s = reinterpret_cast<float2*>(smem);
  float2* ephx = reinterpret_cast<float2*>(smem + XLayout<N>::data_bytes(G));
  float* c2x = reinterpret_cast<float*>(ephx + N);
  const Smem t = load_tables<NV, INTER>(g, smem + XLayout<N>::data_bytes(G) + XLayout<N>::xtab_bytes());
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int x = tid; x < N; x += XB_THREADS) {               // per-x tables (load_tables ended with a barrier)
    const int kx = signed_k(x, N), ax = kx < 0 ? -kx : kx;
    float2 e = INTER ? t.eph[ax] : make_float2(1.f, 0.f);
    if (kx < 0) e.y = -e.y;
    ephx[xswz<N>(x)] = e;
    c2x[xswz<N>(x)] = t.c2[ax];
  }
  __syncthreads();
  const long long gstride = (long long)N * N * P;
  for (int grp = blockIdx.x; grp < g.groups; grp += gridDim.x) {
    for (int it = grp; it < g.items; it += g.groups) {
      const int y = it / g.nkb, kb = it - (it / g.nkb) * g.nkb;
      const float2* src = g.s0 + ((long long)y * P + kb * XB_C);
      auto gin = [src, gstride](int x, int cp) {   // columns 2cp, 2cp+1 (slab = grid cp / 4)
        return __ldcs(reinterpret_cast<const float4*>(src + (cp >> 2) * gstride + (long long)x * N * P) + (cp & 3));
      };
      auto tout = [s](int x, int cp, float4 v) {
        s[(2 * cp) * TST + xswz<N>(x)] = fft::lo2(v);
        s[(2 * cp + 1) * TST + xswz<N>(x)] = fft::hi2(v);
      };
      // from 512^3 up the first stage loads the item from HBM while the previous item's last warps
      // still bin it, and waits for them before it writes the shared buffer (smaller meshes: the
      // registers the early loads hold would spill; they end the binning with a barrier instead)
      fft::col_fft<N, G, XB_THREADS, true, decltype(gin), decltype(tout), XB_EARLY<N>>(s, gin, tout, g.tw, tid);
      xbin_item<N, NV, INTER>(g, t, c2x, ephx, s, warp, lane, y, kb);
      if constexpr (!XB_EARLY<N>) __syncthreads();
    }
    cta_fold<NV>(g, t, grp);
  }
}

// Work groups: a pure function of N, so the summation order is the same on
// every device.
int xbin_groups(int items) { return std::min(items, 1216); }

struct XbLayout {
  int NV, items, nkb, groups;
  size_t smem, ws;
};

int xbin_layout(const gbp_bins_s* B, int G, int ells, XbLayout& L) {
  const int N = B->N;
  L.NV = (ells & GBP_ELL4) ? 3 : ((ells & GBP_ELL2) ? 2 : 1);
  L.nkb = (N / 2 + 8) / XB_C;
  L.items = N * L.nkb;
  L.groups = xbin_groups(L.items);
  size_t data = 0;
  switch (N) {
    case 64: data = XLayout<64>::data_bytes(G); break;
    case 128: data = XLayout<128>::data_bytes(G); break;
    case 256: data = XLayout<256>::data_bytes(G); break;
    case 512: data = XLayout<512>::data_bytes(G); break;
    case 1024: data = XLayout<1024>::data_bytes(G); break;
    default: return GBP_ERR_UNSUPPORTED;
  }
  L.smem = data + (size_t)N * 12 + smem_plan(N, B->nbe, B->lut_n, XB_BINS, L.NV).total;
  if (L.smem > 227 * 1024) return GBP_ERR_UNSUPPORTED;
  L.ws = align256((size_t)L.groups * L.NV * B->nbe * sizeof(float2));
  return GBP_OK;
}

template <int N, int NV, bool INTER>
int launch_xbin(const PowGeom& g, size_t smem, cudaStream_t st) {
  auto k = xbin_kernel<N, NV, INTER>;
  GBP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // one CTA per work group (not a persistent grid): CTAs end every ~14 items, so the block
  // scheduler can start a higher-priority stream's kernels (small serving requests) in between;
  // as fast as the persistent grid at 512^3 (0.775 against 0.781 ms)
  const int grid = std::max(1, g.groups);
  GBP_TRACE("fft_x_bins", st);
  GBP_CUDA_TRY(launch_pdl(k, dim3(grid), dim3(XB_THREADS), smem, st, g));
  return GBP_OK;
}

template <int N>
int dispatch_xbin(const PowGeom& g, int NV, bool inter, size_t smem, cudaStream_t st) {
  if (inter) {
    if (NV == 3) return launch_xbin<N, 3, true>(g, smem, st);
    if (NV == 2) return launch_xbin<N, 2, true>(g, smem, st);
    return launch_xbin<N, 1, true>(g, smem, st);
  }
  if (NV == 3) return launch_xbin<N, 3, false>(g, smem, st);
  if (NV == 2) return launch_xbin<N, 2, false>(g, smem, st);
  return launch_xbin<N, 1, false>(g, smem, st);
}

}  // namespace
}  // namespace gbp

namespace gbp {

int xbin_power_workspace(gbp_fft_plan plan, gbp_bins B, int ells, size_t* bytes) {
  if (!plan || !B || !bytes || plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own || (plan->grids != 1 && plan->grids != 2)) return GBP_ERR_UNSUPPORTED;
  XbLayout L;
  const int st = xbin_layout(B, plan->grids, ells, L);
  if (st) return st;
  *bytes = L.ws;
  return GBP_OK;
}

int xbin_power(gbp_fft_plan plan, float2* spec, gbp_bins B, int mas_order, int ells, const double* mass,
               double* sums_out, long long* nmodes_out, double* ksum_out, void* workspace, size_t ws_bytes,
               cudaStream_t st) {
  if (!plan || !spec || !B || !sums_out || !nmodes_out) return GBP_ERR_INVALID;
  if (plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own || (plan->grids != 1 && plan->grids != 2)) return GBP_ERR_UNSUPPORTED;
  if (mas_order < 0 || mas_order > 8) return GBP_ERR_INVALID;
  if ((ells & (GBP_ELL0 | GBP_ELL2 | GBP_ELL4)) == 0 || (ells & ~15)) return GBP_ERR_INVALID;
  if ((ells & GBP_KSUM) && !ksum_out) return GBP_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(spec) & 15u) != 0) return GBP_ERR_INVALID;
  XbLayout L;
  int r = xbin_layout(B, plan->grids, ells, L);
  if (r) return r;
  if (!workspace || ws_bytes < L.ws) return GBP_ERR_WORKSPACE;
  const int N = B->N, G = plan->grids;
  PowGeom g{};
  g.s0 = spec;
  g.s1 = G == 2 ? spec + (long long)N * N * plan->pitch : nullptr;
  g.N = N;
  g.Lz = N / 2 + 1;
  g.Lzs = plan->pitch;
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
  g.part_ff = static_cast<float2*>(workspace);
  g.warps = XB_BINS;
  g.groups = L.groups;
  g.tw = plan->tw;
  g.items = L.items;
  g.nkb = L.nkb;
  switch (N) {
    case 64: r = dispatch_xbin<64>(g, L.NV, G == 2, L.smem, st); break;
    case 128: r = dispatch_xbin<128>(g, L.NV, G == 2, L.smem, st); break;
    case 256: r = dispatch_xbin<256>(g, L.NV, G == 2, L.smem, st); break;
    case 512: r = dispatch_xbin<512>(g, L.NV, G == 2, L.smem, st); break;
    case 1024: r = dispatch_xbin<1024>(g, L.NV, G == 2, L.smem, st); break;
    default: r = GBP_ERR_UNSUPPORTED;
  }
  if (r) return r;
  GBP_TRACE("power_reduce", st);
  GBP_CUDA_TRY(launch_pdl(power_reduce_kernel, dim3(B->nb), dim3(FOLD_THREADS), 0, st,
                          static_cast<const float2*>(g.part_ff), L.groups, L.NV, B->nb, B->nbe,
                          static_cast<const long long*>(B->d_nmodes), static_cast<const double*>(B->d_ksum), sums_out,
                          nmodes_out, (ells & GBP_KSUM) ? ksum_out : nullptr));
  return GBP_OK;
}

}  // namespace gbp

using namespace gbp;

extern "C" int gbp_fft_power_workspace_size(gbp_fft_plan plan, gbp_bins B, int ells, size_t* bytes) {
  return xbin_power_workspace(plan, B, ells, bytes);
}

extern "C" int gbp_fft_power(gbp_fft_plan plan, const float* mesh, void* spectrum, gbp_bins B, int mas_order,
                             int ells, const double* mass, double* sums_out, long long* nmodes_out, double* ksum_out,
                             void* workspace, size_t ws_bytes, gbp_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!plan || !mesh || !spectrum || !B || !sums_out || !nmodes_out) return GBP_ERR_INVALID;
  if (plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own || (plan->grids != 1 && plan->grids != 2)) return GBP_ERR_UNSUPPORTED;
  if (((reinterpret_cast<uintptr_t>(mesh) | reinterpret_cast<uintptr_t>(spectrum)) & 15u) != 0) return GBP_ERR_INVALID;
  size_t need = 0;
  int r = xbin_power_workspace(plan, B, ells, &need);
  if (r) return r;
  if (!workspace || ws_bytes < need) return GBP_ERR_WORKSPACE;
  float2* spec = static_cast<float2*>(spectrum);
  r = own_fft_zy(B->N, plan->grids, mesh, spec, plan->tw, st);
  if (r) return r;
  return xbin_power(plan, spec, B, mas_order, ells, mass, sums_out, nmodes_out, ksum_out, workspace, ws_bytes, st);
}
