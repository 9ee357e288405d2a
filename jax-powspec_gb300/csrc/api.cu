// Host side of the C ABI: status strings, bin thresholds, bin plans and the
// cuFFT plan wrapper.
#include <cufft.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "gbp_bins.h"
#include "gbp_fft.h"
#include "gbp_internal.cuh"

namespace gbp {

static thread_local cudaError_t g_last_cuda = cudaSuccess;
static thread_local int g_last_cufft = 0;
void set_last_cuda_error(cudaError_t e) { g_last_cuda = e; }
void set_last_cufft_error(int code) { g_last_cufft = code; }

namespace {
struct C2RPlan {
  cufftHandle h;
  size_t ws;
  std::mutex use;      // held while a call sets the stream and work area and enqueues the transform
};

int c2r_entry(int N, int P, int batch, C2RPlan** out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, std::unique_ptr<C2RPlan>> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const auto key = std::make_tuple(dev, N, P, batch);
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it == cache.end()) {
    std::unique_ptr<C2RPlan> e(new (std::nothrow) C2RPlan());
    if (!e) return GBP_ERR_ALLOC;
    GBP_CUFFT_TRY(cufftCreate(&e->h));
    cufftSetAutoAllocation(e->h, 0);
    int n[3] = {N, N, N}, inembed[3] = {N, N, P}, onembed[3] = {N, N, N};
    size_t w = 0;
    const int mr =
        (int)cufftMakePlanMany(e->h, 3, n, inembed, 1, N * N * P, onembed, 1, N * N * N, CUFFT_C2R, batch, &w);
    if (mr != 0) {
      cufftDestroy(e->h);
      set_last_cufft_error(mr);
      return GBP_ERR_CUFFT;
    }
    e->ws = w;
    it = cache.emplace(key, std::move(e)).first;
  }
  *out = it->second.get();
  return GBP_OK;
}
}  // namespace

int c2r_plan(int N, int P, int batch, cufftHandle* out, size_t* ws) {
  C2RPlan* e = nullptr;
  const int r = c2r_entry(N, P, batch, &e);
  if (r) return r;
  *out = e->h;
  *ws = e->ws;
  return GBP_OK;
}

int c2r_exec(int N, int P, int batch, const float2* in, float* out, void* work, cudaStream_t st) {
  C2RPlan* e = nullptr;
  const int r = c2r_entry(N, P, batch, &e);
  if (r) return r;
  std::lock_guard<std::mutex> lock(e->use);
  GBP_CUFFT_TRY(cufftSetStream(e->h, st));
  GBP_CUFFT_TRY(cufftSetWorkArea(e->h, work));
  GBP_CUFFT_TRY(cufftExecC2R(e->h, reinterpret_cast<cufftComplex*>(const_cast<float2*>(in)), out));
  return GBP_OK;
}

namespace {
constexpr int LUT_MAX = 2048;

long long kmax2_of(int N) {
  const long long h = N / 2;
  return 3 * h * h;
}

// The reference's |k| of a mode: jnp.sqrt of the int32 sum, in float32
// (src/correlations.py:34).  sqrtf is correctly rounded (IEEE 754) on every
// host this library targets, as is the int -> float conversion.
inline float kf32(long long m) { return sqrtf((float)m); }
}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" const char* gbp_strerror(int st) {
  switch (st) {
    case GBP_OK: return "ok";
    case GBP_ERR_INVALID: return "invalid argument";
    case GBP_ERR_CUDA: {
      static thread_local char buf[256];
      snprintf(buf, sizeof(buf), "CUDA error: %s", cudaGetErrorString(g_last_cuda));
      return buf;
    }
    case GBP_ERR_CUFFT: {
      static thread_local char buf[64];
      snprintf(buf, sizeof(buf), "cuFFT error (cufftResult %d)", g_last_cufft);
      return buf;
    }
    case GBP_ERR_WORKSPACE: return "workspace too small";
    case GBP_ERR_UNSUPPORTED: return "unsupported configuration";
    case GBP_ERR_ALLOC: return "device allocation failed";
    default: return "unknown status";
  }
}

extern "C" int gbp_version(void) { return 100; }

extern "C" int gbp_bin_thresholds(const float* e, int ne, int N, int32_t* thr, int32_t* last_closed,
                                  int* n_reach) {
  if (!e || ne < 2 || N < 2 || N > 16384 || !thr || !last_closed) return GBP_ERR_INVALID;
  for (int i = 0; i < ne; ++i) {
    if (!isfinite(e[i])) return GBP_ERR_INVALID;
    if (i && e[i] < e[i - 1]) return GBP_ERR_INVALID;
  }
  const long long K = kmax2_of(N);
  for (int b = 0; b < ne; ++b) {
    // smallest m in [0, K+1] with sqrtf(m) >= e[b]   (K+1: no mode reaches it)
    long long lo = 0, hi = K + 1;
    while (lo < hi) {
      const long long mid = (lo + hi) / 2;
      if (kf32(mid) >= e[b]) hi = mid; else lo = mid + 1;
    }
    thr[b] = (int32_t)lo;
  }
  {  // largest m in [0, K] with sqrtf(m) <= e[last], or -1
    const float el = e[ne - 1];
    long long lo = -1, hi = K;
    while (lo < hi) {
      const long long mid = (lo + hi + 1) / 2;
      if (kf32(mid) <= el) lo = mid; else hi = mid - 1;
    }
    *last_closed = (int32_t)lo;
  }
  if (n_reach) {
    int r = 0;
    while (r < ne && thr[r] <= K) ++r;       // thresholds are non-decreasing
    const int nb = ne - 1;
    *n_reach = r < nb ? r : nb;
  }
  return GBP_OK;
}

extern "C" int gbp_bins_create(const float* e, int ne, int N, gbp_bins* out) {
  if (!out) return GBP_ERR_INVALID;
  *out = nullptr;
  std::vector<int32_t> thr((size_t)(ne > 0 ? ne : 1));
  int32_t last = 0;
  int reach = 0;
  int st = gbp_bin_thresholds(e, ne, N, thr.data(), &last, &reach);
  if (st) return st;
  gbp_bins_s* B = new (std::nothrow) gbp_bins_s();
  if (!B) return GBP_ERR_ALLOC;
  B->N = N;
  B->nb = ne - 1;
  B->nbe = reach > 0 ? reach : 1;
  B->last_closed = last;
  const long long K = kmax2_of(N);
  int sh = 0;
  while (((K >> sh) + 1) > LUT_MAX) ++sh;
  B->lut_shift = sh;
  B->lut_n = (int)((K >> sh) + 1);
  const int h = N / 2;

  std::vector<int32_t> h_thr(thr.begin(), thr.begin() + (B->nbe + 1));
  std::vector<int32_t> h_lut(B->lut_n);
  for (int j = 0; j < B->lut_n; ++j) {
    const long long key = (long long)j << sh;
    int r = 0;
    while (r <= B->nbe && h_thr[r] <= key) ++r;
    h_lut[j] = r;
  }
  // Mode counts and sum of |k| per bin depend only on the grid: count the
  // half-space cells per k^2 value once (pairs |kx|,|ky| with multiplicity),
  // then fold them into bins in increasing k^2 order (deterministic).
  std::vector<long long> per_k2((size_t)K + 1, 0);
  for (int ax = 0; ax <= h; ++ax) {
    const long long mx = (ax == 0 || (N % 2 == 0 && ax == h)) ? 1 : 2;
    for (int ay = 0; ay <= h; ++ay) {
      const long long my = (ay == 0 || (N % 2 == 0 && ay == h)) ? 1 : 2;
      const long long kp2 = (long long)ax * ax + (long long)ay * ay;
      for (int kz = 0; kz <= h; ++kz) per_k2[kp2 + (long long)kz * kz] += mx * my;
    }
  }
  std::vector<long long> h_nmodes((size_t)B->nb, 0);
  std::vector<double> h_ksum((size_t)B->nb, 0.0);
  {
    int r = 0;                                   // #thresholds <= k2, non-decreasing in k2
    for (long long k2 = 0; k2 <= K && k2 <= last; ++k2) {
      while (r < ne && thr[r] <= k2) ++r;
      const long long c = per_k2[k2];
      if (!c || r == 0) continue;
      const int b = (r < B->nb ? r : B->nb) - 1;
      h_nmodes[b] += c;
      h_ksum[b] += (double)c * sqrt((double)k2);
    }
  }
  std::vector<float> h_is2(h + 1);
  std::vector<float2> h_eph(h + 1);
  for (int k = 0; k <= h; ++k) {
    const double x = M_PI * (double)k / (double)N;
    const double s = k == 0 ? 1.0 : sin(x) / x;
    h_is2[k] = (float)(1.0 / (s * s));
    h_eph[k] = make_float2((float)cos(x), (float)sin(x));
  }
  const size_t o_thr = 0;
  const size_t o_lut = o_thr + align256(h_thr.size() * 4);
  const size_t o_is2 = o_lut + align256(h_lut.size() * 4);
  const size_t o_eph = o_is2 + align256(h_is2.size() * 4);
  const size_t o_nm = o_eph + align256(h_eph.size() * 8);
  const size_t o_ks = o_nm + align256(h_nmodes.size() * 8);
  const size_t total = o_ks + align256(h_ksum.size() * 8);
  cudaGetDevice(&B->device);
  char* blk = nullptr;
  if (cudaMalloc(&blk, total) != cudaSuccess) {
    delete B;
    return GBP_ERR_ALLOC;
  }
  B->d_block = blk;
  B->d_thr = reinterpret_cast<int*>(blk + o_thr);
  B->d_lut = reinterpret_cast<int*>(blk + o_lut);
  B->d_inv_sinc2 = reinterpret_cast<float*>(blk + o_is2);
  B->d_eph = reinterpret_cast<float2*>(blk + o_eph);
  B->d_nmodes = reinterpret_cast<long long*>(blk + o_nm);
  B->d_ksum = reinterpret_cast<double*>(blk + o_ks);
  cudaError_t ce = cudaSuccess;
  if (ce == cudaSuccess) ce = cudaMemcpy(B->d_nmodes, h_nmodes.data(), h_nmodes.size() * 8, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(B->d_ksum, h_ksum.data(), h_ksum.size() * 8, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(B->d_thr, h_thr.data(), h_thr.size() * 4, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(B->d_lut, h_lut.data(), h_lut.size() * 4, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(B->d_inv_sinc2, h_is2.data(), h_is2.size() * 4, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(B->d_eph, h_eph.data(), h_eph.size() * 8, cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    set_last_cuda_error(ce);
    cudaFree(blk);
    delete B;
    return GBP_ERR_CUDA;
  }
  *out = B;
  return GBP_OK;
}

extern "C" int gbp_bins_destroy(gbp_bins B) {
  if (!B) return GBP_ERR_INVALID;
  cudaFree(B->d_block);
  delete B;
  return GBP_OK;
}

extern "C" int gbp_bins_info(gbp_bins B, int* nb, int* reach, int32_t* last) {
  if (!B) return GBP_ERR_INVALID;
  if (nb) *nb = B->nb;
  if (reach) *reach = B->nbe;
  if (last) *last = B->last_closed;
  return GBP_OK;
}

// ---------------------------------------------------------------------------
// FFT plans.  Power-of-two meshes 64..1024 use the library's own three-pass
// transform (fft.cu), which writes z rows padded to N/2+8 complex; other
// sizes use a cuFFT 3-D R2C plan (batch = grids) with unpadded rows of
// N/2+1.  Setting GBP_FFT_BACKEND=cufft when the plan is created forces
// cuFFT (used to cross-check the two).
extern "C" int gbp_fft_plan_create(int n, int grids, gbp_fft_plan* out, size_t* ws_bytes) {
  if (!out || n < 2 || n > 4096 || grids < 1 || grids > 64) return GBP_ERR_INVALID;
  *out = nullptr;
  const char* env = getenv("GBP_FFT_BACKEND");
  const bool force_cufft = env && strcmp(env, "cufft") == 0;
  if (own_fft_supported(n) && !force_cufft) {
    float2* tw = nullptr;
    const int st = own_fft_twiddles(n, &tw);
    if (st) return st;
    gbp_fft_plan_s* p = new (std::nothrow) gbp_fft_plan_s{true, 0, tw, n, grids, own_fft_pitch(n), 0};
    if (!p) {
      cudaFree(tw);
      return GBP_ERR_ALLOC;
    }
    *out = p;
    if (ws_bytes) *ws_bytes = 0;
    return GBP_OK;
  }
  cufftHandle h;
  if (cufftCreate(&h) != CUFFT_SUCCESS) return GBP_ERR_CUFFT;
  if (cufftSetAutoAllocation(h, 0) != CUFFT_SUCCESS) {
    cufftDestroy(h);
    return GBP_ERR_CUFFT;
  }
  long long dims[3] = {n, n, n};
  size_t ws = 0;
  const long long idist = (long long)n * n * n, odist = (long long)n * n * (n / 2 + 1);
  if (cufftMakePlanMany64(h, 3, dims, nullptr, 1, idist, nullptr, 1, odist, CUFFT_R2C, grids, &ws) !=
      CUFFT_SUCCESS) {
    cufftDestroy(h);
    return GBP_ERR_CUFFT;
  }
  gbp_fft_plan_s* p = new (std::nothrow) gbp_fft_plan_s{false, h, nullptr, n, grids, n / 2 + 1, ws};
  if (!p) {
    cufftDestroy(h);
    return GBP_ERR_ALLOC;
  }
  *out = p;
  if (ws_bytes) *ws_bytes = ws;
  return GBP_OK;
}

extern "C" int gbp_fft_plan_pitch(gbp_fft_plan p, int* z_pitch) {
  if (!p || !z_pitch) return GBP_ERR_INVALID;
  *z_pitch = p->pitch;
  return GBP_OK;
}

extern "C" int gbp_fft_plan_destroy(gbp_fft_plan p) {
  if (!p) return GBP_ERR_INVALID;
  if (p->own) cudaFree(p->tw);
  else cufftDestroy(p->h);
  delete p;
  return GBP_OK;
}

extern "C" int gbp_fft_r2c(gbp_fft_plan p, const float* mesh, void* spec, void* ws, size_t ws_bytes,
                           gbp_stream_t stream) {
  if (!p || !mesh || !spec) return GBP_ERR_INVALID;
  if (p->own) {
    // float4 loads and stores: both buffers must be 16-byte aligned
    if (((reinterpret_cast<uintptr_t>(mesh) | reinterpret_cast<uintptr_t>(spec)) & 15u) != 0) return GBP_ERR_INVALID;
    return own_fft_r2c(p->n, p->grids, mesh, static_cast<float2*>(spec), p->tw,
                       reinterpret_cast<cudaStream_t>(stream));
  }
  if (p->ws > 0 && (!ws || ws_bytes < p->ws)) return GBP_ERR_WORKSPACE;
  if (cufftSetStream(p->h, reinterpret_cast<cudaStream_t>(stream)) != CUFFT_SUCCESS) return GBP_ERR_CUFFT;
  if (p->ws > 0 && cufftSetWorkArea(p->h, ws) != CUFFT_SUCCESS) return GBP_ERR_CUFFT;
  // Out-of-place R2C leaves its input untouched; cuFFT's prototype is non-const.
  GBP_TRACE("cufft_r2c", reinterpret_cast<cudaStream_t>(stream));
  if (cufftExecR2C(p->h, const_cast<cufftReal*>(mesh), static_cast<cufftComplex*>(spec)) != CUFFT_SUCCESS)
    return GBP_ERR_CUFFT;
  return GBP_OK;
}
