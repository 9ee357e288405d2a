// Lognormal mock catalogues generated on the device.
//
// The benchmark workloads are lognormal catalogues (the reference builds its
// mocks this way: tests/create_lognormal.py:42-55 with src/gauss_field.py
// and src/populate_field.py).  Generating them on the host takes seconds per
// million particles, so batched and served throughput runs make them here:
//
//   1. white noise eps on a grid^3 lattice (Philox4x32-10 counter-based
//      generator, Box-Muller),
//   2. eps_k = FFT(eps), g_k = eps_k sqrt(grid^3 P_G(k) / V), g_0 = 0,
//      g = IFFT(g_k) / grid^3 (cuFFT R2C / C2R), with
//      P_G(k) = A k exp(-(k/k_cut)^2) and A set on the host so that the
//      lattice variance sum_k P_G / V is 1,
//   3. rho = exp(g - 1/2) = 1 + delta_LN,
//   4. exactly n particles drawn independently with probability
//      proportional to rho (inclusive prefix sum in double + binary search,
//      i.e. a multinomial sample), placed uniformly inside their cell,
//   5. z shifted by N(0, sigma_v) and wrapped into [0, L); float32
//      positions kept below L.
//
// Everything is a pure function of (seed, grid, box, k_cut, sigma_v, n):
// stream s of the generator is (seed, purpose) and counter i is the cell or
// particle index, so no generator state is stored.
#include <cufft.h>
#include <math.h>

#include <cub/device/device_scan.cuh>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gbp_internal.cuh"

namespace gbp {
namespace {

// Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies with
// the round keys bumped by the Weyl constants.
struct U4 { unsigned a, b, c, d; };

__host__ __device__ inline void mulhilo(unsigned m, unsigned x, unsigned& hi, unsigned& lo) {
  const unsigned long long p = (unsigned long long)m * x;
  hi = (unsigned)(p >> 32);
  lo = (unsigned)p;
}

__host__ __device__ inline U4 philox4x32_10(U4 ctr, unsigned k0, unsigned k1) {
  const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const unsigned W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    unsigned hi0, lo0, hi1, lo1;
    mulhilo(M0, ctr.a, hi0, lo0);
    mulhilo(M1, ctr.c, hi1, lo1);
    ctr = U4{hi1 ^ ctr.b ^ k0, lo1, hi0 ^ ctr.d ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// (0, 1] from 24 random bits
__device__ __forceinline__ float u01(unsigned x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }
// [0, 1) from 53 random bits
__device__ __forceinline__ double u01d(unsigned hi, unsigned lo) {
  return (double)(((unsigned long long)hi << 21) ^ (unsigned long long)(lo >> 11)) * (1.0 / 9007199254740992.0);
}

constexpr unsigned PURPOSE_NOISE = 1u, PURPOSE_SAMPLE = 2u;

__global__ void noise_kernel(float* eps, long long cells, unsigned long long seed) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // one Philox call -> 4 normals
  if (4 * i >= cells) return;
  const U4 r = philox4x32_10(U4{(unsigned)i, (unsigned)(i >> 32), PURPOSE_NOISE, 0u}, (unsigned)seed,
                             (unsigned)(seed >> 32));
  float s0, c0, s1, c1;
  const float r0 = sqrtf(-2.0f * logf(u01(r.a))), r1 = sqrtf(-2.0f * logf(u01(r.c)));
  sincospif(2.0f * u01(r.b), &s0, &c0);
  sincospif(2.0f * u01(r.d), &s1, &c1);
  const float v[4] = {r0 * c0, r0 * s0, r1 * c1, r1 * s1};
  for (int k = 0; k < 4; ++k)
    if (4 * i + k < cells) eps[4 * i + k] = v[k];
}

// g_k = eps_k sqrt(grid^3 P(k) / V) / grid^3 (the C2R that follows is
// unnormalised); the k = 0 mode is removed.
__global__ void shape_kernel(float2* gk, int grid, double kf, double amp_over_v, double k_cut) {
  const int h = grid / 2 + 1;
  const long long total = (long long)grid * grid * h;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int kz = (int)(i % h);
  const int iy = (int)((i / h) % grid), ix = (int)(i / ((long long)h * grid));
  const int kx = signed_k(ix, grid), ky = signed_k(iy, grid);
  const double k = kf * sqrt((double)kx * kx + (double)ky * ky + (double)kz * kz);
  const double g3 = (double)grid * grid * grid;
  const double pk_over_v = amp_over_v * k * exp(-(k / k_cut) * (k / k_cut));
  const float f = i == 0 ? 0.0f : (float)sqrt(pk_over_v / g3);
  const float2 e = gk[i];
  gk[i] = make_float2(e.x * f, e.y * f);
}

// rho = exp(g - 1/2), in double for the prefix sum
__global__ void density_kernel(const float* g, double* rho, long long cells) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells) rho[i] = exp((double)g[i] - 0.5);
}

// Particle i: cell by inverse CDF (cdf = inclusive prefix sum of rho),
// uniform position inside it, Gaussian velocity shift along z, periodic wrap.
__global__ void sample_kernel(const double* __restrict__ cdf, long long cells, int grid, float box,
                              float sigma_v, long long n, unsigned long long seed, float* x, float* y, float* z) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double total = cdf[cells - 1];
  const U4 r = philox4x32_10(U4{(unsigned)i, (unsigned)(i >> 32), PURPOSE_SAMPLE, 0u}, (unsigned)seed,
                             (unsigned)(seed >> 32));
  const U4 r2 = philox4x32_10(U4{(unsigned)i, (unsigned)(i >> 32), PURPOSE_SAMPLE, 1u}, (unsigned)seed,
                              (unsigned)(seed >> 32));
  const double u = u01d(r.a, r.b) * total;
  long long lo = 0, hi = cells - 1;          // first cell with cdf > u
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (cdf[mid] > u) hi = mid;
    else lo = mid + 1;
  }
  const long long c = lo;
  const int cz = (int)(c % grid), cy = (int)((c / grid) % grid), cx = (int)(c / ((long long)grid * grid));
  const float cell = box / (float)grid;
  float px = ((float)cx + u01(r.c) - 0.5f / 16777216.0f) * cell;
  float py = ((float)cy + u01(r.d) - 0.5f / 16777216.0f) * cell;
  float pz = ((float)cz + u01(r2.a) - 0.5f / 16777216.0f) * cell;
  if (sigma_v > 0.0f) {
    float s, co;
    sincospif(2.0f * u01(r2.c), &s, &co);
    pz += sigma_v * sqrtf(-2.0f * logf(u01(r2.b))) * co;
  }
  const float top = nextafterf(box, 0.0f);
  px = fminf(fmodf(fmodf(px, box) + box, box), top);
  py = fminf(fmodf(fmodf(py, box) + box, box), top);
  pz = fminf(fmodf(fmodf(pz, box) + box, box), top);
  x[i] = px;
  y[i] = py;
  z[i] = pz;
}

// Amplitude A / V that makes the lattice variance sum_k P_G(k) / V equal 1
// (each interior kz mode of the half spectrum counts twice).  Cached per
// (grid, box, k_cut): a batch of mocks evaluates it once.
double lognormal_amp_sum(int grid, double box, double k_cut);

double lognormal_amp_over_v(int grid, double box, double k_cut) {
  static std::mutex mu;
  static std::map<std::tuple<int, double, double>, double> cache;
  const auto key = std::make_tuple(grid, box, k_cut);
  {
    std::lock_guard<std::mutex> lock(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const double v = lognormal_amp_sum(grid, box, k_cut);
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = v;
  return v;
}

double lognormal_amp_sum(int grid, double box, double k_cut) {
  const double kf = 2.0 * M_PI / box;
  const int h = grid / 2 + 1;
  std::vector<double> k2(grid);
  for (int i = 0; i < grid; ++i) {
    const int s = signed_k(i, grid);
    k2[i] = (double)s * s;
  }
  double sum = 0.0;
  for (int ix = 0; ix < grid; ++ix)
    for (int iy = 0; iy < grid; ++iy)
      for (int kz = 0; kz < h; ++kz) {
        const double k = kf * sqrt(k2[ix] + k2[iy] + (double)kz * kz);
        const double w = (kz == 0 || (grid % 2 == 0 && kz == grid / 2)) ? 1.0 : 2.0;
        sum += w * k * exp(-(k / k_cut) * (k / k_cut));
      }
  return 1.0 / sum;     // A / V
}

struct LnLayout {
  size_t eps, spec, cdf, scan, fft, total;
};

int lognormal_layout(int grid, LnLayout& L, cufftHandle* r2c, cufftHandle* c2r) {
  const long long cells = (long long)grid * grid * grid;
  const long long modes = (long long)grid * grid * (grid / 2 + 1);
  L.eps = align256((size_t)cells * 4);
  L.spec = align256((size_t)modes * 8);
  L.cdf = align256((size_t)cells * 8);
  L.scan = 0;
  cub::DeviceScan::InclusiveSum(nullptr, L.scan, (double*)nullptr, (double*)nullptr, (int64_t)cells);
  L.scan = align256(L.scan);
  size_t w1 = 0, w2 = 0;
  if (cufftCreate(r2c) != CUFFT_SUCCESS) return GBP_ERR_CUFFT;
  if (cufftCreate(c2r) != CUFFT_SUCCESS) { cufftDestroy(*r2c); return GBP_ERR_CUFFT; }
  cufftSetAutoAllocation(*r2c, 0);
  cufftSetAutoAllocation(*c2r, 0);
  if (cufftMakePlan3d(*r2c, grid, grid, grid, CUFFT_R2C, &w1) != CUFFT_SUCCESS ||
      cufftMakePlan3d(*c2r, grid, grid, grid, CUFFT_C2R, &w2) != CUFFT_SUCCESS) {
    cufftDestroy(*r2c);
    cufftDestroy(*c2r);
    return GBP_ERR_CUFFT;
  }
  L.fft = align256(w1 > w2 ? w1 : w2);
  L.total = L.eps + L.spec + L.cdf + L.scan + L.fft;
  return GBP_OK;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_philox4x32_10(const unsigned* ctr, const unsigned* key, unsigned* out) {
  if (!ctr || !key || !out) return GBP_ERR_INVALID;
  const U4 r = philox4x32_10(U4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
  out[0] = r.a; out[1] = r.b; out[2] = r.c; out[3] = r.d;
  return GBP_OK;
}

extern "C" int gbp_lognormal_workspace_size(int grid, size_t* bytes) {
  if (!bytes || grid < 4 || grid > 1024 || (grid & 1)) return GBP_ERR_INVALID;
  LnLayout L;
  cufftHandle a, b;
  const int st = lognormal_layout(grid, L, &a, &b);
  if (st) return st;
  cufftDestroy(a);
  cufftDestroy(b);
  *bytes = L.total;
  return GBP_OK;
}

namespace gbp {
namespace {

// rho = exp(g - 1/2) as float32, for gbp_lognormal_field
__global__ void rho_out_kernel(const float* g, float* rho, long long cells) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells) rho[i] = (float)exp((double)g[i] - 0.5);
}

// Steps 1-5 (n = 0: steps 1-3 and the prefix sum only).  g_out / rho_out,
// when given, receive the Gaussian field g and rho = 1 + delta_LN.
int lognormal_run(int grid, double box, double k_cut, double sigma_v, int64_t n, unsigned long long seed, float* x,
                  float* y, float* z, float* g_out, float* rho_out, void* workspace, size_t ws_bytes,
                  cudaStream_t st) {
  if (grid < 4 || grid > 1024 || (grid & 1) || !(box > 0.0) || !(k_cut > 0.0) || sigma_v < 0.0 || n < 0)
    return GBP_ERR_INVALID;
  if (n > 0 && (!x || !y || !z)) return GBP_ERR_INVALID;
  LnLayout L;
  cufftHandle r2c, c2r;
  int r = lognormal_layout(grid, L, &r2c, &c2r);
  if (r) return r;
  auto fail = [&](int code) {
    cufftDestroy(r2c);
    cufftDestroy(c2r);
    return code;
  };
  if (!workspace || ws_bytes < L.total) return fail(GBP_ERR_WORKSPACE);
  Carver cv(workspace);
  float* eps = cv.take<float>(L.eps / 4);
  float2* spec = cv.take<float2>(L.spec / 8);
  double* cdf = cv.take<double>(L.cdf / 8);
  void* scan = cv.take<char>(L.scan);
  void* fws = cv.take<char>(L.fft);
  const long long cells = (long long)grid * grid * grid;
  const long long modes = (long long)grid * grid * (grid / 2 + 1);
  {
    GBP_TRACE("lognormal_noise", st);
    noise_kernel<<<(unsigned)((cells / 4 + 256) / 256), 256, 0, st>>>(eps, cells, seed);
    if (cudaGetLastError() != cudaSuccess) return fail(GBP_ERR_CUDA);
  }
  if (cufftSetStream(r2c, st) != CUFFT_SUCCESS || cufftSetWorkArea(r2c, fws) != CUFFT_SUCCESS ||
      cufftExecR2C(r2c, eps, reinterpret_cast<cufftComplex*>(spec)) != CUFFT_SUCCESS)
    return fail(GBP_ERR_CUFFT);
  {
    GBP_TRACE("lognormal_shape", st);
    shape_kernel<<<(unsigned)((modes + 255) / 256), 256, 0, st>>>(spec, grid, 2.0 * M_PI / box,
                                                                   lognormal_amp_over_v(grid, box, k_cut), k_cut);
    if (cudaGetLastError() != cudaSuccess) return fail(GBP_ERR_CUDA);
  }
  if (cufftSetStream(c2r, st) != CUFFT_SUCCESS || cufftSetWorkArea(c2r, fws) != CUFFT_SUCCESS ||
      cufftExecC2R(c2r, reinterpret_cast<cufftComplex*>(spec), eps) != CUFFT_SUCCESS)
    return fail(GBP_ERR_CUFFT);
  if (g_out && cudaMemcpyAsync(g_out, eps, (size_t)cells * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return fail(GBP_ERR_CUDA);
  if (rho_out) {
    rho_out_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(eps, rho_out, cells);
    if (cudaGetLastError() != cudaSuccess) return fail(GBP_ERR_CUDA);
  }
  {
    GBP_TRACE("lognormal_density", st);
    density_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(eps, cdf, cells);
    if (cudaGetLastError() != cudaSuccess) return fail(GBP_ERR_CUDA);
  }
  size_t sb = L.scan;
  if (cub::DeviceScan::InclusiveSum(scan, sb, cdf, cdf, (int64_t)cells, st) != cudaSuccess) return fail(GBP_ERR_CUDA);
  if (n > 0) {
    GBP_TRACE("lognormal_sample", st);
    sample_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cdf, cells, grid, (float)box, (float)sigma_v, n, seed,
                                                               x, y, z);
    if (cudaGetLastError() != cudaSuccess) return fail(GBP_ERR_CUDA);
  }
  // cuFFT plans can be destroyed once their work is enqueued
  return fail(GBP_OK);
}

}  // namespace
}  // namespace gbp

extern "C" int gbp_lognormal(int grid, double box, double k_cut, double sigma_v, int64_t n, unsigned long long seed,
                             float* x, float* y, float* z, void* workspace, size_t ws_bytes, gbp_stream_t stream) {
  return lognormal_run(grid, box, k_cut, sigma_v, n, seed, x, y, z, nullptr, nullptr, workspace, ws_bytes,
                       reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int gbp_lognormal_field(int grid, double box, double k_cut, unsigned long long seed, float* g_out,
                                   float* rho_out, void* workspace, size_t ws_bytes, gbp_stream_t stream) {
  if (!g_out && !rho_out) return GBP_ERR_INVALID;
  return lognormal_run(grid, box, k_cut, 0.0, 0, seed, nullptr, nullptr, nullptr, g_out, rho_out, workspace, ws_bytes,
                       reinterpret_cast<cudaStream_t>(stream));
}
