// 3-D real-to-complex FFT of G meshes of side N (power of two, 64..1024) as
// three passes over HBM, each a batch of 1-D transforms staged in shared
// memory (fft_core.cuh):
//
//   z pass  real [G][N][N][N] -> complex [G][N][N][P], P = N/2 + 8: two real
//           z pencils are packed as one complex pencil (a + i b), transformed,
//           and split into their half spectra A, B (k = 0 .. N/2):
//             A[k] = (C[k] + conj C[N-k]) / 2,  B[k] = -i (C[k] - conj C[N-k]) / 2
//   y pass  in place, 8 adjacent kz columns x N rows per CTA; the first
//           stage reads HBM and the last writes it (fft_pass.cuh)
//   x pass  in place, same with rows N*P apart (the pipeline fuses it with
//           the binning instead: xbin.cu)
//
// The z rows are padded from N/2+1 to P = N/2+8 complex (64-byte multiples)
// so every 8-column block of the y and x passes is a whole number of 32-byte
// sectors; the padding is written as zeros by the z pass.  Same transform as
// cuFFT's R2C (forward, unnormalised) and numpy's rfftn.
#include <math.h>

#include <new>
#include <vector>

#include "fft_core.cuh"
#include "fft_pass.cuh"
#include "gbp_fft.h"
#include "gbp_internal.cuh"

namespace gbp {
namespace {

using fft::cadd;
using fft::cmi;
using fft::csub;

__host__ __device__ constexpr int zpitch(int N) { return N / 2 + 8; }

// ---- z pass ---------------------------------------------------------------
// PAIRS complex columns (2*PAIRS real pencils) per CTA, NT = PAIRS * N / 8.
// Consecutive lanes take consecutive z, so the first stage's loads of each
// pencil are 128-byte coalesced.  Shared memory is column-major, column q
// holding pair q, with row j stored at fft::zsw(j) (conflict-free for every
// stage).  The last stage stays in shared memory, where each half spectrum
// needs C[k] and C[N-k] together.
using fft::zsw;

template <int N, int PAIRS>
__global__ void __launch_bounds__(PAIRS * N / 8)
fftz_kernel(const float* __restrict__ mesh, float2* __restrict__ out, long long npencils,
            const float2* __restrict__ tw) {
  constexpr int NT = PAIRS * N / 8;
  constexpr int P = zpitch(N);
  constexpr int H = N / 2;
  constexpr int LD = N;
  extern __shared__ __align__(16) float2 s[];     // [PAIRS][LD]
  const int tid = threadIdx.x;
  const long long pen0 = (long long)blockIdx.x * 2 * PAIRS;
  const long long left = npencils - pen0;
  const int npen = left < 2 * PAIRS ? (int)left : 2 * PAIRS;
  const float* base = mesh + pen0 * N;

  auto gin = [base, npen](int j, int q) {
    const float a = 2 * q < npen ? __ldcs(base + (2 * q) * N + j) : 0.0f;
    const float b = 2 * q + 1 < npen ? __ldcs(base + (2 * q + 1) * N + j) : 0.0f;
    return make_float2(a, b);
  };
  auto sin_ = [](int j, int q) { return s[q * LD + zsw(j)]; };
  auto sout = [](int j, int q, float2 v) { s[q * LD + zsw(j)] = v; };
  fft::run_stages<N, PAIRS, NT, true, true>(gin, sin_, sout, sout, tw, tid);

  // split the packed spectra and write both pencils' rows (padding -> 0)
  for (int idx = tid; idx < PAIRS * P; idx += NT) {
    const int q = idx / P, k = idx - (idx / P) * P;
    if (2 * q >= npen) continue;
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (k <= H) {
      const float2 c = s[q * LD + zsw(k)];
      const float2 m = s[q * LD + zsw((N - k) & (N - 1))];
      const float2 cm = make_float2(m.x, -m.y);
      const float2 sum = cadd(c, cm), dif = cmi(csub(c, cm));
      a = make_float2(0.5f * sum.x, 0.5f * sum.y);
      b = make_float2(0.5f * dif.x, 0.5f * dif.y);
    }
    __stcs(out + (pen0 + 2 * q) * P + k, a);
    if (2 * q + 1 < npen) __stcs(out + (pen0 + 2 * q + 1) * P + k, b);
  }
}

// ---- y and x passes --------------------------------------------------------
// 8 adjacent kz columns x N rows per CTA, rows `row_stride` complex apart;
// CTA b covers plane (b / nkb) and kz block (b % nkb).  N threads: one
// radix-8 butterfly each per stage; the first stage loads from HBM and the
// last stores to HBM (fft_pass.cuh), in place.
template <int N>
__global__ void __launch_bounds__(N, 2048 / N < 3 ? 2048 / N : 3)
fft_cols_kernel(float2* __restrict__ data, long long plane_stride, long long row_stride, int nplanes, int nkb,
                const float2* __restrict__ tw) {
  extern __shared__ __align__(16) float2 s[];
  const int plane = blockIdx.x / nkb, kb = blockIdx.x % nkb;
  if (plane >= nplanes) return;
  float2* base = data + plane * plane_stride + kb * 8;
  auto gin = [base, row_stride](int j, int col) { return __ldcs(base + j * row_stride + col); };
  auto gout = [base, row_stride](int j, int col, float2 v) { __stcs(base + j * row_stride + col, v); };
  fft::col_fft<N, 1, N, false>(s, gin, gout, tw, threadIdx.x);
}

template <int N>
constexpr int z_pairs() { return N >= 256 ? 8 : 32768 / (N * 8); }   // >= 256 threads
template <int N>
int run_fft(const float* mesh, float2* spec, int G, const float2* tw, cudaStream_t st, bool x_pass = true,
            bool z_pass = true) {
  constexpr int PAIRS = z_pairs<N>();
  constexpr int P = zpitch(N);
  constexpr int C = 8;                    // kz columns per CTA in the y and x passes
  const long long npen = (long long)G * N * N;
  if (z_pass) {
    const size_t smem = (size_t)PAIRS * N * sizeof(float2);
    auto k = fftz_kernel<N, PAIRS>;
    GBP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long blocks = (npen + 2 * PAIRS - 1) / (2 * PAIRS);
    GBP_TRACE("fft_z", st);
    k<<<(unsigned)blocks, PAIRS * N / 8, smem, st>>>(mesh, spec, npen, tw);
    GBP_LAUNCH_CHECK();
  }
  const int nkb = P / C;
  const size_t smem = (size_t)fft::ColBlock<N, 1>::SLAB * sizeof(float2);
  auto kc = fft_cols_kernel<N>;
  GBP_CUDA_TRY(cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  {  // y pass: a plane is one x slab of one grid; rows (y) are P apart
    GBP_TRACE("fft_y", st);
    kc<<<(unsigned)(G * N * nkb), N, smem, st>>>(spec, (long long)N * P, P, G * N, nkb, tw);
    GBP_LAUNCH_CHECK();
  }
  // x pass: a plane is one y row of one grid; rows (x) are N*P apart
  for (int g = 0; x_pass && g < G; ++g) {
    GBP_TRACE("fft_x", st);
    kc<<<(unsigned)(N * nkb), N, smem, st>>>(spec + (long long)g * N * N * P, P, (long long)N * P, N, nkb, tw);
    GBP_LAUNCH_CHECK();
  }
  return GBP_OK;
}

}  // namespace

// Entry used by gbp_fft_r2c for power-of-two meshes (declared in api.cu).
bool own_fft_supported(int N) { return N == 64 || N == 128 || N == 256 || N == 512 || N == 1024; }
int own_fft_pitch(int N) { return zpitch(N); }

int own_fft_twiddles(int N, float2** d_tw) {
  std::vector<float2> h((size_t)N);
  for (int e = 0; e < N; ++e) {
    const double a = -2.0 * M_PI * (double)e / (double)N;
    h[e] = make_float2((float)cos(a), (float)sin(a));
  }
  float2* d = nullptr;
  if (cudaMalloc(&d, (size_t)N * sizeof(float2)) != cudaSuccess) return GBP_ERR_ALLOC;
  const cudaError_t ce = cudaMemcpy(d, h.data(), (size_t)N * sizeof(float2), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    set_last_cuda_error(ce);
    cudaFree(d);
    return GBP_ERR_CUDA;
  }
  *d_tw = d;
  return GBP_OK;
}

int own_fft_r2c(int N, int G, const float* mesh, float2* spec, const float2* tw, cudaStream_t st) {
  switch (N) {
    case 64: return run_fft<64>(mesh, spec, G, tw, st);
    case 128: return run_fft<128>(mesh, spec, G, tw, st);
    case 256: return run_fft<256>(mesh, spec, G, tw, st);
    case 512: return run_fft<512>(mesh, spec, G, tw, st);
    case 1024: return run_fft<1024>(mesh, spec, G, tw, st);
    default: return GBP_ERR_UNSUPPORTED;
  }
}

int own_fft_y(int N, int G, float2* spec, const float2* tw, cudaStream_t st) {
  switch (N) {
    case 64: return run_fft<64>(nullptr, spec, G, tw, st, false, false);
    case 128: return run_fft<128>(nullptr, spec, G, tw, st, false, false);
    case 256: return run_fft<256>(nullptr, spec, G, tw, st, false, false);
    case 512: return run_fft<512>(nullptr, spec, G, tw, st, false, false);
    case 1024: return run_fft<1024>(nullptr, spec, G, tw, st, false, false);
    default: return GBP_ERR_UNSUPPORTED;
  }
}

int own_fft_zy(int N, int G, const float* mesh, float2* spec, const float2* tw, cudaStream_t st) {
  switch (N) {
    case 64: return run_fft<64>(mesh, spec, G, tw, st, false);
    case 128: return run_fft<128>(mesh, spec, G, tw, st, false);
    case 256: return run_fft<256>(mesh, spec, G, tw, st, false);
    case 512: return run_fft<512>(mesh, spec, G, tw, st, false);
    case 1024: return run_fft<1024>(mesh, spec, G, tw, st, false);
    default: return GBP_ERR_UNSUPPORTED;
  }
}

}  // namespace gbp
