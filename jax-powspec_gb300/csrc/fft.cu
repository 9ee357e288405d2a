// 3-D real-to-complex FFT of G meshes of side N (power of two, 64..1024) as
// three passes over HBM, each a batch of 1-D transforms staged in shared
// memory (fft_core.cuh):
//
//   z pass  real [G][N][N][N] -> complex [G][N][N][P], P = N/2 + 8: two real
//           z pencils are packed as one complex pencil (a + i b), transformed,
//           and split into their half spectra A, B (k = 0 .. N/2):
//             A[k] = (C[k] + conj C[N-k]) / 2,  B[k] = -i (C[k] - conj C[N-k]) / 2
//   y pass  in place, 8 adjacent kz columns x N rows per CTA
//   x pass  in place, same with rows N*P apart
//
// The z rows are padded from N/2+1 to P = N/2+8 complex (64-byte multiples)
// so every 8-column block of the y and x passes is a whole number of 32-byte
// sectors; the padding is written as zeros by the z pass.  Same transform as
// cuFFT's R2C (forward, unnormalised) and numpy's rfftn.
#include <math.h>

#include <new>
#include <vector>

#include "fft_core.cuh"
#include "gbp_internal.cuh"

namespace gbp {
namespace {

using fft::cadd;
using fft::cmi;
using fft::csub;

__host__ __device__ constexpr int zpitch(int N) { return N / 2 + 8; }

// ---- z pass ---------------------------------------------------------------
// PAIRS complex columns (2*PAIRS real pencils) per CTA, NT = PAIRS * N / 8.
template <int N, int PAIRS>
__global__ void __launch_bounds__(PAIRS * N / 8)
fftz_kernel(const float* __restrict__ mesh, float2* __restrict__ out, long long npencils,
            const float2* __restrict__ tw) {
  constexpr int NT = PAIRS * N / 8;
  constexpr int P = zpitch(N);
  constexpr int H = N / 2;
  extern __shared__ __align__(16) float2 s[];   // [N][PAIRS]
  const int tid = threadIdx.x;
  const long long pen0 = (long long)blockIdx.x * 2 * PAIRS;
  const long long left = npencils - pen0;
  const int npen = left < 2 * PAIRS ? (int)left : 2 * PAIRS;

  // load: lanes walk 2 float4 of one pencil then the next pencil, so each
  // warp reads 16 pencils x 32 contiguous bytes (whole sectors)
  for (int idx = tid; idx < 2 * PAIRS * (N / 4); idx += NT) {
    const int f = (idx >> 1) % (2 * PAIRS);
    const int i4 = ((idx >> 1) / (2 * PAIRS)) * 2 + (idx & 1);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (f < npen) v = __ldcs(reinterpret_cast<const float4*>(mesh + (pen0 + f) * N) + i4);
    float* row = reinterpret_cast<float*>(s) + (f & 1);
    const int c = f >> 1;
    row[((4 * i4 + 0) * PAIRS + c) * 2] = v.x;
    row[((4 * i4 + 1) * PAIRS + c) * 2] = v.y;
    row[((4 * i4 + 2) * PAIRS + c) * 2] = v.z;
    row[((4 * i4 + 3) * PAIRS + c) * 2] = v.w;
  }
  __syncthreads();
  fft::fft_columns<N, PAIRS, PAIRS, NT>(s, tw, tid);

  // split the packed spectra and write both pencils' rows (padding -> 0)
  for (int idx = tid; idx < PAIRS * P; idx += NT) {
    const int q = idx % PAIRS, k = idx / PAIRS;
    if (2 * q >= npen) continue;
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (k <= H) {
      const float2 c = s[k * PAIRS + q];
      const float2 m = s[((N - k) & (N - 1)) * PAIRS + q];
      const float2 cm = make_float2(m.x, -m.y);
      const float2 sum = cadd(c, cm), dif = cmi(csub(c, cm));
      a = make_float2(0.5f * sum.x, 0.5f * sum.y);
      b = make_float2(0.5f * dif.x, 0.5f * dif.y);
    }
    out[(pen0 + 2 * q) * P + k] = a;
    if (2 * q + 1 < npen) out[(pen0 + 2 * q + 1) * P + k] = b;
  }
}

// ---- y and x passes --------------------------------------------------------
// C columns (adjacent kz) x N rows per CTA, rows `row_stride` complex apart;
// CTA b covers plane (b / nkb) and kz block (b % nkb) of its grid.
template <int N, int C>
__global__ void __launch_bounds__(C * N / 8)
fft_cols_kernel(float2* __restrict__ data, long long plane_stride, long long row_stride, int nplanes, int nkb,
                const float2* __restrict__ tw) {
  constexpr int NT = C * N / 8;
  extern __shared__ __align__(16) float2 s[];   // [N][C]
  const int tid = threadIdx.x;
  const int plane = blockIdx.x / nkb, kb = blockIdx.x % nkb;
  if (plane >= nplanes) return;
  float2* base = data + plane * plane_stride + kb * C;
  for (int idx = tid; idx < N * C / 2; idx += NT) {           // float4 = 2 complex
    const int row = idx / (C / 2), c2 = idx % (C / 2);
    const float4 v = __ldcs(reinterpret_cast<const float4*>(base + row * row_stride) + c2);
    reinterpret_cast<float4*>(s)[idx] = v;
  }
  __syncthreads();
  fft::fft_columns<N, C, C, NT>(s, tw, tid);
  for (int idx = tid; idx < N * C / 2; idx += NT) {
    const int row = idx / (C / 2), c2 = idx % (C / 2);
    __stcs(reinterpret_cast<float4*>(base + row * row_stride) + c2, reinterpret_cast<const float4*>(s)[idx]);
  }
}

template <int N>
constexpr int z_pairs() { return N >= 256 ? 8 : 32768 / (N * 8); }   // >= 256 threads
template <int N>
constexpr int col_block() { return N >= 1024 ? 8 : 8; }

template <int N>
int run_fft(const float* mesh, float2* spec, int G, const float2* tw, cudaStream_t st) {
  constexpr int PAIRS = z_pairs<N>();
  constexpr int P = zpitch(N);
  constexpr int C = col_block<N>();
  const long long npen = (long long)G * N * N;
  {
    const size_t smem = (size_t)N * PAIRS * sizeof(float2);
    auto k = fftz_kernel<N, PAIRS>;
    GBP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long blocks = (npen + 2 * PAIRS - 1) / (2 * PAIRS);
    GBP_TRACE("fft_z", st);
    k<<<(unsigned)blocks, PAIRS * N / 8, smem, st>>>(mesh, spec, npen, tw);
    GBP_LAUNCH_CHECK();
  }
  const int nkb = P / C;
  const size_t smem = (size_t)N * C * sizeof(float2);
  auto kc = fft_cols_kernel<N, C>;
  GBP_CUDA_TRY(cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  {  // y pass: a plane is one x slab of one grid; rows (y) are P apart
    GBP_TRACE("fft_y", st);
    kc<<<(unsigned)(G * N * nkb), C * N / 8, smem, st>>>(spec, (long long)N * P, P, G * N, nkb, tw);
    GBP_LAUNCH_CHECK();
  }
  // x pass: a plane is one y row of one grid; rows (x) are N*P apart
  for (int g = 0; g < G; ++g) {
    GBP_TRACE("fft_x", st);
    kc<<<(unsigned)(N * nkb), C * N / 8, smem, st>>>(spec + (long long)g * N * N * P, P, (long long)N * P, N,
                                                      nkb, tw);
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

}  // namespace gbp
