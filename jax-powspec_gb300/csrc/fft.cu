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
// PAIRS complex columns (2*PAIRS real pencils) per CTA; a thread transforms
// two columns (four pencils) at once, NT = (PAIRS / 2) * N / 8.  Consecutive
// lanes take consecutive z, so the first stage's loads of each pencil are
// 128-byte coalesced.  Shared memory is column-major in 16-byte slots of two
// columns (fft_pass.cuh).  The last stage stays in shared memory, where each
// half spectrum needs C[k] and C[N-k] together.
using fft::zsw;

template <int N, int PAIRS>
__global__ void __launch_bounds__(PAIRS * N / 16)
fftz_kernel(const float* __restrict__ mesh, float2* __restrict__ out, long long npencils,
            const float2* __restrict__ tw) {
  pdl_wait();
  constexpr int NT = PAIRS * N / 16;
  constexpr int CP = PAIRS / 2;
  constexpr int P = zpitch(N);
  constexpr int H = N / 2;
  extern __shared__ __align__(16) float4 s4[];    // [CP][N] slots of two columns
  const int tid = threadIdx.x;
  const long long pen0 = (long long)blockIdx.x * 2 * PAIRS;
  const long long left = npencils - pen0;
  const int npen = left < 2 * PAIRS ? (int)left : 2 * PAIRS;
  const float* base = mesh + pen0 * N;

  auto gin = [base, npen](int j, int cp) {      // pencils 4cp .. 4cp+3 at z = j
    float v[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) v[f] = 4 * cp + f < npen ? __ldcs(base + (4 * cp + f) * N + j) : 0.0f;
    return make_float4(v[0], v[1], v[2], v[3]);
  };
  auto sin_ = [](int j, int cp) { return s4[cp * N + zsw(j)]; };
  auto sout = [](int j, int cp, float4 v) { s4[cp * N + zsw(j)] = v; };
  fft::run_stages2<N, CP, NT, true, false, true>(gin, sin_, sout, sout, tw, tid);

  // split the packed spectra and write both pencils' rows (padding -> 0); two k per thread and
  // 16-byte stores (rows are P = N/2 + 8 complex: 16-byte aligned)
  const float2* s2 = reinterpret_cast<const float2*>(s4);
  constexpr int P2 = P / 2;
  for (int idx = tid; idx < PAIRS * P2; idx += NT) {
    const int q = idx / P2, k0 = 2 * (idx - q * P2);
    if (2 * q >= npen) continue;
    const float2* col = s2 + (q >> 1) * N * 2 + (q & 1);
    float2 a[2], b[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = k0 + h;
      a[h] = b[h] = make_float2(0.f, 0.f);
      if (k <= H) {
        const float2 c = col[zsw(k) * 2];
        const float2 m = col[zsw((N - k) & (N - 1)) * 2];
        const float2 cm = make_float2(m.x, -m.y);
        const float2 sum = cadd(c, cm), dif = cmi(csub(c, cm));
        a[h] = make_float2(0.5f * sum.x, 0.5f * sum.y);
        b[h] = make_float2(0.5f * dif.x, 0.5f * dif.y);
      }
    }
    __stcs(reinterpret_cast<float4*>(out + (pen0 + 2 * q) * P + k0), make_float4(a[0].x, a[0].y, a[1].x, a[1].y));
    if (2 * q + 1 < npen)
      __stcs(reinterpret_cast<float4*>(out + (pen0 + 2 * q + 1) * P + k0),
             make_float4(b[0].x, b[0].y, b[1].x, b[1].y));
  }
}

// ---- y and x passes --------------------------------------------------------
// 8 adjacent kz columns x N rows per CTA, rows `row_stride` complex apart;
// CTA b covers plane (b / nkb) and kz block (b % nkb).  N/2 threads: one
// pair of radix-8 butterflies (two columns) each per stage; the first stage
// loads from HBM and the last stores to HBM (fft_pass.cuh), in place.
template <int N>
__global__ void __launch_bounds__(N / 2, N <= 512 ? 4 : 2)
fft_cols_kernel(float2* __restrict__ data, long long plane_stride, long long row_stride, int nplanes, int nkb,
                const float2* __restrict__ tw) {
  pdl_wait();
  extern __shared__ __align__(16) float2 s[];
  const int plane = blockIdx.x / nkb, kb = blockIdx.x % nkb;
  if (plane >= nplanes) return;
  float2* base = data + plane * plane_stride + kb * 8;
  auto gin = [base, row_stride](int j, int cp) {
    return __ldcs(reinterpret_cast<const float4*>(base + j * row_stride) + cp);
  };
  auto gout = [base, row_stride](int j, int cp, float4 v) {
    __stcs(reinterpret_cast<float4*>(base + j * row_stride) + cp, v);
  };
  fft::col_fft<N, 1, N / 2, false>(s, gin, gout, tw, threadIdx.x);
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
    GBP_CUDA_TRY(launch_pdl(k, dim3((unsigned)blocks), dim3(PAIRS * N / 16), smem, st, mesh, spec, npen, tw));
  }
  const int nkb = P / C;
  const size_t smem = (size_t)fft::ColBlock<N, 1>::SLAB * sizeof(float2);
  auto kc = fft_cols_kernel<N>;
  GBP_CUDA_TRY(cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  {  // y pass: a plane is one x slab of one grid; rows (y) are P apart
    GBP_TRACE("fft_y", st);
    GBP_CUDA_TRY(launch_pdl(kc, dim3((unsigned)(G * N * nkb)), dim3(N / 2), smem, st, spec, (long long)N * P,
                            (long long)P, G * N, nkb, tw));
  }
  // x pass: a plane is one y row of one grid; rows (x) are N*P apart
  for (int g = 0; x_pass && g < G; ++g) {
    GBP_TRACE("fft_x", st);
    GBP_CUDA_TRY(launch_pdl(kc, dim3((unsigned)(N * nkb)), dim3(N / 2), smem, st, spec + (long long)g * N * N * P,
                            (long long)P, (long long)N * P, N, nkb, tw));
  }
  return GBP_OK;
}

}  // namespace

// Entry used by gbp_fft_r2c for power-of-two meshes (declared in api.cu).
bool own_fft_supported(int N) { return N == 64 || N == 128 || N == 256 || N == 512 || N == 1024; }
int own_fft_pitch(int N) { return zpitch(N); }

// Twiddles of an N-point transform: exp(-2 pi i e / N) for e < N, then one
// table per stage of span p > 1 (radix R): entry k * 8 + r holds
// exp(-2 pi i r k / (R p)) for r < R (fft_pass.cuh reads them as float4s).
template <int N>
std::vector<float2> twiddle_tables() {
  std::vector<float2> h((size_t)fft::tw_size<N>(), make_float2(0.f, 0.f));
  for (int e = 0; e < N; ++e) {
    const double a = -2.0 * M_PI * (double)e / (double)N;
    h[e] = make_float2((float)cos(a), (float)sin(a));
  }
  using RD = fft::Radices<N>;
  int p = 1;
  for (int st = 0; st < RD::stages; ++st) {
    const int R = st < RD::n8 ? 8 : (RD::tail == 1 ? 2 : 4);
    if (p > 1) {
      for (int k = 0; k < p; ++k)
        for (int r = 0; r < R; ++r) {
          const double a = -2.0 * M_PI * (double)r * (double)k / ((double)R * (double)p);
          h[(size_t)fft::tw_off<N>(p) + (size_t)k * 8 + r] = make_float2((float)cos(a), (float)sin(a));
        }
    }
    p *= R;
  }
  return h;
}

int own_fft_twiddles(int N, float2** d_tw) {
  std::vector<float2> h;
  switch (N) {
    case 64: h = twiddle_tables<64>(); break;
    case 128: h = twiddle_tables<128>(); break;
    case 256: h = twiddle_tables<256>(); break;
    case 512: h = twiddle_tables<512>(); break;
    case 1024: h = twiddle_tables<1024>(); break;
    default: return GBP_ERR_UNSUPPORTED;
  }
  float2* d = nullptr;
  if (cudaMalloc(&d, h.size() * sizeof(float2)) != cudaSuccess) return GBP_ERR_ALLOC;
  const cudaError_t ce = cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice);
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
