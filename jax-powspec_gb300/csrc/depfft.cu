// C ABI of the fused particles -> multipole sums path (depfft_impl.cuh;
// one translation unit per mesh side, depfft_n<N>.cu) and its tile shapes.
//
// The column tile (TX x TY pencils over all of z) is a plan option:
// gbp_fft_plan_set_tiles picks one of column_tile_variants(N); zero means
// the default (8x4 at 256^3 and 512^3, 4x4 otherwise).  Every shape gives
// the same P_l bit for bit (fixed-point scales per 4x4 block, see
// depfft_impl.cuh); they differ in speed only.
#include <cstdint>

#include "gbp_bins.h"
#include "gbp_fft.h"
#include "gbp_internal.cuh"

namespace gbp {

#define GBP_DEPFFT_DECL(NN)                                                                                        \
  int particles_ws_n##NN(int64_t n, gbp_fft_plan plan, gbp_bins bins, int mas, int ells, int tx, int ty,           \
                         size_t* bytes);                                                                           \
  int particles_power_n##NN(const float* x, const float* y, const float* z, const float* w, int64_t n, float xmin, \
                            float ymin, float zmin, float inv_cell, const gbp_job* job, gbp_fft_plan plan,        \
                            gbp_bins bins, int mas, int ells, int tx, int ty, void* spectrum, double* sums_out,    \
                            long long* nmodes_out, double* ksum_out, gbp_deposit_stats* stats_out,                 \
                            void* workspace, size_t ws_bytes, cudaStream_t st);
GBP_DEPFFT_DECL(64)
GBP_DEPFFT_DECL(128)
GBP_DEPFFT_DECL(256)
GBP_DEPFFT_DECL(512)
GBP_DEPFFT_DECL(1024)
#undef GBP_DEPFFT_DECL

namespace {

// Supported column tiles per mesh side, the default first.  8x8 needs 2x the
// shared memory of 8x4 (and its 64-bit clump kernel 2x again): 128^3 and
// 256^3 only; 1024^3 keeps 4x4 (the clump kernel's 64-bit cells of an 8x4
// tile would not fit).
int tile_variants(int N, int (*v)[2]) {
  switch (N) {
    case 64: v[0][0] = 4; v[0][1] = 4; v[1][0] = 8; v[1][1] = 4; return 2;
    case 128: v[0][0] = 4; v[0][1] = 4; v[1][0] = 8; v[1][1] = 4; v[2][0] = 8; v[2][1] = 8; return 3;
    case 256: v[0][0] = 8; v[0][1] = 4; v[1][0] = 4; v[1][1] = 4; v[2][0] = 8; v[2][1] = 8; return 3;
    case 512: v[0][0] = 8; v[0][1] = 4; v[1][0] = 4; v[1][1] = 4; return 2;
    case 1024: v[0][0] = 4; v[0][1] = 4; return 1;
    default: return 0;
  }
}

bool tile_supported(int N, int tx, int ty) {
  int v[4][2];
  const int k = tile_variants(N, v);
  for (int i = 0; i < k; ++i)
    if (v[i][0] == tx && v[i][1] == ty) return true;
  return false;
}

// The plan's tile shape, or the default for its side.
int plan_tiles(gbp_fft_plan plan, int& tx, int& ty) {
  int v[4][2];
  if (!plan || tile_variants(plan->n, v) == 0) return GBP_ERR_UNSUPPORTED;
  tx = plan->tx ? plan->tx : v[0][0];
  ty = plan->ty ? plan->ty : v[0][1];
  return GBP_OK;
}

int particles_ws(int64_t n, gbp_fft_plan plan, gbp_bins B, int mas, int ells, size_t* bytes) {
  if (!plan || !B || plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own) return GBP_ERR_UNSUPPORTED;
  int tx = 0, ty = 0;
  const int st = plan_tiles(plan, tx, ty);
  if (st) return st;
  switch (B->N) {
    case 64: return particles_ws_n64(n, plan, B, mas, ells, tx, ty, bytes);
    case 128: return particles_ws_n128(n, plan, B, mas, ells, tx, ty, bytes);
    case 256: return particles_ws_n256(n, plan, B, mas, ells, tx, ty, bytes);
    case 512: return particles_ws_n512(n, plan, B, mas, ells, tx, ty, bytes);
    case 1024: return particles_ws_n1024(n, plan, B, mas, ells, tx, ty, bytes);
    default: return GBP_ERR_UNSUPPORTED;
  }
}

int particles_call(const float* x, const float* y, const float* z, const float* w, int64_t n, float xmin, float ymin,
                   float zmin, float inv_cell, const gbp_job* job, gbp_fft_plan plan, gbp_bins B, int mas, int ells,
                   void* spectrum, double* sums_out, long long* nmodes_out, double* ksum_out,
                   gbp_deposit_stats* stats_out, void* workspace, size_t ws_bytes, cudaStream_t st) {
  if (!plan || !B || plan->n != B->N) return GBP_ERR_INVALID;
  if (!plan->own) return GBP_ERR_UNSUPPORTED;
  int tx = 0, ty = 0;
  const int r = plan_tiles(plan, tx, ty);
  if (r) return r;
#define GBP_CALL(NN)                                                                                               \
  particles_power_n##NN(x, y, z, w, n, xmin, ymin, zmin, inv_cell, job, plan, B, mas, ells, tx, ty, spectrum,     \
                        sums_out, nmodes_out, ksum_out, stats_out, workspace, ws_bytes, st)
  switch (B->N) {
    case 64: return GBP_CALL(64);
    case 128: return GBP_CALL(128);
    case 256: return GBP_CALL(256);
    case 512: return GBP_CALL(512);
    case 1024: return GBP_CALL(1024);
    default: return GBP_ERR_UNSUPPORTED;
  }
#undef GBP_CALL
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_column_tile_variants(int n_mesh, int* tx, int* ty, int max, int* count) {
  if (!count || max < 0 || (max > 0 && (!tx || !ty))) return GBP_ERR_INVALID;
  int v[4][2];
  const int k = tile_variants(n_mesh, v);
  for (int i = 0; i < k && i < max; ++i) {
    tx[i] = v[i][0];
    ty[i] = v[i][1];
  }
  *count = k;
  return k ? GBP_OK : GBP_ERR_UNSUPPORTED;
}

extern "C" int gbp_fft_plan_set_tiles(gbp_fft_plan plan, int tx, int ty) {
  if (!plan) return GBP_ERR_INVALID;
  if (tx == 0 && ty == 0) {
    plan->tx = plan->ty = 0;
    return GBP_OK;
  }
  if (!plan->own || !tile_supported(plan->n, tx, ty)) return GBP_ERR_UNSUPPORTED;
  plan->tx = tx;
  plan->ty = ty;
  return GBP_OK;
}

extern "C" int gbp_fft_plan_tiles(gbp_fft_plan plan, int* tx, int* ty) {
  if (!plan || !tx || !ty) return GBP_ERR_INVALID;
  int a = 0, b = 0;
  const int st = plan_tiles(plan, a, b);
  if (st) return st;
  *tx = a;
  *ty = b;
  return GBP_OK;
}

extern "C" int gbp_particles_power_workspace_size(int64_t n, gbp_fft_plan plan, gbp_bins bins, int mas, int ells,
                                                  size_t* bytes) {
  if (!bytes) return GBP_ERR_INVALID;
  return particles_ws(n, plan, bins, mas, ells, bytes);
}

extern "C" int gbp_particles_power(const float* x, const float* y, const float* z, const float* w, int64_t n,
                                   float xmin, float ymin, float zmin, float inv_cell, gbp_fft_plan plan,
                                   gbp_bins bins, int mas, int ells, void* spectrum, double* sums_out,
                                   long long* nmodes_out, double* ksum_out, gbp_deposit_stats* stats_out,
                                   void* workspace, size_t ws_bytes, gbp_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !y || !z))) return GBP_ERR_INVALID;
  if (!plan || !bins) return GBP_ERR_INVALID;
  return particles_call(x, y, z, w, n, xmin, ymin, zmin, inv_cell, nullptr, plan, bins, mas, ells, spectrum,
                        sums_out, nmodes_out, ksum_out, stats_out, workspace, ws_bytes,
                        reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int gbp_particles_power_job(const gbp_job* job, int64_t capacity, gbp_fft_plan plan, gbp_bins bins,
                                       int mas, int ells, void* spectrum, double* sums_out, long long* nmodes_out,
                                       double* ksum_out, gbp_deposit_stats* stats_out, void* workspace,
                                       size_t ws_bytes, gbp_stream_t stream) {
  if (!job || capacity < 0 || !plan || !bins) return GBP_ERR_INVALID;
  return particles_call(nullptr, nullptr, nullptr, nullptr, capacity, 0.f, 0.f, 0.f, 0.f, job, plan, bins, mas,
                        ells, spectrum, sums_out, nmodes_out, ksum_out, stats_out, workspace, ws_bytes,
                        reinterpret_cast<cudaStream_t>(stream));
}
