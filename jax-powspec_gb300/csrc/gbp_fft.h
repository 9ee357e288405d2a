// Internal view of an FFT plan and the library's own three-pass transform
// (fft.cu), shared by the C entry points (api.cu) and the fused x-pass +
// binning (xbin.cu).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include "gbpowspec.h"

struct gbp_fft_plan_s {
  bool own;
  cufftHandle h;
  float2* tw;       // own transform: twiddles exp(-2 pi i e / N)
  int n, grids, pitch;
  size_t ws;
  int tx = 0, ty = 0;   // column tile of the fused particles path (0: the default for n)
};

namespace gbp {
bool own_fft_supported(int N);
int own_fft_pitch(int N);
int own_fft_twiddles(int N, float2** d_tw);
int own_fft_r2c(int N, int G, const float* mesh, float2* spec, const float2* tw, cudaStream_t st);
// z and y passes only: spec holds the transform over z and y, not yet over x
int own_fft_zy(int N, int G, const float* mesh, float2* spec, const float2* tw, cudaStream_t st);
// y pass only (spec already transformed over z)
int own_fft_y(int N, int G, float2* spec, const float2* tw, cudaStream_t st);
// x pass fused with the binning + the fold into per-bin sums (xbin.cu); spec
// holds the transform over z and y
int xbin_power_workspace(gbp_fft_plan plan, gbp_bins bins, int ells, size_t* bytes);
// Cached cuFFT plan (per device) of `batch` unnormalised inverse real 3-D
// transforms: complex input rows of P >= N/2+1 entries ([batch][N][N][P]),
// real output [batch][N][N][N].  No work area of its own: *ws bytes are
// passed with cufftSetWorkArea (0 when the plan needs none).
int c2r_plan(int N, int P, int batch, cufftHandle* h, size_t* ws);
// Enqueue that transform on `st` with `work` (>= ws bytes, its own region:
// not the input) as the work area; the plan's stream and work area are set
// and the transform enqueued under a lock, so concurrent callers cannot mix
// them up.  `in` is overwritten (cuFFT's multi-dimensional C2R).
int c2r_exec(int N, int P, int batch, const float2* in, float* out, void* work, cudaStream_t st);
int xbin_power(gbp_fft_plan plan, float2* spec, gbp_bins bins, int mas_order, int ells, const double* mass,
               double* sums_out, long long* nmodes_out, double* ksum_out, void* ws, size_t ws_bytes,
               cudaStream_t st);
}  // namespace gbp
