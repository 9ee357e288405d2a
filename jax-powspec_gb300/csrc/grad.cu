// Gradients of the P_l(k) estimator with respect to particle positions and
// weights (the adjoint of deposit -> R2C -> |delta_k|^2 L_l binning), the
// derivative the reference obtains from JAX autodiff (tests/lognormal.py:
// 60-103 differentiates a loss of powspec_vec through cic_mas_vec).
//
// With P_l(b) = (2l+1) norm / n_b sum_{k in b} c2(k) L_l(mu_k) |D(k)|^2
// (D = F for one grid, D = (F0 + phi F1) / 2 interlaced, phi = exp(i pi
// (kx+ky+kz) / N), norm = L^3 / M^2, the k = 0 mode excluded) and an
// upstream gradient g = dLoss/dP_l(b):
//
//   dLoss/d rho_0(c) = Re sum_{k in half} 2 f A(k) D(k) exp(+i k.c)
//   dLoss/d rho_1(c) = Re sum_{k in half} 2 f A(k) D(k) conj(phi) exp(+i k.c)
//
// with A(k) = sum_l g_{b(k), l} (2l+1) L_l(mu) c2(k) norm / n_b, f = 1 for
// one grid and 1/2 for each of two.  A C2R of the half spectrum counts every
// kz in (0, N/2) twice and the kz = 0, N/2 planes once, so the adjoint
// spectrum is H = f A D (times conj(phi)) with the two planes doubled, and
// gradient mesh = C2R(H) (unnormalised, as the forward transform).
//
// The deposit's adjoint is a gather: for each particle, the B-spline weights
// W and their derivatives dW/du of its stencil nodes (per grid), times the
// gradient mesh there: dLoss/dw_i = sum grad W, dLoss/du_a = w_i sum grad
// dW/du_a, and dLoss/dx_a = inv_cell dLoss/du_a.  The explicit dependence of
// the normalisation and of the shot noise on the weights is added on the
// host side (gbpowspec/grad.py); it is nb-sized arithmetic.
#include <cufft.h>
#include <math.h>

#include "gbp_bins.h"
#include "gbp_fft.h"
#include "gbp_internal.cuh"

namespace gbp {
namespace {

__device__ __forceinline__ int bin_search(const int* __restrict__ thr, int nbe, int nb, int tu, int k2) {
  if (k2 > tu) return -1;
  int lo = 0, hi = nbe + 1;                      // count thresholds <= k2
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(thr + mid) <= k2) lo = mid + 1;
    else hi = mid;
  }
  const int r = lo;
  return min(min(r, nb), nbe) - 1;
}

// H_g(k) for every half-spectrum entry (row padding -> 0).
__global__ void grad_spec_kernel(const float2* __restrict__ spec, float2* __restrict__ hspec, int N, int P, int G,
                                 const int* __restrict__ thr, int nbe, int nb, int tu,
                                 const float* __restrict__ inv_sinc2, const float2* __restrict__ eph, int mas_order,
                                 const double* __restrict__ grad_pk, const long long* __restrict__ nmodes,
                                 const double* __restrict__ mass, double box) {
  const long long total = (long long)N * N * P;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int kz = (int)(i % P);
  float2 h0 = make_float2(0.f, 0.f), h1 = make_float2(0.f, 0.f);
  const int iy = (int)((i / P) % N), ix = (int)(i / ((long long)P * N));
  const int kx = signed_k(ix, N), ky = signed_k(iy, N);
  const int k2 = kx * kx + ky * ky + kz * kz;
  const int b = (kz <= N / 2 && k2 > 0) ? bin_search(thr, nbe, nb, tu, k2) : -1;
  if (b >= 0 && nmodes[b] > 0) {
    const double m = mass[0];
    const double norm = box * box * box / (m * m) / (double)nmodes[b];
    const float mu2 = (float)(kz * kz) / (float)k2;
    const float l2 = 1.5f * mu2 - 0.5f, l4 = (35.0f * mu2 * mu2 - 30.0f * mu2 + 3.0f) * 0.125f;
    const float gsum = (float)(grad_pk[b * 3 + 0] * norm) + 5.0f * l2 * (float)(grad_pk[b * 3 + 1] * norm) +
                       9.0f * l4 * (float)(grad_pk[b * 3 + 2] * norm);
    const int ax = kx < 0 ? -kx : kx, ay = ky < 0 ? -ky : ky;
    float c2 = 1.0f;
    for (int p = 0; p < mas_order; ++p) c2 *= inv_sinc2[ax] * inv_sinc2[ay] * inv_sinc2[kz];
    const bool plane = (kz == 0) || (kz == N / 2);
    float2 d = spec[i];
    float2 ph = make_float2(1.f, 0.f);
    float f = plane ? 2.0f : 1.0f;
    if (G == 2) {
      float2 ex = eph[ax], ey = eph[ay], ez = eph[kz];
      if (kx < 0) ex.y = -ex.y;
      if (ky < 0) ey.y = -ey.y;
      const float2 exy = make_float2(ex.x * ey.x - ex.y * ey.y, ex.x * ey.y + ex.y * ey.x);
      ph = make_float2(exy.x * ez.x - exy.y * ez.y, exy.x * ez.y + exy.y * ez.x);
      const float2 f1 = spec[i + total];
      d = make_float2(0.5f * (d.x + (f1.x * ph.x - f1.y * ph.y)), 0.5f * (d.y + (f1.x * ph.y + f1.y * ph.x)));
      f *= 0.5f;
    }
    const float a = gsum * c2 * f;
    h0 = make_float2(a * d.x, a * d.y);
    if (G == 2) h1 = make_float2(h0.x * ph.x + h0.y * ph.y, h0.y * ph.x - h0.x * ph.y);   // * conj(phi)
  }
  hspec[i] = h0;
  if (G == 2) hspec[i + total] = h1;
}

// B-spline of order MAS at grid coordinate u (+ half a cell for the second
// grid): first node, weights and their derivatives d/du.  Same node
// convention and arithmetic as the deposit kernels.
template <int MAS>
__device__ __forceinline__ void bspline_dw(float u, int N, int half, int& first, float (&w)[MAS], float (&dw)[MAS]) {
  const float fu = floorf(u);
  float d = __fsub_rn(u, fu);
  int i = pmod(__float2int_rz(fu), N);
  if (half) {
    d = __fadd_rn(d, 0.5f);
    if (d >= 1.0f) { d = __fsub_rn(d, 1.0f); i += 1; }
  }
  if constexpr (MAS == GBP_NGP) {
    first = i + (d >= 0.5f ? 1 : 0);
    w[0] = 1.0f;
    dw[0] = 0.0f;
  } else if constexpr (MAS == GBP_CIC) {
    first = i;
    w[0] = 1.0f - d; w[1] = d;
    dw[0] = -1.0f; dw[1] = 1.0f;
  } else if constexpr (MAS == GBP_TSC) {
    const int up = d >= 0.5f ? 1 : 0;
    const float s = up ? d - 1.0f : d;
    first = i + up - 1;
    const float l = 0.5f - s, r = 0.5f + s;
    w[0] = 0.5f * l * l; w[1] = 0.75f - s * s; w[2] = 0.5f * r * r;
    dw[0] = -l; dw[1] = -2.0f * s; dw[2] = r;
  } else {
    const float t = d, m = 1.0f - d;
    const float c6 = 1.0f / 6.0f;
    first = i - 1;
    w[0] = m * m * m * c6;
    w[1] = (4.0f - 6.0f * t * t + 3.0f * t * t * t) * c6;
    w[2] = (4.0f - 6.0f * m * m + 3.0f * m * m * m) * c6;
    w[3] = t * t * t * c6;
    dw[0] = -0.5f * m * m;
    dw[1] = (-12.0f * t + 9.0f * t * t) * c6;
    dw[2] = (12.0f * m - 9.0f * m * m) * c6;
    dw[3] = 0.5f * t * t;
  }
}

template <int MAS>
__global__ void deposit_gather_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                      const float* __restrict__ z, const float* __restrict__ wts, long long n,
                                      float ox, float oy, float oz, float inv_cell, int N, int G,
                                      const float* __restrict__ grad_mesh, float* gx, float* gy, float* gz,
                                      float* gw) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float u[3] = {__fmul_rn(__fsub_rn(x[i], ox), inv_cell), __fmul_rn(__fsub_rn(y[i], oy), inv_cell),
                      __fmul_rn(__fsub_rn(z[i], oz), inv_cell)};
  const float wi = wts ? wts[i] : 1.0f;
  const long long M = (long long)N * N * N;
  float sw = 0.f, su[3] = {0.f, 0.f, 0.f};
  for (int g = 0; g < G; ++g) {
    int f[3];
    float w[3][MAS], dw[3][MAS];
    for (int a = 0; a < 3; ++a) bspline_dw<MAS>(u[a], N, g, f[a], w[a], dw[a]);
    const float* gm = grad_mesh + g * M;
    for (int rx = 0; rx < MAS; ++rx) {
      const long long cx = pmod(f[0] + rx, N);
      for (int ry = 0; ry < MAS; ++ry) {
        const long long cy = pmod(f[1] + ry, N);
        for (int rz = 0; rz < MAS; ++rz) {
          const int cz = pmod(f[2] + rz, N);
          const float gv = __ldg(gm + (cx * N + cy) * N + cz);
          sw += gv * w[0][rx] * w[1][ry] * w[2][rz];
          su[0] += gv * dw[0][rx] * w[1][ry] * w[2][rz];
          su[1] += gv * w[0][rx] * dw[1][ry] * w[2][rz];
          su[2] += gv * w[0][rx] * w[1][ry] * dw[2][rz];
        }
      }
    }
  }
  gx[i] = wi * su[0] * inv_cell;
  gy[i] = wi * su[1] * inv_cell;
  gz[i] = wi * su[2] * inv_cell;
  if (gw) gw[i] = sw;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_power_backward_workspace_size(gbp_fft_plan plan, size_t* bytes) {
  if (!plan || !bytes) return GBP_ERR_INVALID;
  cufftHandle h;
  size_t w = 0;
  const int st = c2r_plan(plan->n, plan->pitch, 1, &h, &w);
  if (st) return st;
  *bytes = align256((size_t)plan->grids * plan->n * plan->n * plan->pitch * sizeof(float2)) + align256(w > 0 ? w : 1);
  return GBP_OK;
}

extern "C" int gbp_power_backward(const void* spectrum, gbp_fft_plan plan, gbp_bins B, int mas_order,
                                  const double* grad_pk, const long long* nmodes, const double* mass, double box_size,
                                  float* grad_mesh, void* workspace, size_t ws_bytes, gbp_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!spectrum || !plan || !B || !grad_pk || !nmodes || !mass || !grad_mesh || !(box_size > 0.0))
    return GBP_ERR_INVALID;
  if (plan->n != B->N || plan->grids < 1 || plan->grids > 2 || mas_order < 0 || mas_order > 8) return GBP_ERR_INVALID;
  const int N = plan->n, P = plan->pitch, G = plan->grids;
  cufftHandle h;
  size_t w = 0;
  int r = c2r_plan(N, P, 1, &h, &w);
  if (r) return r;
  const long long total = (long long)N * N * P;
  const size_t need = align256((size_t)G * total * sizeof(float2)) + align256(w > 0 ? w : 1);
  if (!workspace || ws_bytes < need) return GBP_ERR_WORKSPACE;
  // The adjoint spectrum first, then a work area of its own (256 bytes when
  // the plan needs none): cuFFT fails to execute with a work area that
  // starts at its input.
  Carver cv(workspace);
  float2* hspec = cv.take<float2>((size_t)G * total);
  void* cws = cv.take<char>(w > 0 ? w : 1);
  {
    GBP_TRACE("grad_spectrum", st);
    grad_spec_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
        static_cast<const float2*>(spectrum), hspec, N, P, G, B->d_thr, B->nbe, B->nb, B->last_closed,
        B->d_inv_sinc2, B->d_eph, mas_order, grad_pk, nmodes, mass, box_size);
    GBP_LAUNCH_CHECK();
  }
  GBP_TRACE("grad_c2r", st);
  for (int g = 0; g < G; ++g) {
    r = c2r_exec(N, P, 1, hspec + g * total, grad_mesh + (long long)g * N * N * N, cws, st);
    if (r) return r;
  }
  return GBP_OK;
}

extern "C" int gbp_deposit_backward(const float* x, const float* y, const float* z, const float* w, int64_t n,
                                    float xmin, float ymin, float zmin, float inv_cell, int N, int mas, int interlace,
                                    const float* grad_mesh, float* grad_x, float* grad_y, float* grad_z,
                                    float* grad_w, gbp_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (n < 0 || N < 1 || mas < GBP_NGP || mas > GBP_PCS || !grad_mesh || !grad_x || !grad_y || !grad_z)
    return GBP_ERR_INVALID;
  if (n == 0) return GBP_OK;
  if (!x || !y || !z) return GBP_ERR_INVALID;
  const int G = interlace ? 2 : 1;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  GBP_TRACE("grad_gather", st);
  switch (mas) {
    case GBP_NGP:
      deposit_gather_kernel<GBP_NGP><<<blocks, 256, 0, st>>>(x, y, z, w, n, xmin, ymin, zmin, inv_cell, N, G,
                                                             grad_mesh, grad_x, grad_y, grad_z, grad_w);
      break;
    case GBP_CIC:
      deposit_gather_kernel<GBP_CIC><<<blocks, 256, 0, st>>>(x, y, z, w, n, xmin, ymin, zmin, inv_cell, N, G,
                                                             grad_mesh, grad_x, grad_y, grad_z, grad_w);
      break;
    case GBP_TSC:
      deposit_gather_kernel<GBP_TSC><<<blocks, 256, 0, st>>>(x, y, z, w, n, xmin, ymin, zmin, inv_cell, N, G,
                                                             grad_mesh, grad_x, grad_y, grad_z, grad_w);
      break;
    default:
      deposit_gather_kernel<GBP_PCS><<<blocks, 256, 0, st>>>(x, y, z, w, n, xmin, ymin, zmin, inv_cell, N, G,
                                                             grad_mesh, grad_x, grad_y, grad_z, grad_w);
  }
  GBP_LAUNCH_CHECK();
  return GBP_OK;
}
