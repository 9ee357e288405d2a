// Internal layout of a gbp_bins plan (see gbp_bins_create in api.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbpowspec.h"

struct gbp_bins_s {
  int N;            // mesh side
  int nb;           // number of bins (n_edges - 1)
  int nbe;          // bins some mode can reach (>= 1)
  int lut_shift;    // lut[k2 >> lut_shift] = #thresholds <= (k2 >> shift) << shift
  int lut_n;
  int32_t last_closed;
  int device;
  int* d_thr;           // [nbe + 1]
  int* d_lut;           // [lut_n]
  float* d_inv_sinc2;   // [N/2 + 1]  1 / sinc(pi k / N)^2
  float2* d_eph;        // [N/2 + 1]  exp(i pi k / N)
  long long* d_nmodes;  // [nb] modes per bin (geometry only, computed once)
  double* d_ksum;       // [nb] sum of |k| per bin, grid units
  void* d_block;        // the single device allocation holding the above
};
