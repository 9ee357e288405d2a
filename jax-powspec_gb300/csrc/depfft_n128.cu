// The fused particles -> multipole sums path for 128^3 meshes (depfft_impl.cuh).
#include "depfft_impl.cuh"

GBP_DEPFFT_INSTANCE(128)
