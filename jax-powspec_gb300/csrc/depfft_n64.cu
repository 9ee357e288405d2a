// The fused particles -> multipole sums path for 64^3 meshes (depfft_impl.cuh).
#include "depfft_impl.cuh"

GBP_DEPFFT_INSTANCE(64)
