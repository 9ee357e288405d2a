// The fused particles -> multipole sums path for 256^3 meshes (depfft_impl.cuh).
#include "depfft_impl.cuh"

GBP_DEPFFT_INSTANCE(256)
