// Internal helpers shared by the gbpowspec CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "gbpowspec.h"

#define GBP_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t e_ = (expr);                                 \
    if (e_ != cudaSuccess) { gbp::set_last_cuda_error(e_); return GBP_ERR_CUDA; } \
  } while (0)

#define GBP_LAUNCH_CHECK()                                   \
  do {                                                       \
    cudaError_t e_ = cudaGetLastError();                     \
    if (e_ != cudaSuccess) { gbp::set_last_cuda_error(e_); return GBP_ERR_CUDA; } \
  } while (0)

#define GBP_TRACE(name, stream) gbp::TraceScope gbp_trace_scope_(name, stream)

namespace gbp {

void set_last_cuda_error(cudaError_t e);
void set_last_cufft_error(int code);   // a cufftResult, reported by gbp_strerror(GBP_ERR_CUFFT)

// Evaluates a cuFFT call; on failure records its result and returns GBP_ERR_CUFFT.
#define GBP_CUFFT_TRY(expr)                                  \
  do {                                                       \
    const int r_ = (int)(expr);                              \
    if (r_ != 0) { gbp::set_last_cufft_error(r_); return GBP_ERR_CUFFT; } \
  } while (0)

// Records CUDA events around the launches in its scope while tracing is on
// (gbp_trace_enable); `name` must be a string literal.
class TraceScope {
 public:
  TraceScope(const char* name, cudaStream_t s);
  ~TraceScope();
  TraceScope(const TraceScope&) = delete;
  TraceScope& operator=(const TraceScope&) = delete;

 private:
  int slot_;
  cudaStream_t s_;
};

// Programmatic dependent launch.  A kernel launched with launch_pdl is
// set up while the kernel before it in the stream finishes (its launch
// latency hides behind that kernel's last blocks); it must call pdl_wait()
// before it touches global memory, which returns once the previous kernel
// has completed and its writes are visible.  Launched the ordinary way,
// pdl_wait() is a no-op.  No kernel triggers its dependents early
// (griddepcontrol.launch_dependents): blocks waiting from the start hold SM
// slots, which cost 3 % on 128^3 batch lanes where the implicit trigger at
// completion gains 3 % (one mock at a time: 2 % at 128^3, 1 % at 512^3).
// GBP_PDL=0 in the environment turns the attribute off.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool pdl_enabled() {
  static const bool on = [] {
    const char* e = getenv("GBP_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Bytes rounded up to a multiple of 256 (keeps every workspace slice aligned).
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Carve consecutive 256-byte-aligned slices out of a caller workspace.
struct Carver {
  char* base;
  size_t used = 0;
  explicit Carver(void* p) : base(static_cast<char*>(p)) {}
  template <class T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base ? base + used : nullptr);
    used += align256(count * sizeof(T));
    return p;
  }
};

__host__ __device__ inline int pmod(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

// pmod for an index that is usually in [0, n) already: one compare on that
// path instead of an integer division.
__host__ __device__ inline int wrap_index(int a, int n) { return (unsigned)a < (unsigned)n ? a : pmod(a, n); }

// Signed wavenumber of FFT index i on an n-point axis, as the reference
// builds it: ki = i if i <= n/2 else i - n (src/correlations.py:25).
__host__ __device__ inline int signed_k(int i, int n) { return i > n / 2 ? i - n : i; }

// ---- float-float ("double-single") arithmetic ----------------------------
// GB300 runs FP64 at a small fraction of its FP32 rate, so wide reductions
// keep a (hi, lo) pair of floats and combine them with error-free sums
// (Knuth TwoSum); only the final per-bin totals are converted to double.
struct ff { float hi, lo; };

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s = __fadd_rn(a.hi, b.hi);
  float v = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  float hi = __fadd_rn(s, e);
  float lo = __fsub_rn(e, __fsub_rn(hi, s));
  return {hi, lo};
}

__device__ __forceinline__ ff ff_add_f(ff a, float b) { return ff_add(a, ff{b, 0.0f}); }

}  // namespace gbp
