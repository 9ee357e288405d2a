// Lanes: resident single-mock pipelines that batching and serving run on.
//
// A lane owns every buffer one mock needs (meshes, spectra, the deposit,
// FFT and binning workspaces, per-mock sums), an FFT plan, and a CUDA graph
// of the whole launch sequence:
//
//   lane_begin    copies job table[cursor] into the lane's job slot
//   P_l sums      gbp_particles_power_job (reads the slot: particles, n,
//                 box): deposit fused with the z pass, y pass, x pass fused
//                 with the binning; or, when the plan uses cuFFT,
//                 gbp_deposit_job + gbp_fft_r2c + gbp_power
//   normalise     gbp_power_normalize_job (box from the slot)
//   lane_end      copies P_l, <k>, counts and deposit statistics to the
//                 caller's per-job arrays at `cursor`, then cursor += stride
//
// The graph holds no per-mock value: everything that changes from mock to
// mock lives in device memory (the job table, the cursor), so one captured
// graph is replayed for every mock of a batch with one cudaGraphLaunch each.
// Kernel launch sizes depend only on the lane's capacity, mesh and bins.
//
// A batch splits its jobs round-robin over several lanes, each on its own
// stream forked from (and joined back into) the caller's stream, so the
// compute-bound deposit of one mock overlaps the bandwidth-bound FFT and
// binning of another, and small meshes fill the GPU together.
#include <new>

#include "gbp_bins.h"
#include "gbp_internal.cuh"

struct LaneDesc {              // device-resident batch state of one lane
  const gbp_job* jobs;
  int n_jobs;
  int next;                    // job the next launch processes
  int stride;
  int active;                  // set by lane_begin: next < n_jobs
  gbp_lane_out out;
};

struct gbp_lane_s {
  int device = 0;
  int N = 0, mas = 0, G = 1, ells = 0, shot = 1, nb = 0, flags = 0;
  long long cap = 0;
  gbp_bins bins = nullptr;      // borrowed
  gbp_fft_plan plan = nullptr;  // owned
  int pitch = 0;
  bool particles = false;       // fused particles -> sums call (library transform sizes)
  size_t dep_ws = 0, fft_ws = 0, pow_ws = 0, bytes = 0;
  char* block = nullptr;        // the lane's single device allocation
  float* mesh = nullptr;
  float2* spec = nullptr;
  void* dws = nullptr;
  void* fws = nullptr;
  void* pws = nullptr;
  double* sums = nullptr;
  long long* nmodes = nullptr;
  double* ksum = nullptr;
  double* pk = nullptr;
  double* kmean = nullptr;
  gbp_deposit_stats* stats = nullptr;
  gbp_job* slot = nullptr;
  LaneDesc* desc = nullptr;
  cudaStream_t stream = nullptr;  // the lane's own stream (batches)
  cudaEvent_t fork = nullptr, done = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace gbp {
namespace {

__global__ void lane_set_desc(LaneDesc* d, LaneDesc v) { *d = v; }

__global__ void lane_begin(LaneDesc* d, gbp_job* slot) {
  pdl_wait();
  const int idx = d->next;
  const bool active = idx >= 0 && idx < d->n_jobs;
  static_assert(sizeof(gbp_job) % 4 == 0, "job copied as 32-bit words");
  constexpr int W = sizeof(gbp_job) / 4;
  unsigned* dst = reinterpret_cast<unsigned*>(slot);
  if (active) {
    const unsigned* src = reinterpret_cast<const unsigned*>(d->jobs + idx);
    if (threadIdx.x < W) dst[threadIdx.x] = src[threadIdx.x];
  } else if (threadIdx.x < W) {
    dst[threadIdx.x] = 0u;      // an empty job: nothing is deposited
  }
  if (threadIdx.x == 0) d->active = active ? 1 : 0;
}

__global__ void lane_end(LaneDesc* d, int nb, const double* pk, const double* kmean, const long long* nmodes,
                         const gbp_deposit_stats* stats) {
  pdl_wait();
  const int idx = d->next;
  if (d->active) {
    const gbp_lane_out o = d->out;
    for (int i = threadIdx.x; i < 3 * nb; i += blockDim.x)
      if (o.pk) o.pk[(long long)idx * 3 * nb + i] = pk[i];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      if (o.kmean) o.kmean[(long long)idx * nb + i] = kmean ? kmean[i] : 0.0;
      if (o.nmodes) o.nmodes[(long long)idx * nb + i] = nmodes[i];
    }
    if (o.stats && threadIdx.x == 0) o.stats[idx] = *stats;
  }
  __syncthreads();
  if (threadIdx.x == 0) d->next = idx + d->stride;
}

struct LaneSizes {
  size_t mesh, spec, dep, fft, pow, small, total;
  int pitch;
  bool particles;   // the fused particles -> sums call serves this shape
};

int lane_sizes(int N, int mas, int interlace, int ells, gbp_bins bins, long long cap, gbp_fft_plan plan,
               LaneSizes& s) {
  const int G = interlace ? 2 : 1;
  int st = gbp_fft_plan_pitch(plan, &s.pitch);
  if (st) return st;
  s.particles = gbp_particles_power_workspace_size(cap, plan, bins, mas, ells, &s.pow) == GBP_OK;
  if (s.particles) {            // one fused call: no mesh, one workspace
    s.mesh = 0;
    s.dep = 0;
    s.fft = 0;
  } else {
    st = gbp_deposit_workspace_size(cap, N, mas, interlace, GBP_COMPAT_NONE, &s.dep);
    if (st) return st;
    st = gbp_power_workspace_size(bins, G, s.pitch, ells, &s.pow);
    if (st) return st;
    s.mesh = align256((size_t)G * N * N * N * sizeof(float));
  }
  s.spec = align256((size_t)G * N * N * s.pitch * sizeof(float2));
  const size_t nb = (size_t)bins->nb;
  s.small = align256(nb * 3 * 8) * 2 + align256(nb * 8) * 3 + align256(sizeof(gbp_deposit_stats)) +
            align256(sizeof(gbp_job)) + align256(sizeof(LaneDesc));
  s.total = s.mesh + s.spec + align256(s.dep) + align256(s.fft) + align256(s.pow) + s.small;
  return GBP_OK;
}

// The launch sequence of one mock (captured into the graph, or run eagerly).
int lane_sequence(gbp_lane L, cudaStream_t st) {
  {
    GBP_TRACE("lane_begin", st);
    lane_begin<<<1, 32, 0, st>>>(L->desc, L->slot);
    GBP_LAUNCH_CHECK();
  }
  const gbp_stream_t s = reinterpret_cast<gbp_stream_t>(st);
  const double* mass = reinterpret_cast<const double*>(L->stats);   // gbp_deposit_stats starts with mass[2]
  double* ksum = (L->ells & GBP_KSUM) ? L->ksum : nullptr;
  int r;
  if (L->particles) {
    r = gbp_particles_power_job(L->slot, L->cap, L->plan, L->bins, L->mas, L->ells, L->spec, L->sums, L->nmodes,
                                ksum, L->stats, L->pws, L->pow_ws, s);
    if (r) return r;
  } else {
    r = gbp_deposit_job(L->slot, L->cap, L->N, L->mas, L->G == 2, L->mesh, L->stats, L->dws, L->dep_ws, s);
    if (r) return r;
    r = gbp_fft_r2c(L->plan, L->mesh, L->spec, L->fws, L->fft_ws, s);
    if (r) return r;
    r = gbp_power(L->spec, L->G, L->pitch, L->bins, L->mas, L->ells, mass, L->sums, L->nmodes, ksum, L->pws,
                  L->pow_ws, s);
    if (r) return r;
  }
  r = gbp_power_normalize_job(L->sums, L->nmodes, ksum, L->nb, L->N, L->slot, mass, L->stats, L->shot, L->pk,
                              (L->ells & GBP_KSUM) ? L->kmean : nullptr, s);
  if (r) return r;
  GBP_TRACE("lane_end", st);
  GBP_CUDA_TRY(launch_pdl(lane_end, dim3(1), dim3(256), 0, st, L->desc, L->nb, L->pk,
                          (L->ells & GBP_KSUM) ? L->kmean : nullptr, L->nmodes, L->stats));
  return GBP_OK;
}

int lane_capture(gbp_lane L) {
  cudaGraph_t graph = nullptr;
  GBP_CUDA_TRY(cudaStreamBeginCapture(L->stream, cudaStreamCaptureModeRelaxed));
  const int r = lane_sequence(L, L->stream);
  const cudaError_t e = cudaStreamEndCapture(L->stream, &graph);
  if (r) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return GBP_ERR_CUDA;
  }
  const cudaError_t ie = cudaGraphInstantiate(&L->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    set_last_cuda_error(ie);
    L->exec = nullptr;
    return GBP_ERR_CUDA;
  }
  return GBP_OK;
}

void lane_free(gbp_lane L) {
  if (!L) return;
  if (L->exec) cudaGraphExecDestroy(L->exec);
  if (L->fork) cudaEventDestroy(L->fork);
  if (L->done) cudaEventDestroy(L->done);
  if (L->stream) cudaStreamDestroy(L->stream);
  if (L->block) cudaFree(L->block);
  if (L->plan) gbp_fft_plan_destroy(L->plan);
  delete L;
}

int launch_one(gbp_lane L, cudaStream_t st) {
  if (L->exec) {
    GBP_CUDA_TRY(cudaGraphLaunch(L->exec, st));
    return GBP_OK;
  }
  return lane_sequence(L, st);
}

int set_desc(gbp_lane L, const gbp_job* jobs, int n_jobs, int first, int stride, const gbp_lane_out* out,
             cudaStream_t st) {
  LaneDesc v{};
  v.jobs = jobs;
  v.n_jobs = n_jobs;
  v.next = first;
  v.stride = stride;
  v.active = 0;
  if (out) v.out = *out;
  lane_set_desc<<<1, 1, 0, st>>>(L->desc, v);
  GBP_LAUNCH_CHECK();
  return GBP_OK;
}

bool lane_args_ok(int N, int mas, int interlace, int ells, gbp_bins bins, long long cap) {
  if (!bins || bins->N != N) return false;
  if (mas < GBP_NGP || mas > GBP_PCS || cap < 1) return false;
  if (interlace != 0 && interlace != 1) return false;
  if ((ells & (GBP_ELL0 | GBP_ELL2 | GBP_ELL4)) == 0 || (ells & ~15)) return false;
  return true;
}

}  // namespace
}  // namespace gbp

using namespace gbp;

extern "C" int gbp_lane_bytes(int N, int mas, int interlace, int ells, gbp_bins bins, int64_t capacity,
                              size_t* bytes) {
  if (!bytes || !lane_args_ok(N, mas, interlace, ells, bins, capacity)) return GBP_ERR_INVALID;
  gbp_fft_plan plan = nullptr;
  size_t fft_ws = 0;
  int st = gbp_fft_plan_create(N, interlace ? 2 : 1, &plan, &fft_ws);
  if (st) return st;
  LaneSizes s{};
  s.fft = fft_ws;
  st = lane_sizes(N, mas, interlace, ells, bins, capacity, plan, s);
  gbp_fft_plan_destroy(plan);
  if (st) return st;
  *bytes = s.total;
  return GBP_OK;
}

extern "C" int gbp_lane_create(int N, int mas, int interlace, int ells, int shot_noise, gbp_bins bins,
                               int64_t capacity, int flags, gbp_lane* out) {
  if (!out || !lane_args_ok(N, mas, interlace, ells, bins, capacity)) return GBP_ERR_INVALID;
  *out = nullptr;
  gbp_lane L = new (std::nothrow) gbp_lane_s();
  if (!L) return GBP_ERR_ALLOC;
  L->N = N; L->mas = mas; L->G = interlace ? 2 : 1; L->ells = ells; L->shot = shot_noise ? 1 : 0;
  L->nb = bins->nb; L->cap = capacity; L->bins = bins; L->flags = flags;
  cudaGetDevice(&L->device);
  int st = gbp_fft_plan_create(N, L->G, &L->plan, &L->fft_ws);
  if (st) { lane_free(L); return st; }
  if (flags & GBP_LANE_TILES(15, 15)) {
    st = gbp_fft_plan_set_tiles(L->plan, (flags >> 8) & 15, (flags >> 12) & 15);
    if (st) { lane_free(L); return st; }
  }
  LaneSizes s{};
  s.fft = L->fft_ws;
  st = lane_sizes(N, mas, interlace, ells, bins, capacity, L->plan, s);
  if (st) { lane_free(L); return st; }
  L->pitch = s.pitch;
  L->particles = s.particles;
  L->dep_ws = s.dep;
  L->pow_ws = s.pow;
  L->bytes = s.total;
  if (cudaMalloc(&L->block, s.total) != cudaSuccess) {
    cudaGetLastError();
    lane_free(L);
    return GBP_ERR_ALLOC;
  }
  Carver cv(L->block);
  const size_t nb = (size_t)L->nb;
  L->mesh = cv.take<float>(s.mesh / sizeof(float));
  L->spec = cv.take<float2>(s.spec / sizeof(float2));
  L->dws = cv.take<char>(s.dep);
  L->fws = cv.take<char>(s.fft);
  L->pws = cv.take<char>(s.pow);
  L->sums = cv.take<double>(nb * 3);
  L->pk = cv.take<double>(nb * 3);
  L->nmodes = cv.take<long long>(nb);
  L->ksum = cv.take<double>(nb);
  L->kmean = cv.take<double>(nb);
  L->stats = cv.take<gbp_deposit_stats>(1);
  L->slot = cv.take<gbp_job>(1);
  L->desc = cv.take<LaneDesc>(1);
  if (cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&L->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    lane_free(L);
    return GBP_ERR_CUDA;
  }
  // an idle descriptor: a launch before the first bind processes no job
  st = set_desc(L, nullptr, 0, 0, 1, nullptr, L->stream);
  if (!st && (flags & GBP_LANE_GRAPH)) st = lane_capture(L);
  if (!st && cudaStreamSynchronize(L->stream) != cudaSuccess) st = GBP_ERR_CUDA;
  if (st) { lane_free(L); return st; }
  *out = L;
  return GBP_OK;
}

extern "C" int gbp_lane_info(gbp_lane L, size_t* bytes, int* n_bins, int* graph) {
  if (!L) return GBP_ERR_INVALID;
  if (bytes) *bytes = L->bytes;
  if (n_bins) *n_bins = L->nb;
  if (graph) *graph = L->exec != nullptr;
  return GBP_OK;
}

extern "C" int gbp_lane_destroy(gbp_lane L) {
  if (!L) return GBP_ERR_INVALID;
  cudaStreamSynchronize(L->stream);
  lane_free(L);
  return GBP_OK;
}

extern "C" int gbp_lane_run(gbp_lane L, const gbp_job* jobs, int n_jobs, int first, int stride,
                            const gbp_lane_out* out, gbp_stream_t stream_) {
  if (!L || !jobs || n_jobs < 0 || first < 0 || stride < 1 || !out) return GBP_ERR_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  int r = set_desc(L, jobs, n_jobs, first, stride, out, st);
  for (int j = first; !r && j < n_jobs; j += stride) r = launch_one(L, st);
  return r;
}

extern "C" int gbp_batch_run(gbp_lane* lanes, int n_lanes, const gbp_job* jobs, int n_jobs,
                             const gbp_lane_out* out, gbp_stream_t stream_) {
  if (!lanes || n_lanes < 1 || !jobs || n_jobs < 0 || !out) return GBP_ERR_INVALID;
  for (int l = 0; l < n_lanes; ++l) {
    if (!lanes[l]) return GBP_ERR_INVALID;
    for (int m = 0; m < l; ++m)
      if (lanes[m] == lanes[l]) return GBP_ERR_INVALID;   // a lane's buffers serve one job at a time
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  const int used = n_lanes < n_jobs ? n_lanes : n_jobs;
  // fork: every lane stream waits for the work already on the caller's stream
  for (int l = 0; l < used; ++l) {
    gbp_lane L = lanes[l];
    GBP_CUDA_TRY(cudaEventRecord(L->fork, st));
    GBP_CUDA_TRY(cudaStreamWaitEvent(L->stream, L->fork, 0));
    const int r = set_desc(L, jobs, n_jobs, l, used, out, L->stream);
    if (r) return r;
  }
  // round-robin issue keeps every lane's queue fed
  for (int j0 = 0; j0 < n_jobs; j0 += used)
    for (int l = 0; l < used && j0 + l < n_jobs; ++l) {
      const int r = launch_one(lanes[l], lanes[l]->stream);
      if (r) return r;
    }
  // join: the caller's stream waits for every lane
  for (int l = 0; l < used; ++l) {
    GBP_CUDA_TRY(cudaEventRecord(lanes[l]->done, lanes[l]->stream));
    GBP_CUDA_TRY(cudaStreamWaitEvent(st, lanes[l]->done, 0));
  }
  return GBP_OK;
}
