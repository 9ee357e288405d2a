/*
 * gbpowspec.h -- C ABI of libgbpowspec.so, the GB300 power-spectrum engine.
 *
 * The library replaces the particle -> mesh -> P_l(k) path of jax-powspec
 * (dforero0896/jax-powspec).  Each entry point below names the reference
 * function it stands in for (path within the reference project, file:line).
 *
 * Conventions shared by every call
 *   - All array arguments are DEVICE pointers owned by the caller; the library
 *     never frees them.  Scratch memory is passed in as (workspace, bytes);
 *     the matching *_workspace_size call says how much is needed.
 *   - Every call is asynchronous on the given stream and returns GBP_OK (0)
 *     or a negative status; gbp_strerror() turns it into text.  Argument
 *     errors are detected on the host before anything is launched.
 *   - Meshes are float32, C order [x][y][z] (z fastest), side n_mesh.
 *     Interlaced deposits write two meshes back to back: grid 0 at mesh_out,
 *     grid 1 (particles shifted by +half a cell on every axis) at
 *     mesh_out + n_mesh^3.
 *   - Spectra are complex64 [x][y][z]: n_mesh/2+1 modes along z in rows of
 *     z_pitch entries (see gbp_fft_plan_pitch), one grid after the other.
 *   - Results are deterministic: the same inputs give bitwise-identical
 *     outputs on every run, whatever else shares the GPU.
 */
#ifndef GBPOWSPEC_H
#define GBPOWSPEC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without pulling in the CUDA headers. */
typedef struct CUstream_st* gbp_stream_t;

/* status codes */
#define GBP_OK                 0
#define GBP_ERR_INVALID       -1  /* bad argument (detected on the host) */
#define GBP_ERR_CUDA          -2  /* a CUDA runtime call failed */
#define GBP_ERR_CUFFT         -3  /* a cuFFT call failed */
#define GBP_ERR_WORKSPACE     -4  /* workspace smaller than *_workspace_size */
#define GBP_ERR_UNSUPPORTED   -5  /* valid request outside what this build supports */
#define GBP_ERR_ALLOC         -6  /* the library could not allocate plan memory */

/* mass-assignment schemes (B-spline order) */
#define GBP_NGP 1
#define GBP_CIC 2
#define GBP_TSC 3
#define GBP_PCS 4

/* deposit semantics */
#define GBP_COMPAT_NONE    0  /* periodic B-spline deposit (mass conserving)        */
#define GBP_COMPAT_VEC     1  /* exactly src/mas.py cic_mas_vec, bugs included      */
#define GBP_COMPAT_SCAN    2  /* exactly src/mas.py cic_mas, bugs included          */

/* multipole selection for gbp_power */
#define GBP_ELL0   1
#define GBP_ELL2   2
#define GBP_ELL4   4
#define GBP_KSUM   8   /* also accumulate sum of |k| per bin (mode-averaged k) */

const char* gbp_strerror(int status);
int gbp_version(void);

/* ------------------------------------------------------------------------
 * Deposit: particles -> density mesh(es).
 * Replaces src/mas.py:88-153 (cic_mas_vec) for compat == GBP_COMPAT_VEC and
 * src/mas.py:5-87 (cic_mas) for compat == GBP_COMPAT_SCAN; with
 * GBP_COMPAT_NONE it adds NGP/TSC/PCS and interlacing (no reference code).
 *
 *   x,y,z        float32[n] positions; w float32[n] weights or NULL (= 1).
 *   xmin,ymin,zmin  mesh origin; inv_cell = float32 (1 / (box/n_mesh)),
 *                computed by the caller exactly as src/mas.py:100-101 does.
 *   mas          GBP_NGP..GBP_PCS (compat modes require GBP_CIC).
 *   interlace    0/1: also deposit the half-cell-shifted grid.
 *   wrap         compat modes only: the reference's `wrap` flag.
 *   mesh_in      NULL, or float32 mesh(es) to which the deposit is added
 *                (src/mas.py returns delta + deposits).
 *   mesh_out     float32 [1+interlace][n_mesh^3]; fully overwritten.
 *   stats_out    NULL or device gbp_deposit_stats (written by the call).
 * Accumulation is exact fixed point (int64, scale 2^s chosen from n and
 * max|w|), so the result does not depend on particle order or scheduling.
 * ---------------------------------------------------------------------- */
typedef struct gbp_deposit_stats {
  double mass[2];       /* sum of the deposited mesh, per grid              */
  double sum_w;         /* sum of weights of the particles that were kept   */
  double sum_w2;        /* sum of squared weights (shot noise)              */
  long long n_kept;     /* particles that deposited at least one cell       */
  long long n_nonfinite;/* particles dropped for a non-finite coordinate    */
  int scale_exp;        /* fixed-point exponent s of the mass totals (the
                           mesh deposit accumulates at 2^s; the fused deposit
                           of gbp_particles_power at 2^(s - t) per tile, t >= 0
                           from the tile's occupancy, its totals shifted to 2^s) */
  int flags;            /* GBP_STATS_* bits below                           */
} gbp_deposit_stats;

/* flags bit: a tile's bucket outgrew the fixed capacity the one-pass
 * bucketing gives it (a strongly clustered catalogue), so the buckets were
 * rebuilt by a scan and a second scatter; the results are the same, the
 * call took longer. */
#define GBP_STATS_REFILLED 1

int gbp_deposit_workspace_size(int64_t n_particles, int n_mesh, int mas,
                               int interlace, int compat, size_t* bytes);

/* A mock described in DEVICE memory, so that a captured CUDA graph can be
 * replayed for a different mock by rewriting these bytes (no new graph):
 * particles, their count, and the box geometry.  inv_cell, xmin.. as for
 * gbp_deposit; box_size feeds gbp_power_normalize_job.  No reference
 * counterpart (the reference has no batching). */
typedef struct gbp_job {
  const float* x;
  const float* y;
  const float* z;
  const float* w;       /* NULL = unit weights */
  long long n;          /* <= the capacity the kernels were sized for */
  float inv_cell, xmin, ymin, zmin;
  double box_size;
} gbp_job;

/* gbp_deposit for a mock held in a device gbp_job (B-spline schemes only,
 * compat = GBP_COMPAT_NONE).  Launch sizes and the workspace
 * (gbp_deposit_workspace_size(capacity, ...)) depend only on `capacity`,
 * never on job->n; particles past `capacity` are not deposited (n_kept in
 * the statistics says how many were). */
int gbp_deposit_job(const gbp_job* job, int64_t capacity, int n_mesh, int mas,
                    int interlace, float* mesh_out,
                    gbp_deposit_stats* stats_out, void* workspace,
                    size_t workspace_bytes, gbp_stream_t stream);

int gbp_deposit(const float* x, const float* y, const float* z, const float* w,
                int64_t n_particles, float xmin, float ymin, float zmin,
                float inv_cell, int n_mesh, int mas, int interlace, int compat,
                int wrap, const float* mesh_in, float* mesh_out,
                gbp_deposit_stats* stats_out, void* workspace,
                size_t workspace_bytes, gbp_stream_t stream);

/* ------------------------------------------------------------------------
 * FFT plans: 3-D real-to-complex transform of n_grids meshes of side n_mesh
 * (forward, unnormalised, as jnp.fft.rfftn).  Replaces the rfftn of
 * src/correlations.py:22.  Power-of-two meshes 64..1024 use the library's
 * own three-pass transform; other sizes a cuFFT plan.  The spectrum rows are
 * z_pitch complex apart (gbp_fft_plan_pitch: n/2+8 for the library's
 * transform, n/2+1 for cuFFT), the first n/2+1 of each row being the modes.
 * A cuFFT plan needs a work area (workspace_bytes); the library's needs none.
 * Buffers passed to gbp_fft_r2c must be 16-byte aligned.
 * ---------------------------------------------------------------------- */
typedef struct gbp_fft_plan_s* gbp_fft_plan;

int gbp_fft_plan_create(int n_mesh, int n_grids, gbp_fft_plan* plan,
                        size_t* workspace_bytes);
int gbp_fft_plan_pitch(gbp_fft_plan plan, int* z_pitch);
int gbp_fft_plan_destroy(gbp_fft_plan plan);
int gbp_fft_r2c(gbp_fft_plan plan, const float* mesh, void* spectrum,
                void* workspace, size_t workspace_bytes, gbp_stream_t stream);

/* ------------------------------------------------------------------------
 * Bin edges -> exact integer thresholds (host-only helper, no GPU).
 * kedges_grid[0..n_edges-1] are float32 bin edges in units of the
 * fundamental frequency, i.e. k_edges / kF computed in float32 as
 * src/correlations.py:12,42 does.  Mode (kx,ky,kz) with k2 = kx^2+ky^2+kz^2
 * falls in bin b (0 <= b < n_edges-1) iff
 *      thr[b] <= k2 < thr[b+1]               for b < n_edges-2,
 *      thr[b] <= k2 <= *thr_last_closed      for the last bin,
 * which is jnp.histogram (searchsorted right, last edge closed) applied to
 * k = sqrtf((float)k2), bit for bit.  thr has n_edges entries.
 * *n_reach = number of bins some mode of an n_mesh^3 grid can fall in.
 * Returns GBP_ERR_INVALID for decreasing or non-finite edges.
 * ---------------------------------------------------------------------- */
int gbp_bin_thresholds(const float* kedges_grid, int n_edges, int n_mesh,
                       int32_t* thr, int32_t* thr_last_closed, int* n_reach);

/* ------------------------------------------------------------------------
 * Bin plans: thresholds, their lookup table and the per-axis window and
 * interlacing-phase tables for one (edges, n_mesh), uploaded once to the
 * current device (the plan owns that memory; gbp_bins_destroy frees it).
 * kedges_grid is a HOST array, as for gbp_bin_thresholds.
 * ---------------------------------------------------------------------- */
typedef struct gbp_bins_s* gbp_bins;

int gbp_bins_create(const float* kedges_grid, int n_edges, int n_mesh,
                    gbp_bins* bins);
int gbp_bins_destroy(gbp_bins bins);
int gbp_bins_info(gbp_bins bins, int* n_bins, int* n_reach,
                  int32_t* thr_last_closed);

/* ------------------------------------------------------------------------
 * Power multipoles: fused window deconvolution, interlacing combination,
 * |delta_k|^2 x L_l(mu) (line of sight = z) and k-shell binning.
 * Replaces src/correlations.py:20-48 (the body of powspec_vec).
 *
 *   spectrum     complex64 [n_grids][n_mesh][n_mesh][z_pitch]; the first
 *                n_mesh/2+1 entries of each z row are the modes.
 *   z_pitch      complex entries per z row (>= n_mesh/2+1; 0 means n_mesh/2+1).
 *   n_grids      1, or 2 for an interlaced pair: the modes are combined as
 *                (F0 + F1 exp(i pi (kx+ky+kz)/n_mesh)) / 2.
 *   mas_order    window: each axis is divided by sinc(pi k_i/n)^mas_order
 *                (0 = no deconvolution; src/correlations.py:20-21,32 uses 2).
 *   ells         GBP_ELL0|GBP_ELL2|GBP_ELL4 [| GBP_KSUM].
 *   mass         NULL, or device double[n_grids]: the mesh totals.  Then the
 *                k=0 mode is taken as (F(0) - mass), so a raw density mesh
 *                gives the spectrum of delta = rho/mean - 1 up to the factor
 *                that gbp_power_normalize applies.
 *   sums_out     double[n_bins][3]: sum over modes of |d|^2 W^2 L_l(mu)
 *                for l = 0,2,4 (zero where not requested).
 *   nmodes_out   int64[n_bins] mode counts (half-space grid cells, as
 *                src/correlations.py:48 counts them).
 *   ksum_out     double[n_bins] sum of |k| in grid units (GBP_KSUM), or NULL.
 * ---------------------------------------------------------------------- */
int gbp_power_workspace_size(gbp_bins bins, int n_grids, int z_pitch, int ells,
                             size_t* bytes);

int gbp_power(const void* spectrum, int n_grids, int z_pitch, gbp_bins bins,
              int mas_order, int ells, const double* mass, double* sums_out,
              long long* nmodes_out, double* ksum_out, void* workspace,
              size_t workspace_bytes, gbp_stream_t stream);

/* ------------------------------------------------------------------------
 * gbp_power without a workspace argument: the same result, with its scratch
 * held in a fixed 16 MiB device array inside the library, for callers that
 * cannot allocate device memory when they call in (a JAX/XLA custom call gets
 * only its operand and result buffers, and its device memory belongs to
 * JAX's allocator, which reserves most of the GPU up front).  This entry
 * point has no counterpart in the reference.
 * Limit: (work groups) x (moments) x (bins) <= 2^21 float2, which holds any
 * 512^3 mesh with up to ~560 bins of l = 0,2,4; larger requests return
 * GBP_ERR_UNSUPPORTED without launching.  The first call on a device looks up
 * the array's address with that device current: make it before any stream
 * capture.  Calls share the array, so calls that overlap on the GPU race.
 * ---------------------------------------------------------------------- */
int gbp_power_noalloc(const void* spectrum, int n_grids, int z_pitch,
                      gbp_bins bins, int mas_order, int ells,
                      const double* mass, double* sums_out,
                      long long* nmodes_out, double* ksum_out,
                      gbp_stream_t stream);

/* ------------------------------------------------------------------------
 * Normalisation of gbp_power's sums into P_l(k), on the device.
 * Replaces src/correlations.py:49-54 (and the caller-side shot-noise
 * subtraction of tests/correlations.py:36,83).
 *   P_l[b] = (2l+1) * sums[b][l] / nmodes[b] * norm  - shot*(l==0)
 *   norm   = (box/n^2)^3            when mass == NULL (delta given)
 *          = box^3 / mass[0]^2      when mass != NULL (raw density mesh)
 *   shot   = box^3 * sum_w2 / mass[0]^2 when subtract_shot and stats given.
 *   kmean[b] = ksum[b] / nmodes[b] * 2 pi / box   (when ksum != NULL)
 * Empty bins give NaN, as in the reference (0/0).
 * ---------------------------------------------------------------------- */
int gbp_power_normalize(const double* sums, const long long* nmodes,
                        const double* ksum, int n_bins, int n_mesh,
                        double box_size, const double* mass,
                        const gbp_deposit_stats* stats, int subtract_shot,
                        double* pk_out, double* kmean_out,
                        gbp_stream_t stream);

/* gbp_power_normalize with the box size read from a device gbp_job. */
int gbp_power_normalize_job(const double* sums, const long long* nmodes,
                            const double* ksum, int n_bins, int n_mesh,
                            const gbp_job* job, const double* mass,
                            const gbp_deposit_stats* stats, int subtract_shot,
                            double* pk_out, double* kmean_out,
                            gbp_stream_t stream);

/* The 3-D FFT fused with the binning (library transform sizes only: power-of
 * two meshes 64..1024 and a plan made without the cuFFT override).  The z and
 * y passes write the partial transform to `spectrum` (the buffer
 * gbp_fft_r2c would fill); the x pass runs inside the binning kernel, so the
 * full spectrum never reaches HBM.  Same outputs and arguments as
 * gbp_fft_r2c followed by gbp_power (src/correlations.py:22-48); the sums
 * agree to float32 round-off (a different, fixed summation order).
 * GBP_ERR_UNSUPPORTED when the plan uses cuFFT. */
int gbp_fft_power_workspace_size(gbp_fft_plan plan, gbp_bins bins, int ells,
                                 size_t* bytes);
int gbp_fft_power(gbp_fft_plan plan, const float* mesh, void* spectrum,
                  gbp_bins bins, int mas_order, int ells, const double* mass,
                  double* sums_out, long long* nmodes_out, double* ksum_out,
                  void* workspace, size_t workspace_bytes,
                  gbp_stream_t stream);

/* Particles -> multipole sums in one call, the deposit fused with the z pass
 * of the FFT (library transform sizes: power-of-two meshes 64..1024 and a
 * plan made without the cuFFT override; B-spline deposits).  The mesh is
 * never written: each column tile of pencils is deposited in shared memory
 * (32-bit fixed point at a scale per 4x4-pencil block that no cell can
 * overflow, exact and order-independent; 64-bit cells for blocks of dense
 * clumps) and transformed along z there; then the y pass and the x pass
 * fused with the binning.  Interlacing follows the plan (2 grids =
 * interlaced); the column tile shape too (gbp_fft_plan_set_tiles).
 * Outputs as gbp_deposit (stats_out, required: it carries the mass the
 * binning and the normalisation use) followed by gbp_fft_power; `spectrum`
 * is scratch of the plan's spectrum size.  The particles are bucketed by
 * column tile in one pass into buckets of fixed capacity (twice the mean
 * fill of a uniform catalogue of n_particles, plus 64); a catalogue that
 * overflows one (a dense clump) is re-bucketed by a scan and a second pass
 * in the same call, same results, GBP_STATS_REFILLED in stats_out->flags.
 * Replaces src/mas.py:88-153 + src/correlations.py:7-56 for the production
 * path. */
int gbp_particles_power_workspace_size(int64_t n_particles, gbp_fft_plan plan,
                                       gbp_bins bins, int mas, int ells,
                                       size_t* bytes);
/* Column tile shapes (tx x ty pencils, all of z) of the fused path for an
 * n_mesh^3 mesh, the default first: up to `max` of them into tx[], ty[];
 * *count = how many there are (no reference counterpart: the tile is the
 * bucket of the particle sort, a tuning choice).  Every shape gives the same
 * results bit for bit; they differ in speed, which the autotuner measures. */
int gbp_column_tile_variants(int n_mesh, int* tx, int* ty, int max, int* count);
/* Tile shape of a plan's fused calls: one of gbp_column_tile_variants, or
 * 0, 0 for the default.  The workspace size depends on it: query after
 * setting. */
int gbp_fft_plan_set_tiles(gbp_fft_plan plan, int tx, int ty);
/* The shape in effect (the default resolved). */
int gbp_fft_plan_tiles(gbp_fft_plan plan, int* tx, int* ty);
int gbp_particles_power(const float* x, const float* y, const float* z,
                        const float* w, int64_t n_particles, float xmin,
                        float ymin, float zmin, float inv_cell,
                        gbp_fft_plan plan, gbp_bins bins, int mas, int ells,
                        void* spectrum, double* sums_out, long long* nmodes_out,
                        double* ksum_out, gbp_deposit_stats* stats_out,
                        void* workspace, size_t workspace_bytes,
                        gbp_stream_t stream);
/* The same for a mock held in a device gbp_job; launch sizes and the
 * workspace depend only on `capacity`. */
int gbp_particles_power_job(const gbp_job* job, int64_t capacity,
                            gbp_fft_plan plan, gbp_bins bins, int mas, int ells,
                            void* spectrum, double* sums_out,
                            long long* nmodes_out, double* ksum_out,
                            gbp_deposit_stats* stats_out, void* workspace,
                            size_t workspace_bytes, gbp_stream_t stream);

/* ---- Lognormal mock catalogues on the device (no reference counterpart;
 * the recipe of tests/create_lognormal.py:42-55, src/gauss_field.py:5-80,
 * src/populate_field.py:11-29 with the benchmark's choices): Gaussian field
 * on grid^3 with P_G(k) = A k exp(-(k/k_cut)^2), unit lattice variance,
 * rho = exp(g - 1/2), exactly n particles drawn with probability
 * proportional to rho, uniform in their cell, z shifted by N(0, sigma_v),
 * periodic.  Philox4x32-10 counter-based random numbers: the catalogue is a
 * pure function of the arguments.  grid even, 4..1024. */
int gbp_lognormal_workspace_size(int grid, size_t* bytes);
int gbp_lognormal(int grid, double box, double k_cut, double sigma_v,
                  int64_t n, unsigned long long seed, float* x, float* y,
                  float* z, void* workspace, size_t workspace_bytes,
                  gbp_stream_t stream);
/* The field behind gbp_lognormal's catalogue for the same (grid, box, k_cut,
 * seed), on the grid^3 lattice (x slowest, z fastest): g_out the Gaussian
 * field g (replaces src/gauss_field.py:5-80 gaussian_field, which returns the
 * field of a tabulated P(k)), rho_out = exp(g - 1/2) = 1 + delta_LN, the
 * density that gbp_lognormal samples its particles from.  Either pointer may
 * be NULL, not both.  Same workspace as gbp_lognormal. */
int gbp_lognormal_field(int grid, double box, double k_cut,
                        unsigned long long seed, float* g_out, float* rho_out,
                        void* workspace, size_t workspace_bytes,
                        gbp_stream_t stream);
/* Host evaluation of the generator's Philox4x32-10 block (known-answer
 * tests): out = philox(ctr[4], key[2]). */
int gbp_philox4x32_10(const unsigned* ctr, const unsigned* key, unsigned* out);

/* Two-point correlation multipoles from a density contrast mesh
 * (src/correlations.py:120-187 xi_vec; the xi half of :641-712
 * compute_2pt_correlations): forward R2C (plan with one grid), |delta_k|^2
 * times (sinc)^(-2 mas_order) per axis (the reference: mas_order 2), inverse
 * C2R into `field` (N^3 floats, unnormalised: N^3 xi), then shells of the
 * separation r on the full grid with the bin plan's thresholds (edges in
 * cell units, the jnp.histogram rule) and L_l(mu), mu = r_z / r.
 * sums_out [nb][3] = sum of field * L_l (double), counts_out [nb] cells per
 * bin; xi_l = (2l+1) sums / counts / N^6.  mu at r = 0 is NaN when
 * nan_mu_at_origin (xi_vec: 0/0) and 0 otherwise (compute_2pt). */
int gbp_xi_workspace_size(gbp_fft_plan plan, gbp_bins bins, size_t* bytes);
int gbp_xi(gbp_fft_plan plan, const float* delta, void* spectrum, float* field,
           gbp_bins bins, int mas_order, int nan_mu_at_origin,
           double* sums_out, long long* counts_out, void* workspace,
           size_t workspace_bytes, gbp_stream_t stream);

/* Bispectrum of a density contrast mesh (src/correlations.py:334-462
 * bispec): shells |k| in [k_i - kF, k_i + kF) around k_1, k_2 and every
 * k_3(theta), each a run of elementary bins of `bins` (edges in kF units:
 * the sorted shell limits); shell_bins [n_shells][2] (device) holds the
 * first and one-past-last elementary bin of shell s (s = 0: k_1, 1: k_2,
 * 2..: k_3).  Amplitude window sinc^(-mas_order) per axis (the reference:
 * 2).  Outputs (device, double): pk_out [n_shells] = P of every shell,
 * bk_out / qk_out [n_shells - 2] = B and the reduced Q per k_3, nmodes_out
 * [n_shells] (nullable) = modes per shell on the full grid.  The estimator
 * is the reference's (real-space sums of squares and triple products of
 * the shell-filtered fields); the sums are evaluated in Fourier space. */
int gbp_bispec_workspace_size(gbp_fft_plan plan, gbp_bins bins, size_t* bytes);
int gbp_bispec(gbp_fft_plan plan, const float* delta, void* spectrum,
               gbp_bins bins, int mas_order, const int32_t* shell_bins,
               int n_shells, double box_size, double* pk_out, double* bk_out,
               double* qk_out, long long* nmodes_out, void* workspace,
               size_t workspace_bytes, gbp_stream_t stream);

/* ---- Gradients (no C counterpart in the reference, which differentiates
 * its P(k) with JAX autodiff, tests/lognormal.py:60-103).
 * gbp_power_backward: given dLoss/dP_l per bin (grad_pk [nb][3], l = 0,2,4),
 * the spectra of the forward pass (gbp_fft_r2c output, the plan's grids:
 * 2 = interlaced), the bins' mode counts and the mesh mass (L^3/M^2
 * normalisation), writes dLoss/d(mesh cell) for every grid (grad_mesh
 * [G][N^3]).  gbp_deposit_backward: the adjoint of a B-spline deposit
 * (compat = GBP_COMPAT_NONE): gathers grad_mesh at each particle's stencil
 * nodes with the weights' derivatives: grad_x/y/z = dLoss/dposition, grad_w
 * (nullable) = dLoss/dweight through the mesh. */
int gbp_power_backward_workspace_size(gbp_fft_plan plan, size_t* bytes);
int gbp_power_backward(const void* spectrum, gbp_fft_plan plan, gbp_bins bins,
                       int mas_order, const double* grad_pk,
                       const long long* nmodes, const double* mass,
                       double box_size, float* grad_mesh, void* workspace,
                       size_t workspace_bytes, gbp_stream_t stream);
int gbp_deposit_backward(const float* x, const float* y, const float* z,
                         const float* w, int64_t n_particles, float xmin,
                         float ymin, float zmin, float inv_cell, int n_mesh,
                         int mas, int interlace, const float* grad_mesh,
                         float* grad_x, float* grad_y, float* grad_z,
                         float* grad_w, gbp_stream_t stream);

/* ---- Lanes: resident per-mock pipelines for batching and serving --------
 * No reference counterpart (the reference computes one mock per call).
 * A lane owns every buffer one mock needs and, with GBP_LANE_GRAPH, a CUDA
 * graph of the whole sequence (job slot <- table[cursor]; deposit; FFT;
 * binning; normalisation; outputs -> caller arrays at cursor; cursor +=
 * stride).  Jobs and outputs are addressed through device memory, so the
 * same graph is replayed for every mock.  A lane serves one job at a time:
 * calls on one lane must be ordered (same stream, or joined streams). */
typedef struct gbp_lane_s* gbp_lane;

#define GBP_LANE_GRAPH 1   /* capture the launch sequence into a CUDA graph */
/* Column tile of the lane's fused calls (gbp_fft_plan_set_tiles), or none
 * for the default: flags |= GBP_LANE_TILES(tx, ty). */
#define GBP_LANE_TILES(tx, ty) ((((tx) & 15) << 8) | (((ty) & 15) << 12))

/* Per-job outputs (device pointers, any may be NULL), indexed by job j:
 * pk[(j*nb + b)*3 + l] (l = 0,2,4 -> 0,1,2), kmean[j*nb + b],
 * nmodes[j*nb + b], stats[j]. */
typedef struct gbp_lane_out {
  double* pk;
  double* kmean;
  long long* nmodes;
  gbp_deposit_stats* stats;
} gbp_lane_out;

/* Device bytes a lane of this shape holds (for admission against a budget). */
int gbp_lane_bytes(int n_mesh, int mas, int interlace, int ells, gbp_bins bins,
                   int64_t capacity, size_t* bytes);
/* bins: borrowed, must outlive the lane; capacity: most particles per job. */
int gbp_lane_create(int n_mesh, int mas, int interlace, int ells,
                    int shot_noise, gbp_bins bins, int64_t capacity, int flags,
                    gbp_lane* lane);
int gbp_lane_info(gbp_lane lane, size_t* bytes, int* n_bins, int* graph);
int gbp_lane_destroy(gbp_lane lane);
/* Runs jobs first, first+stride, ... < n_jobs of the device table `jobs` on
 * `stream`, in order. */
int gbp_lane_run(gbp_lane lane, const gbp_job* jobs, int n_jobs, int first,
                 int stride, const gbp_lane_out* out, gbp_stream_t stream);
/* Splits n_jobs round-robin over n_lanes distinct lanes of one shape, each on
 * its own stream forked from and joined back into `stream`. */
int gbp_batch_run(gbp_lane* lanes, int n_lanes, const gbp_job* jobs,
                  int n_jobs, const gbp_lane_out* out, gbp_stream_t stream);

/* ---- Kernel tracing (no reference counterpart) ---------------------------
 * While enabled, every kernel the library launches outside stream capture is
 * bracketed by CUDA events on its stream.  gbp_trace_collect stops tracing,
 * waits for the recorded launches and returns their names (static strings)
 * and durations in ms, in launch order. */
typedef struct gbp_trace_record {
  const char* kernel;
  float ms;
} gbp_trace_record;

int gbp_trace_enable(int capacity);
int gbp_trace_collect(gbp_trace_record* out, int max_records, int* n_records);

#ifdef __cplusplus
}
#endif

#endif /* GBPOWSPEC_H */
