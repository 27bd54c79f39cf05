/*
 * dsplat_gb300.h -- C ABI of the GB300 (sm_103a) kernels of the Dirichlet-splatting
 * render-and-fit path.
 *
 * Every entry point takes plain device pointers and sizes, launches on the given
 * CUDA stream (a cudaStream_t passed as void*, 0 = legacy default stream) and returns
 * 0 on success or a DSG_ERR_* code; nothing traps, nothing synchronises the stream,
 * and nothing allocates device memory. Buffers that hold intermediate partial sums
 * are passed in by the caller as `workspace`; the *_workspace_bytes queries give
 * their size. Complex values are interleaved float pairs (re, im), the layout of a
 * torch complex64 tensor viewed as real. All tensors are C-contiguous.
 *
 * Each declaration names the reference binding it replaces (path:line within the
 * Asixa/Dirichlet-Splatting project). The reference bindings are Python functions
 * that launch Slang kernels through slangtorch; the Python layer of this project
 * (dirichlet-splatting_gb300/dsplat/kernels/) keeps their signatures and calls these.
 */
#ifndef DSPLAT_GB300_H
#define DSPLAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DSG_OK = 0,
  DSG_ERR_ARGUMENT = 1,      /* a size, pointer or configuration value is invalid   */
  DSG_ERR_UNSUPPORTED = 2,   /* a configuration this build does not handle           */
  DSG_ERR_WORKSPACE = 3,     /* workspace missing or smaller than the query result   */
  DSG_ERR_LAUNCH = 4,        /* cudaGetLastError reported a launch failure            */
  DSG_ERR_LIBRARY = 5        /* a cuBLAS call failed                                  */
};

/* FMCW chirp and sensor constants (reference: dsplat/fmcw.py:62-98, FMCWConfig).
 * num_bins = n_fft / 2, n_fft = samples * pad. pad must divide 8. */
typedef struct DsgChirp {
  int32_t num_bins;
  int32_t n_fft;
  int32_t samples;
  int32_t pad;
  double k0_per_meter;  /* 1 / range_bin_spacing_m                          */
  double fc;            /* carrier, Hz                                      */
  double slope;         /* chirp slope, Hz / s                              */
  double t_start;       /* ADC start time, s                                */
  double lambda_m;      /* c0 / fc                                          */
  double c0;            /* wave speed, m / s                                */
  double fresnel_n;     /* refractive index; <= 1 disables the Fresnel term */
} DsgChirp;

/* Spectral grid (reference: dsplat/spectral.py:16-34, SpectralGrid; taps as built in
 * dsplat/kernels/spectral.py:22-27). window: 0 rect, 1 hann, 2 hamming, 3 kaiser. */
typedef struct DsgGrid {
  int32_t dim;          /* 1..3 axes                                        */
  int32_t nfft[3];
  int32_t samples[3];
  int32_t window;
  int32_t max_taps;     /* row stride of the taps array (kaiser)            */
  float radius;         /* 0: untruncated                                   */
} DsgGrid;

const char* dsg_version(void);
const char* dsg_error_string(int code);
/* Kernels launched by this library since it was loaded (a host-side counter). */
uint64_t dsg_launch_count(void);

/* Launch-shape knobs, set by the autotuner (dsplat/autotune.py); no counterpart in the
 * reference, whose kernels have fixed Slang tile constants (dsplat/kernels/__init__.py:17-21,
 * kernels/surfel.py:42-55: PAD and TILE). 0 restores the automatic choice.
 *   DSG_TUNE_SPLAT_CTAS_PER_SM  splat render / JVP / correlation reductions: target CTAs per
 *                               SM when splitting surfels into segments or apertures into
 *                               chunks (automatic: 6; 1..32)
 *   DSG_TUNE_PROJECT_STAGES     dsg_design_project_bf16x3 pipeline stages (automatic: the
 *                               deepest ring that fits shared memory; 2..4, capped at that)
 *   DSG_TUNE_ORIENT_WARPS       dsg_surfel_correlate_orientations warps per CTA (automatic:
 *                               8; 1..8)
 *   DSG_TUNE_CORRELATION_FORM   how dsg_surfel_correlate(_active, _gradient) and
 *                               dsg_surfel_vjp evaluate their sums over range bins:
 *                               DSG_CORRELATION_INTERP (automatic) interpolates each pair's
 *                               statistics from per-aperture tables (a type-2 nonuniform FFT,
 *                               ~1e-7 relative to the exact sums); DSG_CORRELATION_EXACT sums
 *                               the closed-form kernel over every bin
 * Knobs are process-wide; set them between launches, not while another thread launches. */
#define DSG_TUNE_SPLAT_CTAS_PER_SM 0
#define DSG_TUNE_PROJECT_STAGES 1
#define DSG_TUNE_ORIENT_WARPS 2
#define DSG_TUNE_CORRELATION_FORM 3
#define DSG_TUNE_COUNT 4
#define DSG_CORRELATION_EXACT 1
#define DSG_CORRELATION_INTERP 2
int dsg_tuning_set(int32_t knob, int32_t value);
/* Current value of a knob (0: automatic), or -1 for an unknown knob. */
int32_t dsg_tuning_get(int32_t knob);

/* ---- FMCW surfels: range profiles and derivatives ------------------------------- */

/* One scene of dsg_surfel_render_scenes: its chirp, sensor positions [apertures, 3],
 * surfels (centers, normals [surfels, 3], weights [surfels] complex interleaved) and its
 * output profiles [apertures, num_bins] complex interleaved (all device pointers). */
typedef struct {
  DsgChirp chirp;
  const float* positions;
  int32_t apertures;
  const float* centers;
  const float* normals;
  const float* weights;
  int32_t surfels;
  float* out;
} DsgRenderScene;

/* Workspace of dsg_surfel_render_scenes (the device scene table, work list and queue counter). */
size_t dsg_surfel_render_scenes_workspace_bytes(const DsgRenderScene* scenes, int32_t count);

/* Range profiles of many scenes (a HOST array of count descriptors) in one persistent
 * launch; no counterpart in the reference, which renders one scene per call
 * (dsplat/kernels/surfel.py:167-196). Work items are (scene, 16-aperture tile), the scenes
 * with the most surfel-bins first; CTAs take items from a device counter until none is left
 * (no waits). Scenes may differ in apertures, surfels and chirp; each chirp needs pad 2
 * and 128 or 256 range bins (DSG_ERR_UNSUPPORTED otherwise). status (one int32, zero before
 * the call) becomes 1 if the device met a descriptor it cannot render. The descriptors and
 * the work list are copied to the workspace with one host-to-device copy on stream. */
int dsg_surfel_render_scenes(const DsgRenderScene* scenes, int32_t count, void* workspace, size_t workspace_bytes,
                             int32_t* status, void* stream);

/* Workspace of dsg_surfel_render / dsg_surfel_jvp (segment partials), in bytes. */
size_t dsg_surfel_render_workspace_bytes(const DsgChirp* chirp, int32_t apertures, int32_t surfels);

/* out[A,K] = sum_s weights_s * column_s (reference: dsplat/kernels/surfel.py:58-108
 * _profiles, and :186-196 render). positions [A,3], centers/normals [S,3],
 * weights [S] complex, out [A,K] complex. */
int dsg_surfel_render(const DsgChirp* chirp, const float* positions, int32_t apertures,
                      const float* centers, const float* normals, const float* weights,
                      int32_t surfels, float* out, void* workspace, size_t workspace_bytes,
                      void* stream);

/* Directional derivative of the profiles (reference: dsplat/kernels/surfel.py:140-164 jvp).
 * delta_centers/delta_normals [S,3], delta_weights [S] complex, out [A,K] complex. */
int dsg_surfel_jvp(const DsgChirp* chirp, const float* positions, int32_t apertures,
                   const float* centers, const float* normals, const float* weights,
                   const float* delta_centers, const float* delta_normals,
                   const float* delta_weights, int32_t surfels, float* out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* Workspace of the aperture-reduced kernels (vjp, correlate, correlate_gradient), for
 * either DSG_TUNE_CORRELATION_FORM. The interpolated form keeps per-aperture tables here
 * (apertures x 2 n_fft / pad complex values, twice that with derivatives) and reads fixed
 * per-chirp tables that the library builds on the host and uploads at the first call
 * with that chirp's samples, pad and bins on a device and context (one cudaMalloc and a
 * synchronous copy): make that first call before any stream capture. */
size_t dsg_surfel_reduce_workspace_bytes(const DsgChirp* chirp, int32_t apertures, int32_t surfels,
                                         int32_t values_per_surfel);

/* The forward through the ADC samples instead of the range bins (no counterpart in the
 * reference, whose render_bins sums the closed-form kernel over bins,
 * dsplat/kernels/surfel.slang:87-142): samples [A, samples] complex receives
 * y[a][n] = sum_s w_s c_s / samples exp(2 pi i n k0_s / n_fft), whose n_fft-point FFT
 * (negative exponent, zero padded) has the profiles of dsg_surfel_render as its first
 * num_bins entries. A pair's samples are a geometric sequence: each lane anchors its run of
 * samples / 8 consecutive samples exactly and advances by one complex multiply per sample;
 * surfel chunks are staged in shared memory by bulk copies when centers, normals and
 * weights are 16-byte aligned. samples / 8 must be 2, 4, 8, 16 or 32. status (one int32,
 * zeroed by the caller) becomes 1 if a copy never arrived; the affected samples are NaN.
 * Workspace: dsg_surfel_render_samples_workspace_bytes. */
size_t dsg_surfel_render_samples_workspace_bytes(const DsgChirp* chirp, int32_t apertures, int32_t surfels);
int dsg_surfel_render_samples(const DsgChirp* chirp, const float* positions, int32_t apertures,
                              const float* centers, const float* normals, const float* weights,
                              int32_t surfels, float* samples, void* workspace, size_t workspace_bytes,
                              int32_t* status, void* stream);

/* Gradients of Re(conj(upstream) . profiles) (reference: dsplat/kernels/surfel.py:123-137
 * vjp). upstream [A,K] complex; grad_centers/grad_normals [S,3]; grad_weights [S] complex.
 * Summed over apertures in a fixed order, in double precision across aperture chunks. */
int dsg_surfel_vjp(const DsgChirp* chirp, const float* positions, int32_t apertures,
                   const float* centers, const float* normals, const float* weights,
                   int32_t surfels, const float* upstream, float* grad_centers,
                   float* grad_normals, float* grad_weights, void* workspace,
                   size_t workspace_bytes, void* stream);

/* The fixed tables of the interpolated form (DSG_TUNE_CORRELATION_FORM) for a chirp of
 * `samples` ADC samples (a power of two, at least 8) and zero-padding factor `pad`, built
 * on the host in double precision and returned as float32, without a GPU: correlation
 * [K][2 samples][2] complex interleaved (K = samples pad / 2 bins; per grid cell the
 * coefficients of Z0 and of Z1), norm [4 samples][2] (per grid cell the coefficients of
 * N0 and N1). For checks of the tables; the kernels build their own. */
int dsg_surfel_interp_tables(int32_t samples, int32_t pad, float* correlation, size_t correlation_floats,
                             float* norm, size_t norm_floats);

/* Upper bound of the fixed device scratch of dsg_surfel_vjp_fixed_scratch (4 MiB per GPU). */
#define DSG_VJP_SCRATCH_MAX_BYTES ((size_t)4 << 20)

/* dsg_surfel_vjp for callers that cannot allocate device memory (their device memory is
 * owned by another allocator, or cudaMalloc's device-wide synchronization is not
 * acceptable to them). No counterpart in the reference. Same inputs, outputs and results
 * as dsg_surfel_vjp, but no workspace argument: the chunk partials go to one fixed
 * scratch array of DSG_VJP_SCRATCH_MAX_BYTES in the library, held by every GPU that
 * loads it until the process exits. It always sums over bins (the exact form of
 * DSG_TUNE_CORRELATION_FORM), whose chunk partials are surfels x 8 floats per aperture
 * chunk; it returns DSG_ERR_WORKSPACE, without launching, when they exceed that bound
 * (with the 152-SM grid sizing that is above about 131k surfels). The first call on a
 * device looks up the scratch address there (and may load the module), so make it
 * before any stream capture on that device; the address is remembered per device and
 * CUDA context, so a call after cudaDeviceReset, or from another context, looks it up
 * again (and is again a first call). Calls share the scratch: two calls whose
 * kernels overlap on the GPU race and give wrong gradients; order them on one stream.
 * Allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine. */
int dsg_surfel_vjp_fixed_scratch(const DsgChirp* chirp, const float* positions,
                                 int32_t apertures, const float* centers, const float* normals,
                                 const float* weights, int32_t surfels, const float* upstream,
                                 float* grad_centers, float* grad_normals, float* grad_weights,
                                 void* stream);

/* conj(column) . residual and |column|^2 per candidate, without area (reference:
 * dsplat/kernels/surfel.py:242-260 correlate). corr [C] complex, norm [C]. */
int dsg_surfel_correlate(const DsgChirp* chirp, const float* positions, int32_t apertures,
                         const float* centers, const float* normals, int32_t candidates,
                         const float* residual, float* corr, float* norm, void* workspace,
                         size_t workspace_bytes, void* stream);

/* dsg_surfel_correlate restricted to an active set held on the device: candidate s is
 * computed when s mod period < *active, and the others get corr = norm = 0. No counterpart
 * in the reference: its batched certificate search (dsplat/certificate.py, the backtracking
 * of search_certificate) scores every trial step; here the later backtracking fractions are
 * scored only for the candidates the first fraction did not improve, compacted to the
 * front of each period, without reading the count back to the host. */
int dsg_surfel_correlate_active(const DsgChirp* chirp, const float* positions, int32_t apertures,
                                const float* centers, const float* normals, int32_t candidates,
                                const float* residual, const int32_t* active, int32_t period,
                                float* corr, float* norm, void* workspace, size_t workspace_bytes,
                                void* stream);

/* correlate plus derivatives by centers (and normals) (reference:
 * dsplat/kernels/surfel.py:293-315 correlate_gradient). width = 3 or 6.
 * corr [C] complex, norm [C], dcorr [C,width] complex, dnorm [C,width]. */
int dsg_surfel_correlate_gradient(const DsgChirp* chirp, const float* positions,
                                  int32_t apertures, const float* centers, const float* normals,
                                  int32_t candidates, const float* residual, int32_t width,
                                  float* corr, float* norm, float* dcorr, float* dnorm,
                                  void* workspace, size_t workspace_bytes, void* stream);

/* The residual's aperture tables for the interpolated correlations, computed once and
 * read by any number of the *_tabled calls below. No counterpart in the reference, whose
 * certificate ascent (dsplat/certificate.py:159-194, search_certificate) correlates the
 * same residual with every trial of every iteration; the interpolated form's per-residual
 * work (a [A,K]x[K,2 samples] complex product per table) is done once per search here.
 * tables: [A][2 samples] complex for Z0, then (derivative != 0) the same for Z1;
 * dsg_surfel_residual_tables_bytes gives the size. The first call with a chirp's
 * samples and pad on a device builds its fixed tables (cudaMalloc and a synchronous copy):
 * make it before any stream capture. */
size_t dsg_surfel_residual_tables_bytes(const DsgChirp* chirp, int32_t apertures, int32_t derivative);
int dsg_surfel_residual_tables(const DsgChirp* chirp, const float* residual, int32_t apertures,
                               int32_t derivative, float* tables, size_t tables_bytes, void* stream);
/* Workspace of the tabled calls: the chunk partials only. */
size_t dsg_surfel_tabled_workspace_bytes(int32_t apertures, int32_t candidates, int32_t values_per_surfel);
/* dsg_surfel_correlate (active == NULL) or dsg_surfel_correlate_active from a residual's
 * tables: the same outputs, bitwise, as those calls in the interpolated form. values per
 * surfel 3. */
int dsg_surfel_correlate_tabled(const DsgChirp* chirp, const float* positions, int32_t apertures,
                                const float* centers, const float* normals, int32_t candidates,
                                const float* tables, const int32_t* active, int32_t period, float* corr,
                                float* norm, void* workspace, size_t workspace_bytes, void* stream);
/* dsg_surfel_correlate_gradient from a residual's tables (made with derivative != 0); the
 * same outputs, bitwise, as that call in the interpolated form. values per surfel 3 + 3 width. */
int dsg_surfel_correlate_gradient_tabled(const DsgChirp* chirp, const float* positions, int32_t apertures,
                                         const float* centers, const float* normals, int32_t candidates,
                                         const float* tables, int32_t width, float* corr, float* norm,
                                         float* dcorr, float* dnorm, void* workspace, size_t workspace_bytes,
                                         void* stream);

/* Scores of each candidate's own normal and every bank normal (reference:
 * dsplat/kernels/surfel.py:263-290 correlate_orientations). bank [Nb,3];
 * out [C, 1+Nb, 3] = (Re corr, Im corr, norm). range_table [A, n_fft*oversample, 2] and
 * norm_table [n_fft*oversample] select the FFT-interpolated mode when non-null. */
int dsg_surfel_correlate_orientations(const DsgChirp* chirp, const float* positions,
                                      int32_t apertures, const float* centers,
                                      const float* normals, int32_t candidates, const float* bank,
                                      int32_t bank_size, const float* residual,
                                      const float* range_table, const float* norm_table,
                                      int32_t oversample, float* out, void* stream);

/* The best normal of each candidate among its own and the bank's, with its certificate, in one
 * launch: dsg_surfel_correlate_orientations followed by the selection of
 * dsplat/certificate.py orient_candidates (reference: dsplat/certificate.py, the normal-bank
 * scoring of the spatial search), without writing the [C, 1 + Nb, 3] scores. Per normal the
 * certificate is |Re corr|^2 (real_mode) or |corr|^2 over max(norm, 1e-60) * energy in
 * double precision, corr and norm scaled first by sqrt(area) and area in float32; which [C]
 * receives the winning index (0 = the candidate's own normal, j = bank row j - 1; NaN
 * first, then the largest, ties to the lowest index) and top [C] its certificate. energy is
 * one double on the device (the residual's energy); areas [C]. */
int dsg_surfel_orient_best(const DsgChirp* chirp, const float* positions, int32_t apertures,
                           const float* centers, const float* normals, const float* areas, int32_t candidates,
                           const float* bank, int32_t bank_size, const float* residual, const float* range_table,
                           const float* norm_table, int32_t oversample, const double* energy, int32_t real_mode,
                           int32_t* which, float* top, void* stream);

/* Dictionary rows including sqrt(area) (reference: dsplat/kernels/surfel.py:199-220 design).
 * real != 0: out [2*A*K, S] with row (2k+part)*A + a; else out [A*K, S] complex. */
int dsg_surfel_design(const DsgChirp* chirp, const float* positions, int32_t apertures,
                      const float* centers, const float* normals, const float* areas,
                      int32_t surfels, int32_t real, float* out, void* stream);

/* Explicit columns [A,K,S] complex and their center/normal derivatives [A,K,S,6] complex,
 * without area (reference: dsplat/kernels/surfel.py:223-239 jacobian). */
int dsg_surfel_jacobian(const DsgChirp* chirp, const float* positions, int32_t apertures,
                        const float* centers, const float* normals, int32_t surfels,
                        float* columns, float* derivatives, void* stream);

/* ---- Spectral atoms --------------------------------------------------------------- */

/* Per-axis tables of the separable spectral atoms (the redesign of the reference's
 * per-bin evaluation, dsplat/kernels/spectral.slang:4-47): for axis d < dim, bin
 * u < nfft[d] and atom s, values[d][u][s] = K_d(u - centers[s][d]) and derivatives the
 * same of dK_d / d(delta), complex interleaved, with width = max nfft: values and
 * derivatives hold dim * width * count complex values (rows u >= nfft[d] untouched). The
 * grid's forward, JVP and VJP are then products of these [nfft[d], count] tables. */
int dsg_spectral_axis_tables(const DsgGrid* grid, const float* taps, const float* centers, int32_t count,
                             float* values, float* derivatives, void* stream);

/* out[M] = sum_s a_ms coeff_s (reference: dsplat/kernels/spectral.py:168-189). */
int dsg_spectral_render(const DsgGrid* grid, const float* taps, const float* centers,
                        int32_t count, const float* coeff, const float* bins, int32_t size,
                        float* out, void* stream);
/* Directional derivative (reference: dsplat/kernels/spectral.py:192-201 jvp). */
int dsg_spectral_jvp(const DsgGrid* grid, const float* taps, const float* centers,
                     int32_t count, const float* coeff, const float* delta_centers,
                     const float* delta_coeff, const float* bins, int32_t size, float* out,
                     void* stream);
/* Workspace of dsg_spectral_vjp, in bytes. */
size_t dsg_spectral_vjp_workspace_bytes(const DsgGrid* grid, int32_t count, int32_t size);
/* Gradients for centers [S,D] and complex coefficients [S] (reference:
 * dsplat/kernels/spectral.py:157-165,204-209). Deterministic two-stage sum. */
int dsg_spectral_vjp(const DsgGrid* grid, const float* taps, const float* centers,
                     int32_t count, const float* coeff, const float* upstream,
                     const float* bins, int32_t size, float* grad_centers, float* grad_coeff,
                     void* workspace, size_t workspace_bytes, void* stream);
/* Dictionary [M,S] complex and optionally d/dcenters [M,S,D] complex
 * (reference: dsplat/kernels/spectral.py:146-154 design). jacobian may be null. */
int dsg_spectral_design(const DsgGrid* grid, const float* taps, const float* centers,
                        int32_t count, const float* bins, int32_t size, float* out,
                        float* jacobian, void* stream);

/* ---- Search ----------------------------------------------------------------------- */

/* Range gate (reference: dsplat/kernels/search.py:10-24). intervals [Ap, bins] int32,
 * output [count] int32 0/1. */
int dsg_range_gate(const float* points, int32_t count, const float* positions,
                   int32_t apertures, const int32_t* intervals, int32_t bins, float spacing,
                   int32_t required, int32_t* output, void* stream);
/* Greedy separated peaks (reference: dsplat/kernels/search.py:27-39). order [count]
 * lists the candidate indices by descending score, ties in index order (a stable
 * descending sort); non-finite scores are never taken. output [peaks] int32 receives
 * the chosen indices best first, -1 past the last; peaks <= 4096. */
int dsg_peaks(const float* scores, const int32_t* order, const float* centers, int32_t count,
              int32_t dimension, int32_t peaks, float separation, int32_t* output, void* stream);
/* Candidates (visited in the given descending-score order, non-finite skipped) that
 * lie at least separation from every occupied point and every earlier kept candidate,
 * and never at distance zero; periodic axes fold when period [dimension] is non-null.
 * output [width] receives the kept indices, kept_count (device) their number
 * (reference: dsplat/replacement.py:142-175 _distinct). */
int dsg_distinct(const float* scores, const int32_t* order, const float* points, int32_t count,
                 int32_t dimension, const float* occupied, int32_t n_occupied, const float* period,
                 float separation, int32_t width, int32_t* output, int32_t* kept_count,
                 void* stream);
/* Quasi-Newton direction per candidate (reference: dsplat/kernels/search.py:42-56). */
int dsg_direction(const float* inverse, const float* gradient, const float* normals,
                  const float* mask, int32_t count, int32_t width, float radius, float* output,
                  void* stream);
/* Trial step (reference: dsplat/kernels/search.py:59-77). controls [4,6]. */
int dsg_trial(const float* centers, const float* normals, const float* direction,
              const float* controls, int32_t count, int32_t width, float fraction,
              float* out_centers, float* out_normals, void* stream);

/* dsg_trial for every backtracking fraction in one launch: fractions is a HOST array of
 * fraction_count <= 16 values; out_centers / out_normals [fraction_count, count, 3]
 * (reference: dsplat/certificate.py:164-167, the trials of search_certificate). */
int dsg_trials(const float* centers, const float* normals, const float* direction,
               const float* controls, int32_t count, int32_t width, const float* fractions,
               int32_t fraction_count, float* out_centers, float* out_normals, void* stream);

/* Constants of one certificate ascent: width 3 (centers) or 6 (centers and normals)
 * and, per group (0 centers, 1 normals), whether it is a unit vector, the length of one
 * solver step and the free components (mask 1) (reference: dsplat/parameters.py:15-83
 * ParameterConfig.mask / scale / normalize). */
typedef struct {
  int32_t width;
  int32_t normalize[2];
  float scale[2];
  float mask[6];
} DsgAscentSpec;

/* Batched backtracking, first phase. corr [count, 2] and norm [count] are the unscaled
 * correlations of the full-step trials (dsg_surfel_correlate); with areas [count] and
 * the residual power |r|^2 (one device double) they give each candidate's certificate
 * (reference: dsplat/certificate.py:11-37), compared with value [count]. improved[i] is
 * 1 where the full step raised it; the others ("pending") come first in a stable
 * partition: position[i] is candidate i's slot, pending (device) their number, and batch
 * row r - 1 of batch_centers / batch_normals [(fraction_count - 1) * count, 3] holds
 * trial fraction r of trial_centers / trial_normals [fraction_count, count, 3] at the
 * slots (reference: dsplat/certificate.py:163-177, the backtracking loop). One CTA.
 * stuck [count] (optional) marks candidates that rejected every fraction in an earlier
 * iteration: their state is unchanged, so they reject them again and are never pending
 * (no smaller fraction is scored for them). */
int dsg_ascent_partition(const float* corr, const float* norm, const float* areas, const double* power,
                         int32_t real_mode, const float* value, int32_t count, const float* trial_centers,
                         const float* trial_normals, int32_t fraction_count, const uint8_t* stuck, uint8_t* improved,
                         int32_t* position, int32_t* pending, float* batch_centers, float* batch_normals,
                         void* stream);
/* Batched backtracking, second phase: corr / norm [(fraction_count - 1) * count] are the
 * correlations of the batch rows (dsg_surfel_correlate_active with the pending count).
 * Each candidate takes the first fraction whose finite certificate exceeds value:
 * new_centers / new_normals receive the trial (normals only if move_normals) or the
 * current parameters, accepted[i] whether one was taken; a stuck candidate (optional
 * stuck [count], as for dsg_ascent_partition) takes none. */
int dsg_ascent_select(const float* corr, const float* norm, const float* areas, const double* power,
                      int32_t real_mode, const float* value, int32_t count, const uint8_t* improved,
                      const int32_t* position, const float* trial_centers, const float* trial_normals,
                      int32_t fraction_count, const uint8_t* stuck, const float* centers, const float* normals,
                      int32_t move_normals, float* new_centers, float* new_normals, uint8_t* accepted,
                      void* stream);
/* End of a batched ascent iteration: corr, norm, dcorr [count, width, 2] and dnorm
 * [count, width] are the unscaled correlation gradient at new_centers / new_normals
 * (dsg_surfel_correlate_gradient). Writes the certificate value, the negated gradient in
 * scaled tangent coordinates and the damped BFGS update of inverse [count, width, width]
 * (only where accepted and the curvature condition holds), and moves centers / normals
 * to the new parameters; all in place (reference: dsplat/certificate.py:136-142 ascent,
 * :178-194 the BFGS update). */
int dsg_ascent_update(const DsgAscentSpec* spec, const float* corr, const float* norm, const float* dcorr,
                      const float* dnorm, const float* areas, const double* power, int32_t real_mode,
                      int32_t count, const float* new_centers, const float* new_normals, const uint8_t* accepted,
                      float* centers, float* normals, float* value, float* gradient, float* inverse,
                      void* stream);

/* ---- Reductions and the row-basis response ----------------------------------------- */

/* Workspace of dsg_energy, in bytes. */
size_t dsg_energy_workspace_bytes(int64_t count);
/* out[0] = sum |value - reference|^2 in double precision, fixed order
 * (reference: dsplat/kernels/reduce.py:8-18 energy). out is one double. */
int dsg_energy(const float* value, const float* reference, int64_t count, double* out,
               void* workspace, size_t workspace_bytes, void* stream);

/* Float64 Dirichlet responses [bins, count] complex of count peak positions spread
 * evenly over [low, high] (reference: dsplat/kernels/response.py:8-20). */
int dsg_range_response(double low, double high, int32_t count, int32_t bins, int32_t samples,
                       int32_t nfft, double* out, void* stream);

/* ---- Gram products of the streamed normal equations --------------------------------- */

/* Plain FP32: add rows^T rows to the upper triangle of the row-major [n, n] matrix out
 * (cuBLAS SSYRK; reference: dsplat/kernels/cublas.py:31-44 syrk). rows [m, n] row-major. */
int dsg_syrk_f32(const float* rows, int64_t m, int32_t n, float* out, void* stream);

/* Row-major C[m, n] = A[m, k] B[k, n] + beta C on the tensor cores with FP32-accurate
 * BF16x9 emulation (cuBLAS CUBLAS_COMPUTE_32F_EMULATED_16BFX9). The mixed path's row-basis
 * projection of design blocks (replaces the FP32 GEMM of dsplat/fmcw.py:128-131). */
int dsg_gemm_f32_bf16x9(int32_t m, int32_t n, int32_t k, const float* a, int32_t lda, const float* b,
                        int32_t ldb, float beta, float* c, int32_t ldc, void* stream);

/* Mixed precision, fused: evaluate the real dictionary rows of every (aperture, surfel)
 * pair of the block (as dsg_surfel_design with real != 0) on chip, project them with the
 * block's interleaved row basis U [rank2, 2K] given as bf16 hi/lo [128, 2K] (rows >= rank2
 * zero) on the tcgen05 tensor cores (split-BF16x3), and store the projected rows split
 * and transposed: pt_hi/pt_lo[s * ld + column_offset + a * rank2 + rho]. pt must have at
 * least ceil(surfels / 32) * 32 rows. num_bins <= 128, pad in {1, 2, 4}. status as for
 * dsg_gram_bf16x3. Replaces dsplat/kernels/surfel.py:199-220 (design) followed by
 * dsplat/fmcw.py:128-131 (RowBasis.reduce_major) on the mixed path. */
int dsg_design_project_bf16x3(const DsgChirp* chirp, const float* positions, int32_t apertures,
                              const float* centers, const float* normals, const float* areas,
                              int32_t surfels, const void* basis_hi, const void* basis_lo,
                              int32_t rank2, void* pt_hi, void* pt_lo, int64_t ld,
                              int64_t column_offset, int32_t* status, void* stream);

/* Mixed precision: split FP32 rows [m, n] into bf16 hi + lo and store them transposed,
 * hi[s * ld + column_offset + r] = bf16(rows[r, s]) and lo the bf16 of the remainder.
 * Feeds dsg_gram_bf16x3 (replaces the FP32 operand of the reference's SYRK,
 * dsplat/varpro.py:108-118). */
int dsg_split_transpose_bf16(const float* rows, int64_t m, int32_t n, int64_t column_offset,
                             void* hi, void* lo, int64_t ld, void* stream);

/* Workspace of dsg_gram_bf16x3 in bytes: one FP32 128 x 128 slab per (tile, K split)
 * when k_splits > 1 (after capping k_splits at k_pad / 64), else 0. */
size_t dsg_gram_bf16x3_workspace_bytes(int32_t n_pad, int64_t k_pad, int32_t column_from, int32_t k_splits);

/* Mixed precision: out[n, n] (float64, row-major, leading dimension ldo) += the upper
 * 128 x 128 tiles of PT PT^T, PT = hi + lo of shape [n_pad, k_pad] bf16 (n_pad a multiple
 * of 128, k_pad of 64, zero padded), on the tcgen05 tensor cores in split-BF16x3 with FP32
 * accumulation; k_splits CTAs share each tile's reduction, write their FP32 parts to the
 * workspace, and a second kernel adds the parts in split order (bitwise reproducible).
 * Only tiles whose columns reach column_from or beyond are computed (0: the whole upper
 * triangle; the pooled cross-Gram of dsplat/replacement.py:178-199 needs the new columns).
 * status (one int32, zero before the call) becomes 1 if a bounded wait ran out.
 * Replaces dsplat/kernels/cublas.py:31-44 (cublasSsyrk_v2) on the mixed path. */
int dsg_gram_bf16x3(const void* hi, const void* lo, int32_t n, int32_t n_pad, int64_t k_pad,
                    int32_t column_from, int32_t k_splits, double* out, int32_t ldo, void* workspace,
                    size_t workspace_bytes, int32_t* status, void* stream);

/* ADC-domain synthesis of an FMCW scan in float64 (reference: dsplat/groundtruth.py:58-90
 * synthesize, :40-55 _echoes): adc[a, n] = sum_s amplitudes_s * (echo of surfel s at
 * aperture a) * exp(2 pi i beat n / sample_rate), n < chirp->samples (at most 256).
 * positions [A,3], centers/normals [S,3] and amplitudes [S] complex (interleaved) are
 * float64; adc [A, samples] complex128 (interleaved). The range FFT (n_fft points, first
 * num_bins, divided by samples) is left to the caller's FFT library. */
int dsg_synthesize_adc(const DsgChirp* chirp, double sample_rate, const double* positions, int32_t apertures,
                       const double* centers, const double* normals, const double* amplitudes, int32_t surfels,
                       double* adc, void* stream);

/* Angular-spectrum focusing of the range-migration initializer (reference:
 * dsplat/fmcw.py:361-454, migration, its per-depth frequency sum): focused [depth_count,
 * qu, qv] complex = sum_f spectrum[f, iu, iv] kz exp(-i kz depths[d]), kz = sqrt(max(k_f^2 -
 * kx^2 - ky^2, 0)), iu = (x - qu/2 + pu/2) mod pu (likewise iv). spectrum [frequencies, pu,
 * pv] complex, k [frequencies], kx [qu], ky [qv], depths [depth_count] float32. */
int dsg_migration_focus(const float* spectrum, int32_t frequencies, int32_t pu, int32_t pv, const float* k,
                        const float* kx, const float* ky, int32_t qu, int32_t qv, const float* depths,
                        int32_t depth_count, float* focused, void* stream);

/* Workspace of dsg_backward_elimination, in bytes. */
size_t dsg_elimination_workspace_bytes(int32_t n, int32_t count, int32_t is_complex);

/* Backward elimination of the merged replacement (reference: dsplat/replacement.py:104-140,
 * backward_elimination): with the float64 inverse W [n,n] (complex128 when is_complex,
 * row-major) of the pooled system and its right-hand side q [n], remove count unknowns one
 * at a time, each the cheapest |b_j|^2 / W_jj (b = W q) of those still allowed, continuing
 * with the rank-one-updated inverse; at most limit of the unknowns with limited[j] != 0
 * (uint8 [n], or NULL for no limit) are removed. removed [count] (int64) receives the
 * indices in order. Launches 2 + count kernels (3 + count in the factor form); ties go to the
 * lowest index. */
int dsg_backward_elimination(const void* inverse, const void* rhs, int32_t n, int32_t count,
                             const uint8_t* limited, int64_t limit, int32_t is_complex, void* workspace,
                             size_t workspace_bytes, int64_t* removed, void* stream);

/* Backward elimination from the lower-triangular inverse factor X = L^-1 (row-major,
 * strictly upper part zero) of the pooled system's Cholesky factor L instead of the
 * inverse W = X^H X itself (reference: dsplat/replacement.py:93-140, regularized_inverse
 * followed by backward_elimination): the same removals, W's columns formed on the fly. */
int dsg_backward_elimination_factor(const void* factor_inverse, const void* rhs, int32_t n, int32_t count,
                                    const uint8_t* limited, int64_t limit, int32_t is_complex, void* workspace,
                                    size_t workspace_bytes, int64_t* removed, void* stream);

/* Device workspace of dsg_triangular_inverse, in bytes. */
size_t dsg_triangular_inverse_workspace_bytes(int32_t n, int32_t is_complex);

/* In place: a row-major lower-triangular float64 (complex128 when is_complex) factor L [n,n]
 * becomes L^-1 (every 64-row diagonal block inverted by forward substitution in one launch,
 * then recursive halving with cuBLAS trmm for the off-diagonal blocks). info (one int32 on the device) receives the
 * 1-based row of the first zero diagonal element, 0 when L is nonsingular. Replaces the potri inside dsplat/replacement.py:93-101 (cholesky_inverse) on
 * the batched path. */
int dsg_triangular_inverse(void* factor, int32_t n, int32_t is_complex, void* workspace, size_t workspace_bytes,
                           int32_t* info, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DSPLAT_GB300_H */
