/*
 * amb_gb300.h — C ABI of the GB300-native Active Model B+ integrator.
 *
 * Drop-in boundary for the reference's plain integrator (tranqui/active-model-bplus).
 * The reference exposes its integrator to Python through a pybind11 module
 * (src/integrator.cc:31-123) over the C++ class Integrator
 * (src/integrator.h:24-81, src/integrator.cu:288-538). This header replaces that
 * boundary with plain C: opaque handles, plain pointers and sizes, int status.
 *
 * Two layers:
 *   1. amb_integrator_*  — the reference's Integrator class, one call per method,
 *                          host buffers in and out (what a cgo / JNI / ctypes
 *                          binding of the reference's class would bind).
 *   2. amb_step_*, amb_terms_*, amb_mass_*, amb_check_finite_* — stateless,
 *                          stream-ordered calls on caller-owned DEVICE buffers
 *                          (what the Python host layer drives with torch tensors).
 *
 * Conventions
 *   - Fields are row-major (nrows, ncols), index = col + row * ncols, axis 0 = y
 *     (src/integrator.cu:59, src/integrator.cc:108-109). Periodic in both axes.
 *     Any nrows, ncols >= 1 is accepted (the reference needs multiples of 8).
 *   - Every call returns AMB_OK (0) or an AMB_ERR_* code; amb_last_error() gives
 *     the calling thread's message for the last failing call. Calls never throw.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).
 *   - Parameters travel with each call or handle: there is no process-global
 *     state (the reference keeps them in __constant__ memory, src/parameters.cu:6-8),
 *     so independent integrators may run concurrently on different streams.
 */
#ifndef AMB_GB300_H
#define AMB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define AMB_OK 0
#define AMB_ERR_INVALID 1     /* bad argument: size, pointer, precision, kernel id */
#define AMB_ERR_CUDA 2        /* CUDA runtime error (reference: kernel::throw_errors, src/integrator.cu:21-30) */
#define AMB_ERR_NONFINITE 3   /* field became NaN/Inf (reference: src/integrator.cu:524-537) */
#define AMB_ERR_NOMEM 4       /* device or host allocation failed */
#define AMB_ERR_UNSUPPORTED 5 /* valid request the chosen kernel cannot serve */

/* --------------------------------------------------------------- parameters */
/* HostStencilParams (src/parameters.h:23-41). */
typedef struct amb_stencil
{
    double dt, dx, dy;
} amb_stencil;

/* ActiveModelBPlusParams (src/parameters.h:54-77): mu = a phi + b phi^2 + c phi^3 - kappa lap phi,
 * active terms lambda |grad phi|^2 and zeta (lap phi) grad phi, noise temperature T. */
typedef struct amb_model
{
    double a, b, c, kappa, lambda, zeta, temperature;
} amb_model;

/* Storage precisions. The reference has FP64 only (src/math_primitives.h:5). */
#define AMB_F64 0  /* double field; parity path */
#define AMB_F32 1  /* float field, float arithmetic */
#define AMB_F32C 2 /* float field + 16-bit (bf16) Kahan residual plane: compensated update */

/* Selectors for the current / chemical-potential getters (src/integrator.h:41-51). */
#define AMB_CURRENT_TOTAL 0         /* get_current */
#define AMB_CURRENT_DETERMINISTIC 1 /* get_deterministic_current */
#define AMB_CURRENT_PASSIVE 2       /* get_passive_current */
#define AMB_CURRENT_ACTIVE 3        /* get_active_current */
#define AMB_CURRENT_LAMBDA 4        /* get_lambda_current */
#define AMB_CURRENT_CIRCULATING 5   /* get_circulating_current */
#define AMB_CURRENT_RANDOM 6        /* get_random_current */
#define AMB_MU_TOTAL 0              /* get_chemical_potential */
#define AMB_MU_PASSIVE 1            /* get_passive_chemical_potential */
#define AMB_MU_ACTIVE 2             /* get_active_chemical_potential */

/* Kernel selectors for amb_step_f32 (AMB_KERNEL_AUTO picks the fastest valid one). */
#define AMB_KERNEL_AUTO 0
#define AMB_KERNEL_TILE 1    /* shared-memory tile kernel, any grid */
#define AMB_KERNEL_SLIDING 2 /* warp-pair sliding FP32 kernel (ncols % 4 == 0, ncols >= 112, 16-byte aligned) */

/* Explicit kernel configuration for amb_step_f32_ex / amb_step_f64_ex (zeros mean defaults).
 * seg_rows: rows per warp-pair task of the sliding kernel.
 * pairs_per_cta: sliding kernel: warp pairs per CTA (1, 2 or 4); tile kernel: groups of 256
 *   threads per CTA (1, 2 or 4).
 * flags: AMB_FLAG_PERSISTENT (tile kernel): all nsteps of the call in one cooperative launch,
 *   a grid-wide barrier between the steps (for grids too small to fill the GPU, where a launch
 *   per step costs more than the step; ignored while the stream is being captured). The
 *   results are bitwise those of one launch per step.
 *   AMB_FLAG_FUSED (sliding kernel): one warp per strip runs every stage (no producer/consumer
 *   warp pair); pairs_per_cta then counts warps per CTA (1, 2 or 4). Bitwise the same results.
 *   AMB_FLAG_TILE_ROWS_28 (tile kernel): output tiles of 28 rows x 32 columns instead of 32 x 32
 *   (balances small grids over the SMs: 512 x 512 is 304 tiles, two per SM). Bitwise the same
 *   results. */
typedef struct amb_kernel_config
{
    int kernel;
    int seg_rows;
    int pairs_per_cta;
    int flags;
} amb_kernel_config;
#define AMB_FLAG_PERSISTENT 1
#define AMB_FLAG_FUSED 2
#define AMB_FLAG_TILE_ROWS_28 4

/* Number of FP64 planes written by amb_terms_*: mu_p, mu_a, J_p(y,x), J_l(y,x), J_c(y,x), J_r(y,x). */
#define AMB_NTERMS 10

const char* amb_version(void);
/* Message of the calling thread's last failing call ("" if none). Replaces the
 * reference's CudaError what() string (src/integrator.h:10-14). */
const char* amb_last_error(void);

/* ====================================================== layer 1: Integrator */
typedef struct amb_integrator amb_integrator;

/* Integrator::Integrator(field, stencil, model) (src/integrator.cu:288-333).
 * host_field: nrows*ncols doubles. precision: AMB_F64 / AMB_F32 / AMB_F32C.
 * seed keys the Philox noise (the reference draws a non-deterministic curand seed,
 * src/integrator.cu:320-323); the same seed reproduces a run exactly. */
int amb_integrator_create(const double* host_field, int nrows, int ncols, const amb_stencil* stencil,
                          const amb_model* model, int precision, uint64_t seed, amb_integrator** out);
/* Integrator::~Integrator (src/integrator.cu:353-366). NULL is ignored. */
void amb_integrator_destroy(amb_integrator* h);
/* Integrator::run(nsteps) (src/integrator.cu:497-538): advances nsteps steps, blocks until
 * done, then checks the field is finite (AMB_ERR_NONFINITE otherwise). As in the
 * reference, the timestep counter advances by nsteps even when nsteps <= 0. */
int amb_integrator_run(amb_integrator* h, int nsteps);
/* Integrator::get_field (src/integrator.cu:378-383): copies the field out as doubles. */
int amb_integrator_get_field(amb_integrator* h, double* host_out);
/* No reference counterpart: replace the field (resume from a checkpoint); residual cleared. */
int amb_integrator_set_field(amb_integrator* h, const double* host_field);
/* get_chemical_potential / get_passive_... / get_active_... (src/integrator.cu:385-404). */
int amb_integrator_get_chemical_potential(amb_integrator* h, int which, double* host_out);
/* get_current and friends (src/integrator.cu:406-465): two planes (y then x component). */
int amb_integrator_get_current(amb_integrator* h, int which, double* host_y, double* host_x);
/* get_timestep / get_time (src/integrator.h:53-61). */
int amb_integrator_get_timestep(const amb_integrator* h, int64_t* out);
int amb_integrator_get_time(const amb_integrator* h, double* out);
/* No reference counterpart: jump the step counter (exact resume of (field, step, seed)). */
int amb_integrator_set_timestep(amb_integrator* h, int64_t timestep);
/* get_stencil / get_model (src/integrator.cu:368-376). */
int amb_integrator_get_stencil(const amb_integrator* h, amb_stencil* out);
int amb_integrator_get_model(const amb_integrator* h, amb_model* out);
int amb_integrator_get_shape(const amb_integrator* h, int* nrows, int* ncols, int* precision);

/* ============================================ layer 2: device-pointer calls */

/* nsteps fused explicit-Euler steps on a device field (the reference's run loop,
 * src/integrator.cu:507-518, whose three kernels per step become one launch).
 * field and spare are two device buffers of nrows*ncols elements; the steps
 * ping-pong between them, and *result_in_spare (if not NULL) is set to 1 when the
 * result ended in `spare`, 0 when in `field`.
 * The update from step s to s+1 uses currents at step s with noise keyed on
 * (seed, s): steps run from step0 to step0 + nsteps.
 * injected_noise: NULL for Philox noise (or none when temperature == 0); otherwise
 * nsteps * 2 * nrows * ncols standard normals, per step the y plane then the x plane
 * (J_r = sqrt(2T/(dt dx dy)) * xi, src/integrator.cu:106-109).
 * Asynchronous on `stream`. */
int amb_step_f64(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                 double* field, double* spare, int64_t step0, int nsteps, const double* injected_noise,
                 void* stream, int* result_in_spare);
/* amb_step_f64 with an explicit tile-kernel configuration (kernel AMB_KERNEL_AUTO or
 * AMB_KERNEL_TILE; pairs_per_cta and flags as in amb_kernel_config; NULL = defaults). */
int amb_step_f64_ex(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                    double* field, double* spare, int64_t step0, int nsteps, const double* injected_noise,
                    const amb_kernel_config* config, void* stream, int* result_in_spare);
/* FP32 storage. residual: NULL for plain FP32 (AMB_F32), else a device plane of
 * nrows*ncols bf16 words updated in place (AMB_F32C; zero it before the first step).
 * kernel: AMB_KERNEL_*. */
int amb_step_f32(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                 float* field, float* spare, uint16_t* residual, int64_t step0, int nsteps,
                 const float* injected_noise, int kernel, void* stream, int* result_in_spare);

/* Measured kernel choice (no reference counterpart): times the tile kernel and the sliding
 * kernel over a range of row-segment heights and warp pairs per CTA, a few steps each on
 * scratch buffers of this shape (zero field, this model's noise on or off), and returns the
 * fastest configuration and its time per step. The result is cached per (device, shape,
 * compensated, noise); later calls return the cached entry, and AMB_KERNEL_AUTO in
 * amb_step_f32 / amb_step_f32_ex uses it. Synchronous; allocates 2-3 fields of scratch. The
 * FP32 kernels evaluate the same operations in the same order at every site, so their results
 * are bitwise equal: what the autotuner picks changes the time, never the field. */
int amb_autotune_f32(const amb_stencil* stencil, const amb_model* model, int nrows, int ncols, int compensated,
                     int probe_steps, void* stream, amb_kernel_config* best, double* us_per_step);

/* amb_step_f32 with an explicit kernel configuration (NULL = defaults). */
int amb_step_f32_ex(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                    float* field, float* spare, uint16_t* residual, int64_t step0, int nsteps,
                    const float* injected_noise, const amb_kernel_config* config, void* stream,
                    int* result_in_spare);

/* Every term of the reference's forces/currents kernels (src/integrator.cu:46-176) at
 * timestep `step`, as AMB_NTERMS FP64 device planes in `out` (order in AMB_NTERMS).
 * injected_noise: NULL (Philox) or 2 planes (y, x) of standard normals. */
int amb_terms_f64(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                  const double* field, int64_t step, const double* injected_noise, double* out, void* stream);
int amb_terms_f32(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                  const float* field, int64_t step, const float* injected_noise, double* out, void* stream);

/* FP64 compensated sum of a device field into out_sum (one double, device memory).
 * scratch: device memory of at least amb_mass_scratch_bytes(n) bytes. */
size_t amb_mass_scratch_bytes(int64_t n);
int amb_mass_f64(const double* field, int64_t n, double* out_sum, void* scratch, size_t scratch_bytes, void* stream);
int amb_mass_f32(const float* field, int64_t n, double* out_sum, void* scratch, size_t scratch_bytes, void* stream);

/* No counterpart in the reference. amb_mass_f32 without any device allocation, for
 * callers that cannot allocate (their allocator already holds the device memory, they
 * only receive device pointers, or they cannot afford cudaMalloc's synchronization).
 * Scratch is a file-scope device array (256 KiB per GPU, held until process exit);
 * fields above 2^30 sites are rejected with AMB_ERR_INVALID. The first call on each
 * device looks up the array's address and should precede any stream capture; the address
 * is cached per device ordinal for the life of the process, so it is stale after a
 * cudaDeviceReset of that device. All calls share the array: calls that overlap on the
 * GPU race. An error already pending from an earlier CUDA call is reported (AMB_ERR_CUDA)
 * and left pending; nothing is launched then. */
int amb_mass_f32_noalloc(const float* field, int64_t n, double* out_sum, void* stream);

/* ORs 1 into *flag (device int) when any element of the field is NaN or Inf
 * (src/integrator.cu:265-272). The caller zeroes the flag. */
int amb_check_finite_f64(const double* field, int64_t n, int* flag, void* stream);
int amb_check_finite_f32(const float* field, int64_t n, int* flag, void* stream);

/* ================================================================ ensemble */
/* No reference counterpart (the reference runs one integrator per process). Many
 * independent replicas — any mix of sizes (ncols >= 112, ncols % 4 == 0) and model
 * parameters, FP32 storage (AMB_F32 or AMB_F32C), one Philox seed each — advanced
 * together: one launch per step covers every replica, and graph_steps (even; 0 = no
 * graph) steps are captured once into a CUDA graph and replayed. Creation times a few
 * launches to choose the row-segment height of each replica shape (the fields are left as
 * given). Each replica's result is bitwise that of a single-field run. */
typedef struct amb_ensemble amb_ensemble;
int amb_ensemble_create(int nreplicas, const int* nrows, const int* ncols, const double* const* host_fields,
                        const amb_stencil* stencils, const amb_model* models, const uint64_t* seeds, int precision,
                        int graph_steps, amb_ensemble** out);
void amb_ensemble_destroy(amb_ensemble* h);
/* Advance every replica nsteps steps, then check all fields are finite (AMB_ERR_NONFINITE). */
int amb_ensemble_run(amb_ensemble* h, int nsteps);
int amb_ensemble_get_field(amb_ensemble* h, int replica, double* host_out);
/* timestep, warp-pair tasks per step, and the row-segment height of the tallest replicas' tasks
 * (heights are chosen per replica shape by measurement when the ensemble is created). */
int amb_ensemble_info(const amb_ensemble* h, int64_t* timestep, int* ntasks, int* seg_rows);
/* The step kernel's form: 0 = a producer/consumer warp pair per task, 1 = one warp per task
 * running every stage. Creation chooses the faster by measurement; set = 0 or 1 sets the form,
 * set = -1 leaves it; *form (may be NULL) receives the form in effect. Both forms give bitwise the
 * same fields. */
int amb_ensemble_form(amb_ensemble* h, int set, int* form);
/* Device-to-device copy of every replica's current field into dst / from src (FP32, packed
 * back to back in replica order, replica r at offset sum_{q<r} nrows_q*ncols_q). Scatter also
 * zeroes the compensation residuals. Synchronous. */
int amb_ensemble_gather(amb_ensemble* h, float* dst);
int amb_ensemble_scatter(amb_ensemble* h, const float* src);

/* ================================================================ analysis */

/* Radial binning of a power spectrum (device arrays). power: nrows*ncols values |phi_q|^2 in
 * FFT order; mode (r, c) has |k| from numpy's fftfreq convention with spacings dx, dy. Adds
 * each mode to bin l with edges[l-1] < |k| <= edges[l] (np.digitize right=True, the binning of
 * the reference's analysis notebook examples/structureFactor.ipynb); sum[l] and count[l]
 * (nedges each) are zeroed first. */
int amb_radial_spectrum(const double* power, int nrows, int ncols, double dx, double dy, const double* edges,
                        int nedges, double* sum, unsigned long long* count, void* stream);

/* 4-connected components of {field > threshold} on the periodic grid (no reference
 * counterpart; the droplet count of the analysis). labels: nrows*ncols ints, set to the
 * smallest linear index of each site's component, -1 for background. *ncomp (device int)
 * receives the number of components. Grids below 2^31 sites. */
int amb_label_components_f64(const double* field, int nrows, int ncols, double threshold, int* labels, int* ncomp,
                             void* stream);
int amb_label_components_f32(const float* field, int nrows, int ncols, double threshold, int* labels, int* ncomp,
                             void* stream);


/* ========================================================== learned stepper */
/* No reference counterpart. Building blocks of the learned coarse stepper: a
 * periodic CNN of 5x5 circular convolutions that predicts a face flux over many
 * Euler steps. All buffers are DEVICE pointers; calls are stream-ordered.
 *
 * Activations are bf16 "chunk planes": [batch][C/8][nrows][ncols][8] (16-byte
 * aligned). Requirements: ncols % 128 == 0, nrows >= 3, C in {16, 32}.
 * Convolution weights are passed as a bf16 B-operand image
 * [5 (kx)][Cin/8][5 (4 - ky)][npad][8]: element (ky, kx, ci, co) at
 * (((kx*Cin/8 + ci/8)*5 + 4 - ky)*npad + co)*8 + ci%8, co < npad zero-padded.
 * *error (device int, may be NULL) receives a non-zero code if a kernel gave up
 * waiting on its own pipeline (the outputs are then incomplete). */

/* Tensor-core self-test: d (128 x n, row-major FP32) = a (128 x k) * b (n x k)^T,
 * a and b row-major bf16, staged K-major (flag 0) or MN-major (flag 1).
 * n in {16, 32}, k in {16, 32, 48, 64}. One CTA. */
int amb_tc_selftest(const void* a, const void* b, float* d, int n, int k, int a_mn_major, int b_mn_major, int* error,
                    void* stream);

/* Epilogues of amb_conv5x5_forward */
#define AMB_EPI_GELU 0     /* out = bf16(gelu(acc + bias)) (tanh-form GELU); pre (optional) = bf16(acc + bias) */
#define AMB_EPI_F32 1      /* out_f32[batch][cout][nrows][ncols] = acc + bias (first cout channels) */
#define AMB_EPI_GELU_BWD 2 /* out = bf16(acc * gelu'(gate)), gate = pre-activation, same layout as out */

/* Circular 5x5 convolution, BF16 tensor cores, FP32 accumulation:
 * acc[b][co][r][c] = sum_{ci,ky,kx} w[co][ci][ky][kx] in[b][ci][(r+ky-2) mod nrows][(c+kx-2) mod ncols].
 * in: [batch][cin/8][nrows][ncols][8]; out/pre/gate: [batch][npad/8][nrows][ncols][8]. The data
 * gradient of the same convolution is this call with the kernel flipped in (ky, kx) and the
 * channel roles swapped. */
int amb_conv5x5_forward(const void* in, int batch, int nrows, int ncols, int cin, const void* wimg, const float* bias,
                        int npad, int cout, int epilogue, void* out, void* pre, const void* gate, float* out_f32,
                        int* error, void* stream);

/* Weight gradient: dw[tap][ci][co] (FP32, 25*cin*npad) = sum over batch and sites of
 * x[b][ci][(r+ky-2) mod nrows][(c+kx-2) mod ncols] * dz[b][co][r][c]. x: [batch][cin/8][...][8],
 * dz: [batch][npad/8][...][8]. Deterministic (fixed reduction order); scratch must hold
 * amb_conv5x5_wgrad_scratch_bytes(...) bytes. */
size_t amb_conv5x5_wgrad_scratch_bytes(int batch, int nrows, int ncols, int cin, int npad);
int amb_conv5x5_wgrad(const void* x, const void* dz, int batch, int nrows, int ncols, int cin, int npad, float* dw,
                      float* scratch, size_t scratch_bytes, int* error, void* stream);

/* Network input planes (16 channels, 2 chunks): bf16(phi), 256*(phi - bf16(phi)), zeta/4,
 * lambda, 10*T, zeros. phi: [batch][nrows][ncols] FP32; params: [batch][3] = (zeta, lambda, T). */
int amb_learned_input(const float* phi, const float* params, int batch, int nrows, int ncols, void* x, void* stream);

/* Two standard normals per site, xi[2][nrows][ncols], Philox keyed (seed, *step, site,
 * component) exactly as the integrator's noise (the step is read from device memory so that
 * a captured graph can advance it). */
int amb_learned_noise(int nrows, int ncols, uint64_t seed, const int64_t* step, float* xi, void* stream);

/* One macro step of the learned stepper on a fixed-point field phi_q (int32, phi * 2^24):
 * phi -= dt_macro * div F with div the face difference
 * (F_x(r,c) - F_x(r,c-1))/dx + (F_y(r,c) - F_y(r-1,c))/dy. F = flux + extra (extra may be
 * NULL), both [2][nrows][ncols] FP32 (component 0 = y face after (r,c), 1 = x face), plus, if
 * xi is non-NULL, the order-8 central derivative of noise_mag * xi written as face sums (xi as
 * from amb_learned_noise). Face values are formed in FP32 with explicitly rounded operations,
 * scaled by dt_macro/d * 2^24 and rounded to an integer once; each face increment is applied
 * with opposite signs to its two sites, so sum(phi_q) is conserved exactly. phi_f receives
 * phi_q * 2^-24. *flag |= 1 if a flux is non-finite or |phi| exceeds bound (then clamped).
 * step_to_advance (device int64, may be NULL) is incremented once, for the next macro step's
 * noise key. */
int amb_learned_update(const float* flux, const float* extra, int nrows, int ncols, double dt_macro, double dx,
                       double dy, const float* xi, double noise_mag, int32_t* phi_q, float* phi_f, double bound,
                       int* flag, int64_t* step_to_advance, void* stream);

/* amb_learned_update that also writes channel chunk 0 of the next network input (x_next, bf16
 * chunk planes [2][nrows][ncols][8], 16-byte aligned) from the updated field and params
 * (zeta, lambda, T), exactly as amb_learned_input does; chunk 1 (zeros) is left untouched. */
int amb_learned_update_input(const float* flux, const float* extra, int nrows, int ncols, double dt_macro,
                             double dx, double dy, const float* xi, double noise_mag, int32_t* phi_q, float* phi_f,
                             double bound, int* flag, int64_t* step_to_advance, const float* params, void* x_next,
                             void* stream);

/* The rfft2 spectra of two real white-noise fields (unit variance per site), drawn directly in
 * the spectral domain: complex64 out[2][nrows][ncols/2+1], mode (r, k) of component c at element
 * c*nrows*(ncols/2+1) + r*row_stride + k*col_stride. Complex normals with E|z|^2 = nrows*ncols,
 * Hermitian-consistent in the k = 0 and k = ncols/2 columns (so an inverse real FFT sees the
 * spectrum of a real field); Philox keyed (seed, *step, mode). */
int amb_learned_noise_spectral(int nrows, int ncols, uint64_t seed, const int64_t* step, void* out,
                               int64_t row_stride, int64_t col_stride, void* stream);

/* Spectral step of the learned stepper's linear part and noise: for n complex rfft2 modes
 * (complex64 arrays), out_y = phi_hat * my + noise_mag * xi_hat_y * ny and
 * out_x = phi_hat * mx + noise_mag * xi_hat_x * nx, xi_hat = [2][n] (y then x) or NULL.
 * Element-wise in memory order: all arrays must share one dense layout (of any dimension
 * order), e.g. the layout the FFT produced. */
int amb_learned_spectral_combine(const void* phi_hat, const void* xi_hat, const void* my, const void* mx,
                                 const void* ny, const void* nx, double noise_mag, int64_t n, void* out_y,
                                 void* out_x, void* stream);

/* cuFFT plans for the learned stepper's spectral pass on nrows x ncols fields, created (with
 * their work areas) by amb_learned_fft_create: amb_learned_fft_forward is the real-to-complex
 * transform of one field into a row-major [nrows][ncols/2+1] complex64 spectrum;
 * amb_learned_fft_inverse2 the unnormalised complex-to-real transform of two such spectra
 * (consecutive, overwritten) into two consecutive fields. Both are stream-ordered and can be
 * captured in a CUDA graph. */
int amb_learned_fft_create(int nrows, int ncols, void** handle);
int amb_learned_fft_forward(void* handle, const float* field, void* spectrum, void* stream);
int amb_learned_fft_inverse2(void* handle, void* spectra, float* fields, void* stream);
void amb_learned_fft_destroy(void* handle);

/* amb_learned_spectral_combine with xi_hat drawn in place: the draw amb_learned_noise_spectral
 * makes for the same seed and *step. All spectra are [nrows][ncols/2+1] complex64 in one dense
 * layout given by its strides (row-major: col_stride 1, row_stride ncols/2+1; column-major:
 * row_stride 1, col_stride nrows); other layouts are rejected. */
int amb_learned_spectral_combine_noise(const void* phi_hat, const void* my, const void* mx, const void* ny,
                                       const void* nx, double noise_mag, int nrows, int ncols, int64_t row_stride,
                                       int64_t col_stride, uint64_t seed, const int64_t* step, void* out_y,
                                       void* out_x, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* AMB_GB300_H */
