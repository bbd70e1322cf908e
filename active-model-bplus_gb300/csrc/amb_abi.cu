// C-ABI entry points (include/amb_gb300.h): argument checking, error strings,
// the stream-ordered device-pointer layer, and the Integrator handle.
#include "amb_gb300.h"
#include "amb_kernels.h"
#include "amb_step_tile.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace
{
    thread_local std::string g_last_error;

    int fail(int code, const std::string& msg)
    {
        g_last_error = msg;
        return code;
    }

    int cuda_fail(cudaError_t e, const char* where)
    {
        return fail(AMB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    }

    constexpr int kMaxDim = 1 << 30;

    int check_shape(int nrows, int ncols)
    {
        if (nrows < 1 || ncols < 1 || nrows > kMaxDim || ncols > kMaxDim)
            return fail(AMB_ERR_INVALID, "grid shape must have nrows, ncols >= 1 (got " + std::to_string(nrows) + " x "
                                             + std::to_string(ncols) + ")");
        if (int64_t(nrows) * ncols > (int64_t(1) << 36))
            return fail(AMB_ERR_INVALID, "grid has too many sites");
        return AMB_OK;
    }

    int check_params(const amb_stencil* s, const amb_model* m)
    {
        if (!s || !m) return fail(AMB_ERR_INVALID, "stencil and model must not be NULL");
        return AMB_OK;
    }

    // Device-side parameter block for one launch (src/parameters.h:43-51,79-87 derive
    // dxInv, dyInv and the two noise strengths the same way).
    amb::StepParams make_params(const amb_stencil* s, const amb_model* m, uint64_t seed, int nrows, int ncols,
                                int64_t step)
    {
        amb::StepParams p{};
        p.ny = nrows;
        p.nx = ncols;
        p.dt = s->dt;
        p.dxInv = 1 / s->dx;
        p.dyInv = 1 / s->dy;
        p.a = m->a;
        p.b = m->b;
        p.c = m->c;
        p.kappa = m->kappa;
        p.lambda = m->lambda;
        p.zeta = m->zeta;
        p.noise_mag = std::sqrt(2 * m->temperature) * std::sqrt(1. / (s->dt * s->dx * s->dy));
        p.seed = seed;
        p.step = step;
        return p;
    }

    int noise_mode_for(const amb_model* m, const void* injected)
    {
        if (injected) return amb::NOISE_INJECTED;
        return m->temperature != 0 ? amb::NOISE_PHILOX : amb::NOISE_OFF;
    }

    cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }
}

void amb::set_last_error(const std::string& msg) { g_last_error = msg; }

extern "C" const char* amb_version(void) { return "amb_gb300 0.1 (sm_103a)"; }

extern "C" const char* amb_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------------------ steps

namespace
{
    bool capturing(cudaStream_t s)
    {
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
    }

    // Steps of the tile kernel: one launch per step, or all of them in one persistent launch.
    template <typename Real>
    int tile_steps(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                   Real* field, Real* spare, __nv_bfloat16* res, int comp, int64_t step0, int nsteps,
                   const Real* injected_noise, const amb_kernel_config& cfg, cudaStream_t stream,
                   int* result_in_spare, const char* name)
    {
        const size_t n = size_t(nrows) * ncols;
        const int mode = noise_mode_for(model, injected_noise);
        // default CTA width: 512 threads (measured fastest for FP64 at 1024^2-4096^2 and for FP32
        // small grids; the FP32 autotuner names its own)
        const int groups = cfg.pairs_per_cta == 0 ? 2 : cfg.pairs_per_cta;
        const bool rows28 = (cfg.flags & AMB_FLAG_TILE_ROWS_28) != 0;
        if ((cfg.flags & AMB_FLAG_PERSISTENT) && nsteps > 1 && !capturing(stream))
        {
            amb::StepParams p = make_params(stencil, model, seed, nrows, ncols, step0);
            cudaError_t e = amb::launch_steps_tile_persistent<Real>(field, spare, res, comp, p, mode, injected_noise,
                                                                    nsteps, groups, rows28, stream);
            if (e != cudaSuccess) return cuda_fail(e, name);
            if (result_in_spare) *result_in_spare = nsteps & 1;
            return AMB_OK;
        }
        Real* cur = field;
        Real* nxt = spare;
        for (int s = 0; s < nsteps; ++s)
        {
            amb::StepParams p = make_params(stencil, model, seed, nrows, ncols, step0 + s);
            const Real* inj = injected_noise ? injected_noise + size_t(s) * 2 * n : nullptr;
            cudaError_t e = amb::launch_step_tile<Real>(cur, nxt, res, comp, p, mode, inj, groups, rows28, stream);
            if (e != cudaSuccess) return cuda_fail(e, name);
            std::swap(cur, nxt);
        }
        if (result_in_spare) *result_in_spare = (cur == spare) ? 1 : 0;
        return AMB_OK;
    }

    int check_config(const amb_kernel_config& cfg, int max_kernel)
    {
        if (cfg.kernel < AMB_KERNEL_AUTO || cfg.kernel > max_kernel) return fail(AMB_ERR_INVALID, "unknown kernel selector");
        if (cfg.seg_rows < 0 || cfg.pairs_per_cta < 0 || cfg.pairs_per_cta > 4 || cfg.pairs_per_cta == 3)
            return fail(AMB_ERR_INVALID, "kernel config: seg_rows >= 0, pairs_per_cta in {0, 1, 2, 4}");
        if (cfg.flags & ~(AMB_FLAG_PERSISTENT | AMB_FLAG_FUSED | AMB_FLAG_TILE_ROWS_28))
            return fail(AMB_ERR_INVALID, "kernel config: unknown flags");
        return AMB_OK;
    }
}

extern "C" int amb_step_f64_ex(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows,
                               int ncols, double* field, double* spare, int64_t step0, int nsteps,
                               const double* injected_noise, const amb_kernel_config* config, void* stream,
                               int* result_in_spare)
{
    if (int rc = check_shape(nrows, ncols)) return rc;
    if (int rc = check_params(stencil, model)) return rc;
    if (!field || !spare || field == spare) return fail(AMB_ERR_INVALID, "field and spare must be distinct device buffers");
    if (nsteps < 0) return fail(AMB_ERR_INVALID, "nsteps must be >= 0");
    amb_kernel_config cfg{AMB_KERNEL_AUTO, 0, 0, 0};
    if (config) cfg = *config;
    if (int rc = check_config(cfg, AMB_KERNEL_TILE)) return rc;
    return tile_steps<double>(stencil, model, seed, nrows, ncols, field, spare, nullptr, amb::COMP_NONE, step0, nsteps,
                              injected_noise, cfg, as_stream(stream), result_in_spare, "amb_step_f64");
}

extern "C" int amb_step_f64(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                            double* field, double* spare, int64_t step0, int nsteps, const double* injected_noise,
                            void* stream, int* result_in_spare)
{
    return amb_step_f64_ex(stencil, model, seed, nrows, ncols, field, spare, step0, nsteps, injected_noise, nullptr,
                           stream, result_in_spare);
}

namespace
{
    bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }
}

extern "C" int amb_step_f32_ex(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows,
                               int ncols, float* field, float* spare, uint16_t* residual, int64_t step0, int nsteps,
                               const float* injected_noise, const amb_kernel_config* config, void* stream,
                               int* result_in_spare)
{
    if (int rc = check_shape(nrows, ncols)) return rc;
    if (int rc = check_params(stencil, model)) return rc;
    if (!field || !spare || field == spare) return fail(AMB_ERR_INVALID, "field and spare must be distinct device buffers");
    if (nsteps < 0) return fail(AMB_ERR_INVALID, "nsteps must be >= 0");
    amb_kernel_config cfg{AMB_KERNEL_AUTO, 0, 0, 0};
    if (config) cfg = *config;
    if (cfg.kernel == AMB_KERNEL_AUTO && cfg.seg_rows == 0 && cfg.pairs_per_cta == 0)
    {
        amb_kernel_config tuned;
        if (amb::autotune_lookup(nrows, ncols, residual != nullptr, model->temperature > 0 && !injected_noise, &tuned))
            cfg = tuned;  // a sliding choice still falls back to the tile kernel on unaligned buffers below
    }
    if (int rc = check_config(cfg, AMB_KERNEL_SLIDING)) return rc;
    const size_t n = size_t(nrows) * ncols;
    const int mode = noise_mode_for(model, injected_noise);
    const int comp = residual ? amb::COMP_BF16 : amb::COMP_NONE;
    auto* res = reinterpret_cast<__nv_bfloat16*>(residual);
    const bool fits = amb::step_f32_sliding_supported(nrows, ncols, 0) && aligned(field, 16) && aligned(spare, 16)
                      && (!residual || aligned(residual, 8)) && (!injected_noise || aligned(injected_noise, 16));
    bool sliding = false;
    if (cfg.kernel == AMB_KERNEL_SLIDING && !fits && !(config && config->kernel == AMB_KERNEL_SLIDING))
        cfg = amb_kernel_config{AMB_KERNEL_TILE, 0, 0, 0};
    if (cfg.kernel == AMB_KERNEL_SLIDING)
    {
        if (!fits)
            return fail(AMB_ERR_UNSUPPORTED, "sliding kernel needs ncols % 4 == 0, ncols >= 112 and 16-byte aligned "
                                             "field buffers (8-byte residual)");
        sliding = true;
    }
    else if (cfg.kernel == AMB_KERNEL_AUTO)
        sliding = fits;
    if (!sliding)
        return tile_steps<float>(stencil, model, seed, nrows, ncols, field, spare, res, comp, step0, nsteps,
                                 injected_noise, cfg, as_stream(stream), result_in_spare, "amb_step_f32");
    const int pairs_code = cfg.pairs_per_cta == 1 ? 1 : cfg.pairs_per_cta == 4 ? 3 : cfg.pairs_per_cta == 2 ? 2 : 0;
    const int variant = (cfg.seg_rows << 4) | ((cfg.flags & AMB_FLAG_FUSED) ? 8 : 0) | pairs_code;
    float* cur = field;
    float* nxt = spare;
    for (int s = 0; s < nsteps; ++s)
    {
        amb::StepParams p = make_params(stencil, model, seed, nrows, ncols, step0 + s);
        const float* inj = injected_noise ? injected_noise + size_t(s) * 2 * n : nullptr;
        cudaError_t e = amb::launch_step_f32_sliding(cur, nxt, res, comp, p, mode, inj, variant, as_stream(stream));
        if (e != cudaSuccess) return cuda_fail(e, "amb_step_f32");
        std::swap(cur, nxt);
    }
    if (result_in_spare) *result_in_spare = (cur == spare) ? 1 : 0;
    return AMB_OK;
}

extern "C" int amb_step_f32(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                            float* field, float* spare, uint16_t* residual, int64_t step0, int nsteps,
                            const float* injected_noise, int kernel, void* stream, int* result_in_spare)
{
    amb_kernel_config cfg{kernel, 0, 0, 0};
    return amb_step_f32_ex(stencil, model, seed, nrows, ncols, field, spare, residual, step0, nsteps, injected_noise,
                           &cfg, stream, result_in_spare);
}

// ------------------------------------------------------------------ terms

extern "C" int amb_terms_f64(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                             const double* field, int64_t step, const double* injected_noise, double* out, void* stream)
{
    if (int rc = check_shape(nrows, ncols)) return rc;
    if (int rc = check_params(stencil, model)) return rc;
    if (!field || !out) return fail(AMB_ERR_INVALID, "field and out must not be NULL");
    amb::StepParams p = make_params(stencil, model, seed, nrows, ncols, step);
    cudaError_t e = amb::launch_terms<double>(field, out, p, noise_mode_for(model, injected_noise), injected_noise,
                                              as_stream(stream));
    return e == cudaSuccess ? AMB_OK : cuda_fail(e, "amb_terms_f64");
}

extern "C" int amb_terms_f32(const amb_stencil* stencil, const amb_model* model, uint64_t seed, int nrows, int ncols,
                             const float* field, int64_t step, const float* injected_noise, double* out, void* stream)
{
    if (int rc = check_shape(nrows, ncols)) return rc;
    if (int rc = check_params(stencil, model)) return rc;
    if (!field || !out) return fail(AMB_ERR_INVALID, "field and out must not be NULL");
    amb::StepParams p = make_params(stencil, model, seed, nrows, ncols, step);
    cudaError_t e = amb::launch_terms<float>(field, out, p, noise_mode_for(model, injected_noise), injected_noise,
                                             as_stream(stream));
    return e == cudaSuccess ? AMB_OK : cuda_fail(e, "amb_terms_f32");
}

// ------------------------------------------------------------- reductions

extern "C" size_t amb_mass_scratch_bytes(int64_t n)
{
    if (n < 1) return 0;
    return size_t(amb::mass_partials(size_t(n))) * 2 * sizeof(double);
}

namespace
{
    template <typename Real>
    int mass_impl(const Real* field, int64_t n, double* out_sum, void* scratch, size_t scratch_bytes, void* stream,
                  const char* name)
    {
        if (!field || !out_sum || !scratch || n < 1) return fail(AMB_ERR_INVALID, std::string(name) + ": bad arguments");
        if (scratch_bytes < amb_mass_scratch_bytes(n))
            return fail(AMB_ERR_INVALID, std::string(name) + ": scratch smaller than amb_mass_scratch_bytes(n)");
        int parts = amb::mass_partials(size_t(n));
        cudaError_t e = amb::launch_mass<Real>(field, size_t(n), out_sum, static_cast<double*>(scratch), parts,
                                               as_stream(stream));
        return e == cudaSuccess ? AMB_OK : cuda_fail(e, name);
    }

    template <typename Real>
    int finite_impl(const Real* field, int64_t n, int* flag, void* stream, const char* name)
    {
        if (!field || !flag || n < 1) return fail(AMB_ERR_INVALID, std::string(name) + ": bad arguments");
        cudaError_t e = amb::launch_nonfinite<Real>(field, size_t(n), flag, as_stream(stream));
        return e == cudaSuccess ? AMB_OK : cuda_fail(e, name);
    }
}

extern "C" int amb_mass_f64(const double* field, int64_t n, double* out_sum, void* scratch, size_t scratch_bytes,
                            void* stream)
{
    return mass_impl(field, n, out_sum, scratch, scratch_bytes, stream, "amb_mass_f64");
}

extern "C" int amb_mass_f32(const float* field, int64_t n, double* out_sum, void* scratch, size_t scratch_bytes,
                            void* stream)
{
    return mass_impl(field, n, out_sum, scratch, scratch_bytes, stream, "amb_mass_f32");
}

extern "C" int amb_check_finite_f64(const double* field, int64_t n, int* flag, void* stream)
{
    return finite_impl(field, n, flag, stream, "amb_check_finite_f64");
}

extern "C" int amb_check_finite_f32(const float* field, int64_t n, int* flag, void* stream)
{
    return finite_impl(field, n, flag, stream, "amb_check_finite_f32");
}

// ------------------------------------------------------------ Integrator

struct amb_integrator
{
    amb_stencil stencil;
    amb_model model;
    int nrows, ncols, precision;
    uint64_t seed;
    int64_t timestep = 0;
    int64_t terms_timestep = -1;  // timestep the cached terms belong to (src/integrator.cu:477-495)
    cudaStream_t stream = nullptr;
    void* buf[2] = {nullptr, nullptr};  // field ping-pong
    int cur = 0;
    uint16_t* residual = nullptr;
    double* stage = nullptr;  // float64 staging plane for FP32 fields, allocated on first transfer
    double* terms = nullptr;  // AMB_NTERMS planes, allocated on first getter call
    int* flag = nullptr;
    std::vector<double> host_terms;

    size_t n() const { return size_t(nrows) * ncols; }
    size_t elem() const { return precision == AMB_F64 ? sizeof(double) : sizeof(float); }
};

namespace
{
    void release(amb_integrator* h)
    {
        if (!h) return;
        if (h->stream) cudaStreamSynchronize(h->stream);
        cudaFree(h->buf[0]);
        cudaFree(h->buf[1]);
        cudaFree(h->residual);
        cudaFree(h->stage);
        cudaFree(h->terms);
        cudaFree(h->flag);
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
    }

    cudaError_t ensure_stage(amb_integrator* h)
    {
        if (h->stage) return cudaSuccess;
        return cudaMalloc(&h->stage, h->n() * sizeof(double));
    }

    // Host float64 -> device field (FP32 fields convert on the device).
    int upload(amb_integrator* h, const double* host_field)
    {
        cudaError_t e;
        if (h->precision == AMB_F64)
            e = cudaMemcpyAsync(h->buf[h->cur], host_field, h->n() * sizeof(double), cudaMemcpyHostToDevice, h->stream);
        else
        {
            e = ensure_stage(h);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(h->stage, host_field, h->n() * sizeof(double), cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess)
                e = amb::launch_convert_f64_to_f32(h->stage, static_cast<float*>(h->buf[h->cur]), h->n(), h->stream);
        }
        if (e == cudaSuccess && h->residual) e = cudaMemsetAsync(h->residual, 0, h->n() * sizeof(uint16_t), h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        h->terms_timestep = -1;
        return e == cudaSuccess ? AMB_OK : cuda_fail(e, "upload field");
    }

    int compute_terms(amb_integrator* h)
    {
        if (h->terms_timestep == h->timestep) return AMB_OK;
        if (!h->terms)
        {
            cudaError_t e = cudaMalloc(&h->terms, h->n() * AMB_NTERMS * sizeof(double));
            if (e != cudaSuccess) return fail(AMB_ERR_NOMEM, "terms buffer: " + std::string(cudaGetErrorString(e)));
        }
        int rc = h->precision == AMB_F64
                     ? amb_terms_f64(&h->stencil, &h->model, h->seed, h->nrows, h->ncols,
                                     static_cast<const double*>(h->buf[h->cur]), h->timestep, nullptr, h->terms, h->stream)
                     : amb_terms_f32(&h->stencil, &h->model, h->seed, h->nrows, h->ncols,
                                     static_cast<const float*>(h->buf[h->cur]), h->timestep, nullptr, h->terms, h->stream);
        if (rc) return rc;
        h->host_terms.resize(h->n() * AMB_NTERMS);
        cudaError_t e = cudaMemcpyAsync(h->host_terms.data(), h->terms, h->n() * AMB_NTERMS * sizeof(double),
                                        cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return cuda_fail(e, "terms readback");
        h->terms_timestep = h->timestep;
        return AMB_OK;
    }

    const double* plane(const amb_integrator* h, int k) { return h->host_terms.data() + size_t(k) * h->n(); }
}

extern "C" int amb_integrator_create(const double* host_field, int nrows, int ncols, const amb_stencil* stencil,
                                     const amb_model* model, int precision, uint64_t seed, amb_integrator** out)
{
    if (!out) return fail(AMB_ERR_INVALID, "out must not be NULL");
    *out = nullptr;
    if (!host_field) return fail(AMB_ERR_INVALID, "host_field must not be NULL");
    if (int rc = check_shape(nrows, ncols)) return rc;
    if (int rc = check_params(stencil, model)) return rc;
    if (precision != AMB_F64 && precision != AMB_F32 && precision != AMB_F32C)
        return fail(AMB_ERR_INVALID, "precision must be AMB_F64, AMB_F32 or AMB_F32C");
    auto* h = new (std::nothrow) amb_integrator;
    if (!h) return fail(AMB_ERR_NOMEM, "host allocation failed");
    h->stencil = *stencil;
    h->model = *model;
    h->nrows = nrows;
    h->ncols = ncols;
    h->precision = precision;
    h->seed = seed;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMalloc(&h->buf[i], h->n() * h->elem());
    if (e == cudaSuccess && precision == AMB_F32C) e = cudaMalloc(&h->residual, h->n() * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->flag, sizeof(int));
    if (e != cudaSuccess)
    {
        release(h);
        return fail(e == cudaErrorMemoryAllocation ? AMB_ERR_NOMEM : AMB_ERR_CUDA,
                    std::string("amb_integrator_create: ") + cudaGetErrorString(e));
    }
    if (int rc = upload(h, host_field))
    {
        release(h);
        return rc;
    }
    *out = h;
    return AMB_OK;
}

extern "C" void amb_integrator_destroy(amb_integrator* h) { release(h); }

extern "C" int amb_integrator_run(amb_integrator* h, int nsteps)
{
    if (!h) return fail(AMB_ERR_INVALID, "NULL integrator");
    if (nsteps > 0)
    {
        int in_spare = 0;
        int rc;
        void* other = h->buf[1 - h->cur];
        if (h->precision == AMB_F64)
            rc = amb_step_f64(&h->stencil, &h->model, h->seed, h->nrows, h->ncols, static_cast<double*>(h->buf[h->cur]),
                              static_cast<double*>(other), h->timestep, nsteps, nullptr, h->stream, &in_spare);
        else
            rc = amb_step_f32(&h->stencil, &h->model, h->seed, h->nrows, h->ncols, static_cast<float*>(h->buf[h->cur]),
                              static_cast<float*>(other), h->residual, h->timestep, nsteps, nullptr, AMB_KERNEL_AUTO,
                              h->stream, &in_spare);
        if (rc) return rc;
        if (in_spare) h->cur = 1 - h->cur;
    }
    h->timestep += nsteps;  // as src/integrator.cu:520, also for nsteps <= 0

    cudaError_t e = cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream);
    int rc = AMB_OK;
    if (e == cudaSuccess)
        rc = h->precision == AMB_F64
                 ? amb_check_finite_f64(static_cast<const double*>(h->buf[h->cur]), int64_t(h->n()), h->flag, h->stream)
                 : amb_check_finite_f32(static_cast<const float*>(h->buf[h->cur]), int64_t(h->n()), h->flag, h->stream);
    if (rc) return rc;
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "amb_integrator_run");
    if (flag) return fail(AMB_ERR_NONFINITE, "an unknown numerical error occurred during simulation");
    return AMB_OK;
}

extern "C" int amb_integrator_get_field(amb_integrator* h, double* host_out)
{
    if (!h || !host_out) return fail(AMB_ERR_INVALID, "NULL argument");
    cudaError_t e;
    if (h->precision == AMB_F64)
    {
        e = cudaMemcpyAsync(host_out, h->buf[h->cur], h->n() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    else
    {
        e = ensure_stage(h);
        if (e == cudaSuccess)
            e = amb::launch_convert_f32_to_f64(static_cast<const float*>(h->buf[h->cur]), h->stage, h->n(), h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(host_out, h->stage, h->n() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    return e == cudaSuccess ? AMB_OK : cuda_fail(e, "amb_integrator_get_field");
}

extern "C" int amb_integrator_set_field(amb_integrator* h, const double* host_field)
{
    if (!h || !host_field) return fail(AMB_ERR_INVALID, "NULL argument");
    return upload(h, host_field);
}

extern "C" int amb_integrator_get_chemical_potential(amb_integrator* h, int which, double* host_out)
{
    if (!h || !host_out) return fail(AMB_ERR_INVALID, "NULL argument");
    if (which < AMB_MU_TOTAL || which > AMB_MU_ACTIVE) return fail(AMB_ERR_INVALID, "unknown chemical potential");
    if (int rc = compute_terms(h)) return rc;
    const size_t n = h->n();
    const double *mp = plane(h, 0), *ma = plane(h, 1);
    for (size_t i = 0; i < n; ++i)
        host_out[i] = which == AMB_MU_PASSIVE ? mp[i] : which == AMB_MU_ACTIVE ? ma[i] : mp[i] + ma[i];
    return AMB_OK;
}

extern "C" int amb_integrator_get_current(amb_integrator* h, int which, double* host_y, double* host_x)
{
    if (!h || !host_y || !host_x) return fail(AMB_ERR_INVALID, "NULL argument");
    if (which < AMB_CURRENT_TOTAL || which > AMB_CURRENT_RANDOM) return fail(AMB_ERR_INVALID, "unknown current");
    if (int rc = compute_terms(h)) return rc;
    const size_t n = h->n();
    double* out[2] = {host_y, host_x};
    for (int c = 0; c < 2; ++c)
    {
        const double *jp = plane(h, 2 + c), *jl = plane(h, 4 + c), *jc = plane(h, 6 + c), *jr = plane(h, 8 + c);
        for (size_t i = 0; i < n; ++i)
        {
            // Sums in the reference's order (src/integrator.cu:406-465).
            double active = jc[i] + jl[i];
            double det = active + jp[i];
            double v = 0;
            switch (which)
            {
            case AMB_CURRENT_TOTAL: v = det + jr[i]; break;
            case AMB_CURRENT_DETERMINISTIC: v = det; break;
            case AMB_CURRENT_PASSIVE: v = jp[i]; break;
            case AMB_CURRENT_ACTIVE: v = active; break;
            case AMB_CURRENT_LAMBDA: v = jl[i]; break;
            case AMB_CURRENT_CIRCULATING: v = jc[i]; break;
            default: v = jr[i]; break;
            }
            out[c][i] = v;
        }
    }
    return AMB_OK;
}

extern "C" int amb_integrator_get_timestep(const amb_integrator* h, int64_t* out)
{
    if (!h || !out) return fail(AMB_ERR_INVALID, "NULL argument");
    *out = h->timestep;
    return AMB_OK;
}

extern "C" int amb_integrator_get_time(const amb_integrator* h, double* out)
{
    if (!h || !out) return fail(AMB_ERR_INVALID, "NULL argument");
    *out = double(h->timestep) * h->stencil.dt;  // src/integrator.h:58-61
    return AMB_OK;
}

extern "C" int amb_integrator_set_timestep(amb_integrator* h, int64_t timestep)
{
    if (!h) return fail(AMB_ERR_INVALID, "NULL integrator");
    h->timestep = timestep;
    h->terms_timestep = -1;
    return AMB_OK;
}

extern "C" int amb_integrator_get_stencil(const amb_integrator* h, amb_stencil* out)
{
    if (!h || !out) return fail(AMB_ERR_INVALID, "NULL argument");
    *out = h->stencil;
    return AMB_OK;
}

extern "C" int amb_integrator_get_model(const amb_integrator* h, amb_model* out)
{
    if (!h || !out) return fail(AMB_ERR_INVALID, "NULL argument");
    *out = h->model;
    return AMB_OK;
}

extern "C" int amb_integrator_get_shape(const amb_integrator* h, int* nrows, int* ncols, int* precision)
{
    if (!h) return fail(AMB_ERR_INVALID, "NULL integrator");
    if (nrows) *nrows = h->nrows;
    if (ncols) *ncols = h->ncols;
    if (precision) *precision = h->precision;
    return AMB_OK;
}
