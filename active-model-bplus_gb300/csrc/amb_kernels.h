// Internal launch interface between the C-ABI layer (amb_abi.cu) and the
// kernel translation units. Not part of the public header.
#pragma once

#include "amb_common.cuh"
#include "amb_gb300.h"
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

namespace amb
{
    // Fused single-step tile kernel (amb_step_tile.cuh), one launch = one step; groups x 256
    // threads per CTA (groups in {1, 2, 4}); 32 x 32 output tiles, or 28 x 32 with rows28.
    template <typename Real>
    cudaError_t launch_step_tile(const Real* phi_in, Real* phi_out, __nv_bfloat16* comp, int comp_mode,
                                 const StepParams& p, int noise_mode, const Real* injected, int groups, bool rows28,
                                 cudaStream_t stream);
    // nsteps steps of the tile kernel in one cooperative launch (grid barrier between steps); the
    // result is in a when nsteps is even, in b when odd. injected: nsteps * 2 planes or nullptr.
    template <typename Real>
    cudaError_t launch_steps_tile_persistent(Real* a, Real* b, __nv_bfloat16* comp, int comp_mode,
                                             const StepParams& p, int noise_mode, const Real* injected, int nsteps,
                                             int groups, bool rows28, cudaStream_t stream);

    // Register-sliding FP32 kernel (amb_step_f32.cu). Returns cudaErrorNotSupported
    // when the grid shape is outside its fast-path constraints.
    cudaError_t launch_step_f32_sliding(const float* phi_in, float* phi_out, __nv_bfloat16* comp, int comp_mode,
                                        const StepParams& p, int noise_mode, const float* injected, int variant,
                                        cudaStream_t stream);
    bool step_f32_sliding_supported(int ny, int nx, int variant);
    int sliding_default_seg_h(int ny, int nx);

    // ------------------------------------------------------------- ensemble
    // One replica of a batched ensemble (device array of these, filled by the host).
    struct EnsembleReplica
    {
        float* phi[2];               // ping-pong pair
        __nv_bfloat16* residual;     // bf16 Kahan residual or nullptr
        StepParams p;                // p.step unused: the launch reads the step from the device counter
    };
    // One warp-pair task: rows [r0, r1) of column strip `strip` of replica `replica`.
    struct EnsembleTask
    {
        int replica, strip, r0, r1;
    };
    size_t sliding_coef_bytes();
    void sliding_make_coef(const StepParams& p, void* out);  // host: per-replica coefficient block
    int sliding_default_seg_h_for(int ny, int nx, int resident_pairs);
    // fused: one warp per task running every stage (otherwise a producer/consumer warp pair).
    cudaError_t launch_sliding_ensemble(const EnsembleReplica* reps, const void* coefs, const EnsembleTask* tasks,
                                        int ntasks, int parity, const int64_t* step_counter, int step_offset,
                                        int comp_mode, int noise_mode, bool fused, cudaStream_t stream);
    cudaError_t ensemble_resident_pairs(int* out, bool fused);

    template <typename Real>
    cudaError_t launch_terms(const Real* phi, double* out, const StepParams& p, int noise_mode, const Real* injected,
                             cudaStream_t stream);

    int mass_partials(size_t n);
    template <typename Real>
    cudaError_t launch_mass(const Real* f, size_t n, double* out, double* scratch, int nparts, cudaStream_t stream);

    template <typename Real>
    cudaError_t launch_nonfinite(const Real* f, size_t n, int* flag, cudaStream_t stream);

    // Tuned FP32 step configuration for this shape (amb_autotune_f32's cache), if any.
    bool autotune_lookup(int nrows, int ncols, int compensated, int noise, amb_kernel_config* out);

    // Sets the message amb_last_error() returns on the calling thread.
    void set_last_error(const std::string& msg);

    cudaError_t launch_convert_f64_to_f32(const double* src, float* dst, size_t n, cudaStream_t stream);
    cudaError_t launch_convert_f32_to_f64(const float* src, double* dst, size_t n, cudaStream_t stream);
}
