// Launchers for the shared-memory tile step kernel (amb_step_tile.cuh).
#include "amb_kernels.h"
#include "amb_step_tile.cuh"

namespace amb
{
    namespace
    {
        template <typename Real, int TY, int TX, int COMP>
        cudaError_t launch_tile(const Real* phi_in, Real* phi_out, __nv_bfloat16* comp, const StepParams& p,
                                int noise_mode, const Real* injected, cudaStream_t stream)
        {
            using G = TileGeom<TY, TX>;
            constexpr size_t smem = G::template smem_bytes<Real>();
            auto kern = step_tile_kernel<Real, TY, TX, COMP>;
            static bool configured = false;  // attribute is per-function; setting it twice is harmless
            if (!configured)
            {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                configured = true;
            }
            dim3 grid((p.nx + TX - 1) / TX, (p.ny + TY - 1) / TY);
            kern<<<grid, 256, smem, stream>>>(phi_in, phi_out, comp, comp, p, Canon<Real>(p), noise_mode, injected);
            return cudaGetLastError();
        }
    }

    template <>
    cudaError_t launch_step_tile<double>(const double* phi_in, double* phi_out, __nv_bfloat16* comp, int comp_mode,
                                         const StepParams& p, int noise_mode, const double* injected,
                                         cudaStream_t stream)
    {
        (void)comp;
        if (comp_mode != COMP_NONE) return cudaErrorInvalidValue;
        return launch_tile<double, 32, 32, COMP_NONE>(phi_in, phi_out, nullptr, p, noise_mode, injected, stream);
    }

    template <>
    cudaError_t launch_step_tile<float>(const float* phi_in, float* phi_out, __nv_bfloat16* comp, int comp_mode,
                                        const StepParams& p, int noise_mode, const float* injected, cudaStream_t stream)
    {
        if (comp_mode == COMP_BF16)
            return launch_tile<float, 32, 32, COMP_BF16>(phi_in, phi_out, comp, p, noise_mode, injected, stream);
        return launch_tile<float, 32, 32, COMP_NONE>(phi_in, phi_out, nullptr, p, noise_mode, injected, stream);
    }
}
