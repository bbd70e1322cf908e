// Launchers for the shared-memory tile step kernel (amb_step_tile.cuh): one launch per step, or
// (small grids) one cooperative launch for many steps with a grid barrier between them.
#include "amb_kernels.h"
#include "amb_step_tile.cuh"

namespace amb
{
    namespace
    {
        // Output tiles of TY rows x 32 columns: 32 x 32, or 28 x 32, which the autotuner picks for
        // small grids (a 512^2 grid is then 19 x 16 = 304 tiles, two per SM on 152 SMs, against 256
        // tiles of 32 x 32 that leave 48 SMs with one).

        template <typename Real, int COMP, int NT, int TY, int TX>
        cudaError_t launch_tile(const Real* phi_in, Real* phi_out, __nv_bfloat16* comp, const StepParams& p,
                                int noise_mode, const Real* injected, cudaStream_t stream)
        {
            using G = TileGeom<TY, TX>;
            constexpr size_t smem = G::template smem_bytes<Real>();
            auto kern = step_tile_kernel<Real, TY, TX, COMP, NT>;
            static bool configured = false;  // attribute is per-function; setting it twice is harmless
            if (!configured)
            {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                configured = true;
            }
            dim3 grid((p.nx + TX - 1) / TX, (p.ny + TY - 1) / TY);
            kern<<<grid, NT, smem, stream>>>(phi_in, phi_out, comp, comp, p, Canon<Real>(p), noise_mode, injected);
            return cudaGetLastError();
        }

        // All nsteps in one cooperative launch (grid = the resident CTAs, at most one per tile).
        // The grid barrier's arrival counter and error word come from the stream-ordered allocator
        // (cudaMallocAsync), so concurrent launches on other streams never share them.
        template <typename Real, int COMP, int NT, int TY, int TX>
        cudaError_t launch_tile_persistent(Real* buf0, Real* buf1, __nv_bfloat16* comp, const StepParams& p,
                                           int noise_mode, const Real* injected, int nsteps, cudaStream_t stream)
        {
            using G = TileGeom<TY, TX>;
            constexpr size_t smem = G::template smem_bytes<Real>();
            auto kern = step_tile_persistent_kernel<Real, TY, TX, COMP, NT>;
            static int resident = 0;  // co-resident CTAs on this device type
            if (resident == 0)
            {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                int dev = 0, sms = 0, blocks = 0, coop = 0;
                if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
                if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
                if (!coop) return cudaErrorNotSupported;
                if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
                if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, NT, smem)) != cudaSuccess) return e;
                resident = blocks * sms;
                if (resident < 1) return cudaErrorNotSupported;
            }
            const int ntiles = ((p.nx + TX - 1) / TX) * ((p.ny + TY - 1) / TY);
            const int grid = ntiles < resident ? ntiles : resident;
            void* ws = nullptr;
            cudaError_t e = cudaMallocAsync(&ws, 2 * sizeof(unsigned), stream);
            if (e != cudaSuccess) return e;
            e = cudaMemsetAsync(ws, 0, 2 * sizeof(unsigned), stream);
            unsigned* count = static_cast<unsigned*>(ws);
            int* error = reinterpret_cast<int*>(count + 1);
            const Canon<Real> k(p);
            StepParams pp = p;
            if (e == cudaSuccess)
            {
                void* args[] = {&buf0, &buf1, &comp, &pp, const_cast<Canon<Real>*>(&k), &noise_mode,
                                const_cast<Real**>(&injected), &nsteps, &count, &error};
                e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(grid), dim3(NT), args, smem,
                                                stream);
            }
            const cudaError_t ef = cudaFreeAsync(ws, stream);
            return e != cudaSuccess ? e : ef;
        }

        template <typename Real, int COMP, int TY>
        cudaError_t by_threads(const Real* phi_in, Real* phi_out, __nv_bfloat16* comp, const StepParams& p,
                               int noise_mode, const Real* injected, int groups, cudaStream_t stream)
        {
            if (groups == 4)
                return launch_tile<Real, COMP, 1024, TY, 32>(phi_in, phi_out, comp, p, noise_mode, injected, stream);
            if (groups == 2)
                return launch_tile<Real, COMP, 512, TY, 32>(phi_in, phi_out, comp, p, noise_mode, injected, stream);
            return launch_tile<Real, COMP, 256, TY, 32>(phi_in, phi_out, comp, p, noise_mode, injected, stream);
        }

        template <typename Real, int COMP, int TY>
        cudaError_t by_threads_persistent(Real* a, Real* b, __nv_bfloat16* comp, const StepParams& p, int noise_mode,
                                          const Real* injected, int nsteps, int groups, cudaStream_t stream)
        {
            if (groups == 4)
                return launch_tile_persistent<Real, COMP, 1024, TY, 32>(a, b, comp, p, noise_mode, injected, nsteps,
                                                                        stream);
            if (groups == 2)
                return launch_tile_persistent<Real, COMP, 512, TY, 32>(a, b, comp, p, noise_mode, injected, nsteps,
                                                                       stream);
            return launch_tile_persistent<Real, COMP, 256, TY, 32>(a, b, comp, p, noise_mode, injected, nsteps, stream);
        }

        template <typename Real, int COMP>
        cudaError_t by_shape(const Real* phi_in, Real* phi_out, __nv_bfloat16* comp, const StepParams& p,
                             int noise_mode, const Real* injected, int groups, bool rows28, cudaStream_t stream)
        {
            if (rows28) return by_threads<Real, COMP, 28>(phi_in, phi_out, comp, p, noise_mode, injected, groups, stream);
            return by_threads<Real, COMP, 32>(phi_in, phi_out, comp, p, noise_mode, injected, groups, stream);
        }

        template <typename Real, int COMP>
        cudaError_t by_shape_persistent(Real* a, Real* b, __nv_bfloat16* comp, const StepParams& p, int noise_mode,
                                        const Real* injected, int nsteps, int groups, bool rows28, cudaStream_t stream)
        {
            if (rows28)
                return by_threads_persistent<Real, COMP, 28>(a, b, comp, p, noise_mode, injected, nsteps, groups, stream);
            return by_threads_persistent<Real, COMP, 32>(a, b, comp, p, noise_mode, injected, nsteps, groups, stream);
        }
    }

    template <>
    cudaError_t launch_step_tile<double>(const double* phi_in, double* phi_out, __nv_bfloat16* comp, int comp_mode,
                                         const StepParams& p, int noise_mode, const double* injected, int groups,
                                         bool rows28, cudaStream_t stream)
    {
        (void)comp;
        if (comp_mode != COMP_NONE) return cudaErrorInvalidValue;
        return by_shape<double, COMP_NONE>(phi_in, phi_out, nullptr, p, noise_mode, injected, groups, rows28, stream);
    }

    template <>
    cudaError_t launch_step_tile<float>(const float* phi_in, float* phi_out, __nv_bfloat16* comp, int comp_mode,
                                        const StepParams& p, int noise_mode, const float* injected, int groups,
                                        bool rows28, cudaStream_t stream)
    {
        if (comp_mode == COMP_BF16)
            return by_shape<float, COMP_BF16>(phi_in, phi_out, comp, p, noise_mode, injected, groups, rows28, stream);
        return by_shape<float, COMP_NONE>(phi_in, phi_out, nullptr, p, noise_mode, injected, groups, rows28, stream);
    }

    template <>
    cudaError_t launch_steps_tile_persistent<double>(double* a, double* b, __nv_bfloat16* comp, int comp_mode,
                                                     const StepParams& p, int noise_mode, const double* injected,
                                                     int nsteps, int groups, bool rows28, cudaStream_t stream)
    {
        (void)comp;
        if (comp_mode != COMP_NONE) return cudaErrorInvalidValue;
        return by_shape_persistent<double, COMP_NONE>(a, b, nullptr, p, noise_mode, injected, nsteps, groups, rows28,
                                                      stream);
    }

    template <>
    cudaError_t launch_steps_tile_persistent<float>(float* a, float* b, __nv_bfloat16* comp, int comp_mode,
                                                    const StepParams& p, int noise_mode, const float* injected,
                                                    int nsteps, int groups, bool rows28, cudaStream_t stream)
    {
        if (comp_mode == COMP_BF16)
            return by_shape_persistent<float, COMP_BF16>(a, b, comp, p, noise_mode, injected, nsteps, groups, rows28,
                                                         stream);
        return by_shape_persistent<float, COMP_NONE>(a, b, nullptr, p, noise_mode, injected, nsteps, groups, rows28,
                                                     stream);
    }
}
