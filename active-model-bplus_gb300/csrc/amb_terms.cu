// Per-term diagnostics and field reductions.
//
// amb_terms_*: every term the reference's forces/currents kernels produce
// (src/integrator.cu:46-110, 112-176), evaluated at the current field and
// written as ten FP64 planes: mu_p, mu_a, J_p(y,x), J_l(y,x), J_c(y,x),
// J_r(y,x). This backs the Integrator's current and chemical-potential
// getters (src/integrator.cu:385-465); it is off the time-stepping path.
//
// Reductions: FP64 compensated mass (sum of phi) and the non-finite check
// (src/integrator.cu:265-272,524-537).
#include "amb_common.cuh"
#include "amb_kernels.h"

#include <cmath>

namespace amb
{
    template <typename Real>
    __device__ __forceinline__ double at(const Real* f, int ny, int nx, int r, int c)
    {
        return double(f[(size_t)wrap_index(r, ny) * nx + wrap_index(c, nx)]);
    }

    // Pass A: mu_p, mu_a, J_c, J_r at each site.
    template <typename Real>
    __global__ void terms_local_kernel(const Real* __restrict__ phi, double* __restrict__ out, StepParams p,
                                       int noise_mode, const Real* __restrict__ injected)
    {
        const int ny = p.ny, nx = p.nx;
        const size_t n = (size_t)ny * nx;
        for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < n; s += (size_t)gridDim.x * blockDim.x)
        {
            int r = int(s / nx), c = int(s % nx);
            double f[3][3];
#pragma unroll
            for (int di = 0; di < 3; ++di)
#pragma unroll
                for (int dj = 0; dj < 3; ++dj) f[di][dj] = at(phi, ny, nx, r + di - 1, c + dj - 1);
            double second_x = -0.25 * ((f[0][0] - 2 * f[0][1] + f[0][2]) + (f[2][0] - 2 * f[2][1] + f[2][2]))
                            + 1.5 * (f[1][0] - 2 * f[1][1] + f[1][2]);
            double second_y = -0.25 * ((f[0][0] - 2 * f[1][0] + f[2][0]) + (f[0][2] - 2 * f[1][2] + f[2][2]))
                             + 1.5 * (f[0][1] - 2 * f[1][1] + f[2][1]);
            double lap = p.dxInv * p.dxInv * second_x + p.dyInv * p.dyInv * second_y;
            double gx = p.dxInv * (0.1 * ((f[0][2] - f[0][0]) + (f[2][2] - f[2][0])) + 0.3 * (f[1][2] - f[1][0]));
            double gy = p.dyInv * (0.1 * ((f[2][0] - f[0][0]) + (f[2][2] - f[0][2])) + 0.3 * (f[2][1] - f[0][1]));
            double v = f[1][1];
            out[0 * n + s] = (p.a * v + p.b * v * v + p.c * v * v * v) - p.kappa * lap;
            out[1 * n + s] = p.lambda * (gy * gy + gx * gx);
            out[6 * n + s] = p.zeta * lap * gy;
            out[7 * n + s] = p.zeta * lap * gx;
            double xy = 0, xx = 0;
            if (noise_mode == 1)
            {
                xy = double(noise_normal(p.seed, p.step, r, c, 0));
                xx = double(noise_normal(p.seed, p.step, r, c, 1));
            }
            else if (noise_mode == 2)
            {
                xy = double(injected[s]);
                xx = double(injected[n + s]);
            }
            out[8 * n + s] = p.noise_mag * xy;
            out[9 * n + s] = p.noise_mag * xx;
        }
    }

    // Pass B: J_p = -D8 mu_p and J_l = -Tj mu_a.
    __global__ void terms_currents_kernel(double* __restrict__ out, StepParams p)
    {
        const int ny = p.ny, nx = p.nx;
        const size_t n = (size_t)ny * nx;
        const double* mup = out;
        const double* mua = out + n;
        for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < n; s += (size_t)gridDim.x * blockDim.x)
        {
            int r = int(s / nx), c = int(s % nx);
            double dy8 = 0, dx8 = 0;
#pragma unroll
            for (int kk = 1; kk <= 4; ++kk)
            {
                dy8 += d8_tap(kk) * (at(mup, ny, nx, r + kk, c) - at(mup, ny, nx, r - kk, c));
                dx8 += d8_tap(kk) * (at(mup, ny, nx, r, c + kk) - at(mup, ny, nx, r, c - kk));
            }
            double ty = 0.1 * ((at(mua, ny, nx, r + 1, c - 1) - at(mua, ny, nx, r - 1, c - 1))
                             + (at(mua, ny, nx, r + 1, c + 1) - at(mua, ny, nx, r - 1, c + 1)))
                      + 0.3 * (at(mua, ny, nx, r + 1, c) - at(mua, ny, nx, r - 1, c));
            double tx = 0.1 * ((at(mua, ny, nx, r - 1, c + 1) - at(mua, ny, nx, r - 1, c - 1))
                             + (at(mua, ny, nx, r + 1, c + 1) - at(mua, ny, nx, r + 1, c - 1)))
                      + 0.3 * (at(mua, ny, nx, r, c + 1) - at(mua, ny, nx, r, c - 1));
            out[2 * n + s] = -(p.dyInv * dy8);
            out[3 * n + s] = -(p.dxInv * dx8);
            out[4 * n + s] = -(p.dyInv * ty);
            out[5 * n + s] = -(p.dxInv * tx);
        }
    }

    static int grid_for(size_t n, int block)
    {
        size_t g = (n + block - 1) / block;
        return int(g > 152 * 16 ? 152 * 16 : (g == 0 ? 1 : g));
    }

    template <typename Real>
    cudaError_t launch_terms(const Real* phi, double* out, const StepParams& p, int noise_mode, const Real* injected,
                             cudaStream_t stream)
    {
        size_t n = (size_t)p.ny * p.nx;
        int g = grid_for(n, 256);
        terms_local_kernel<Real><<<g, 256, 0, stream>>>(phi, out, p, noise_mode, injected);
        terms_currents_kernel<<<g, 256, 0, stream>>>(out, p);
        return cudaGetLastError();
    }

    template cudaError_t launch_terms<double>(const double*, double*, const StepParams&, int, const double*, cudaStream_t);
    template cudaError_t launch_terms<float>(const float*, double*, const StepParams&, int, const float*, cudaStream_t);

    // ----------------------------------------------------------- reductions

    constexpr int kReduceBlock = 256;

    // Neumaier-compensated pair (sum, compensation).
    struct CSum
    {
        double s, c;
        __device__ __forceinline__ void add(double v)
        {
            double t = s + v;
            c += fabs(s) >= fabs(v) ? (s - t) + v : (v - t) + s;
            s = t;
        }
        __device__ __forceinline__ void merge(const CSum& o)
        {
            add(o.s);
            c += o.c;
        }
    };

    __device__ __forceinline__ CSum block_reduce(CSum v)
    {
        __shared__ double ss[kReduceBlock / 32], sc[kReduceBlock / 32];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
        {
            CSum o{__shfl_down_sync(0xffffffffu, v.s, off), __shfl_down_sync(0xffffffffu, v.c, off)};
            v.merge(o);
        }
        int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0) { ss[warp] = v.s; sc[warp] = v.c; }
        __syncthreads();
        if (warp == 0)
        {
            v = lane < kReduceBlock / 32 ? CSum{ss[lane], sc[lane]} : CSum{0, 0};
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
            {
                CSum o{__shfl_down_sync(0xffffffffu, v.s, off), __shfl_down_sync(0xffffffffu, v.c, off)};
                v.merge(o);
            }
        }
        return v;
    }

    // Pass 1: each block writes its compensated partial sum (s, c) to scratch[2*block].
    template <typename Real>
    __global__ void __launch_bounds__(kReduceBlock) mass_partial_kernel(const Real* __restrict__ f, size_t n,
                                                                       double* __restrict__ scratch)
    {
        CSum v{0, 0};
        for (size_t i = blockIdx.x * (size_t)kReduceBlock + threadIdx.x; i < n; i += (size_t)gridDim.x * kReduceBlock)
            v.add(double(f[i]));
        v = block_reduce(v);
        if (threadIdx.x == 0)
        {
            scratch[2 * blockIdx.x] = v.s;
            scratch[2 * blockIdx.x + 1] = v.c;
        }
    }

    // Pass 2: one block folds the partials into out[0] = sum.
    __global__ void __launch_bounds__(kReduceBlock) mass_final_kernel(const double* __restrict__ scratch, int nparts,
                                                                     double* __restrict__ out)
    {
        CSum v{0, 0};
        for (int i = threadIdx.x; i < nparts; i += kReduceBlock) v.merge(CSum{scratch[2 * i], scratch[2 * i + 1]});
        v = block_reduce(v);
        if (threadIdx.x == 0) out[0] = v.s + v.c;
    }

    int mass_partials(size_t n)
    {
        size_t g = (n + kReduceBlock - 1) / kReduceBlock;
        return int(g > 152 * 8 ? 152 * 8 : (g == 0 ? 1 : g));
    }

    template <typename Real>
    cudaError_t launch_mass(const Real* f, size_t n, double* out, double* scratch, int nparts, cudaStream_t stream)
    {
        mass_partial_kernel<Real><<<nparts, kReduceBlock, 0, stream>>>(f, n, scratch);
        mass_final_kernel<<<1, kReduceBlock, 0, stream>>>(scratch, nparts, out);
        return cudaGetLastError();
    }

    template cudaError_t launch_mass<double>(const double*, size_t, double*, double*, int, cudaStream_t);
    template cudaError_t launch_mass<float>(const float*, size_t, double*, double*, int, cudaStream_t);

    template <typename Real>
    __global__ void nonfinite_kernel(const Real* __restrict__ f, size_t n, int* __restrict__ flag)
    {
        bool bad = false;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
            bad |= !isfinite(f[i]);
        if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
    }

    template <typename Real>
    cudaError_t launch_nonfinite(const Real* f, size_t n, int* flag, cudaStream_t stream)
    {
        nonfinite_kernel<Real><<<grid_for(n, 256), 256, 0, stream>>>(f, n, flag);
        return cudaGetLastError();
    }

    template cudaError_t launch_nonfinite<double>(const double*, size_t, int*, cudaStream_t);
    template cudaError_t launch_nonfinite<float>(const float*, size_t, int*, cudaStream_t);

    // Element-wise precision conversion (host-facing float64 <-> FP32 field storage).
    template <typename To, typename From>
    __global__ void convert_kernel(const From* __restrict__ src, To* __restrict__ dst, size_t n)
    {
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
            dst[i] = To(src[i]);
    }

    cudaError_t launch_convert_f64_to_f32(const double* src, float* dst, size_t n, cudaStream_t stream)
    {
        convert_kernel<float, double><<<grid_for(n, 256), 256, 0, stream>>>(src, dst, n);
        return cudaGetLastError();
    }

    cudaError_t launch_convert_f32_to_f64(const float* src, double* dst, size_t n, cudaStream_t stream)
    {
        convert_kernel<double, float><<<grid_for(n, 256), 256, 0, stream>>>(src, dst, n);
        return cudaGetLastError();
    }
}
