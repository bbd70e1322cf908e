// amb_mass_f32_noalloc: the FP64 compensated mass of an FP32 field without any
// device allocation.
//
// Some callers cannot allocate device memory at the point where they need the
// mass: a host program whose allocator has already reserved all device memory
// for its own pool, a plugin (cgo, JNI, another framework's custom op) that is
// handed device pointers but no allocator, or a time-critical loop that cannot
// afford cudaMalloc/cudaFree, which may synchronize the device. amb_mass_f32
// needs caller-provided scratch; this entry point instead keeps its scratch in
// a file-scope device array that every GPU loading the library holds until the
// process exits.
//
// Decomposition: one partial sum per fixed chunk of 65536 sites (Neumaier-
// compensated FP64), then one block folds the partials. The partials of one
// call fit the static array when the field has at most 2^30 sites; larger
// fields are rejected. Because the chunking does not depend on the GPU, the
// result is the same on any device.
//
// Sharing: every call on a device uses the same array, which keeps the last
// call's partials. Each call writes every slot it later reads, so nothing has
// to be cleared first. Calls that overlap on the GPU (on different streams, or
// from different host threads without ordering) race on the array and may
// return wrong sums; order them on one stream.
//
// Set-up: the array's device address is looked up with cudaGetSymbolAddress
// on the first call made on each device, with that device current; that first
// call on a device should come before any stream capture begins.
#include "amb_gb300.h"
#include "amb_kernels.h"

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

namespace
{
    constexpr int kChunk = 1 << 16;          // sites per partial sum
    constexpr int kMaxPartials = 1 << 14;    // partial sums the static array holds
    constexpr int64_t kMaxSites = int64_t(kChunk) * kMaxPartials;  // 2^30
    constexpr int kBlock = 256;
    constexpr int kMaxDevices = 64;

    // (sum, compensation) of each chunk: 2 doubles per partial, 256 KiB in total.
    static __device__ __align__(256) double g_noalloc_partials[2 * kMaxPartials];

    struct Neumaier
    {
        double s = 0, c = 0;
        __device__ void add(double v)
        {
            double t = s + v;
            c += fabs(s) >= fabs(v) ? (s - t) + v : (v - t) + s;
            s = t;
        }
    };

    __device__ Neumaier reduce_block(Neumaier v)
    {
        __shared__ double ss[kBlock], sc[kBlock];
        ss[threadIdx.x] = v.s;
        sc[threadIdx.x] = v.c;
        __syncthreads();
        for (int off = kBlock / 2; off > 0; off >>= 1)
        {
            if (threadIdx.x < off)
            {
                Neumaier a{ss[threadIdx.x], sc[threadIdx.x]};
                a.add(ss[threadIdx.x + off]);
                a.c += sc[threadIdx.x + off];
                ss[threadIdx.x] = a.s;
                sc[threadIdx.x] = a.c;
            }
            __syncthreads();
        }
        return Neumaier{ss[0], sc[0]};
    }

    // Block b sums sites [b * kChunk, min(n, (b + 1) * kChunk)).
    __global__ void __launch_bounds__(kBlock) chunk_sum_kernel(const float* __restrict__ f, int64_t n,
                                                               double* __restrict__ partials)
    {
        const int64_t lo = int64_t(blockIdx.x) * kChunk;
        const int64_t hi = lo + kChunk < n ? lo + kChunk : n;
        Neumaier v;
        for (int64_t i = lo + threadIdx.x; i < hi; i += kBlock) v.add(double(f[i]));
        v = reduce_block(v);
        if (threadIdx.x == 0)
        {
            partials[2 * blockIdx.x] = v.s;
            partials[2 * blockIdx.x + 1] = v.c;
        }
    }

    __global__ void __launch_bounds__(kBlock) fold_kernel(const double* __restrict__ partials, int nparts,
                                                          double* __restrict__ out)
    {
        Neumaier v;
        for (int i = threadIdx.x; i < nparts; i += kBlock)
        {
            v.add(partials[2 * i]);
            v.c += partials[2 * i + 1];
        }
        v = reduce_block(v);
        if (threadIdx.x == 0) out[0] = v.s + v.c;
    }

    std::mutex g_setup_mutex;
    double* g_scratch[kMaxDevices] = {};

    // Device address of the static array on the current device (looked up once per device).
    int scratch_on_current_device(double** out)
    {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess)
        {
            amb::set_last_error(std::string("amb_mass_f32_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
            return AMB_ERR_CUDA;
        }
        if (dev < 0 || dev >= kMaxDevices)
        {
            amb::set_last_error("amb_mass_f32_noalloc: device ordinal beyond 63");
            return AMB_ERR_UNSUPPORTED;
        }
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch[dev])
        {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (e != cudaSuccess || !p)
            {
                amb::set_last_error(std::string("amb_mass_f32_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
                return AMB_ERR_CUDA;
            }
            g_scratch[dev] = static_cast<double*>(p);
        }
        *out = g_scratch[dev];
        return AMB_OK;
    }
}

extern "C" int amb_mass_f32_noalloc(const float* field, int64_t n, double* out_sum, void* stream)
{
    if (!field || !out_sum || n < 1)
    {
        amb::set_last_error("amb_mass_f32_noalloc: field and out_sum must be device pointers and n >= 1");
        return AMB_ERR_INVALID;
    }
    if (n > kMaxSites)
    {
        amb::set_last_error("amb_mass_f32_noalloc: " + std::to_string(n) + " sites exceed the static scratch limit of "
                            + std::to_string(kMaxSites) + " (2^30); use amb_mass_f32 with caller scratch");
        return AMB_ERR_INVALID;
    }
    double* scratch = nullptr;
    if (int rc = scratch_on_current_device(&scratch)) return rc;
    const int parts = int((n + kChunk - 1) / kChunk);
    auto s = static_cast<cudaStream_t>(stream);
    // An error left pending by an earlier, unrelated call is not this call's: it is reported
    // without being cleared, so the caller's own error check still sees it.
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
    {
        amb::set_last_error(std::string("amb_mass_f32_noalloc: an earlier CUDA error is pending: ")
                            + cudaGetErrorString(pending));
        return AMB_ERR_CUDA;
    }
    chunk_sum_kernel<<<parts, kBlock, 0, s>>>(field, n, scratch);
    fold_kernel<<<1, kBlock, 0, s>>>(scratch, parts, out_sum);
    const cudaError_t e = cudaGetLastError();  // nothing was pending, so this is a launch error of ours
    if (e != cudaSuccess)
    {
        amb::set_last_error(std::string("amb_mass_f32_noalloc: ") + cudaGetErrorString(e));
        return AMB_ERR_CUDA;
    }
    return AMB_OK;
}
