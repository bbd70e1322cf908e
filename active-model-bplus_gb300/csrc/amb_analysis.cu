// Field analysis on the device: radial binning of a power spectrum (structure
// factor S(k)) and periodic connected-component labelling (droplet count).
//
// S(k) follows the reference's analysis notebook (examples/structureFactor.ipynb,
// cells 5-7): phi_q = FFT2(phi - phi0) dx dy, |phi_q|^2 averaged over the modes whose
// |k| falls in each bin, bins given by np.digitize(|k|, edges, right=True), i.e.
// bin l holds edges[l-1] < |k| <= edges[l]. The FFT itself is a library call made
// by the caller (cuFFT through torch.fft); this file does the binning.
//
// Droplets: 4-connected components of {phi > threshold} on the periodic grid, by
// union-find with atomic hooking of the larger root onto the smaller (a standard
// GPU connected-components scheme), then full path compression. Labels are the
// smallest linear index in each component; background sites get -1.
#include "amb_gb300.h"
#include "amb_kernels.h"

#include <cuda_runtime.h>

namespace
{
    // |k| of FFT mode (r, c) with numpy's fftfreq ordering: frequency index f maps to
    // f (f < (n+1)/2) or f - n, times 2 pi / (n d).
    __device__ __forceinline__ double mode_k(int r, int c, int ny, int nx, double dx, double dy)
    {
        const double twopi = 6.283185307179586;
        int fr = r < (ny + 1) / 2 ? r : r - ny;
        int fc = c < (nx + 1) / 2 ? c : c - nx;
        double ky = twopi * (double(fr) * (1.0 / (double(ny) * dy)));
        double kx = twopi * (double(fc) * (1.0 / (double(nx) * dx)));
        return sqrt(kx * kx + ky * ky);
    }

    // Index l with edges[l-1] < k <= edges[l] (np.digitize right=True); nedges if beyond.
    __device__ __forceinline__ int digitize_right(double k, const double* __restrict__ edges, int nedges)
    {
        int lo = 0, hi = nedges;  // first index with edges[i] >= k
        while (lo < hi)
        {
            int mid = (lo + hi) >> 1;
            if (edges[mid] < k) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    }

    __global__ void radial_bin_kernel(const double* __restrict__ power, int ny, int nx, double dx, double dy,
                                      const double* __restrict__ edges, int nedges, double* __restrict__ sum,
                                      unsigned long long* __restrict__ count)
    {
        const size_t n = size_t(ny) * nx;
        for (size_t s = blockIdx.x * size_t(blockDim.x) + threadIdx.x; s < n; s += size_t(gridDim.x) * blockDim.x)
        {
            int r = int(s / nx), c = int(s % nx);
            int l = digitize_right(mode_k(r, c, ny, nx, dx, dy), edges, nedges);
            if (l < nedges)
            {
                atomicAdd(&sum[l], power[s]);
                atomicAdd(&count[l], 1ull);
            }
        }
    }

    // ----------------------------------------------------------- components

    __device__ __forceinline__ int find_root(const int* __restrict__ parent, int i)
    {
        while (true)
        {
            int p = parent[i];
            if (p == i) return i;
            i = p;
        }
    }

    template <typename Real>
    __global__ void ccl_init(const Real* __restrict__ f, int n, double threshold, int* __restrict__ parent)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            parent[i] = double(f[i]) > threshold ? i : -1;
    }

    // Union of two foreground roots: hook the larger index under the smaller with atomicCAS
    // (retry while another thread moved the root).
    __device__ void unite(int* parent, int a, int b)
    {
        while (true)
        {
            a = find_root(parent, a);
            b = find_root(parent, b);
            if (a == b) return;
            if (a > b)
            {
                int t = a;
                a = b;
                b = t;
            }
            int old = atomicCAS(&parent[b], b, a);
            if (old == b) return;
            b = old;
        }
    }

    __global__ void ccl_merge(int ny, int nx, int* parent)
    {
        const int n = ny * nx;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            if (parent[i] < 0) continue;
            int r = i / nx, c = i - r * nx;
            int right = r * nx + (c + 1 == nx ? 0 : c + 1);
            int down = (r + 1 == ny ? 0 : r + 1) * nx + c;
            if (parent[right] >= 0) unite(parent, i, right);
            if (parent[down] >= 0) unite(parent, i, down);
        }
    }

    __global__ void ccl_compress(int n, int* parent, int* __restrict__ ncomp)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            if (parent[i] < 0) continue;
            int root = find_root(parent, i);
            if (root == i) atomicAdd(ncomp, 1);
            parent[i] = root;
        }
    }

    int grid_for(size_t n)
    {
        size_t g = (n + 255) / 256;
        return int(g > 152 * 16 ? 152 * 16 : (g == 0 ? 1 : g));
    }
}

extern "C" int amb_radial_spectrum(const double* power, int nrows, int ncols, double dx, double dy,
                                   const double* edges, int nedges, double* sum, unsigned long long* count,
                                   void* stream)
{
    if (!power || !edges || !sum || !count || nrows < 1 || ncols < 1 || nedges < 1 || !(dx > 0) || !(dy > 0))
    {
        amb::set_last_error("amb_radial_spectrum: bad arguments");
        return AMB_ERR_INVALID;
    }
    auto s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(sum, 0, sizeof(double) * nedges, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(unsigned long long) * nedges, s);
    if (e == cudaSuccess)
    {
        radial_bin_kernel<<<grid_for(size_t(nrows) * ncols), 256, 0, s>>>(power, nrows, ncols, dx, dy, edges, nedges,
                                                                        sum, count);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
    {
        amb::set_last_error(std::string("amb_radial_spectrum: ") + cudaGetErrorString(e));
        return AMB_ERR_CUDA;
    }
    return AMB_OK;
}

namespace
{
    template <typename Real>
    int label_impl(const Real* field, int nrows, int ncols, double threshold, int* labels, int* ncomp, void* stream)
    {
        if (!field || !labels || !ncomp || nrows < 1 || ncols < 1 || int64_t(nrows) * ncols > (int64_t(1) << 31) - 1)
        {
            amb::set_last_error("amb_label_components: bad arguments (grid must have < 2^31 sites)");
            return AMB_ERR_INVALID;
        }
        auto s = static_cast<cudaStream_t>(stream);
        const int n = nrows * ncols;
        cudaError_t e = cudaMemsetAsync(ncomp, 0, sizeof(int), s);
        if (e == cudaSuccess)
        {
            ccl_init<Real><<<grid_for(n), 256, 0, s>>>(field, n, threshold, labels);
            ccl_merge<<<grid_for(n), 256, 0, s>>>(nrows, ncols, labels);
            ccl_compress<<<grid_for(n), 256, 0, s>>>(n, labels, ncomp);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess)
        {
            amb::set_last_error(std::string("amb_label_components: ") + cudaGetErrorString(e));
            return AMB_ERR_CUDA;
        }
        return AMB_OK;
    }
}

extern "C" int amb_label_components_f64(const double* field, int nrows, int ncols, double threshold, int* labels,
                                        int* ncomp, void* stream)
{
    return label_impl(field, nrows, ncols, threshold, labels, ncomp, stream);
}

extern "C" int amb_label_components_f32(const float* field, int nrows, int ncols, double threshold, int* labels,
                                        int* ncomp, void* stream)
{
    return label_impl(field, nrows, ncols, threshold, labels, ncomp, stream);
}
