// Spectral transforms of the learned stepper's linear-part and noise pass, on cuFFT plans owned
// by a handle: one real-to-complex 2D transform of the field and one batched complex-to-real
// 2D transform of the two flux components. Spectra are row-major [nrows][ncols/2 + 1]
// complex64; the inverse is unnormalised (callers fold 1/(nrows ncols) into their spectral
// filters) and overwrites its input spectra, which are scratch. Plans and their work areas are
// allocated when the handle is created, so the transforms can be captured in a CUDA graph.
#include "amb_gb300.h"
#include "amb_kernels.h"

#include <cuda_runtime.h>
#include <cufft.h>

#include <new>
#include <string>

namespace
{
    struct LearnedFft
    {
        cufftHandle r2c = 0, c2r = 0;
        bool has_r2c = false, has_c2r = false;
        int nrows = 0, ncols = 0;
    };

    int fail(const char* what, int code)
    {
        amb::set_last_error(what);
        return code;
    }

    int fail_cufft(const char* what, cufftResult r)
    {
        amb::set_last_error(std::string(what) + ": cuFFT error " + std::to_string(int(r)));
        return AMB_ERR_CUDA;
    }

    void destroy(LearnedFft* f)
    {
        if (!f) return;
        if (f->has_r2c) cufftDestroy(f->r2c);
        if (f->has_c2r) cufftDestroy(f->c2r);
        delete f;
    }
}

extern "C" int amb_learned_fft_create(int nrows, int ncols, void** out)
{
    if (!out || nrows < 2 || ncols < 2 || (long long)nrows * ncols >= (1ll << 31))
        return fail("amb_learned_fft_create: bad arguments", AMB_ERR_INVALID);
    *out = nullptr;
    LearnedFft* f = new (std::nothrow) LearnedFft;
    if (!f) return fail("amb_learned_fft_create: out of host memory", AMB_ERR_NOMEM);
    f->nrows = nrows;
    f->ncols = ncols;
    int n[2] = {nrows, ncols};
    const int nk = ncols / 2 + 1;
    cufftResult r = cufftPlan2d(&f->r2c, nrows, ncols, CUFFT_R2C);
    if (r != CUFFT_SUCCESS)
    {
        destroy(f);
        return fail_cufft("amb_learned_fft_create (R2C plan)", r);
    }
    f->has_r2c = true;
    // two inverse transforms: inputs nrows*nk complex apart, outputs nrows*ncols reals apart
    r = cufftPlanMany(&f->c2r, 2, n, nullptr, 1, nrows * nk, nullptr, 1, nrows * ncols, CUFFT_C2R, 2);
    if (r != CUFFT_SUCCESS)
    {
        destroy(f);
        return fail_cufft("amb_learned_fft_create (C2R plan)", r);
    }
    f->has_c2r = true;
    *out = f;
    return AMB_OK;
}

extern "C" int amb_learned_fft_forward(void* handle, const float* field, void* spectrum, void* stream)
{
    auto* f = static_cast<LearnedFft*>(handle);
    if (!f || !field || !spectrum) return fail("amb_learned_fft_forward: bad arguments", AMB_ERR_INVALID);
    cufftResult r = cufftSetStream(f->r2c, static_cast<cudaStream_t>(stream));
    if (r == CUFFT_SUCCESS)
        r = cufftExecR2C(f->r2c, const_cast<cufftReal*>(field), static_cast<cufftComplex*>(spectrum));
    return r == CUFFT_SUCCESS ? AMB_OK : fail_cufft("amb_learned_fft_forward", r);
}

extern "C" int amb_learned_fft_inverse2(void* handle, void* spectra, float* fields, void* stream)
{
    auto* f = static_cast<LearnedFft*>(handle);
    if (!f || !spectra || !fields) return fail("amb_learned_fft_inverse2: bad arguments", AMB_ERR_INVALID);
    cufftResult r = cufftSetStream(f->c2r, static_cast<cudaStream_t>(stream));
    if (r == CUFFT_SUCCESS) r = cufftExecC2R(f->c2r, static_cast<cufftComplex*>(spectra), fields);
    return r == CUFFT_SUCCESS ? AMB_OK : fail_cufft("amb_learned_fft_inverse2", r);
}

extern "C" void amb_learned_fft_destroy(void* handle)
{
    destroy(static_cast<LearnedFft*>(handle));
}
