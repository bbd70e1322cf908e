// Host driver for the reference's own CUDA integrator — baseline/test
// infrastructure, not the product.
//
// The reference's device code (src/integrator.cu + src/parameters.cu) is compiled
// from the read-only reference checkout into one relinked cubin by
// oracle/build.py (output oracle/_ref/ref_integrator.cubin, git-ignored). This
// driver loads that cubin with the CUDA driver API and replays what the
// reference's host class does, call for call:
//   ctor  (src/integrator.cu:288-333): device buffers, zeroed currents, curand
//         state, __constant__ parameters (src/integrator.cu:467-475),
//         init_random_state<<<grid, 8x8>>>.
//   run   (src/integrator.cu:497-538): lazily calculate_forces +
//         calculate_local_currents, then per step step / calculate_forces /
//         calculate_local_currents, timestep += n, synchronise, check_finite.
// Launch shapes follow src/integrator.cu:482-484 (8x8 blocks). Kernel and symbol
// names are the C++ names of the reference's kernels (mangled).
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace
{
    struct Stencil4 { double dt, dxInv, dyInv, noise_strength; };                 // DeviceStencilParams
    struct Model8 { double a, b, c, kappa, lambda, zeta, temperature, noise; };    // DeviceModelParams
    struct Pair { double* p[2]; };                                                // DeviceCurrent

    constexpr size_t kCurandStateBytes = 48;  // sizeof(curandStateXORWOW)

    std::string g_err;
    CUmodule g_mod = nullptr;
    CUfunction f_step, f_forces, f_currents, f_init, f_finite;
    CUdeviceptr c_stencil, c_nrows, c_ncols, c_model;

    int fail(CUresult r, const char* where)
    {
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        g_err = std::string(where) + ": " + (s ? s : "CUDA driver error");
        return 1;
    }

    struct RefIntegrator
    {
        int nrows, ncols;
        Stencil4 st;
        Model8 md;
        CUdeviceptr field, mup, mua, state;
        Pair pass, lamb, circ, rand;
        long long timestep = 0, computed = -1;
        size_t bytes() const { return size_t(nrows) * ncols * sizeof(double); }
    };

    int set_params(RefIntegrator* h)
    {
        CUresult r;
        if ((r = cuMemcpyHtoD(c_stencil, &h->st, sizeof(h->st)))) return fail(r, "stencil");
        if ((r = cuMemcpyHtoD(c_nrows, &h->nrows, sizeof(int)))) return fail(r, "nrows");
        if ((r = cuMemcpyHtoD(c_ncols, &h->ncols, sizeof(int)))) return fail(r, "ncols");
        if ((r = cuMemcpyHtoD(c_model, &h->md, sizeof(h->md)))) return fail(r, "model");
        return 0;
    }

    int launch(CUfunction f, RefIntegrator* h, void** args)
    {
        unsigned gx = (h->ncols + 7) / 8, gy = (h->nrows + 7) / 8;
        CUresult r = cuLaunchKernel(f, gx, gy, 1, 8, 8, 1, 0, nullptr, args, nullptr);
        return r ? fail(r, "launch") : 0;
    }

    int forces_and_currents(RefIntegrator* h)
    {
        void* a1[] = {&h->field, &h->mup, &h->mua, &h->circ, &h->rand, &h->state};
        if (launch(f_forces, h, a1)) return 1;
        void* a2[] = {&h->mup, &h->mua, &h->pass, &h->lamb};
        return launch(f_currents, h, a2);
    }
}

extern "C"
{
    const char* refgpu_last_error(void) { return g_err.c_str(); }

    // Load the cubin into the current (primary) context of device 0.
    int refgpu_load(const char* cubin_path)
    {
        CUresult r;
        if ((r = cuInit(0))) return fail(r, "cuInit");
        CUdevice dev;
        if ((r = cuDeviceGet(&dev, 0))) return fail(r, "cuDeviceGet");
        CUcontext ctx;
        if ((r = cuDevicePrimaryCtxRetain(&ctx, dev))) return fail(r, "cuDevicePrimaryCtxRetain");
        if ((r = cuCtxSetCurrent(ctx))) return fail(r, "cuCtxSetCurrent");
        if (g_mod) return 0;
        if ((r = cuModuleLoad(&g_mod, cubin_path))) return fail(r, "cuModuleLoad");
        struct { CUfunction* f; const char* name; } fns[] = {
            {&f_step, "_ZN6kernel4stepEPdSt5arrayIS0_Lm2EES2_S2_S2_"},
            {&f_forces, "_ZN6kernel16calculate_forcesEPdS0_S0_St5arrayIS0_Lm2EES2_P17curandStateXORWOW"},
            {&f_currents, "_ZN6kernel24calculate_local_currentsEPdS0_St5arrayIS0_Lm2EES2_"},
            {&f_init, "_ZN6kernel17init_random_stateEP17curandStateXORWOWy"},
            {&f_finite, "_ZN6kernel12check_finiteEPdPb"},
        };
        for (auto& e : fns)
            if ((r = cuModuleGetFunction(e.f, g_mod, e.name))) return fail(r, e.name);
        size_t sz;
        if ((r = cuModuleGetGlobal(&c_stencil, &sz, g_mod, "_ZN6kernel7stencilE")) || sz != sizeof(Stencil4))
            return fail(r ? r : CUDA_ERROR_INVALID_VALUE, "kernel::stencil");
        if ((r = cuModuleGetGlobal(&c_nrows, &sz, g_mod, "_ZN6kernel5nrowsE"))) return fail(r, "kernel::nrows");
        if ((r = cuModuleGetGlobal(&c_ncols, &sz, g_mod, "_ZN6kernel5ncolsE"))) return fail(r, "kernel::ncols");
        if ((r = cuModuleGetGlobal(&c_model, &sz, g_mod, "_ZN6kernel5modelE")) || sz != sizeof(Model8))
            return fail(r ? r : CUDA_ERROR_INVALID_VALUE, "kernel::model");
        return 0;
    }

    // Integrator(field, stencil, model) with an explicit curand seed.
    int refgpu_create(const double* host_field, int nrows, int ncols, const double stencil[3], const double model[7],
                      unsigned long long seed, void** out)
    {
        if (!g_mod) { g_err = "refgpu_load first"; return 1; }
        if (nrows < 8 || ncols < 8 || nrows % 8 || ncols % 8)
        {
            g_err = "the reference integrator needs nrows, ncols multiples of 8";
            return 1;
        }
        auto* h = new RefIntegrator{};
        h->nrows = nrows;
        h->ncols = ncols;
        h->st = {stencil[0], 1 / stencil[1], 1 / stencil[2], std::sqrt(1. / (stencil[0] * stencil[1] * stencil[2]))};
        h->md = {model[0], model[1], model[2], model[3], model[4], model[5], model[6], std::sqrt(2 * model[6])};
        CUresult r = CUDA_SUCCESS;
        std::vector<CUdeviceptr*> planes = {&h->field, &h->mup, &h->mua};
        for (Pair* pr : {&h->pass, &h->lamb, &h->circ, &h->rand})
            for (int c = 0; c < 2; ++c) planes.push_back(reinterpret_cast<CUdeviceptr*>(&pr->p[c]));
        for (CUdeviceptr* p : planes)
        {
            if ((r = cuMemAlloc(p, h->bytes()))) break;
            if ((r = cuMemsetD8(*p, 0, h->bytes()))) break;
        }
        if (!r) r = cuMemAlloc(&h->state, size_t(nrows) * ncols * kCurandStateBytes);
        if (!r) r = cuMemcpyHtoD(h->field, host_field, h->bytes());
        if (r) { delete h; return fail(r, "refgpu_create"); }
        if (set_params(h)) { delete h; return 1; }
        void* args[] = {&h->state, &seed};
        if (launch(f_init, h, args)) { delete h; return 1; }
        if ((r = cuCtxSynchronize())) { delete h; return fail(r, "init_random_state"); }
        *out = h;
        return 0;
    }

    // Integrator::run(nsteps). Returns 2 when the field is no longer finite.
    int refgpu_run(void* handle, int nsteps)
    {
        auto* h = static_cast<RefIntegrator*>(handle);
        if (h->computed != h->timestep)
        {
            if (set_params(h) || forces_and_currents(h)) return 1;
            h->computed = h->timestep;
        }
        if (set_params(h)) return 1;
        for (int i = 0; i < nsteps; ++i)
        {
            void* a[] = {&h->field, &h->pass, &h->lamb, &h->circ, &h->rand};
            if (launch(f_step, h, a) || forces_and_currents(h)) return 1;
        }
        h->timestep += nsteps;
        h->computed = h->timestep;
        CUresult r = cuCtxSynchronize();
        if (r) return fail(r, "run");
        CUdeviceptr flag;
        if ((r = cuMemAlloc(&flag, 1))) return fail(r, "flag");
        unsigned char one = 1, got = 1;
        cuMemcpyHtoD(flag, &one, 1);
        void* a[] = {&h->field, &flag};
        if (launch(f_finite, h, a)) { cuMemFree(flag); return 1; }
        r = cuMemcpyDtoH(&got, flag, 1);
        cuMemFree(flag);
        if (r) return fail(r, "finite flag");
        if (!got) { g_err = "an unknown numerical error occurred during simulation"; return 2; }
        return 0;
    }

    int refgpu_get_field(void* handle, double* out)
    {
        auto* h = static_cast<RefIntegrator*>(handle);
        CUresult r = cuMemcpyDtoH(out, h->field, h->bytes());
        return r ? fail(r, "get_field") : 0;
    }

    // Device time of nsteps of run()'s loop (3 launches per step), CUDA events.
    int refgpu_time_steps(void* handle, int nsteps, float* ms)
    {
        auto* h = static_cast<RefIntegrator*>(handle);
        CUevent e0, e1;
        cuEventCreate(&e0, CU_EVENT_DEFAULT);
        cuEventCreate(&e1, CU_EVENT_DEFAULT);
        if (set_params(h)) return 1;
        cuEventRecord(e0, nullptr);
        for (int i = 0; i < nsteps; ++i)
        {
            void* a[] = {&h->field, &h->pass, &h->lamb, &h->circ, &h->rand};
            if (launch(f_step, h, a) || forces_and_currents(h)) return 1;
        }
        cuEventRecord(e1, nullptr);
        CUresult r = cuEventSynchronize(e1);
        if (!r) r = cuEventElapsedTime(ms, e0, e1);
        cuEventDestroy(e0);
        cuEventDestroy(e1);
        h->timestep += nsteps;
        h->computed = h->timestep;
        return r ? fail(r, "time") : 0;
    }

    void refgpu_destroy(void* handle)
    {
        auto* h = static_cast<RefIntegrator*>(handle);
        if (!h) return;
        cuCtxSynchronize();
        for (CUdeviceptr p : {h->field, h->mup, h->mua, h->state}) cuMemFree(p);
        for (Pair* pr : {&h->pass, &h->lamb, &h->circ, &h->rand})
            for (int c = 0; c < 2; ++c) cuMemFree(reinterpret_cast<CUdeviceptr>(pr->p[c]));
        delete h;
    }
}
