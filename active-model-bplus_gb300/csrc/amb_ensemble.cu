// Batched ensemble: many independent replicas (any mix of grid sizes and model
// parameters, FP32 storage) advanced together. Every step is ONE launch of the
// warp-pair sliding kernel over a task table that spans all replicas; K steps
// are captured once into a CUDA graph and replayed, and the step index lives in
// device memory so the same graph serves every chunk.
//
// Task table: each replica is cut into 112-column strips and row segments, larger
// tasks first. The segment height is chosen per size class (replicas of one shape) by
// measurement at creation, starting from the occupancy model's choice for the whole
// ensemble (waves x (rows + pipeline fill) minimised).
// The reference has no counterpart: it runs one integrator per process.
#include "amb_gb300.h"
#include "amb_kernels.h"
#include "amb_step_tile.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

struct amb_ensemble
{
    int nrep = 0, precision = AMB_F32C, graph_steps = 0, parity = 0;
    bool noise = false;
    std::vector<int> ny, nx;
    std::vector<amb::EnsembleReplica> host_reps;
    std::vector<void*> allocations;
    amb::EnsembleReplica* d_reps = nullptr;
    void* d_coefs = nullptr;
    amb::EnsembleTask* d_tasks = nullptr;
    int ntasks = 0, seg_h = 0;
    bool fused = false;  // one warp per task (fused form) instead of a warp pair; chosen by measurement
    struct SizeClass
    {
        int ny, nx, seg_h;  // shape and the segment height of its tasks
    };
    std::vector<SizeClass> classes;
    std::vector<int> class_of;  // replica -> size class
    int64_t* d_step = nullptr;
    int64_t step = 0;
    int* d_flag = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one per starting parity
};

namespace
{
    int efail(int code, const std::string& msg)
    {
        amb::set_last_error(msg);
        return code;
    }

    int ecuda(cudaError_t e, const char* where)
    {
        return efail(AMB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    }

    __global__ void advance_step_kernel(int64_t* counter, int n) { *counter += n; }

    void release(amb_ensemble* h)
    {
        if (!h) return;
        if (h->stream) cudaStreamSynchronize(h->stream);
        for (auto g : h->graph)
            if (g) cudaGraphExecDestroy(g);
        for (void* p : h->allocations) cudaFree(p);
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
    }

    template <typename T>
    cudaError_t dalloc(amb_ensemble* h, T** p, size_t bytes)
    {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes);
        if (e == cudaSuccess)
        {
            h->allocations.push_back(q);
            *p = static_cast<T*>(q);
        }
        return e;
    }

    // One step for all replicas: launch with the current parity and step offset.
    cudaError_t launch_step(amb_ensemble* h, int parity, int offset)
    {
        return amb::launch_sliding_ensemble(h->d_reps, h->d_coefs, h->d_tasks, h->ntasks, parity, h->d_step, offset,
                                            h->precision == AMB_F32C ? amb::COMP_BF16 : amb::COMP_NONE,
                                            h->noise ? amb::NOISE_PHILOX : amb::NOISE_OFF, h->fused, h->stream);
    }

    // Tasks of every replica (112-column strips x row segments of its class's height), the
    // tallest first.
    std::vector<amb::EnsembleTask> make_tasks(const amb_ensemble* h)
    {
        std::vector<amb::EnsembleTask> tasks;
        for (int r = 0; r < h->nrep; ++r)
        {
            const int h_r = std::min(h->classes[h->class_of[r]].seg_h, h->ny[r]);
            const int strips = (h->nx[r] + 111) / 112;
            for (int r0 = 0; r0 < h->ny[r]; r0 += h_r)
                for (int sidx = 0; sidx < strips; ++sidx)
                    tasks.push_back({r, sidx, r0, std::min(r0 + h_r, h->ny[r])});
        }
        std::stable_sort(tasks.begin(), tasks.end(),
                         [](const amb::EnsembleTask& a, const amb::EnsembleTask& b) { return a.r1 - a.r0 > b.r1 - b.r0; });
        return tasks;
    }

    // Most tasks any segment height from 16 rows up can give (the table's capacity).
    size_t max_tasks(const amb_ensemble* h)
    {
        size_t n = 0;
        for (int r = 0; r < h->nrep; ++r) n += size_t((h->nx[r] + 111) / 112) * ((h->ny[r] + 15) / 16);
        return n;
    }

    // Segment height per size class by measurement: one pass over the classes (most sites
    // first), each trying heights of its rows / 1, 2, 3, 4, 6, 8 (at least 16) with the other
    // classes fixed, timing three whole-ensemble launches per candidate (CUDA events) and keeping
    // the fastest; one such pass with the warp-pair kernel and one with the fused single-warp
    // kernel, and the faster of the two is kept. The launches read the initial fields (parity 0) and write the spare buffers; the
    // compensation residuals they touch are zeroed afterwards, so the ensemble starts unchanged.
    // Every candidate gives bitwise the same fields: only the time differs.
    cudaError_t tune_segments(amb_ensemble* h)
    {
        cudaEvent_t t0, t1;
        cudaError_t e = cudaEventCreate(&t0);
        if (e == cudaSuccess) e = cudaEventCreate(&t1);
        const auto time_table = [&](float* ms) -> cudaError_t {
            std::vector<amb::EnsembleTask> tasks = make_tasks(h);
            h->ntasks = int(tasks.size());
            cudaError_t err = cudaMemcpyAsync(h->d_tasks, tasks.data(), sizeof(amb::EnsembleTask) * tasks.size(),
                                              cudaMemcpyHostToDevice, h->stream);
            if (err == cudaSuccess) err = launch_step(h, 0, 0);  // warm-up
            if (err == cudaSuccess) err = cudaEventRecord(t0, h->stream);
            for (int i = 0; i < 3 && err == cudaSuccess; ++i) err = launch_step(h, 0, 0);
            if (err == cudaSuccess) err = cudaEventRecord(t1, h->stream);
            if (err == cudaSuccess) err = cudaEventSynchronize(t1);
            if (err == cudaSuccess) err = cudaEventElapsedTime(ms, t0, t1);
            return err;
        };
        std::vector<size_t> order(h->classes.size());
        for (size_t c = 0; c < order.size(); ++c) order[c] = c;
        std::vector<double> sites(h->classes.size(), 0.0);
        for (int r = 0; r < h->nrep; ++r) sites[h->class_of[r]] += double(h->ny[r]) * h->nx[r];
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return sites[a] > sites[b]; });
        // one coordinate-descent pass per form (warp pair, fused single warp); the faster form wins
        const auto pass = [&](float* best_ms) {
            if (e == cudaSuccess) e = time_table(best_ms);
            for (size_t c : order)
            {
                auto& cl = h->classes[c];
                const int keep = cl.seg_h;
                int best_h = keep;
                for (int div : {1, 2, 3, 4, 6, 8})
                {
                    const int H = std::max(16, (cl.ny + div - 1) / div);
                    if (e != cudaSuccess || H == keep || (div > 1 && H >= cl.ny)) continue;
                    cl.seg_h = H;
                    float ms = 0.f;
                    e = time_table(&ms);
                    if (e == cudaSuccess && ms < *best_ms)
                    {
                        *best_ms = ms;
                        best_h = H;
                    }
                }
                cl.seg_h = best_h;
            }
        };
        const std::vector<amb_ensemble::SizeClass> start = h->classes;
        float pair_ms = 0.f, fused_ms = 0.f;
        h->fused = false;
        pass(&pair_ms);
        const std::vector<amb_ensemble::SizeClass> pair_classes = h->classes;
        h->classes = start;
        h->fused = true;
        pass(&fused_ms);
        if (e == cudaSuccess && pair_ms <= fused_ms)
        {
            h->fused = false;
            h->classes = pair_classes;
        }
        if (e == cudaSuccess)
        {
            std::vector<amb::EnsembleTask> tasks = make_tasks(h);
            h->ntasks = int(tasks.size());
            e = cudaMemcpyAsync(h->d_tasks, tasks.data(), sizeof(amb::EnsembleTask) * tasks.size(),
                                cudaMemcpyHostToDevice, h->stream);
        }
        for (int r = 0; r < h->nrep && e == cudaSuccess; ++r)
            if (h->host_reps[r].residual)
                e = cudaMemsetAsync(h->host_reps[r].residual, 0, size_t(h->ny[r]) * h->nx[r] * sizeof(uint16_t),
                                    h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        return e;
    }

    // Capture graph_steps (even) steps from the current parity, and the counter advance,
    // into one executable graph.
    int build_graph(amb_ensemble* h)
    {
        cudaGraphExec_t* slot = &h->graph[h->parity];
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return ecuda(e, "amb_ensemble graph capture");
        for (int s = 0; s < h->graph_steps && e == cudaSuccess; ++s) e = launch_step(h, (h->parity + s) & 1, s);
        if (e == cudaSuccess)
        {
            advance_step_kernel<<<1, 1, 0, h->stream>>>(h->d_step, h->graph_steps);
            e = cudaGetLastError();
        }
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(slot, g, 0);
        if (g) cudaGraphDestroy(g);
        return e == cudaSuccess ? AMB_OK : ecuda(e, "amb_ensemble graph");
    }
}

extern "C" int amb_ensemble_create(int nreplicas, const int* nrows, const int* ncols, const double* const* host_fields,
                                   const amb_stencil* stencils, const amb_model* models, const uint64_t* seeds,
                                   int precision, int graph_steps, amb_ensemble** out)
{
    if (!out) return efail(AMB_ERR_INVALID, "out must not be NULL");
    *out = nullptr;
    if (nreplicas < 1 || !nrows || !ncols || !host_fields || !stencils || !models || !seeds)
        return efail(AMB_ERR_INVALID, "amb_ensemble_create: bad arguments");
    if (precision != AMB_F32 && precision != AMB_F32C)
        return efail(AMB_ERR_INVALID, "amb_ensemble_create: precision must be AMB_F32 or AMB_F32C");
    if (graph_steps < 0 || graph_steps % 2)
        return efail(AMB_ERR_INVALID, "amb_ensemble_create: graph_steps must be even and >= 0");
    for (int r = 0; r < nreplicas; ++r)
        if (nrows[r] < 1 || ncols[r] < 112 || ncols[r] % 4 || !host_fields[r])
            return efail(AMB_ERR_INVALID, "amb_ensemble_create: replica " + std::to_string(r)
                                              + " needs nrows >= 1, ncols >= 112 and ncols % 4 == 0");

    auto* h = new (std::nothrow) amb_ensemble;
    if (!h) return efail(AMB_ERR_NOMEM, "host allocation failed");
    h->nrep = nreplicas;
    h->precision = precision;
    h->graph_steps = graph_steps;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    std::vector<unsigned char> coefs(amb::sliding_coef_bytes() * size_t(nreplicas));
    for (int r = 0; r < nreplicas && e == cudaSuccess; ++r)
    {
        const size_t n = size_t(nrows[r]) * ncols[r];
        h->ny.push_back(nrows[r]);
        h->nx.push_back(ncols[r]);
        amb::EnsembleReplica rep{};
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) e = dalloc(h, &rep.phi[b], n * sizeof(float));
        if (e == cudaSuccess && precision == AMB_F32C)
        {
            e = dalloc(h, &rep.residual, n * sizeof(uint16_t));
            if (e == cudaSuccess) e = cudaMemsetAsync(rep.residual, 0, n * sizeof(uint16_t), h->stream);
        }
        if (e == cudaSuccess)
        {
            std::vector<float> tmp(n);
            for (size_t i = 0; i < n; ++i) tmp[i] = float(host_fields[r][i]);
            e = cudaMemcpy(rep.phi[0], tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice);
        }
        const amb_stencil& st = stencils[r];
        const amb_model& md = models[r];
        amb::StepParams p{};
        p.ny = nrows[r];
        p.nx = ncols[r];
        p.dt = st.dt;
        p.dxInv = 1 / st.dx;
        p.dyInv = 1 / st.dy;
        p.a = md.a; p.b = md.b; p.c = md.c; p.kappa = md.kappa; p.lambda = md.lambda; p.zeta = md.zeta;
        p.noise_mag = std::sqrt(2 * md.temperature) * std::sqrt(1. / (st.dt * st.dx * st.dy));
        p.seed = seeds[r];
        if (md.temperature != 0) h->noise = true;
        rep.p = p;
        amb::sliding_make_coef(p, coefs.data() + amb::sliding_coef_bytes() * r);
        h->host_reps.push_back(rep);
    }

    // task table: a start from the occupancy model, then segment heights per size class chosen by
    // measurement (below, once the replicas are on the device)
    int resident = 0;
    if (e == cudaSuccess) e = amb::ensemble_resident_pairs(&resident, false);
    if (e == cudaSuccess)
    {
        double best = 1e300;
        for (int H = 16; H <= 1024; H += 8)
        {
            long long ntask = 0;
            for (int r = 0; r < nreplicas; ++r)
            {
                int h_r = std::min(H, h->ny[r]);
                ntask += (long long)((h->nx[r] + 111) / 112) * ((h->ny[r] + h_r - 1) / h_r);
            }
            long long waves = (ntask + resident - 1) / resident;
            double cost = double(waves) * double(H + 10);
            if (cost < best - 1e-9)
            {
                best = cost;
                h->seg_h = H;
            }
        }
        // size classes: replicas of one shape share a segment height
        for (int r = 0; r < nreplicas; ++r)
        {
            size_t c = 0;
            while (c < h->classes.size() && (h->classes[c].ny != h->ny[r] || h->classes[c].nx != h->nx[r])) ++c;
            if (c == h->classes.size()) h->classes.push_back({h->ny[r], h->nx[r], std::min(h->seg_h, h->ny[r])});
            h->class_of.push_back(int(c));
        }
    }
    std::vector<amb::EnsembleTask> tasks;
    if (e == cudaSuccess)
    {
        tasks = make_tasks(h);
        h->ntasks = int(tasks.size());
    }
    if (e == cudaSuccess) e = dalloc(h, &h->d_reps, sizeof(amb::EnsembleReplica) * nreplicas);
    if (e == cudaSuccess) e = dalloc(h, &h->d_coefs, coefs.size());
    if (e == cudaSuccess) e = dalloc(h, &h->d_tasks, sizeof(amb::EnsembleTask) * max_tasks(h));
    if (e == cudaSuccess) e = dalloc(h, &h->d_step, sizeof(int64_t));
    if (e == cudaSuccess) e = dalloc(h, &h->d_flag, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_reps, h->host_reps.data(), sizeof(amb::EnsembleReplica) * nreplicas, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_coefs, coefs.data(), coefs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_tasks, tasks.data(), sizeof(amb::EnsembleTask) * tasks.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->d_step, 0, sizeof(int64_t));
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess && h->classes.size() > 0) e = tune_segments(h);
    if (e != cudaSuccess)
    {
        int code = e == cudaErrorMemoryAllocation ? AMB_ERR_NOMEM : AMB_ERR_CUDA;
        release(h);
        return efail(code, std::string("amb_ensemble_create: ") + cudaGetErrorString(e));
    }
    *out = h;
    return AMB_OK;
}

extern "C" void amb_ensemble_destroy(amb_ensemble* h) { release(h); }

extern "C" int amb_ensemble_run(amb_ensemble* h, int nsteps)
{
    if (!h || nsteps < 0) return efail(AMB_ERR_INVALID, "amb_ensemble_run: bad arguments");
    cudaError_t e = cudaSuccess;
    int done = 0;
    if (h->graph_steps > 0 && nsteps >= h->graph_steps)
    {
        if (!h->graph[h->parity])
            if (int rc = build_graph(h)) return rc;
        for (; done + h->graph_steps <= nsteps && e == cudaSuccess; done += h->graph_steps)
            e = cudaGraphLaunch(h->graph[h->parity], h->stream);  // parity unchanged: graph_steps is even
    }
    for (int s = 0; done < nsteps && e == cudaSuccess; ++done, ++s)
    {
        e = launch_step(h, h->parity, s);
        h->parity ^= 1;
        if (e == cudaSuccess && done + 1 == nsteps)
        {
            advance_step_kernel<<<1, 1, 0, h->stream>>>(h->d_step, s + 1);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) return ecuda(e, "amb_ensemble_run");
    h->step += nsteps;
    // finite check over every replica's current field
    e = cudaMemsetAsync(h->d_flag, 0, sizeof(int), h->stream);
    for (int r = 0; r < h->nrep && e == cudaSuccess; ++r)
        e = amb::launch_nonfinite<float>(h->host_reps[r].phi[h->parity], size_t(h->ny[r]) * h->nx[r], h->d_flag,
                                         h->stream);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return ecuda(e, "amb_ensemble_run");
    if (flag) return efail(AMB_ERR_NONFINITE, "an unknown numerical error occurred during simulation");
    return AMB_OK;
}

extern "C" int amb_ensemble_get_field(amb_ensemble* h, int replica, double* host_out)
{
    if (!h || !host_out || replica < 0 || replica >= h->nrep)
        return efail(AMB_ERR_INVALID, "amb_ensemble_get_field: bad arguments");
    const size_t n = size_t(h->ny[replica]) * h->nx[replica];
    std::vector<float> tmp(n);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), h->host_reps[replica].phi[h->parity], n * sizeof(float),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return ecuda(e, "amb_ensemble_get_field");
    for (size_t i = 0; i < n; ++i) host_out[i] = double(tmp[i]);
    return AMB_OK;
}

extern "C" int amb_ensemble_form(amb_ensemble* h, int set, int* form)
{
    if (!h || set < -1 || set > 1) return efail(AMB_ERR_INVALID, "amb_ensemble_form: bad arguments");
    if (set >= 0 && (set == 1) != h->fused)
    {
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return ecuda(e, "amb_ensemble_form");
        for (auto& g : h->graph)  // captured with the other kernel
            if (g)
            {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
        h->fused = set == 1;
    }
    if (form) *form = h->fused ? 1 : 0;
    return AMB_OK;
}

extern "C" int amb_ensemble_info(const amb_ensemble* h, int64_t* timestep, int* ntasks, int* seg_rows)
{
    if (!h) return efail(AMB_ERR_INVALID, "NULL ensemble");
    if (timestep) *timestep = h->step;
    if (ntasks) *ntasks = h->ntasks;
    if (seg_rows)  // the segment height of the tallest size class
    {
        int tallest = 0;
        *seg_rows = 0;
        for (const auto& c : h->classes)
            if (c.ny > tallest)
            {
                tallest = c.ny;
                *seg_rows = c.seg_h;
            }
    }
    return AMB_OK;
}

// Device-to-device copies of every replica's current field, packed back to back in
// replica order (replica r at offset sum_{q<r} nrows_q * ncols_q). Synchronous.
extern "C" int amb_ensemble_gather(amb_ensemble* h, float* dst)
{
    if (!h || !dst) return efail(AMB_ERR_INVALID, "amb_ensemble_gather: bad arguments");
    cudaError_t e = cudaSuccess;
    size_t off = 0;
    for (int r = 0; r < h->nrep && e == cudaSuccess; ++r)
    {
        const size_t n = size_t(h->ny[r]) * h->nx[r];
        e = cudaMemcpyAsync(dst + off, h->host_reps[r].phi[h->parity], n * sizeof(float), cudaMemcpyDeviceToDevice,
                            h->stream);
        off += n;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? AMB_OK : ecuda(e, "amb_ensemble_gather");
}

extern "C" int amb_ensemble_scatter(amb_ensemble* h, const float* src)
{
    if (!h || !src) return efail(AMB_ERR_INVALID, "amb_ensemble_scatter: bad arguments");
    cudaError_t e = cudaSuccess;
    size_t off = 0;
    for (int r = 0; r < h->nrep && e == cudaSuccess; ++r)
    {
        const size_t n = size_t(h->ny[r]) * h->nx[r];
        e = cudaMemcpyAsync(h->host_reps[r].phi[h->parity], src + off, n * sizeof(float), cudaMemcpyDeviceToDevice,
                            h->stream);
        if (e == cudaSuccess && h->host_reps[r].residual)
            e = cudaMemsetAsync(h->host_reps[r].residual, 0, n * sizeof(__nv_bfloat16), h->stream);
        off += n;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? AMB_OK : ecuda(e, "amb_ensemble_scatter");
}
