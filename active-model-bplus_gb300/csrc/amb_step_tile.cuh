// Fused explicit-Euler step, shared-memory tile form.
//
// One CTA produces a TY x TX tile of phi(t+dt) from a (TY+18) x (TX+18) tile
// of phi(t): the one-step dependency radius is 9 along each axis (mu_p needs a
// 3x3 box, J_p = -D8 mu_p and div J_p = D8 J_p add 4 + 4 along the axis).
// All five stages of the reference's three kernels (src/integrator.cu:46-110,
// 112-176, 178-262) run out of shared memory in one launch, so HBM sees one read
// and one write of phi per site-update instead of ~280 B.
//
// This is the general form: any grid size >= 1 (periodic wrap by index
// arithmetic on the halo load), FP64 or FP32 storage, Philox or injected noise.
// It is the correctness vehicle and the FP64 path; the FP32 headline path is the
// register-sliding kernel in amb_step_f32.cu.
#pragma once

#include "amb_canon.cuh"
#include "amb_common.cuh"
#include <cuda_bf16.h>

namespace amb
{
    enum NoiseMode : int { NOISE_OFF = 0, NOISE_PHILOX = 1, NOISE_INJECTED = 2 };

    // Compensation residual storage for FP32 fields: none, or a bf16 residual plane.
    enum CompMode : int { COMP_NONE = 0, COMP_BF16 = 1 };

    template <int TY, int TX>
    struct TileGeom
    {
        static constexpr int H = 9;               // phi halo
        static constexpr int LY = TY + 2 * H, LX = TX + 2 * H;
        static constexpr int MY = TY + 16, MX = TX + 16;   // mu_p box, offset 8
        static constexpr int AY = TY + 4, AX = TX + 4;     // mu_a box, offset 2
        static constexpr int CY = TY + 2, CX = TX + 2;     // J2 = J_l + J_c box, offset 1
        static constexpr int PY = TY + 8;                  // J1_y rows [-4, TY+4), cols [0, TX)
        static constexpr int QX = TX + 8;                  // J1_x rows [0, TY), cols [-4, TX+4)
        template <typename Real>
        static constexpr size_t smem_bytes()
        {
            return sizeof(Real) * (size_t(LY) * LX + size_t(MY) * MX + size_t(AY) * AX + 2 * size_t(CY) * CX
                                   + size_t(PY) * TX + size_t(TY) * QX);
        }
    };

    // Loads of the field a step reads. A persistent launch reads rows that other CTAs wrote
    // earlier in the same launch: those loads go through L2 only (ld.global.cg), never a stale L1.
    template <typename Real, bool COHERENT>
    __device__ __forceinline__ Real load_field(const Real* p)
    {
        if constexpr (COHERENT) return __ldcg(p);
        else return *p;
    }

    // Work over a W-wide, H-tall index box by the CTA's NT threads: thread t owns column t % W and
    // rows t / W, t / W + NT / W, ... (threads past the last whole row of threads idle), so the
    // index arithmetic is one division per thread and box rather than one per element.
    template <int W, int H, int NT, typename F>
    __device__ __forceinline__ void for_box(F&& f)
    {
        static_assert(W <= NT, "box wider than the CTA");
        constexpr int R = NT / W, K = (H + R - 1) / R;
        const int t = threadIdx.x;
        if (t < R * W)
        {
            const int j = t % W, i0 = t / W;
#pragma unroll
            for (int q = 0; q < K; ++q)
                if (i0 + q * R < H) f(i0 + q * R, j);
        }
    }

    // One step of one TY x TX output tile (origin r0, c0): the whole body of the tile kernel.
    template <typename Real, int TY, int TX, int COMP, bool COHERENT, int NT>
    __device__ __forceinline__ void tile_step(const Real* __restrict__ phi_in, Real* __restrict__ phi_out,
                                              const __nv_bfloat16* comp_in, __nv_bfloat16* comp_out,
                                              const StepParams& p, const Canon<Real>& k, int noise_mode,
                                              const Real* __restrict__ injected, int r0, int c0,
                                              unsigned char* smem_raw)
    {
        using G = TileGeom<TY, TX>;
        Real* PHI = reinterpret_cast<Real*>(smem_raw);
        Real* MUP = PHI + G::LY * G::LX;
        Real* MUA = MUP + G::MY * G::MX;
        Real* J2Y = MUA + G::AY * G::AX;
        Real* J2X = J2Y + G::CY * G::CX;
        Real* J1Y = J2X + G::CY * G::CX;
        Real* J1X = J1Y + G::PY * TX;

        const int ny = p.ny, nx = p.nx;
        const int tid = threadIdx.x;

        // Load phi(t) with a 9-site periodic halo: each thread owns one column of the halo tile
        // (its periodic image computed once) and issues all its rows' loads before storing any.
        {
            constexpr int W = G::LX, R = NT / W, K = (G::LY + R - 1) / R;
            static_assert(W <= NT, "halo tile wider than the CTA");
            if (tid < R * W)
            {
                const int j = tid % W, i0 = tid / W;
                const int gc = wrap_index(c0 + j - G::H, nx);
                Real v[K];
#pragma unroll
                for (int q = 0; q < K; ++q)
                {
                    const int i = i0 + q * R;
                    if (i < G::LY)
                        v[q] = load_field<Real, COHERENT>(phi_in + (size_t)wrap_index(r0 + i - G::H, ny) * nx + gc);
                }
#pragma unroll
                for (int q = 0; q < K; ++q)
                {
                    const int i = i0 + q * R;
                    if (i < G::LY) PHI[i * G::LX + j] = v[q];
                }
            }
        }
        __syncthreads();

        // Stage A: mu_p on the (TY+16) x (TX+16) plus-shaped box; mu_a on (TY+4)^2; J_c on (TY+2)^2.
        for_box<G::MX, G::MY, NT>([&](int bi, int bj) {  // box coords, offset 8
            const int i = bi - 8, j = bj - 8;               // tile coords
            const bool in_plus = (i >= 0 && i < TY) || (j >= 0 && j < TX);
            const bool in_a = i >= -2 && i < TY + 2 && j >= -2 && j < TX + 2;
            if (!in_plus && !in_a) return;
            const int e = bi * G::MX + bj;
            const Real* m = PHI + (i + G::H) * G::LX + (j + G::H);
            if (!in_a)  // the arms of the plus need mu_p only
            {
                MUP[e] = canon_mu_p(m - G::LX, m, m + G::LX, k);
                return;
            }
            const SiteA<Real> s = canon_stage_a(m - G::LX, m, m + G::LX, k);
            MUP[e] = s.mup;
            MUA[(i + 2) * G::AX + (j + 2)] = s.mua;
            if (i >= -1 && i < TY + 1 && j >= -1 && j < TX + 1)
            {
                J2Y[(i + 1) * G::CX + (j + 1)] = s.jcy;
                J2X[(i + 1) * G::CX + (j + 1)] = s.jcx;
            }
        });
        __syncthreads();

        // Stage B: J1 = -D8 mu_p + mag xi on the two arms, J2 = -Tj mu_a + J_c on the box. With
        // Philox noise and ncols % 4 == 0 the arms are walked by column quads, one Philox call per
        // quad (the tile origin is a multiple of 4, so quads align with the noise's quads).
        const size_t plane = (size_t)ny * nx;
        const auto j1y_at = [&](int i, int j, Real xi) {  // row i in [-4, TY+4), column j in [0, TX)
            const Real* c = MUP + (i + 8) * G::MX + (j + 8);
            constexpr int L = G::MX;
            return rfma(k.mag, xi, canon_d8(k.ny8, c[-L], c[L], c[-2 * L], c[2 * L], c[-3 * L], c[3 * L], c[-4 * L],
                                            c[4 * L]));
        };
        const auto j1x_at = [&](int i, int j, Real xi) {  // row i in [0, TY), column j in [-4, TX+4)
            const Real* c = MUP + (i + 8) * G::MX + (j + 8);
            return rfma(k.mag, xi, canon_d8(k.nx8, c[-1], c[1], c[-2], c[2], c[-3], c[3], c[-4], c[4]));
        };
        if (noise_mode == NOISE_PHILOX && nx % 4 == 0)
        {
            constexpr int QY = TX / 4, QQ = G::QX / 4;
            for_box<QY, G::PY, NT>([&](int ii, int qj) {  // J1_y rows ii - 4, column quad qj
                const int i = ii - 4, j = qj * 4;
                float z[4];
                noise_quad(p.seed, p.step, wrap_index(r0 + i, ny), wrap_index(c0 + j, nx), 0, z);
#pragma unroll
                for (int q = 0; q < 4; ++q) J1Y[ii * TX + j + q] = j1y_at(i, j + q, Real(z[q]));
            });
            for_box<QQ, TY, NT>([&](int i, int qj) {  // J1_x row i, column quad qj (columns from -4)
                const int j = qj * 4 - 4;
                float z[4];
                noise_quad(p.seed, p.step, wrap_index(r0 + i, ny), wrap_index(c0 + j, nx), 1, z);
#pragma unroll
                for (int q = 0; q < 4; ++q) J1X[i * G::QX + j + q + 4] = j1x_at(i, j + q, Real(z[q]));
            });
        }
        else
        {
            for_box<TX, G::PY, NT>([&](int ii, int j) {
                const int i = ii - 4;
                Real xi = 0;
                if (noise_mode != NOISE_OFF)
                {
                    int gr = wrap_index(r0 + i, ny), gc = wrap_index(c0 + j, nx);
                    xi = noise_mode == NOISE_PHILOX ? Real(noise_normal(p.seed, p.step, gr, gc, 0))
                                                    : injected[(size_t)gr * nx + gc];
                }
                J1Y[ii * TX + j] = j1y_at(i, j, xi);
            });
            for_box<G::QX, TY, NT>([&](int i, int jj) {
                const int j = jj - 4;
                Real xi = 0;
                if (noise_mode != NOISE_OFF)
                {
                    int gr = wrap_index(r0 + i, ny), gc = wrap_index(c0 + j, nx);
                    xi = noise_mode == NOISE_PHILOX ? Real(noise_normal(p.seed, p.step, gr, gc, 1))
                                                    : injected[plane + (size_t)gr * nx + gc];
                }
                J1X[i * G::QX + jj] = j1x_at(i, j, xi);
            });
        }
        for_box<G::CX, G::CY, NT>([&](int ci, int cj) {
            const int e = ci * G::CX + cj;
            const Real* a0 = MUA + ci * G::AX + cj + 1;     // mu_a row above, centre column
            const Real* a1 = a0 + G::AX;                    // (box offset 1: rows ci-1..ci+1 of mu_a are its rows ci..ci+2)
            const Real* a2 = a1 + G::AX;
            const Real sx_m = canon_smooth(a0[-1], a0[0], a0[1], k), sx_p = canon_smooth(a2[-1], a2[0], a2[1], k);
            const Real dx_m = rsub(a0[1], a0[-1]), dx_0 = rsub(a1[1], a1[-1]), dx_p = rsub(a2[1], a2[-1]);
            J2Y[e] = canon_j2y(sx_m, sx_p, J2Y[e], k);
            J2X[e] = canon_j2x(dx_m, dx_0, dx_p, J2X[e], k);
        });
        __syncthreads();

        // Stage C: div J and the update.
        for_box<TX, TY, NT>([&](int i, int j) {
            const int gr = r0 + i, gc = c0 + j;
            if (gr >= ny || gc >= nx) return;
            const Real* y0 = J2Y + i * G::CX + j + 1;       // J2 rows i-1, i, i+1 at J2 rows i, i+1, i+2
            const Real* y2 = y0 + 2 * G::CX;
            const Real* x0 = J2X + i * G::CX + j + 1;
            const Real* x1 = x0 + G::CX;
            const Real* x2 = x1 + G::CX;
            const Real divtj = canon_divtj(canon_smooth(y0[-1], y0[0], y0[1], k), canon_smooth(y2[-1], y2[0], y2[1], k),
                                           rsub(x0[1], x0[-1]), rsub(x1[1], x1[-1]), rsub(x2[1], x2[-1]), k);
            const Real* cy = J1Y + (i + 4) * TX + j;
            const Real dy8 = canon_d8(k.py8, cy[-TX], cy[TX], cy[-2 * TX], cy[2 * TX], cy[-3 * TX], cy[3 * TX],
                                      cy[-4 * TX], cy[4 * TX]);
            const Real* cx = J1X + i * G::QX + j + 4;
            const Real dx8 = canon_d8(k.px8, cx[-1], cx[1], cx[-2], cx[2], cx[-3], cx[3], cx[-4], cx[4]);
            const Real f = PHI[(i + G::H) * G::LX + (j + G::H)];
            const size_t gi = (size_t)gr * nx + gc;
            if constexpr (COMP == COMP_BF16)
            {
                float r = __bfloat162float(load_field<__nv_bfloat16, COHERENT>(comp_in + gi));
                phi_out[gi] = canon_update_comp(f, dx8, divtj, dy8, r, k);
                comp_out[gi] = __float2bfloat16_rn(r);
            }
            else
            {
                phi_out[gi] = canon_update(f, dx8, divtj, dy8, k);
            }
        });
    }

    // One step, one tile per CTA (grid = tiles). Both tile kernels are built for 1024 threads per
    // SM (at most 64 registers per thread).
    template <typename Real, int TY, int TX, int COMP, int NT>
    __global__ void __launch_bounds__(NT, 1024 / NT)
    step_tile_kernel(const Real* __restrict__ phi_in, Real* __restrict__ phi_out,
                     const __nv_bfloat16* comp_in, __nv_bfloat16* comp_out,  // may alias: each site reads/writes only its own
                     StepParams p, const Canon<Real> k, int noise_mode, const Real* __restrict__ injected)
    {
        extern __shared__ __align__(16) unsigned char smem_raw[];
        tile_step<Real, TY, TX, COMP, false, NT>(phi_in, phi_out, comp_in, comp_out, p, k, noise_mode, injected,
                                             blockIdx.y * TY, blockIdx.x * TX, smem_raw);
    }

    constexpr long long kGridBarrierSpin = 1ll << 24;  // ~1 s of polling at >= 64 ns per poll

    // Bounded grid-wide barrier of a cooperative launch: every CTA adds one arrival to *count and
    // waits until `target` arrivals are there. Returns false (and sets *error) if the wait gave up.
    __device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned target, int* error, int* ok_smem)
    {
        __syncthreads();
        if (threadIdx.x == 0)
        {
            __threadfence();
            atomicAdd(count, 1u);
            bool done = false;
            for (long long it = 0; it < kGridBarrierSpin; ++it)
            {
                if (*reinterpret_cast<volatile unsigned*>(count) >= target)
                {
                    done = true;
                    break;
                }
                __nanosleep(64);
            }
            if (!done) atomicOr(error, 1);
            __threadfence();
            *ok_smem = done ? 1 : 0;
        }
        __syncthreads();
        return *ok_smem != 0;
    }

    // nsteps steps in one cooperative launch: each CTA owns tiles blockIdx.x, +gridDim.x, ... for
    // the whole launch, and a bounded grid barrier separates the steps. Step s reads buf[s % 2]
    // and writes buf[(s + 1) % 2]. The per-site arithmetic is the tile kernel's (tile_step), so
    // the result is bitwise that of nsteps single-step launches. If a barrier gives up, the CTA
    // fills its tiles of both buffers with NaN (caught by the finite check) and leaves.
    template <typename Real, int TY, int TX, int COMP, int NT>
    __global__ void __launch_bounds__(NT, 1024 / NT)
    step_tile_persistent_kernel(Real* buf0, Real* buf1, __nv_bfloat16* comp, StepParams p, const Canon<Real> k,
                                int noise_mode, const Real* __restrict__ injected, int nsteps, unsigned* count,
                                int* error)
    {
        extern __shared__ __align__(16) unsigned char smem_raw[];
        __shared__ int ok;
        const int tx = (p.nx + TX - 1) / TX, ty = (p.ny + TY - 1) / TY;
        const int ntiles = tx * ty;
        const size_t plane = (size_t)p.ny * p.nx;
        const int64_t step0 = p.step;
        for (int s = 0; s < nsteps; ++s)
        {
            const Real* in = (s & 1) ? buf1 : buf0;
            Real* out = (s & 1) ? buf0 : buf1;
            p.step = step0 + s;
            const Real* inj = injected ? injected + (size_t)s * 2 * plane : nullptr;
            for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
            {
                tile_step<Real, TY, TX, COMP, true, NT>(in, out, comp, comp, p, k, noise_mode, inj, (tile / tx) * TY,
                                                    (tile % tx) * TX, smem_raw);
                __syncthreads();
            }
            if (s + 1 < nsteps && !grid_barrier(count, unsigned(s + 1) * gridDim.x, error, &ok))
            {
                const Real nan = Real(__int_as_float(0x7fc00000));
                for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
                    for (int e = threadIdx.x; e < TY * TX; e += blockDim.x)
                    {
                        const int r = (tile / tx) * TY + e / TX, c = (tile % tx) * TX + e % TX;
                        if (r < p.ny && c < p.nx)
                        {
                            buf0[(size_t)r * p.nx + c] = nan;
                            buf1[(size_t)r * p.nx + c] = nan;
                        }
                    }
                return;
            }
        }
    }
}
