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

    template <typename Real>
    struct Coefs
    {
        Real dt, dxInv, dyInv, ex, ey, a, b, c, kappa, lambda, zeta, mag;
        __device__ __forceinline__ explicit Coefs(const StepParams& p)
            : dt(Real(p.dt)), dxInv(Real(p.dxInv)), dyInv(Real(p.dyInv)),
              ex(Real(p.dxInv * p.dxInv)), ey(Real(p.dyInv * p.dyInv)),
              a(Real(p.a)), b(Real(p.b)), c(Real(p.c)), kappa(Real(p.kappa)),
              lambda(Real(p.lambda)), zeta(Real(p.zeta)), mag(Real(p.noise_mag)) {}
    };

    // Tjhung first derivative along x of a row-major array at (i, j), unscaled.
    template <typename Real>
    __device__ __forceinline__ Real tj_x(const Real* f, int ld, int i, int j)
    {
        const Real* u = f + (i - 1) * ld + j;
        const Real* m = f + i * ld + j;
        const Real* d = f + (i + 1) * ld + j;
        return Real(0.1) * ((u[1] - u[-1]) + (d[1] - d[-1])) + Real(0.3) * (m[1] - m[-1]);
    }

    template <typename Real>
    __device__ __forceinline__ Real tj_y(const Real* f, int ld, int i, int j)
    {
        const Real* u = f + (i - 1) * ld + j;
        const Real* d = f + (i + 1) * ld + j;
        return Real(0.1) * ((d[-1] - u[-1]) + (d[1] - u[1])) + Real(0.3) * (d[0] - u[0]);
    }

    template <typename Real>
    __device__ __forceinline__ Real d8_x(const Real* f, int ld, int i, int j)
    {
        const Real* m = f + i * ld + j;
        return Real(d8_tap(1)) * (m[1] - m[-1]) + Real(d8_tap(2)) * (m[2] - m[-2])
             + Real(d8_tap(3)) * (m[3] - m[-3]) + Real(d8_tap(4)) * (m[4] - m[-4]);
    }

    template <typename Real>
    __device__ __forceinline__ Real d8_y(const Real* f, int ld, int i, int j)
    {
        const Real* m = f + i * ld + j;
        return Real(d8_tap(1)) * (m[ld] - m[-ld]) + Real(d8_tap(2)) * (m[2 * ld] - m[-2 * ld])
             + Real(d8_tap(3)) * (m[3 * ld] - m[-3 * ld]) + Real(d8_tap(4)) * (m[4 * ld] - m[-4 * ld]);
    }

    // Stage 1 at one site: Laplacian and gradient of phi from its 3x3 box.
    template <typename Real>
    struct LocalTerms { Real lap, gy, gx; };

    template <typename Real>
    __device__ __forceinline__ LocalTerms<Real> local_terms(const Real* f, int ld, int i, int j, const Coefs<Real>& k)
    {
        const Real* u = f + (i - 1) * ld + j;
        const Real* m = f + i * ld + j;
        const Real* d = f + (i + 1) * ld + j;
        // second differences along x per row, along y per column
        Real sx_u = u[-1] - Real(2) * u[0] + u[1];
        Real sx_m = m[-1] - Real(2) * m[0] + m[1];
        Real sx_d = d[-1] - Real(2) * d[0] + d[1];
        Real sy_l = u[-1] - Real(2) * m[-1] + d[-1];
        Real sy_c = u[0] - Real(2) * m[0] + d[0];
        Real sy_r = u[1] - Real(2) * m[1] + d[1];
        Real second_x = Real(-0.25) * (sx_u + sx_d) + Real(1.5) * sx_m;
        Real second_y = Real(-0.25) * (sy_l + sy_r) + Real(1.5) * sy_c;
        LocalTerms<Real> t;
        t.lap = k.ex * second_x + k.ey * second_y;
        t.gx = k.dxInv * (Real(0.1) * ((u[1] - u[-1]) + (d[1] - d[-1])) + Real(0.3) * (m[1] - m[-1]));
        t.gy = k.dyInv * (Real(0.1) * ((d[-1] - u[-1]) + (d[1] - u[1])) + Real(0.3) * (d[0] - u[0]));
        return t;
    }

    // Compensated (Kahan) update phi += inc with residual `comp` carried between steps.
    __device__ __forceinline__ float kahan_add(float phi, float inc, float& comp)
    {
        float y = inc - comp;
        float t = phi + y;
        comp = (t - phi) - y;
        return t;
    }

    template <typename Real, int TY, int TX, int COMP>
    __global__ void __launch_bounds__(256)
    step_tile_kernel(const Real* __restrict__ phi_in, Real* __restrict__ phi_out,
                     const __nv_bfloat16* comp_in, __nv_bfloat16* comp_out,  // may alias: each site reads/writes only its own
                     StepParams p, int noise_mode, const Real* __restrict__ injected)
    {
        using G = TileGeom<TY, TX>;
        extern __shared__ __align__(16) unsigned char smem_raw[];
        Real* PHI = reinterpret_cast<Real*>(smem_raw);
        Real* MUP = PHI + G::LY * G::LX;
        Real* MUA = MUP + G::MY * G::MX;
        Real* J2Y = MUA + G::AY * G::AX;
        Real* J2X = J2Y + G::CY * G::CX;
        Real* J1Y = J2X + G::CY * G::CX;
        Real* J1X = J1Y + G::PY * TX;

        const Coefs<Real> k(p);
        const int ny = p.ny, nx = p.nx;
        const int r0 = blockIdx.y * TY, c0 = blockIdx.x * TX;
        const int tid = threadIdx.x, nthr = blockDim.x;

        // Load phi(t) with a 9-site periodic halo.
        for (int e = tid; e < G::LY * G::LX; e += nthr)
        {
            int i = e / G::LX, j = e - i * G::LX;
            int gr = wrap_index(r0 + i - G::H, ny);
            int gc = wrap_index(c0 + j - G::H, nx);
            PHI[e] = phi_in[(size_t)gr * nx + gc];
        }
        __syncthreads();

        // Stage 1: mu_p on the (TY+16) x (TX+16) box; mu_a on (TY+4)^2; J_c on (TY+2)^2.
        for (int e = tid; e < G::MY * G::MX; e += nthr)
        {
            int bi = e / G::MX, bj = e - bi * G::MX;      // box coords, offset 8
            int i = bi - 8, j = bj - 8;                     // tile coords
            bool in_plus = (i >= 0 && i < TY) || (j >= 0 && j < TX);
            bool in_a = i >= -2 && i < TY + 2 && j >= -2 && j < TX + 2;
            if (!in_plus && !in_a) continue;
            int pi = i + G::H, pj = j + G::H;
            LocalTerms<Real> t = local_terms(PHI, G::LX, pi, pj, k);
            Real f = PHI[pi * G::LX + pj];
            MUP[e] = f * (k.a + f * (k.b + k.c * f)) - k.kappa * t.lap;
            if (in_a)
            {
                MUA[(i + 2) * G::AX + (j + 2)] = k.lambda * (t.gy * t.gy + t.gx * t.gx);
                if (i >= -1 && i < TY + 1 && j >= -1 && j < TX + 1)
                {
                    Real zl = k.zeta * t.lap;
                    J2Y[(i + 1) * G::CX + (j + 1)] = zl * t.gy;
                    J2X[(i + 1) * G::CX + (j + 1)] = zl * t.gx;
                }
            }
        }
        __syncthreads();

        // Stage 2: J1 = J_p + J_r on the two arms, J2 = J_l + J_c on the box. With Philox
        // noise and ncols % 4 == 0 the arms are walked by column quads, one Philox call per
        // quad (the tile origin is a multiple of 4, so quads align with the noise's quads).
        const size_t plane = (size_t)ny * nx;
        if (noise_mode == NOISE_PHILOX && nx % 4 == 0)
        {
            constexpr int QY = TX / 4, QQ = G::QX / 4;
            for (int e = tid; e < G::PY * QY; e += nthr)
            {
                int i = e / QY - 4, j = (e % QY) * 4;
                float z[4];
                noise_quad(p.seed, p.step, wrap_index(r0 + i, ny), wrap_index(c0 + j, nx), 0, z);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    J1Y[(i + 4) * TX + j + q] = -(k.dyInv * d8_y(MUP, G::MX, i + 8, j + q + 8)) + k.mag * Real(z[q]);
            }
            for (int e = tid; e < TY * QQ; e += nthr)
            {
                int i = e / QQ, j = (e % QQ) * 4 - 4;
                float z[4];
                noise_quad(p.seed, p.step, wrap_index(r0 + i, ny), wrap_index(c0 + j, nx), 1, z);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    J1X[i * G::QX + j + q + 4] = -(k.dxInv * d8_x(MUP, G::MX, i + 8, j + q + 8)) + k.mag * Real(z[q]);
            }
        }
        else
        {
            for (int e = tid; e < G::PY * TX; e += nthr)
            {
                int i = e / TX - 4, j = e % TX;
                Real xi = 0;
                if (noise_mode != NOISE_OFF)
                {
                    int gr = wrap_index(r0 + i, ny), gc = wrap_index(c0 + j, nx);
                    xi = noise_mode == NOISE_PHILOX ? Real(noise_normal(p.seed, p.step, gr, gc, 0))
                                                    : injected[(size_t)gr * nx + gc];
                }
                J1Y[e] = -(k.dyInv * d8_y(MUP, G::MX, i + 8, j + 8)) + k.mag * xi;
            }
            for (int e = tid; e < TY * G::QX; e += nthr)
            {
                int i = e / G::QX, j = e % G::QX - 4;
                Real xi = 0;
                if (noise_mode != NOISE_OFF)
                {
                    int gr = wrap_index(r0 + i, ny), gc = wrap_index(c0 + j, nx);
                    xi = noise_mode == NOISE_PHILOX ? Real(noise_normal(p.seed, p.step, gr, gc, 1))
                                                    : injected[plane + (size_t)gr * nx + gc];
                }
                J1X[e] = -(k.dxInv * d8_x(MUP, G::MX, i + 8, j + 8)) + k.mag * xi;
            }
        }
        for (int e = tid; e < G::CY * G::CX; e += nthr)
        {
            int ci = e / G::CX, cj = e - ci * G::CX;      // offset 1
            J2Y[e] += -(k.dyInv * tj_y(MUA, G::AX, ci + 1, cj + 1));
            J2X[e] += -(k.dxInv * tj_x(MUA, G::AX, ci + 1, cj + 1));
        }
        __syncthreads();

        // Stage 3: div J and the update.
        for (int e = tid; e < TY * TX; e += nthr)
        {
            int i = e / TX, j = e - i * TX;
            int gr = r0 + i, gc = c0 + j;
            if (gr >= ny || gc >= nx) continue;
            Real div = k.dyInv * tj_y(J2Y, G::CX, i + 1, j + 1) + k.dxInv * tj_x(J2X, G::CX, i + 1, j + 1)
                     + k.dyInv * d8_y(J1Y, TX, i + 4, j) + k.dxInv * d8_x(J1X, G::QX, i, j + 4);
            Real f = PHI[(i + G::H) * G::LX + (j + G::H)];
            size_t gi = (size_t)gr * nx + gc;
            if constexpr (COMP == COMP_BF16)
            {
                float comp = __bfloat162float(comp_in[gi]);
                float nf = kahan_add(float(f), -float(k.dt) * float(div), comp);
                phi_out[gi] = Real(nf);
                comp_out[gi] = __float2bfloat16_rn(comp);
            }
            else
            {
                phi_out[gi] = f - k.dt * div;
            }
        }
    }
}
