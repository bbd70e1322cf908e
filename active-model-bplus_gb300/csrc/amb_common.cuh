// Shared device-side definitions for the Active Model B+ step kernels:
// per-launch parameters, the discrete operators, and the counter-based noise.
//
// Discrete operators (reference tranqui/active-model-bplus):
//   D8   order-8 central first derivative, taps (1/280, -4/105, 1/5, -4/5, 0,
//        4/5, -1/5, 4/105, -1/280) over offsets -4..4 (src/finite_difference.h:69-75);
//        antisymmetric, applied here as sum_k d_k (g[+k] - g[-k]).
//   Tj   Tjhung 3x3 first derivative [0.1, 0.3, 0.1] (smoothing, across) x
//        [-1, 0, 1] (difference, along) (src/finite_difference.h:379-387,404-407).
//   Lap  Tjhung Laplacian dxInv^2 [-.25, 1.5, -.25]_y x [1, -2, 1]_x +
//        dyInv^2 [1, -2, 1]_y x [-.25, 1.5, -.25]_x (src/finite_difference.h:389-412,
//        src/finite_difference.cuh:178-183).
// All are applied in separable form; the rounding order therefore differs from
// the reference's tap-by-tap sums, by O(1e-16) relative in FP64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace amb
{
    // Everything one step needs, passed by value per launch (the reference keeps
    // these in process-global __constant__ memory, src/parameters.cu:6-8).
    struct StepParams
    {
        int ny, nx;                 // rows (y), cols (x)
        double dt, dxInv, dyInv;
        double a, b, c, kappa, lambda, zeta;
        double noise_mag;           // sqrt(2T) sqrt(1/(dt dx dy)) (src/parameters.h:43-51,79-87)
        uint64_t seed;
        int64_t step;               // timestep whose currents drive the first update of the launch
    };

    // D8 antisymmetric taps d_1..d_4 (offset +k has +d_k, offset -k has -d_k).
    __host__ __device__ constexpr double d8_tap(int k)
    {
        return k == 1 ? 4.0 / 5 : k == 2 ? -1.0 / 5 : k == 3 ? 4.0 / 105 : -1.0 / 280;
    }

    // Periodic index in [0, n). The common cases (already inside, or one period
    // out) take no division; only grids smaller than the stencil reach the
    // general remainder. |i| < 2^31 for every caller (n < 2^30).
    __host__ __device__ __forceinline__ int wrap_index(int i, int n)
    {
        if ((unsigned)i < (unsigned)n) return i;
        if (i < 0 && i >= -n) return i + n;
        if (i >= n && i - n < n) return i - n;
        int r = i % n;
        return r < 0 ? r + n : r;
    }

    // ------------------------------------------------------------ Philox noise

    // Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds with the
    // published multipliers and Weyl key increments.
    struct U4 { uint32_t x, y, z, w; };

    // One 32 x 32 -> 64-bit product per multiplier (a single wide multiply gives both halves).
    __device__ __forceinline__ void mulhilo(uint32_t m, uint32_t x, uint32_t& hi, uint32_t& lo)
    {
        const uint64_t p = uint64_t(m) * x;
        hi = uint32_t(p >> 32);
        lo = uint32_t(p);
    }

    __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
    {
        constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
        constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
        for (int round = 0; round < 10; ++round)
        {
            uint32_t hi0, lo0, hi1, lo1;
            mulhilo(M0, c.x, hi0, lo0);
            mulhilo(M1, c.z, hi1, lo1);
            c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
            k0 += W0;
            k1 += W1;
        }
        return c;
    }

    // Philox4x32-10 with the ten round keys precomputed (rk0[i] = k0 + i W0,
    // rk1[i] = k1 + i W1): same output as philox4x32_10, no key arithmetic per call.
    __device__ __forceinline__ U4 philox4x32_10_rk(U4 c, const uint32_t (&rk0)[10], const uint32_t (&rk1)[10])
    {
        constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
#pragma unroll
        for (int round = 0; round < 10; ++round)
        {
            uint32_t hi0, lo0, hi1, lo1;
            mulhilo(M0, c.x, hi0, lo0);
            mulhilo(M1, c.z, hi1, lo1);
            c = U4{hi1 ^ c.y ^ rk0[round], lo1, hi0 ^ c.w ^ rk1[round], lo0};
        }
        return c;
    }

    // Counter of the noise quad holding (row, col) for component comp (0 = y, 1 = x):
    // (col >> 2, row, step mod 2^32, (step >> 32) << 1 | comp), key = seed.
    __device__ __forceinline__ U4 noise_bits(uint64_t seed, int64_t step, int row, int col, int comp)
    {
        U4 ctr{uint32_t(col) >> 2, uint32_t(row), uint32_t(uint64_t(step)),
               (uint32_t(uint64_t(step) >> 32) << 1) | uint32_t(comp)};
        return philox4x32_10(ctr, uint32_t(seed), uint32_t(seed >> 32));
    }

    // Box-Muller on one pair of 32-bit words with 24-bit uniforms:
    // ua = ((xa >> 8) + 1) 2^-24 in (0,1], ub = (xb >> 8) 2^-24 in [0,1);
    // r = sqrt(-2 ln ua), theta = 2 pi (ub - 1/2); returns (r cos theta, r sin theta).
    // Evaluated in single precision, every operation rounded once as written (no contraction),
    // so the scalar and the packed form below give the same bits. -ln(ua) uses the fast
    // hardware logarithm (__logf) where ua <= 31/32; closer to 1 its absolute
    // error would rival ln(ua) itself, so there -ln(1 - v), v = 1 - ua (exact),
    // is summed from the Mercator series v + v^2/2 + ... + v^5/5 (truncation
    // below 1e-8 relative for v < 1/32), as 2v (1 + v (1/2 + v (1/3 + v (1/4 + v/5)))).
    // |theta| <= pi keeps __sincosf in its accurate range.
    __device__ __forceinline__ float2 box_muller_f32(uint32_t xa, uint32_t xb)
    {
        const uint32_t ka = xa >> 8;
        const float ua = __fmul_rn(float(ka + 1u), 1.0f / 16777216.0f);
        const float v = __fmul_rn(float(16777215u - ka), 1.0f / 16777216.0f);
        const float ub = __fmul_rn(float(xb >> 8), 1.0f / 16777216.0f);
        // both branches evaluated and selected: a divergent branch would make most warps run both anyway
        float ser = __fmaf_rn(v, 0.2f, 0.25f);
        ser = __fmaf_rn(v, ser, 0.333333343f);
        ser = __fmaf_rn(v, ser, 0.5f);
        ser = __fmaf_rn(v, ser, 1.0f);
        const float t_series = __fmul_rn(__fmul_rn(2.0f, v), ser);
        const float t_log = __fmul_rn(-2.0f, __logf(ua));
        const float t = v < 0.03125f ? t_series : t_log;
        const float r = __fmul_rn(t, rsqrtf(fmaxf(t, 1e-30f)));
        float sn, cs;
        __sincosf(__fmul_rn(6.283185307179586f, __fadd_rn(ub, -0.5f)), &sn, &cs);
        return make_float2(__fmul_rn(r, cs), __fmul_rn(r, sn));
    }

    // box_muller_f32 on two independent pairs of words, (xa.x, xb.x) and (xa.y, xb.y): the
    // integer steps and the hardware approximations per pair, the floating-point steps as packed
    // FP32 pairs (each half rounded as the scalar operation). zc = (r cos) and zs = (r sin) of the
    // two pairs: box_muller_f32(xa.x, xb.x) == (zc.x, zs.x), box_muller_f32(xa.y, xb.y) == (zc.y, zs.y).
    __device__ __forceinline__ void box_muller_f32x2(uint2 xa, uint2 xb, float2& zc, float2& zs)
    {
        const auto d = [](float c) { return make_float2(c, c); };
        const uint32_t kx = xa.x >> 8, ky = xa.y >> 8;
        const float2 inv24 = d(1.0f / 16777216.0f);
        const float2 ua = __fmul2_rn(make_float2(float(kx + 1u), float(ky + 1u)), inv24);
        const float2 v = __fmul2_rn(make_float2(float(16777215u - kx), float(16777215u - ky)), inv24);
        const float2 ub = __fmul2_rn(make_float2(float(xb.x >> 8), float(xb.y >> 8)), inv24);
        float2 ser = __ffma2_rn(v, d(0.2f), d(0.25f));
        ser = __ffma2_rn(v, ser, d(0.333333343f));
        ser = __ffma2_rn(v, ser, d(0.5f));
        ser = __ffma2_rn(v, ser, d(1.0f));
        const float2 t_series = __fmul2_rn(__fmul2_rn(d(2.0f), v), ser);
        const float2 t_log = __fmul2_rn(d(-2.0f), make_float2(__logf(ua.x), __logf(ua.y)));
        const float2 t = make_float2(v.x < 0.03125f ? t_series.x : t_log.x, v.y < 0.03125f ? t_series.y : t_log.y);
        const float2 r = __fmul2_rn(t, make_float2(rsqrtf(fmaxf(t.x, 1e-30f)), rsqrtf(fmaxf(t.y, 1e-30f))));
        const float2 th = __fmul2_rn(d(6.283185307179586f), __fadd2_rn(ub, d(-0.5f)));
        float sx, cx, sy, cy;
        __sincosf(th.x, &sx, &cx);
        __sincosf(th.y, &sy, &cy);
        zc = __fmul2_rn(r, make_float2(cx, cy));
        zs = __fmul2_rn(r, make_float2(sx, sy));
    }

    // One standard normal of the (seed, step) noise field at (row, col, comp). Both field
    // precisions draw the same single-precision Box-Muller normals: the noise only needs
    // statistical accuracy, and GB300's FP64 rate would make a double-precision transform
    // cost more than the stencil itself.
    __device__ __forceinline__ float noise_normal(uint64_t seed, int64_t step, int row, int col, int comp)
    {
        U4 q = noise_bits(seed, step, row, col, comp);
        int lane = col & 3;
        uint32_t xa = (lane < 2) ? q.x : q.z;
        uint32_t xb = (lane < 2) ? q.y : q.w;
        float2 z = box_muller_f32(xa, xb);
        return (lane & 1) ? z.y : z.x;
    }

    // All four normals of a quad (columns 4q..4q+3; col4 is any column of the quad).
    __device__ __forceinline__ void noise_quad(uint64_t seed, int64_t step, int row, int col4, int comp, float z[4])
    {
        U4 q = noise_bits(seed, step, row, col4, comp);
        float2 p0 = box_muller_f32(q.x, q.y), p1 = box_muller_f32(q.z, q.w);
        z[0] = p0.x; z[1] = p0.y; z[2] = p1.x; z[3] = p1.y;
    }
}
