// Register-sliding FP32 step kernel: the FP32 performance path.
//
// Work decomposition: one warp owns a strip of 128 computed columns (4 per
// lane) whose middle 112 are its output, and slides down a segment of rows.
// Nothing is shared between warps, so there is no CTA barrier: x-neighbours
// come from warp shuffles (radius 1) or a per-warp smem row (radius 4), and the
// y-direction order-8 stencils (D8_y o D8_y of the passive current, radius 8)
// run on register rings of nine rows held per lane.
//
// Pipeline, with k the row whose mu_p is formed this iteration:
//   stage A (row k)     lap, grad phi, mu_p, mu_a, zeta*lap*grad phi from phi rows k-1..k+1
//   J1_y   (row k-4)    -D8_y mu_p + mag xi_y                      mu_p ring, rows k-8..k
//   DY8    (row k-8)    D8_y J1_y                                   J1_y ring
//   J2     (row k-1)    -Tj mu_a + J_c                              mu_a partials, rows k-2..k
//   divTj  (row k-2)    Tj . J2                                     J2 partials, rows k-3..k-1
//   output (row k-8)    J1_x = -D8_x mu_p + mag xi_x, DX8 = D8_x J1_x (smem row exchange),
//                       div J = DX8 + DY8 + divTj (delayed 6 rows in smem), compensated update.
// The phi rows stream through a 16-row shared-memory ring filled by TMA bulk
// copies (cp.async.bulk, completion on one mbarrier per ring slot) issued 8
// rows ahead of use; a row window that crosses the periodic x boundary is
// fetched as several aligned pieces. Every mbarrier wait is bounded: on timeout the
// warp poisons its outputs with NaN (caught by the Integrator's finite check),
// drains its own copies with a bounded wait, and leaves.
//
// Requirements (checked by step_f32_sliding_supported): ncols % 4 == 0 and
// ncols >= 112 (one strip's output width); any nrows >= 1.
//
// Arithmetic per site follows the same separable operators as the tile kernel
// (amb_step_tile.cuh); the noise is the shared Philox definition (amb_common.cuh),
// one Philox4x32-10 call per lane per row and component, so the result does
// not depend on the strip or segment decomposition.
#include "amb_kernels.h"
#include "amb_step_tile.cuh"

#include <cstdint>
#include <cstring>
#include <type_traits>

namespace amb
{
    namespace sliding
    {
        constexpr int kCols = 128;              // columns computed per warp (4 per lane)
        constexpr int kHalo = 8;                // mu_p halo on each side
        constexpr int kOut = kCols - 2 * kHalo; // 112 output columns per warp
        constexpr int kRing = 16;               // phi rows in the smem ring
        constexpr int kLead = 6;                // rows fetched ahead of use
        constexpr int kRowF = 136;              // floats per ring row: columns -12 .. 123 of the strip
        constexpr int kRowBytes = kRowF * 4;
        constexpr int kDelay = 8;               // divTj delay ring (6 rows of delay needed)
        constexpr int kMupRing = 10;            // mu_p ring: 9 rows in use + 1 the producer fills while the consumer reads
        constexpr int kJ1Ring = 9;              // J1_y ring: the 9 rows of one D8_y
        constexpr long long kSpinLimit = 1ll << 22;

        // Shared memory of one producer/consumer warp pair.
        struct __align__(16) PairSmem
        {
            float phi[kRing][kRowF];     // phi row ring (TMA destination)
            float mup[kMupRing][kCols];  // mu_p rows k-9..k (producer writes k, D8_y reads k-8..k, consumer reads k-8)
            float j1y[kJ1Ring][kCols];   // J1_y rows k-12..k-4 (producer only)
            float hand[2][4][kCols];     // producer -> consumer rows: mu_a(k), J_c,y(k), J_c,x(k), DY8(k-8)
            float xch[kCols];            // consumer's J1_x row exchange
            float dtj[kDelay][kCols];    // divTj delay ring
            uint64_t bar[kRing];         // one mbarrier per phi ring slot
            int abort;                   // set by the producer when a row never arrived
        };

        // Shared memory of one warp that runs every stage of its strip (the fused form).
        struct __align__(16) WarpSmem
        {
            float phi[kRing][kRowF];     // phi row ring (TMA destination)
            float mup[kMupRing][kCols];  // mu_p rows k-9..k (D8_y reads k-8..k-1, J1_x reads k-8)
            float j1y[kJ1Ring][kCols];   // J1_y rows k-12..k-4
            float xch[kCols];            // J1_x row exchange
            float dtj[kDelay][kCols];    // divTj delay ring
            uint64_t bar[kRing];         // one mbarrier per phi ring slot
        };

        __device__ __forceinline__ uint32_t smem_u32(const void* p)
        {
            return static_cast<uint32_t>(__cvta_generic_to_shared(p));
        }

        __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
        {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
        }

        __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
        {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                         : "memory");
        }

        __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
        {
            uint32_t ok;
            asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                         : "=r"(ok)
                         : "r"(smem_u32(bar)), "r"(parity)
                         : "memory");
            return ok != 0;
        }

        // Bounded wait; returns false on timeout.
        __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
        {
            for (long long i = 0; i < kSpinLimit; ++i)
                if (mbar_try_wait(bar, parity)) return true;
            return false;
        }

        __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
        {
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                             smem_u32(dst)),
                         "l"(src), "r"(bytes), "r"(smem_u32(bar))
                         : "memory");
        }

        __device__ __forceinline__ void fence_proxy_async()
        {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }

        struct Task
        {
            int c0;        // first computed... strip origin: output columns [c0, c0 + 112)
            int store_lo;  // first column this strip stores (overlapping last strip)
            int r0, r1;    // output rows [r0, r1)
        };

        // Lane 0 fetches local row m (global row r0 - 9 + m) of the strip window into ring slot m % 16.
        template <typename Smem>
        __device__ __forceinline__ void issue_row(Smem& sm, const float* __restrict__ phi, int ny, int nx,
                                                  const Task& t, int m)
        {
            int slot = m & (kRing - 1);
            int gr = wrap_index(t.r0 - 9 + m, ny);
            int gc = wrap_index(t.c0 - 12, nx);
            const float* row = phi + (size_t)gr * nx;
            mbar_expect_tx(&sm.bar[slot], kRowBytes);
            // the window is one aligned piece, or several where it wraps round a narrow grid
            for (int dst = 0; dst < kRowF;)
            {
                int n = nx - gc < kRowF - dst ? nx - gc : kRowF - dst;
                bulk_g2s(&sm.phi[slot][dst], row + gc, uint32_t(n) * 4u, &sm.bar[slot]);
                dst += n;
                gc = 0;
            }
        }

        struct Coef
        {
            float dt, mag;
            float a, b, c, kappa, lambda, zeta;
            float lA, lB, lC, lD;      // lap = lA (A-+A+) + lB (f-+f+) + lC A0 + lD f0
            float gxa, gxb, gya, gyb;  // gx = gxa (D-+D+) + gxb D0 ; gy = gya (A+-A-) + gyb (f+-f-)
            float ny8[4], nx8[4];      // -dyInv d_j, -dxInv d_j (J1 = -D8 mu_p)
            float py8[4], px8[4];      // dyInv d_j, dxInv d_j (D8 J1)
            float ndy, jx1, jx3;       // J_l,y = ndy (sx(k) - sx(k-2)); J_l,x = jx1 (dx(k)+dx(k-2)) + jx3 dx(k-1)
            float dyInv, tx1, tx3;     // divTj = dyInv (sxJ(k-1)-sxJ(k-3)) + tx1 (dxJ(k-3)+dxJ(k-1)) + tx3 dxJ(k-2)
            // duplicated pairs for the packed (f32x2) arithmetic on a lane's column pairs
            float2 ny8p[4], py8p[4], magp;
            float2 cp, bp, ap, nkappap, lambdap, zetap;  // c, b, a, -kappa, lambda, zeta
            float2 ndyp, jx1p, jx3p, tx1p, tx3p, dyInvp;
            float2 dtp, ndtp;                             // dt, -dt
            uint32_t rk0[10], rk1[10]; // Philox round keys of the seed
            __host__ __device__ explicit Coef(const StepParams& p)
            {
                for (int r = 0; r < 10; ++r)
                {
                    rk0[r] = uint32_t(p.seed) + uint32_t(r) * 0x9E3779B9u;
                    rk1[r] = uint32_t(p.seed >> 32) + uint32_t(r) * 0xBB67AE85u;
                }
                double ex = p.dxInv * p.dxInv, ey = p.dyInv * p.dyInv;
                dt = float(p.dt);
                mag = float(p.noise_mag);
                a = float(p.a); b = float(p.b); c = float(p.c);
                kappa = float(p.kappa); lambda = float(p.lambda); zeta = float(p.zeta);
                lA = float(-0.25 * (ex + ey));
                lB = float(0.5 * ex + 1.5 * ey);
                lC = float(1.5 * ex + 0.5 * ey);
                lD = float(-3.0 * (ex + ey));
                gxa = float(0.1 * p.dxInv); gxb = float(0.3 * p.dxInv);
                gya = float(0.1 * p.dyInv); gyb = float(0.3 * p.dyInv);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                {
                    ny8[j] = float(-p.dyInv * d8_tap(j + 1));
                    nx8[j] = float(-p.dxInv * d8_tap(j + 1));
                    py8[j] = float(p.dyInv * d8_tap(j + 1));
                    px8[j] = float(p.dxInv * d8_tap(j + 1));
                    ny8p[j] = make_float2(ny8[j], ny8[j]);
                    py8p[j] = make_float2(py8[j], py8[j]);
                }
                ndy = float(-p.dyInv);
                jx1 = float(-0.1 * p.dxInv); jx3 = float(-0.3 * p.dxInv);
                dyInv = float(p.dyInv);
                tx1 = float(0.1 * p.dxInv); tx3 = float(0.3 * p.dxInv);
                const auto dup = [](float v) { return make_float2(v, v); };
                magp = dup(mag);
                cp = dup(c); bp = dup(b); ap = dup(a); nkappap = dup(-kappa); lambdap = dup(lambda);
                zetap = dup(zeta);
                ndyp = dup(ndy); jx1p = dup(jx1); jx3p = dup(jx3); tx1p = dup(tx1); tx3p = dup(tx3);
                dyInvp = dup(dyInv); dtp = dup(dt); ndtp = dup(-dt);
            }
        };

        __device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

        // Packed FP32 pairs (sm_100+ f32x2): each lane rounds exactly as the scalar operation.
        __device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }

        // One order-8 y derivative c . (r[5+j] - r[3-j]) of four columns, in column pairs, in the
        // scalar code's operation order: c0 (r5 - r3), then fused c_j (r[5+j] - r[3-j]) + acc.
        __device__ __forceinline__ void d8y_pairs(const float4 (&r)[9], const float2 (&c)[4], float2& lo, float2& hi)
        {
            const auto L = [](const float4& v) { return make_float2(v.x, v.y); };
            const auto H = [](const float4& v) { return make_float2(v.z, v.w); };
            lo = __fmul2_rn(c[0], sub2(L(r[5]), L(r[3])));
            hi = __fmul2_rn(c[0], sub2(H(r[5]), H(r[3])));
#pragma unroll
            for (int j = 1; j < 4; ++j)
            {
                lo = __ffma2_rn(c[j], sub2(L(r[5 + j]), L(r[3 - j])), lo);
                hi = __ffma2_rn(c[j], sub2(H(r[5 + j]), H(r[3 - j])), hi);
            }
        }
        __device__ __forceinline__ void sts4(float* p, const float (&v)[4])
        {
            *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
        }

        // Four normals of this lane's quad (global quad at column gcol) for one row and component.
        template <int NOISE>
        __device__ __forceinline__ void normals(const StepParams& p, const Coef& k, const float* __restrict__ injected,
                                                int grow, int gcol, int comp, float (&z)[4])
        {
            if constexpr (NOISE == NOISE_PHILOX)
            {
                U4 ctr{uint32_t(gcol) >> 2, uint32_t(grow), uint32_t(uint64_t(p.step)),
                       (uint32_t(uint64_t(p.step) >> 32) << 1) | uint32_t(comp)};
                U4 q = philox4x32_10_rk(ctr, k.rk0, k.rk1);
                float2 zc, zs;  // (r cos, r sin) of the draws (x, y) and (z, w)
                box_muller_f32x2(make_uint2(q.x, q.z), make_uint2(q.y, q.w), zc, zs);
                z[0] = zc.x; z[1] = zs.x; z[2] = zc.y; z[3] = zs.y;
            }
            else if constexpr (NOISE == NOISE_INJECTED)
            {
                float4 v = *reinterpret_cast<const float4*>(injected + (size_t)comp * p.ny * p.nx
                                                            + (size_t)grow * p.nx + gcol);
                z[0] = v.x; z[1] = v.y; z[2] = v.z; z[3] = v.w;
            }
            else
            {
                z[0] = z[1] = z[2] = z[3] = 0.f;
            }
        }

        __device__ __forceinline__ void pair_sync(int id)
        {
            asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
        }

        __device__ __forceinline__ Task make_task(int task, int nstrips, int seg_h, int ny, int nx)
        {
            Task t;
            int strip = task % nstrips, seg = task / nstrips;
            int c0 = strip * kOut;
            t.store_lo = c0;
            if (c0 + kOut > nx) c0 = nx - kOut;  // last strip overlaps its neighbour; stores only its own part
            t.c0 = c0;
            t.r0 = seg * seg_h;
            t.r1 = min(t.r0 + seg_h, ny);
            return t;
        }

        // Pointer to row slot i (0 <= i < 8) of a window of 8 consecutive ring rows that starts at
        // slot b of a ring of N slots: slots b..N-1 from `at_b`, the wrapped ones from `at_b` - N rows.
        // One compare and one select per row; the row offset is a constant of the load.
        template <int N>
        __device__ __forceinline__ const float* ring_row(const float* at_b, int b, int i)
        {
            return (b < N - i ? at_b : at_b - N * kCols) + i * kCols;
        }

        // Producer warp: stage A, the mu_p ring, J1_y and its noise; streams phi rows in by TMA.
        // Rounds 1..8 feed no J1_y row that an output reads and rounds 1..16 no DY8 row: they run
        // the body without those parts (the rounds' other results are the same).
        template <int NOISE>
        __device__ __forceinline__ void producer(PairSmem& sm, const float* __restrict__ phi_in, const StepParams& p,
                                                 const Coef& k, const float* __restrict__ injected, const Task& t,
                                                 int lane, int bar_id)
        {
            const int ny = p.ny, nx = p.nx;
            const int H = t.r1 - t.r0;
            const int nrows = H + 18;   // local rows 0 .. H+17 (global r0-9 .. r1+8)
            const int total = H + 16;   // rounds kl = 1 .. H+16
            const int gcol = wrap_index(t.c0 - 8 + 4 * lane, nx);
            const int own = 4 + 4 * lane;

            if (lane == 0)
            {
                for (int s = 0; s < kRing; ++s) mbar_init(&sm.bar[s], 1);
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                sm.abort = 0;
                for (int m = 0; m <= kLead && m < nrows; ++m) issue_row(sm, phi_in, ny, nx, t, m);
            }
            __syncwarp();
            int issued = min(kLead, nrows - 1);
            bool ok = mbar_wait(&sm.bar[0], 0);
            ok &= mbar_wait(&sm.bar[1], 0);
            bool failed = !__all_sync(0xffffffffu, ok);
            int waited = failed ? -1 : 1;

            float fm[6], fz[6];
#pragma unroll
            for (int q = 0; q < 6; ++q)
            {
                fm[q] = sm.phi[0][own - 1 + q];
                fz[q] = sm.phi[1][own - 1 + q];
            }
            float xin[4] = {0.f, 0.f, 0.f, 0.f};  // xi_y of this round's J1_y row, formed one round ahead
            int nrow = 0;    // global row of the next round's J1_y noise
            int ms = 1;      // mu_p ring slot of row kl  (kl mod 10)
            int js = 5;      // J1_y ring slot of row kl-4 ((kl - 4) mod 9), from round 9 on

            const auto round = [&](int kl, auto j1_tag, auto dy_tag) {
                constexpr bool J1 = decltype(j1_tag)::value, DY = decltype(dy_tag)::value;
                const int mnew = kl + 1;
                if (!failed)
                {
                    bool okw = mbar_wait(&sm.bar[mnew & (kRing - 1)], (mnew >> 4) & 1);
                    if (__all_sync(0xffffffffu, okw)) waited = mnew;
                    else
                    {
                        failed = true;
                        if (lane == 0) sm.abort = 1;
                    }
                }
                // ---- stage A at local row kl
                float lap[4], gx[4], gy[4], f0[4];
                {
                    const float* rp = sm.phi[mnew & (kRing - 1)];
                    float4 vp = lds4(rp + own);
                    float pL = __shfl_up_sync(0xffffffffu, vp.w, 1);
                    float pR = __shfl_down_sync(0xffffffffu, vp.x, 1);
                    if (lane == 0) pL = rp[own - 1];
                    if (lane == 31) pR = rp[own + 4];
                    float fp[6] = {pL, vp.x, vp.y, vp.z, vp.w, pR};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        float Am = fm[q] + fm[q + 2], Dm = fm[q + 2] - fm[q];
                        float A0 = fz[q] + fz[q + 2], D0 = fz[q + 2] - fz[q];
                        float Ap = fp[q] + fp[q + 2], Dp = fp[q + 2] - fp[q];
                        float f = fz[q + 1];
                        float l = k.lA * (Am + Ap);
                        l = fmaf(k.lB, fm[q + 1] + fp[q + 1], l);
                        l = fmaf(k.lC, A0, l);
                        lap[q] = fmaf(k.lD, f, l);
                        gx[q] = fmaf(k.gxb, D0, k.gxa * (Dm + Dp));
                        gy[q] = fmaf(k.gyb, fp[q + 1] - fm[q + 1], k.gya * (Ap - Am));
                        f0[q] = f;
                    }
#pragma unroll
                    for (int q = 0; q < 6; ++q)
                    {
                        fm[q] = fz[q];
                        fz[q] = fp[q];
                    }
                }
                float mup[4], mua[4], jcy[4], jcx[4];
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2)  // column pairs (0, 1) and (2, 3), packed
                {
                    const int q = 2 * h2;
                    const float2 f = make_float2(f0[q], f0[q + 1]), l2 = make_float2(lap[q], lap[q + 1]);
                    const float2 x2 = make_float2(gx[q], gx[q + 1]), y2 = make_float2(gy[q], gy[q + 1]);
                    const float2 poly = __fmul2_rn(__ffma2_rn(__ffma2_rn(k.cp, f, k.bp), f, k.ap), f);
                    const float2 mp = __ffma2_rn(k.nkappap, l2, poly);
                    const float2 ma = __fmul2_rn(k.lambdap, __ffma2_rn(y2, y2, __fmul2_rn(x2, x2)));
                    const float2 zl = __fmul2_rn(k.zetap, l2);
                    const float2 cy = __fmul2_rn(zl, y2), cx = __fmul2_rn(zl, x2);
                    mup[q] = mp.x; mup[q + 1] = mp.y;
                    mua[q] = ma.x; mua[q + 1] = ma.y;
                    jcy[q] = cy.x; jcy[q + 1] = cy.y;
                    jcx[q] = cx.x; jcx[q + 1] = cx.y;
                }
                sts4(&sm.mup[ms][4 * lane], mup);
                float(*h)[kCols] = sm.hand[kl & 1];
                sts4(&h[0][4 * lane], mua);
                sts4(&h[1][4 * lane], jcy);
                sts4(&h[2][4 * lane], jcx);
                if constexpr (J1)
                {
                    // ---- J1_y at local row kl-4 from mu_p rows kl-8..kl (this lane's own columns)
                    const int bm = ms + 2 < kMupRing ? ms + 2 : ms + 2 - kMupRing;  // slot of row kl-8
                    const float* mb = &sm.mup[bm][4 * lane];
                    float4 m[9];
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        if (i != 4) m[i] = lds4(ring_row<kMupRing>(mb, bm, i));
                    m[4] = make_float4(0.f, 0.f, 0.f, 0.f);  // the centre tap has weight 0
                    m[8] = make_float4(mup[0], mup[1], mup[2], mup[3]);
                    const float2 xlo = make_float2(xin[0], xin[1]), xhi = make_float2(xin[2], xin[3]);
                    // noise of the next round's J1_y row, formed now so its Philox chain overlaps this round
                    normals<NOISE>(p, k, injected, nrow, gcol, 0, xin);
                    nrow = nrow + 1 == ny ? 0 : nrow + 1;
                    float2 slo, shi;
                    d8y_pairs(m, k.ny8p, slo, shi);
                    slo = __ffma2_rn(k.magp, xlo, slo);
                    shi = __ffma2_rn(k.magp, xhi, shi);
                    const float j1y[4] = {slo.x, slo.y, shi.x, shi.y};
                    sts4(&sm.j1y[js][4 * lane], j1y);
                    if constexpr (DY)
                    {
                        // ---- DY8 at local row kl-8 from J1_y rows kl-12..kl-4
                        const int bj = js + 1 < kJ1Ring ? js + 1 : js + 1 - kJ1Ring;  // slot of row kl-12
                        const float* jb = &sm.j1y[bj][4 * lane];
                        float4 j[9];
#pragma unroll
                        for (int i = 0; i < 8; ++i)
                            if (i != 4) j[i] = lds4(ring_row<kJ1Ring>(jb, bj, i));
                        j[4] = make_float4(0.f, 0.f, 0.f, 0.f);
                        j[8] = make_float4(j1y[0], j1y[1], j1y[2], j1y[3]);
                        float2 dlo, dhi;
                        d8y_pairs(j, k.py8p, dlo, dhi);
                        const float dy8[4] = {dlo.x, dlo.y, dhi.x, dhi.y};
                        sts4(&h[3][4 * lane], dy8);
                    }
                    js = js + 1 == kJ1Ring ? 0 : js + 1;
                }
                ms = ms + 1 == kMupRing ? 0 : ms + 1;
                // ---- refill: local row kl-10 has been read by everyone (barrier kl-1); fetch row kl+6
                if (lane == 0 && !failed && kl + 6 < nrows)
                {
                    fence_proxy_async();
                    issue_row(sm, phi_in, ny, nx, t, kl + 6);
                }
                if (!failed && kl + 6 < nrows) issued = kl + 6;
                pair_sync(bar_id);
            };
            using F = std::false_type;
            using T = std::true_type;
#pragma unroll 1
            for (int kl = 1; kl <= 8; ++kl) round(kl, F{}, F{});
            // J1_y rows from local row 5 (round 9) on: xi_y of that row (global r0 - 4) now
            nrow = wrap_index(t.r0 - 4, ny);
            normals<NOISE>(p, k, injected, nrow, gcol, 0, xin);
            nrow = nrow + 1 == ny ? 0 : nrow + 1;
#pragma unroll 1
            for (int kl = 9; kl <= 16; ++kl) round(kl, T{}, F{});
#pragma unroll 1
            for (int kl = 17; kl <= total; ++kl) round(kl, T{}, T{});
            if (failed)  // drain this pair's copies in flight (bounded) before the CTA can exit
                for (int m = waited + 1; m <= issued; ++m) mbar_wait(&sm.bar[m & (kRing - 1)], (m >> 4) & 1);
        }

        // Consumer warp: Tjhung chain, J1_x and DX8, compensated update and stores. The first 16
        // rounds output nothing: they run the Tjhung chain only.
        template <int COMP, int NOISE>
        __device__ __forceinline__ void consumer(PairSmem& sm, float* __restrict__ phi_out,
                                                 __nv_bfloat16* residual, const StepParams& p, const Coef& k,
                                                 const float* __restrict__ injected, const Task& t, int lane,
                                                 int bar_id)
        {
            const int ny = p.ny, nx = p.nx;
            const int H = t.r1 - t.r0;
            const int total = H + 16;
            const int gcol = wrap_index(t.c0 - 8 + 4 * lane, nx);
            const int scol = t.c0 - 8 + 4 * lane;
            const bool out_lane = lane >= 2 && lane < 30 && scol >= t.store_lo && scol < nx;
            const int own = 4 + 4 * lane;

            float sxm[3][4], dxm[3][4], sxj[3][4], dxj[3][4];
            float jcy[4], jcx[4];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int q = 0; q < 4; ++q) sxm[i][q] = dxm[i][q] = sxj[i][q] = dxj[i][q] = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) jcy[q] = jcx[q] = 0.f;

            // ---- Tjhung chain of round kl: J2 at row kl-1, divTj at row kl-2 (first needed: divTj of row 9)
            const auto tjhung = [&](int kl) {
                const float(*h)[kCols] = sm.hand[kl & 1];
                float4 m4 = lds4(&h[0][4 * lane]);
                float mL = __shfl_up_sync(0xffffffffu, m4.w, 1);
                float mR = __shfl_down_sync(0xffffffffu, m4.x, 1);
                float mm[6] = {mL, m4.x, m4.y, m4.z, m4.w, mR};
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                    sxm[0][q] = sxm[1][q]; sxm[1][q] = sxm[2][q];
                    dxm[0][q] = dxm[1][q]; dxm[1][q] = dxm[2][q];
                    sxm[2][q] = fmaf(0.1f, mm[q] + mm[q + 2], 0.3f * mm[q + 1]);
                    dxm[2][q] = mm[q + 2] - mm[q];
                }
                float j2y[4], j2x[4];
#pragma unroll
                for (int q = 0; q < 4; q += 2)
                {
                    const auto P = [q](const float (&v)[4]) { return make_float2(v[q], v[q + 1]); };
                    const float2 vy = __ffma2_rn(k.ndyp, sub2(P(sxm[2]), P(sxm[0])), P(jcy));
                    const float2 vx = __ffma2_rn(k.jx3p, P(dxm[1]),
                                                 __ffma2_rn(k.jx1p, __fadd2_rn(P(dxm[2]), P(dxm[0])), P(jcx)));
                    j2y[q] = vy.x; j2y[q + 1] = vy.y;
                    j2x[q] = vx.x; j2x[q + 1] = vx.y;
                }
                float4 cy4 = lds4(&h[1][4 * lane]), cx4 = lds4(&h[2][4 * lane]);
                jcy[0] = cy4.x; jcy[1] = cy4.y; jcy[2] = cy4.z; jcy[3] = cy4.w;  // J_c at row kl
                jcx[0] = cx4.x; jcx[1] = cx4.y; jcx[2] = cx4.z; jcx[3] = cx4.w;
                float yL = __shfl_up_sync(0xffffffffu, j2y[3], 1);
                float yR = __shfl_down_sync(0xffffffffu, j2y[0], 1);
                float xL = __shfl_up_sync(0xffffffffu, j2x[3], 1);
                float xR = __shfl_down_sync(0xffffffffu, j2x[0], 1);
                float yy[6] = {yL, j2y[0], j2y[1], j2y[2], j2y[3], yR};
                float xx[6] = {xL, j2x[0], j2x[1], j2x[2], j2x[3], xR};
                float dtj[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                    sxj[0][q] = sxj[1][q]; sxj[1][q] = sxj[2][q];
                    dxj[0][q] = dxj[1][q]; dxj[1][q] = dxj[2][q];
                    sxj[2][q] = fmaf(0.1f, yy[q] + yy[q + 2], 0.3f * yy[q + 1]);
                    dxj[2][q] = xx[q + 2] - xx[q];
                }
#pragma unroll
                for (int q = 0; q < 4; q += 2)
                {
                    const auto P = [q](const float (&v)[4]) { return make_float2(v[q], v[q + 1]); };
                    float2 v = __fmul2_rn(k.tx1p, __fadd2_rn(P(dxj[0]), P(dxj[2])));
                    v = __ffma2_rn(k.tx3p, P(dxj[1]), v);
                    v = __ffma2_rn(k.dyInvp, sub2(P(sxj[2]), P(sxj[0])), v);
                    dtj[q] = v.x; dtj[q + 1] = v.y;
                }
                sts4(&sm.dtj[(kl - 2) & (kDelay - 1)][4 * lane], dtj);
            };

            // Rounds 1..16: the chain only (unrolled by 3 so the 3-row rings rotate by renaming).
            for (int base = 0; base < 15; base += 3)
            {
#pragma unroll
                for (int ph = 1; ph <= 3; ++ph)
                {
                    pair_sync(bar_id);
                    tjhung(base + ph);
                }
            }
            pair_sync(bar_id);
            tjhung(16);

            // Output rows: round kl (17 .. H+16) writes global row r0 + kl - 17 (never wraps). Its
            // xi_x and bf16 residual are fetched one round ahead.
            int grow = t.r0;
            int mo = 9;        // mu_p ring slot of the output row ((kl - 8) mod 10)
            float xnx[4];
            normals<NOISE>(p, k, injected, grow, gcol, 1, xnx);
            uint2 rnext = make_uint2(0u, 0u);
            if constexpr (COMP == COMP_BF16)
                rnext = *reinterpret_cast<const uint2*>(residual + (size_t)grow * nx + gcol);
            const auto output = [&](int kl) {
                const int lo = kl - 8;
                const float(*h)[kCols] = sm.hand[kl & 1];
                const float* mrow = sm.mup[mo];
                mo = mo + 1 == kMupRing ? 0 : mo + 1;
                float4 ml = lds4(&mrow[(4 * lane - 4) & (kCols - 1)]);
                float4 mc = lds4(&mrow[4 * lane]);
                float4 mr = lds4(&mrow[(4 * lane + 4) & (kCols - 1)]);
                float mu[12] = {ml.x, ml.y, ml.z, ml.w, mc.x, mc.y, mc.z, mc.w, mr.x, mr.y, mr.z, mr.w};
                float xi[4] = {xnx[0], xnx[1], xnx[2], xnx[3]};
                // next round's xi_x and residual are fetched now, off this round's critical path
                const int gnext = grow + 1 == ny ? 0 : grow + 1;
                normals<NOISE>(p, k, injected, gnext, gcol, 1, xnx);
                uint2 rv = rnext;
                if constexpr (COMP == COMP_BF16)
                    rnext = *reinterpret_cast<const uint2*>(residual + (size_t)gnext * nx + gcol);
                float j1x[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                    float s = k.nx8[0] * (mu[q + 5] - mu[q + 3]);
                    s = fmaf(k.nx8[1], mu[q + 6] - mu[q + 2], s);
                    s = fmaf(k.nx8[2], mu[q + 7] - mu[q + 1], s);
                    s = fmaf(k.nx8[3], mu[q + 8] - mu[q], s);
                    j1x[q] = fmaf(k.mag, xi[q], s);
                }
                sts4(&sm.xch[4 * lane], j1x);
                __syncwarp();
                float4 jl = lds4(&sm.xch[(4 * lane - 4) & (kCols - 1)]);
                float4 jr = lds4(&sm.xch[(4 * lane + 4) & (kCols - 1)]);
                float jj[12] = {jl.x, jl.y, jl.z, jl.w, j1x[0], j1x[1], j1x[2], j1x[3], jr.x, jr.y, jr.z, jr.w};
                __syncwarp();
                float4 dt4 = lds4(&sm.dtj[lo & (kDelay - 1)][4 * lane]);
                float4 dy4 = lds4(&h[3][4 * lane]);
                const float dtv[4] = {dt4.x, dt4.y, dt4.z, dt4.w}, dyv[4] = {dy4.x, dy4.y, dy4.z, dy4.w};
                float4 ph4 = lds4(&sm.phi[lo & (kRing - 1)][own]);
                float fo[4] = {ph4.x, ph4.y, ph4.z, ph4.w};
                const size_t gi = (size_t)grow * nx + gcol;
                grow = gnext;
                float rr[4] = {0.f, 0.f, 0.f, 0.f};
                if constexpr (COMP == COMP_BF16)
                {
                    rr[0] = __uint_as_float(rv.x << 16);
                    rr[1] = __uint_as_float(rv.x & 0xffff0000u);
                    rr[2] = __uint_as_float(rv.y << 16);
                    rr[3] = __uint_as_float(rv.y & 0xffff0000u);
                }
                float dx8[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                    float d = k.px8[0] * (jj[q + 5] - jj[q + 3]);
                    d = fmaf(k.px8[1], jj[q + 6] - jj[q + 2], d);
                    d = fmaf(k.px8[2], jj[q + 7] - jj[q + 1], d);
                    dx8[q] = fmaf(k.px8[3], jj[q + 8] - jj[q], d);
                }
                // div = DX8 + (divTj + DY8); compensated update phi += y, y = -dt div - r,
                // in column pairs: y = -F with F = fma(dt, div, r) (the same rounding),
                // new phi = phi - F, new r = (new phi - phi) + F
                float nf[4], nr[4];
#pragma unroll
                for (int q = 0; q < 4; q += 2)
                {
                    const auto P = [q](const float (&v)[4]) { return make_float2(v[q], v[q + 1]); };
                    const float2 div = __fadd2_rn(P(dx8), __fadd2_rn(P(dtv), P(dyv)));
                    float2 vf, vr;
                    if constexpr (COMP == COMP_BF16)
                    {
                        const float2 F = __ffma2_rn(k.dtp, div, P(rr));
                        vf = sub2(P(fo), F);
                        vr = __fadd2_rn(sub2(vf, P(fo)), F);
                    }
                    else
                    {
                        vf = __ffma2_rn(k.ndtp, div, P(fo));
                        vr = make_float2(0.f, 0.f);
                    }
                    nf[q] = vf.x; nf[q + 1] = vf.y;
                    nr[q] = vr.x; nr[q + 1] = vr.y;
                }
                if (*reinterpret_cast<volatile int*>(&sm.abort))
                    nf[0] = nf[1] = nf[2] = nf[3] = __int_as_float(0x7fc00000);
                if (out_lane)
                {
                    *reinterpret_cast<float4*>(phi_out + gi) = make_float4(nf[0], nf[1], nf[2], nf[3]);
                    if constexpr (COMP == COMP_BF16)
                    {
                        __nv_bfloat162 lo2 = __floats2bfloat162_rn(nr[0], nr[1]);
                        __nv_bfloat162 hi2 = __floats2bfloat162_rn(nr[2], nr[3]);
                        uint2 w;
                        w.x = *reinterpret_cast<uint32_t*>(&lo2);
                        w.y = *reinterpret_cast<uint32_t*>(&hi2);
                        *reinterpret_cast<uint2*>(residual + gi) = w;
                    }
                }
            };

            // Rounds 17 .. H+16: chain and output (unrolled by 3, as the fill rounds).
            for (int base = 16; base < total; base += 3)
            {
#pragma unroll
                for (int ph = 1; ph <= 3; ++ph)
                {
                    const int kl = base + ph;
                    if (kl > total) break;
                    pair_sync(bar_id);
                    tjhung(kl);
                    output(kl);
                }
            }
        }

        // One warp runs every stage of its strip: the producer's and the consumer's work of each
        // round in one instruction stream, with no hand-off buffers and no barrier between warps
        // (the only synchronisation is the warp's own, around the J1_x row exchange). The same
        // operations in the same order as the warp pair, so the same bits.
        template <int COMP, int NOISE>
        __device__ __forceinline__ void fused_strip(WarpSmem& sm, const float* __restrict__ phi_in,
                                                    float* __restrict__ phi_out, __nv_bfloat16* residual,
                                                    const StepParams& p, const Coef& k,
                                                    const float* __restrict__ injected, const Task& t, int lane)
        {
            const int ny = p.ny, nx = p.nx;
            const int H = t.r1 - t.r0;
            const int nrows = H + 18;   // local rows 0 .. H+17 (global r0-9 .. r1+8)
            const int total = H + 16;   // rounds kl = 1 .. H+16
            const int gcol = wrap_index(t.c0 - 8 + 4 * lane, nx);
            const int scol = t.c0 - 8 + 4 * lane;
            const bool out_lane = lane >= 2 && lane < 30 && scol >= t.store_lo && scol < nx;
            const int own = 4 + 4 * lane;

            if (lane == 0)
            {
                for (int s = 0; s < kRing; ++s) mbar_init(&sm.bar[s], 1);
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                for (int m = 0; m <= kLead && m < nrows; ++m) issue_row(sm, phi_in, ny, nx, t, m);
            }
            __syncwarp();
            int issued = min(kLead, nrows - 1);
            bool ok = mbar_wait(&sm.bar[0], 0);
            ok &= mbar_wait(&sm.bar[1], 0);
            bool failed = !__all_sync(0xffffffffu, ok);
            int waited = failed ? -1 : 1;

            float fm[6], fz[6];
#pragma unroll
            for (int q = 0; q < 6; ++q)
            {
                fm[q] = sm.phi[0][own - 1 + q];
                fz[q] = sm.phi[1][own - 1 + q];
            }
            float xin[4] = {0.f, 0.f, 0.f, 0.f};  // xi_y of this round's J1_y row, formed one round ahead
            int nrow = 0;
            int ms = 1;      // mu_p ring slot of row kl  (kl mod 10)
            int js = 5;      // J1_y ring slot of row kl-4 ((kl - 4) mod 9), from round 9 on
            float sxm[3][4], dxm[3][4], sxj[3][4], dxj[3][4];
            float jcy[4], jcx[4];  // J_c of row kl-1
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int q = 0; q < 4; ++q) sxm[i][q] = dxm[i][q] = sxj[i][q] = dxj[i][q] = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) jcy[q] = jcx[q] = 0.f;
            int grow = t.r0;   // output row of the next output round
            int mo = 9;        // mu_p ring slot of the output row ((kl - 8) mod 10)
            float xnx[4] = {0.f, 0.f, 0.f, 0.f};
            uint2 rnext = make_uint2(0u, 0u);

            const auto round = [&](int kl, auto j1_tag, auto dy_tag) {
                constexpr bool J1 = decltype(j1_tag)::value, OUT = decltype(dy_tag)::value;
                const int mnew = kl + 1;
                if (!failed)
                {
                    bool okw = mbar_wait(&sm.bar[mnew & (kRing - 1)], (mnew >> 4) & 1);
                    if (__all_sync(0xffffffffu, okw)) waited = mnew;
                    else failed = true;
                }
                // ---- stage A at local row kl
                float lap[4], gx[4], gy[4], f0[4];
                {
                    const float* rp = sm.phi[mnew & (kRing - 1)];
                    float4 vp = lds4(rp + own);
                    float pL = __shfl_up_sync(0xffffffffu, vp.w, 1);
                    float pR = __shfl_down_sync(0xffffffffu, vp.x, 1);
                    if (lane == 0) pL = rp[own - 1];
                    if (lane == 31) pR = rp[own + 4];
                    float fp[6] = {pL, vp.x, vp.y, vp.z, vp.w, pR};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        float Am = fm[q] + fm[q + 2], Dm = fm[q + 2] - fm[q];
                        float A0 = fz[q] + fz[q + 2], D0 = fz[q + 2] - fz[q];
                        float Ap = fp[q] + fp[q + 2], Dp = fp[q + 2] - fp[q];
                        float f = fz[q + 1];
                        float l = k.lA * (Am + Ap);
                        l = fmaf(k.lB, fm[q + 1] + fp[q + 1], l);
                        l = fmaf(k.lC, A0, l);
                        lap[q] = fmaf(k.lD, f, l);
                        gx[q] = fmaf(k.gxb, D0, k.gxa * (Dm + Dp));
                        gy[q] = fmaf(k.gyb, fp[q + 1] - fm[q + 1], k.gya * (Ap - Am));
                        f0[q] = f;
                    }
#pragma unroll
                    for (int q = 0; q < 6; ++q)
                    {
                        fm[q] = fz[q];
                        fz[q] = fp[q];
                    }
                }
                float mup[4], mua[4], ncy[4], ncx[4];
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2)
                {
                    const int q = 2 * h2;
                    const float2 f = make_float2(f0[q], f0[q + 1]), l2 = make_float2(lap[q], lap[q + 1]);
                    const float2 x2 = make_float2(gx[q], gx[q + 1]), y2 = make_float2(gy[q], gy[q + 1]);
                    const float2 poly = __fmul2_rn(__ffma2_rn(__ffma2_rn(k.cp, f, k.bp), f, k.ap), f);
                    const float2 mp = __ffma2_rn(k.nkappap, l2, poly);
                    const float2 ma = __fmul2_rn(k.lambdap, __ffma2_rn(y2, y2, __fmul2_rn(x2, x2)));
                    const float2 zl = __fmul2_rn(k.zetap, l2);
                    const float2 cy = __fmul2_rn(zl, y2), cx = __fmul2_rn(zl, x2);
                    mup[q] = mp.x; mup[q + 1] = mp.y;
                    mua[q] = ma.x; mua[q + 1] = ma.y;
                    ncy[q] = cy.x; ncy[q + 1] = cy.y;
                    ncx[q] = cx.x; ncx[q + 1] = cx.y;
                }
                sts4(&sm.mup[ms][4 * lane], mup);
                float dy8[4] = {0.f, 0.f, 0.f, 0.f};
                if constexpr (J1)
                {
                    // ---- J1_y at local row kl-4 from mu_p rows kl-8..kl (own columns)
                    const int bm = ms + 2 < kMupRing ? ms + 2 : ms + 2 - kMupRing;
                    const float* mb = &sm.mup[bm][4 * lane];
                    float4 m[9];
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        if (i != 4) m[i] = lds4(ring_row<kMupRing>(mb, bm, i));
                    m[4] = make_float4(0.f, 0.f, 0.f, 0.f);
                    m[8] = make_float4(mup[0], mup[1], mup[2], mup[3]);
                    const float2 xlo = make_float2(xin[0], xin[1]), xhi = make_float2(xin[2], xin[3]);
                    normals<NOISE>(p, k, injected, nrow, gcol, 0, xin);
                    nrow = nrow + 1 == ny ? 0 : nrow + 1;
                    float2 slo, shi;
                    d8y_pairs(m, k.ny8p, slo, shi);
                    slo = __ffma2_rn(k.magp, xlo, slo);
                    shi = __ffma2_rn(k.magp, xhi, shi);
                    const float j1y[4] = {slo.x, slo.y, shi.x, shi.y};
                    sts4(&sm.j1y[js][4 * lane], j1y);
                    if constexpr (OUT)
                    {
                        // ---- DY8 at local row kl-8 from J1_y rows kl-12..kl-4
                        const int bj = js + 1 < kJ1Ring ? js + 1 : js + 1 - kJ1Ring;
                        const float* jb = &sm.j1y[bj][4 * lane];
                        float4 j[9];
#pragma unroll
                        for (int i = 0; i < 8; ++i)
                            if (i != 4) j[i] = lds4(ring_row<kJ1Ring>(jb, bj, i));
                        j[4] = make_float4(0.f, 0.f, 0.f, 0.f);
                        j[8] = make_float4(j1y[0], j1y[1], j1y[2], j1y[3]);
                        float2 dlo, dhi;
                        d8y_pairs(j, k.py8p, dlo, dhi);
                        dy8[0] = dlo.x; dy8[1] = dlo.y; dy8[2] = dhi.x; dy8[3] = dhi.y;
                    }
                    js = js + 1 == kJ1Ring ? 0 : js + 1;
                }
                // ---- Tjhung chain: J2 at row kl-1, divTj at row kl-2
                {
                    float mL = __shfl_up_sync(0xffffffffu, mua[3], 1);
                    float mR = __shfl_down_sync(0xffffffffu, mua[0], 1);
                    float mm[6] = {mL, mua[0], mua[1], mua[2], mua[3], mR};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        sxm[0][q] = sxm[1][q]; sxm[1][q] = sxm[2][q];
                        dxm[0][q] = dxm[1][q]; dxm[1][q] = dxm[2][q];
                        sxm[2][q] = fmaf(0.1f, mm[q] + mm[q + 2], 0.3f * mm[q + 1]);
                        dxm[2][q] = mm[q + 2] - mm[q];
                    }
                    float j2y[4], j2x[4];
#pragma unroll
                    for (int q = 0; q < 4; q += 2)
                    {
                        const auto P = [q](const float (&v)[4]) { return make_float2(v[q], v[q + 1]); };
                        const float2 vy = __ffma2_rn(k.ndyp, sub2(P(sxm[2]), P(sxm[0])), P(jcy));
                        const float2 vx = __ffma2_rn(k.jx3p, P(dxm[1]),
                                                     __ffma2_rn(k.jx1p, __fadd2_rn(P(dxm[2]), P(dxm[0])), P(jcx)));
                        j2y[q] = vy.x; j2y[q + 1] = vy.y;
                        j2x[q] = vx.x; j2x[q + 1] = vx.y;
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        jcy[q] = ncy[q];  // J_c at row kl, for the next round
                        jcx[q] = ncx[q];
                    }
                    float yL = __shfl_up_sync(0xffffffffu, j2y[3], 1);
                    float yR = __shfl_down_sync(0xffffffffu, j2y[0], 1);
                    float xL = __shfl_up_sync(0xffffffffu, j2x[3], 1);
                    float xR = __shfl_down_sync(0xffffffffu, j2x[0], 1);
                    float yy[6] = {yL, j2y[0], j2y[1], j2y[2], j2y[3], yR};
                    float xx[6] = {xL, j2x[0], j2x[1], j2x[2], j2x[3], xR};
                    float dtj[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        sxj[0][q] = sxj[1][q]; sxj[1][q] = sxj[2][q];
                        dxj[0][q] = dxj[1][q]; dxj[1][q] = dxj[2][q];
                        sxj[2][q] = fmaf(0.1f, yy[q] + yy[q + 2], 0.3f * yy[q + 1]);
                        dxj[2][q] = xx[q + 2] - xx[q];
                    }
#pragma unroll
                    for (int q = 0; q < 4; q += 2)
                    {
                        const auto P = [q](const float (&v)[4]) { return make_float2(v[q], v[q + 1]); };
                        float2 v = __fmul2_rn(k.tx1p, __fadd2_rn(P(dxj[0]), P(dxj[2])));
                        v = __ffma2_rn(k.tx3p, P(dxj[1]), v);
                        v = __ffma2_rn(k.dyInvp, sub2(P(sxj[2]), P(sxj[0])), v);
                        dtj[q] = v.x; dtj[q + 1] = v.y;
                    }
                    sts4(&sm.dtj[(kl - 2) & (kDelay - 1)][4 * lane], dtj);
                }
                if constexpr (OUT)
                {
                    // ---- output local row kl-8 (global row grow)
                    const int lo = kl - 8;
                    const float* mrow = sm.mup[mo];
                    mo = mo + 1 == kMupRing ? 0 : mo + 1;
                    __syncwarp();  // the mu_p row's neighbour columns were written by other lanes
                    float4 ml = lds4(&mrow[(4 * lane - 4) & (kCols - 1)]);
                    float4 mc = lds4(&mrow[4 * lane]);
                    float4 mr = lds4(&mrow[(4 * lane + 4) & (kCols - 1)]);
                    float mu[12] = {ml.x, ml.y, ml.z, ml.w, mc.x, mc.y, mc.z, mc.w, mr.x, mr.y, mr.z, mr.w};
                    float xi[4] = {xnx[0], xnx[1], xnx[2], xnx[3]};
                    const int gnext = grow + 1 == ny ? 0 : grow + 1;
                    normals<NOISE>(p, k, injected, gnext, gcol, 1, xnx);
                    uint2 rv = rnext;
                    if constexpr (COMP == COMP_BF16)
                        rnext = *reinterpret_cast<const uint2*>(residual + (size_t)gnext * nx + gcol);
                    float j1x[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        float s = k.nx8[0] * (mu[q + 5] - mu[q + 3]);
                        s = fmaf(k.nx8[1], mu[q + 6] - mu[q + 2], s);
                        s = fmaf(k.nx8[2], mu[q + 7] - mu[q + 1], s);
                        s = fmaf(k.nx8[3], mu[q + 8] - mu[q], s);
                        j1x[q] = fmaf(k.mag, xi[q], s);
                    }
                    sts4(&sm.xch[4 * lane], j1x);
                    __syncwarp();
                    float4 jl = lds4(&sm.xch[(4 * lane - 4) & (kCols - 1)]);
                    float4 jr = lds4(&sm.xch[(4 * lane + 4) & (kCols - 1)]);
                    float jj[12] = {jl.x, jl.y, jl.z, jl.w, j1x[0], j1x[1], j1x[2], j1x[3], jr.x, jr.y, jr.z, jr.w};
                    __syncwarp();
                    float4 dt4 = lds4(&sm.dtj[lo & (kDelay - 1)][4 * lane]);
                    const float dtv[4] = {dt4.x, dt4.y, dt4.z, dt4.w};
                    float4 ph4 = lds4(&sm.phi[lo & (kRing - 1)][own]);
                    float fo[4] = {ph4.x, ph4.y, ph4.z, ph4.w};
                    const size_t gi = (size_t)grow * nx + gcol;
                    grow = gnext;
                    float rr[4] = {0.f, 0.f, 0.f, 0.f};
                    if constexpr (COMP == COMP_BF16)
                    {
                        rr[0] = __uint_as_float(rv.x << 16);
                        rr[1] = __uint_as_float(rv.x & 0xffff0000u);
                        rr[2] = __uint_as_float(rv.y << 16);
                        rr[3] = __uint_as_float(rv.y & 0xffff0000u);
                    }
                    float dx8[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        float d = k.px8[0] * (jj[q + 5] - jj[q + 3]);
                        d = fmaf(k.px8[1], jj[q + 6] - jj[q + 2], d);
                        d = fmaf(k.px8[2], jj[q + 7] - jj[q + 1], d);
                        dx8[q] = fmaf(k.px8[3], jj[q + 8] - jj[q], d);
                    }
                    float nf[4], nr[4];
#pragma unroll
                    for (int q = 0; q < 4; q += 2)
                    {
                        const auto P = [q](const float (&v)[4]) { return make_float2(v[q], v[q + 1]); };
                        const float2 div = __fadd2_rn(P(dx8), __fadd2_rn(P(dtv), P(dy8)));
                        float2 vf, vr;
                        if constexpr (COMP == COMP_BF16)
                        {
                            const float2 F = __ffma2_rn(k.dtp, div, P(rr));
                            vf = sub2(P(fo), F);
                            vr = __fadd2_rn(sub2(vf, P(fo)), F);
                        }
                        else
                        {
                            vf = __ffma2_rn(k.ndtp, div, P(fo));
                            vr = make_float2(0.f, 0.f);
                        }
                        nf[q] = vf.x; nf[q + 1] = vf.y;
                        nr[q] = vr.x; nr[q + 1] = vr.y;
                    }
                    if (failed) nf[0] = nf[1] = nf[2] = nf[3] = __int_as_float(0x7fc00000);
                    if (out_lane)
                    {
                        *reinterpret_cast<float4*>(phi_out + gi) = make_float4(nf[0], nf[1], nf[2], nf[3]);
                        if constexpr (COMP == COMP_BF16)
                        {
                            __nv_bfloat162 lo2 = __floats2bfloat162_rn(nr[0], nr[1]);
                            __nv_bfloat162 hi2 = __floats2bfloat162_rn(nr[2], nr[3]);
                            uint2 w;
                            w.x = *reinterpret_cast<uint32_t*>(&lo2);
                            w.y = *reinterpret_cast<uint32_t*>(&hi2);
                            *reinterpret_cast<uint2*>(residual + gi) = w;
                        }
                    }
                }
                ms = ms + 1 == kMupRing ? 0 : ms + 1;
                // ---- refill: this warp read local row kl-10 last in round kl-2; fetch row kl+6 into its slot
                __syncwarp();
                if (lane == 0 && !failed && kl + 6 < nrows)
                {
                    fence_proxy_async();
                    issue_row(sm, phi_in, ny, nx, t, kl + 6);
                }
                if (!failed && kl + 6 < nrows) issued = kl + 6;
            };
            using F = std::false_type;
            using T = std::true_type;
            for (int base = 0; base < 6; base += 3)
            {
#pragma unroll
                for (int ph = 1; ph <= 3; ++ph) round(base + ph, F{}, F{});  // rounds 1..6
            }
            round(7, F{}, F{});
            round(8, F{}, F{});
            // J1_y rows from local row 5 (round 9) on: xi_y of that row (global r0 - 4) now
            nrow = wrap_index(t.r0 - 4, ny);
            normals<NOISE>(p, k, injected, nrow, gcol, 0, xin);
            nrow = nrow + 1 == ny ? 0 : nrow + 1;
            for (int base = 8; base < 14; base += 3)
            {
#pragma unroll
                for (int ph = 1; ph <= 3; ++ph) round(base + ph, T{}, F{});  // rounds 9..14
            }
            round(15, T{}, F{});
            round(16, T{}, F{});
            // output rounds: xi_x and residual of the first output row (global r0)
            normals<NOISE>(p, k, injected, grow, gcol, 1, xnx);
            if constexpr (COMP == COMP_BF16)
                rnext = *reinterpret_cast<const uint2*>(residual + (size_t)grow * nx + gcol);
            for (int base = 16; base < total; base += 3)
            {
#pragma unroll
                for (int ph = 1; ph <= 3; ++ph)
                {
                    const int kl = base + ph;
                    if (kl > total) break;
                    round(kl, T{}, T{});
                }
            }
            if (failed)  // drain this warp's copies in flight (bounded) before the CTA can exit
                for (int m = waited + 1; m <= issued; ++m) mbar_wait(&sm.bar[m & (kRing - 1)], (m >> 4) & 1);
        }

        template <int COMP, int NOISE, int WARPS>
        __global__ void __launch_bounds__(32 * WARPS)
        sliding_fused_kernel(const float* __restrict__ phi_in, float* __restrict__ phi_out, __nv_bfloat16* residual,
                             const StepParams p, const Coef k, const float* __restrict__ injected, int seg_h,
                             int nstrips, int ntasks)
        {
            extern __shared__ __align__(16) unsigned char smem_raw[];
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            const int task = blockIdx.x * WARPS + warp;
            if (task >= ntasks) return;
            WarpSmem& sm = reinterpret_cast<WarpSmem*>(smem_raw)[warp];
            const Task t = make_task(task, nstrips, seg_h, p.ny, p.nx);
            fused_strip<COMP, NOISE>(sm, phi_in, phi_out, residual, p, k, injected, t, lane);
        }

        template <int COMP, int NOISE, int PAIRS>
        __global__ void __launch_bounds__(64 * PAIRS)
        sliding_kernel(const float* __restrict__ phi_in, float* __restrict__ phi_out, __nv_bfloat16* residual,
                       const StepParams p, const Coef k, const float* __restrict__ injected, int seg_h, int nstrips,
                       int ntasks)
        {
            extern __shared__ __align__(16) unsigned char smem_raw[];
            const int pair = threadIdx.x >> 6, role = (threadIdx.x >> 5) & 1, lane = threadIdx.x & 31;
            const int task = blockIdx.x * PAIRS + pair;
            if (task >= ntasks) return;  // both warps of the pair leave together
            PairSmem& sm = reinterpret_cast<PairSmem*>(smem_raw)[pair];
            const Task t = make_task(task, nstrips, seg_h, p.ny, p.nx);
            if (role == 0)
                producer<NOISE>(sm, phi_in, p, k, injected, t, lane, 1 + pair);
            else
                consumer<COMP, NOISE>(sm, phi_out, residual, p, k, injected, t, lane, 1 + pair);
        }
    }

    namespace sliding
    {
        // Batched form: one warp pair per task of a task table that spans many replicas of
        // different sizes and parameters; the step index comes from device memory so that
        // a captured CUDA graph of several steps can be replayed.
        // The per-replica coefficients are copied from their table into the pair's shared memory
        // at the start of the task and read from there (8 one-pair CTAs per SM, as the
        // single-field kernel: at most 128 registers).
        template <int COMP, int NOISE>
        __global__ void __launch_bounds__(64, 8)
        sliding_ensemble_kernel(const EnsembleReplica* __restrict__ reps, const Coef* __restrict__ coefs,
                                const EnsembleTask* __restrict__ tasks, int parity,
                                const int64_t* __restrict__ step_counter, int step_offset)
        {
            extern __shared__ __align__(16) unsigned char smem_raw[];
            const int role = (threadIdx.x >> 5) & 1, lane = threadIdx.x & 31;
            PairSmem& sm = *reinterpret_cast<PairSmem*>(smem_raw);
            const EnsembleTask bt = tasks[blockIdx.x];
            const EnsembleReplica& rd = reps[bt.replica];
            StepParams p = rd.p;
            p.step = *step_counter + step_offset;
            Coef* kc = reinterpret_cast<Coef*>(smem_raw + sizeof(PairSmem));
            {
                const uint32_t* src = reinterpret_cast<const uint32_t*>(coefs + bt.replica);
                uint32_t* dst = reinterpret_cast<uint32_t*>(kc);
                for (int i = threadIdx.x; i < int(sizeof(Coef) / 4); i += 64) dst[i] = src[i];
            }
            __syncthreads();
            const Coef& k = *kc;
            Task t;
            int c0 = bt.strip * kOut;
            t.store_lo = c0;
            if (c0 + kOut > p.nx) c0 = p.nx - kOut;
            t.c0 = c0;
            t.r0 = bt.r0;
            t.r1 = bt.r1;
            if (role == 0)
                producer<NOISE>(sm, rd.phi[parity], p, k, nullptr, t, lane, 1);
            else
                consumer<COMP, NOISE>(sm, rd.phi[parity ^ 1], rd.residual, p, k, nullptr, t, lane, 1);
        }

        // The batched form with one warp per task running every stage (the fused form), its
        // replica's coefficient block in shared memory beside the warp's rings.
        template <int COMP, int NOISE>
        __global__ void __launch_bounds__(32)
        sliding_ensemble_fused_kernel(const EnsembleReplica* __restrict__ reps, const Coef* __restrict__ coefs,
                                      const EnsembleTask* __restrict__ tasks, int parity,
                                      const int64_t* __restrict__ step_counter, int step_offset)
        {
            extern __shared__ __align__(16) unsigned char smem_raw[];
            const int lane = threadIdx.x & 31;
            WarpSmem& sm = *reinterpret_cast<WarpSmem*>(smem_raw);
            const EnsembleTask bt = tasks[blockIdx.x];
            const EnsembleReplica& rd = reps[bt.replica];
            StepParams p = rd.p;
            p.step = *step_counter + step_offset;
            Coef* kc = reinterpret_cast<Coef*>(smem_raw + sizeof(WarpSmem));
            {
                const uint32_t* src = reinterpret_cast<const uint32_t*>(coefs + bt.replica);
                uint32_t* dst = reinterpret_cast<uint32_t*>(kc);
                for (int i = lane; i < int(sizeof(Coef) / 4); i += 32) dst[i] = src[i];
            }
            __syncwarp();
            const Coef& k = *kc;
            Task t;
            int c0 = bt.strip * kOut;
            t.store_lo = c0;
            if (c0 + kOut > p.nx) c0 = p.nx - kOut;
            t.c0 = c0;
            t.r0 = bt.r0;
            t.r1 = bt.r1;
            fused_strip<COMP, NOISE>(sm, rd.phi[parity], rd.phi[parity ^ 1], rd.residual, p, k, nullptr, t, lane);
        }
    }

    bool step_f32_sliding_supported(int ny, int nx, int variant)
    {
        (void)variant;
        return ny >= 1 && nx >= sliding::kOut && nx % 4 == 0;
    }

    namespace
    {
        // Rows of one segment that minimise waves x (rows + pipeline fill), given how many
        // warp pairs the device keeps resident. Fill rounds cost about 10 full rows.
        int choose_seg_h(int ny, int nx, int resident_pairs)
        {
            const int nstrips = (nx + sliding::kOut - 1) / sliding::kOut;
            double best = 1e300;
            int best_h = ny;
            for (int nsegs = 1; nsegs <= ny; ++nsegs)
            {
                int h = (ny + nsegs - 1) / nsegs;
                if (h < 16 && nsegs > 1) break;
                long long tasks = (long long)nstrips * ((ny + h - 1) / h);
                long long waves = (tasks + resident_pairs - 1) / resident_pairs;
                double cost = double(waves) * (h + 10);
                if (cost < best - 1e-9)
                {
                    best = cost;
                    best_h = h;
                }
            }
            return best_h;
        }

        template <int COMP, int NOISE, int WPB>
        cudaError_t launch_variant(const float* phi_in, float* phi_out, __nv_bfloat16* comp, const StepParams& p,
                                   const float* injected, int seg_h, cudaStream_t stream)
        {
            using namespace sliding;
            const size_t smem = sizeof(PairSmem) * WPB;
            auto kern = sliding_kernel<COMP, NOISE, WPB>;
            static int resident_pairs = 0;  // per kernel variant; the process drives one device type
            if (resident_pairs == 0)
            {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                int dev = 0, sms = 0, blocks = 0;
                if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
                if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
                if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, 64 * WPB, smem)) != cudaSuccess)
                    return e;
                resident_pairs = blocks * WPB * sms > 0 ? blocks * WPB * sms : WPB;
            }
            if (seg_h <= 0) seg_h = choose_seg_h(p.ny, p.nx, resident_pairs);
            const int nstrips = (p.nx + kOut - 1) / kOut;
            const int nsegs = (p.ny + seg_h - 1) / seg_h;
            const int ntasks = nstrips * nsegs;
            const Coef k(p);
            kern<<<(ntasks + WPB - 1) / WPB, 64 * WPB, smem, stream>>>(phi_in, phi_out, comp, p, k, injected, seg_h,
                                                                       nstrips, ntasks);
            return cudaGetLastError();
        }

        template <int COMP, int NOISE, int WARPS>
        cudaError_t launch_fused(const float* phi_in, float* phi_out, __nv_bfloat16* comp, const StepParams& p,
                                 const float* injected, int seg_h, cudaStream_t stream)
        {
            using namespace sliding;
            const size_t smem = sizeof(WarpSmem) * WARPS;
            auto kern = sliding_fused_kernel<COMP, NOISE, WARPS>;
            static int resident = 0;  // per kernel variant; the process drives one device type
            if (resident == 0)
            {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                int dev = 0, sms = 0, blocks = 0;
                if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
                if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
                if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, 32 * WARPS, smem)) != cudaSuccess)
                    return e;
                resident = blocks * WARPS * sms > 0 ? blocks * WARPS * sms : WARPS;
            }
            if (seg_h <= 0) seg_h = choose_seg_h(p.ny, p.nx, resident);
            const int nstrips = (p.nx + kOut - 1) / kOut;
            const int nsegs = (p.ny + seg_h - 1) / seg_h;
            const int ntasks = nstrips * nsegs;
            const Coef k(p);
            kern<<<(ntasks + WARPS - 1) / WARPS, 32 * WARPS, smem, stream>>>(phi_in, phi_out, comp, p, k, injected,
                                                                            seg_h, nstrips, ntasks);
            return cudaGetLastError();
        }

        template <int COMP, int WARPS>
        cudaError_t by_noise_fused(const float* phi_in, float* phi_out, __nv_bfloat16* comp, const StepParams& p,
                                   int noise_mode, const float* injected, int seg_h, cudaStream_t stream)
        {
            switch (noise_mode)
            {
            case NOISE_PHILOX: return launch_fused<COMP, NOISE_PHILOX, WARPS>(phi_in, phi_out, comp, p, injected, seg_h, stream);
            case NOISE_INJECTED: return launch_fused<COMP, NOISE_INJECTED, WARPS>(phi_in, phi_out, comp, p, injected, seg_h, stream);
            default: return launch_fused<COMP, NOISE_OFF, WARPS>(phi_in, phi_out, comp, p, injected, seg_h, stream);
            }
        }

        template <int COMP, int WPB>
        cudaError_t by_noise(const float* phi_in, float* phi_out, __nv_bfloat16* comp, const StepParams& p,
                             int noise_mode, const float* injected, int seg_h, cudaStream_t stream)
        {
            switch (noise_mode)
            {
            case NOISE_PHILOX: return launch_variant<COMP, NOISE_PHILOX, WPB>(phi_in, phi_out, comp, p, injected, seg_h, stream);
            case NOISE_INJECTED: return launch_variant<COMP, NOISE_INJECTED, WPB>(phi_in, phi_out, comp, p, injected, seg_h, stream);
            default: return launch_variant<COMP, NOISE_OFF, WPB>(phi_in, phi_out, comp, p, injected, seg_h, stream);
            }
        }
    }

    int sliding_default_seg_h(int ny, int nx)
    {
        return choose_seg_h(ny, nx, 152 * 8);
    }

    // variant: 0 = defaults; otherwise (seg_h << 4) | fused (8) | code, code 1 -> 1, 2 -> 2, 3 -> 4 warp
    // pairs (fused: warps) per CTA.
    cudaError_t launch_step_f32_sliding(const float* phi_in, float* phi_out, __nv_bfloat16* comp, int comp_mode,
                                        const StepParams& p, int noise_mode, const float* injected, int variant,
                                        cudaStream_t stream)
    {
        if (!step_f32_sliding_supported(p.ny, p.nx, variant)) return cudaErrorNotSupported;
        int seg_h = variant >> 4;
        int wpb = variant & 7;
        if (variant & 8)
        {
            if (comp_mode == COMP_BF16)
            {
                if (wpb == 1) return by_noise_fused<COMP_BF16, 1>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
                if (wpb == 2) return by_noise_fused<COMP_BF16, 2>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
                return by_noise_fused<COMP_BF16, 4>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
            }
            if (wpb == 1) return by_noise_fused<COMP_NONE, 1>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
            if (wpb == 2) return by_noise_fused<COMP_NONE, 2>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
            return by_noise_fused<COMP_NONE, 4>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
        }
        if (wpb == 0) wpb = 1;
        if (comp_mode == COMP_BF16)
        {
            if (wpb == 1) return by_noise<COMP_BF16, 1>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
            if (wpb == 3) return by_noise<COMP_BF16, 4>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
            return by_noise<COMP_BF16, 2>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
        }
        if (wpb == 1) return by_noise<COMP_NONE, 1>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
        if (wpb == 3) return by_noise<COMP_NONE, 4>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
        return by_noise<COMP_NONE, 2>(phi_in, phi_out, comp, p, noise_mode, injected, seg_h, stream);
    }
}

namespace amb
{
    size_t sliding_coef_bytes() { return sizeof(sliding::Coef); }

    namespace
    {
        // A pair's (or, fused, a warp's) shared memory plus its replica's coefficient block.
        constexpr size_t ensemble_smem_bytes() { return sizeof(sliding::PairSmem) + sizeof(sliding::Coef); }
        constexpr size_t ensemble_fused_smem_bytes() { return sizeof(sliding::WarpSmem) + sizeof(sliding::Coef); }
    }

    void sliding_make_coef(const StepParams& p, void* out)
    {
        sliding::Coef k(p);
        std::memcpy(out, &k, sizeof(k));
    }

    int sliding_default_seg_h_for(int ny, int nx, int resident_pairs)
    {
        return choose_seg_h(ny, nx, resident_pairs);
    }

    namespace
    {
        template <int COMP, int NOISE, bool FUSED>
        cudaError_t launch_ensemble_variant(const EnsembleReplica* reps, const void* coefs, const EnsembleTask* tasks,
                                            int ntasks, int parity, const int64_t* step_counter, int step_offset,
                                            cudaStream_t stream)
        {
            using namespace sliding;
            auto kern = FUSED ? sliding_ensemble_fused_kernel<COMP, NOISE> : sliding_ensemble_kernel<COMP, NOISE>;
            const size_t smem = FUSED ? ensemble_fused_smem_bytes() : ensemble_smem_bytes();
            static bool configured = false;
            if (!configured)
            {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                configured = true;
            }
            kern<<<ntasks, FUSED ? 32 : 64, smem, stream>>>(reps, static_cast<const Coef*>(coefs), tasks, parity,
                                                           step_counter, step_offset);
            return cudaGetLastError();
        }

        template <bool FUSED>
        cudaError_t launch_ensemble_form(const EnsembleReplica* reps, const void* coefs, const EnsembleTask* tasks,
                                         int ntasks, int parity, const int64_t* step_counter, int step_offset,
                                         int comp_mode, bool noise, cudaStream_t stream)
        {
            if (comp_mode == COMP_BF16)
                return noise ? launch_ensemble_variant<COMP_BF16, NOISE_PHILOX, FUSED>(reps, coefs, tasks, ntasks, parity,
                                                                                       step_counter, step_offset, stream)
                             : launch_ensemble_variant<COMP_BF16, NOISE_OFF, FUSED>(reps, coefs, tasks, ntasks, parity,
                                                                                    step_counter, step_offset, stream);
            return noise ? launch_ensemble_variant<COMP_NONE, NOISE_PHILOX, FUSED>(reps, coefs, tasks, ntasks, parity,
                                                                                   step_counter, step_offset, stream)
                         : launch_ensemble_variant<COMP_NONE, NOISE_OFF, FUSED>(reps, coefs, tasks, ntasks, parity,
                                                                                step_counter, step_offset, stream);
        }
    }

    cudaError_t ensemble_resident_pairs(int* out, bool fused)
    {
        using namespace sliding;
        const void* kern = fused ? reinterpret_cast<const void*>(sliding_ensemble_fused_kernel<COMP_BF16, NOISE_PHILOX>)
                                 : reinterpret_cast<const void*>(sliding_ensemble_kernel<COMP_BF16, NOISE_PHILOX>);
        const size_t smem = fused ? ensemble_fused_smem_bytes() : ensemble_smem_bytes();
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        int dev = 0, sms = 0, blocks = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, fused ? 32 : 64, smem);
        if (e == cudaSuccess) *out = blocks * sms > 0 ? blocks * sms : 1;
        return e;
    }

    cudaError_t launch_sliding_ensemble(const EnsembleReplica* reps, const void* coefs, const EnsembleTask* tasks,
                                        int ntasks, int parity, const int64_t* step_counter, int step_offset,
                                        int comp_mode, int noise_mode, bool fused, cudaStream_t stream)
    {
        if (ntasks <= 0) return cudaSuccess;
        const bool noise = noise_mode == NOISE_PHILOX;
        return fused ? launch_ensemble_form<true>(reps, coefs, tasks, ntasks, parity, step_counter, step_offset,
                                                  comp_mode, noise, stream)
                     : launch_ensemble_form<false>(reps, coefs, tasks, ntasks, parity, step_counter, step_offset,
                                                   comp_mode, noise, stream);
    }
}
