// Learned coarse stepper kernels (no reference counterpart): 5x5 circular
// convolutions as BF16 implicit GEMMs on the tcgen05 tensor cores with FP32
// accumulation in TMEM, for both inference and training, plus the
// mass-conserving fixed-point update that applies the predicted flux.
//
// Activation layout ("chunk planes"): bf16 [batch][C/8][nrows][ncols][8], i.e.
// for each group of 8 channels a plane of 16-byte sites. One 16-byte site row
// is one row of a tensor-core core matrix, so a tap shift of one site along x
// is a 16-byte move of the operand start address.
//
// Forward / data-gradient kernel (conv_fwd_kernel): one CTA owns a 128-site
// window of up to 16 output rows and stages all of its input rows (the rows plus
// a 2-row halo above and below, periodic wrap in both axes) in shared memory, one
// bulk copy per (row, channel chunk) for the in-range sites and, in the first and
// last windows, plain copies of the 2 periodically wrapped sites on each side by
// the epilogue warps; one mbarrier per row. Each staged input row, shifted by one of the
// five x taps, is the A operand (M = 128 sites, K-major, LBO = one channel-chunk
// plane, SBO = 8 sites) of ONE MMA per 16 input channels whose B operand stacks
// the five y taps along N (N = 5 x Cout): its five N slices are the contributions
// of that input row to the five output rows it touches, whose FP32 accumulators
// sit side by side in TMEM (zeroed first). One 128 x 160 x 16 MMA thus replaces
// five 128 x 32 x 16 ones and the A tile is read from shared memory once instead
// of five times. Rows at the edges of the CTA's range issue only the slices of
// the output rows they own. Warp 0 stages rows, warp 1 issues the MMAs and
// commits one mbarrier per finished output row, warps 2-9 zero TMEM and then run
// the epilogue (bias, GELU, its derivative, or FP32 output). The data gradient of
// a circular convolution is the forward convolution with the kernel flipped and
// the channel roles swapped, so the same kernel serves it with the
// GELU-derivative epilogue.
//
// Weight-gradient kernel (conv_wgrad_kernel): dW[tap][ci][co] = sum over sites
// of X[ci][site + tap] dZ[co][site]. Per MMA: M = 128 rows = (ky block, ci), with
// 16/(Cin/8) ky values stacked along M (the staged rows sit at a uniform pitch,
// so (ky, chunk) is one uniform M stride), N = Cout, K = 16 sites; both operands
// MN-major. Partial sums per CTA go to scratch and a second kernel reduces them
// in a fixed order (deterministic gradients).
#include "amb_gb300.h"
#include "amb_kernels.h"
#include "amb_tc.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

namespace
{
    using namespace amb::tc;

    constexpr int kTile = 128;              // output sites per tile (one row window)
    constexpr int kSites = kTile + 4;       // staged input sites per row (halo 2 on each side)
    constexpr int kRowPlane = kSites * 16;  // bytes of one channel chunk of one staged row
    constexpr int kThreads = 192;           // wgrad: warp 0 loads, warp 1 issues MMAs, warps 2-5 epilogue
    constexpr int kFwdThreads = 320;        // forward: warp 0 loads, warp 1 issues MMAs, warps 2-9 epilogue
    constexpr int kMaxFwdRows = 16;         // forward: most output rows per CTA (all inputs staged at once)
    constexpr uint32_t kSmemLimit = 227u * 1024u;
    constexpr int kTaps = 25;

    enum Epilogue
    {
        EPI_GELU = 0,      // out = bf16(gelu(acc + bias)), pre = bf16(acc + bias)
        EPI_F32 = 1,       // out_f32 = acc + bias (first `cout` channels)
        EPI_GELU_BWD = 2,  // out = bf16(acc * gelu'(gate))
    };

    struct FwdArgs
    {
        const uint16_t* in;     // [batch][cin/8][nrows][ncols][8]
        const uint16_t* wimg;   // [5 kx][cin/8][5 (4 - ky)][npad][8] (B operand image, K-major)
        const float* bias;      // [npad] or null
        uint16_t* out;          // [batch][npad/8][nrows][ncols][8]
        uint16_t* pre;          // optional, same layout as out
        const uint16_t* gate;   // EPI_GELU_BWD: same layout as out
        float* out_f32;         // [batch][cout][nrows][ncols]
        int batch, nrows, ncols, cin_chunks, npad, cout, epilogue, rows_per_cta;
        int* error;
    };

    struct WgradArgs
    {
        const uint16_t* x;   // [batch][cin/8][nrows][ncols][8]
        const uint16_t* dz;  // [batch][npad/8][nrows][ncols][8]
        float* partial;      // [grid][25][cin][npad]
        int batch, nrows, ncols, cin_chunks, npad, rows_per_cta;
        int* error;
    };

    __host__ __device__ constexpr uint32_t align128(uint32_t x) { return (x + 127u) & ~127u; }

    __host__ __device__ inline uint32_t fwd_weight_bytes(int cc, int npad) { return uint32_t(kTaps) * cc * npad * 16u; }
    __host__ __device__ inline uint32_t fwd_rows_offset(int cc, int npad) { return align128(fwd_weight_bytes(cc, npad)); }
    __host__ __device__ inline uint32_t fwd_bar_offset(int cc, int npad, int rows)
    {
        return fwd_rows_offset(cc, npad) + uint32_t(rows + 4) * cc * kRowPlane;
    }
    // barriers: full[rows + 4], accf[rows], zero, wbar, done; then the TMEM slot and abort flag
    __host__ __device__ inline uint32_t fwd_smem_bytes(int cc, int npad, int rows)
    {
        return fwd_bar_offset(cc, npad, rows) + uint32_t(2 * rows + 4 + 3) * 8u + 16u;
    }
    // TMEM columns: one npad-wide accumulator per output row, rounded up to a power of two
    __host__ __device__ inline uint32_t fwd_tmem_cols(int npad, int rows)
    {
        uint32_t need = uint32_t(npad * rows), c = 32;
        while (c < need) c <<= 1;
        return c;
    }

    // wgrad: ky blocks per MMA along M, staged X rows per output-row range
    __host__ __device__ inline int wg_kb(int cc) { return 16 / cc; }
    __host__ __device__ inline int wg_nstarts(int cc) { return wg_kb(cc) >= 5 ? 1 : 2; }
    __host__ __device__ inline int wg_start(int cc, int si) { return si == 0 ? 0 : 5 - wg_kb(cc); }
    __host__ __device__ inline int wg_extra_rows(int cc) { return wg_kb(cc) - 1 > 4 ? wg_kb(cc) - 1 : 4; }
    __host__ __device__ inline uint32_t wg_x_bytes(int cc, int rows) { return uint32_t(rows + wg_extra_rows(cc)) * cc * kRowPlane; }
    __host__ __device__ inline uint32_t wg_dz_bytes(int npad, int rows) { return uint32_t(rows) * (npad / 8) * kTile * 16u; }
    __host__ __device__ inline uint32_t wg_bar_offset(int cc, int npad, int rows)
    {
        return align128(wg_x_bytes(cc, rows)) + align128(wg_dz_bytes(npad, rows));
    }
    constexpr uint32_t kWgradMinSmem = 120u * 1024u;  // keeps one wgrad CTA per SM (it owns all of TMEM)
    __host__ __device__ inline uint32_t wg_smem_bytes(int cc, int npad, int rows)
    {
        uint32_t need = wg_bar_offset(cc, npad, rows) + 256u;
        return need > kWgradMinSmem ? need : kWgradMinSmem;
    }

    __device__ __forceinline__ void give_up(int* error, volatile int* abort, int code)
    {
        *abort = 1;
        if (error) atomicExch(error, code);
    }

    __device__ __forceinline__ int wrap_row(int r, int n)
    {
        r %= n;
        return r < 0 ? r + n : r;
    }

    // GELU in its tanh form (Hendrycks and Gimpel): 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))),
    // with the hardware tanh approximation (relative error about 2^-11, below the bf16 rounding
    // of the stored activations; end-state statistics of long learned runs are unchanged by it).
    constexpr float kGeluC0 = 0.7978845608028654f;  // sqrt(2 / pi)
    constexpr float kGeluC1 = 0.044715f;

    __device__ __forceinline__ float tanh_hw(float u)
    {
        float t;
        asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
        return t;
    }

    __device__ __forceinline__ float gelu_f(float z)
    {
        const float t = tanh_hw(kGeluC0 * z * (1.f + kGeluC1 * z * z));
        return 0.5f * z * (1.f + t);
    }

    __device__ __forceinline__ float gelu_grad_f(float z)
    {
        const float z2 = z * z;
        const float t = tanh_hw(kGeluC0 * z * (1.f + kGeluC1 * z2));
        return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * kGeluC0 * (1.f + 3.f * kGeluC1 * z2);
    }

    __device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
    {
        __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
        return *reinterpret_cast<uint32_t*>(&h);
    }

    __device__ __forceinline__ void unpack_bf16x8(const uint4& u, float (&f)[8])
    {
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            f[2 * i] = __uint_as_float(w[i] << 16);
            f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
        }
    }

    // ================================================================ self-test
    // One CTA: D (128 x n) = A (128 x k) * B (n x k)^T from row-major inputs, with A
    // and B staged in the K-major or MN-major core-matrix layout. Layout constants:
    //   K-major  A: SBO = 128 (8-row groups along M), LBO = 16 * 128 (K chunks)
    //   MN-major A: LBO = 128 (8-row K groups),       SBO = (k / 8) * 128 (M groups)
    //   (B likewise with n in place of 128.)
    __global__ void __launch_bounds__(128) tc_selftest_kernel(const uint16_t* __restrict__ A,
                                                              const uint16_t* __restrict__ B, float* __restrict__ D,
                                                              int n, int k, int a_mn, int b_mn, int* error)
    {
        extern __shared__ __align__(1024) uint8_t smem[];
        uint8_t* sa = smem;             // 64 KB region (A uses at most 16 KB)
        uint8_t* sb = smem + 65536;     // 32 KB region (B uses at most 4 KB)
        uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 98304);
        uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 98304 + 64);
        volatile int* abort = reinterpret_cast<volatile int*>(smem + 98304 + 128);
        const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

        // zero both regions, then scatter the operands
        for (int i = tid; i < 98304 / 16; i += 128) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        for (int idx = tid; idx < 128 * k; idx += 128)
        {
            int m = idx / k, kk = idx % k;
            uint32_t off = a_mn ? (m / 8) * (k / 8) * 128 + (kk / 8) * 128 + (kk % 8) * 16 + (m % 8) * 2
                                : (kk / 8) * 16 * 128 + (m / 8) * 128 + (m % 8) * 16 + (kk % 8) * 2;
            *reinterpret_cast<uint16_t*>(sa + off) = A[idx];
        }
        for (int idx = tid; idx < n * k; idx += 128)
        {
            int r = idx / k, kk = idx % k;
            uint32_t off = b_mn ? (r / 8) * (k / 8) * 128 + (kk / 8) * 128 + (kk % 8) * 16 + (r % 8) * 2
                                : (kk / 8) * (n / 8) * 128 + (r / 8) * 128 + (r % 8) * 16 + (kk % 8) * 2;
            *reinterpret_cast<uint16_t*>(sb + off) = B[idx];
        }
        if (tid == 0)
        {
            mbar_init(bar, 1);
            *abort = 0;
            fence_mbar_init();
        }
        fence_proxy_async();
        if (warp == 0)
        {
            tmem_alloc(tslot, 32);
            tmem_relinquish();
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        const uint32_t tbase = *tslot;

        if (tid == 0)
        {
            const uint32_t idesc = idesc_bf16(128, n, a_mn != 0, b_mn != 0);
            const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
            for (int ks = 0; ks < k / 16; ++ks)
            {
                uint64_t ad = a_mn ? smem_desc(a0 + 2 * ks * 128, 128, (k / 8) * 128)
                                   : smem_desc(a0 + 2 * ks * 16 * 128, 16 * 128, 128);
                uint64_t bd = b_mn ? smem_desc(b0 + 2 * ks * 128, 128, (k / 8) * 128)
                                   : smem_desc(b0 + 2 * ks * (n / 8) * 128, (n / 8) * 128, 128);
                mma_bf16(tbase, ad, bd, idesc, ks > 0 ? 1u : 0u);
            }
            mma_commit(bar);
        }
        bool ok = mbar_wait(bar, 0, nullptr);
        ok = __all_sync(0xffffffffu, ok);
        if (ok)
        {
            tc_fence_after();
            float v[32];
            const uint32_t taddr = tbase + (uint32_t(warp * 32) << 16);
            if (n == 32) tmem_ld32(taddr, v);
            else tmem_ld16(taddr, v);
            tmem_wait_ld();
            const int m = warp * 32 + lane;
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (c < n) D[m * n + c] = v[c];
        }
        else if (lane == 0)
            give_up(error, abort, 1);
        tc_fence_before();
        __syncthreads();
        if (warp == 0)
        {
            tc_fence_after();
            tmem_dealloc(tbase, 32);
        }
    }

    // ============================================================== forward
    // CC = input channel chunks (2 or 4), a compile-time constant so that the MMA issue loop
    // unrolls and every descriptor is a base plus a constant.
    template <int CC>
    __global__ void __launch_bounds__(kFwdThreads, 1) conv_fwd_kernel(const FwdArgs a)
    {
        extern __shared__ __align__(1024) uint8_t smem[];
        constexpr int cc = CC;
        const int npad = a.npad, R = a.rows_per_cta;
        const uint32_t wbytes = fwd_weight_bytes(cc, npad);
        const uint32_t slot_bytes = uint32_t(cc) * kRowPlane;
        const uint32_t tcols = fwd_tmem_cols(npad, R);
        uint8_t* wsm = smem;
        uint8_t* rows = smem + fwd_rows_offset(cc, npad);
        uint64_t* full = reinterpret_cast<uint64_t*>(smem + fwd_bar_offset(cc, npad, R));
        uint64_t* accf = full + R + 4;
        uint64_t* zbar = accf + R;
        uint64_t* wbar = zbar + 1;
        uint64_t* done = wbar + 1;
        uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
        volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);

        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int nwin = a.ncols / kTile;
        const int ngroups = (a.nrows + R - 1) / R;
        int t = blockIdx.x;
        const int cw = t % nwin;
        t /= nwin;
        const int rg = t % ngroups;
        const int b = t / ngroups;
        const int c0 = cw * kTile;
        const int r0 = rg * R;
        const int nout = min(R, a.nrows - r0);
        const int nin = nout + 4;

        if (threadIdx.x == 0)
        {
            // a row completes with its bulk copies and one arrival per wrapped site (below)
            const int wrapped = (c0 == 0 ? 2 : 0) + (c0 + kTile == a.ncols ? 2 : 0);
            for (int i = 0; i < R + 4; ++i) mbar_init(&full[i], 1 + cc * wrapped);
            for (int i = 0; i < R; ++i) mbar_init(&accf[i], 1);
            mbar_init(zbar, 256);
            mbar_init(wbar, 1);
            mbar_init(done, 1);
            *abort = 0;
            fence_mbar_init();
        }
        if (warp == 0)
        {
            tmem_alloc(tslot, tcols);
            tmem_relinquish();
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        const uint32_t tbase = *tslot;

        if (warp == 0)
        {
            // The window's sites c0-2 .. c0+129 of each (row, channel chunk): the in-range run by
            // ONE bulk copy here; where the window wraps round the periodic row (first and last
            // windows, 2 sites each side) the epilogue warps copy the wrapped 16-byte sites
            // before their first wait (one mbarrier arrival each).
            const int left = c0 == 0 ? 2 : 0;
            const int right = c0 + kTile == a.ncols ? 2 : 0;
            const int lo = c0 - 2 + left;          // first in-range column of the window
            const int run = kSites - left - right; // in-range sites
            if (lane == 0)
            {
                // every input row of this CTA at once, one mbarrier per row, in the order
                // the MMAs consume them
                mbar_expect_tx(wbar, wbytes);
                bulk_g2s(wsm, a.wimg, wbytes, wbar);
                for (int i = 0; i < nin; ++i)
                {
                    const int row = wrap_row(r0 - 2 + i, a.nrows);
                    mbar_expect_tx(&full[i], uint32_t(cc * run) * 16u);
                    uint8_t* dst = rows + i * slot_bytes;
                    for (int q = 0; q < cc; ++q)
                    {
                        const uint16_t* src = a.in + (size_t(b * cc + q) * a.nrows + row) * size_t(a.ncols) * 8;
                        bulk_g2s(dst + q * kRowPlane + left * 16, src + size_t(lo) * 8, uint32_t(run) * 16u,
                                 &full[i]);
                    }
                }
                // no copy may still be in flight when the CTA exits
                mbar_wait(wbar, 0, nullptr);
                for (int i = 0; i < nin; ++i) mbar_wait(&full[i], 0, nullptr);
            }
        }
        else if (warp == 1)
        {
            if (lane == 0)
            {
                const uint32_t wsa = smem_u32(wsm), rsa = smem_u32(rows);
                const uint32_t kblock = 5u * npad * 16u;  // one (x tap, channel chunk) block of the image
                bool ok = mbar_wait(wbar, 0, abort) && mbar_wait(zbar, 0, abort);
                tc_fence_after();
                bool issued_any = false;
                for (int i = 0; ok && i < nin; ++i)
                {
                    if (!mbar_wait(&full[i], 0, abort))
                    {
                        ok = false;
                        break;
                    }
                    // slice s of this row's MMA feeds output row i - 4 + s (y tap 4 - s)
                    const int s_lo = i < 4 ? 4 - i : 0;
                    const int s_hi = nout + 3 - i < 4 ? nout + 3 - i : 4;
                    if (s_lo <= s_hi)
                    {
                        const int n = npad * (s_hi - s_lo + 1);
                        const uint32_t idesc = idesc_bf16(128, n, false, false);
                        const uint32_t d = tbase + uint32_t((i - 4 + s_lo) * npad);
                        // base descriptors of this row; every MMA adds (byte offset >> 4) to the start
                        // address field (addresses stay below 256 KiB, so the 14-bit field never carries)
                        const uint64_t a0 = smem_desc(rsa + i * slot_bytes, kRowPlane, 128);
                        const uint64_t b0 = smem_desc(wsa + uint32_t(s_lo * npad * 16), kblock, 128);
                        const uint64_t bstep = kblock >> 4;
#pragma unroll
                        for (int kx = 0; kx < 5; ++kx)
#pragma unroll
                            for (int ks = 0; ks < cc / 2; ++ks)
                                mma_bf16(d, a0 + uint64_t((2 * ks * kRowPlane + kx * 16) >> 4),
                                         b0 + uint64_t(kx * cc + 2 * ks) * bstep, idesc, 1u);
                        issued_any = true;
                    }
                    if (i >= 4) mma_commit(&accf[i - 4]);  // output row i - 4 has all five y taps
                }
                if (!ok) give_up(a.error, abort, 2);
                if (issued_any)
                {
                    mma_commit(done);
                    mbar_wait(done, 0, nullptr);
                }
            }
        }
        else
        {
            // warps 2-9: lane quarter (warp % 4) of the tile, column half (warp - 2) / 4
            const int q4 = warp & 3;  // the TMEM lane quarter this warp may access
            const int half = (warp - 2) >> 2;
            const int m = q4 * 32 + lane;
            const int col = c0 + m;
            const int nq = npad / 8;
            const bool active = half * 16 < npad;  // npad 16: the second half has no columns
            const size_t plane = size_t(a.nrows) * a.ncols;
            float bias[16];
#pragma unroll
            for (int e = 0; e < 16; ++e)
            {
                const int n = half * 16 + e;
                bias[e] = (a.bias && n < npad) ? a.bias[n] : 0.f;
            }
            // zero this warp's half of the accumulator columns in its lane quarter
            const uint32_t lanes = uint32_t(q4 * 32) << 16;
            for (uint32_t c = half * (tcols / 2); c < (half + 1) * (tcols / 2); c += 16)
                tmem_st16_zero(tbase + lanes + c);
            tmem_wait_st();
            tc_fence_before();
            mbar_arrive(zbar);
            {
                // the wrapped sites of the staged rows (see warp 0): 16-byte plain copies, made
                // visible to the async proxy, one arrival on the row's mbarrier each
                const int left = c0 == 0 ? 2 : 0;
                const int right = c0 + kTile == a.ncols ? 2 : 0;
                const int per_chunk = left + right, per_row = cc * per_chunk;
                for (int it = int(threadIdx.x) - 64; it < nin * per_row; it += kFwdThreads - 64)
                {
                    const int i = it / per_row, rem = it - i * per_row;
                    const int q = rem / per_chunk, s = rem - q * per_chunk;
                    const bool at_left = s < left;
                    const int wsite = at_left ? s : kSites - right + (s - left);  // site in the window
                    const int gcol = at_left ? a.ncols - 2 + s : s - left;        // its periodic column
                    const int row = wrap_row(r0 - 2 + i, a.nrows);
                    const uint4 v = *reinterpret_cast<const uint4*>(
                        a.in + ((size_t(b * cc + q) * a.nrows + row) * size_t(a.ncols) + gcol) * 8);
                    *reinterpret_cast<uint4*>(rows + i * slot_bytes + q * kRowPlane + wsite * 16) = v;
                    fence_proxy_async();
                    mbar_arrive(&full[i]);
                }
            }
            for (int j = 0; j < nout; ++j)
            {
                bool ok = mbar_wait(&accf[j], 0, abort);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok)
                {
                    if (lane == 0) give_up(a.error, abort, 3);
                    break;
                }
                tc_fence_after();
                if (!active) continue;
                float v[32];
                tmem_ld16(tbase + lanes + uint32_t(j * npad + half * 16), v);
                tmem_wait_ld();

                const int row = r0 + j;
                const size_t site = size_t(row) * a.ncols + col;
                if (a.epilogue == EPI_F32)
                {
#pragma unroll
                    for (int e = 0; e < 16; ++e)
                    {
                        const int n = half * 16 + e;
                        if (n < a.cout) a.out_f32[(size_t(b) * a.cout + n) * plane + site] = v[e] + bias[e];
                    }
                }
                else
                {
#pragma unroll
                    for (int qq = 0; qq < 2; ++qq)
                    {
                        const int q = half * 2 + qq;
                        if (q >= nq) break;
                        const size_t off = ((size_t(b) * nq + q) * plane + site) * 8;
                        float o[8];
                        if (a.epilogue == EPI_GELU)
                        {
                            float z[8];
#pragma unroll
                            for (int e = 0; e < 8; ++e)
                            {
                                z[e] = v[8 * qq + e] + bias[8 * qq + e];
                                o[e] = gelu_f(z[e]);
                            }
                            if (a.pre)
                                *reinterpret_cast<uint4*>(a.pre + off) =
                                    make_uint4(pack_bf16x2(z[0], z[1]), pack_bf16x2(z[2], z[3]),
                                               pack_bf16x2(z[4], z[5]), pack_bf16x2(z[6], z[7]));
                        }
                        else
                        {
                            float g[8];
                            unpack_bf16x8(*reinterpret_cast<const uint4*>(a.gate + off), g);
#pragma unroll
                            for (int e = 0; e < 8; ++e) o[e] = v[8 * qq + e] * gelu_grad_f(g[e]);
                        }
                        *reinterpret_cast<uint4*>(a.out + off) =
                            make_uint4(pack_bf16x2(o[0], o[1]), pack_bf16x2(o[2], o[3]), pack_bf16x2(o[4], o[5]),
                                       pack_bf16x2(o[6], o[7]));
                    }
                }
            }
        }

        tc_fence_before();
        __syncthreads();
        if (warp == 0)
        {
            tc_fence_after();
            tmem_dealloc(tbase, tcols);
        }
    }

    // =========================================================== weight grad
    __global__ void __launch_bounds__(kThreads) conv_wgrad_kernel(const WgradArgs a)
    {
        extern __shared__ __align__(1024) uint8_t smem[];
        const int cc = a.cin_chunks, npad = a.npad, nq = npad / 8;
        const int R = a.rows_per_cta;
        const uint32_t xrow = uint32_t(cc) * kRowPlane;    // bytes per staged X row
        const uint32_t dzrow = uint32_t(nq) * kTile * 16;  // bytes per staged dZ row
        uint8_t* xs = smem;
        uint8_t* dzs = smem + align128(wg_x_bytes(cc, R));
        uint64_t* bars = reinterpret_cast<uint64_t*>(smem + wg_bar_offset(cc, npad, R));
        uint64_t* ld = bars;
        uint64_t* done = bars + 1;
        uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
        volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);

        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const int nwin = a.ncols / kTile;
        const int ngroups = (a.nrows + R - 1) / R;
        int t = blockIdx.x;
        const int cw = t % nwin;
        t /= nwin;
        const int rg = t % ngroups;
        const int b = t / ngroups;
        const int c0 = cw * kTile;
        const int r0 = rg * R;
        const int nout = min(R, a.nrows - r0);
        const int nx_rows = nout + wg_extra_rows(cc);
        const int kb = wg_kb(cc), nst = wg_nstarts(cc);

        // the X windows' wrapped sites (first and last windows) are copied by the epilogue
        // warps, one arrival on `ld` each (see the forward kernel)
        const int wleft = c0 == 0 ? 2 : 0, wright = c0 + kTile == a.ncols ? 2 : 0;
        if (threadIdx.x == 0)
        {
            mbar_init(ld, 1 + nx_rows * cc * (wleft + wright));
            mbar_init(done, 1);
            *abort = 0;
            fence_mbar_init();
        }
        if (warp == 0)
        {
            tmem_alloc(tslot, 512);
            tmem_relinquish();
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        const uint32_t tbase = *tslot;

        if (warp == 0)
        {
            if (lane == 0)
            {
                const int lo = c0 - 2 + wleft, run = kSites - wleft - wright;  // in-range run of a window
                const uint32_t bytes = uint32_t(nx_rows * cc * run) * 16u + uint32_t(nout) * dzrow;
                mbar_expect_tx(ld, bytes);
                for (int i = 0; i < nx_rows; ++i)
                {
                    const int row = wrap_row(r0 - 2 + i, a.nrows);
                    for (int q = 0; q < cc; ++q)
                    {
                        const uint16_t* src = a.x + (size_t(b * cc + q) * a.nrows + row) * size_t(a.ncols) * 8;
                        bulk_g2s(xs + i * xrow + q * kRowPlane + wleft * 16, src + size_t(lo) * 8,
                                 uint32_t(run) * 16u, ld);
                    }
                }
                for (int j = 0; j < nout; ++j)
                    for (int q = 0; q < nq; ++q)
                    {
                        const uint16_t* src =
                            a.dz + ((size_t(b * nq + q) * a.nrows + (r0 + j)) * size_t(a.ncols) + c0) * 8;
                        bulk_g2s(dzs + j * dzrow + q * (kTile * 16), src, kTile * 16, ld);
                    }
                if (!mbar_wait(ld, 0, nullptr)) give_up(a.error, abort, 4);
            }
        }
        else if (warp == 1)
        {
            if (lane == 0)
            {
                const uint32_t idesc = idesc_bf16(128, npad, true, true);
                const uint32_t xa = smem_u32(xs), za = smem_u32(dzs);
                bool ok = mbar_wait(ld, 0, abort);
                if (ok)
                {
                    for (int j = 0; j < nout; ++j)
                        for (int ks = 0; ks < kTile / 16; ++ks)
                            for (int kx = 0; kx < 5; ++kx)
                                for (int si = 0; si < nst; ++si)
                                {
                                    const uint32_t astart =
                                        xa + (j + wg_start(cc, si)) * xrow + (ks * 16 + kx) * 16;
                                    const uint64_t ad = smem_desc(astart, 128, kRowPlane);
                                    const uint64_t bd = smem_desc(za + j * dzrow + ks * 256, 128, kTile * 16);
                                    const uint32_t d = tbase + uint32_t((kx * nst + si) * npad);
                                    mma_bf16(d, ad, bd, idesc, (j | ks) ? 1u : 0u);
                                }
                    mma_commit(done);
                    if (!mbar_wait(done, 0, nullptr)) give_up(a.error, abort, 5);
                }
                else
                    give_up(a.error, abort, 6);
            }
        }
        else
        {
            const int q4 = warp & 3;
            const int m = q4 * 32 + lane;  // accumulator row = (ky block, channel chunk, channel)
            const int g = m >> 3, e = m & 7;
            const int kyb = g / cc, ci = (g % cc) * 8 + e;
            const int cin = cc * 8;
            {
                const int per_chunk = wleft + wright, per_row = cc * per_chunk;
                for (int it = int(threadIdx.x) - 64; it < nx_rows * per_row; it += kThreads - 64)
                {
                    const int i = it / per_row, rem = it - i * per_row;
                    const int q = rem / per_chunk, s = rem - q * per_chunk;
                    const bool at_left = s < wleft;
                    const int wsite = at_left ? s : kSites - wright + (s - wleft);
                    const int gcol = at_left ? a.ncols - 2 + s : s - wleft;
                    const int row = wrap_row(r0 - 2 + i, a.nrows);
                    const uint4 v = *reinterpret_cast<const uint4*>(
                        a.x + ((size_t(b * cc + q) * a.nrows + row) * size_t(a.ncols) + gcol) * 8);
                    *reinterpret_cast<uint4*>(xs + i * xrow + q * kRowPlane + wsite * 16) = v;
                    fence_proxy_async();
                    mbar_arrive(ld);
                }
            }
            bool ok = mbar_wait(done, 0, abort);
            ok = __all_sync(0xffffffffu, ok);
            if (ok)
            {
                tc_fence_after();
                for (int kx = 0; kx < 5; ++kx)
                    for (int si = 0; si < nst; ++si)
                    {
                        float v[32];
                        const uint32_t taddr = tbase + (uint32_t(q4 * 32) << 16) + uint32_t((kx * nst + si) * npad);
                        if (npad == 32) tmem_ld32(taddr, v);
                        else tmem_ld16(taddr, v);
                        tmem_wait_ld();
                        const int ky = wg_start(cc, si) + kyb;
                        // keep each ky once: start 0 covers [0, kb), the second start only ky >= kb
                        const bool keep = ky < 5 && (si == 0 || ky >= kb);
                        if (keep)
                        {
                            float* dst = a.partial + ((size_t(blockIdx.x) * kTaps + ky * 5 + kx) * cin + ci) * npad;
#pragma unroll
                            for (int n = 0; n < 32; n += 4)
                                if (n < npad)
                                    *reinterpret_cast<float4*>(dst + n) =
                                        make_float4(v[n], v[n + 1], v[n + 2], v[n + 3]);
                        }
                    }
            }
            else if (lane == 0)
                give_up(a.error, abort, 7);
        }

        tc_fence_before();
        __syncthreads();
        if (warp == 0)
        {
            tc_fence_after();
            tmem_dealloc(tbase, 512);
        }
    }

    __global__ void wgrad_reduce_kernel(const float* __restrict__ partial, int nparts, int total, float* __restrict__ dw)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        {
            float s = 0.f;
            for (int p = 0; p < nparts; ++p) s += partial[size_t(p) * total + i];
            dw[i] = s;
        }
    }

    // ================================================== learned-step helpers
    // Network input planes from the field and per-sample parameters: channel 0 =
    // bf16(phi), 1 = 256 (phi - bf16(phi)) (the rounding remainder, so phi is
    // carried to ~16 significant bits), 2 = zeta / 4, 3 = lambda, 4 = 10 T, 5-15 = 0.
    __global__ void learned_input_kernel(const float* __restrict__ phi, const float* __restrict__ params, int batch,
                                         int nrows, int ncols, uint16_t* __restrict__ x)
    {
        const size_t plane = size_t(nrows) * ncols;
        const size_t n = size_t(batch) * plane;
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        {
            const int b = int(i / plane);
            const size_t s = i - size_t(b) * plane;
            const float f = phi[i];
            const __nv_bfloat16 hi = __float2bfloat16_rn(f);
            const float lo = (f - __bfloat162float(hi)) * 256.f;
            const float* pr = params + 3 * b;
            uint4 c0 = make_uint4(pack_bf16x2(__bfloat162float(hi), lo), pack_bf16x2(pr[0] * 0.25f, pr[1]),
                                  pack_bf16x2(pr[2] * 10.f, 0.f), 0u);
            reinterpret_cast<uint4*>(x)[(size_t(b) * 2 + 0) * plane + s] = c0;
            reinterpret_cast<uint4*>(x)[(size_t(b) * 2 + 1) * plane + s] = make_uint4(0, 0, 0, 0);
        }
    }

    // Two standard normals per site for the macro-step noise flux, Philox keyed
    // (seed, *step, site, component).
    __global__ void learned_noise_kernel(float* __restrict__ xi, int nrows, int ncols, uint64_t seed,
                                         const int64_t* __restrict__ step)
    {
        const int64_t st = *step;
        const size_t plane = size_t(nrows) * ncols;
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < plane; i += size_t(gridDim.x) * blockDim.x)
        {
            const int r = int(i / ncols), c = int(i - size_t(r) * ncols);
            xi[i] = amb::noise_normal(seed, st, r, c, 0);
            xi[plane + i] = amb::noise_normal(seed, st, r, c, 1);
        }
    }

    // The rfft2 spectra of two real white-noise fields of unit variance per site, drawn directly:
    // out[comp][r][k] at out + comp * n + r * rs + k * ks (complex64; k < ncols/2 + 1). Off the
    // self-conjugate columns (k = 0 and, for even ncols, k = ncols/2) each mode is a complex
    // normal with E|z|^2 = nrows ncols; in those columns mode r is the conjugate of mode
    // nrows - r, and the self-conjugate modes (r = 0, r = nrows/2) are real with the same
    // variance. One Philox call per (r, k) (keyed by the lower of r and nrows - r in those
    // columns) gives both components.
    __device__ __forceinline__ void spectral_noise_mode(uint64_t seed, int64_t st, int r, int k, int nrows, int ncols,
                                                        float2& vy, float2& vx)
    {
        const float s_half = sqrtf(0.5f * float(nrows) * float(ncols));
        const float s_full = sqrtf(float(nrows) * float(ncols));
        const bool herm = k == 0 || (ncols % 2 == 0 && k == ncols / 2);
        int rr = r;
        bool conj = false;
        if (herm && r > nrows / 2)
        {
            rr = nrows - r;
            conj = true;
        }
        const amb::U4 b = amb::noise_bits(seed, st, rr, 4 * k, 0);
        const float2 z0 = amb::box_muller_f32(b.x, b.y), z1 = amb::box_muller_f32(b.z, b.w);
        vy = make_float2(z0.x * s_half, z0.y * s_half);
        vx = make_float2(z1.x * s_half, z1.y * s_half);
        if (herm && (rr == 0 || (nrows % 2 == 0 && rr == nrows / 2)))
        {
            vy = make_float2(z0.x * s_full, 0.f);
            vx = make_float2(z1.x * s_full, 0.f);
        }
        if (conj)
        {
            vy.y = -vy.y;
            vx.y = -vx.y;
        }
    }

    __global__ void learned_noise_spectral_kernel(float2* __restrict__ out, int nrows, int ncols, int64_t rs,
                                                  int64_t ks, int64_t n, uint64_t seed,
                                                  const int64_t* __restrict__ step)
    {
        const int nk = ncols / 2 + 1;
        const int64_t st = *step;
        const int64_t total = int64_t(nrows) * nk;
        for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
             i += int64_t(gridDim.x) * blockDim.x)
        {
            const int r = int(i / nk), k = int(i - int64_t(r) * nk);
            float2 vy, vx;
            spectral_noise_mode(seed, st, r, k, nrows, ncols, vy, vx);
            out[int64_t(r) * rs + int64_t(k) * ks] = vy;
            out[n + int64_t(r) * rs + int64_t(k) * ks] = vx;
        }
    }

    // The spectral combine with the noise spectrum drawn in place (the draw of
    // learned_noise_spectral_kernel for the same seed and step): the spectra are dense in
    // memory with row stride rs and column stride ks, one of them 1.
    __global__ void spectral_combine_noise_kernel(const float2* __restrict__ phi_hat, const float2* __restrict__ my,
                                                  const float2* __restrict__ mx, const float2* __restrict__ ny_,
                                                  const float2* __restrict__ nx_, float noise_mag, int nrows,
                                                  int ncols, int64_t rs, int64_t ks, uint64_t seed,
                                                  const int64_t* __restrict__ step, float2* __restrict__ out_y,
                                                  float2* __restrict__ out_x)
    {
        const int64_t n = int64_t(nrows) * (ncols / 2 + 1);
        const int64_t st = *step;
        for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        {
            int r, k;
            if (n <= INT32_MAX)  // 32-bit division (a 64-bit one costs several times the instructions)
            {
                const int ii = int(i);
                if (ks == 1)
                {
                    r = ii / int(rs);
                    k = ii - r * int(rs);
                }
                else
                {
                    k = ii / int(ks);
                    r = ii - k * int(ks);
                }
            }
            else if (ks == 1)
            {
                r = int(i / rs);
                k = int(i - int64_t(r) * rs);
            }
            else
            {
                k = int(i / ks);
                r = int(i - int64_t(k) * ks);
            }
            float2 u, v;
            spectral_noise_mode(seed, st, r, k, nrows, ncols, u, v);
            const float2 p = phi_hat[i], a = my[i], b = mx[i], c = ny_[i], d = nx_[i];
            float2 y = make_float2(p.x * a.x - p.y * a.y, p.x * a.y + p.y * a.x);
            float2 x = make_float2(p.x * b.x - p.y * b.y, p.x * b.y + p.y * b.x);
            y.x += noise_mag * (u.x * c.x - u.y * c.y);
            y.y += noise_mag * (u.x * c.y + u.y * c.x);
            x.x += noise_mag * (v.x * d.x - v.y * d.y);
            x.y += noise_mag * (v.x * d.y + v.y * d.x);
            out_y[i] = y;
            out_x[i] = x;
        }
    }

    // Face weights of the order-8 central derivative written as a difference of face sums:
    // D8 f(j) = F(j + 1/2) - F(j - 1/2) with F(j + 1/2) = sum_e w_e f(j + e), e = -3..4,
    // w_e = sum of c_d over d >= max(e, 1 - e), c = (4/5, -1/5, 4/105, -1/280) (the sum in
    // double, in increasing d, then rounded to float).
    constexpr double kC1 = 4.0 / 5.0, kC2 = -1.0 / 5.0, kC3 = 4.0 / 105.0, kC4 = -1.0 / 280.0;

    __device__ __forceinline__ float d8_face_weight(int e)
    {
        const int d0 = e > 1 - e ? e : 1 - e;
        return d0 == 1 ? float(kC1 + kC2 + kC3 + kC4)
                       : d0 == 2 ? float(kC2 + kC3 + kC4) : d0 == 3 ? float(kC3 + kC4) : float(kC4);
    }

    // Integer face increment through the face after site (r, c) along the axis (dr, dc), in
    // FP32 with explicitly rounded operations, so the two sites sharing the face compute the
    // same integer.
    __device__ __forceinline__ long long face_q(const float* __restrict__ f, const float* __restrict__ extra,
                                                const float* __restrict__ xi, float noise_mag, float scale, int r,
                                                int c, int dr, int dc, int nrows, int ncols)
    {
        const size_t k = size_t(r) * ncols + c;
        float v = f[k];
        if (extra) v = __fadd_rn(v, extra[k]);
        if (xi)
        {
            float s = 0.f;
#pragma unroll
            for (int e = -3; e <= 4; ++e)
            {
                int rr = r + dr * e, cc = c + dc * e;
                rr = rr < 0 ? rr + nrows : (rr >= nrows ? rr - nrows : rr);
                cc = cc < 0 ? cc + ncols : (cc >= ncols ? cc - ncols : cc);
                s = __fadd_rn(s, __fmul_rn(d8_face_weight(e), xi[size_t(rr) * ncols + cc]));
            }
            v = __fadd_rn(v, __fmul_rn(noise_mag, s));
        }
        float q = __fmul_rn(scale, v);
        q = q > 1e9f ? 1e9f : (q < -1e9f ? -1e9f : q);
        return (long long)__float2int_rn(q);  // |q| <= 1e9 < 2^31: the same value as a 64-bit conversion
    }

    // phi_q -= sum of integer face increments (each face computed identically by the two
    // sites that share it, so the sum over all sites is unchanged: exact conservation).
    __global__ void learned_update_kernel(const float* __restrict__ flux, const float* __restrict__ extra,
                                          const float* __restrict__ xi, int nrows, int ncols, float scale_y,
                                          float scale_x, float noise_mag, int32_t* __restrict__ phi_q,
                                          float* __restrict__ phi_f, long long bound, int* __restrict__ flag,
                                          int64_t* __restrict__ advance, const float* __restrict__ params,
                                          uint4* __restrict__ x_next)
    {
        // the next macro step's noise key (nothing in this launch reads it)
        if (advance && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *advance += 1;
        const size_t plane = size_t(nrows) * ncols;
        const float* fy = flux;
        const float* fx = flux + plane;
        const float* ey = extra;
        const float* ex = extra ? extra + plane : nullptr;
        const float* xy = xi;
        const float* xx = xi ? xi + plane : nullptr;
        // rows by blockIdx.y (grid-stride), columns by blockIdx.x and the thread: no division per site
        const int c = blockIdx.x * blockDim.x + threadIdx.x;
        if (c >= ncols) return;
        const int cm = c == 0 ? ncols - 1 : c - 1;
        for (int r = blockIdx.y; r < nrows; r += gridDim.y)
        {
            const size_t i = size_t(r) * ncols + c;
            const int rm = r == 0 ? nrows - 1 : r - 1;
            long long dq = face_q(fx, ex, xx, noise_mag, scale_x, r, c, 0, 1, nrows, ncols) -
                           face_q(fx, ex, xx, noise_mag, scale_x, r, cm, 0, 1, nrows, ncols) +
                           face_q(fy, ey, xy, noise_mag, scale_y, r, c, 1, 0, nrows, ncols) -
                           face_q(fy, ey, xy, noise_mag, scale_y, rm, c, 1, 0, nrows, ncols);
            long long q = (long long)phi_q[i] - dq;
            bool bad = !isfinite(fx[i]) || !isfinite(fy[i]) || q > bound || q < -bound;
            if (extra) bad = bad || !isfinite(ex[i]) || !isfinite(ey[i]);
            if (bad)
            {
                atomicOr(flag, 1);
                q = q > bound ? bound : (q < -bound ? -bound : q);
            }
            phi_q[i] = int32_t(q);
            // q * 2^-24 rounded once to FP32: rounding q to FP32 and scaling by a power of two gives the
            // same value (|q| <= 2e9, so the scaled value is a normal number or zero)
            const float f = __fmul_rn(__int2float_rn(int(q)), 1.0f / 16777216.0f);
            phi_f[i] = f;
            if (x_next)  // channel chunk 0 of the next network input, as learned_input_kernel forms it
            {
                const __nv_bfloat16 hi = __float2bfloat16_rn(f);
                const float lo = (f - __bfloat162float(hi)) * 256.f;
                x_next[i] = make_uint4(pack_bf16x2(__bfloat162float(hi), lo), pack_bf16x2(params[0] * 0.25f, params[1]),
                                       pack_bf16x2(params[2] * 10.f, 0.f), 0u);
            }
        }
    }

    // out_c = phi_hat * m_c + noise_mag * xi_hat_c * n_c for c = y, x (complex rfft2 spectra,
    // [ny][nx/2+1] each; xi_hat may be null).
    __global__ void spectral_combine_kernel(const float2* __restrict__ phi_hat, const float2* __restrict__ xi_hat,
                                            const float2* __restrict__ my, const float2* __restrict__ mx,
                                            const float2* __restrict__ ny_, const float2* __restrict__ nx_,
                                            float noise_mag, size_t n, float2* __restrict__ out_y,
                                            float2* __restrict__ out_x)
    {
        for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        {
            const float2 p = phi_hat[i], a = my[i], b = mx[i];
            float2 y = make_float2(p.x * a.x - p.y * a.y, p.x * a.y + p.y * a.x);
            float2 x = make_float2(p.x * b.x - p.y * b.y, p.x * b.y + p.y * b.x);
            if (xi_hat)
            {
                const float2 u = xi_hat[i], v = xi_hat[n + i], c = ny_[i], d = nx_[i];
                y.x += noise_mag * (u.x * c.x - u.y * c.y);
                y.y += noise_mag * (u.x * c.y + u.y * c.x);
                x.x += noise_mag * (v.x * d.x - v.y * d.y);
                x.y += noise_mag * (v.x * d.y + v.y * d.x);
            }
            out_y[i] = y;
            out_x[i] = x;
        }
    }

    int g_sms = 0;
    std::once_flag g_sms_once;

    int sm_count()
    {
        std::call_once(g_sms_once, [] {
            int dev = 0;
            cudaGetDevice(&dev);
            if (cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || g_sms < 1)
                g_sms = 148;
        });
        return g_sms;
    }

    // Rows per CTA for the forward kernel: every CTA stages all its input rows at once, so
    // shared memory and TMEM per CTA grow with the rows (at most kMaxFwdRows); one CTA per
    // SM (320 threads at ~150 registers); cost = waves x (rows + about three row times of
    // pipeline fill).
    int choose_fwd_rows(int batch, int nrows, int nwin, int cc, int npad)
    {
        const int sms = sm_count();
        int best = 1;
        double best_cost = 1e30;
        for (int r = 1; r <= kMaxFwdRows && r <= nrows; ++r)
        {
            if (fwd_smem_bytes(cc, npad, r) > kSmemLimit || npad * r > 512) break;
            const long long grid = (long long)batch * nwin * ((nrows + r - 1) / r);
            const long long waves = (grid + sms - 1) / sms;
            const double cost = double(waves) * (r + 3);
            if (cost < best_cost - 1e-9)
            {
                best_cost = cost;
                best = r;
            }
        }
        return best;
    }

    constexpr int kWgradRows = 8;

    // Raises a kernel's dynamic shared-memory limit once per device (so that later
    // launches, e.g. inside a stream capture, make no attribute calls).
    std::mutex g_attr_mutex;
    int g_attr_selftest[64], g_attr_fwd[64], g_attr_fwd2[64], g_attr_wgrad[64];

    cudaError_t set_smem_attr(const void* fn, uint32_t bytes, int (&done)[64])
    {
        std::lock_guard<std::mutex> lock(g_attr_mutex);
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
        if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = 1;
        return e;
    }

    bool valid_geometry(int batch, int nrows, int ncols)
    {
        return batch >= 1 && nrows >= 3 && ncols >= kTile && ncols % kTile == 0 &&
               (long long)batch * nrows * ncols < (1ll << 31);
    }

    int fail_invalid(const char* what)
    {
        amb::set_last_error(what);
        return AMB_ERR_INVALID;
    }

    int fail_cuda(const char* what, cudaError_t e)
    {
        amb::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        return AMB_ERR_CUDA;
    }
}

// ============================================================= C ABI

extern "C" int amb_tc_selftest(const void* a, const void* b, float* d, int n, int k, int a_mn_major, int b_mn_major,
                               int* error, void* stream)
{
    if (!a || !b || !d || (n != 16 && n != 32) || k < 16 || k > 64 || k % 16 != 0)
        return fail_invalid("amb_tc_selftest: n must be 16 or 32, k in {16, 32, 48, 64}");
    const uint32_t smem = 98304 + 256;
    cudaError_t e = set_smem_attr(reinterpret_cast<const void*>(tc_selftest_kernel), smem, g_attr_selftest);
    if (e == cudaSuccess)
    {
        tc_selftest_kernel<<<1, 128, smem, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const uint16_t*>(a), static_cast<const uint16_t*>(b), d, n, k, a_mn_major, b_mn_major, error);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_tc_selftest", e);
}

extern "C" int amb_conv5x5_forward(const void* in, int batch, int nrows, int ncols, int cin, const void* wimg,
                                   const float* bias, int npad, int cout, int epilogue, void* out, void* pre,
                                   const void* gate, float* out_f32, int* error, void* stream)
{
    if (!in || !wimg || !valid_geometry(batch, nrows, ncols) || (cin != 16 && cin != 32) ||
        (npad != 16 && npad != 32) || epilogue < 0 || epilogue > 2)
        return fail_invalid("amb_conv5x5_forward: need ncols % 128 == 0, nrows >= 3, cin and npad in {16, 32}");
    if (epilogue == EPI_F32 && (!out_f32 || cout < 1 || cout > npad))
        return fail_invalid("amb_conv5x5_forward: FP32 epilogue needs out_f32 and 1 <= cout <= npad");
    if (epilogue != EPI_F32 && !out) return fail_invalid("amb_conv5x5_forward: bf16 epilogue needs out");
    if (epilogue == EPI_GELU_BWD && !gate) return fail_invalid("amb_conv5x5_forward: GELU' epilogue needs gate");
    const auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    if (!al16(in) || !al16(wimg) || (out && !al16(out)) || (pre && !al16(pre)) || (gate && !al16(gate)))
        return fail_invalid("amb_conv5x5_forward: bf16 buffers must be 16-byte aligned");

    FwdArgs a{};
    a.in = static_cast<const uint16_t*>(in);
    a.wimg = static_cast<const uint16_t*>(wimg);
    a.bias = bias;
    a.out = static_cast<uint16_t*>(out);
    a.pre = static_cast<uint16_t*>(pre);
    a.gate = static_cast<const uint16_t*>(gate);
    a.out_f32 = out_f32;
    a.batch = batch;
    a.nrows = nrows;
    a.ncols = ncols;
    a.cin_chunks = cin / 8;
    a.npad = npad;
    a.cout = epilogue == EPI_F32 ? cout : npad;
    a.epilogue = epilogue;
    const int nwin = ncols / kTile;
    a.rows_per_cta = choose_fwd_rows(batch, nrows, nwin, a.cin_chunks, npad);
    a.error = error;
    const uint32_t smem = fwd_smem_bytes(a.cin_chunks, npad, a.rows_per_cta);
    auto kern = a.cin_chunks == 4 ? conv_fwd_kernel<4> : conv_fwd_kernel<2>;
    cudaError_t e = set_smem_attr(reinterpret_cast<const void*>(kern), kSmemLimit,
                                  a.cin_chunks == 4 ? g_attr_fwd : g_attr_fwd2);
    if (e == cudaSuccess)
    {
        const long long grid = (long long)batch * nwin * ((nrows + a.rows_per_cta - 1) / a.rows_per_cta);
        kern<<<unsigned(grid), kFwdThreads, smem, static_cast<cudaStream_t>(stream)>>>(a);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_conv5x5_forward", e);
}

static long long wgrad_grid(int batch, int nrows, int ncols)
{
    return (long long)batch * (ncols / kTile) * ((nrows + kWgradRows - 1) / kWgradRows);
}

extern "C" size_t amb_conv5x5_wgrad_scratch_bytes(int batch, int nrows, int ncols, int cin, int npad)
{
    if (!valid_geometry(batch, nrows, ncols)) return 0;
    return size_t(wgrad_grid(batch, nrows, ncols)) * kTaps * cin * npad * sizeof(float);
}

extern "C" int amb_conv5x5_wgrad(const void* x, const void* dz, int batch, int nrows, int ncols, int cin, int npad,
                                 float* dw, float* scratch, size_t scratch_bytes, int* error, void* stream)
{
    if (!x || !dz || !dw || !scratch || !valid_geometry(batch, nrows, ncols) || (cin != 16 && cin != 32) ||
        (npad != 16 && npad != 32))
        return fail_invalid("amb_conv5x5_wgrad: need ncols % 128 == 0, nrows >= 3, cin and npad in {16, 32}");
    if (scratch_bytes < amb_conv5x5_wgrad_scratch_bytes(batch, nrows, ncols, cin, npad))
        return fail_invalid("amb_conv5x5_wgrad: scratch too small (see amb_conv5x5_wgrad_scratch_bytes)");
    WgradArgs a{};
    a.x = static_cast<const uint16_t*>(x);
    a.dz = static_cast<const uint16_t*>(dz);
    a.partial = scratch;
    a.batch = batch;
    a.nrows = nrows;
    a.ncols = ncols;
    a.cin_chunks = cin / 8;
    a.npad = npad;
    a.rows_per_cta = kWgradRows;
    a.error = error;
    const uint32_t smem = wg_smem_bytes(a.cin_chunks, npad, kWgradRows);
    cudaError_t e = set_smem_attr(reinterpret_cast<const void*>(conv_wgrad_kernel),
                                  std::max(wg_smem_bytes(4, 32, kWgradRows), wg_smem_bytes(2, 32, kWgradRows)),
                                  g_attr_wgrad);
    auto s = static_cast<cudaStream_t>(stream);
    const long long grid = wgrad_grid(batch, nrows, ncols);
    if (e == cudaSuccess)
    {
        conv_wgrad_kernel<<<unsigned(grid), kThreads, smem, s>>>(a);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
    {
        const int total = kTaps * cin * npad;
        wgrad_reduce_kernel<<<(total + 255) / 256, 256, 0, s>>>(scratch, int(grid), total, dw);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_conv5x5_wgrad", e);
}

extern "C" int amb_learned_input(const float* phi, const float* params, int batch, int nrows, int ncols, void* x,
                                 void* stream)
{
    if (!phi || !params || !x || !valid_geometry(batch, nrows, ncols))
        return fail_invalid("amb_learned_input: bad arguments");
    const size_t n = size_t(batch) * nrows * ncols;
    const int grid = int(std::min<size_t>((n + 255) / 256, size_t(sm_count()) * 16));
    learned_input_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(phi, params, batch, nrows, ncols,
                                                                            static_cast<uint16_t*>(x));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_learned_input", e);
}

extern "C" int amb_learned_noise(int nrows, int ncols, uint64_t seed, const int64_t* step, float* xi, void* stream)
{
    if (!step || !xi || nrows < 1 || ncols < 1) return fail_invalid("amb_learned_noise: bad arguments");
    const size_t n = size_t(nrows) * ncols;
    const int grid = int(std::min<size_t>((n + 255) / 256, size_t(sm_count()) * 16));
    learned_noise_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(xi, nrows, ncols, seed, step);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_learned_noise", e);
}

static int learned_update_launch(const float* flux, const float* extra, int nrows, int ncols, double dt_macro,
                                 double dx, double dy, const float* xi, double noise_mag, int32_t* phi_q, float* phi_f,
                                 double bound, int* flag, int64_t* step_to_advance, const float* params, void* x_next,
                                 void* stream)
{
    auto s = static_cast<cudaStream_t>(stream);
    const dim3 grid((ncols + 255) / 256, std::min(nrows, 65535));
    const double fix = 16777216.0;
    const double qb = std::min(bound * fix, 2.0e9);
    const bool noisy = xi && noise_mag > 0;
    learned_update_kernel<<<grid, 256, 0, s>>>(flux, extra, noisy ? xi : nullptr, nrows, ncols,
                                               float(dt_macro / dy * fix), float(dt_macro / dx * fix),
                                               noisy ? float(noise_mag) : 0.f, phi_q, phi_f, (long long)qb, flag,
                                               step_to_advance, params, static_cast<uint4*>(x_next));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_learned_update", e);
}

static bool learned_update_args_ok(const float* flux, const int32_t* phi_q, const float* phi_f, const int* flag,
                                   int nrows, int ncols, double dt_macro, double dx, double dy, double noise_mag,
                                   double bound)
{
    return flux && phi_q && phi_f && flag && nrows >= 1 && ncols >= 1 && dt_macro > 0 && dx > 0 && dy > 0 &&
           noise_mag >= 0 && bound > 0;
}

extern "C" int amb_learned_update(const float* flux, const float* extra, int nrows, int ncols, double dt_macro,
                                  double dx, double dy, const float* xi, double noise_mag, int32_t* phi_q,
                                  float* phi_f, double bound, int* flag, int64_t* step_to_advance, void* stream)
{
    if (!learned_update_args_ok(flux, phi_q, phi_f, flag, nrows, ncols, dt_macro, dx, dy, noise_mag, bound))
        return fail_invalid("amb_learned_update: bad arguments");
    return learned_update_launch(flux, extra, nrows, ncols, dt_macro, dx, dy, xi, noise_mag, phi_q, phi_f, bound,
                                 flag, step_to_advance, nullptr, nullptr, stream);
}

extern "C" int amb_learned_update_input(const float* flux, const float* extra, int nrows, int ncols, double dt_macro,
                                        double dx, double dy, const float* xi, double noise_mag, int32_t* phi_q,
                                        float* phi_f, double bound, int* flag, int64_t* step_to_advance,
                                        const float* params, void* x_next, void* stream)
{
    if (!learned_update_args_ok(flux, phi_q, phi_f, flag, nrows, ncols, dt_macro, dx, dy, noise_mag, bound) ||
        !params || !x_next || (reinterpret_cast<uintptr_t>(x_next) & 15) != 0)
        return fail_invalid("amb_learned_update_input: bad arguments");
    return learned_update_launch(flux, extra, nrows, ncols, dt_macro, dx, dy, xi, noise_mag, phi_q, phi_f, bound,
                                 flag, step_to_advance, params, x_next, stream);
}

extern "C" int amb_learned_spectral_combine(const void* phi_hat, const void* xi_hat, const void* my, const void* mx,
                                            const void* ny, const void* nx, double noise_mag, int64_t n,
                                            void* out_y, void* out_x, void* stream)
{
    if (!phi_hat || !my || !mx || !out_y || !out_x || n < 1 || (xi_hat && (!ny || !nx)))
        return fail_invalid("amb_learned_spectral_combine: bad arguments");
    const int grid = int(std::min<int64_t>((n + 255) / 256, int64_t(sm_count()) * 8));
    spectral_combine_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float2*>(phi_hat), static_cast<const float2*>(xi_hat), static_cast<const float2*>(my),
        static_cast<const float2*>(mx), static_cast<const float2*>(ny), static_cast<const float2*>(nx),
        float(noise_mag), size_t(n), static_cast<float2*>(out_y), static_cast<float2*>(out_x));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_learned_spectral_combine", e);
}

extern "C" int amb_learned_noise_spectral(int nrows, int ncols, uint64_t seed, const int64_t* step, void* out,
                                          int64_t row_stride, int64_t col_stride, void* stream)
{
    if (!step || !out || nrows < 1 || ncols < 2 || row_stride < 1 || col_stride < 1)
        return fail_invalid("amb_learned_noise_spectral: bad arguments");
    const int64_t n = int64_t(nrows) * (ncols / 2 + 1);
    const int grid = int(std::min<int64_t>((n + 255) / 256, int64_t(sm_count()) * 8));
    learned_noise_spectral_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<float2*>(out), nrows, ncols, row_stride, col_stride, n, seed ^ 0x5bd1e995a5a5a5a5ull, step);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_learned_noise_spectral", e);
}

extern "C" int amb_learned_spectral_combine_noise(const void* phi_hat, const void* my, const void* mx, const void* ny,
                                                  const void* nx, double noise_mag, int nrows, int ncols,
                                                  int64_t row_stride, int64_t col_stride, uint64_t seed,
                                                  const int64_t* step, void* out_y, void* out_x, void* stream)
{
    const int64_t nk = ncols / 2 + 1;
    const bool row_major = col_stride == 1 && row_stride == nk;
    const bool col_major = row_stride == 1 && col_stride == nrows;
    if (!phi_hat || !my || !mx || !ny || !nx || !step || !out_y || !out_x || nrows < 1 || ncols < 2 ||
        !(row_major || col_major))
        return fail_invalid("amb_learned_spectral_combine_noise: bad arguments (spectra must be dense)");
    const int64_t n = int64_t(nrows) * nk;
    const int grid = int(std::min<int64_t>((n + 255) / 256, int64_t(sm_count()) * 8));
    spectral_combine_noise_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float2*>(phi_hat), static_cast<const float2*>(my), static_cast<const float2*>(mx),
        static_cast<const float2*>(ny), static_cast<const float2*>(nx), float(noise_mag), nrows, ncols, row_stride,
        col_stride, seed ^ 0x5bd1e995a5a5a5a5ull, step, static_cast<float2*>(out_y), static_cast<float2*>(out_x));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AMB_OK : fail_cuda("amb_learned_spectral_combine_noise", e);
}
