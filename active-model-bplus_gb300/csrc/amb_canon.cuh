// The step's arithmetic, defined once for every kernel that evaluates it.
//
// Every FP32/FP64 step kernel (the shared-memory tile kernel, the warp-pair sliding kernel)
// evaluates the same operations in the same order at every site,
// each rounded exactly once as written here (explicit round-to-nearest intrinsics: the
// compiler may not contract or reorder them), from the same constants (computed once on the
// host by Canon's constructor). The results of the kernels are therefore bitwise equal to
// each other for a given precision, whatever the kernel, tile or launch shape: no result
// depends on which kernel an autotuner picked.
//
// The operators are those of the reference (tranqui/active-model-bplus): the Tjhung 3x3
// gradient and Laplacian (src/finite_difference.h:371-453, src/finite_difference.cuh:166-190)
// and the order-8 central first derivative D8 (src/finite_difference.h:69-75), applied in
// separable form:
//   lap  = lA (Am + Ap) + lB (u0 + d0) + lC A0 + lD f   (A = left + right, per row above (m),
//          centre (0) and below (p); u0, d0 the centre column above and below)
//   gx   = gxb D0 + gxa (Dm + Dp)                      (D = right - left, per row)
//   gy   = gyb (d0 - u0) + gya (Ap - Am)
//   mu_p = ((c f + b) f + a) f - kappa lap;  mu_a = lambda (gy^2 + gx^2);  J_c = zeta lap grad
//   J1   = -D8 mu_p + mag xi (per axis),  D8 g = sum_j d_j (g[+j] - g[-j]) in order j = 1..4
//   J2_y = -dyInv (sx(r+1) - sx(r-1)) + J_c,y,  sx = 0.1 (left + right) + 0.3 centre of mu_a
//   J2_x = jx3 dx(r) + (jx1 (dx(r+1) + dx(r-1)) + J_c,x),  dx = right - left of mu_a
//   divTj = dyInv (sxj(r+1) - sxj(r-1)) + (tx3 dxj(r) + tx1 (dxj(r-1) + dxj(r+1)))  (of J2)
//   div  = D8_x J1_x + (divTj + D8_y J1_y)
//   update: plain phi - dt div (one fused multiply-add); compensated (Kahan, residual r):
//          F = dt div + r (fused), phi' = phi - F, r' = (phi' - phi) + F.
#pragma once

#include "amb_common.cuh"

#include <type_traits>

namespace amb
{
    // Rounded-once arithmetic, never contracted by the compiler.
    __device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
    __device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
    __device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
    __device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
    __device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
    __device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }

    // The constants of one step in the storage precision, computed on the host.
    template <typename Real>
    struct Canon
    {
        Real lA, lB, lC, lD;          // Laplacian weights
        Real gxa, gxb, gya, gyb;      // gradient weights
        Real ny8[4], nx8[4];          // -dyInv d_j, -dxInv d_j   (J1 = -D8 mu_p)
        Real py8[4], px8[4];          // dyInv d_j, dxInv d_j     (D8 J1)
        Real a, b, c, nkappa, lambda, zeta, mag;
        Real ndy, jx1, jx3;           // J2 weights
        Real dyInv, tx1, tx3;         // divTj weights
        Real dt, ndt;
        Real p1, p3;                  // 0.1, 0.3 (x smoothing of mu_a and J2_y)

        __host__ explicit Canon(const StepParams& p)
        {
            const auto R = [](double v) { return Real(v); };
            const double ex = p.dxInv * p.dxInv, ey = p.dyInv * p.dyInv;
            lA = R(-0.25 * (ex + ey));
            lB = R(0.5 * ex + 1.5 * ey);
            lC = R(1.5 * ex + 0.5 * ey);
            lD = R(-3.0 * (ex + ey));
            gxa = R(0.1 * p.dxInv);
            gxb = R(0.3 * p.dxInv);
            gya = R(0.1 * p.dyInv);
            gyb = R(0.3 * p.dyInv);
            for (int j = 0; j < 4; ++j)
            {
                ny8[j] = R(-p.dyInv * d8_tap(j + 1));
                nx8[j] = R(-p.dxInv * d8_tap(j + 1));
                py8[j] = R(p.dyInv * d8_tap(j + 1));
                px8[j] = R(p.dxInv * d8_tap(j + 1));
            }
            a = R(p.a);
            b = R(p.b);
            c = R(p.c);
            nkappa = -R(p.kappa);
            lambda = R(p.lambda);
            zeta = R(p.zeta);
            mag = R(p.noise_mag);
            ndy = R(-p.dyInv);
            jx1 = R(-0.1 * p.dxInv);
            jx3 = R(-0.3 * p.dxInv);
            dyInv = R(p.dyInv);
            tx1 = R(0.1 * p.dxInv);
            tx3 = R(0.3 * p.dxInv);
            dt = R(p.dt);
            ndt = -R(p.dt);
            if constexpr (std::is_same<Real, float>::value)
            {
                p1 = 0.1f;
                p3 = 0.3f;
            }
            else
            {
                p1 = 0.1;
                p3 = 0.3;
            }
        }
    };

    // Stage A at one site from its 3x3 box: rows u (above), m (centre), d (below), each at
    // columns -1, 0, +1 (pointers to the centre column).
    template <typename Real>
    struct SiteA
    {
        Real f, mup, mua, jcy, jcx;
    };

    template <typename Real>
    __device__ __forceinline__ SiteA<Real> canon_stage_a(const Real* u, const Real* m, const Real* d,
                                                         const Canon<Real>& k)
    {
        const Real Am = radd(u[-1], u[1]), Dm = rsub(u[1], u[-1]);
        const Real A0 = radd(m[-1], m[1]), D0 = rsub(m[1], m[-1]);
        const Real Ap = radd(d[-1], d[1]), Dp = rsub(d[1], d[-1]);
        const Real f = m[0];
        Real l = rmul(k.lA, radd(Am, Ap));
        l = rfma(k.lB, radd(u[0], d[0]), l);
        l = rfma(k.lC, A0, l);
        const Real lap = rfma(k.lD, f, l);
        const Real gx = rfma(k.gxb, D0, rmul(k.gxa, radd(Dm, Dp)));
        const Real gy = rfma(k.gyb, rsub(d[0], u[0]), rmul(k.gya, rsub(Ap, Am)));
        SiteA<Real> s;
        s.f = f;
        s.mup = rfma(k.nkappa, lap, rmul(rfma(rfma(k.c, f, k.b), f, k.a), f));
        s.mua = rmul(k.lambda, rfma(gy, gy, rmul(gx, gx)));
        const Real zl = rmul(k.zeta, lap);
        s.jcy = rmul(zl, gy);
        s.jcx = rmul(zl, gx);
        return s;
    }

    // mu_p alone at one site (the same operations as canon_stage_a's mu_p).
    template <typename Real>
    __device__ __forceinline__ Real canon_mu_p(const Real* u, const Real* m, const Real* d, const Canon<Real>& k)
    {
        const Real Am = radd(u[-1], u[1]);
        const Real A0 = radd(m[-1], m[1]);
        const Real Ap = radd(d[-1], d[1]);
        const Real f = m[0];
        Real l = rmul(k.lA, radd(Am, Ap));
        l = rfma(k.lB, radd(u[0], d[0]), l);
        l = rfma(k.lC, A0, l);
        const Real lap = rfma(k.lD, f, l);
        return rfma(k.nkappa, lap, rmul(rfma(rfma(k.c, f, k.b), f, k.a), f));
    }

    // sum_j c_j (g[+j] - g[-j]), j = 1..4, in that order (first a product, then fused).
    template <typename Real>
    __device__ __forceinline__ Real canon_d8(const Real (&c)[4], Real m1, Real p1, Real m2, Real p2, Real m3, Real p3,
                                             Real m4, Real p4)
    {
        Real s = rmul(c[0], rsub(p1, m1));
        s = rfma(c[1], rsub(p2, m2), s);
        s = rfma(c[2], rsub(p3, m3), s);
        return rfma(c[3], rsub(p4, m4), s);
    }

    // 0.1 (left + right) + 0.3 centre (fused).
    template <typename Real>
    __device__ __forceinline__ Real canon_smooth(Real l, Real c, Real r, const Canon<Real>& k)
    {
        return rfma(k.p1, radd(l, r), rmul(k.p3, c));
    }

    // J2_y and J2_x at row r from the x-smoothed (sx) and x-differenced (dx) mu_a rows r-1, r, r+1.
    template <typename Real>
    __device__ __forceinline__ Real canon_j2y(Real sx_m, Real sx_p, Real jcy, const Canon<Real>& k)
    {
        return rfma(k.ndy, rsub(sx_p, sx_m), jcy);
    }

    template <typename Real>
    __device__ __forceinline__ Real canon_j2x(Real dx_m, Real dx_0, Real dx_p, Real jcx, const Canon<Real>& k)
    {
        return rfma(k.jx3, dx_0, rfma(k.jx1, radd(dx_p, dx_m), jcx));
    }

    // Tjhung divergence of J2 at row r from sxj (x-smoothed J2_y) and dxj (x-differenced J2_x)
    // of rows r-1, r, r+1.
    template <typename Real>
    __device__ __forceinline__ Real canon_divtj(Real sxj_m, Real sxj_p, Real dxj_m, Real dxj_0, Real dxj_p,
                                                const Canon<Real>& k)
    {
        Real v = rmul(k.tx1, radd(dxj_m, dxj_p));
        v = rfma(k.tx3, dxj_0, v);
        return rfma(k.dyInv, rsub(sxj_p, sxj_m), v);
    }

    // The update of one site: plain, or compensated with residual r (in/out).
    template <typename Real>
    __device__ __forceinline__ Real canon_update(Real f, Real dx8, Real divtj, Real dy8, const Canon<Real>& k)
    {
        const Real div = radd(dx8, radd(divtj, dy8));
        return rfma(k.ndt, div, f);
    }

    __device__ __forceinline__ float canon_update_comp(float f, float dx8, float divtj, float dy8, float& r,
                                                       const Canon<float>& k)
    {
        const float div = radd(dx8, radd(divtj, dy8));
        const float F = rfma(k.dt, div, r);
        const float nf = rsub(f, F);
        r = radd(rsub(nf, f), F);
        return nf;
    }
}
