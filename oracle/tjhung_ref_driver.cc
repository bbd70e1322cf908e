// C-ABI driver around the reference's own serial CPU scheme,
// test/tjhung_ambplus.h (struct TjhungIntegrator). Test infrastructure only:
// it is compiled by the recipe oracle/build.py from an unmodified, git-ignored
// staged copy of the reference's sources (oracle/_ref/src) into oracle/_ref/,
// and used to pin the oracle and to time the reference CPU baseline. Nothing of
// the reference is copied into this file.
//
// Axis convention (test/test_tjhung.cc:17-23): the reference Integrator takes
// a (rows=y, cols=x) array; TjhungIntegrator's first index is its "x". The
// reference's parity test passes the same (rows, cols) array to both, so
// Tjhung "x" == Integrator "y" (rows). This driver follows that mapping: the
// caller passes a row-major (nrows, ncols) field, Tjhung's Nx := nrows and
// Ny := ncols, Tjhung dx := row spacing, dy := column spacing. Tjhung's
// Laplacian divides by dx*dy (test/tjhung_ambplus.h:138-140), so callers
// must use equal spacings. Noise is off (D = 0) in the parity entry points:
// the scheme draws from the global drand48 stream (test/tjhung_ambplus.h:80-100),
// which no test can pin. tjhung_ref_run_noisy runs it with that noise on, for
// timing the scheme as it ships.
#include "tjhung_ambplus.h"

#include <cstring>

namespace
{
    void load(TjhungIntegrator& t, const double* phi)
    {
        std::memcpy(t.phi.data(), phi, sizeof(double) * t.Nx * t.Ny);
    }

    void store(const Field& f, double* out)
    {
        if (out) std::memcpy(out, f.data(), sizeof(double) * f.rows() * f.cols());
    }
}

extern "C"
{
    // One call of TjhungIntegrator::calculate_dphi (test/tjhung_ambplus.h:192-251)
    // on `phi`; copies out dphi and the intermediate fields the reference's
    // parity test reads (test/test_tjhung.cc:24-40). Any output may be null.
    // A = -a = c (model a=-A, b=0, c=A), K = kappa.
    int tjhung_ref_dphi(int nrows, int ncols, double dt, double h,
                        double A, double K, double lambda, double zeta,
                        const double* phi, double* dphi, double* mueq, double* muact,
                        double* jxeq, double* jyeq, double* jxact, double* jyact)
    {
        if (nrows < 9 || ncols < 9) return 1;
        TjhungIntegrator t(nrows, ncols, dt, h, h, A, K, lambda, zeta, 0.0);
        load(t, phi);
        t.calculate_dphi();
        store(t.dphi, dphi);
        store(t.mueq, mueq);
        store(t.muact, muact);
        store(t.Jxeq, jxeq);
        store(t.Jyeq, jyeq);
        store(t.Jxact, jxact);
        store(t.Jyact, jyact);
        return 0;
    }

    // TjhungIntegrator::run(nsteps) (test/tjhung_ambplus.h:70-77) on `phi`, in place.
    int tjhung_ref_run(int nrows, int ncols, double dt, double h,
                       double A, double K, double lambda, double zeta,
                       double* phi, int nsteps)
    {
        if (nrows < 9 || ncols < 9 || nsteps < 0) return 1;
        TjhungIntegrator t(nrows, ncols, dt, h, h, A, K, lambda, zeta, 0.0);
        load(t, phi);
        t.run(nsteps);
        store(t.phi, phi);
        return 0;
    }

    // TjhungIntegrator::run(nsteps) with noise strength D (= the model's T), drand48 seeded
    // with `seed` after construction (the constructor seeds it from the clock,
    // test/tjhung_ambplus.h:64).
    int tjhung_ref_run_noisy(int nrows, int ncols, double dt, double h,
                             double A, double K, double lambda, double zeta, double D,
                             double* phi, int nsteps, long seed)
    {
        if (nrows < 9 || ncols < 9 || nsteps < 0 || D < 0) return 1;
        TjhungIntegrator t(nrows, ncols, dt, h, h, A, K, lambda, zeta, D);
        srand48(seed);
        load(t, phi);
        t.run(nsteps);
        store(t.phi, phi);
        return 0;
    }
}
