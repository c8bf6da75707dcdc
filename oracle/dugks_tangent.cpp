/*
 * Tangent-linear (forward-mode) model of the reference DUGKS step, from the
 * oracle's own restatement: dugks_oracle_impl.h compiled with REAL = a dual
 * number (value, derivative), so that every operation of the step carries its
 * exact directional derivative alongside the value.  Running it from (f, df)
 * gives S^n(f) and its tangent dS^n(f)[df] to rounding: the FP64 reference
 * gradient <grad J, d> against which the engine's hand-written adjoint is
 * checked (no finite-difference truncation).
 *
 * TEST INFRASTRUCTURE ONLY (built into oracle/libtangent.so, called by tests/).
 */
#include <cmath>
#include <cstdlib>
#include <omp.h>

#include "dugks_oracle.h"

/* D3Q19 velocity set in the reference's population order, src/lbm_d3q19.cu:12-15. */
static const int CIX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CIY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CIZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};

namespace {

// dual number: v + d*eps with eps^2 = 0
struct dual {
    double v, d;
    dual() : v(0), d(0) {}
    dual(double x) : v(x), d(0) {}  // constants carry no derivative
    dual(double x, double dx) : v(x), d(dx) {}
};
inline dual operator+(const dual &a, const dual &b) { return dual(a.v + b.v, a.d + b.d); }
inline dual operator-(const dual &a, const dual &b) { return dual(a.v - b.v, a.d - b.d); }
inline dual operator-(const dual &a) { return dual(-a.v, -a.d); }
inline dual operator*(const dual &a, const dual &b) { return dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline dual operator/(const dual &a, const dual &b)
{
    const double q = a.v / b.v;
    return dual(q, (a.d - q * b.d) / b.v);
}
inline dual &operator+=(dual &a, const dual &b) { return a = a + b; }
inline dual &operator-=(dual &a, const dual &b) { return a = a - b; }
inline dual &operator*=(dual &a, const dual &b) { return a = a * b; }
inline dual &operator/=(dual &a, const dual &b) { return a = a / b; }
inline dual fabs(const dual &a) { return a.v < 0 ? -a : a; }
inline dual sin(const dual &a) { return dual(std::sin(a.v), std::cos(a.v) * a.d); }
inline dual cos(const dual &a) { return dual(std::cos(a.v), -std::sin(a.v) * a.d); }
inline dual pow(const dual &a, int n) { return n == 2 ? a * a : dual(std::pow(a.v, n), n * std::pow(a.v, n - 1) * a.d); }

}  // namespace

#define ORACLE_TANGENT 1
#define REAL dual
#define SFX _tan
#include "dugks_oracle_impl.h"
#undef REAL
#undef SFX

/* nsteps steps from the ghosted AoS state f (value) and df (direction), in
 * place: f <- S^n(f), df <- dS^n(f)[df]. */
extern "C" int oracle_tangent_run(const oracle_cfg *c, double *f, double *df, int istep0, int nsteps, int nthreads)
{
    const size_t n = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2) * 19;
    dual *g = static_cast<dual *>(std::calloc(n, sizeof(dual)));
    if (!g) return -10;
    for (size_t q = 0; q < n; ++q) g[q] = dual(f[q], df[q]);
    const int rc = oracle_run_tan(c, g, istep0, nsteps, nthreads);
    for (size_t q = 0; q < n; ++q) {
        f[q] = g[q].v;
        df[q] = g[q].d;
    }
    std::free(g);
    return rc;
}
