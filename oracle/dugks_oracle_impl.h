/*
 * CPU restatement of the reference DUGKS time step, precision-generic body.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: it is compiled into
 * oracle/liboracle.so and called by tests/, by __graft_entry__.smoke() and by
 * the cpu_baseline / --impl reference legs of bench.py.  The product library
 * never links or calls it.
 *
 * It is included twice by dugks_oracle.c, once with REAL=double (suffix _f64)
 * and once with REAL=float (suffix _f32), mirroring the reference's
 * compile-time `real` switch (src/precision.h:4-8).  Literal types follow the
 * reference expression by expression, so that the float instance reproduces
 * the reference PREC4 build's promotions to double (e.g. `0.5*(a+b)`).
 *
 * Layout is the reference's: AoS with one ghost layer,
 *   f[((k*(ny+2)+j)*(nx+2)+i)*19+ip]            (src/dugks.cu:15-16)
 * Single rank, so lx=nx, ly=ny, lz=nz and the z halo exchange with itself is a
 * plane copy (src/parallel.cu:185-234 with zprev=znext=self).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

#define IDX(ip, i, j, k) ((((size_t)(k) * (size_t)(ny + 2) + (size_t)(j)) * (size_t)(nx + 2) + (size_t)(i)) * 19 + (size_t)(ip))
#define SIDX(i, j, k) (((size_t)(k) * (size_t)(ny + 2) + (size_t)(j)) * (size_t)(nx + 2) + (size_t)(i))

typedef struct {
    REAL visc, RT, hdt;
    REAL bw0, bw1, bw2;
    REAL fw0, fw1, fw2;
    REAL dx, dy, dz, dt;
    REAL xwidth, ywidth, zwidth;
    REAL ambient_fx, ambient_fy, ambient_fz;
    REAL tp[19];
} FN(coef_t);

/* Coefficient block, src/dugks.cu:97-125 (and the weights, 137-142). */
static void FN(make_coef)(const oracle_cfg *c, FN(coef_t) *q)
{
    const REAL RT = (REAL)(1. / 3.);              /* src/lbm_d3q19.cu:21 */
    const REAL visc = (REAL)c->visc;
    const REAL dt = (REAL)c->dt;
    const REAL tau = visc / RT;
    REAL hdt = dt / 2.;
    q->visc = visc;
    q->RT = RT;
    q->hdt = hdt;
    q->bw0 = (3. * tau * hdt) / (2. * tau + dt);
    q->bw1 = (2. * tau - hdt) / (2. * tau + dt);
    q->bw2 = 3. * hdt / (2. * tau + dt);
    q->fw0 = tau * hdt / (2. * tau + hdt);
    q->fw1 = 2. * tau / (2. * tau + hdt);
    q->fw2 = hdt / (2. * tau + hdt);
    q->dx = (REAL)c->dx;
    q->dy = (REAL)c->dy;
    q->dz = (REAL)c->dz;
    q->dt = dt;
    q->xwidth = (REAL)c->xwidth;
    q->ywidth = (REAL)c->ywidth;
    q->zwidth = (REAL)c->zwidth;
    q->ambient_fx = (REAL)c->Fx;
    q->ambient_fy = (REAL)c->Fy;
    q->ambient_fz = (REAL)c->Fz;
    {
        const REAL ww0 = 1.0 / 3.0, ww1 = 1.0 / 18.0, ww2 = 1.0 / 36.0; /* src/lbm_d3q19.cu:17-19 */
        int ip;
        q->tp[0] = ww0;
        for (ip = 1; ip <= 6; ip++) q->tp[ip] = ww1;
        for (ip = 7; ip < 19; ip++) q->tp[ip] = ww2;
    }
}

#ifndef ORACLE_TANGENT
int FN(oracle_coefficients)(const oracle_cfg *c, double *out13)
{
    FN(coef_t) q;
    FN(make_coef)(c, &q);
    out13[0] = q.visc; out13[1] = q.RT; out13[2] = q.hdt;
    out13[3] = q.bw0; out13[4] = q.bw1; out13[5] = q.bw2;
    out13[6] = q.fw0; out13[7] = q.fw1; out13[8] = q.fw2;
    out13[9] = q.dx; out13[10] = q.dy; out13[11] = q.dz; out13[12] = q.dt;
    return 0;
}
#endif /* ORACLE_TANGENT */

/* Equilibrium, src/dugks.cu:1201-1207 (feq_s) and 1183-1190 (inline in calc_fb1). */
static inline REAL FN(feq_s)(REAL r, REAL u, REAL v, REAL w, REAL tp, int cx, int cy, int cz)
{
    const REAL RT = 1. / 3.f;
    REAL eu = (cx * u + cy * v + cz * w) / RT;
    REAL uv = (u * u + v * v + w * w) / (RT);
    return tp * r * (1.0f + eu + 0.5f * (eu * eu - uv));
}

/* Host equilibrium used for initial conditions, src/dugks.cu:304-309. */
static inline REAL FN(feq_host)(int ip, const REAL *tp, REAL r, REAL u, REAL v, REAL w)
{
    const REAL RT = (REAL)(1. / 3.);
    REAL eu = (CIX[ip] * u + CIY[ip] * v + CIZ[ip] * w) / RT;
    REAL uv = (u * u + v * v + w * w) / RT;
    return tp[ip] * r * (1.0 + eu + 0.5 * (eu * eu - uv));
}

/* Initial condition f=feq(rho,u) on the whole ghosted box, src/dugks.cu:222-281.
 * kind 0: tg_eq, 1: channel.  */
int FN(oracle_init)(const oracle_cfg *c, int kind, REAL *f)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    FN(coef_t) q;
    const REAL pi = 3.141592653589793;   /* src/constants.cu:3-4 */
    const REAL pi2 = pi * 2;
    const REAL xoffset = 0, yoffset = 0, zoffset = 0;
    int i, j, k, ip;
    FN(make_coef)(c, &q);
    for (k = 0; k < nz + 2; k++) {
        REAL z = (k - 0.5) * q.dz + zoffset;
        for (j = 0; j < ny + 2; j++) {
            REAL y = (j - 0.5) * q.dy + yoffset;
            for (i = 0; i < nx + 2; i++) {
                REAL x = (i - 0.5) * q.dx + xoffset;
                REAL rho, ux, uy, uz;
                if (kind == 0) {
                    REAL vel_scale = 0.1;
                    rho = 1.0 + 1.0 * vel_scale * vel_scale / 16 * (cos(2 * pi2 / q.xwidth * x) + cos(2 * pi2 / q.ywidth * y)) * (cos(2 * pi2 / q.zwidth * z) + 2) / q.RT;
                    ux = vel_scale * sin(pi2 / q.xwidth * x) * cos(pi2 / q.ywidth * y) * cos(pi2 / q.zwidth * z);
                    uy = -vel_scale * cos(pi2 / q.xwidth * x) * sin(pi2 / q.ywidth * y) * cos(pi2 / q.zwidth * z);
                    uz = 0;
                } else if (kind == 1) {
                    rho = 1.0; ux = 0.0; uy = 0.0; uz = 0.1;
                } else {
                    return -1;
                }
                for (ip = 0; ip < 19; ip++) f[IDX(ip, i, j, k)] = FN(feq_host)(ip, q.tp, rho, ux, uy, uz);
            }
        }
    }
    return 0;
}

/* splitmix64 finaliser and the uniform value in [-1, 1) of (seed, cell,
 * component) that defines the seeded synthetic channel start: the 53 high bits
 * of splitmix64(seed*0xD1B54A32D192ED03 + 3*cell + component). */
static inline unsigned long long FN(smix)(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline double FN(usym)(unsigned long long seed, unsigned long long cell, int comp)
{
    const unsigned long long z = FN(smix)(seed * 0xD1B54A32D192ED03ull + cell * 3ull + (unsigned long long)comp);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

/* Initial states by case, interior cells of the ghosted box (ghosts untouched).
 *   kind 0  tg_eq (src/dugks.cu:222-238) with the amplitude par[0] in place of
 *           the reference's fixed 0.1, in the velocity and the density term;
 *   kind 1  channel (src/dugks.cu:239-255);
 *   kind 2  the seeded turbulent-channel start of the benchmark workloads (no
 *           counterpart in the reference, whose channel restarts from a DNS
 *           dump): along the streamwise axis a (the largest ambient force
 *           component) the laminar profile 6 ub eta (1 - eta), eta = x/xwidth,
 *           x the cell centre (c->xc on a stretched mesh); on every component
 *           amp*ub*usym(seed, cell, component); along a the near-wall streaks
 *           streak*ub*sin(2 pi m s) e exp(1 - e), e = y+/10 = min(x, xwidth - x)
 *           re_tau/(xwidth/2)/10, s = the spanwise coordinate / its width (y
 *           when a = z, else z).  par = {ub, re_tau, amp, streak, seed, m}.
 * f = feq(rho, u) with the host equilibrium (src/dugks.cu:304-309). */
int FN(oracle_init_case)(const oracle_cfg *c, int kind, const double *par, REAL *f)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    FN(coef_t) q;
    const double pi = 3.141592653589793, pi2 = 2 * pi;
    int i, j, k, ip;
    int sa = 2;
    FN(make_coef)(c, &q);
    (void)q;
    if (kind < 0 || kind > 2) return -1;
    const double Fa[3] = {c->Fx, c->Fy, c->Fz};
    if (fabs(Fa[0]) > fabs(Fa[sa])) sa = 0;
    if (fabs(Fa[1]) > fabs(Fa[sa])) sa = 1;
    for (k = 1; k <= nz; k++) {
        const double z = (k - 0.5) * c->dz;
        for (j = 1; j <= ny; j++) {
            const double y = (j - 0.5) * c->dy;
            for (i = 1; i <= nx; i++) {
                const double x = c->mesh == 1 ? c->xc[i] : (i - 0.5) * c->dx;
                double rho = 1, u[3] = {0, 0, 0};
                if (kind == 0) {
                    const double vs = par[0];
                    rho = 1.0 + 1.0 * vs * vs / 16 * (cos(2 * pi2 / c->xwidth * x) + cos(2 * pi2 / c->ywidth * y)) *
                                    (cos(2 * pi2 / c->zwidth * z) + 2) / (1. / 3.);
                    u[0] = vs * sin(pi2 / c->xwidth * x) * cos(pi2 / c->ywidth * y) * cos(pi2 / c->zwidth * z);
                    u[1] = -vs * cos(pi2 / c->xwidth * x) * sin(pi2 / c->ywidth * y) * cos(pi2 / c->zwidth * z);
                } else if (kind == 1) {
                    u[2] = 0.1;
                } else {
                    const double ub = par[0], re_tau = par[1], amp = par[2], streak = par[3];
                    const unsigned long long seed = (unsigned long long)par[4];
                    const int m = (int)par[5];
                    const unsigned long long cell = ((unsigned long long)(k - 1) * ny + (j - 1)) * nx + (i - 1);
                    const double eta = x / c->xwidth, H = 0.5 * c->xwidth;
                    const double wall = x < c->xwidth - x ? x : c->xwidth - x;
                    const double e = wall * (re_tau / H) / 10.0;
                    const double s = sa == 2 ? y / c->ywidth : z / c->zwidth;
                    int a;
                    u[sa] = 6.0 * ub * eta * (1 - eta);
                    for (a = 0; a < 3; a++) u[a] += amp * ub * FN(usym)(seed, cell, a);
                    u[sa] += streak * ub * sin(pi2 * m * s) * e * exp(1 - e);
                }
                for (ip = 0; ip < 19; ip++) {
                    const double RT = 1. / 3.;
                    const double tp = ip == 0 ? 1.0 / 3.0 : (ip <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
                    const double eu = (CIX[ip] * u[0] + CIY[ip] * u[1] + CIZ[ip] * u[2]) / RT;
                    const double uv = (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / RT;
                    f[IDX(ip, i, j, k)] = (REAL)(tp * rho * (1.0 + eu + 0.5 * (eu * eu - uv)));
                }
            }
        }
    }
    return 0;
}

/* Per-cell body force, src/dugks.cu:1066-1126 (calc_force / calc_perturb_force).
 * Writes interior cells of the three ghosted force arrays. */
static void FN(force_field)(const oracle_cfg *c, const FN(coef_t) *q, int step, REAL *fxa, REAL *fya, REAL *fza)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    int i, j, k;
    const REAL pi = 3.141592653589793;
    const REAL pi2 = pi * 2;
    for (k = 1; k <= nz; k++)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                size_t s = SIDX(i, j, k);
                if (c->perturb) {
                    const REAL beta = 3, Tpd = 2000, gamma = 2, Re_tau = 180;
                    const REAL zoffset = 0;
                    const REAL ustar = 2 * Re_tau * q->visc / q->xwidth;
                    const REAL FF = 2 * pow(ustar, 2) / q->xwidth;
                    REAL A0 = 5 * 40.0 / nx * beta * sin(pi2 * step * q->dt / Tpd);
                    if (3 < i && i < nx / 4 + 2) {
                        REAL xx = pi2 * (i - 3) * q->dx / (q->xwidth / 4.);
                        REAL yy = pi2 * (j - 0.5) * q->dy / q->ywidth;
                        REAL zz = pi2 * ((k - 0.5) * q->dz + zoffset) / q->zwidth;
                        fxa[s] = 0.5 * FF * A0 * q->xwidth / 4 * (1 - cos(xx)) * cos(beta * yy) * cos(gamma * zz);
                        fya[s] = 0.5 * FF * A0 * q->ywidth / gamma * sin(xx) * cos(beta * yy) * sin(gamma * zz);
                        fza[s] = FF * (1 - A0 * q->zwidth / beta * sin(xx) * sin(beta * yy) * cos(gamma * zz));
                        continue;
                    }
                }
                fxa[s] = q->ambient_fx;
                fya[s] = q->ambient_fy;
                fza[s] = q->ambient_fz;
            }
}

/* Stage (a): f-bar-plus from f-tilde, src/dugks.cu:1131-1196 (calc_fb1);
 * the stretched-mesh kernel src/fortran/channel/src/dugks.cuf:337-363 is the
 * same arithmetic with the ambient force. */
static void FN(stage_fbar)(const oracle_cfg *c, const FN(coef_t) *q, const REAL *f, REAL *fb,
                           const REAL *fxa, const REAL *fya, const REAL *fza)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    int k;
#pragma omp parallel for schedule(static)
    for (k = 1; k <= nz; k++) {
        int i, j, ip;
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                const size_t s = SIDX(i, j, k);
                REAL ff[19], feqa[19];
                REAL rr, uu, vv, ww;
                const REAL RT = 1. / 3.f;
                rr = uu = vv = ww = 0;
                for (ip = 0; ip < 19; ip++) {
                    ff[ip] = f[IDX(ip, i, j, k)];
                    rr += ff[ip];
                    uu += CIX[ip] * ff[ip];
                    vv += CIY[ip] * ff[ip];
                    ww += CIZ[ip] * ff[ip];
                }
                uu /= rr;
                vv /= rr;
                ww /= rr;
                uu += q->hdt * fxa[s];
                vv += q->hdt * fya[s];
                ww += q->hdt * fza[s];
                for (ip = 0; ip < 19; ip++) {
                    REAL eu = (CIX[ip] * uu + CIY[ip] * vv + CIZ[ip] * ww) / RT;
                    REAL uv = (uu * uu + vv * vv + ww * ww) / (RT);
                    feqa[ip] = q->tp[ip] * rr * (1.0f + eu + 0.5f * (eu * eu - uv));
                }
                for (ip = 0; ip < 19; ip++) {
                    REAL temp = ((CIX[ip] - uu) * fxa[s] + (CIY[ip] - vv) * fya[s] + (CIZ[ip] - ww) * fza[s]) / RT;
                    fb[IDX(ip, i, j, k)] = q->bw1 * ff[ip] + (q->bw2 + q->bw0 * temp) * feqa[ip];
                }
            }
    }
}

/* Ghost fill of f-bar-plus in the reference's order: x (wall extrapolation or
 * periodic copy, over all ghosted j,k), then periodic y (over all ghosted i,k),
 * then periodic z (whole planes).
 *   src/dugks.cu:1212-1229 extend_fb_x, 1234-1251 extend_fb_x_wall,
 *   1256-1273 extend_fb_y, src/parallel.cu:185-234 exchange (self).
 * Stretched mesh: src/fortran/channel/src/dugks.cuf:365-374 (qqq weights),
 * src/fortran/channel/src/main.cuf:71-74 (periodic y, z). */
static void FN(stage_ghost)(const oracle_cfg *c, REAL *fb)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    int i, j, k, ip;
    REAL q0 = 2, q1 = 2;
    if (c->mesh == 1) {
        const double *xc = c->xc;
        q0 = (REAL)((xc[2] - xc[0]) / (xc[2] - xc[1]));
        q1 = (REAL)((xc[nx + 1] - xc[nx - 1]) / (xc[nx] - xc[nx - 1]));
    }
    for (k = 0; k < nz + 2; k++)
        for (j = 0; j < ny + 2; j++)
            for (ip = 0; ip < 19; ip++) {
                if (c->periodic_x) {
                    fb[IDX(ip, 0, j, k)] = fb[IDX(ip, nx, j, k)];
                    fb[IDX(ip, nx + 1, j, k)] = fb[IDX(ip, 1, j, k)];
                } else if (c->mesh == 1) {
                    fb[IDX(ip, 0, j, k)] = q0 * fb[IDX(ip, 1, j, k)] + (1. - q0) * fb[IDX(ip, 2, j, k)];
                    fb[IDX(ip, nx + 1, j, k)] = q1 * fb[IDX(ip, nx, j, k)] + (1. - q1) * fb[IDX(ip, nx - 1, j, k)];
                } else {
                    fb[IDX(ip, 0, j, k)] = 2 * fb[IDX(ip, 1, j, k)] - fb[IDX(ip, 2, j, k)];
                    fb[IDX(ip, nx + 1, j, k)] = 2 * fb[IDX(ip, nx, j, k)] - fb[IDX(ip, nx - 1, j, k)];
                }
            }
    for (k = 0; k < nz + 2; k++)
        for (i = 0; i < nx + 2; i++)
            for (ip = 0; ip < 19; ip++) {
                fb[IDX(ip, i, 0, k)] = fb[IDX(ip, i, ny, k)];
                fb[IDX(ip, i, ny + 1, k)] = fb[IDX(ip, i, 1, k)];
            }
    for (j = 0; j < ny + 2; j++)
        for (i = 0; i < nx + 2; i++)
            for (ip = 0; ip < 19; ip++) {
                fb[IDX(ip, i, j, 0)] = fb[IDX(ip, i, j, nz)];
                fb[IDX(ip, i, j, nz + 1)] = fb[IDX(ip, i, j, 1)];
            }
}

/* src/dugks.cu:964-978 */
static inline REAL FN(trilinear)(REAL a, REAL b, REAL c, REAL d, REAL e, REAL f, REAL g, REAL h, REAL mx, REAL my, REAL mz)
{
    REAL x00, x01, x10, x11, y00, y11;
    x00 = (1 - mx) * a + mx * b;
    x01 = (1 - mx) * c + mx * d;
    x10 = (1 - mx) * e + mx * f;
    x11 = (1 - mx) * g + mx * h;
    y00 = (1 - my) * x00 + my * x01;
    y11 = (1 - my) * x10 + my * x11;
    return (1 - mz) * y00 + mz * y11;
}

/* Face moments with the half-step ambient shift, src/dugks.cu:675-709 (f2ruvwh). */
static inline void FN(f2ruvwh)(REAL *r, REAL *u, REAL *v, REAL *w, const REAL *ft, REAL *force1, const FN(coef_t) *q)
{
    int ip;
    *r = *u = *v = *w = 0;
    for (ip = 0; ip < 19; ip++) {
        *r += ft[ip];
        *u += CIX[ip] * ft[ip];
        *v += CIY[ip] * ft[ip];
        *w += CIZ[ip] * ft[ip];
    }
    *u /= *r;
    *v /= *r;
    *w /= *r;
    *u += 0.5 * q->hdt * q->ambient_fx;
    *v += 0.5 * q->hdt * q->ambient_fy;
    *w += 0.5 * q->hdt * q->ambient_fz;
    for (ip = 0; ip < 19; ip++)
        force1[ip] = (q->ambient_fx * (CIX[ip] - *u) + q->ambient_fy * (CIY[ip] - *v) + q->ambient_fz * (CIZ[ip] - *w)) / q->RT;
}

/* Fortran channel face moments, src/fortran/channel/src/dugks.cuf:842-876. */
static inline void FN(macro_plain)(const REAL *ft, REAL *r, REAL *u, REAL *v, REAL *w)
{
    int ip;
    *u = 0; *v = 0; *w = 0; *r = 0;
    for (ip = 0; ip < 19; ip++) {
        *r = *r + ft[ip];
        *u = *u + CIX[ip] * ft[ip];
        *v = *v + CIY[ip] * ft[ip];
        *w = *w + CIZ[ip] * ft[ip];
    }
    *u = *u / *r;
    *v = *v / *r;
    *w = *w / *r;
}

static inline void FN(feq_plain)(REAL *feq, const REAL *tp, REAL r, REAL u, REAL v, REAL w)
{
    const REAL RT = (REAL)(1. / 3.);
    int ip;
    for (ip = 0; ip < 19; ip++) {
        REAL eu = (CIX[ip] * u + CIY[ip] * v + CIZ[ip] * w) / RT;
        REAL uv = (u * u + v * v + w * w) / RT;
        feq[ip] = tp[ip] * r * (1 + eu + 0.5 * (eu * eu - uv));
    }
}

/* Bounce-back at the x walls, src/dugks.cu:807-823. */
static inline void FN(bounce_back)(const oracle_cfg *c, int i, REAL ft[6][19])
{
    if (c->periodic_x) return;
    if (i == 1) {
        ft[0][1] = ft[0][2];
        ft[0][7] = ft[0][10];
        ft[0][9] = ft[0][8];
        ft[0][11] = ft[0][14];
        ft[0][13] = ft[0][12];
    }
    if (i == c->nx) {
        ft[1][2] = ft[1][1];
        ft[1][10] = ft[1][7];
        ft[1][8] = ft[1][9];
        ft[1][14] = ft[1][11];
        ft[1][12] = ft[1][13];
    }
}

/* Stage (d) and (e) for one cell: face equilibrium with the ambient force and
 * the finite-volume update written in place, src/dugks.cu:908-956.
 * face_force==1 restates the Fortran channel treatment instead
 * (src/fortran/channel/src/dugks.cuf:765-839): no force on x and z faces,
 * force on y faces only, feq taken before the half-step shift. */
static void FN(face_fluxes_and_update)(const oracle_cfg *c, const FN(coef_t) *q, REAL *f, const REAL *fb,
                                       int i, int j, int k, REAL ft[6][19])
{
    const int nx = c->nx, ny = c->ny;
    REAL r, u, v, w;
    REAL force1[19], feq[19];
    int s, ip;
    if (c->face_force == 0) {
        for (s = 0; s < 6; s++) {
            FN(f2ruvwh)(&r, &u, &v, &w, ft[s], force1, q);
            for (ip = 0; ip < 19; ip++)
                ft[s][ip] = q->fw1 * ft[s][ip] + (q->fw2 + q->fw0 * force1[ip]) * FN(feq_s)(r, u, v, w, q->tp[ip], CIX[ip], CIY[ip], CIZ[ip]);
        }
    } else {
        const REAL RT = (REAL)(1. / 3.);
        const REAL F1 = q->ambient_fx, F2 = q->ambient_fy, F3 = q->ambient_fz;
        static const int plain_faces[4] = {1, 0, 5, 4};
        int n;
        for (n = 0; n < 4; n++) {
            s = plain_faces[n];
            FN(macro_plain)(ft[s], &r, &u, &v, &w);
            FN(feq_plain)(feq, q->tp, r, u, v, w);
            for (ip = 0; ip < 19; ip++) ft[s][ip] = q->fw1 * ft[s][ip] + q->fw2 * feq[ip];
        }
        FN(macro_plain)(ft[3], &r, &u, &v, &w);
        FN(feq_plain)(feq, q->tp, r, u, v, w);
        v = v + 0.5 * q->hdt * F2;
        for (ip = 0; ip < 19; ip++)
            force1[ip] = (1. / RT) * (F1 * (CIX[ip] - u) + F2 * (CIY[ip] - v) + F3 * (CIZ[ip] - w));
        for (ip = 0; ip < 19; ip++) ft[3][ip] = q->fw1 * ft[3][ip] + (q->fw2 + q->fw0 * force1[ip]) * feq[ip];
        FN(macro_plain)(ft[2], &r, &u, &v, &w);
        FN(feq_plain)(feq, q->tp, r, u, v, w);
        for (ip = 0; ip < 19; ip++)
            force1[ip] = (1. / RT) * (F1 * (CIX[ip] - u) + F2 * (CIY[ip] - v) + F3 * (CIZ[ip] - w));
        for (ip = 0; ip < 19; ip++) ft[2][ip] = q->fw1 * ft[2][ip] + (q->fw2 + q->fw0 * force1[ip]) * feq[ip];
    }
    {
        REAL cx = (q->dt) / (q->dx);
        const REAL cy = (q->dt) / (q->dy);
        const REAL cz = (q->dt) / (q->dz);
        if (c->mesh == 1) cx = q->dt / (REAL)c->dxx[i];
        for (ip = 0; ip < 19; ip++) {
            u = ft[1][ip] - ft[0][ip];
            v = ft[3][ip] - ft[2][ip];
            w = ft[5][ip] - ft[4][ip];
            r = fb[IDX(ip, i, j, k)] * 4. / 3. - f[IDX(ip, i, j, k)] * 1. / 3.;
            f[IDX(ip, i, j, k)] = r - cx * CIX[ip] * u - cy * CIY[ip] * v - cz * CIZ[ip] * w;
        }
    }
}

/* Stages (c)(d)(e) for one cell with trilinear reconstruction,
 * src/dugks.cu:715-959 (calc_fx_tri).  With mesh==1 the x fractions and the
 * update width follow src/fortran/channel/src/dugks.cuf:541,546,595,658,833. */
static void FN(cell_tri)(const oracle_cfg *c, const FN(coef_t) *q, REAL *f, const REAL *fb, int i, int j, int k)
{
    const int nx = c->nx, ny = c->ny;
    const REAL hdt = q->hdt, dx = q->dx, dy = q->dy, dz = q->dz;
    REAL ft[6][19];
    int ip, ii, jj, kk;
    REAL mx0, my0, mz0, mx1, my1, mz1;
    const double *dxx = c->dxx;
#define FBV(ip_, a_, b_, c_) fb[IDX(ip_, a_, b_, c_)]
    ft[1][0] = 0.5 * (FBV(0, i, j, k) + FBV(0, i + 1, j, k));
    ft[0][0] = 0.5 * (FBV(0, i, j, k) + FBV(0, i - 1, j, k));
    ft[3][0] = 0.5 * (FBV(0, i, j, k) + FBV(0, i, j + 1, k));
    ft[2][0] = 0.5 * (FBV(0, i, j, k) + FBV(0, i, j - 1, k));
    ft[5][0] = 0.5 * (FBV(0, i, j, k) + FBV(0, i, j, k + 1));
    ft[4][0] = 0.5 * (FBV(0, i, j, k) + FBV(0, i, j, k - 1));

    for (ip = 1; ip < 19; ip++) {
        if (c->mesh == 1) {
            REAL di = (REAL)dxx[i], dip = (REAL)dxx[i + 1], dim = (REAL)dxx[i - 1];
            mx1 = (di / 2 - hdt * CIX[ip]) / (0.5 * di + 0.5 * dip);
            mx0 = (di / 2 + hdt * CIX[ip]) / (0.5 * di + 0.5 * dim);
        } else {
            mx1 = (dx / 2. - hdt * CIX[ip]) / dx;
            mx0 = 1 - mx1;
        }
        my1 = (-hdt * CIY[ip]) / dy;
        mz1 = (-hdt * CIZ[ip]) / dz;
        my0 = my1;
        mz0 = mz1;
        ii = 1; jj = -CIY[ip]; kk = -CIZ[ip];
        ft[1][ip] = FN(trilinear)(FBV(ip, i, j, k), FBV(ip, i + ii, j, k), FBV(ip, i, j + jj, k), FBV(ip, i + ii, j + jj, k),
                                  FBV(ip, i, j, k + kk), FBV(ip, i + ii, j, k + kk), FBV(ip, i, j + jj, k + kk), FBV(ip, i + ii, j + jj, k + kk),
                                  (mx1), fabs(my1), fabs(mz1));
        ii = -1;
        ft[0][ip] = FN(trilinear)(FBV(ip, i, j, k), FBV(ip, i + ii, j, k), FBV(ip, i, j + jj, k), FBV(ip, i + ii, j + jj, k),
                                  FBV(ip, i, j, k + kk), FBV(ip, i + ii, j, k + kk), FBV(ip, i, j + jj, k + kk), FBV(ip, i + ii, j + jj, k + kk),
                                  (mx0), fabs(my0), fabs(mz0));
    }

    if (c->face_force == 0) FN(bounce_back)(c, i, ft);

    for (ip = 1; ip < 19; ip++) {
        if (c->mesh == 1)
            mx1 = (-hdt * CIX[ip]) / (0.5 * (REAL)dxx[i] + 0.5 * (REAL)dxx[i - CIX[ip]]);
        else
            mx1 = (-hdt * CIX[ip]) / dx;
        my1 = (dy / 2. - hdt * CIY[ip]) / dy;
        mz1 = (-hdt * CIZ[ip]) / dz;
        mx0 = mx1;
        my0 = 1 - my1;
        mz0 = mz1;
        ii = -CIX[ip]; jj = 1; kk = -CIZ[ip];
        ft[3][ip] = FN(trilinear)(FBV(ip, i, j, k), FBV(ip, i + ii, j, k), FBV(ip, i, j + jj, k), FBV(ip, i + ii, j + jj, k),
                                  FBV(ip, i, j, k + kk), FBV(ip, i + ii, j, k + kk), FBV(ip, i, j + jj, k + kk), FBV(ip, i + ii, j + jj, k + kk),
                                  fabs(mx1), (my1), fabs(mz1));
        jj = -1;
        ft[2][ip] = FN(trilinear)(FBV(ip, i, j, k), FBV(ip, i + ii, j, k), FBV(ip, i, j + jj, k), FBV(ip, i + ii, j + jj, k),
                                  FBV(ip, i, j, k + kk), FBV(ip, i + ii, j, k + kk), FBV(ip, i, j + jj, k + kk), FBV(ip, i + ii, j + jj, k + kk),
                                  fabs(mx0), (my0), fabs(mz0));
    }

    for (ip = 1; ip < 19; ip++) {
        if (c->mesh == 1)
            mx1 = (-hdt * CIX[ip]) / (0.5 * (REAL)dxx[i] + 0.5 * (REAL)dxx[i - CIX[ip]]);
        else
            mx1 = (-hdt * CIX[ip]) / dx;
        my1 = (-hdt * CIY[ip]) / dy;
        mz1 = (dz / 2. - hdt * CIZ[ip]) / dz;
        mx0 = mx1;
        my0 = my1;
        mz0 = 1 - mz1;
        ii = -CIX[ip]; jj = -CIY[ip]; kk = 1;
        ft[5][ip] = FN(trilinear)(FBV(ip, i, j, k), FBV(ip, i + ii, j, k), FBV(ip, i, j + jj, k), FBV(ip, i + ii, j + jj, k),
                                  FBV(ip, i, j, k + kk), FBV(ip, i + ii, j, k + kk), FBV(ip, i, j + jj, k + kk), FBV(ip, i + ii, j + jj, k + kk),
                                  fabs(mx1), fabs(my1), (mz1));
        kk = -1;
        ft[4][ip] = FN(trilinear)(FBV(ip, i, j, k), FBV(ip, i + ii, j, k), FBV(ip, i, j + jj, k), FBV(ip, i + ii, j + jj, k),
                                  FBV(ip, i, j, k + kk), FBV(ip, i + ii, j, k + kk), FBV(ip, i, j + jj, k + kk), FBV(ip, i + ii, j + jj, k + kk),
                                  fabs(mx0), fabs(my0), (mz0));
    }

    if (c->face_force == 1) FN(bounce_back)(c, i, ft);

    FN(face_fluxes_and_update)(c, q, f, fb, i, j, k, ft);
#undef FBV
}

/* The gradient reconstruction on a stretched x mesh (no counterpart in the
 * reference, whose stretched-mesh channel reconstructs trilinearly; this is
 * calc_fx's rule on non-uniform centres): an x face between cells a and a+1
 * takes the cell values interpolated linearly to the face, weight
 * lam = (dxx_a/2)/(xc_{a+1} - xc_a) on cell a+1, and the normal derivative
 * (f_{a+1} - f_a)/(xc_{a+1} - xc_a); the x derivative on y and z faces is the
 * three-point central difference of the face-averaged values on the centres
 * xc_{i-1}, xc_i, xc_{i+1}.  On a uniform mesh both reduce to calc_fx. */
static void FN(cell_grad_stretched)(const oracle_cfg *c, const FN(coef_t) *q, REAL *f, const REAL *fb, int i, int j,
                                    int k)
{
    const int nx = c->nx, ny = c->ny;
    const REAL hdt = q->hdt, dy = q->dy, dz = q->dz;
    const double *xc = c->xc, *dxx = c->dxx;
    REAL ft[6][19];
    int ip, s;
    const double hm = xc[i] - xc[i - 1], hp = xc[i + 1] - xc[i];
    const REAL wm = (REAL)(-hp / (hm * (hp + hm))), w0 = (REAL)((hp - hm) / (hp * hm)), wp = (REAL)(hm / (hp * (hp + hm)));
#define FBV(ip_, a_, b_, c_) fb[IDX(ip_, a_, b_, c_)]
    for (s = 0; s < 2; s++) {               /* x faces: s = 1 between i and i+1, s = 0 between i-1 and i */
        const int a = s == 1 ? i : i - 1, b = a + 1;
        const REAL lam = (REAL)(0.5 * dxx[a] / (xc[b] - xc[a])), id = (REAL)(1.0 / (xc[b] - xc[a]));
        for (ip = 0; ip < 19; ip++) {
            REAL temp = FBV(ip, a, j, k) + lam * (FBV(ip, b, j, k) - FBV(ip, a, j, k));
            REAL gradx = (FBV(ip, b, j, k) - FBV(ip, a, j, k)) * id;
            REAL aa = FBV(ip, a, j + 1, k) + lam * (FBV(ip, b, j + 1, k) - FBV(ip, a, j + 1, k));
            REAL bb = FBV(ip, a, j - 1, k) + lam * (FBV(ip, b, j - 1, k) - FBV(ip, a, j - 1, k));
            REAL grady = (aa - bb) / (2 * dy);
            aa = FBV(ip, a, j, k + 1) + lam * (FBV(ip, b, j, k + 1) - FBV(ip, a, j, k + 1));
            bb = FBV(ip, a, j, k - 1) + lam * (FBV(ip, b, j, k - 1) - FBV(ip, a, j, k - 1));
            REAL gradz = (aa - bb) / (2 * dz);
            ft[s][ip] = ip == 0 ? temp : temp - hdt * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
        }
    }
    FN(bounce_back)(c, i, ft);
    for (s = 2; s < 6; s++) {               /* y faces (2: j-1|j, 3: j|j+1), z faces (4: k-1|k, 5: k|k+1) */
        const int y = s < 4, up = s & 1;
        const int j0 = y ? (up ? j : j - 1) : j, k0 = y ? k : (up ? k : k - 1);
        const int j1 = y ? j0 + 1 : j0, k1 = y ? k0 : k0 + 1;
        for (ip = 0; ip < 19; ip++) {
            REAL temp = 0.5 * (FBV(ip, i, j1, k1) + FBV(ip, i, j0, k0));
            REAL gradx = wm * (0.5 * (FBV(ip, i - 1, j0, k0) + FBV(ip, i - 1, j1, k1))) + w0 * temp +
                         wp * (0.5 * (FBV(ip, i + 1, j0, k0) + FBV(ip, i + 1, j1, k1)));
            REAL gn = y ? (FBV(ip, i, j1, k1) - FBV(ip, i, j0, k0)) / dy : (FBV(ip, i, j1, k1) - FBV(ip, i, j0, k0)) / dz;
            REAL gt;   /* transverse: z on a y face, y on a z face, central over 2 cells */
            if (y) {
                REAL aa = 0.5 * (FBV(ip, i, j0, k + 1) + FBV(ip, i, j1, k + 1));
                REAL bb = 0.5 * (FBV(ip, i, j0, k - 1) + FBV(ip, i, j1, k - 1));
                gt = (aa - bb) / (2 * dz);
            } else {
                REAL aa = 0.5 * (FBV(ip, i, j + 1, k0) + FBV(ip, i, j + 1, k1));
                REAL bb = 0.5 * (FBV(ip, i, j - 1, k0) + FBV(ip, i, j - 1, k1));
                gt = (aa - bb) / (2 * dy);
            }
            {
                const REAL grady = y ? gn : gt, gradz = y ? gt : gn;
                ft[s][ip] = temp - hdt * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
            }
        }
    }
    FN(face_fluxes_and_update)(c, q, f, fb, i, j, k, ft);
#undef FBV
}

/* Stages (b)(c) with the central-difference ("gradient") reconstruction,
 * src/dugks.cu:421-584 (calc_fx), followed by the shared (d)(e). */
static void FN(cell_grad)(const oracle_cfg *c, const FN(coef_t) *q, REAL *f, const REAL *fb, int i, int j, int k)
{
    const int nx = c->nx, ny = c->ny;
    const REAL hdt = q->hdt, dx = q->dx, dy = q->dy, dz = q->dz;
    REAL ft[6][19];
    int ip;
    REAL temp, aa, bb, gradx, grady, gradz;
    if (c->mesh == 1) {
        FN(cell_grad_stretched)(c, q, f, fb, i, j, k);
        return;
    }
#define FBV(ip_, a_, b_, c_) fb[IDX(ip_, a_, b_, c_)]
    for (ip = 0; ip < 19; ip++) {
        temp = 0.5 * (FBV(ip, i + 1, j, k) + FBV(ip, i, j, k));
        gradx = (FBV(ip, i + 1, j, k) - FBV(ip, i, j, k)) / (dx);
        aa = 0.5 * (FBV(ip, i, j + 1, k) + FBV(ip, i + 1, j + 1, k));
        bb = 0.5 * (FBV(ip, i, j - 1, k) + FBV(ip, i + 1, j - 1, k));
        grady = (aa - bb) / (2 * dy);
        aa = 0.5 * (FBV(ip, i, j, k + 1) + FBV(ip, i + 1, j, k + 1));
        bb = 0.5 * (FBV(ip, i, j, k - 1) + FBV(ip, i + 1, j, k - 1));
        gradz = (aa - bb) / (2 * dz);
        ft[1][ip] = temp - (hdt) * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
    }
    for (ip = 0; ip < 19; ip++) {
        temp = 0.5 * (FBV(ip, i, j, k) + FBV(ip, i - 1, j, k));
        gradx = (FBV(ip, i, j, k) - FBV(ip, i - 1, j, k)) / (dx);
        aa = 0.5 * (FBV(ip, i, j + 1, k) + FBV(ip, i - 1, j + 1, k));
        bb = 0.5 * (FBV(ip, i, j - 1, k) + FBV(ip, i - 1, j - 1, k));
        grady = (aa - bb) / (2 * dy);
        aa = 0.5 * (FBV(ip, i, j, k + 1) + FBV(ip, i - 1, j, k + 1));
        bb = 0.5 * (FBV(ip, i, j, k - 1) + FBV(ip, i - 1, j, k - 1));
        gradz = (aa - bb) / (2 * dz);
        ft[0][ip] = temp - (hdt) * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
    }
    FN(bounce_back)(c, i, ft);
    for (ip = 0; ip < 19; ip++) {
        temp = 0.5 * (FBV(ip, i, j + 1, k) + FBV(ip, i, j, k));
        aa = 0.5 * (FBV(ip, i + 1, j, k) + FBV(ip, i + 1, j + 1, k));
        bb = 0.5 * (FBV(ip, i - 1, j, k) + FBV(ip, i - 1, j + 1, k));
        gradx = (aa - bb) / (2 * dx);
        grady = (FBV(ip, i, j + 1, k) - FBV(ip, i, j, k)) / (dy);
        aa = 0.5 * (FBV(ip, i, j, k + 1) + FBV(ip, i, j + 1, k + 1));
        bb = 0.5 * (FBV(ip, i, j, k - 1) + FBV(ip, i, j + 1, k - 1));
        gradz = (aa - bb) / (2 * dz);
        ft[3][ip] = temp - (hdt) * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
    }
    for (ip = 0; ip < 19; ip++) {
        temp = 0.5 * (FBV(ip, i, j, k) + FBV(ip, i, j - 1, k));
        aa = 0.5 * (FBV(ip, i + 1, j - 1, k) + FBV(ip, i + 1, j, k));
        bb = 0.5 * (FBV(ip, i - 1, j - 1, k) + FBV(ip, i - 1, j, k));
        gradx = (aa - bb) / (2 * dx);
        grady = (FBV(ip, i, j, k) - FBV(ip, i, j - 1, k)) / (dy);
        aa = 0.5 * (FBV(ip, i, j - 1, k + 1) + FBV(ip, i, j, k + 1));
        bb = 0.5 * (FBV(ip, i, j - 1, k - 1) + FBV(ip, i, j, k - 1));
        gradz = (aa - bb) / (2 * dz);
        ft[2][ip] = temp - (hdt) * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
    }
    for (ip = 0; ip < 19; ip++) {
        temp = 0.5 * (FBV(ip, i, j, k + 1) + FBV(ip, i, j, k));
        aa = 0.5 * (FBV(ip, i + 1, j, k) + FBV(ip, i + 1, j, k + 1));
        bb = 0.5 * (FBV(ip, i - 1, j, k) + FBV(ip, i - 1, j, k + 1));
        gradx = (aa - bb) / (2 * dx);
        aa = 0.5 * (FBV(ip, i, j + 1, k) + FBV(ip, i, j + 1, k + 1));
        bb = 0.5 * (FBV(ip, i, j - 1, k) + FBV(ip, i, j - 1, k + 1));
        grady = (aa - bb) / (2 * dy);
        gradz = (FBV(ip, i, j, k + 1) - FBV(ip, i, j, k)) / (dz);
        ft[5][ip] = temp - (hdt) * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
    }
    for (ip = 0; ip < 19; ip++) {
        temp = 0.5 * (FBV(ip, i, j, k) + FBV(ip, i, j, k - 1));
        aa = 0.5 * (FBV(ip, i + 1, j, k) + FBV(ip, i + 1, j, k - 1));
        bb = 0.5 * (FBV(ip, i - 1, j, k) + FBV(ip, i - 1, j, k - 1));
        gradx = (aa - bb) / (2 * dx);
        aa = 0.5 * (FBV(ip, i, j + 1, k) + FBV(ip, i, j + 1, k - 1));
        bb = 0.5 * (FBV(ip, i, j - 1, k) + FBV(ip, i, j - 1, k - 1));
        grady = (aa - bb) / (2 * dy);
        gradz = (FBV(ip, i, j, k) - FBV(ip, i, j, k - 1)) / (dz);
        ft[4][ip] = temp - (hdt) * (CIX[ip] * gradx + CIY[ip] * grady + CIZ[ip] * gradz);
    }
    FN(face_fluxes_and_update)(c, q, f, fb, i, j, k, ft);
#undef FBV
}

/* Stages (c)(d)(e) over the interior, written in place into f (the
 * reference's calc_fx_tri / calc_fx read f only at their own cell). */
static void FN(stage_flux)(const oracle_cfg *c, const FN(coef_t) *q, REAL *f, const REAL *fb)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    int k;
#pragma omp parallel for schedule(static)
    for (k = 1; k <= nz; k++) {
        int i, j;
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                if (c->recon == 1) FN(cell_grad)(c, q, f, fb, i, j, k);
                else FN(cell_tri)(c, q, f, fb, i, j, k);
            }
    }
}

static int FN(check_cfg)(const oracle_cfg *c)
{
    if (c->nx < 3 || c->ny < 1 || c->nz < 1) return -1;
    if (c->mesh == 1 && (c->xc == 0 || c->dxx == 0)) return -2;
    return 0;
}

/* Stage (a) plus the ghost fill: fb is the ghosted f-bar-plus after
 * calc_fb1 and the x / y / z extensions of step `step`. */
int FN(oracle_fbar)(const oracle_cfg *c, const REAL *f, REAL *fb, int step, int nthreads)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    size_t ncell = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    FN(coef_t) q;
    REAL *fxa, *fya, *fza;
    int rc = FN(check_cfg)(c);
    if (rc) return rc;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    FN(make_coef)(c, &q);
    fxa = (REAL *)calloc(ncell, sizeof(REAL));
    fya = (REAL *)calloc(ncell, sizeof(REAL));
    fza = (REAL *)calloc(ncell, sizeof(REAL));
    if (!fxa || !fya || !fza) { free(fxa); free(fya); free(fza); return -10; }
    FN(force_field)(c, &q, step, fxa, fya, fza);
    FN(stage_fbar)(c, &q, f, fb, fxa, fya, fza);
    FN(stage_ghost)(c, fb);
    free(fxa); free(fya); free(fza);
    return 0;
}

/* nsteps DUGKS steps istep0 .. istep0+nsteps-1 on the ghosted AoS state f,
 * in the order of src/dugks.cu:322-391. */
int FN(oracle_run)(const oracle_cfg *c, REAL *f, int istep0, int nsteps, int nthreads)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    size_t ncell = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    FN(coef_t) q;
    REAL *fb, *fxa, *fya, *fza;
    int s, rc = FN(check_cfg)(c);
    if (rc) return rc;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    FN(make_coef)(c, &q);
    fb = (REAL *)calloc(ncell * 19, sizeof(REAL));
    fxa = (REAL *)calloc(ncell, sizeof(REAL));
    fya = (REAL *)calloc(ncell, sizeof(REAL));
    fza = (REAL *)calloc(ncell, sizeof(REAL));
    if (!fb || !fxa || !fya || !fza) { free(fb); free(fxa); free(fya); free(fza); return -10; }
    for (s = 0; s < nsteps; s++) {
        FN(force_field)(c, &q, istep0 + s, fxa, fya, fza);
        FN(stage_fbar)(c, &q, f, fb, fxa, fya, fza);
        FN(stage_ghost)(c, fb);
        FN(stage_flux)(c, &q, f, fb);
    }
    free(fb); free(fxa); free(fya); free(fza);
    return 0;
}

/* Density and velocity for output, src/dugks.cu:1021-1064 (calc_macro):
 * interior cells of ghosted scalar arrays; u includes +hdt*F_ambient. */
int FN(oracle_macro)(const oracle_cfg *c, const REAL *f, REAL *rho, REAL *ux, REAL *uy, REAL *uz)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    FN(coef_t) q;
    int i, j, k, ip;
    FN(make_coef)(c, &q);
    for (k = 1; k <= nz; k++)
        for (j = 1; j <= ny; j++)
            for (i = 1; i <= nx; i++) {
                REAL rr, uu, vv, ww;
                size_t s = SIDX(i, j, k);
                rr = uu = vv = ww = 0;
                for (ip = 0; ip < 19; ip++) {
                    REAL ff = f[IDX(ip, i, j, k)];
                    rr += ff;
                    uu += CIX[ip] * ff;
                    vv += CIY[ip] * ff;
                    ww += CIZ[ip] * ff;
                }
                uu /= rr;
                vv /= rr;
                ww /= rr;
                rho[s] = rr;
                ux[s] = uu + q.ambient_fx * q.hdt;
                uy[s] = vv + q.ambient_fy * q.hdt;
                uz[s] = ww + q.ambient_fz * q.hdt;
            }
    return 0;
}

#ifndef ORACLE_TANGENT
/* diag.dat and profiles-2.dat statistics, src/output.cu:223-334
 * (statistics_serial), on global non-ghosted arrays ijk=(k*ny+j)*nx+i.
 * diag: mean rho,u,v,w; min rho,u,v,w; max rho,u,v,w.
 * prof: per x index 9 values (uave, vave, wave, <uw>', <uv>', <vw>', <u'u'>, <v'v'>, <w'w'>). */
int FN(oracle_stats)(int nx, int ny, int nz, const REAL *rhg, const REAL *uxg, const REAL *uyg, const REAL *uzg,
                     double *diag, double *prof)
{
    REAL rhomean, umean, vmean, wmean;
    REAL rhomin, uxmin, uymin, uzmin;
    REAL rhomax, uxmax, uymax, uzmax;
    int i, j, k;
    rhomean = umean = vmean = wmean = 0;
    rhomin = uxmin = uymin = uzmin = 99999;
    rhomax = uxmax = uymax = uzmax = -99999;
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                size_t ijk = ((size_t)k * ny + j) * nx + i;
                rhomean += rhg[ijk];
                umean += uxg[ijk];
                vmean += uyg[ijk];
                wmean += uzg[ijk];
                if (rhg[ijk] < rhomin) rhomin = rhg[ijk];
                if (uxg[ijk] < uxmin) uxmin = uxg[ijk];
                if (uyg[ijk] < uymin) uymin = uyg[ijk];
                if (uzg[ijk] < uzmin) uzmin = uzg[ijk];
                if (rhg[ijk] > rhomax) rhomax = rhg[ijk];
                if (uxg[ijk] > uxmax) uxmax = uxg[ijk];
                if (uyg[ijk] > uymax) uymax = uyg[ijk];
                if (uzg[ijk] > uzmax) uzmax = uzg[ijk];
            }
    rhomean /= nx * ny * nz;
    umean /= nx * ny * nz;
    vmean /= nx * ny * nz;
    wmean /= nx * ny * nz;
    diag[0] = rhomean; diag[1] = umean; diag[2] = vmean; diag[3] = wmean;
    diag[4] = rhomin; diag[5] = uxmin; diag[6] = uymin; diag[7] = uzmin;
    diag[8] = rhomax; diag[9] = uxmax; diag[10] = uymax; diag[11] = uzmax;
    for (i = 0; i < nx; i++) {
        REAL uave, vave, wave, sxz, sxy, syz, usq, vsq, wsq;
        uave = vave = wave = 0;
        sxz = sxy = syz = 0;
        usq = vsq = wsq = 0;
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++) {
                size_t ijk = ((size_t)k * ny + j) * nx + i;
                uave += uxg[ijk];
                vave += uyg[ijk];
                wave += uzg[ijk];
                sxz += uxg[ijk] * uzg[ijk];
                sxy += uxg[ijk] * uyg[ijk];
                syz += uyg[ijk] * uzg[ijk];
                usq += uxg[ijk] * uxg[ijk];
                vsq += uyg[ijk] * uyg[ijk];
                wsq += uzg[ijk] * uzg[ijk];
            }
        uave /= (ny * nz);
        vave /= (ny * nz);
        wave /= (ny * nz);
        sxz /= (ny * nz);
        sxy /= (ny * nz);
        syz /= (ny * nz);
        usq /= (ny * nz);
        vsq /= (ny * nz);
        wsq /= (ny * nz);
        usq -= uave * uave;
        vsq -= vave * vave;
        wsq -= wave * wave;
        sxz -= uave * wave;
        sxy -= uave * vave;
        syz -= vave * wave;
        prof[9 * i + 0] = uave; prof[9 * i + 1] = vave; prof[9 * i + 2] = wave;
        prof[9 * i + 3] = sxz; prof[9 * i + 4] = sxy; prof[9 * i + 5] = syz;
        prof[9 * i + 6] = usq; prof[9 * i + 7] = vsq; prof[9 * i + 8] = wsq;
    }
    return 0;
}
#endif /* ORACLE_TANGENT */
