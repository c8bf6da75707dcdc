// DUGKS D3Q19 step kernels for sm_103a.
//
// Layout in HBM: structure of arrays, one plane per population.
//   f-tilde:         f[p*ps + ((k*ny + j)*pitch + i)]           (0-based i, j, k; interior only)
//   f-bar-plus:     fb[p*ps_b + (((k+1)*(ny+2) + j+1)*pitch_b + i + 1)]
//                   with one ghost layer on every side (periodic images, wall
//                   extrapolation), which replaces the reference's extend_fb_x /
//                   extend_fb_x_wall / extend_fb_y kernels and the MPI z exchange
//                   (src/dugks.cu:348-377, src/parallel.cu:185-234): written by
//                   fb_ghost_kernel (FP64; 16-bit forms with periodic x), by
//                   fbar_kernel itself (FP32; 16-bit forms between walls: the y / z
//                   images, the wall columns formed by the flux kernel in shared memory).
//
// Kernels:
//   fbar_kernel      stage (a), src/dugks.cu:1131-1196 (calc_fb1), with or without
//                    the ghost writes
//   fb_ghost_kernel  the ghost layer of f-bar-plus in a separate pass
//   flux_kernel      stages (c) (d) (e), src/dugks.cu:715-959 (calc_fx_tri) or the
//                    central-difference variant 421-649 (calc_fx); every face
//                    evaluated once, z-marching warp rows
//   macro_kernel     src/dugks.cu:1021-1064 (calc_macro)
//
// Template parameters: T is the arithmetic type, S the storage type of f and
// f-bar-plus (double, float, or the 16-bit deviation codecs of storage.cuh).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "d3q19.cuh"
#include "storage.cuh"

namespace dg {

// ---------------------------------------------------------------------------
// Parameters (host-filled, passed by value; T-typed so that no conversion from
// double runs in an FP32 kernel)
// ---------------------------------------------------------------------------
// Rows of the corner-weight table (products of the face_tri lerp weights that
// involve an x weight; column = face index I for the x-face rows, cell column
// for the y- and z-face rows).  class = xrep(p).
constexpr int CW_XY = 0;     // + 4 (class-1) + q   x face, c_y != 0 = c_z
constexpr int CW_XZ = 12;    // + 4 (class-1) + q   x face, c_z != 0 = c_y
constexpr int CW_XYZ = 24;   // + q (q < 8)         x face, c_y, c_z != 0 (c_x = 0)
constexpr int CW_Y4 = 32;    // + 4 slot4y(p) + q   y face, c_x != 0 = c_z (p = 1, 2, 7..10)
constexpr int CW_Y8 = 56;    // + 8 (class-1) + q   y face, c_x, c_z != 0 (c_y = 0)
constexpr int CW_Z4 = 72;    // + 4 slot4z(p) + q   z face, c_x != 0 = c_y (p = 1, 2, 11..14)
constexpr int CW_Z8 = 96;    // + 8 (class-1) + q   z face, c_x, c_y != 0 (c_z = 0)
constexpr int CW_ROWS = 112;

// Rows of the stretched-mesh gradient table P.gw (recon=gradient, mesh != uniform)
constexpr int GW_LAM = 0;     // x face I: interpolation weight of cell I+1 at the face
constexpr int GW_IDX = 1;     // x face I: 1 / (xc_{I+1} - xc_I)
constexpr int GW_WM = 2;      // column i: three-point x derivative weights on xc_{i-1}, xc_i, xc_{i+1}
constexpr int GW_W0 = 3;
constexpr int GW_WP = 4;
constexpr int GW_ROWS = 5;
__host__ __device__ constexpr int slot4y(int p) { return p == 1 ? 0 : (p == 2 ? 1 : p - 5); }
__host__ __device__ constexpr int slot4z(int p) { return p == 1 ? 0 : (p == 2 ? 1 : p - 9); }

// Forms whose throughput is set by the FP64 instruction count: they take the
// corner-weight faces and the one-axis force paths, which trade FP64
// operations for table loads and integer selects.
template <class T>
struct Fp64Form { static constexpr bool value = false; };
template <>
struct Fp64Form<double> { static constexpr bool value = true; };

template <class T, class S>
struct StepParams {
    int nx, ny, nz, pitch;
    long long ps;          // population stride of f-tilde (elements)
    int pitch_b;           // x pitch of f-bar-plus (>= nx+2: ghost columns 0 and nx+1 stored)
    long long ps_b;        // population stride of f-bar-plus (>= pitch_b*(ny+2)*(nz+2))
    int periodic_x;        // 0: bounce-back walls on the two x faces
    int perturb;           // per-cell perturbation force in stage (a)
    int force_on;          // ambient force non-zero
    int fax;               // the axis of the ambient force if at most one component is non-zero, else -1
    // stage (a)
    T hdt, bw1, bw2, bw0x3;      // bw0x3 = 3*bw0
    T F[3];                      // ambient force
    PopArr<T> Kb;                // 3*bw0*(c_p . F)
    T Fa, hFa, Kba, Kfa;         // fax >= 0: F, (0.5*hdt)*F, Kb, Kfs of the force axis (c_p = +1 on it)
    // faces
    T fw1, fw2, fw0x3;           // fw0x3 = 3*fw0
    T hF[3];                     // (0.5*hdt)*F, the face velocity shift (src/dugks.cu:698-700)
    T Kf[NPOP];                  // 3*fw0*(c_p . F)
    T fw2s, fw0x3s;              // fw2, 3*fw0 divided by fw1 (fluxes are kept divided by fw1)
    PopArr<T> Kfs;               // Kf divided by fw1
    T bwF;                       // bw2*hdt + bw0: momentum of f-bar-plus = j + rho F bwF (exact arithmetic)
    T cyuf, czuf;                // fw1*dt/dy, fw1*dt/dz
    // interpolation weights, (1-m, m) pairs in the reference's lerp form
    T ty_om, ty_m;               // transverse y, |hdt/dy|
    T tz_om, tz_m;               // transverse z, |hdt/dz|
    PopArr<T> yn_om, yn_m;       // y-face normal (dy/2 - hdt*cy)/dy
    PopArr<T> zn_om, zn_m;       // z-face normal (dz/2 - hdt*cz)/dz
    T cyu, czu;                  // dt/dy, dt/dz
    T q0, q1;                    // wall ghost extrapolation weights (2 on a uniform mesh)
    T g_idx, g_idy, g_idz;       // gradient reconstruction: 1/dx, 1/dy, 1/dz
    T g_i2dx, g_i2dy, g_i2dz;    // 1/(2dx), 1/(2dy), 1/(2dz)
    T ycw[NPOP][4];              // y face, c_x = 0, c_z != 0: z-lerp x y-lerp weight products
    T zcw[NPOP][4];              // z face, c_x = 0, c_y != 0: z-lerp x y-lerp weight products
    const T *cw;                 // [CW_ROWS][xws] corner weights of the FP64 faces (face_tri_cw)
    const T *xw;                 // [19*2][xws] x-face normal (1-m, m) of face I (between cells I, I+1, 1-based)
    const T *txw;                // [19*2][xws] transverse x (1-t, t) per column 0..nx+1
    int xws;                     // row stride of xw / txw (nx+2)
    const T *gw;                 // [GW_ROWS][xws] gradient reconstruction weights of a stretched x mesh
    int grad_st;                 // 1: recon=gradient on a stretched x mesh (face_grad reads gw)
    const T *cxu;                // [nx+2] dt/dxx(i)
    const T *cxuf;               // [nx+2] fw1*dt/dxx(i)
    // perturbation forcing (src/dugks.cu:1086-1126) as separable factors
    const T *pert_x;             // [nx+2][3]: (1-cos xx), sin xx, in-zone flag
    const T *pert_y;             // [ny+2][3]: cos(beta yy), sin(beta yy), 0
    const T *pert_z;             // [nz+2][3]: cos(gamma zz), sin(gamma zz), 0
    T pert_ax, pert_ay, pert_az, pert_FF;  // per-step amplitude prefactors
    int *err;                    // device error flag (bit 0: a TMA pipeline wait gave up)
    // optional per-cell body-force field phi (an extension): F(cell) = F_ambient + phi(cell) e_ffaxis in
    // stage (a), F(face) = F_ambient + (phi(c1) + phi(c2))/2 e_ffaxis on a face between c1 and c2
    const T *ffield;             // [k][j][pitch] like one population of f-tilde; nullptr = none
    int ffaxis;
    Codec<T, S> codec;           // storage decode / encode constants
};

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T lerp2(T om, T m, T a, T b)
{
    return om * a + m * b;  // (1-m)*a + m*b, src/dugks.cu:969-977
}

// Equilibrium of the pair (p, opp(p)) from eu = 3 c_p.u, base = 1 - 1.5|u|^2
// and wr = w_p*rho:  feq = wr*(1 + eu + eu^2/2 - 1.5|u|^2)
// (src/dugks.cu:1201-1207 with 1/RT = 3), as wr*t +- wr*eu: five operations
// for the pair.
template <class T>
__device__ __forceinline__ void feq_pair(T eu, T base, T wr, T &fp, T &fm)
{
    const T wt = wr * fma(T(0.5) * eu, eu, base);
    fp = fma(wr, eu, wt);
    fm = fma(-wr, eu, wt);
}

// Zeroth and first moments of 19 values, from the sums and differences of the
// nine opposite pairs (18 operations): rho from the nine sums, each momentum
// component from its five differences -- 39 operations instead of 45 for the
// direct sums (the reference sums sequentially over ip, src/dugks.cu:687-693:
// same values to rounding), in short dependency chains for the reduced-rate
// FP64 pipe of GB300.
template <class T>
__device__ __forceinline__ void moments(const T v[NPOP], T &r, T &jx, T &jy, T &jz)
{
    const T s1 = v[1] + v[2], d1 = v[1] - v[2];          // (+-1, 0, 0)
    const T s3 = v[3] + v[4], d3 = v[3] - v[4];          // (0, +-1, 0)
    const T s5 = v[5] + v[6], d5 = v[5] - v[6];          // (0, 0, +-1)
    const T s7 = v[7] + v[10], d7 = v[7] - v[10];        // 7 = (1, 1, 0)
    const T s8 = v[8] + v[9], d8 = v[8] - v[9];          // 8 = (-1, 1, 0)
    const T s11 = v[11] + v[14], d11 = v[11] - v[14];    // 11 = (1, 0, 1)
    const T s12 = v[12] + v[13], d12 = v[12] - v[13];    // 12 = (-1, 0, 1)
    const T s15 = v[15] + v[18], d15 = v[15] - v[18];    // 15 = (0, 1, 1)
    const T s16 = v[16] + v[17], d16 = v[16] - v[17];    // 16 = (0, -1, 1)
    r = ((v[0] + s1) + (s3 + s5)) + ((s7 + s8) + (s11 + s12)) + (s15 + s16);
    jx = ((d1 + d7) - d8) + (d11 - d12);
    jy = ((d3 + d7) + d8) + (d15 - d16);
    jz = ((d5 + d11) + d12) + (d15 + d16);
}

// moments for FP32 arithmetic on the population pairs (2m-1, 2m), m = 1..9, as
// packed FP32x2 sums (sm_100+ FADD2/FFMA2): rho from the nine pairs summed
// pairwise, each momentum component from the pairs that move along it, whose
// c pattern within a pair is (+, -), (+, +) or (-, -) -- 27 operations instead
// of 39 (same values to rounding).
__device__ __forceinline__ float2 sub_x2(float2 a, float2 b)
{
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);  // a - b, one rounding
}
__device__ __forceinline__ void moments_x2(const float v[NPOP], float &r, float &jx, float &jy, float &jz)
{
    auto V = [&](int m) { return make_float2(v[2 * m - 1], v[2 * m]); };
    const float2 a = __fadd2_rn(__fadd2_rn(V(1), V(2)), __fadd2_rn(V(3), V(4)));
    const float2 b = __fadd2_rn(__fadd2_rn(V(5), V(6)), __fadd2_rn(V(7), V(8)));
    const float2 sr = __fadd2_rn(__fadd2_rn(a, b), V(9));
    r = v[0] + (sr.x + sr.y);
    // x: pairs 1, 4, 5, 6, 7 are (+, -)
    const float2 X = __fadd2_rn(__fadd2_rn(V(1), V(4)), __fadd2_rn(__fadd2_rn(V(5), V(6)), V(7)));
    jx = X.x - X.y;
    // y: pairs 2, 8, 9 (+, -); 4 (+, +); 5 (-, -)
    const float2 Y1 = __fadd2_rn(__fadd2_rn(V(2), V(8)), V(9)), Y2 = sub_x2(V(4), V(5));
    jy = (Y1.x - Y1.y) + (Y2.x + Y2.y);
    // z: pair 3 (+, -); 6, 8 (+, +); 7, 9 (-, -)
    const float2 Z = sub_x2(__fadd2_rn(V(6), V(8)), __fadd2_rn(V(7), V(9)));
    const float2 V3 = V(3);
    jz = (V3.x - V3.y) + (Z.x + Z.y);
}

// 1/r: FP64 from a single-precision seed x (relative error e ~ 2^-23) and one
// third-order correction x (1 + e + e^2) (truncation error ~e^3, far below the
// rounding level): three dependent FMAs, cheaper than the full-precision
// divide on the FP64 pipe; the correctly rounded FP32 reciprocal (same result
// as 1.0f / r, without the division's multi-instruction sequence) for FP32.
__device__ __forceinline__ double recip(double r)
{
    const double x = double(__frcp_rn(float(r)));
    const double e = fma(-r, x, 1.0);
    return fma(x, fma(e, e, e), x);
}
__device__ __forceinline__ float recip(float r) { return __frcp_rn(r); }

// First term of the update, 4/3 f-bar-plus - 1/3 f (src/dugks.cu:954).  FP64:
// as written.  FP32 arithmetic: fb + (fb - f)/3, whose coefficients sum to one
// exactly; float(4/3) - float(1/3) = 1 + 3e-8 would make the mass and momentum
// grow by that factor every step (the reference evaluates this line in double).
template <class T>
__device__ __forceinline__ T upd_base(T fb, T fo, T c43, T c13)
{
    return sizeof(T) == 8 ? fma(fb, c43, -(fo * c13)) : fma(fb - fo, c13, fb);
}

// New f-tilde of one population of a cell: the first term (upd_base of its
// f-bar-plus and f-tilde as stored) plus coef x (flux difference) along each
// axis it moves on (src/dugks.cu:949-956), then the stored value.  Plain
// forms: the terms are added to the first term in axis order.  16-bit forms:
// the first term is in deviation units (an affine combination of stored
// deviations, coefficients summing to one) and the flux terms in f units with
// the rest state cancelled, so they are summed apart and scaled once,
// d = base + sum / s_p, then rounded as every stored deviation.
template <class T, class S>
struct UpdateSum {
    T r, acc = T(0);
    int nt = 0;
    __device__ __forceinline__ explicit UpdateSum(T base) : r(base) {}
    __device__ __forceinline__ void add(T coef, T diff)
    {
        if constexpr (Codec<T, S>::deviation)
            acc = nt ? fma(coef, diff, acc) : coef * diff;
        else
            r = fma(coef, diff, r);
        ++nt;
    }
    __device__ __forceinline__ S encode(const Codec<T, S> &c, int p, unsigned hc) const
    {
        if constexpr (Codec<T, S>::deviation)
            return c.encode_dh(p, nt ? fma(c.is[p], acc, r) : r, hc);
        else
            return c.encode_h(p, r, hc);
    }
};

// The update's pairing rule: the pair (2m-1, 2m) moves along the same axes
// and sits in adjacent slots of each of their flux lists.
__host__ __device__ constexpr bool update_pairs_ok()
{
    for (int m = 1; m <= 9; ++m) {
        const int p = 2 * m - 1, q = 2 * m;
        for (int a = 0; a < 3; ++a) {
            if ((cc(a, p) != 0) != (cc(a, q) != 0)) return false;
            if (cc(a, p) != 0 && flux_slot(a, q) != flux_slot(a, p) + 1) return false;
        }
    }
    return true;
}
static_assert(update_pairs_ok(), "update population pairs must share their axes and adjacent flux slots");

// UpdateSum for the population pair (2m-1, 2m) in FP32 arithmetic, two at a
// time (FFMA2 / FMUL2): the same operations in the same order for each.
template <class S>
struct UpdatePair {
    float2 r, acc = make_float2(0.0f, 0.0f);
    int nt = 0;
    __device__ __forceinline__ explicit UpdatePair(float2 fb, float2 fo)
        : r(__ffma2_rn(__ffma2_rn(fo, make_float2(-1.0f, -1.0f), fb), make_float2(1.0f / 3.0f, 1.0f / 3.0f), fb))
    {
    }  // upd_base, FP32 form: fb + (fb - fo) / 3
    __device__ __forceinline__ void add(float2 coef, float2 diff)
    {
        if constexpr (Codec<float, S>::deviation)
            acc = nt ? __ffma2_rn(coef, diff, acc) : __fmul2_rn(coef, diff);
        else
            r = __ffma2_rn(coef, diff, r);
        ++nt;
    }
    __device__ __forceinline__ void store(const Codec<float, S> &c, S *out, long long ip, long long iq, int p, int q,
                                          unsigned hc) const
    {
        if constexpr (Codec<float, S>::deviation) {
            const float2 d = nt ? __ffma2_rn(make_float2(c.is[p], c.is[q]), acc, r) : r;
            out[ip] = c.encode_dh(p, d.x, hc);
            out[iq] = c.encode_dh(q, d.y, hc);
        } else {
            out[ip] = c.encode_h(p, r.x, hc);
            out[iq] = c.encode_h(q, r.y, hc);
        }
    }
};

// All 19 equilibria for density r and velocity (u, v, w).
template <class T>
__device__ __forceinline__ void feq_all(T r, T u, T v, T w, T fe[NPOP])
{
    const T u3 = T(3) * u, v3 = T(3) * v, w3 = T(3) * w;
    const T base = fma(T(-1.5), fma(u, u, fma(v, v, w * w)), T(1));
    const T wr1 = weight<T>(1) * r, wr2 = weight<T>(7) * r;
    fe[0] = (weight<T>(0) * r) * base;
    feq_pair(u3, base, wr1, fe[1], fe[2]);
    feq_pair(v3, base, wr1, fe[3], fe[4]);
    feq_pair(w3, base, wr1, fe[5], fe[6]);
    feq_pair(u3 + v3, base, wr2, fe[7], fe[10]);
    feq_pair(v3 - u3, base, wr2, fe[8], fe[9]);
    feq_pair(u3 + w3, base, wr2, fe[11], fe[14]);
    feq_pair(w3 - u3, base, wr2, fe[12], fe[13]);
    feq_pair(v3 + w3, base, wr2, fe[15], fe[18]);
    feq_pair(w3 - v3, base, wr2, fe[16], fe[17]);
}

// The equilibria of the 10 populations that cross a face normal to AX (the
// others are left unset).
template <class T, int AX>
__device__ __forceinline__ void feq_face(T r, T u, T v, T w, T fe[NPOP])
{
    const T u3 = T(3) * u, v3 = T(3) * v, w3 = T(3) * w;
    const T base = fma(T(-1.5), fma(u, u, fma(v, v, w * w)), T(1));
    const T wr1 = weight<T>(1) * r, wr2 = weight<T>(7) * r;
    if (AX == 0) feq_pair(u3, base, wr1, fe[1], fe[2]);
    else if (AX == 1) feq_pair(v3, base, wr1, fe[3], fe[4]);
    else feq_pair(w3, base, wr1, fe[5], fe[6]);
    if (AX != 2) {
        feq_pair(u3 + v3, base, wr2, fe[7], fe[10]);
        feq_pair(v3 - u3, base, wr2, fe[8], fe[9]);
    }
    if (AX != 1) {
        feq_pair(u3 + w3, base, wr2, fe[11], fe[14]);
        feq_pair(w3 - u3, base, wr2, fe[12], fe[13]);
    }
    if (AX != 0) {
        feq_pair(v3 + w3, base, wr2, fe[15], fe[18]);
        feq_pair(w3 - v3, base, wr2, fe[16], fe[17]);
    }
}

// ---------------------------------------------------------------------------
// Stage (a): f-bar-plus = bw1 f + (bw2 + bw0 F.(c-u)/RT) feq(rho, u + hdt F)
// ---------------------------------------------------------------------------
template <class T, class S>
__device__ __forceinline__ void cell_force(const StepParams<T, S> &P, int i, int j, int k, T &Fx, T &Fy, T &Fz)
{
    Fx = P.F[0]; Fy = P.F[1]; Fz = P.F[2];
    if (P.ffield) {
        const T phi = __ldg(P.ffield + ((long long)k * P.ny + j) * P.pitch + i);
        if (P.ffaxis == 0) Fx += phi; else if (P.ffaxis == 1) Fy += phi; else Fz += phi;
    }
    if (P.perturb) {
        // 1-based cell (i+1, j+1, k+1); zone flag set for 3 < i < nx/4 + 2 (src/dugks.cu:1112)
        const T *px = P.pert_x + 3 * (i + 1);
        if (px[2] != T(0)) {
            const T *py = P.pert_y + 3 * (j + 1);
            const T *pz = P.pert_z + 3 * (k + 1);
            Fx = P.pert_ax * px[0] * py[0] * pz[0];
            Fy = P.pert_ay * px[1] * py[0] * pz[1];
            Fz = P.pert_FF * (T(1) - P.pert_az * px[1] * py[1] * pz[0]);
        }
    }
}

// Copies the 19 f-bar-plus values of stored column I, row J, plane K (written
// by this thread) to their periodic images in y and z when ny or nz is 1, so
// that both ghost rows (planes) are images of the one interior row (plane).
template <class S>
__device__ __forceinline__ void copy_images(S *fb, long long ps_b, int I, int J, int K, int ny, int nz, int pitch_b)
{
    int js[3], ks[3], nj = 0, nk = 0;
    js[nj++] = J;
    if (J == 1) js[nj++] = ny + 1;
    if (J == ny) js[nj++] = 0;
    ks[nk++] = K;
    if (K == 1) ks[nk++] = nz + 1;
    if (K == nz) ks[nk++] = 0;
    const long long src = ((long long)K * (ny + 2) + J) * pitch_b + I;
    for (int p = 0; p < NPOP; ++p) {
        const S v = fb[p * ps_b + src];
        for (int a = 0; a < nk; ++a)
            for (int b = 0; b < nj; ++b)
                if (a || b) fb[p * ps_b + ((long long)ks[a] * (ny + 2) + js[b]) * pitch_b + I] = v;
    }
}

// Stage (a) for one cell.  GHOST = 0: the interior of f-bar-plus only
// (fb_ghost_kernel fills the ghost layer).  GHOST = 2: the interior and its
// periodic images in y and z only (the 16-bit forms between walls, whose flux
// kernel forms the wall ghost columns itself).  GHOST = 1: the ghost layer is
// written by the threads that hold its sources, in the same launch -- a cell
// of the first/last row or plane also writes its periodic images in y and z
// (src/dugks.cu:1256-1273, src/parallel.cu:192-199), the first/last cell of a
// row writes the periodic x copy (src/dugks.cu:1212-1229), and between walls
// each warp next to a wall forms the extrapolation g0 = q0 fb(1) + (1-q0) fb(2),
// g_{nx+1} = q1 fb(nx) + (1-q1) fb(nx-1) of the stored values (src/dugks.cu:1234-1251;
// stretched mesh src/fortran/channel/src/dugks.cuf:365-374), one population per
// lane.  Warps away from walls, x ends and boundary rows/planes take the
// plain path.  xoff shifts the cells by one thread when nx = 1 (mod 32) so
// that cells nx-1 and nx share a warp.  The result equals the reference's
// x -> y -> z fill order.
// Stage (a) with a force along axis A only (FP64 form): f-bar-plus_p =
// (B + K_p) feq_p + bw1 f_p with K_p in {0, +-Kb}, fused per opposite pair
// (p, q): feq_{p,q} = w r (t +- eu), t = base + eu^2/2.  A pair with c_A = 0
// shares K = B w r:  K t + (bw1 f_p) +- K eu  (7 operations for the pair, 9
// for the equilibria followed by the combines); a pair along A has
// K_{p,q} = (B +- Kb) w r:  K_p (t + eu) + bw1 f_p  (8 operations).
template <class T, int A>
__device__ __forceinline__ void fbar_one_axis(T r, T u, T vv, T w, T B, T Kb, T bw1, const T v[NPOP], T ob[NPOP])
{
    const T u3 = T(3) * u, v3 = T(3) * vv, w3 = T(3) * w;
    const T base = fma(T(-1.5), fma(u, u, fma(vv, vv, w * w)), T(1));
    const T wr0 = weight<T>(0) * r, wr1 = weight<T>(1) * r, wr2 = weight<T>(7) * r;
    const T Bp = B + Kb, Bm = B - Kb;
    const T K1 = B * wr1, K2 = B * wr2, Kp1 = Bp * wr1, Km1 = Bm * wr1, Kp2 = Bp * wr2, Km2 = Bm * wr2;
    ob[0] = fma(B * wr0, base, bw1 * v[0]);
    auto pair = [&](int p, int q, T eu, int cls) {
        const T t = fma(T(0.5) * eu, eu, base);
        const int ca = cc(A, p);
        if (ca == 0) {
            const T K = cls == 1 ? K1 : K2;
            const T X = K * t;
            ob[p] = fma(K, eu, fma(bw1, v[p], X));
            ob[q] = fma(-K, eu, fma(bw1, v[q], X));
        } else {
            const T Kp = cls == 1 ? (ca > 0 ? Kp1 : Km1) : (ca > 0 ? Kp2 : Km2);
            const T Kq = cls == 1 ? (ca > 0 ? Km1 : Kp1) : (ca > 0 ? Km2 : Kp2);
            ob[p] = fma(Kp, t + eu, bw1 * v[p]);
            ob[q] = fma(Kq, t - eu, bw1 * v[q]);
        }
    };
    pair(1, 2, u3, 1);
    pair(3, 4, v3, 1);
    pair(5, 6, w3, 1);
    pair(7, 10, u3 + v3, 2);
    pair(8, 9, v3 - u3, 2);
    pair(11, 14, u3 + w3, 2);
    pair(12, 13, w3 - u3, 2);
    pair(15, 18, v3 + w3, 2);
    pair(16, 17, w3 - v3, 2);
}

template <class T, class S, int GHOST>
__global__ void __launch_bounds__(256) fbar_kernel(const S *__restrict__ f, S *__restrict__ fb, const StepParams<T, S> P,
                                                   int xoff)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x - xoff;
    const int j = blockIdx.y;
    const int k = blockIdx.z;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const bool in = i >= 0 && i < nx;
    const int wbase = blockIdx.x * blockDim.x + (threadIdx.x & ~31) - xoff;  // cell of lane 0
    const bool wall_warp =
        GHOST == 1 && !P.periodic_x && ((wbase <= 1 && wbase + 31 >= 0) || (wbase <= nx - 1 && wbase + 31 >= nx - 2));
    if (!in && !wall_warp) return;
    const int ic = in ? i : (i < 0 ? 0 : nx - 1);  // lanes past the row read a valid cell and store nothing
    const long long c = ((long long)k * ny + j) * P.pitch + ic;
    const long long cb = ((long long)(k + 1) * (ny + 2) + (j + 1)) * P.pitch_b + ic + 1;

    T v[NPOP];
    if constexpr (Codec<T, S>::deviation) {
        // decoded two populations at a time (pairs 2m-1, 2m)
        v[0] = P.codec.load_nc(f, c, 0);
#pragma unroll
        for (int m = 1; m <= 9; ++m) {
            const int p = 2 * m - 1, q = 2 * m;
            const float2 x = P.codec.dec2(p, q, make_float2(P.codec.raw_nc(f, p * P.ps + c), P.codec.raw_nc(f, q * P.ps + c)));
            v[p] = x.x;
            v[q] = x.y;
        }
    } else {
#pragma unroll
        for (int p = 0; p < NPOP; ++p) v[p] = P.codec.load_nc(f, p * P.ps + c, p);
    }

    // the 16-bit forms' moments two at a time; the FP32 form keeps the pair sums, whose
    // density, as the target of the moment correction below, measured a ten times smaller
    // mass drift (2e-7 against 2e-6 over 50,000 turbulent-channel steps)
    T r, jx, jy, jz;
    if constexpr (Codec<T, S>::deviation)
        moments_x2(v, r, jx, jy, jz);
    else
        moments(v, r, jx, jy, jz);
    const T inv = recip(r);
    T u = jx * inv, vv = jy * inv, w = jz * inv;

    T Fx, Fy, Fz;
    cell_force(P, ic, j, k, Fx, Fy, Fz);
    const bool forced = P.force_on || P.perturb || P.ffield;
    // one ambient force component and no per-cell force: the same values from
    // that component alone, and B + K_p in three values (FP64 form)
    const bool one_axis = Fp64Form<T>::value && P.fax >= 0 && !P.perturb && !P.ffield;
    // coefficient of feq: bw2 + 3 bw0 (F.c - F.u) = B + K_p
    T B = P.bw2;
    if (one_axis) {
        if (P.force_on) {
            const int a = P.fax;
            const T ua = fma(P.hdt, P.Fa, a == 0 ? u : (a == 1 ? vv : w));
            u = a == 0 ? ua : u;
            vv = a == 1 ? ua : vv;
            w = a == 2 ? ua : w;
            B = fma(-P.bw0x3, P.Fa * ua, P.bw2);
        }
    } else if (forced) {
        u = fma(P.hdt, Fx, u);
        vv = fma(P.hdt, Fy, vv);
        w = fma(P.hdt, Fz, w);
        B = fma(-P.bw0x3, fma(Fx, u, fma(Fy, vv, Fz * w)), P.bw2);
    }

    const unsigned hc = P.codec.cell_hash(cb);
    T ob[NPOP];
    if (one_axis) {
        if (P.fax == 0)
            fbar_one_axis<T, 0>(r, u, vv, w, B, P.Kba, P.bw1, v, ob);
        else if (P.fax == 1)
            fbar_one_axis<T, 1>(r, u, vv, w, B, P.Kba, P.bw1, v, ob);
        else
            fbar_one_axis<T, 2>(r, u, vv, w, B, P.Kba, P.bw1, v, ob);
    } else {
        T fe[NPOP];
        feq_all(r, u, vv, w, fe);
        auto kcoef = [&](int p) {
            T K = P.Kb[p];
            if (P.perturb || P.ffield) {
                T cf = T(0);
                if (cx(p)) cf += cx(p) > 0 ? Fx : -Fx;
                if (cy(p)) cf += cy(p) > 0 ? Fy : -Fy;
                if (cz(p)) cf += cz(p) > 0 ? Fz : -Fz;
                K = P.bw0x3 * cf;
            }
            return K;
        };
        if constexpr (std::is_same<T, float>::value) {
            // the same operations on the pairs (2m-1, 2m), two at a time; B + K_p as the
            // one-population form rounds it (with a per-cell force, K_p = 3 bw0 (c_p . F) and
            // B + K_p is one fused multiply-add)
            auto bk = [&](int p) {
                if (P.perturb || P.ffield) {
                    T cf = T(0);
                    if (cx(p)) cf += cx(p) > 0 ? Fx : -Fx;
                    if (cy(p)) cf += cy(p) > 0 ? Fy : -Fy;
                    if (cz(p)) cf += cz(p) > 0 ? Fz : -Fz;
                    return fma(P.bw0x3, cf, B);
                }
                return B + P.Kb[p];
            };
            ob[0] = fma(bk(0), fe[0], P.bw1 * v[0]);
            const float2 bw = make_float2(P.bw1, P.bw1);
#pragma unroll
            for (int m = 1; m <= 9; ++m) {
                const int p = 2 * m - 1, q = 2 * m;
                const float2 o = __ffma2_rn(make_float2(bk(p), bk(q)), make_float2(fe[p], fe[q]),
                                            __fmul2_rn(bw, make_float2(v[p], v[q])));
                ob[p] = o.x;
                ob[q] = o.y;
            }
        } else {
#pragma unroll
            for (int p = 0; p < NPOP; ++p) ob[p] = fma(B + kcoef(p), fe[p], P.bw1 * v[p]);
        }
    }
    if (sizeof(T) == 4) {
        // FP32 arithmetic: the moments of f-bar-plus are set to their exact values
        // (exact arithmetic: sum f-bar-plus = rho, sum c f-bar-plus = j + rho F
        // (bw2 hdt + bw0)).  The float weights and bw1, bw2 carry rounding biases
        // of ~1e-8 that would otherwise add up, step after step, into a drift of
        // the total mass and momentum.  The momentum defect goes to the +- pair of
        // each axis (mass unchanged), the mass defect to the rest population.
        T r2, mx, my, mz;
        if constexpr (Codec<T, S>::deviation)
            moments_x2(ob, r2, mx, my, mz);
        else
            moments(ob, r2, mx, my, mz);
        T tx = jx, ty = jy, tz = jz;
        if (forced) {
            const T g = r * P.bwF;
            tx = fma(g, Fx, jx);
            ty = fma(g, Fy, jy);
            tz = fma(g, Fz, jz);
        }
        const T dx = T(0.5) * (tx - mx), dy = T(0.5) * (ty - my), dz = T(0.5) * (tz - mz);
        ob[1] += dx; ob[2] -= dx;
        ob[3] += dy; ob[4] -= dy;
        ob[5] += dz; ob[6] -= dz;
        const T a = (ob[1] + ob[2]) + (ob[3] + ob[4]), b = (ob[5] + ob[6]) + (ob[7] + ob[8]);
        const T c2 = (ob[9] + ob[10]) + (ob[11] + ob[12]), d = (ob[13] + ob[14]) + (ob[15] + ob[16]);
        ob[0] = r - ((((a + b) + (c2 + d)) + ob[17]) + ob[18]);
    }

    // periodic images of this row and plane (uniform over the warp): J = 1 -> ny+1,
    // J = ny -> 0, likewise K, and the corner image
    const long long rstep = P.pitch_b, pstep = (long long)(ny + 2) * P.pitch_b;
    const long long dj = j == 0 ? ny * rstep : (j == ny - 1 ? -(long long)ny * rstep : 0);
    const long long dk = k == 0 ? nz * pstep : (k == nz - 1 ? -(long long)nz * pstep : 0);
    const bool small = ny == 1 || nz == 1;  // two images along one axis: copied at the end
    const bool img = !small && (dj != 0 || dk != 0);
    const bool xend = wbase <= 0 || wbase + 31 >= nx - 1;
    S enc[NPOP];  // the stored values (16-bit forms: deviations of the pairs formed two at a time)
    if constexpr (Codec<T, S>::deviation) {
        enc[0] = P.codec.encode_h(0, ob[0], hc);
#pragma unroll
        for (int m = 1; m <= 9; ++m) {
            const int p = 2 * m - 1, q = 2 * m;
            const float2 d = P.codec.dev2(p, q, make_float2(ob[p], ob[q]));
            enc[p] = P.codec.encode_dh(p, d.x, hc);
            enc[q] = P.codec.encode_dh(q, d.y, hc);
        }
    } else {
#pragma unroll
        for (int p = 0; p < NPOP; ++p) enc[p] = P.codec.encode_h(p, ob[p], hc);
    }
    if (GHOST == 0 || (!wall_warp && !img && !small && !(P.periodic_x && xend))) {
#pragma unroll
        for (int p = 0; p < NPOP; ++p) fb[p * P.ps_b + cb] = enc[p];
        return;
    }
    __shared__ T wv[4][4][NPOP];  // per warp: values of cells 1, 2, nx, nx-1 (blocks of at most 128 threads)
    auto put = [&](S *q, S val) {  // a value and its images
        q[0] = val;
        if (img) {
            if (dj) q[dj] = val;
            if (dk) q[dk] = val;
            if (dj && dk) q[dj + dk] = val;
        }
    };
    const long long rowb = cb - (ic + 1);  // stored column 0 of this row and plane
    const int wl = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < NPOP; ++p) {
        const T out = ob[p];
        S *pl = fb + p * P.ps_b + rowb;
        const S e = enc[p];
        if (in) {
            put(pl + ic + 1, e);
            if (P.periodic_x) {
                if (ic == 0) put(pl + nx + 1, e);
                if (ic == nx - 1) put(pl, e);
            }
        }
        if (wall_warp) {
            // the stored values of the two cells next to each wall
            const T mine = Codec<T, S>::deviation ? P.codec.dec(p, T(e)) : out;
            if (in && ic == 0) wv[wl][0][p] = mine;
            if (in && ic == 1) wv[wl][1][p] = mine;
            if (in && ic == nx - 1) wv[wl][2][p] = mine;
            if (in && ic == nx - 2) wv[wl][3][p] = mine;
        }
    }
    if (wall_warp) {
        __syncwarp();
        const int lane = threadIdx.x & 31;
        if (lane < NPOP) {
            const int p = lane;
            S *pl = fb + p * P.ps_b + rowb;
            if (wbase <= 0) put(pl, P.codec.encode_h(p, P.q0 * wv[wl][0][p] + (T(1) - P.q0) * wv[wl][1][p], hc));
            if (wbase + 31 >= nx - 1)
                put(pl + nx + 1, P.codec.encode_h(p, P.q1 * wv[wl][2][p] + (T(1) - P.q1) * wv[wl][3][p], hc));
        }
        __syncwarp();
    }
    if (small && in) {
        copy_images(fb, P.ps_b, ic + 1, j + 1, k + 1, ny, nz, P.pitch_b);
        if (GHOST == 1 && ic == 0) copy_images(fb, P.ps_b, P.periodic_x ? nx + 1 : 0, j + 1, k + 1, ny, nz, P.pitch_b);
        if (GHOST == 1 && ic == nx - 1)
            copy_images(fb, P.ps_b, P.periodic_x ? 0 : nx + 1, j + 1, k + 1, ny, nz, P.pitch_b);
    }
}

// ---------------------------------------------------------------------------
// Ghost layer of f-bar-plus: every ghost cell takes its value from the
// interior -- the periodic image in y and z (the reference's extend_fb_y and
// z exchange, src/dugks.cu:1256-1273, src/parallel.cu:192-199) and in x the
// periodic copy (extend_fb_x, src/dugks.cu:1212-1229) or the linear wall
// extrapolation (extend_fb_x_wall, src/dugks.cu:1234-1251; stretched mesh
// src/fortran/channel/src/dugks.cuf:365-374).  The result equals the
// reference's x -> y -> z fill order.
// Ghost cells, by group: x columns 0 and nx+1 for all stored rows and planes,
// y rows 0 and ny+1 for interior columns and all planes, z planes 0 and nz+1
// for the interior columns and rows.
// ---------------------------------------------------------------------------
template <class T, class S>
__global__ void __launch_bounds__(256) fb_ghost_kernel(S *__restrict__ fb, const StepParams<T, S> P)
{
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long nxg = 2LL * (ny + 2) * (nz + 2);
    const long long nyg = 2LL * nx * (nz + 2);
    const long long nzg = 2LL * nx * ny;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int gi, gj, gk;
    if (q < nxg) {
        gi = (q & 1) ? nx + 1 : 0;
        q >>= 1;
        gj = int(q % (ny + 2));
        gk = int(q / (ny + 2));
    } else if ((q -= nxg) < nyg) {
        gj = (q & 1) ? ny + 1 : 0;
        q >>= 1;
        gi = int(q % nx) + 1;
        gk = int(q / nx);
    } else if ((q -= nyg) < nzg) {
        gk = (q & 1) ? nz + 1 : 0;
        q >>= 1;
        gi = int(q % nx) + 1;
        gj = int(q / nx) + 1;
    } else {
        return;
    }
    // periodic images in y and z
    const int sj = gj == 0 ? ny : (gj == ny + 1 ? 1 : gj);
    const int sk = gk == 0 ? nz : (gk == nz + 1 ? 1 : gk);
    const long long dst = ((long long)gk * (ny + 2) + gj) * P.pitch_b + gi;
    const long long row = ((long long)sk * (ny + 2) + sj) * P.pitch_b;
    if (gi >= 1 && gi <= nx) {
#pragma unroll
        for (int p = 0; p < NPOP; ++p) fb[p * P.ps_b + dst] = fb[p * P.ps_b + row + gi];
    } else if (P.periodic_x) {
        const int si = gi == 0 ? nx : 1;
#pragma unroll
        for (int p = 0; p < NPOP; ++p) fb[p * P.ps_b + dst] = fb[p * P.ps_b + row + si];
    } else {
        const int a = gi == 0 ? 1 : nx, b = gi == 0 ? 2 : nx - 1;
        const T q0 = gi == 0 ? P.q0 : P.q1;
#pragma unroll
        for (int p = 0; p < NPOP; ++p) {
            const T va = P.codec.load(fb, p * P.ps_b + row + a, p);
            const T vb = P.codec.load(fb, p * P.ps_b + row + b, p);
            P.codec.store(fb, p * P.ps_b + dst, p, q0 * va + (T(1) - q0) * vb);
        }
    }
}

// ---------------------------------------------------------------------------
// Stages (b)/(c), (d), (e): face reconstruction, face flux, finite-volume update.
//
// A CTA is W warps.  Warps 1..W-1 each own one row of 32 cells (lane = x)
// and march over a chunk of z planes; per plane every thread evaluates the
// +x, +y and +z faces of its cell once, takes the -x face from lane-1
// (warp shuffle), the -y face from the warp below (shared memory) and the
// -z face from its own previous plane (register), and updates its cell.
// Warp 0 is the halo: it evaluates the -y faces of the first row and, one
// lane per row, the -x faces of the first column.  f-bar-plus is read through
// L1 (no shared-memory staging); its ghost columns are stored by
// fb_ghost_kernel and its y / z images are index wraps.
// ---------------------------------------------------------------------------
// f-bar-plus through L1: rows and planes are stored indices 0..n+1 (ghosts included)
template <class T, class S>
struct FbRead {
    const S *fb;
    long long ps;
    int pitch, ny, nz;
    const Codec<T, S> &codec;
    __device__ __forceinline__ long long rb(int j, int k) const
    {
        return ((long long)k * (ny + 2) + j) * pitch;
    }
    __device__ __forceinline__ T operator()(int p, long long row, int col) const
    {
        return codec.load_nc(fb, p * ps + row + col, p);
    }
    __device__ __forceinline__ T raw(int p, long long row, int col) const { return codec.raw_nc(fb, p * ps + row + col); }
    __device__ __forceinline__ S bits(int p, long long row, int col) const { return __ldg(fb + p * ps + row + col); }
    __device__ __forceinline__ T dec(int p, T x) const { return codec.dec(p, x); }
    __device__ __forceinline__ T dec_e(int p, T x) const { return codec.dec_e(p, x); }
    __device__ __forceinline__ float2 dec_e2(int p, int q, float2 x) const { return codec.dec_e2(p, q, x); }
};

// 19 reconstructed values of one face, trilinear characteristic interpolation
// (src/dugks.cu:756-906) in the reference's x -> y -> z lerp order:
//   AX=0: face I between columns I and I+1 (I = 0: anchor column 1, other 0)
//   AX=1: face J between rows J and J+1 at column i
//   AX=2: face K between planes K and K+1 at column i
template <class T, class S, int AX, class RD>
__device__ __forceinline__ void face_tri(const StepParams<T, S> &P, const RD &R, int i, int j, int k, T v[NPOP])
{
    using RI = decltype(R.rb(0, 0));
    // j, k are stored indices (ghost rows / planes 0 and n+1 hold the periodic images).
    // The stencil is read undecoded (R.raw) and each face value scaled once
    // (R.dec_e): the interpolation is affine with weights summing to one, so for
    // the 16-bit deviation forms s (sum w d) is the face value less its rest
    // state w_p (the form the face flux takes); for FP64 / FP32 both are the
    // identity and the arithmetic is unchanged.
    const int jm = j - 1, jp = j + 1, jc = j;
    const int km = k - 1, kp = k + 1, kc = k;
    if (AX == 0) {
        const int A = i == 0 ? 1 : i, B = i == 0 ? 0 : i + 1;
        // the x weights depend on p only through cx(p): read them at the
        // representative population (1: cx>0, 2: cx<0, 3: cx=0), one load per class
        const T *xw = P.xw + i;
        const RI r00 = R.rb(jc, kc);
        v[0] = R.dec_e(0, T(0.5) * (R.raw(0, r00, A) + R.raw(0, r00, B)));
#pragma unroll
        for (int p = 1; p < NPOP; ++p) {
            const int ay = cy(p), az = cz(p);
            const int rp = xrep(p);
            const T om = __ldg(xw + (2 * rp) * P.xws), m = __ldg(xw + (2 * rp + 1) * P.xws);
            const int jt = ay > 0 ? jm : (ay < 0 ? jp : jc);
            const int kt = az > 0 ? km : (az < 0 ? kp : kc);
            const T x00 = lerp2(om, m, R.raw(p, r00, A), R.raw(p, r00, B));
            T y00 = x00;
            if (ay) {
                const RI r10 = R.rb(jt, kc);
                y00 = lerp2(P.ty_om, P.ty_m, x00, lerp2(om, m, R.raw(p, r10, A), R.raw(p, r10, B)));
            }
            if (az) {
                const RI r01 = R.rb(jc, kt);
                const T x10 = lerp2(om, m, R.raw(p, r01, A), R.raw(p, r01, B));
                T y11 = x10;
                if (ay) {
                    const RI r11 = R.rb(jt, kt);
                    y11 = lerp2(P.ty_om, P.ty_m, x10, lerp2(om, m, R.raw(p, r11, A), R.raw(p, r11, B)));
                }
                v[p] = R.dec_e(p, lerp2(P.tz_om, P.tz_m, y00, y11));
            } else {
                v[p] = R.dec_e(p, y00);
            }
        }
    } else if (AX == 1) {
        // rows j (anchor) and j+1 (other); transverse x to column i - cx, z to plane k - cz
        const RI rA = R.rb(jc, kc), rB = R.rb(jp, kc);
        v[0] = R.dec_e(0, T(0.5) * (R.raw(0, rA, i) + R.raw(0, rB, i)));
        const T *tw = P.txw + i;
#pragma unroll
        for (int p = 1; p < NPOP; ++p) {
            const int ax = cx(p), az = cz(p);
            const int io = i - ax;
            const int kt = az > 0 ? km : (az < 0 ? kp : kc);
            T txo = T(1), txm = T(0);
            if (ax) { txo = __ldg(tw + (2 * xrep(p)) * P.xws); txm = __ldg(tw + (2 * xrep(p) + 1) * P.xws); }
            T x00 = R.raw(p, rA, i), x01 = R.raw(p, rB, i);
            if (ax) {
                x00 = lerp2(txo, txm, x00, R.raw(p, rA, io));
                x01 = lerp2(txo, txm, x01, R.raw(p, rB, io));
            }
            const T y00 = lerp2(P.yn_om[p], P.yn_m[p], x00, x01);
            if (az) {
                const RI sA = R.rb(jc, kt), sB = R.rb(jp, kt);
                T x10 = R.raw(p, sA, i), x11 = R.raw(p, sB, i);
                if (ax) {
                    x10 = lerp2(txo, txm, x10, R.raw(p, sA, io));
                    x11 = lerp2(txo, txm, x11, R.raw(p, sB, io));
                }
                v[p] = R.dec_e(p, lerp2(P.tz_om, P.tz_m, y00, lerp2(P.yn_om[p], P.yn_m[p], x10, x11)));
            } else {
                v[p] = R.dec_e(p, y00);
            }
        }
    } else {
        // planes k (anchor) and k+1 (other); transverse x to i - cx, y to row j - cy
        const RI rA = R.rb(jc, kc), rB = R.rb(jc, kp);
        v[0] = R.dec_e(0, T(0.5) * (R.raw(0, rA, i) + R.raw(0, rB, i)));
        const T *tw = P.txw + i;
#pragma unroll
        for (int p = 1; p < NPOP; ++p) {
            const int ax = cx(p), ay = cy(p);
            const int io = i - ax;
            const int jt = ay > 0 ? jm : (ay < 0 ? jp : jc);
            T txo = T(1), txm = T(0);
            if (ax) { txo = __ldg(tw + (2 * xrep(p)) * P.xws); txm = __ldg(tw + (2 * xrep(p) + 1) * P.xws); }
            T x00 = R.raw(p, rA, i), x10 = R.raw(p, rB, i);
            if (ax) {
                x00 = lerp2(txo, txm, x00, R.raw(p, rA, io));
                x10 = lerp2(txo, txm, x10, R.raw(p, rB, io));
            }
            T y00 = x00, y11 = x10;
            if (ay) {
                const RI sA = R.rb(jt, kc), sB = R.rb(jt, kp);
                T x01 = R.raw(p, sA, i), x11 = R.raw(p, sB, i);
                if (ax) {
                    x01 = lerp2(txo, txm, x01, R.raw(p, sA, io));
                    x11 = lerp2(txo, txm, x11, R.raw(p, sB, io));
                }
                y00 = lerp2(P.ty_om, P.ty_m, x00, x01);
                y11 = lerp2(P.ty_om, P.ty_m, x10, x11);
            }
            v[p] = R.dec_e(p, lerp2(P.zn_om[p], P.zn_m[p], y00, y11));
        }
    }
}

// face_tri for the FP32 form on packed pairs (sm_100+ FMUL2/FFMA2): the 18
// moving populations of a face form nine pairs (p, q) with the same stencil
// shape -- the same rows, planes and lerps, weights of the same kind -- whose
// lerps run two per instruction, each half rounded as the scalar instruction.
// A lerp is m b + (om a) here (one rounding order of face_tri's om a + m b).
// Pairs per face orientation: first populations kPairP[AX], second kPairQ[AX];
// a mixed-class pair has its c_x > 0 population first.
__host__ __device__ constexpr int pair_p(int ax, int n)
{
    return ax == 0 ? (n == 0 ? 1 : n == 1 ? 3 : n == 2 ? 7 : n == 3 ? 9 : n == 4 ? 5 : n == 5 ? 11 : n == 6 ? 13 : n == 7 ? 15 : 17)
         : ax == 1 ? (n == 0 ? 3 : n == 1 ? 1 : n == 2 ? 7 : n == 3 ? 9 : n == 4 ? 5 : n == 5 ? 15 : n == 6 ? 17 : n == 7 ? 11 : 13)
                   : (n == 0 ? 5 : n == 1 ? 1 : n == 2 ? 11 : n == 3 ? 13 : n == 4 ? 3 : n == 5 ? 15 : n == 6 ? 17 : n == 7 ? 7 : 9);
}
__host__ __device__ constexpr int pair_q(int ax, int n) { return pair_p(ax, n) + 1; }

// The pairing rule, checked at compile time: per orientation every moving
// population once; the two of a pair with the same transverse lerps (c != 0
// on the same transverse axes) and x weights of one kind: both c_x = 0, or
// c_x > 0 first and c_x < 0 second (the packed x-weight pairs).
__host__ __device__ constexpr bool face_pairs_ok()
{
    for (int ax = 0; ax < 3; ++ax) {
        int seen = 0;
        for (int n = 0; n < 9; ++n) {
            const int p = pair_p(ax, n), q = pair_q(ax, n);
            if (p < 1 || q > 18) return false;
            seen |= (1 << p) | (1 << q);
            for (int t = 0; t < 3; ++t)
                if (t != ax && (cc(t, p) != 0) != (cc(t, q) != 0)) return false;
            const bool x_lerp = ax != 0 && cx(p) != 0;   // transverse x lerp (y, z faces)
            const bool x_face = ax == 0;                   // x-face normal weights by class
            if ((x_lerp || x_face) && !(cx(p) == 0 && cx(q) == 0) && !(cx(p) > 0 && cx(q) < 0)) return false;
        }
        if (seen != ((1 << 19) - 2)) return false;
    }
    return true;
}
static_assert(face_pairs_ok(), "face population pairs of face_tri_x2 must share their stencil shape");

__device__ __forceinline__ float2 lerp_x2(float2 om, float2 m, float2 a, float2 b)
{
    return __ffma2_rn(m, b, __fmul2_rn(om, a));
}

// b - a for a stored 16-bit value b and a float a, in one mixed-precision
// subtraction (sm_100+: the 16-bit operand is widened exactly inside the
// instruction, the difference rounded once to FP32).
__device__ __forceinline__ float sub_stored(__half b, float a)
{
    float d;
    asm("sub.rn.f32.f16 %0, %1, %2;" : "=f"(d) : "h"(__half_as_ushort(b)), "f"(a));
    return d;
}
__device__ __forceinline__ float sub_stored(__nv_bfloat16 b, float a)
{
    float d;
    asm("sub.rn.f32.bf16 %0, %1, %2;" : "=f"(d) : "h"(__bfloat16_as_ushort(b)), "f"(a));
    return d;
}

// First lerp of a stencil, between two stored values of each of the pair
// (a = (ap, aq) weighted om, b = (bp, bq) weighted m).  FP32: lerp_x2.  16-bit
// forms: a + m (b - a), a widened and b - a taken by sub_stored (three
// instructions per pair of values instead of four widenings and two packed
// products); this uses om = 1 - m, which the weight tables hold to the last
// bit of FP32.
template <class S>
__device__ __forceinline__ float2 lerp_first_x2(float2 om, float2 m, S ap, S aq, S bp, S bq)
{
    if constexpr (sizeof(S) == 2) {
        const float2 af = make_float2(float(ap), float(aq));
        return __ffma2_rn(m, make_float2(sub_stored(bp, af.x), sub_stored(bq, af.y)), af);
    } else {
        (void)om;
        return lerp_x2(om, m, make_float2(ap, aq), make_float2(bp, bq));
    }
}

template <class S, int AX, class RD>
__device__ __forceinline__ void face_tri_x2(const StepParams<float, S> &P, const RD &R, int i, int j, int k,
                                            float v[NPOP])
{
    using RI = decltype(R.rb(0, 0));
    const int jm = j - 1, jp = j + 1, jc = j;
    const int km = k - 1, kp = k + 1, kc = k;
    const int xs = P.xws;
    const float2 ty_o = make_float2(P.ty_om, P.ty_om), ty_m = make_float2(P.ty_m, P.ty_m);
    const float2 tz_o = make_float2(P.tz_om, P.tz_om), tz_m = make_float2(P.tz_m, P.tz_m);
    // first lerp of populations p, q between (row ra, column ca) and (row rb, column cb) of each
    auto L1 = [&](float2 om, float2 m, int p, int q, RI rap, int cap, RI raq, int caq, RI rbp, int cbp, RI rbq,
                  int cbq) {
        return lerp_first_x2<S>(om, m, R.bits(p, rap, cap), R.bits(q, raq, caq), R.bits(p, rbp, cbp),
                                R.bits(q, rbq, cbq));
    };
    if (AX == 0) {
        const int A = i == 0 ? 1 : i, B = i == 0 ? 0 : i + 1;
        const float *xw = P.xw + i;
        const float2 om12 = make_float2(__ldg(xw + 2 * xs), __ldg(xw + 4 * xs));
        const float2 m12 = make_float2(__ldg(xw + 3 * xs), __ldg(xw + 5 * xs));
        const float om3 = __ldg(xw + 6 * xs), m3 = __ldg(xw + 7 * xs);
        const float2 om33 = make_float2(om3, om3), m33 = make_float2(m3, m3);
        const RI r00 = R.rb(jc, kc);
        v[0] = R.dec_e(0, 0.5f * (R.raw(0, r00, A) + R.raw(0, r00, B)));
#pragma unroll
        for (int n = 0; n < 9; ++n) {
            const int p = pair_p(0, n), q = pair_q(0, n);
            const bool ay = cy(p) != 0, az = cz(p) != 0;
            const float2 om = xrep(p) == 3 ? om33 : om12, m = xrep(p) == 3 ? m33 : m12;
            const int jtp = cy(p) > 0 ? jm : (cy(p) < 0 ? jp : jc), jtq = cy(q) > 0 ? jm : (cy(q) < 0 ? jp : jc);
            const int ktp = cz(p) > 0 ? km : (cz(p) < 0 ? kp : kc), ktq = cz(q) > 0 ? km : (cz(q) < 0 ? kp : kc);
            const float2 x00 = L1(om, m, p, q, r00, A, r00, A, r00, B, r00, B);
            float2 y00 = x00;
            if (ay) {
                const RI sp = R.rb(jtp, kc), sq = R.rb(jtq, kc);
                const float2 x01 = L1(om, m, p, q, sp, A, sq, A, sp, B, sq, B);
                y00 = lerp_x2(ty_o, ty_m, x00, x01);
            }
            float2 res = y00;
            if (az) {
                const RI tp = R.rb(jc, ktp), tq = R.rb(jc, ktq);
                const float2 x10 = L1(om, m, p, q, tp, A, tq, A, tp, B, tq, B);
                float2 y11 = x10;
                if (ay) {
                    const RI up = R.rb(jtp, ktp), uq = R.rb(jtq, ktq);
                    const float2 x11 = L1(om, m, p, q, up, A, uq, A, up, B, uq, B);
                    y11 = lerp_x2(ty_o, ty_m, x10, x11);
                }
                res = lerp_x2(tz_o, tz_m, y00, y11);
            }
            const float2 e = R.dec_e2(p, q, res);
            v[p] = e.x;
            v[q] = e.y;
        }
    } else if (AX == 1) {
        // rows j (A) and j+1 (B); transverse x to column i - cx, z to plane k - cz
        const RI rA = R.rb(jc, kc), rB = R.rb(jp, kc);
        v[0] = R.dec_e(0, 0.5f * (R.raw(0, rA, i) + R.raw(0, rB, i)));
        const float *tw = P.txw + i;
        const float2 tx_o = make_float2(__ldg(tw + 2 * xs), __ldg(tw + 4 * xs));
        const float2 tx_m = make_float2(__ldg(tw + 3 * xs), __ldg(tw + 5 * xs));
#pragma unroll
        for (int n = 0; n < 9; ++n) {
            const int p = pair_p(1, n), q = pair_q(1, n);
            const bool ax = cx(p) != 0, az = cz(p) != 0;
            const int iop = i - cx(p), ioq = i - cx(q);
            const int ktp = cz(p) > 0 ? km : (cz(p) < 0 ? kp : kc), ktq = cz(q) > 0 ? km : (cz(q) < 0 ? kp : kc);
            const float2 yo = make_float2(P.yn_om[p], P.yn_om[q]), ym = make_float2(P.yn_m[p], P.yn_m[q]);
            // normal lerp between rows A and B of the values at column i, x-lerped first when c_x != 0
            auto yl = [&](RI sAp, RI sAq, RI sBp, RI sBq) {
                if (ax) {
                    const float2 x0 = L1(tx_o, tx_m, p, q, sAp, i, sAq, i, sAp, iop, sAq, ioq);
                    const float2 x1 = L1(tx_o, tx_m, p, q, sBp, i, sBq, i, sBp, iop, sBq, ioq);
                    return lerp_x2(yo, ym, x0, x1);
                }
                return L1(yo, ym, p, q, sAp, i, sAq, i, sBp, i, sBq, i);
            };
            const float2 y00 = yl(rA, rA, rB, rB);
            float2 res = y00;
            if (az) {
                const RI sAp = R.rb(jc, ktp), sBp = R.rb(jp, ktp), sAq = R.rb(jc, ktq), sBq = R.rb(jp, ktq);
                res = lerp_x2(tz_o, tz_m, y00, yl(sAp, sAq, sBp, sBq));
            }
            const float2 e = R.dec_e2(p, q, res);
            v[p] = e.x;
            v[q] = e.y;
        }
    } else {
        // planes k (A) and k+1 (B); transverse x to column i - cx, y to row j - cy
        const RI rA = R.rb(jc, kc), rB = R.rb(jc, kp);
        v[0] = R.dec_e(0, 0.5f * (R.raw(0, rA, i) + R.raw(0, rB, i)));
        const float *tw = P.txw + i;
        const float2 tx_o = make_float2(__ldg(tw + 2 * xs), __ldg(tw + 4 * xs));
        const float2 tx_m = make_float2(__ldg(tw + 3 * xs), __ldg(tw + 5 * xs));
#pragma unroll
        for (int n = 0; n < 9; ++n) {
            const int p = pair_p(2, n), q = pair_q(2, n);
            const bool ax = cx(p) != 0, ay = cy(p) != 0;
            const int iop = i - cx(p), ioq = i - cx(q);
            const int jtp = cy(p) > 0 ? jm : (cy(p) < 0 ? jp : jc), jtq = cy(q) > 0 ? jm : (cy(q) < 0 ? jp : jc);
            const float2 zo = make_float2(P.zn_om[p], P.zn_om[q]), zm = make_float2(P.zn_m[p], P.zn_m[q]);
            // value at column i of rows sp / sq, x-lerped when c_x != 0 (first lerps)
            auto xl = [&](RI sp, RI sq) {
                return L1(tx_o, tx_m, p, q, sp, i, sq, i, sp, iop, sq, ioq);
            };
            float2 res;
            if (!ax && !ay) {
                res = L1(zo, zm, p, q, rA, i, rA, i, rB, i, rB, i);
            } else {
                float2 y00, y11;
                if (ay) {
                    const RI sAp = R.rb(jtp, kc), sBp = R.rb(jtp, kp), sAq = R.rb(jtq, kc), sBq = R.rb(jtq, kp);
                    if (ax) {
                        y00 = lerp_x2(ty_o, ty_m, xl(rA, rA), xl(sAp, sAq));
                        y11 = lerp_x2(ty_o, ty_m, xl(rB, rB), xl(sBp, sBq));
                    } else {
                        y00 = L1(ty_o, ty_m, p, q, rA, i, rA, i, sAp, i, sAq, i);
                        y11 = L1(ty_o, ty_m, p, q, rB, i, rB, i, sBp, i, sBq, i);
                    }
                } else {
                    y00 = xl(rA, rA);
                    y11 = xl(rB, rB);
                }
                res = lerp_x2(zo, zm, y00, y11);
            }
            const float2 e = R.dec_e2(p, q, res);
            v[p] = e.x;
            v[q] = e.y;
        }
    }
}

// Corner-weight form of face_tri for the FP64 step, whose throughput is set by
// the FP64 instruction count: each face value is sum_q w_q f_q over its 2, 4
// or 8 stencil points (one multiply and FMAs) instead of the nested lerps
// (two operations per lerp: 6 for a bilinear, 14 for a trilinear value).  The
// weights are the products of the lerp weights, from the corner-weight table
// P.cw (rows of the CW_* layout, column-dependent through the x weights) and,
// where no x weight enters, from the uniform products in P.ycw / P.zcw.  Same
// stencil points and weights as face_tri; the sums differ only by rounding.
template <class T, class S, int AX, class RD>
__device__ __forceinline__ void face_tri_cw(const StepParams<T, S> &P, const RD &R, int i, int j, int k, T v[NPOP])
{
    using RI = decltype(R.rb(0, 0));
    const int jm = j - 1, jp = j + 1, jc = j;
    const int km = k - 1, kp = k + 1, kc = k;
    const int xs = P.xws;
    const T *cw = P.cw + i;
    if (AX == 0) {
        const int A = i == 0 ? 1 : i, B = i == 0 ? 0 : i + 1;
        const T *xw = P.xw + i;
        const RI r00 = R.rb(jc, kc);
        v[0] = R.dec_e(0, T(0.5) * (R.raw(0, r00, A) + R.raw(0, r00, B)));
#pragma unroll
        for (int p = 1; p < NPOP; ++p) {
            const int ay = cy(p), az = cz(p), c = xrep(p);
            const int jt = ay > 0 ? jm : (ay < 0 ? jp : jc);
            const int kt = az > 0 ? km : (az < 0 ? kp : kc);
            T t;
            if (!ay && !az) {
                t = lerp2(__ldg(xw + (2 * c) * xs), __ldg(xw + (2 * c + 1) * xs), R.raw(p, r00, A), R.raw(p, r00, B));
            } else if (!az) {
                const RI r10 = R.rb(jt, kc);
                const T *w = cw + (CW_XY + 4 * (c - 1)) * xs;
                t = __ldg(w) * R.raw(p, r00, A);
                t = fma(__ldg(w + xs), R.raw(p, r00, B), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, r10, A), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, r10, B), t);
            } else if (!ay) {
                const RI r01 = R.rb(jc, kt);
                const T *w = cw + (CW_XZ + 4 * (c - 1)) * xs;
                t = __ldg(w) * R.raw(p, r00, A);
                t = fma(__ldg(w + xs), R.raw(p, r00, B), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, r01, A), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, r01, B), t);
            } else {
                const RI r10 = R.rb(jt, kc), r01 = R.rb(jc, kt), r11 = R.rb(jt, kt);
                const T *w = cw + CW_XYZ * xs;
                t = __ldg(w) * R.raw(p, r00, A);
                t = fma(__ldg(w + xs), R.raw(p, r00, B), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, r10, A), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, r10, B), t);
                t = fma(__ldg(w + 4 * xs), R.raw(p, r01, A), t);
                t = fma(__ldg(w + 5 * xs), R.raw(p, r01, B), t);
                t = fma(__ldg(w + 6 * xs), R.raw(p, r11, A), t);
                t = fma(__ldg(w + 7 * xs), R.raw(p, r11, B), t);
            }
            v[p] = R.dec_e(p, t);
        }
    } else if (AX == 1) {
        // rows j (A) and j+1 (B); transverse x to column i - cx, z to plane k - cz
        const RI rA = R.rb(jc, kc), rB = R.rb(jp, kc);
        v[0] = R.dec_e(0, T(0.5) * (R.raw(0, rA, i) + R.raw(0, rB, i)));
#pragma unroll
        for (int p = 1; p < NPOP; ++p) {
            const int ax = cx(p), az = cz(p), c = xrep(p);
            const int io = i - ax;
            const int kt = az > 0 ? km : (az < 0 ? kp : kc);
            T t;
            if (!ax && !az) {
                t = lerp2(P.yn_om[p], P.yn_m[p], R.raw(p, rA, i), R.raw(p, rB, i));
            } else if (!az) {
                const T *w = cw + (CW_Y4 + 4 * slot4y(p)) * xs;
                t = __ldg(w) * R.raw(p, rA, i);
                t = fma(__ldg(w + xs), R.raw(p, rA, io), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, rB, i), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, rB, io), t);
            } else if (!ax) {
                const RI sA = R.rb(jc, kt), sB = R.rb(jp, kt);
                t = P.ycw[p][0] * R.raw(p, rA, i);
                t = fma(P.ycw[p][1], R.raw(p, rB, i), t);
                t = fma(P.ycw[p][2], R.raw(p, sA, i), t);
                t = fma(P.ycw[p][3], R.raw(p, sB, i), t);
            } else {
                const RI sA = R.rb(jc, kt), sB = R.rb(jp, kt);
                const T *w = cw + (CW_Y8 + 8 * (c - 1)) * xs;
                t = __ldg(w) * R.raw(p, rA, i);
                t = fma(__ldg(w + xs), R.raw(p, rA, io), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, rB, i), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, rB, io), t);
                t = fma(__ldg(w + 4 * xs), R.raw(p, sA, i), t);
                t = fma(__ldg(w + 5 * xs), R.raw(p, sA, io), t);
                t = fma(__ldg(w + 6 * xs), R.raw(p, sB, i), t);
                t = fma(__ldg(w + 7 * xs), R.raw(p, sB, io), t);
            }
            v[p] = R.dec_e(p, t);
        }
    } else {
        // planes k (A) and k+1 (B); transverse x to column i - cx, y to row j - cy
        const RI rA = R.rb(jc, kc), rB = R.rb(jc, kp);
        v[0] = R.dec_e(0, T(0.5) * (R.raw(0, rA, i) + R.raw(0, rB, i)));
#pragma unroll
        for (int p = 1; p < NPOP; ++p) {
            const int ax = cx(p), ay = cy(p), c = xrep(p);
            const int io = i - ax;
            const int jt = ay > 0 ? jm : (ay < 0 ? jp : jc);
            T t;
            if (!ax && !ay) {
                t = lerp2(P.zn_om[p], P.zn_m[p], R.raw(p, rA, i), R.raw(p, rB, i));
            } else if (!ay) {
                const T *w = cw + (CW_Z4 + 4 * slot4z(p)) * xs;
                t = __ldg(w) * R.raw(p, rA, i);
                t = fma(__ldg(w + xs), R.raw(p, rA, io), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, rB, i), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, rB, io), t);
            } else if (!ax) {
                const RI sA = R.rb(jt, kc), sB = R.rb(jt, kp);
                t = P.zcw[p][0] * R.raw(p, rA, i);
                t = fma(P.zcw[p][1], R.raw(p, sA, i), t);
                t = fma(P.zcw[p][2], R.raw(p, rB, i), t);
                t = fma(P.zcw[p][3], R.raw(p, sB, i), t);
            } else {
                const RI sA = R.rb(jt, kc), sB = R.rb(jt, kp);
                const T *w = cw + (CW_Z8 + 8 * (c - 1)) * xs;
                t = __ldg(w) * R.raw(p, rA, i);
                t = fma(__ldg(w + xs), R.raw(p, rA, io), t);
                t = fma(__ldg(w + 2 * xs), R.raw(p, sA, i), t);
                t = fma(__ldg(w + 3 * xs), R.raw(p, sA, io), t);
                t = fma(__ldg(w + 4 * xs), R.raw(p, rB, i), t);
                t = fma(__ldg(w + 5 * xs), R.raw(p, rB, io), t);
                t = fma(__ldg(w + 6 * xs), R.raw(p, sB, i), t);
                t = fma(__ldg(w + 7 * xs), R.raw(p, sB, io), t);
            }
            v[p] = R.dec_e(p, t);
        }
    }
}

// 19 face values of the central-difference ("gradient") reconstruction,
// f_face = mean - hdt (c . grad), src/dugks.cu:459-583 (calc_fx): normal
// gradient across the face, transverse gradients of face-averaged neighbours
// over two cells.  Uniform mesh.
template <class T, class S, int AX, class RD>
__device__ __forceinline__ void face_grad(const StepParams<T, S> &P, const RD &R, int i, int j, int k, T v[NPOP])
{
    using RI = decltype(R.rb(0, 0));
    const int jm = j - 1, jp = j + 1, jc = j;
    const int km = k - 1, kp = k + 1, kc = k;
    const T h = P.hdt;
#pragma unroll
    for (int p = 0; p < NPOP; ++p) {
        T temp, gx, gy, gz;
        if (AX == 0) {
            const int L = i, Rr = i + 1;  // left / right column of face I = i
            const RI r = R.rb(jc, kc);
            const T a = R(p, r, Rr), b = R(p, r, L);
            const RI ru = R.rb(jp, kc), rd = R.rb(jm, kc);
            const RI rt = R.rb(jc, kp), rbo = R.rb(jc, km);
            if (P.grad_st) {
                // stretched x mesh: values interpolated to the face, normal difference over the centre spacing
                const T lam = __ldg(P.gw + GW_LAM * P.xws + i), idx = __ldg(P.gw + GW_IDX * P.xws + i);
                temp = fma(lam, a - b, b);
                gx = (a - b) * idx;
                const T bu = R(p, ru, L), bd = R(p, rd, L), bt = R(p, rt, L), bb = R(p, rbo, L);
                gy = (fma(lam, R(p, ru, Rr) - bu, bu) - fma(lam, R(p, rd, Rr) - bd, bd)) * P.g_i2dy;
                gz = (fma(lam, R(p, rt, Rr) - bt, bt) - fma(lam, R(p, rbo, Rr) - bb, bb)) * P.g_i2dz;
            } else {
                temp = T(0.5) * (a + b);
                gx = (a - b) * P.g_idx;
                gy = (T(0.5) * (R(p, ru, L) + R(p, ru, Rr)) - T(0.5) * (R(p, rd, L) + R(p, rd, Rr))) * P.g_i2dy;
                gz = (T(0.5) * (R(p, rt, L) + R(p, rt, Rr)) - T(0.5) * (R(p, rbo, L) + R(p, rbo, Rr))) * P.g_i2dz;
            }
        } else if (AX == 1) {
            const RI rD = R.rb(jc, kc), rU = R.rb(jp, kc);
            const T a = R(p, rU, i), b = R(p, rD, i);
            temp = T(0.5) * (a + b);
            if (P.grad_st) {
                // three-point x derivative of the face averages on the non-uniform centres
                gx = __ldg(P.gw + GW_WM * P.xws + i) * (T(0.5) * (R(p, rD, i - 1) + R(p, rU, i - 1)));
                gx = fma(__ldg(P.gw + GW_W0 * P.xws + i), temp, gx);
                gx = fma(__ldg(P.gw + GW_WP * P.xws + i), T(0.5) * (R(p, rD, i + 1) + R(p, rU, i + 1)), gx);
            } else {
                gx = (T(0.5) * (R(p, rD, i + 1) + R(p, rU, i + 1)) - T(0.5) * (R(p, rD, i - 1) + R(p, rU, i - 1))) * P.g_i2dx;
            }
            gy = (a - b) * P.g_idy;
            const RI tD = R.rb(jc, kp), tU = R.rb(jp, kp), bD = R.rb(jc, km), bU = R.rb(jp, km);
            gz = (T(0.5) * (R(p, tD, i) + R(p, tU, i)) - T(0.5) * (R(p, bD, i) + R(p, bU, i))) * P.g_i2dz;
        } else {
            const RI rB = R.rb(jc, kc), rT = R.rb(jc, kp);
            const T a = R(p, rT, i), b = R(p, rB, i);
            temp = T(0.5) * (a + b);
            if (P.grad_st) {
                gx = __ldg(P.gw + GW_WM * P.xws + i) * (T(0.5) * (R(p, rB, i - 1) + R(p, rT, i - 1)));
                gx = fma(__ldg(P.gw + GW_W0 * P.xws + i), temp, gx);
                gx = fma(__ldg(P.gw + GW_WP * P.xws + i), T(0.5) * (R(p, rB, i + 1) + R(p, rT, i + 1)), gx);
            } else {
                gx = (T(0.5) * (R(p, rB, i + 1) + R(p, rT, i + 1)) - T(0.5) * (R(p, rB, i - 1) + R(p, rT, i - 1))) * P.g_i2dx;
            }
            const RI uB = R.rb(jp, kc), uT = R.rb(jp, kp), dB = R.rb(jm, kc), dT = R.rb(jm, kp);
            gy = (T(0.5) * (R(p, uB, i) + R(p, uT, i)) - T(0.5) * (R(p, dB, i) + R(p, dT, i))) * P.g_i2dy;
            gz = (a - b) * P.g_idz;
        }
        T s = T(0);
        if (cx(p)) s += cx(p) > 0 ? gx : -gx;
        if (cy(p)) s += cy(p) > 0 ? gy : -gy;
        if (cz(p)) s += cz(p) > 0 ? gz : -gz;
        v[p] = p == 0 ? temp : temp - h * s;
    }
}

// Face equilibrium and flux (src/dugks.cu:675-709 f2ruvwh, 912-943):
//   F_p = fw1 v_p + (fw2 + fw0 F.(c_p - u)/RT) feq_p(rho, u + hdt/2 F)
// for the 10 populations crossing a face normal to AX.  Stored divided by fw1
// (out_s = F_p / fw1, one FMA each); the update multiplies the flux
// differences by fw1 dt/dx instead.
template <class T, class S, int AX, bool FF>
__device__ __forceinline__ void face_flux(const StepParams<T, S> &P, const T v[NPOP], T out[10], T fadd)
{
    T r, jx, jy, jz;
    if constexpr (std::is_same<T, float>::value)
        moments_x2(v, r, jx, jy, jz);
    else
        moments(v, r, jx, jy, jz);
    // 16-bit forms: v holds f_p - w_p; the rest state adds sum w_p = 1 to the
    // density and nothing to the momentum, and out carries F_p - w_p, which the
    // update only differences between the two faces of a cell
    if constexpr (Codec<T, S>::deviation) r += T(1);
    const T inv = recip(r);
    T u = jx * inv, vv = jy * inv, w = jz * inv;
    T B = P.fw2s;
    T Ff[3] = {P.F[0], P.F[1], P.F[2]};
    if (FF) {
        // face force with the field: shift (hdt/2) F_face
        Ff[0] += P.ffaxis == 0 ? fadd : T(0);  // selects: no dynamically indexed local array
        Ff[1] += P.ffaxis == 1 ? fadd : T(0);
        Ff[2] += P.ffaxis == 2 ? fadd : T(0);
        const T hh = T(0.5) * P.hdt;
        u = fma(hh, Ff[0], u);
        vv = fma(hh, Ff[1], vv);
        w = fma(hh, Ff[2], w);
        B = fma(-P.fw0x3s, fma(Ff[0], u, fma(Ff[1], vv, Ff[2] * w)), P.fw2s);
    } else if (Fp64Form<T>::value && P.force_on && P.fax >= 0) {
        // one force component: the same values from that component alone
        const int a = P.fax;
        const T ua = (a == 0 ? u : (a == 1 ? vv : w)) + P.hFa;
        u = a == 0 ? ua : u;
        vv = a == 1 ? ua : vv;
        w = a == 2 ? ua : w;
        B = fma(-P.fw0x3s, P.Fa * ua, P.fw2s);
    } else if (P.force_on) {
        u += P.hF[0];
        vv += P.hF[1];
        w += P.hF[2];
        B = fma(-P.fw0x3s, fma(Ff[0], u, fma(Ff[1], vv, Ff[2] * w)), P.fw2s);
    }
    const T u3 = T(3) * u, v3 = T(3) * vv, w3 = T(3) * w;
    const T base = fma(T(-1.5), fma(u, u, fma(vv, vv, w * w)), T(1));
    const T wr1 = weight<T>(1) * r, wr2 = weight<T>(7) * r;
    T fe[NPOP];
    if (AX == 0) {
        feq_pair(u3, base, wr1, fe[1], fe[2]);
    } else if (AX == 1) {
        feq_pair(v3, base, wr1, fe[3], fe[4]);
    } else {
        feq_pair(w3, base, wr1, fe[5], fe[6]);
    }
    if (AX != 2) {
        feq_pair(u3 + v3, base, wr2, fe[7], fe[10]);
        feq_pair(v3 - u3, base, wr2, fe[8], fe[9]);
    }
    if (AX != 1) {
        feq_pair(u3 + w3, base, wr2, fe[11], fe[14]);
        feq_pair(w3 - u3, base, wr2, fe[12], fe[13]);
    }
    if (AX != 0) {
        feq_pair(v3 + w3, base, wr2, fe[15], fe[18]);
        feq_pair(w3 - v3, base, wr2, fe[16], fe[17]);
    }
    if (Fp64Form<T>::value && !FF && P.fax >= 0) {
        // B + K_p takes three values: B, B + Kfa, B - Kfa
        const T Bp = B + P.Kfa, Bm = B - P.Kfa;
        const int a = P.fax;
#pragma unroll
        for (int s = 0; s < 10; ++s) {
            const int p = flux_pop(AX, s);
            const int ca = a == 0 ? cx(p) : (a == 1 ? cy(p) : cz(p));
            out[s] = fma(ca > 0 ? Bp : (ca < 0 ? Bm : B), fe[p], v[p]);
        }
        return;
    }
    auto coef = [&](int p) {
        T K = P.Kfs[p];
        if (FF) {
            const int ca = P.ffaxis == 0 ? cx(p) : (P.ffaxis == 1 ? cy(p) : cz(p));
            if (ca) K = fma(ca > 0 ? P.fw0x3s : -P.fw0x3s, fadd, K);
        }
        return K;
    };
    if constexpr (std::is_same<T, float>::value) {
        // slots (2t, 2t+1) hold the pair (2m-1, 2m): the same operations two at a time
        const float2 B2 = make_float2(B, B);
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            const int p = flux_pop(AX, 2 * t), q = flux_pop(AX, 2 * t + 1);
            const float2 o = __ffma2_rn(__fadd2_rn(B2, make_float2(coef(p), coef(q))), make_float2(fe[p], fe[q]),
                                        make_float2(v[p], v[q]));
            out[2 * t] = o.x;
            out[2 * t + 1] = o.y;
        }
    } else {
#pragma unroll
        for (int s = 0; s < 10; ++s) {
            const int p = flux_pop(AX, s);
            out[s] = fma(B + coef(p), fe[p], v[p]);
        }
    }
}

// Force-field contribution on a face: the mean of phi over the two cells
// across the face (one cell on a wall face).  i, j, k: the face's stored
// indices as passed to face_fluxes.
template <class T, class S, int AX>
__device__ __forceinline__ T face_field(const StepParams<T, S> &P, int i, int j, int k)
{
    if (!P.ffield) return T(0);
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    auto wr1 = [](int a, int n) { return a < 1 ? a + n : (a > n ? a - n : a); };
    int i1 = i, i2 = i, j1 = wr1(j, ny), j2 = j1, k1 = wr1(k, nz), k2 = k1;
    if (AX == 0) {
        i1 = i == 0 ? (P.periodic_x ? nx : 1) : i;
        i2 = i + 1 <= nx ? i + 1 : (P.periodic_x ? 1 : nx);
    } else if (AX == 1) {
        j2 = wr1(j + 1, ny);
    } else {
        k2 = wr1(k + 1, nz);
    }
    const T a = __ldg(P.ffield + ((long long)(k1 - 1) * ny + (j1 - 1)) * P.pitch + (i1 - 1));
    const T b = __ldg(P.ffield + ((long long)(k2 - 1) * ny + (j2 - 1)) * P.pitch + (i2 - 1));
    return T(0.5) * (a + b);
}

// Bounce-back on the wall faces (src/dugks.cu:807-823): the populations
// entering the fluid take the value of their opposites on the same face.
template <class T>
__device__ __forceinline__ void bounce_back(T v[NPOP], bool lo, bool hi)
{
    if (lo) {
        v[1] = v[2]; v[7] = v[10]; v[9] = v[8]; v[11] = v[14]; v[13] = v[12];
    }
    if (hi) {
        v[2] = v[1]; v[10] = v[7]; v[8] = v[9]; v[14] = v[11]; v[12] = v[13];
    }
}

// Fluxes of one face: reconstruction + bounce-back + face equilibrium.
template <class T, class S, int AX, int RECON, bool FF, class RD>
__device__ __forceinline__ void face_fluxes(const StepParams<T, S> &P, const RD &R, int i, int j, int k, T out[10])
{
    T v[NPOP];
    if constexpr (RECON == 0 && Fp64Form<T>::value)
        face_tri_cw<T, S, AX>(P, R, i, j, k, v);
    else if constexpr (RECON == 0 && std::is_same<T, float>::value)
        face_tri_x2<S, AX>(P, R, i, j, k, v);  // packed lerps: FP32, FP16, BF16
    else if constexpr (RECON == 0)
        face_tri<T, S, AX>(P, R, i, j, k, v);
    else
        face_grad<T, S, AX>(P, R, i, j, k, v);
    if constexpr (RECON != 0 && Codec<T, S>::deviation) {
        // the face values less their rest state, as the interpolating forms give them
#pragma unroll
        for (int p = 0; p < NPOP; ++p) v[p] -= P.codec.w[p];
    }
    if (AX == 0 && !P.periodic_x) bounce_back(v, i == 0, i == P.nx);
    face_flux<T, S, AX, FF>(P, v, out, FF ? face_field<T, S, AX>(P, i, j, k) : T(0));
}

template <class T, class S, int W, int RECON, int MINB, bool FF>
__global__ void __launch_bounds__(32 * W, MINB) flux_kernel(const S *__restrict__ fb, const S *f_in, S *f_out,
                                                       const StepParams<T, S> P, int kchunk)
{
    static_assert(4 * (W - 1) <= 32, "the halo warp evaluates 4 planes x (W-1) rows of -x faces at once");
    __shared__ T ysh[2][W][10][32];  // +y face fluxes of every warp row (double buffer)
    __shared__ T xsh[2][4][W][10];   // -x face fluxes of the first column: [batch parity][plane of batch][row]
    const int lane = threadIdx.x, wr = threadIdx.y;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int i0 = blockIdx.x * 32 + 1;           // first column of the tile (1-based)
    const int j0 = blockIdx.y * (W - 1) + 1;      // first row of the tile (1-based)
    const int kb = blockIdx.z * kchunk + 1;
    const int ke = min(kb + kchunk, nz + 1);
    const FbRead<T, S> R{fb, P.ps_b, P.pitch_b, ny, nz, P.codec};

    // warps 1..W-1: cell (gi, gj); warp 0: halo
    const int gi = i0 + lane;
    const int gj = j0 + wr - 1;
    const bool cell = wr >= 1 && gi <= nx && gj <= ny;
    const int ci = min(gi, nx);                     // clamped column for unused lanes
    const int cj = wr >= 1 ? min(gj, ny) : 1;
    // warp 0 tasks: y face J = j0-1 at column gi every plane; every fourth plane the -x faces
    // of the first column for the next four planes, lane = q (W-1) + r -> plane +q, row j0+r
    // (28 of 32 lanes busy, instead of W-1 lanes every plane)
    const int hq = lane / (W - 1), hr = lane - hq * (W - 1);
    const int hj = j0 + hr;                         // halo x-face row
    const bool hx = wr == 0 && hq < 4 && hj <= ny;

    T fzd[10], fzu[10], fx[10], fy[10];
    int buf = 0;
    if (kb >= ke) return;
    if (wr >= 1) face_fluxes<T, S, 2, RECON, FF>(P, R, ci, cj, kb - 1, fzd);  // z face kb-1/2
    for (int k = kb; k < ke; ++k) {
        const int bq = (k - kb) & 3, bp = ((k - kb) >> 2) & 1;  // plane within its batch of four, batch parity
        if (wr >= 1) {
            face_fluxes<T, S, 0, RECON, FF>(P, R, ci, cj, k, fx);   // +x face I = gi
            face_fluxes<T, S, 1, RECON, FF>(P, R, ci, cj, k, fy);   // +y face J = gj
            face_fluxes<T, S, 2, RECON, FF>(P, R, ci, cj, k, fzu);  // +z face k+1/2
#pragma unroll
            for (int s = 0; s < 10; ++s) ysh[buf][wr][s][lane] = fy[s];
        } else {
            face_fluxes<T, S, 1, RECON, FF>(P, R, ci, j0 - 1, k, fy);  // y face J = j0-1 (may be 0: periodic image)
#pragma unroll
            for (int s = 0; s < 10; ++s) ysh[buf][0][s][lane] = fy[s];
            // the batch's slots were last read before the barrier of the plane 4 back
            if (bq == 0 && hx && k + hq < ke) {
                T hxf[10];
                face_fluxes<T, S, 0, RECON, FF>(P, R, i0 - 1, hj, k + hq, hxf);  // x face I = i0-1, row hj
#pragma unroll
                for (int s = 0; s < 10; ++s) xsh[bp][hq][hr + 1][s] = hxf[s];
            }
        }
        __syncthreads();
        if (wr >= 1) {
            T fxl[10];
#pragma unroll
            for (int s = 0; s < 10; ++s) {
                const T up = __shfl_up_sync(0xffffffffu, fx[s], 1);
                fxl[s] = lane == 0 ? xsh[bp][bq][wr][s] : up;
            }
            if (cell) {
                const long long c = ((long long)(k - 1) * ny + (gj - 1)) * P.pitch + (gi - 1);
                const unsigned hc = P.codec.cell_hash(c);
                const long long cb = R.rb(gj, k) + gi;
                const T cxg = __ldg(P.cxuf + gi);
                const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0);
#pragma unroll
                for (int p = 0; p < NPOP; ++p) {
                    UpdateSum<T, S> u(upd_base(R.raw(p, cb, 0), P.codec.raw(f_in, p * P.ps + c), c43, c13));
                    if (cx(p)) {
                        const int s = flux_slot(0, p);
                        u.add(cx(p) > 0 ? -cxg : cxg, fx[s] - fxl[s]);
                    }
                    if (cy(p)) {
                        const int s = flux_slot(1, p);
                        u.add(cy(p) > 0 ? -P.cyuf : P.cyuf, fy[s] - ysh[buf][wr - 1][s][lane]);
                    }
                    if (cz(p)) {
                        const int s = flux_slot(2, p);
                        u.add(cz(p) > 0 ? -P.czuf : P.czuf, fzu[s] - fzd[s]);
                    }
                    f_out[p * P.ps + c] = u.encode(P.codec, p, hc);
                }
            }
#pragma unroll
            for (int s = 0; s < 10; ++s) fzd[s] = fzu[s];
        }
        buf ^= 1;
    }
}

// ---------------------------------------------------------------------------
// TMA-fed variant of flux_kernel.  The CTA's window of f-bar-plus -- columns
// i0-1 .. i0+32, rows j0-1 .. j0+W-1, all 19 populations of one plane -- is
// one 4-D tile of the ghosted f-bar-plus tensor (x, y, z, population); it
// arrives in a 4-stage shared-memory ring through cp.async.bulk.tensor with
// mbarrier completion, two planes ahead of use.  The faces read the ring
// instead of global memory; everything else is flux_kernel.
// ---------------------------------------------------------------------------
template <class S>
struct TmaTile {
    // tile width in elements: >= 34 columns, row bytes a multiple of 16
    static constexpr int BXT = sizeof(S) == 8 ? 34 : (sizeof(S) == 4 ? 36 : 40);
};

template <class T, class S, int W>
struct SmemRead {
    static constexpr int BXT = TmaTile<S>::BXT, RH = W + 1, POPS = BXT * RH;
    static constexpr int STAGE_BYTES = ((NPOP * POPS * int(sizeof(S))) + 127) / 128 * 128;
    static constexpr int STAGE = STAGE_BYTES / int(sizeof(S));
    const S *ring;
    int i0m1, j0m1;
    const Codec<T, S> &codec;
    __device__ __forceinline__ int rb(int j, int k) const { return (k & 3) * STAGE + (j - j0m1) * BXT - i0m1; }
    __device__ __forceinline__ T operator()(int p, int row, int col) const
    {
        return codec.load_s(ring, p * POPS + row + col, p);
    }
    __device__ __forceinline__ T raw(int p, int row, int col) const { return codec.raw_s(ring, p * POPS + row + col); }
    __device__ __forceinline__ S bits(int p, int row, int col) const { return ring[p * POPS + row + col]; }
    __device__ __forceinline__ T dec(int p, T x) const { return codec.dec(p, x); }
    __device__ __forceinline__ T dec_e(int p, T x) const { return codec.dec_e(p, x); }
    __device__ __forceinline__ float2 dec_e2(int p, int q, float2 x) const { return codec.dec_e2(p, q, x); }
};

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Polls of a bounded pipeline wait before it gives up.  A try_wait on a phase
// that does not complete suspends the thread for a few microseconds before it
// reports (about 7,800 SM cycles per poll measured on GB300), so 2^18 polls
// last about a second, far beyond any legitimate wait for one TMA plane.
// After a first time-out a CTA waits only kWaitPollsAfterFailure polls, so
// that a failed pipeline finishes quickly instead of waiting out every plane.
constexpr int kWaitPolls = 1 << 18;
constexpr int kWaitPollsAfterFailure = 64;

// bounded wait on an mbarrier phase; false if it did not complete within
// `limit` polls
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit = kWaitPolls)
{
    for (int it = 0; it < limit; ++it) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

template <class T, class S, int W, int RECON, int MINB, bool FF>
__global__ void __launch_bounds__(32 * W, MINB) flux_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                 const S *f_in, S *f_out,
                                                                 const StepParams<T, S> P, int kchunk)
{
    using RD = SmemRead<T, S, W>;
    extern __shared__ __align__(128) unsigned char smem[];
    S *ring = reinterpret_cast<S *>(smem);
    T(*ysh)[W][10][32] = reinterpret_cast<T(*)[W][10][32]>(smem + 4 * RD::STAGE_BYTES);
    T(*xsh)[W][10] = reinterpret_cast<T(*)[W][10]>(smem + 4 * RD::STAGE_BYTES + 2 * W * 10 * 32 * sizeof(T));
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(
        smem + 4 * RD::STAGE_BYTES + 2 * W * 10 * 32 * sizeof(T) + 2 * W * 10 * sizeof(T));
    constexpr unsigned TILE_BYTES = unsigned(NPOP * RD::POPS * sizeof(S));

    const int lane = threadIdx.x, wr = threadIdx.y, tid = wr * 32 + lane;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int i0 = blockIdx.x * 32 + 1;
    const int j0 = blockIdx.y * (W - 1) + 1;
    const int kb = blockIdx.z * kchunk + 1;
    const int ke = min(kb + kchunk, nz + 1);
    if (kb >= ke) return;
    const RD R{ring, i0 - 1, j0 - 1, P.codec};

    if (tid == 0) {
        for (int s = 0; s < 4; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar + s)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int g) {  // stored plane g -> stage g & 3
        if (tid == 0 && g <= ke) {
            const unsigned bar = smem_u32(mbar + (g & 3));
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(TILE_BYTES)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(ring + (g & 3) * RD::STAGE)),
                "l"(reinterpret_cast<unsigned long long>(&tmap)), "r"(i0 - 1), "r"(j0 - 1), "r"(g), "r"(0), "r"(bar)
                : "memory");
        }
    };
    unsigned phase = 0;  // bit s: parity of the next completion of stage s
    int wait_limit = kWaitPolls;
    auto wait = [&](int g) {
        const int s = g & 3;
        if (!mbar_wait(smem_u32(mbar + s), (phase >> s) & 1u, wait_limit)) {
            atomicOr(P.err, 1);
            wait_limit = kWaitPollsAfterFailure;
        }
        phase ^= 1u << s;
    };

    // 16-bit forms between walls: the wall ghost columns 0 and nx+1 of f-bar-plus
    // are not stored (stage (a) writes the interior and its y / z images only);
    // the tiles that read them form
    // them in shared memory from the landed plane, g0 = q0 d(1) + (1-q0) d(2),
    // g_{nx+1} = q1 d(nx) + (1-q1) d(nx-1) (src/dugks.cu:1234-1251; stretched
    // mesh src/fortran/channel/src/dugks.cuf:365-374), on the stored deviations
    // (the decode is affine) and rounded as the engine rounds every stored value
    // (stochastically, from the ghost cell's index; every tile that forms the
    // same ghost gets the same value).  Column 0
    // is read only by the first tile, column nx+1 only by the tile holding nx.
    // (Formed by the whole CTA after each plane lands, with one more block
    // barrier in those tiles; done by the halo warp one plane ahead instead, it
    // measured slower.)
    constexpr bool WALL_GHOST = sizeof(S) == 2;
    const int cwall_lo = (WALL_GHOST && !P.periodic_x && i0 == 1) ? 0 : -1;
    const int cwall_hi = (WALL_GHOST && !P.periodic_x && i0 <= nx && nx <= i0 + 31) ? nx + 1 - (i0 - 1) : -1;
    auto wall_ghosts = [&](int g) {
        if constexpr (WALL_GHOST) {
            S *st = reinterpret_cast<S *>(smem) + (g & 3) * RD::STAGE;
            for (int t = tid; t < 2 * NPOP * RD::RH; t += 32 * W) {
                const int side = t / (NPOP * RD::RH), seg = t - side * (NPOP * RD::RH);
                const int c = side ? cwall_hi : cwall_lo;
                if (c < 0) continue;
                S *row = st + seg * RD::BXT;  // segment = one row of one population
                const int d = side ? -1 : 1;
                const float q = side ? float(P.q1) : float(P.q0);
                const float a = float(row[c + d]), b = float(row[c + 2 * d]);
                // rounded as a stored value of that ghost cell (stochastically, by its index)
                const int p = seg / RD::RH, r = seg - p * RD::RH;
                const long long dst = ((long long)g * (ny + 2) + (j0 - 1 + r)) * P.pitch_b + (i0 - 1 + c);
                row[c] = P.codec.encode_dev(p * P.ps_b + dst, p, q * a + (1.0f - q) * b);
            }
        }
    };

    const int gi = i0 + lane;
    const int gj = j0 + wr - 1;
    const bool cell = wr >= 1 && gi <= nx && gj <= ny;
    const int ci = min(gi, nx);
    const int cj = wr >= 1 ? min(gj, ny) : 1;
    const int hj = j0 + lane;
    const bool hx = wr == 0 && lane < W - 1 && hj <= ny;

    for (int g = kb - 1; g <= kb + 2; ++g) issue(g);
    T fzd[10], fzu[10], fx[10], fy[10], fo[NPOP];
    int buf = 0;
    wait(kb - 1);
    wait(kb);
    const bool wall_tile = cwall_lo >= 0 || cwall_hi >= 0;  // the same for the whole CTA
    if (wall_tile) {
        wall_ghosts(kb - 1);
        wall_ghosts(kb);
        __syncthreads();
    }
    if (wr >= 1) face_fluxes<T, S, 2, RECON, FF>(P, R, ci, cj, kb - 1, fzd);
    for (int k = kb; k < ke; ++k) {
        wait(k + 1);
        if (wall_tile) {
            wall_ghosts(k + 1);
            __syncthreads();
        }
        if (wr >= 1) {
            face_fluxes<T, S, 0, RECON, FF>(P, R, ci, cj, k, fx);
            face_fluxes<T, S, 1, RECON, FF>(P, R, ci, cj, k, fy);
            face_fluxes<T, S, 2, RECON, FF>(P, R, ci, cj, k, fzu);
#pragma unroll
            for (int s = 0; s < 10; ++s) ysh[buf][wr][s][lane] = fy[s];
            // the cell's f-tilde, loaded before the barrier so its latency overlaps the exchange
            if (cell) {
                const long long c = ((long long)(k - 1) * ny + (gj - 1)) * P.pitch + (gi - 1);
#pragma unroll
                for (int p = 0; p < NPOP; ++p) fo[p] = P.codec.raw(f_in, p * P.ps + c);
            }
        } else {
            face_fluxes<T, S, 1, RECON, FF>(P, R, ci, j0 - 1, k, fy);
#pragma unroll
            for (int s = 0; s < 10; ++s) ysh[buf][0][s][lane] = fy[s];
            if (hx) {
                T hxf[10];
                face_fluxes<T, S, 0, RECON, FF>(P, R, i0 - 1, hj, k, hxf);
#pragma unroll
                for (int s = 0; s < 10; ++s) xsh[buf][lane + 1][s] = hxf[s];
            }
        }
        __syncthreads();
        issue(k + 3);  // plane k-1 (same stage) is no longer read
        if (wr >= 1) {
            T fxl[10];
#pragma unroll
            for (int s = 0; s < 10; ++s) {
                const T up = __shfl_up_sync(0xffffffffu, fx[s], 1);
                fxl[s] = lane == 0 ? xsh[buf][wr][s] : up;
            }
            if (cell) {
                const long long c = ((long long)(k - 1) * ny + (gj - 1)) * P.pitch + (gi - 1);
                const unsigned hc = P.codec.cell_hash(c);
                const int cb = R.rb(gj, k) + gi;
                const T cxg = __ldg(P.cxuf + gi);
                const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0);
                {
                    const UpdateSum<T, S> u(upd_base(R.raw(0, cb, 0), fo[0], c43, c13));  // rest population
                    f_out[c] = u.encode(P.codec, 0, hc);
                }
                // the pairs (2m-1, 2m): they move along the same axes, and their flux
                // slots along each are adjacent
                auto sgn = [](int a, T cval) { return a > 0 ? -cval : cval; };
#pragma unroll
                for (int m = 1; m <= 9; ++m) {
                    const int p = 2 * m - 1, q = 2 * m;
                    UpdatePair<S> u(make_float2(R.raw(p, cb, 0), R.raw(q, cb, 0)), make_float2(fo[p], fo[q]));
                    if (cx(p)) {
                        const int s = flux_slot(0, p);
                        u.add(make_float2(sgn(cx(p), cxg), sgn(cx(q), cxg)),
                              sub_x2(make_float2(fx[s], fx[s + 1]), make_float2(fxl[s], fxl[s + 1])));
                    }
                    if (cy(p)) {
                        const int s = flux_slot(1, p);
                        u.add(make_float2(sgn(cy(p), P.cyuf), sgn(cy(q), P.cyuf)),
                              sub_x2(make_float2(fy[s], fy[s + 1]),
                                     make_float2(ysh[buf][wr - 1][s][lane], ysh[buf][wr - 1][s + 1][lane])));
                    }
                    if (cz(p)) {
                        const int s = flux_slot(2, p);
                        u.add(make_float2(sgn(cz(p), P.czuf), sgn(cz(q), P.czuf)),
                              sub_x2(make_float2(fzu[s], fzu[s + 1]), make_float2(fzd[s], fzd[s + 1])));
                    }
                    u.store(P.codec, f_out, p * P.ps + c, q * P.ps + c, p, q, hc);
                }
            }
#pragma unroll
            for (int s = 0; s < 10; ++s) fzd[s] = fzu[s];
        }
        buf ^= 1;
    }
    // every plane issued (g <= ke) has been waited for: no bulk copy is left in flight
}


template <class T, class S, int W>
constexpr size_t flux_tma_smem_bytes()
{
    using RD = SmemRead<T, S, W>;
    return 4 * size_t(RD::STAGE_BYTES) + 2 * W * 10 * 32 * sizeof(T) + 2 * W * 10 * sizeof(T) + 4 * 8;
}

// ---------------------------------------------------------------------------
// Density and velocity for output, src/dugks.cu:1021-1064: ghosted scalar
// arrays, u = j/rho + hdt*F_ambient.  FP64 outputs whatever the storage.
// ---------------------------------------------------------------------------
template <class T, class S>
__global__ void __launch_bounds__(256) macro_kernel(const S *__restrict__ f, const StepParams<T, S> P, double hdt,
                                                    double fxa, double fya, double fza,
                                                    double *rho, double *ux, double *uy, double *uz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= P.nx) return;
    const long long c = ((long long)k * P.ny + j) * P.pitch + i;
    double v[NPOP];
#pragma unroll
    for (int p = 0; p < NPOP; ++p) v[p] = double(P.codec.load_nc(f, p * P.ps + c, p));
    double r, jx, jy, jz;
    moments(v, r, jx, jy, jz);
    const size_t g = ((size_t)(k + 1) * (P.ny + 2) + (j + 1)) * (P.nx + 2) + (i + 1);
    rho[g] = r;
    ux[g] = jx / r + fxa * hdt;
    uy[g] = jy / r + fya * hdt;
    uz[g] = jz / r + fza * hdt;
}

}  // namespace dg
