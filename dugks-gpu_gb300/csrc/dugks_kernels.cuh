// DUGKS D3Q19 step kernels for sm_103a.
//
// Layout in HBM: structure of arrays, interior cells only, one plane per
// population: a[p*ps + ((k*ny + j)*pitch + i)] (0-based i, j, k).  There is no
// ghost layer: the periodic images and the wall extrapolation of f-bar-plus
// are formed while the flux kernel stages a tile in shared memory, which
// replaces the reference's extend_fb_x / extend_fb_x_wall / extend_fb_y
// kernels and the MPI z exchange (src/dugks.cu:348-377, src/parallel.cu:185-234).
//
// Kernels:
//   fbar_kernel      stage (a), src/dugks.cu:1131-1196 (calc_fb1)
//   flux_kernel      stages (c) (d) (e), src/dugks.cu:715-959 (calc_fx_tri),
//                    each face evaluated once, z-marching tile in shared memory
//   macro_kernel     src/dugks.cu:1021-1064 (calc_macro)
//
// Template parameters: T is the arithmetic type, S the storage type of f and
// f-bar-plus (double, float, or the 16-bit deviation codecs of storage.cuh).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "d3q19.cuh"
#include "storage.cuh"

namespace dg {

// ---------------------------------------------------------------------------
// Parameters (host-filled, passed by value; T-typed so that no conversion from
// double runs in an FP32 kernel)
// ---------------------------------------------------------------------------
template <class T, class S>
struct StepParams {
    int nx, ny, nz, pitch;
    long long ps;          // population stride (elements)
    int periodic_x;        // 0: bounce-back walls on the two x faces
    int perturb;           // per-cell perturbation force in stage (a)
    int force_on;          // ambient force non-zero
    // stage (a)
    T hdt, bw1, bw2, bw0x3;      // bw0x3 = 3*bw0
    T F[3];                      // ambient force
    T Kb[NPOP];                  // 3*bw0*(c_p . F)
    // faces
    T fw1, fw2, fw0x3;           // fw0x3 = 3*fw0
    T hF[3];                     // (0.5*hdt)*F, the face velocity shift (src/dugks.cu:698-700)
    T Kf[NPOP];                  // 3*fw0*(c_p . F)
    // interpolation weights, (1-m, m) pairs in the reference's lerp form
    T ty_om, ty_m;               // transverse y, |hdt/dy|
    T tz_om, tz_m;               // transverse z, |hdt/dz|
    T yn_om[NPOP], yn_m[NPOP];   // y-face normal (dy/2 - hdt*cy)/dy
    T zn_om[NPOP], zn_m[NPOP];   // z-face normal (dz/2 - hdt*cz)/dz
    T cyu, czu;                  // dt/dy, dt/dz
    T q0, q1;                    // wall ghost extrapolation weights (2 on a uniform mesh)
    const T *xw;                 // [(nx+1)*19*2] x-face normal (1-m, m); face I lies between cells I, I+1 (1-based)
    const T *txw;                // [(nx+2)*19*2] transverse x (1-t, t) per column 0..nx+1
    const T *cxu;                // [nx+2] dt/dxx(i)
    // perturbation forcing (src/dugks.cu:1086-1126) as separable factors
    const T *pert_x;             // [nx+2][3]: (1-cos xx), sin xx, in-zone flag
    const T *pert_y;             // [ny+2][3]: cos(beta yy), sin(beta yy), 0
    const T *pert_z;             // [nz+2][3]: cos(gamma zz), sin(gamma zz), 0
    T pert_ax, pert_ay, pert_az, pert_FF;  // per-step amplitude prefactors
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
// (src/dugks.cu:1201-1207 with 1/RT = 3).
template <class T>
__device__ __forceinline__ void feq_pair(T eu, T base, T wr, T &fp, T &fm)
{
    const T t = fma(T(0.5) * eu, eu, base);
    fp = wr * (t + eu);
    fm = wr * (t - eu);
}

// Zeroth and first moments of 19 values in the reference's summation order
// (src/dugks.cu:687-693): sequential over ip; the terms with c=0 add an exact
// zero there and are skipped here.
template <class T>
__device__ __forceinline__ void moments(const T v[NPOP], T &r, T &jx, T &jy, T &jz)
{
    r = v[0];
#pragma unroll
    for (int p = 1; p < NPOP; ++p) r += v[p];
    jx = v[1] - v[2];
    jx += v[7]; jx -= v[8]; jx += v[9]; jx -= v[10]; jx += v[11]; jx -= v[12]; jx += v[13]; jx -= v[14];
    jy = v[3] - v[4];
    jy += v[7]; jy += v[8]; jy -= v[9]; jy -= v[10]; jy += v[15]; jy -= v[16]; jy += v[17]; jy -= v[18];
    jz = v[5] - v[6];
    jz += v[11]; jz += v[12]; jz -= v[13]; jz -= v[14]; jz += v[15]; jz += v[16]; jz -= v[17]; jz -= v[18];
}

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

// ---------------------------------------------------------------------------
// Stage (a): f-bar-plus = bw1 f + (bw2 + bw0 F.(c-u)/RT) feq(rho, u + hdt F)
// ---------------------------------------------------------------------------
template <class T, class S>
__device__ __forceinline__ void cell_force(const StepParams<T, S> &P, int i, int j, int k, T &Fx, T &Fy, T &Fz)
{
    Fx = P.F[0]; Fy = P.F[1]; Fz = P.F[2];
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

template <class T, class S>
__global__ void __launch_bounds__(256) fbar_kernel(const S *__restrict__ f, S *__restrict__ fb, const StepParams<T, S> P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int k = blockIdx.z;
    if (i >= P.nx) return;
    const long long c = ((long long)k * P.ny + j) * P.pitch + i;

    T v[NPOP];
#pragma unroll
    for (int p = 0; p < NPOP; ++p) v[p] = P.codec.load_nc(f, p * P.ps + c, p);

    T r, jx, jy, jz;
    moments(v, r, jx, jy, jz);
    const T inv = T(1) / r;
    T u = jx * inv, vv = jy * inv, w = jz * inv;

    T Fx, Fy, Fz;
    cell_force(P, i, j, k, Fx, Fy, Fz);
    const bool forced = P.force_on || P.perturb;
    if (forced) {
        u = fma(P.hdt, Fx, u);
        vv = fma(P.hdt, Fy, vv);
        w = fma(P.hdt, Fz, w);
    }
    // coefficient of feq: bw2 + 3 bw0 (F.c - F.u) = B + K_p
    T B = P.bw2;
    if (forced) B = fma(-P.bw0x3, fma(Fx, u, fma(Fy, vv, Fz * w)), P.bw2);

    T fe[NPOP];
    feq_all(r, u, vv, w, fe);

#pragma unroll
    for (int p = 0; p < NPOP; ++p) {
        T K = P.Kb[p];
        if (P.perturb) {
            T cf = T(0);
            if (cx(p)) cf += cx(p) > 0 ? Fx : -Fx;
            if (cy(p)) cf += cy(p) > 0 ? Fy : -Fy;
            if (cz(p)) cf += cz(p) > 0 ? Fz : -Fz;
            K = P.bw0x3 * cf;
        }
        const T out = fma(B + K, fe[p], P.bw1 * v[p]);
        P.codec.store(fb, p * P.ps + c, p, out);
    }
}

// ---------------------------------------------------------------------------
// Stages (c) (d) (e): face reconstruction, face flux, finite-volume update.
//
// One CTA owns a BX x BY column of cells and marches over a chunk of z
// planes.  Three planes of f-bar-plus (k-1, k, k+1) with a one-cell halo in x
// and y live in shared memory; every face of plane k is reconstructed once:
//   x faces I-1/2 .. I+BX-1/2 of each row, y faces likewise, z face k+1/2;
// the 10 fluxes of each face (populations with c_normal != 0) go to shared
// memory and the cells of plane k are updated from them.
// ---------------------------------------------------------------------------
template <class T, int BX, int BY>
struct FluxTile {
    static constexpr int PW = BX + 2, PH = BY + 2, PL = PW * PH;
    static constexpr int NXF = (BX + 1) * BY, NYF = BX * (BY + 1), NZF = BX * BY;
    static constexpr int pad32(int n) { return (n + 31) / 32 * 32; }
    static constexpr int NXFP = pad32(NXF), NYFP = pad32(NYF), NZFP = pad32(NZF);
    static constexpr size_t elems = 3 * NPOP * PL + 10 * (NXF + NYF + 2 * NZF);
    static constexpr size_t bytes = sizeof(T) * elems;
};

// Reconstruct the 19 values of one face from the staged planes and return the
// 10 fluxes of the populations crossing it.
//   AX = 0: x face between anchor column sa and other column sa+dxo (row sj)
//   AX = 1: y face between anchor row and the row above
//   AX = 2: z face between plane k (anchor) and plane k+1
// `pA` / `pB`: planes holding the anchor / other side along the normal for
// AX=2; for AX=0,1 pA is plane k, and pM / pP are planes k-1 / k+1 used by
// the transverse z shift (c_z = +1 reads plane k-1).
template <class T, class S, int AX, int BX, int BY>
__device__ __forceinline__ void face_values(const StepParams<T, S> &P, const T *pA, const T *pB, const T *pM, const T *pP,
                                            int sa, int dxo, int gi, const T *xw_face, T v[NPOP])
{
    using Tile = FluxTile<T, BX, BY>;
    constexpr int PW = Tile::PW, PL = Tile::PL;
#pragma unroll
    for (int p = 0; p < NPOP; ++p) {
        const T *base = pA + p * PL;
        if (p == 0) {
            // rest population: mean of the two cells across the face (src/dugks.cu:756-763)
            const int o = AX == 0 ? dxo : (AX == 1 ? PW : 0);
            const T a = base[sa];
            const T b = AX == 2 ? pB[sa] : base[sa + o];
            v[0] = T(0.5) * (a + b);
            continue;
        }
        const int ax = cx(p), ay = cy(p), az = cz(p);
        if (AX == 0) {
            // x normal; y shift jj=-cy; z shift kk=-cz (plane k-cz)
            const T om = __ldg(xw_face + 2 * p), m = __ldg(xw_face + 2 * p + 1);
            const int jo = -ay * PW;
            const T *b0 = base;
            const T *b1 = az > 0 ? pM + p * PL : (az < 0 ? pP + p * PL : base);
            const T x00 = lerp2(om, m, b0[sa], b0[sa + dxo]);
            T y00 = x00;
            if (ay != 0) {
                const T x01 = lerp2(om, m, b0[sa + jo], b0[sa + jo + dxo]);
                y00 = lerp2(P.ty_om, P.ty_m, x00, x01);
            }
            if (az != 0) {
                const T x10 = lerp2(om, m, b1[sa], b1[sa + dxo]);
                T y11 = x10;
                if (ay != 0) {
                    const T x11 = lerp2(om, m, b1[sa + jo], b1[sa + jo + dxo]);
                    y11 = lerp2(P.ty_om, P.ty_m, x10, x11);
                }
                v[p] = lerp2(P.tz_om, P.tz_m, y00, y11);
            } else {
                v[p] = y00;
            }
        } else if (AX == 1) {
            // x shift ii=-cx (transverse, per-column weight); y normal (anchor row, row above); z shift kk=-cz
            const int io = -ax;
            const T *b0 = base;
            const T *b1 = az > 0 ? pM + p * PL : (az < 0 ? pP + p * PL : base);
            T txo = T(1), txm = T(0);
            if (ax != 0) {
                txo = __ldg(P.txw + (size_t)gi * 38 + 2 * p);
                txm = __ldg(P.txw + (size_t)gi * 38 + 2 * p + 1);
            }
            T x00 = b0[sa], x01 = b0[sa + PW];
            if (ax != 0) {
                x00 = lerp2(txo, txm, x00, b0[sa + io]);
                x01 = lerp2(txo, txm, x01, b0[sa + PW + io]);
            }
            const T y00 = lerp2(P.yn_om[p], P.yn_m[p], x00, x01);
            if (az != 0) {
                T x10 = b1[sa], x11 = b1[sa + PW];
                if (ax != 0) {
                    x10 = lerp2(txo, txm, x10, b1[sa + io]);
                    x11 = lerp2(txo, txm, x11, b1[sa + PW + io]);
                }
                const T y11 = lerp2(P.yn_om[p], P.yn_m[p], x10, x11);
                v[p] = lerp2(P.tz_om, P.tz_m, y00, y11);
            } else {
                v[p] = y00;
            }
        } else {
            // x shift ii=-cx, y shift jj=-cy, z normal (plane k anchor, plane k+1 other)
            const int io = -ax, jo = -ay * PW;
            const T *b0 = base, *b1 = pB + p * PL;
            T txo = T(1), txm = T(0);
            if (ax != 0) {
                txo = __ldg(P.txw + (size_t)gi * 38 + 2 * p);
                txm = __ldg(P.txw + (size_t)gi * 38 + 2 * p + 1);
            }
            T x00 = b0[sa], x10 = b1[sa];
            if (ax != 0) {
                x00 = lerp2(txo, txm, x00, b0[sa + io]);
                x10 = lerp2(txo, txm, x10, b1[sa + io]);
            }
            T y00 = x00, y11 = x10;
            if (ay != 0) {
                T x01 = b0[sa + jo], x11 = b1[sa + jo];
                if (ax != 0) {
                    x01 = lerp2(txo, txm, x01, b0[sa + jo + io]);
                    x11 = lerp2(txo, txm, x11, b1[sa + jo + io]);
                }
                y00 = lerp2(P.ty_om, P.ty_m, x00, x01);
                y11 = lerp2(P.ty_om, P.ty_m, x10, x11);
            }
            v[p] = lerp2(P.zn_om[p], P.zn_m[p], y00, y11);
        }
    }
}

// Face equilibrium and flux (src/dugks.cu:675-709 f2ruvwh, 912-943):
//   F_p = fw1 v_p + (fw2 + fw0 F.(c_p - u)/RT) feq_p(rho, u + hdt/2 F)
// for the 10 populations crossing a face normal to AX, written to out[s*stride].
template <class T, class S, int AX>
__device__ __forceinline__ void face_flux(const StepParams<T, S> &P, const T v[NPOP], T *out, int stride)
{
    T r, jx, jy, jz;
    moments(v, r, jx, jy, jz);
    const T inv = T(1) / r;
    T u = jx * inv, vv = jy * inv, w = jz * inv;
    T B = P.fw2;
    if (P.force_on) {
        u += P.hF[0];
        vv += P.hF[1];
        w += P.hF[2];
        B = fma(-P.fw0x3, fma(P.F[0], u, fma(P.F[1], vv, P.F[2] * w)), P.fw2);
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
#pragma unroll
    for (int s = 0; s < 10; ++s) {
        const int p = flux_pop(AX, s);
        out[s * stride] = fma(B + P.Kf[p], fe[p], P.fw1 * v[p]);
    }
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

template <class T, class S, int BX, int BY, int NT>
__global__ void __launch_bounds__(NT) flux_kernel(const S *__restrict__ fb, const S *f_in, S *f_out,
                                                   const StepParams<T, S> P, int kchunk)
{
    using Tile = FluxTile<T, BX, BY>;
    constexpr int PW = Tile::PW, PL = Tile::PL;
    constexpr int NXF = Tile::NXF, NYF = Tile::NYF, NZF = Tile::NZF;
    constexpr int NXFP = Tile::NXFP, NYFP = Tile::NYFP, NZFP = Tile::NZFP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *planes = reinterpret_cast<T *>(smem_raw);     // [3][19][PL]
    T *fxs = planes + 3 * NPOP * PL;                  // [10][NXF]
    T *fys = fxs + 10 * NXF;                          // [10][NYF]
    T *fzs = fys + 10 * NYF;                          // [2][10][NZF]

    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int i0 = blockIdx.x * BX + 1;  // 1-based first cell of the tile
    const int j0 = blockIdx.y * BY + 1;
    const int kb = blockIdx.z * kchunk + 1;
    const int ke = min(kb + kchunk, nz + 1);  // exclusive
    const int tid = threadIdx.x;
    const long long ps = P.ps;

    // ---- stage plane g (1-based, 0..nz+1) of f-bar-plus into its buffer ----
    auto load_plane = [&](int g) {
        const int gz = g == 0 ? nz : (g == nz + 1 ? 1 : g);
        T *dst = planes + (g % 3) * NPOP * PL;
        const long long zoff = (long long)(gz - 1) * ny * P.pitch;
        for (int e = tid; e < PL; e += NT) {
            const int sj = e / PW, si = e - sj * PW;
            int gi = i0 - 1 + si, gj = j0 - 1 + sj;
            gj = gj == 0 ? ny : (gj == ny + 1 ? 1 : (gj > ny + 1 ? ny : gj));
            int mode = 0;  // 0 plain, 1 left wall ghost, 2 right wall ghost
            if (gi == 0) {
                if (P.periodic_x) gi = nx; else mode = 1;
            } else if (gi == nx + 1) {
                if (P.periodic_x) gi = 1; else mode = 2;
            } else if (gi > nx + 1) {
                gi = nx;
            }
            const long long row = zoff + (long long)(gj - 1) * P.pitch;
            if (mode == 0) {
                const long long o = row + (gi - 1);
#pragma unroll
                for (int p = 0; p < NPOP; ++p) dst[p * PL + e] = P.codec.load_nc(fb, p * ps + o, p);
            } else {
                // linear extrapolation to the ghost cell centre (src/dugks.cu:1247-1248;
                // stretched: src/fortran/channel/src/dugks.cuf:368-373)
                const long long o1 = row + (mode == 1 ? 0 : nx - 1);
                const long long o2 = row + (mode == 1 ? 1 : nx - 2);
                const T q = mode == 1 ? P.q0 : P.q1;
#pragma unroll
                for (int p = 0; p < NPOP; ++p) {
                    const T a = P.codec.load_nc(fb, p * ps + o1, p);
                    const T b = P.codec.load_nc(fb, p * ps + o2, p);
                    dst[p * PL + e] = q * a + (T(1) - q) * b;
                }
            }
        }
    };
    auto plane = [&](int g) -> const T * { return planes + (g % 3) * NPOP * PL; };

    // ---- reconstruct + flux of the faces of plane k (x, y and z=k+1/2) ----
    auto faces = [&](int k, int zbuf, bool xy) {
        const T *pk = plane(k), *pm = plane(k - 1), *pp = plane(k + 1);
        const int njobs = xy ? NXFP + NYFP + NZFP : NZFP;
        for (int q0 = tid; q0 < njobs; q0 += NT) {
            int q = xy ? q0 : q0 + NXFP + NYFP;
            T v[NPOP];
            if (q < NXFP) {
                if (q >= NXF) continue;
                const int sj = q / (BX + 1), fi = q - sj * (BX + 1);
                const int I = i0 - 1 + fi, gj = j0 + sj;
                if (I > nx || gj > ny) continue;
                const int sa = (sj + 1) * PW + (I == 0 ? fi + 1 : fi);
                const int dxo = I == 0 ? -1 : 1;
                face_values<T, S, 0, BX, BY>(P, pk, nullptr, pm, pp, sa, dxo, 0, P.xw + (size_t)I * 38, v);
                if (!P.periodic_x) bounce_back(v, I == 0, I == nx);
                face_flux<T, S, 0>(P, v, fxs + q, NXF);
            } else if (q < NXFP + NYFP) {
                q -= NXFP;
                if (q >= NYF) continue;
                const int fj = q / BX, si = q - fj * BX;
                const int gi = i0 + si, J = j0 - 1 + fj;
                if (gi > nx || J > ny) continue;
                const int sa = fj * PW + si + 1;
                face_values<T, S, 1, BX, BY>(P, pk, nullptr, pm, pp, sa, 0, gi, nullptr, v);
                face_flux<T, S, 1>(P, v, fys + q, NYF);
            } else {
                q -= NXFP + NYFP;
                if (q >= NZF) continue;
                const int sj = q / BX, si = q - sj * BX;
                const int gi = i0 + si, gj = j0 + sj;
                if (gi > nx || gj > ny) continue;
                const int sa = (sj + 1) * PW + si + 1;
                face_values<T, S, 2, BX, BY>(P, pk, pp, nullptr, nullptr, sa, 0, gi, nullptr, v);
                face_flux<T, S, 2>(P, v, fzs + zbuf * 10 * NZF + q, NZF);
            }
        }
    };

    // ---- finite-volume update of plane k (src/dugks.cu:945-956) ----
    auto update = [&](int k, int zbot, int ztop) {
        const T *pk = plane(k);
        const T c43 = T(4.0 / 3.0), c13 = T(1.0 / 3.0);
        for (int q = tid; q < BX * BY; q += NT) {
            const int sj = q / BX, si = q - sj * BX;
            const int gi = i0 + si, gj = j0 + sj;
            if (gi > nx || gj > ny) continue;
            const long long c = ((long long)(k - 1) * ny + (gj - 1)) * P.pitch + (gi - 1);
            const T cxg = __ldg(P.cxu + gi);
            const int sc = (sj + 1) * PW + si + 1;
#pragma unroll
            for (int p = 0; p < NPOP; ++p) {
                const T fo = P.codec.load(f_in, p * ps + c, p);
                T r = fma(pk[p * PL + sc], c43, -(fo * c13));
                if (cx(p)) {
                    const int s = flux_slot(0, p);
                    const T d = fxs[s * NXF + sj * (BX + 1) + si + 1] - fxs[s * NXF + sj * (BX + 1) + si];
                    r = fma(cx(p) > 0 ? -cxg : cxg, d, r);
                }
                if (cy(p)) {
                    const int s = flux_slot(1, p);
                    const T d = fys[s * NYF + (sj + 1) * BX + si] - fys[s * NYF + sj * BX + si];
                    r = fma(cy(p) > 0 ? -P.cyu : P.cyu, d, r);
                }
                if (cz(p)) {
                    const int s = flux_slot(2, p);
                    const T d = fzs[ztop * 10 * NZF + s * NZF + q] - fzs[zbot * 10 * NZF + s * NZF + q];
                    r = fma(cz(p) > 0 ? -P.czu : P.czu, d, r);
                }
                P.codec.store(f_out, p * ps + c, p, r);
            }
        }
    };

    if (kb >= ke) return;
    load_plane(kb - 1);
    load_plane(kb);
    load_plane(kb + 1);
    __syncthreads();
    {
        // bottom z face of the chunk (kb-1/2): anchor plane kb-1, other plane kb
        const T *pa = plane(kb - 1), *pb = plane(kb);
        for (int q = tid; q < NZF; q += NT) {
            const int sj = q / BX, si = q - sj * BX;
            const int gi = i0 + si, gj = j0 + sj;
            if (gi > nx || gj > ny) continue;
            T v[NPOP];
            face_values<T, S, 2, BX, BY>(P, pa, pb, nullptr, nullptr, (sj + 1) * PW + si + 1, 0, gi, nullptr, v);
            face_flux<T, S, 2>(P, v, fzs + q, NZF);
        }
    }
    faces(kb, 1, true);
    __syncthreads();
    for (int k = kb; k < ke; ++k) {
        const int zbot = (k - kb) & 1, ztop = zbot ^ 1;
        if (k + 2 <= ke) load_plane(k + 2);
        update(k, zbot, ztop);
        __syncthreads();
        if (k + 1 < ke) faces(k + 1, zbot, true);
        __syncthreads();
    }
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
