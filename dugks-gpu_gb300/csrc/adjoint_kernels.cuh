// Hand-written adjoint (transposed Jacobian) of one DUGKS step.
//
// The forward step S (dugks_kernels.cuh) is
//   fb   = A(f)                         stage (a), per cell
//   v    = L(G fb)                      ghost formation G, interpolation L (linear)
//   v'   = B v                          bounce-back on the wall faces (linear)
//   F    = phi(v')                      face equilibrium + flux, per face
//   f'   = 4/3 fb - 1/3 f - D F         finite-volume update (linear)
// Given lam' = dJ/df', the adjoint step returns lam = (dS/df)^T lam':
//   lamF = -D^T lam'                    (per face, the two adjacent cells)
//   lamv = B^T (dphi/dv')^T lamF        adj_face_kernel, one thread per face
//   mu   = 4/3 lam' + G^T L^T lamv      adj_gather_kernel (gather form, deterministic)
//   lam  = (dA/df)^T mu - 1/3 lam'      adj_gather_kernel
// For a face or a cell with density r, first moment j, u0 = j/r,
// u = u0 + shift, coefficient c_p = fw2 + 3 fw0 (F.c_p - F.u) and
// feq_p = w_p r (1 + 3 c_p.u + 4.5 (c_p.u)^2 - 1.5 u.u), the map
// out_p = w1 x_p + c_p feq_p has the transposed Jacobian
//   lam_x_q = w1 lamo_q + (S0 + G.(c_q - u0)) / r
//   S0 = sum_p lamo_p c_p feq_p
//   G  = sum_p lamo_p [c_p w_p r (3 c_p + 9 (c_p.u) c_p - 3 u) - 3 w0 F feq_p].
#pragma once
#include "dugks_kernels.cuh"

namespace dg {

// Accumulators of S0 and G over the populations, without multiplications by
// zero velocity components:
//   S0 = sum lam_p coef_p feq_p,  Lf = sum lam_p feq_p,
//   A = sum a_p,  Bd_d = sum a_p b_p c_pd   (a_p = lam_p coef_p w_p r, b_p = 3 + 9 c_p.u)
// so that G_d = Bd_d - 3 u_d A - 3 w0 F_d Lf.
template <class T>
struct AdjJac {
    T S0, Lf, A, Bd[3];
};

// c_p . u from the non-zero components only
template <class T>
__device__ __forceinline__ T cdot(int p, T u, T v, T w)
{
    T s = T(0);
    bool any = false;
    if (cx(p)) { s = cx(p) > 0 ? u : -u; any = true; }
    if (cy(p)) { s = any ? (cy(p) > 0 ? s + v : s - v) : (cy(p) > 0 ? v : -v); any = true; }
    if (cz(p)) s = any ? (cz(p) > 0 ? s + w : s - w) : (cz(p) > 0 ? w : -w);
    return s;
}

// One population's terms; lam is the adjoint of out_p = w1 x_p + coef_p feq_p
// and wr = w_p r.
template <class T>
__device__ __forceinline__ void adj_accum(AdjJac<T> &J, int p, T lam, T wr, T u, T v, T w, T coef, T feq)
{
    const T lc = lam * coef;
    J.S0 = fma(lc, feq, J.S0);
    J.Lf = fma(lam, feq, J.Lf);
    const T a = lc * wr;
    J.A += a;
    const T b = fma(T(9), cdot(p, u, v, w), T(3));
    if (cx(p)) J.Bd[0] = fma(cx(p) > 0 ? a : -a, b, J.Bd[0]);
    if (cy(p)) J.Bd[1] = fma(cy(p) > 0 ? a : -a, b, J.Bd[1]);
    if (cz(p)) J.Bd[2] = fma(cz(p) > 0 ? a : -a, b, J.Bd[2]);
}

// G without the force term (Gq_d = Bd_d - 3 u_d A) and with it (G_d = Gq_d - w0x3 F_d Lf)
template <class T>
__device__ __forceinline__ void adj_G(const AdjJac<T> &J, T u, T v, T w, T w0x3, const T F[3], T Gq[3], T G[3])
{
    Gq[0] = fma(T(-3) * u, J.A, J.Bd[0]);
    Gq[1] = fma(T(-3) * v, J.A, J.Bd[1]);
    Gq[2] = fma(T(-3) * w, J.A, J.Bd[2]);
    const T fl = w0x3 * J.Lf;
    G[0] = fma(-fl, F[0], Gq[0]);
    G[1] = fma(-fl, F[1], Gq[1]);
    G[2] = fma(-fl, F[2], Gq[2]);
}

// g_p = S0 + G.(c_p - u0) as K0 + G.c_p with K0 = S0 - G.u0
template <class T>
__device__ __forceinline__ T adj_g(int p, T K0, const T G[3])
{
    T g = K0;
    if (cx(p)) g = cx(p) > 0 ? g + G[0] : g - G[0];
    if (cy(p)) g = cy(p) > 0 ? g + G[1] : g - G[1];
    if (cz(p)) g = cz(p) > 0 ? g + G[2] : g - G[2];
    return g;
}

// w_p r of population p from the three class values
template <class T>
__device__ __forceinline__ T wr_of(int p, T wr0, T wr1, T wr2)
{
    return p == 0 ? wr0 : (p <= 6 ? wr1 : wr2);
}

template <class T, class S>
__device__ __forceinline__ T lam_at(const S *lam, const StepParams<T, S> &P, int p, int gi, int gj, int gk)
{
    const long long c = ((long long)(gk - 1) * P.ny + (gj - 1)) * P.pitch + (gi - 1);
    return T(lam[p * P.ps + c]);
}

// Number of faces of each orientation in the per-face adjoint buffers.
//   x faces: I = 0..nx (face I between cells I and I+1), per (j, k)
//   y faces: J = 1..ny (between J and J+1, periodic), per (i, k)
//   z faces: K = 1..nz, per (i, j)
__host__ __device__ inline long long adj_nface(int ax, int nx, int ny, int nz)
{
    return ax == 0 ? (long long)(nx + 1) * ny * nz : (long long)nx * ny * nz;
}
__host__ __device__ inline long long adj_xface(int I, int j, int k, int nx, int ny)
{
    return ((long long)(k - 1) * ny + (j - 1)) * (nx + 1) + I;
}
__host__ __device__ inline long long adj_cell(int i, int j, int k, int nx, int ny)
{
    return ((long long)(k - 1) * ny + (j - 1)) * nx + (i - 1);
}

// Per-face adjoint: reconstruct the face values (the forward's face_tri with
// reader RD), take the flux adjoint from the two adjacent cells' lam', apply
// (dphi/dv)^T and the bounce-back transpose.  F: the face's first index (x
// faces: I = 0..nx, between columns I and I+1; y / z faces: the column i);
// j, k: row and plane (1-based).  lv: the 19 adjoint face values; lf: dJ/dF
// of the face force along the field axis (0 without a field).
template <class T, class S, int AX, class RD>
__device__ __forceinline__ void adj_face_values(const StepParams<T, S> &P, const RD &R,
                                                const S *__restrict__ lam_next, int F, int j, int k, T lv[NPOP],
                                                T &lf)
{
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int I = AX == 0 ? F : 0, i = AX == 0 ? 1 : F;
    T v[NPOP];
    if (Fp64Form<T>::value)
        face_tri_cw<T, S, AX>(P, R, F, j, k, v);  // the forward's own face values
    else
        face_tri<T, S, AX>(P, R, F, j, k, v);
    const bool lo = AX == 0 && !P.periodic_x && I == 0;
    const bool hi = AX == 0 && !P.periodic_x && I == nx;
    bounce_back(v, lo, hi);

    // --- lamF of the 10 crossing populations from the adjacent cells ---
    T lamF[NPOP];
#pragma unroll
    for (int p = 0; p < NPOP; ++p) lamF[p] = T(0);
    if (AX == 0) {
        const int L = I, Rc = I + 1 <= nx ? I + 1 : (P.periodic_x ? 1 : 0);
        const T cl = L >= 1 ? __ldg(P.cxu + L) : T(0);
        const T cr = Rc >= 1 ? __ldg(P.cxu + Rc) : T(0);
#pragma unroll
        for (int s = 0; s < 10; ++s) {
            const int p = flux_pop(0, s);
            T a = T(0);
            if (Rc >= 1) a += cr * lam_at(lam_next, P, p, Rc, j, k);
            if (L >= 1) a -= cl * lam_at(lam_next, P, p, L, j, k);
            lamF[p] = T(cx(p)) * a;
        }
    } else if (AX == 1) {
        const int J2 = j + 1 <= ny ? j + 1 : 1;
#pragma unroll
        for (int s = 0; s < 10; ++s) {
            const int p = flux_pop(1, s);
            lamF[p] = T(cy(p)) * P.cyu * (lam_at(lam_next, P, p, i, J2, k) - lam_at(lam_next, P, p, i, j, k));
        }
    } else {
        const int K2 = k + 1 <= nz ? k + 1 : 1;
#pragma unroll
        for (int s = 0; s < 10; ++s) {
            const int p = flux_pop(2, s);
            lamF[p] = T(cz(p)) * P.czu * (lam_at(lam_next, P, p, i, j, K2) - lam_at(lam_next, P, p, i, j, k));
        }
    }

    // --- (dphi/dv)^T ---
    T r, jx, jy, jz;
    moments(v, r, jx, jy, jz);
    const T inv = recip(r);
    const T u0 = jx * inv, v0 = jy * inv, w0 = jz * inv;
    // face force: ambient plus the field averaged over the two cells
    T Ff[3] = {P.F[0], P.F[1], P.F[2]};
    const T fadd = P.ffield ? face_field<T, S, AX>(P, F, j, k) : T(0);
    if (P.ffield) {
        // add along the field axis with selects (no dynamically indexed local array)
        Ff[0] += P.ffaxis == 0 ? fadd : T(0);
        Ff[1] += P.ffaxis == 1 ? fadd : T(0);
        Ff[2] += P.ffaxis == 2 ? fadd : T(0);
    }
    const T hh = T(0.5) * P.hdt;
    T u = u0, vv = v0, w = w0, B = P.fw2;
    if (P.force_on || P.ffield) {
        u = fma(hh, Ff[0], u);
        vv = fma(hh, Ff[1], vv);
        w = fma(hh, Ff[2], w);
        B = fma(-P.fw0x3, fma(Ff[0], u, fma(Ff[1], vv, Ff[2] * w)), P.fw2);
    }
    T fe[NPOP];
    feq_face<T, AX>(r, u, vv, w, fe);
    AdjJac<T> Jc = {T(0), T(0), T(0), {T(0), T(0), T(0)}};
    // with a field: L1 = sum lamF_p c_{a,p} feq_p along the field axis a (Jc.Lf = sum lamF_p feq_p)
    const int fax = P.ffaxis;
    const T wr1 = weight<T>(1) * r, wr2 = weight<T>(7) * r;
    T L1 = T(0);
#pragma unroll
    for (int s = 0; s < 10; ++s) {
        const int p = flux_pop(AX, s);
        // coef_p = fw2 + 3 fw0 (F.c_p - F.u): the table value without a field
        const T coef = P.ffield ? fma(P.fw0x3, cdot(p, Ff[0], Ff[1], Ff[2]), B) : B + P.Kf[p];
        adj_accum(Jc, p, lamF[p], wr_of(p, wr1, wr1, wr2), u, vv, w, coef, fe[p]);
        if (P.ffield) {
            const int ca = fax == 0 ? cx(p) : (fax == 1 ? cy(p) : cz(p));
            if (ca) L1 = fma(ca > 0 ? lamF[p] : -lamF[p], fe[p], L1);
        }
    }
    T Gq[3], G[3];
    adj_G(Jc, u, vv, w, P.fw0x3, Ff, Gq, G);
    if (P.ffield) {
        // dJ/dF_a = 3 fw0 sum lamF (c_a - u_a - hh F_a) feq + hh sum lamF coef d feq / d u_a
        //         = 3 fw0 (L1 - (u_a + hh F_a) Lf) + hh Gq_a
        const T ua = fax == 0 ? u : (fax == 1 ? vv : w);
        const T Fa = fax == 0 ? Ff[0] : (fax == 1 ? Ff[1] : Ff[2]);
        const T Gqa = fax == 0 ? Gq[0] : (fax == 1 ? Gq[1] : Gq[2]);
        const T Sc = L1 - (ua + hh * Fa) * Jc.Lf;
        lf = P.fw0x3 * Sc + hh * Gqa;
    } else {
        lf = T(0);
    }
    const T K0 = fma(-G[2], w0, fma(-G[1], v0, fma(-G[0], u0, Jc.S0)));
#pragma unroll
    for (int p = 0; p < NPOP; ++p) lv[p] = fma(P.fw1, lamF[p], adj_g(p, K0, G) * inv);
    // bounce-back transpose
    if (lo) {
        lv[2] += lv[1]; lv[1] = T(0); lv[10] += lv[7]; lv[7] = T(0); lv[8] += lv[9]; lv[9] = T(0);
        lv[14] += lv[11]; lv[11] = T(0); lv[12] += lv[13]; lv[13] = T(0);
    }
    if (hi) {
        lv[1] += lv[2]; lv[2] = T(0); lv[7] += lv[10]; lv[10] = T(0); lv[9] += lv[8]; lv[8] = T(0);
        lv[11] += lv[14]; lv[14] = T(0); lv[13] += lv[12]; lv[12] = T(0);
    }
}

// One thread per face of orientation AX (f-bar-plus through L1), storing
// lamv[19] of the face (population-major, stride nface) and dJ/dF.
// only_x0: x faces I = 0 only (one thread per row and plane).
template <class T, class S, int AX>
__global__ void __launch_bounds__(128) adj_face_kernel(const S *__restrict__ fb, const S *__restrict__ lam_next,
                                                       T *__restrict__ lamv, T *__restrict__ lamF_face,
                                                       const StepParams<T, S> P, int only_x0)
{
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long nface = adj_nface(AX, nx, ny, nz);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long q;
    int F, j, k;
    if (AX == 0) {
        if (only_x0) {
            if (t >= (long long)ny * nz) return;
            q = t * (nx + 1);
        } else {
            q = t;
        }
        if (q >= nface) return;
        F = int(q % (nx + 1));
        const long long r = q / (nx + 1);
        j = int(r % ny) + 1;
        k = int(r / ny) + 1;
        if (P.periodic_x && F == 0) {
            for (int p = 0; p < NPOP; ++p) lamv[p * nface + q] = T(0);  // periodic: face 0 is face nx
            if (lamF_face) lamF_face[q] = T(0);
            return;
        }
    } else {
        q = t;
        if (q >= nface) return;
        F = int(q % nx) + 1;
        const long long r = q / nx;
        j = int(r % ny) + 1;
        k = int(r / ny) + 1;
    }
    const FbRead<T, S> R{fb, P.ps_b, P.pitch_b, ny, nz, P.codec};
    T lv[NPOP], lf;
    adj_face_values<T, S, AX>(P, R, lam_next, F, j, k, lv, lf);
    if (lamF_face) lamF_face[q] = lf;
#pragma unroll
    for (int p = 0; p < NPOP; ++p) lamv[p * nface + q] = lv[p];
}

// The three faces +x (I = i), +y (J = j) and +z (K = k) of every cell, with
// f-bar-plus staged through the same 4-plane TMA ring as the forward flux
// kernel: W warps, one row of 32 cells each, marching a chunk of z planes.
// The box holds rows j0-1 .. j0+W (the stencil's transverse and +y rows).
// x faces I = 0 are left to adj_face_kernel (only_x0).
template <class T, class S, int W>
constexpr size_t adj_faces_tma_smem_bytes()
{
    return 4 * size_t(SmemRead<T, S, W + 1>::STAGE_BYTES) + 4 * 8;
}

template <class T, class S, int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) adj_faces_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                      const S *__restrict__ lam_next,
                                                                      T *__restrict__ LX, T *__restrict__ LY,
                                                                      T *__restrict__ LZ, T *__restrict__ LFX,
                                                                      T *__restrict__ LFY, T *__restrict__ LFZ,
                                                                      const StepParams<T, S> P, int kchunk)
{
    using RD = SmemRead<T, S, W + 1>;
    extern __shared__ __align__(128) unsigned char smem[];
    S *ring = reinterpret_cast<S *>(smem);
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(smem + 4 * RD::STAGE_BYTES);
    constexpr unsigned TILE_BYTES = unsigned(NPOP * RD::POPS * sizeof(S));

    const int lane = threadIdx.x, wr = threadIdx.y, tid = wr * 32 + lane;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int i0 = blockIdx.x * 32 + 1;
    const int j0 = blockIdx.y * W + 1;
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
    unsigned phase = 0;
    int wait_limit = kWaitPolls;
    auto wait = [&](int g) {
        const int s = g & 3;
        if (!mbar_wait(smem_u32(mbar + s), (phase >> s) & 1u, wait_limit)) {
            atomicOr(P.err, 1);
            wait_limit = kWaitPollsAfterFailure;
        }
        phase ^= 1u << s;
    };

    const int gi = i0 + lane, gj = j0 + wr;
    const bool cell = gi <= nx && gj <= ny;
    const long long nfx = adj_nface(0, nx, ny, nz), nfc = adj_nface(1, nx, ny, nz);
    for (int g = kb - 1; g <= kb + 2; ++g) issue(g);
    wait(kb - 1);
    wait(kb);
    for (int k = kb; k < ke; ++k) {
        wait(k + 1);
        if (cell) {
            T lv[NPOP], lf;
            const long long qx = adj_xface(gi, gj, k, nx, ny), qc = adj_cell(gi, gj, k, nx, ny);
            adj_face_values<T, S, 0>(P, R, lam_next, gi, gj, k, lv, lf);
            LFX[qx] = lf;
#pragma unroll
            for (int p = 0; p < NPOP; ++p) LX[p * nfx + qx] = lv[p];
            adj_face_values<T, S, 1>(P, R, lam_next, gi, gj, k, lv, lf);
            LFY[qc] = lf;
#pragma unroll
            for (int p = 0; p < NPOP; ++p) LY[p * nfc + qc] = lv[p];
            adj_face_values<T, S, 2>(P, R, lam_next, gi, gj, k, lv, lf);
            LFZ[qc] = lf;
#pragma unroll
            for (int p = 0; p < NPOP; ++p) LZ[p * nfc + qc] = lv[p];
        }
        __syncthreads();
        issue(k + 3);  // plane k-1 (same stage) is no longer read
    }
    // every plane issued (g <= ke) has been waited for: no bulk copy is left in flight
}

// Row / plane offsets of the face arrays around one interior cell (the
// periodic images in y and z folded in): x faces ((k-1)*ny + (j-1))*(nx+1),
// y / z faces ((k-1)*ny + (j-1))*nx, for j-1..j+1 and k-1..k+1.
struct AdjRows {
    int kx[3], jx[3];  // x faces: plane part ((k'-1)*ny)*(nx+1) and row part (j'-1)*(nx+1), k' = k-1..k+1
    int kc[3], jc[3];  // y / z faces: the same with nx
    __device__ __forceinline__ int x(int dk, int dj) const { return kx[dk] + jx[dj]; }  // [dk+1][dj+1]
    __device__ __forceinline__ int c(int dk, int dj) const { return kc[dk] + jc[dj]; }
};

__device__ __forceinline__ AdjRows adj_rows(int j, int k, int nx, int ny, int nz)
{
    AdjRows R;
    const int js[3] = {j == 1 ? ny : j - 1, j, j == ny ? 1 : j + 1};
    const int ks[3] = {k == 1 ? nz : k - 1, k, k == nz ? 1 : k + 1};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        R.kx[a] = (ks[a] - 1) * ny * (nx + 1);
        R.jx[a] = (js[a] - 1) * (nx + 1);
        R.kc[a] = (ks[a] - 1) * ny * nx;
        R.jc[a] = (js[a] - 1) * nx;
    }
    return R;
}

// Transposed-stencil sums of one population p (a compile-time constant)
// around row j, plane k: the adjoint that an f-bar-plus value at column gi
// receives from the x faces I (xsum) and from the y and z faces at column i
// (colsum), with the stencil offsets resolved at compile time.
template <int p, class T, class S>
struct AdjPop {
    const T *__restrict__ LX;
    const T *__restrict__ LY;
    const T *__restrict__ LZ;
    const StepParams<T, S> &P;
    const AdjRows &R;
    long long nfx, nfc;
    static constexpr int ax = cx(p), ay = cy(p), az = cz(p), rp = xrep(p);

    __device__ __forceinline__ T xsum(int I) const
    {
        const T tyo = p == 0 ? T(1) : P.ty_om, tym = P.ty_m, tzo = p == 0 ? T(1) : P.tz_om, tzm = P.tz_m;
        const T *base = LX + (long long)p * nfx;
        T s = (ay ? tyo : T(1)) * (az ? tzo : T(1)) * base[R.x(1, 1) + I];
        if (ay) s += tym * (az ? tzo : T(1)) * base[R.x(1, 1 + ay) + I];
        if (az) s += (ay ? tyo : T(1)) * tzm * base[R.x(1 + az, 1) + I];
        if (ay && az) s += tym * tzm * base[R.x(1 + az, 1 + ay) + I];
        return s;
    }
    // x weight of face I: anchor (which = 0) or other column (which = 1)
    __device__ __forceinline__ T xw(int I, int which) const
    {
        return p == 0 ? T(0.5) : __ldg(P.xw + (2 * rp + which) * P.xws + I);
    }
    // transverse x weight of the y / z faces at column i: own column (0) or column i - cx (1)
    __device__ __forceinline__ T tw(int i, int which) const { return __ldg(P.txw + (2 * rp + which) * P.xws + i); }
    __device__ __forceinline__ T colsum(int i) const
    {
        const T tyo = p == 0 ? T(1) : P.ty_om, tym = P.ty_m, tzo = p == 0 ? T(1) : P.tz_om, tzm = P.tz_m;
        const int c = i - 1;
        T sy, sz;
        {
            const T *base = LY + (long long)p * nfc;
            const T yo = p == 0 ? T(0.5) : P.yn_om[p], ym = p == 0 ? T(0.5) : P.yn_m[p];
            sy = yo * base[R.c(1, 1) + c] + ym * base[R.c(1, 0) + c];
            if (az) {
                sy = tzo * sy;
                sy += tzm * (yo * base[R.c(1 + az, 1) + c] + ym * base[R.c(1 + az, 0) + c]);
            }
        }
        {
            const T *base = LZ + (long long)p * nfc;
            const T zo = p == 0 ? T(0.5) : P.zn_om[p], zm = p == 0 ? T(0.5) : P.zn_m[p];
            sz = zo * base[R.c(1, 1) + c] + zm * base[R.c(0, 1) + c];
            if (ay) {
                sz = tyo * sz;
                sz += tym * (zo * base[R.c(1, 1 + ay) + c] + zm * base[R.c(0, 1 + ay) + c]);
            }
        }
        return sy + sz;
    }
    // interior column gi (1..nx); Ix2 / x2_anchor: the second x face holding the
    // column (face gi-1 as "other", face 0 as anchor for gi = 1 between walls,
    // face nx as "other" for gi = 1 when periodic); i2: the column i with
    // i - cx = gi of the y / z faces, 0 if none
    __device__ __forceinline__ T interior(int gi, int Ix2, bool x2_anchor, int i2) const
    {
        T acc = xw(gi, 0) * xsum(gi) + xw(Ix2, x2_anchor ? 0 : 1) * xsum(Ix2);
        if (ax) {
            acc += tw(gi, 0) * colsum(gi);
            if (i2 >= 1) acc += tw(i2, 1) * colsum(i2);
        } else {
            acc += colsum(gi);
        }
        return acc;
    }
    // wall ghost column 0 (side 0) or nx+1 (side 1): the other column of x face
    // 0 / nx, and the y / z faces at column 1 (cx > 0) / nx (cx < 0)
    __device__ __forceinline__ T ghost(int side) const
    {
        const int nx = P.nx;
        const int I = side ? nx : 0;
        T acc = xw(I, 1) * xsum(I);
        if (!side && ax > 0) acc += tw(1, 1) * colsum(1);
        if (side && ax < 0) acc += tw(nx, 1) * colsum(nx);
        return acc;
    }
};

// Adjoint received by the wall ghost columns (0 and nx+1) of f-bar-plus, per
// population, row and plane: GH[(side*19 + p) * ny*nz + (k-1)*ny + (j-1)].
// The gather folds it into columns 1, 2 and nx-1, nx with the extrapolation
// weights.
template <class T, class S, int p = 0>
__device__ __forceinline__ void adj_ghost_pops(const T *LX, const T *LY, const T *LZ, const StepParams<T, S> &P,
                                               const AdjRows &R, long long nfx, long long nfc, int side,
                                               T *__restrict__ GH, long long o)
{
    const AdjPop<p, T, S> A{LX, LY, LZ, P, R, nfx, nfc};
    GH[(long long)(side * NPOP + p) * P.ny * P.nz + o] = A.ghost(side);
    if constexpr (p + 1 < NPOP) adj_ghost_pops<T, S, p + 1>(LX, LY, LZ, P, R, nfx, nfc, side, GH, o);
}

template <class T, class S>
__global__ void __launch_bounds__(128) adj_ghost_kernel(const T *__restrict__ LX, const T *__restrict__ LY,
                                                        const T *__restrict__ LZ, T *__restrict__ GH,
                                                        const StepParams<T, S> P)
{
    const long long nyz = (long long)P.ny * P.nz;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * nyz) return;
    const int side = int(q / nyz);
    const long long o = q % nyz;
    const int j = int(o % P.ny) + 1, k = int(o / P.ny) + 1;
    const AdjRows R = adj_rows(j, k, P.nx, P.ny, P.nz);
    adj_ghost_pops<T, S>(LX, LY, LZ, P, R, adj_nface(0, P.nx, P.ny, P.nz), adj_nface(1, P.nx, P.ny, P.nz), side,
                         GH, o);
}

// Transposed interpolation stencil of every population at one cell (the
// part of mu that comes from the faces), stored population by population:
// MU[p * ncell + cell], cell = ((k-1)*ny + (j-1))*nx + (i-1).
template <class T, class S, int p, int pend>
__device__ __forceinline__ void adj_stencil_pops(const T *__restrict__ LX, const T *__restrict__ LY,
                                                 const T *__restrict__ LZ, const T *__restrict__ GH,
                                                 const StepParams<T, S> &P, const AdjRows &R, int i, long long o,
                                                 int Ix2, bool x2_anchor, long long nfx, long long nfc,
                                                 T *__restrict__ MU, long long cc)
{
    constexpr int ax = cx(p);
    // second column of the y / z faces: i + cx (periodic image, or none past a wall)
    int i2 = 0;
    if (ax) {
        i2 = i + ax;
        if (P.periodic_x) i2 = i2 < 1 ? P.nx : (i2 > P.nx ? 1 : i2);
        else if (i2 < 1 || i2 > P.nx) i2 = 0;
    }
    const AdjPop<p, T, S> A{LX, LY, LZ, P, R, nfx, nfc};
    T m = A.interior(i, Ix2, x2_anchor, i2);
    if (!P.periodic_x && (i <= 2 || i >= P.nx - 1)) {
        // wall ghosts: g0 = q0 fb1 + (1-q0) fb2, g_{nx+1} = q1 fb_nx + (1-q1) fb_{nx-1}
        const long long nyz = (long long)P.ny * P.nz;
        const T g0 = GH[(long long)p * nyz + o], g1 = GH[(long long)(NPOP + p) * nyz + o];
        if (i == 1) m += P.q0 * g0;
        if (i == 2) m += (T(1) - P.q0) * g0;
        if (i == P.nx) m += P.q1 * g1;
        if (i == P.nx - 1) m += (T(1) - P.q1) * g1;
    }
    MU[(long long)p * nfc + cc] = m;
    if constexpr (p + 1 < pend)
        adj_stencil_pops<T, S, p + 1, pend>(LX, LY, LZ, GH, P, R, i, o, Ix2, x2_anchor, nfx, nfc, MU, cc);
}

// Transposed stencil pass of the gather, split from the stage-(a) transpose so
// that it runs with few registers and many warps in flight (it is bound by
// the latency of its ~250 scattered loads per cell).  The populations are
// split into four groups, one per block (blockIdx.z = plane * 4 + group), so
// that each thread carries a quarter of the loads.
template <class T, class S>
__global__ void __launch_bounds__(128, 12) adj_stencil_kernel(const T *__restrict__ LX, const T *__restrict__ LY,
                                                             const T *__restrict__ LZ, const T *__restrict__ GH,
                                                             T *__restrict__ MU, const StepParams<T, S> P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1, k = blockIdx.z / 4 + 1, grp = blockIdx.z % 4;
    if (i > P.nx || j > P.ny) return;
    const AdjRows R = adj_rows(j, k, P.nx, P.ny, P.nz);
    const long long nfx = adj_nface(0, P.nx, P.ny, P.nz), nfc = adj_nface(1, P.nx, P.ny, P.nz);
    // second x face holding column i: face i-1 ("other" column), face 0 (anchor) at a wall,
    // face nx ("other") for i = 1 when periodic
    const bool wall1 = !P.periodic_x && i == 1;
    const int Ix2 = i == 1 ? (P.periodic_x ? P.nx : 0) : i - 1;
    const long long o = (long long)(k - 1) * P.ny + (j - 1);
    const long long cc = adj_cell(i, j, k, P.nx, P.ny);
    if (grp == 0) adj_stencil_pops<T, S, 0, 5>(LX, LY, LZ, GH, P, R, i, o, Ix2, wall1, nfx, nfc, MU, cc);
    else if (grp == 1) adj_stencil_pops<T, S, 5, 10>(LX, LY, LZ, GH, P, R, i, o, Ix2, wall1, nfx, nfc, MU, cc);
    else if (grp == 2) adj_stencil_pops<T, S, 10, 15>(LX, LY, LZ, GH, P, R, i, o, Ix2, wall1, nfx, nfc, MU, cc);
    else adj_stencil_pops<T, S, 15, NPOP>(LX, LY, LZ, GH, P, R, i, o, Ix2, wall1, nfx, nfc, MU, cc);
}

// mu = 4/3 lam' + (G^T L^T lamv); lam = (dA/df)^T mu - 1/3 lam'.
// d(face field)/d(phi at column gi) of x face I: (phi(i1) + phi(i2))/2
template <class T, class S>
__device__ __forceinline__ T xface_share(const StepParams<T, S> &P, int I, int gi)
{
    const int i1 = I == 0 ? (P.periodic_x ? P.nx : 1) : I;
    const int i2 = I + 1 <= P.nx ? I + 1 : (P.periodic_x ? 1 : P.nx);
    return T(0.5) * (T(i1 == gi) + T(i2 == gi));
}

template <class T, class S>
__global__ void __launch_bounds__(128) adj_gather_kernel(const S *__restrict__ f, const S *__restrict__ lam_next,
                                                         const T *__restrict__ LX, const T *__restrict__ LY,
                                                         const T *__restrict__ LZ, S *__restrict__ lam_out,
                                                         const T *__restrict__ LFX, const T *__restrict__ LFY,
                                                         const T *__restrict__ LFZ, double *__restrict__ dphi,
                                                         const T *__restrict__ MU, const StepParams<T, S> P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1, k = blockIdx.z + 1;
    if (i > P.nx || j > P.ny) return;
    const long long c = ((long long)(k - 1) * P.ny + (j - 1)) * P.pitch + (i - 1);
    T mu[NPOP];
    {
        const long long nfc = adj_nface(1, P.nx, P.ny, P.nz), cc = adj_cell(i, j, k, P.nx, P.ny);
#pragma unroll
        for (int p = 0; p < NPOP; ++p) mu[p] = T(4.0 / 3.0) * T(lam_next[p * P.ps + c]) + MU[p * nfc + cc];
    }
    // stage (a) transpose at this cell
    T v[NPOP];
#pragma unroll
    for (int p = 0; p < NPOP; ++p) v[p] = T(f[p * P.ps + c]);
    T r, jx, jy, jz;
    moments(v, r, jx, jy, jz);
    const T inv = recip(r);
    const T u0 = jx * inv, v0 = jy * inv, w0 = jz * inv;
    T Fx, Fy, Fz;
    cell_force(P, i - 1, j - 1, k - 1, Fx, Fy, Fz);
    const T Fc[3] = {Fx, Fy, Fz};
    const bool forced = P.force_on || P.perturb || P.ffield;
    T u = u0, vv = v0, w = w0, B = P.bw2;
    if (forced) {
        u = fma(P.hdt, Fx, u);
        vv = fma(P.hdt, Fy, vv);
        w = fma(P.hdt, Fz, w);
        B = fma(-P.bw0x3, fma(Fx, u, fma(Fy, vv, Fz * w)), P.bw2);
    }
    T fe[NPOP];
    feq_all(r, u, vv, w, fe);
    AdjJac<T> Jc = {T(0), T(0), T(0), {T(0), T(0), T(0)}};
    // with a field: L1 = sum mu_p c_{a,p} feq_p along the field axis a (Jc.Lf = sum mu_p feq_p)
    const int fax = P.ffaxis;
    const T wr0 = weight<T>(0) * r, wr1 = weight<T>(1) * r, wr2 = weight<T>(7) * r;
    T L1 = T(0);
#pragma unroll
    for (int p = 0; p < NPOP; ++p) {
        T K = P.Kb[p];
        if (P.perturb || P.ffield) {
            T cf = T(0);
            if (cx(p)) cf += cx(p) > 0 ? Fx : -Fx;
            if (cy(p)) cf += cy(p) > 0 ? Fy : -Fy;
            if (cz(p)) cf += cz(p) > 0 ? Fz : -Fz;
            K = P.bw0x3 * cf;
        }
        adj_accum(Jc, p, mu[p], wr_of(p, wr0, wr1, wr2), u, vv, w, B + K, fe[p]);
        if (P.ffield) {
            const int ca = fax == 0 ? cx(p) : (fax == 1 ? cy(p) : cz(p));
            if (ca) L1 = fma(ca > 0 ? mu[p] : -mu[p], fe[p], L1);
        }
    }
    T Gq[3], G[3];
    adj_G(Jc, u, vv, w, P.bw0x3, Fc, Gq, G);
    const T K0 = fma(-G[2], w0, fma(-G[1], v0, fma(-G[0], u0, Jc.S0)));
#pragma unroll
    for (int p = 0; p < NPOP; ++p) {
        const T out = P.bw1 * mu[p] + adj_g(p, K0, G) * inv - T(1.0 / 3.0) * T(lam_next[p * P.ps + c]);
        lam_out[p * P.ps + c] = S(out);
    }
    if (dphi && P.ffield) {
        // stage (a): d fb_p / dF_a = 3 bw0 (c_ap - u_a - hdt F_a) feq_p + coef_p hdt d feq_p / d u_a;
        // summed with mu: Sc = L1 - (u_a + hdt F_a) Lf and the second sum Gq_a
        const T ua = fax == 0 ? u : (fax == 1 ? vv : w);
        const T Fa = fax == 0 ? Fx : (fax == 1 ? Fy : Fz);
        const T Gqa = fax == 0 ? Gq[0] : (fax == 1 ? Gq[1] : Gq[2]);
        const T Sc = L1 - (ua + P.hdt * Fa) * Jc.Lf;
        // this step's contribution in the arithmetic type, accumulated over steps in FP64
        T g = P.bw0x3 * Sc + P.hdt * Gqa;
        // faces: the field enters each face through the mean over its two cells
        const int nx = P.nx, ny = P.ny, nz = P.nz;
        const int Il = P.periodic_x && i == 1 ? nx : i - 1;
        g += xface_share(P, Il, i) * LFX[adj_xface(Il, j, k, nx, ny)];
        g += xface_share(P, i, i) * LFX[adj_xface(i, j, k, nx, ny)];
        const int jl = j == 1 ? ny : j - 1, kl = k == 1 ? nz : k - 1;
        g += T(0.5) * (LFY[adj_cell(i, jl, k, nx, ny)] + LFY[adj_cell(i, j, k, nx, ny)]);
        g += T(0.5) * (LFZ[adj_cell(i, j, kl, nx, ny)] + LFZ[adj_cell(i, j, k, nx, ny)]);
        dphi[adj_cell(i, j, k, nx, ny)] += double(g);
    }
}

}  // namespace dg
