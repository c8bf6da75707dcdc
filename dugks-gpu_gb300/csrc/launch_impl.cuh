// Template bodies of the launchers declared in launch.cuh.
#pragma once
#include <algorithm>
#include <type_traits>
#include <cudaTypedefs.h>
#include "launch.cuh"

namespace dg {

template <class T, class S>
cudaError_t Kern<T, S>::fbar(const S *f, S *fb, const StepParams<T, S> &P, cudaStream_t st)
{
    if constexpr (std::is_same<S, float>::value) {
        // FP32: stage (a) writes the ghost layer itself (one launch); cells nx-1 and nx
        // must share a warp for the wall extrapolation: shift by one when nx = 1 (mod 32)
        const int xoff = (!P.periodic_x && P.nx % 32 == 1) ? 1 : 0;
        const int bx = P.nx + xoff >= 128 ? 128 : ((P.nx + xoff + 31) / 32) * 32;
        dim3 grid((P.nx + xoff + bx - 1) / bx, P.ny, P.nz);
        fbar_kernel<T, S, 1><<<grid, bx, 0, st>>>(f, fb, P, xoff);
    } else {
        const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
        dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
        if (sizeof(S) == 2 && !P.periodic_x) {
            // 16-bit storage between walls: stage (a) also writes the y / z images (the same
            // encoded values); the flux kernel forms the wall ghost columns in shared memory
            fbar_kernel<T, S, 2><<<grid, bx, 0, st>>>(f, fb, P, 0);
        } else {
            // FP64 and periodic 16-bit storage: the fused ghost writes cost more issue in
            // stage (a) (FP64 pipe, 16-bit encode) than the separate pass saves
            fbar_kernel<T, S, 0><<<grid, bx, 0, st>>>(f, fb, P, 0);
            const long long ghosts = 2LL * (P.ny + 2) * (P.nz + 2) + 2LL * P.nx * (P.nz + 2) + 2LL * P.nx * P.ny;
            fb_ghost_kernel<T, S><<<unsigned((ghosts + 255) / 256), 256, 0, st>>>(fb, P);
        }
    }
    return cudaGetLastError();
}

// Chunk length along z for a grid of `cols` CTA columns and `slots` resident
// CTAs: every chunk re-evaluates one bottom z face (1/(3k) of the face work
// for k planes) and refills the plane pipeline (about half a plane), and the
// last wave of CTAs may be partly empty; maximise
// (useful waves / launched waves) * (1 - 1/(3k)) * (1 - 1/(2k)) over chunk
// lengths k >= 4, keeping at least two waves where the grid allows it so that
// the scheduler can even out tiles of unequal work (partial rows).
static int choose_kchunk(int nz, long long cols, long long slots)
{
    const int kmin = std::min(nz, 4);
    const long long max_chunks = (nz + kmin - 1) / kmin;
    const double min_waves = std::min(2.0, double(cols * max_chunks) / double(slots));
    int best_k = nz;
    double best = -1.0;
    for (int k = kmin; k <= nz; ++k) {
        const long long nch = (nz + k - 1) / k;
        if (k > kmin && (nz + k - 2) / (k - 1) == nch) continue;  // same chunk count as k-1
        const double waves = double(cols * nch) / double(slots);
        if (waves < min_waves - 1e-9) break;  // fewer chunks only lower the wave count further
        const double fill = waves / std::ceil(waves);
        const double score = fill * (1.0 - 1.0 / (3.0 * k)) * (1.0 - 0.5 / k) * std::min(1.0, waves);
        if (score > best + 1e-9) {
            best = score;
            best_k = k;
        }
    }
    return best_k;
}

static int device_sms()
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

template <class T, class S>
int Kern<T, S>::flux_kchunk(const StepParams<T, S> &P)
{
    constexpr int W = TileCfg<T, S>::W, MB = TileCfg<T, S>::MINB;
    const int sms = device_sms();
    int occ = 1;
    if constexpr (TileCfg<T, S>::TMA)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, flux_tma_kernel<T, S, W, 0, MB, false>, 32 * W,
                                                      flux_tma_smem_bytes<T, S, W>());
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, flux_kernel<T, S, W, 0, MB, false>, 32 * W, 0);
    occ = std::max(occ, 1);
    const long long cols = (long long)((P.nx + 31) / 32) * ((P.ny + W - 2) / (W - 1));
    return choose_kchunk(P.nz, cols, (long long)sms * occ);
}

// one launch of the flux kernel variant <RECON, FF>
template <class T, class S, int RECON, bool FF>
static cudaError_t flux_launch(const S *fb, const S *f_in, S *f_out, const StepParams<T, S> &P,
                               const CUtensorMap *tmap, int kchunk, cudaStream_t st)
{
    constexpr int W = TileCfg<T, S>::W, MB = TileCfg<T, S>::MINB;
    dim3 grid((P.nx + 31) / 32, (P.ny + W - 2) / (W - 1), (P.nz + kchunk - 1) / kchunk);
    dim3 block(32, W);
    if constexpr (TileCfg<T, S>::TMA) {
        auto kern = flux_tma_kernel<T, S, W, RECON, MB, FF>;
        const int bytes = int(flux_tma_smem_bytes<T, S, W>());
        static bool attr_set = false;
        if (!attr_set) {
            const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e != cudaSuccess) return e;
            attr_set = true;
        }
        if (!tmap) return cudaErrorInvalidValue;
        kern<<<grid, block, bytes, st>>>(*tmap, f_in, f_out, P, kchunk);
    } else {
        (void)tmap;
        flux_kernel<T, S, W, RECON, MB, FF><<<grid, block, 0, st>>>(fb, f_in, f_out, P, kchunk);
    }
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::flux(const S *fb, const S *f_in, S *f_out, const StepParams<T, S> &P, int recon,
                             const CUtensorMap *tmap, cudaStream_t st)
{
    const int kchunk = flux_kchunk(P);
    const bool ff = P.ffield != nullptr;
    if (recon == 1)
        return ff ? flux_launch<T, S, 1, true>(fb, f_in, f_out, P, tmap, kchunk, st)
                  : flux_launch<T, S, 1, false>(fb, f_in, f_out, P, tmap, kchunk, st);
    return ff ? flux_launch<T, S, 0, true>(fb, f_in, f_out, P, tmap, kchunk, st)
              : flux_launch<T, S, 0, false>(fb, f_in, f_out, P, tmap, kchunk, st);
}

template <class T, class S>
cudaError_t Kern<T, S>::macro(const S *f, const StepParams<T, S> &P, double hdt, const double F[3], double *rho,
                              double *ux, double *uy, double *uz, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    macro_kernel<T, S><<<grid, bx, 0, st>>>(f, P, hdt, F[0], F[1], F[2], rho, ux, uy, uz);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::aos_to_soa(const double *src, S *dst, const StepParams<T, S> &P, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    aos_to_soa_kernel<T, S><<<grid, bx, 0, st>>>(src, dst, P);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::soa_to_aos(const S *src, double *dst, const StepParams<T, S> &P, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    soa_to_aos_kernel<T, S><<<grid, bx, 0, st>>>(src, dst, P);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::stats_partials(const S *f, const StepParams<T, S> &P, double hdt, const double F[3],
                                       double *partial, int nblocks, cudaStream_t st)
{
    const int bx = P.nx >= 256 ? 256 : ((P.nx + 31) / 32) * 32;
    dim3 grid(nblocks, (P.nx + bx - 1) / bx);
    stats_partials_kernel<T, S><<<grid, bx, 0, st>>>(f, P, hdt, F[0], F[1], F[2], partial);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::moments_partials(const S *f, const StepParams<T, S> &P, double *partial, int nblocks,
                                         cudaStream_t st)
{
    moments_partials_kernel<T, S><<<nblocks, 256, 0, st>>>(f, P, partial);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::adjoint(const S *f_n, S *fb, const S *lam_next, S *lam_out, T *lamv,
                                const StepParams<T, S> &P, double *dphi, const CUtensorMap *tmap_adj,
                                cudaStream_t st)
{
    if constexpr (!std::is_same<T, S>::value) {
        return cudaErrorNotSupported;
    } else {
        cudaError_t e = fbar(f_n, fb, P, st);
        if (e != cudaSuccess) return e;
        const long long nfx = adj_nface(0, P.nx, P.ny, P.nz), nfc = adj_nface(1, P.nx, P.ny, P.nz);
        T *LX = lamv, *LY = lamv + NPOP * nfx, *LZ = LY + NPOP * nfc;
        T *LFX = LZ + NPOP * nfc, *LFY = LFX + nfx, *LFZ = LFY + nfc;  // per-face dJ/dF (force field)
        if constexpr (TileCfg<T, S>::TMA) {
            // +x, +y, +z faces of every cell from the TMA-staged tile; x faces I = 0 apart
            if (!tmap_adj) return cudaErrorInvalidValue;
            constexpr int W = AdjCfg<T, S>::W, MB = AdjCfg<T, S>::MINB;
            auto kern = adj_faces_tma_kernel<T, S, W, MB>;
            const size_t smem = adj_faces_tma_smem_bytes<T, S, W>();
            static bool attr_set = false;
            if (!attr_set) {
                e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                attr_set = true;
            }
            int occ = 1;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * W, smem);
            const long long cols = (long long)((P.nx + 31) / 32) * ((P.ny + W - 1) / W);
            const int kchunk = choose_kchunk(P.nz, cols, (long long)device_sms() * std::max(occ, 1));
            dim3 grid((P.nx + 31) / 32, (P.ny + W - 1) / W, (P.nz + kchunk - 1) / kchunk);
            kern<<<grid, dim3(32, W), smem, st>>>(*tmap_adj, lam_next, LX, LY, LZ, LFX, LFY, LFZ, P, kchunk);
            // one warp per block: the few wall faces spread over every SM
            const long long n0 = (long long)P.ny * P.nz;
            adj_face_kernel<T, S, 0><<<unsigned((n0 + 31) / 32), 32, 0, st>>>(fb, lam_next, LX, LFX, P, 1);
        } else {
            adj_face_kernel<T, S, 0><<<unsigned((nfx + 127) / 128), 128, 0, st>>>(fb, lam_next, LX, LFX, P, 0);
            adj_face_kernel<T, S, 1><<<unsigned((nfc + 127) / 128), 128, 0, st>>>(fb, lam_next, LY, LFY, P, 0);
            adj_face_kernel<T, S, 2><<<unsigned((nfc + 127) / 128), 128, 0, st>>>(fb, lam_next, LZ, LFZ, P, 0);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        T *GH = LFZ + nfc;  // wall-ghost sums, 2 * 19 * ny * nz
        if (!P.periodic_x) {
            const long long ng = 2LL * P.ny * P.nz;
            adj_ghost_kernel<T, S><<<unsigned((ng + 31) / 32), 32, 0, st>>>(LX, LY, LZ, GH, P);
        }
        T *MU = GH + 2LL * NPOP * P.ny * P.nz;  // transposed-stencil sums, 19 * nx * ny * nz
        // 128-thread blocks of whole warps over x (one to four rows when nx < 128), so
        // that narrow grids leave no lanes idle
        const int bx = P.nx >= 128 ? 128 : (P.nx + 31) / 32 * 32, by = 128 / bx;
        const dim3 blk(bx, by), grid((P.nx + bx - 1) / bx, (P.ny + by - 1) / by, P.nz);
        adj_stencil_kernel<T, S><<<dim3(grid.x, grid.y, 4 * P.nz), blk, 0, st>>>(LX, LY, LZ, GH, MU, P);
        adj_gather_kernel<T, S><<<grid, blk, 0, st>>>(f_n, lam_next, LX, LY, LZ, lam_out, LFX, LFY, LFZ, dphi, MU, P);
        return cudaGetLastError();
    }
}

template <class T, class S>
int Kern<T, S>::make_tmap(const S *fb, int nx, int ny, int nz, int pitch_b, long long ps_b, int box_rows,
                          CUtensorMap *out)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return -1;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const CUtensorMapDataType dt = sizeof(S) == 8   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                   : sizeof(S) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : std::is_same<S, __half>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                    : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    const cuuint64_t dims[4] = {cuuint64_t(nx + 2), cuuint64_t(ny + 2), cuuint64_t(nz + 2), cuuint64_t(NPOP)};
    const cuuint64_t strides[3] = {cuuint64_t(pitch_b) * sizeof(S), cuuint64_t(pitch_b) * (ny + 2) * sizeof(S),
                                   cuuint64_t(ps_b) * sizeof(S)};
    const cuuint32_t box[4] = {cuuint32_t(TmaTile<S>::BXT), cuuint32_t(box_rows), 1u, cuuint32_t(NPOP)};
    const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
    const CUresult r = encode(out, dt, 4, const_cast<S *>(fb), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : int(r);
}

}  // namespace dg
