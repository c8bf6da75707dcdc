/*
 * Runs the reference's own, unmodified CUDA-C step kernels (compiled from
 * Kairzhan/DUGKS-GPU src/dugks.cu into oracle/_ref/dugks_f64.cubin and
 * dugks_f32.cubin by oracle/build_ref.sh) on the GPU, single rank, in the
 * launch order and with the launch shapes of dugks_step (src/dugks.cu:322-391).
 *
 * TEST INFRASTRUCTURE ONLY: the reference oracle for parity tests, golden
 * fixture generation and the reference-GPU timing; never part of the product.
 *
 * The parameter structs below repeat the field order of the reference's
 * DugksParameters / NumericalParameters / HydroParameters
 * (src/dugks.cu:36-61) because the reference kernels read them through
 * pointers; their values follow init_dugks (src/dugks.cu:101-179).
 * The single-rank z "exchange" (src/parallel.cu:192-200, CUDA-aware path with
 * zprev = znext = self) is two device-to-device plane copies.
 */
#include <cuda.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

template <class R>
struct RefDugksParameters {
    R visc, RT, hdt, bw0, bw1, bw2, fw0, fw1, fw2, qw1, qw2, gw1, gw2;
    R *tp;
    int *cixyzo;
};
template <class R>
struct RefNumericalParameters {
    int npop, lx, ly, lz, nx, ny, nz;
    R dx, dy, dz, dt, xwidth, ywidth, zwidth, zoffset;
    int periods[3];
};
template <class R>
struct RefHydroParameters {
    R ambient_fx, ambient_fy, ambient_fz;
};

struct Module {
    CUmodule mod = nullptr;
    CUfunction calc_force = nullptr, calc_perturb_force = nullptr, calc_fb1 = nullptr, extend_fb_x = nullptr,
               extend_fb_x_wall = nullptr, extend_fb_y = nullptr, calc_fx_tri = nullptr, calc_fx = nullptr,
               calc_macro = nullptr;
};

CUcontext g_ctx = nullptr;
Module g_mod[2];  // [0] fp64, [1] fp32
std::string g_err;

#define DRV(call)                                                            \
    do {                                                                     \
        CUresult r_ = (call);                                                \
        if (r_ != CUDA_SUCCESS) {                                            \
            const char *s_ = nullptr;                                        \
            cuGetErrorString(r_, &s_);                                       \
            g_err = std::string(#call) + ": " + (s_ ? s_ : "?");             \
            return -4;                                                       \
        }                                                                    \
    } while (0)

// Itanium-mangled kernel names start with _Z<len><name>
bool name_is(const char *mangled, const char *plain)
{
    char pre[96];
    std::snprintf(pre, sizeof(pre), "_Z%zu%s", std::strlen(plain), plain);
    return std::strncmp(mangled, pre, std::strlen(pre)) == 0;
}

int ensure_ctx()
{
    if (g_ctx) return 0;
    DRV(cuInit(0));
    CUdevice dev;
    DRV(cuDeviceGet(&dev, 0));
    DRV(cuDevicePrimaryCtxRetain(&g_ctx, dev));
    DRV(cuCtxSetCurrent(g_ctx));
    return 0;
}

}  // namespace

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }

/* Load one of the reference cubins; prec 0 = FP64 build, 1 = PREC4 build. */
int ref_open(const char *cubin_path, int prec)
{
    if (prec < 0 || prec > 1) return -6;
    int rc = ensure_ctx();
    if (rc) return rc;
    Module &m = g_mod[prec];
    if (m.mod) return 0;
    DRV(cuModuleLoad(&m.mod, cubin_path));
    unsigned int n = 0;
    DRV(cuModuleGetFunctionCount(&n, m.mod));
    std::vector<CUfunction> fns(n);
    DRV(cuModuleEnumerateFunctions(fns.data(), n, m.mod));
    for (CUfunction fn : fns) {
        const char *name = nullptr;
        DRV(cuFuncGetName(&name, fn));
        if (name_is(name, "calc_force")) m.calc_force = fn;
        else if (name_is(name, "calc_perturb_force")) m.calc_perturb_force = fn;
        else if (name_is(name, "calc_fb1")) m.calc_fb1 = fn;
        else if (name_is(name, "extend_fb_x")) m.extend_fb_x = fn;
        else if (name_is(name, "extend_fb_x_wall")) m.extend_fb_x_wall = fn;
        else if (name_is(name, "extend_fb_y")) m.extend_fb_y = fn;
        else if (name_is(name, "calc_fx_tri")) m.calc_fx_tri = fn;
        else if (name_is(name, "calc_fx")) m.calc_fx = fn;
        else if (name_is(name, "calc_macro")) m.calc_macro = fn;
    }
    if (!m.calc_force || !m.calc_perturb_force || !m.calc_fb1 || !m.extend_fb_x || !m.extend_fb_x_wall ||
        !m.extend_fb_y || !m.calc_fx_tri || !m.calc_fx || !m.calc_macro) {
        g_err = "reference kernel missing from cubin";
        return -1;
    }
    return 0;
}

typedef struct {
    int nx, ny, nz;
    int periods[3];
    int perturb;
    int recon;             /* 0 calc_fx_tri (dugks_step), 1 calc_fx */
    double CFL, xwidth, ywidth, zwidth, visc; /* as parsed by std::stof, widened */
    double F[3];
} ref_cfg;

}  // extern "C"

namespace {

template <class R>
int run_impl(const Module &m, const ref_cfg *c, double *f_host, int istep0, int nsteps, double *ms_out)
{
    const int lx = c->nx, ly = c->ny, lz = c->nz;
    if (lx % 16 || ly % 8 || lz % 2) {
        g_err = "reference launch shapes need nx%16==0, ny%8==0, nz%2==0";
        return -3;
    }
    if (!c->periods[1] || !c->periods[2]) {
        g_err = "reference supports walls in x only";
        return -7;
    }
    // Numerics (src/numerics.cu:101-105) and init_dugks (src/dugks.cu:101-125)
    const R RT = 1. / 3.;
    RefNumericalParameters<R> np;
    std::memset(&np, 0, sizeof(np));
    np.npop = 19; np.lx = lx; np.ly = ly; np.lz = lz; np.nx = lx; np.ny = ly; np.nz = lz;
    const R xwidth = R(c->xwidth), ywidth = R(c->ywidth), zwidth = R(c->zwidth), CFL = R(c->CFL);
    np.dx = xwidth / lx; np.dy = ywidth / ly; np.dz = zwidth / lz;
    np.dt = CFL * np.dx / std::sqrt(6 * RT);
    np.xwidth = xwidth; np.ywidth = ywidth; np.zwidth = zwidth; np.zoffset = 0;
    for (int a = 0; a < 3; ++a) np.periods[a] = c->periods[a];
    const R dt = np.dt, visc = R(c->visc), tau = visc / RT;
    R hdt = dt / 2.;
    RefDugksParameters<R> dp;
    std::memset(&dp, 0, sizeof(dp));
    dp.visc = visc; dp.RT = RT; dp.hdt = hdt;
    dp.bw0 = (3. * tau * hdt) / (2. * tau + dt);
    dp.bw1 = (2. * tau - hdt) / (2. * tau + dt);
    dp.bw2 = 3. * hdt / (2. * tau + dt);
    dp.gw1 = 2. * tau / (2. * tau + dt);
    dp.gw2 = dt / (2. * tau + dt);
    dp.qw1 = (2. * tau + dt) / (2. * tau);
    dp.qw2 = -dt / (2. * tau);
    dp.fw0 = tau * hdt / (2. * tau + hdt);
    dp.fw1 = 2. * tau / (2. * tau + hdt);
    dp.fw2 = hdt / (2. * tau + hdt);
    RefHydroParameters<R> hp = {R(c->F[0]), R(c->F[1]), R(c->F[2])};
    static const int cix[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
    static const int ciy[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
    static const int ciz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    static const int opp[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
    int cixyzo[76];
    R tp[19];
    for (int ip = 0; ip < 19; ++ip) {
        cixyzo[ip] = opp[ip]; cixyzo[ip + 19] = cix[ip]; cixyzo[ip + 38] = ciy[ip]; cixyzo[ip + 57] = ciz[ip];
        tp[ip] = ip == 0 ? R(1.0 / 3.0) : (ip <= 6 ? R(1.0 / 18.0) : R(1.0 / 36.0));
    }
    const size_t g = size_t(lx + 2) * (ly + 2) * (lz + 2);
    CUdeviceptr d_f, d_fb, d_fx, d_fy, d_fz, d_tp, d_cix, d_np, d_dp, d_hp;
    DRV(cuMemAlloc(&d_f, 19 * g * sizeof(R)));
    DRV(cuMemAlloc(&d_fb, 19 * g * sizeof(R)));
    DRV(cuMemAlloc(&d_fx, g * sizeof(R)));
    DRV(cuMemAlloc(&d_fy, g * sizeof(R)));
    DRV(cuMemAlloc(&d_fz, g * sizeof(R)));
    DRV(cuMemAlloc(&d_tp, sizeof(tp)));
    DRV(cuMemAlloc(&d_cix, sizeof(cixyzo)));
    DRV(cuMemAlloc(&d_np, sizeof(np)));
    DRV(cuMemAlloc(&d_dp, sizeof(dp)));
    DRV(cuMemAlloc(&d_hp, sizeof(hp)));
    dp.tp = reinterpret_cast<R *>(d_tp);
    dp.cixyzo = reinterpret_cast<int *>(d_cix);
    DRV(cuMemsetD8(d_fb, 0, 19 * g * sizeof(R)));
    DRV(cuMemsetD8(d_fx, 0, g * sizeof(R)));
    DRV(cuMemsetD8(d_fy, 0, g * sizeof(R)));
    DRV(cuMemsetD8(d_fz, 0, g * sizeof(R)));
    DRV(cuMemcpyHtoD(d_tp, tp, sizeof(tp)));
    DRV(cuMemcpyHtoD(d_cix, cixyzo, sizeof(cixyzo)));
    DRV(cuMemcpyHtoD(d_np, &np, sizeof(np)));
    DRV(cuMemcpyHtoD(d_dp, &dp, sizeof(dp)));
    DRV(cuMemcpyHtoD(d_hp, &hp, sizeof(hp)));
    std::vector<R> hf(19 * g);
    for (size_t q = 0; q < hf.size(); ++q) hf[q] = R(f_host[q]);
    DRV(cuMemcpyHtoD(d_f, hf.data(), hf.size() * sizeof(R)));

    CUevent e0, e1;
    DRV(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    DRV(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    const int smem = 19 * (8 + 2) * (4 + 2) * (2 + 2) * int(sizeof(R));  // src/dugks.cu:382
    const size_t plane = size_t(19) * (lx + 2) * (ly + 2) * sizeof(R);
    DRV(cuEventRecord(e0, 0));
    for (int s = 0; s < nsteps; ++s) {
        int step = istep0 + s;
        {
            void *args[] = {&step, &d_fx, &d_fy, &d_fz, &d_np, &d_dp, &d_hp};
            DRV(cuLaunchKernel(c->perturb ? m.calc_perturb_force : m.calc_force, lx / 16, ly / 8, lz, 16, 8, 1, 0, 0,
                               args, nullptr));
        }
        {
            void *args[] = {&d_fb, &d_f, &d_fx, &d_fy, &d_fz, &d_np, &d_dp};
            DRV(cuLaunchKernel(m.calc_fb1, lx / 16, ly / 8, lz, 16, 8, 1, 0, 0, args, nullptr));
        }
        {
            void *args[] = {&d_fb, &d_np, &d_dp};
            DRV(cuLaunchKernel(c->periods[0] ? m.extend_fb_x : m.extend_fb_x_wall, 1, (ly + 2 + 16) / 16,
                               (lz + 2 + 16) / 16, 1, 16, 16, 0, 0, args, nullptr));
            DRV(cuLaunchKernel(m.extend_fb_y, (lx + 2 + 16) / 16, 1, (lz + 2 + 16) / 16, 16, 1, 16, 0, 0, args,
                               nullptr));
        }
        // exchange(fb) with itself: plane 1 -> lz+1, plane lz -> 0
        DRV(cuMemcpyDtoDAsync(d_fb + plane * (lz + 1), d_fb + plane * 1, plane, 0));
        DRV(cuMemcpyDtoDAsync(d_fb + plane * 0, d_fb + plane * lz, plane, 0));
        {
            void *args[] = {&d_f, &d_fb, &d_np, &d_dp, &d_hp};
            DRV(cuLaunchKernel(c->recon ? m.calc_fx : m.calc_fx_tri, lx / 8, ly / 4, lz / 2, 8, 4, 2, smem, 0, args,
                               nullptr));
        }
    }
    DRV(cuEventRecord(e1, 0));
    DRV(cuEventSynchronize(e1));
    float ms = 0;
    DRV(cuEventElapsedTime(&ms, e0, e1));
    if (ms_out) *ms_out = nsteps > 0 ? double(ms) / nsteps : 0.0;
    DRV(cuCtxSynchronize());
    DRV(cuMemcpyDtoH(hf.data(), d_f, hf.size() * sizeof(R)));
    for (size_t q = 0; q < hf.size(); ++q) f_host[q] = double(hf[q]);
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    CUdeviceptr all[] = {d_f, d_fb, d_fx, d_fy, d_fz, d_tp, d_cix, d_np, d_dp, d_hp};
    for (CUdeviceptr p : all) cuMemFree(p);
    return 0;
}

}  // namespace

extern "C" {

/* nsteps reference steps istep0.. on the ghosted AoS state f (double on the
 * host whatever the build; converted to the build's real).  ms_per_step gets
 * the CUDA-event time per step. */
int ref_run(int prec, const ref_cfg *c, double *f_ghosted, int istep0, int nsteps, double *ms_per_step)
{
    if (prec < 0 || prec > 1 || !c || !f_ghosted) return -6;
    if (!g_mod[prec].mod) {
        g_err = "ref_open not called for this precision";
        return -6;
    }
    return prec == 0 ? run_impl<double>(g_mod[0], c, f_ghosted, istep0, nsteps, ms_per_step)
                     : run_impl<float>(g_mod[1], c, f_ghosted, istep0, nsteps, ms_per_step);
}

}  // extern "C"
