// Host side of the engine: configuration, mesh and coefficient tables, device
// state, step dispatch, macro output, statistics and checkpoint I/O, behind the
// C ABI of include/dugks_gb300.h.
//
// Reference counterparts (Kairzhan/DUGKS-GPU):
//   Numerics::init_numerics  src/numerics.cu:62-106   -> load_config()
//   init_parallel (single rank, periods) src/parallel.cu:75-180
//   init_cuda                src/cuda.cu:13-33        (gpusPerThread parsed, current device used)
//   init_dugks               src/dugks.cu:95-302      -> build_tables(), set_initial()
//   dugks_step               src/dugks.cu:322-391     -> dg_step()
//   upload_macro / copy_vel / copy_ddf  src/dugks.cu:311-320, 393-416
//   dump / read_dump         src/output.cu:22-89
//   output_2d / save_tecplot_serial / statistics_serial  src/output.cu:118-334
//   stretched mesh           src/fortran/channel/src/dugks.cuf:107-138, run/mesh.py:21-25
//   spectral statistics      src/fortran/dhit/src/stat.f90:5-205, main.cuf:83-119 -> dg_spectral_stats()
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>
#include <algorithm>

#include <cufft.h>
#include <dlfcn.h>

#include "../../include/dugks_gb300.h"
#include "config.h"
#include "launch.cuh"
#include "spectral_kernels.cuh"

using namespace dg;

namespace {

size_t storage_bytes(int prec) { return prec == DG_PREC_FP64 ? 8 : (prec == DG_PREC_FP32 ? 4 : 2); }

thread_local std::string g_create_error;

// Coefficients computed in the reference's `real` (R = double, or float for
// the PREC4 build), expression by expression (src/numerics.cu:101-105,
// src/dugks.cu:101-125, src/fortran/channel/src/dugks.cuf:138-153).
template <class R>
struct RefCoef {
    R RT, visc, tau, dx, dy, dz, dt, hdt;
    R bw0, bw1, bw2, fw0, fw1, fw2;
    R F[3];
};

template <class R>
RefCoef<R> ref_coef(double visc, double cfl, double xw, double yw, double zw, int nx, int ny, int nz,
                    const double F[3], bool stretched, double dxx1)
{
    RefCoef<R> c;
    c.RT = R(1. / 3.);
    c.visc = R(visc);
    const R xwidth = R(xw), ywidth = R(yw), zwidth = R(zw), CFL = R(cfl);
    c.dx = xwidth / nx;
    c.dy = ywidth / ny;
    c.dz = zwidth / nz;
    if (stretched)
        c.dt = CFL * R(dxx1) / std::sqrt(R(6) * c.RT);
    else
        c.dt = CFL * c.dx / std::sqrt(R(6) * c.RT);
    const R dt = c.dt;
    c.tau = c.visc / c.RT;
    const R tau = c.tau;
    c.hdt = dt / 2.;
    const R hdt = c.hdt;
    c.bw0 = (3. * tau * hdt) / (2. * tau + dt);
    c.bw1 = (2. * tau - hdt) / (2. * tau + dt);
    c.bw2 = 3. * hdt / (2. * tau + dt);
    c.fw0 = tau * hdt / (2. * tau + hdt);
    c.fw1 = 2. * tau / (2. * tau + hdt);
    c.fw2 = hdt / (2. * tau + hdt);
    for (int a = 0; a < 3; ++a) c.F[a] = R(F[a]);
    return c;
}

// splitmix64 finaliser: the synthetic-input generator's RNG
uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// uniform in [-1, 1) from (seed, cell, component)
double rng_sym(uint64_t seed, uint64_t cell, int comp)
{
    const uint64_t z = splitmix64(seed * 0xD1B54A32D192ED03ull + cell * 3ull + uint64_t(comp));
    return double(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

}  // namespace

struct dg_ctx {
    std::string err;
    std::string workdir;
    // configuration (reference keys)
    std::string casename;
    int nx = 0, ny = 0, nz = 0;
    int istep0 = 1, nsteps = 0, noutput2 = 1, noutput3 = 1, ndump = 1, restart = 0, nrestart = 0, perturb = 0;
    int periodic[3] = {1, 1, 1};
    int gpus_per_thread = 1;
    double cfl = 0, xwidth = 0, ywidth = 0, zwidth = 0, visc = 0, F[3] = {0, 0, 0};
    // extension keys
    int prec = DG_PREC_FP64;
    int mesh = 0;           // 0 uniform, 1 tanh, 2 file
    int recon = 0;          // 0 trilinear
    int stochastic = 1;     // 16-bit forms: stochastic rounding of the stored deviations
    double mesh_alpha = 0.85;
    double xwidth_d = 0;    // xwidth parsed in double precision (stretched meshes)
    double tg_u0 = 0.1;     // velocity amplitude of case=tg_eq (the reference's fixed 0.1 by default)
    std::string mesh_file;
    // derived
    int pitch = 0;
    long long ps = 0;
    int pitch_b = 0;        // f-bar-plus: x ghost columns stored
    long long ps_b = 0;
    std::vector<double> xf, xc, dxx;  // stretched mesh, xc/dxx indexed 0..nx+1
    RefCoef<double> c64{};
    RefCoef<float> c32{};
    float dev_w[19] = {}, dev_s[19] = {};
    // device memory
    int device = 0;
    cudaStream_t stream = nullptr;
    void *f = nullptr, *fb = nullptr;
    void *tab = nullptr;          // xw | txw | cxu | pert_x | pert_y | pert_z | cxuf | cw | gw (T-typed)
    size_t tab_off[9] = {};
    double *macro = nullptr;      // rho|ux|uy|uz ghosted
    double *scratch = nullptr;    // statistics partial sums / moments partials
    size_t scratch_bytes = 0;
    void *adj = nullptr;          // per-face adjoint scratch (allocated on first dg_adjoint_step)
    void *ffield = nullptr;       // body-force field phi, T-typed, [k][j][pitch] (dg_set_force_field)
    int ffaxis = 0;
    double *dphi = nullptr;       // accumulated dJ/dphi, [k][j][i] (adjoint steps with a field)
    double *acc = nullptr;        // running sums of the per-x statistics (dg_stats_accumulate)
    int *dev_err = nullptr;       // device error flag written by the kernels (TMA wait time-outs)
    CUtensorMap tmap;             // f-bar-plus tensor map of the TMA flux kernel (64-byte aligned type)
    CUtensorMap tmap_adj;         // the same array with the adjoint face kernel's box
    bool have_tmap = false;
    // spectral statistics (dg_spectral_stats): U, V, W (complex), ET, ETS, partial sums; the
    // modes grouped by shell (spec_order, spec_off); the cuFFT plan
    void *spec = nullptr;
    int *spec_order = nullptr;
    int *spec_off = nullptr;
    int spec_nbins = 0;
    int spec_plan = 0;
    bool spec_have_plan = false;
    // CUDA graph of kGraphSteps steps, replayed by dg_run when the step's launch
    // parameters do not change from step to step (captured on a private stream)
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t step_graph = nullptr;
    long long acc_count = 0;
    bool macro_valid = false;

    ~dg_ctx()
    {
        if (f) cudaFree(f);
        if (fb) cudaFree(fb);
        if (tab) cudaFree(tab);
        if (macro) cudaFree(macro);
        if (scratch) cudaFree(scratch);
        if (adj) cudaFree(adj);
        if (ffield) cudaFree(ffield);
        if (dphi) cudaFree(dphi);
        if (acc) cudaFree(acc);
        if (dev_err) cudaFree(dev_err);
        if (step_graph) cudaGraphExecDestroy(step_graph);
        if (cap_stream) cudaStreamDestroy(cap_stream);
        if (spec) cudaFree(spec);
        if (spec_order) cudaFree(spec_order);
        if (spec_off) cudaFree(spec_off);
        release_spec_plan();
    }
    void release_spec_plan();
    void drop_graph()
    {
        if (step_graph) cudaGraphExecDestroy(step_graph);
        step_graph = nullptr;
    }
    int fail(int code, const std::string &msg)
    {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return DG_ERR_CUDA;
    }
    size_t ncell() const { return size_t(nx) * ny * nz; }
    size_t ghosted() const { return size_t(nx + 2) * (ny + 2) * (nz + 2); }
    double hdt() const { return prec == DG_PREC_FP64 ? c64.hdt : double(c32.hdt); }
};

namespace {

#define CK(call, what)                                    \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return h->cuda_fail(e_, what); \
    } while (0)

// ---------------------------------------------------------------------------
// configuration
// ---------------------------------------------------------------------------
int load_config(dg_ctx *h, const ConfigFile &cf)
{
    std::string e;
    auto need_i = [&](const char *k, int &v) { return cf.get_int(k, v, e); };
    auto need_f = [&](const char *k, double &v) { return cf.get_float(k, v, e); };
    if (!cf.get_string("case", h->casename, e)) return h->fail(DG_ERR_CONFIG, e);
    if (!need_f("CFL", h->cfl) || !need_f("xwidth", h->xwidth) || !need_f("ywidth", h->ywidth) ||
        !need_f("zwidth", h->zwidth) || !need_i("nx", h->nx) || !need_i("ny", h->ny) || !need_i("nz", h->nz) ||
        !need_i("istep0", h->istep0) || !need_i("nsteps", h->nsteps) || !need_i("noutput2", h->noutput2) ||
        !need_i("noutput3", h->noutput3) || !need_i("ndump", h->ndump) || !need_i("restart", h->restart) ||
        !need_i("nrestart", h->nrestart) || !need_i("perturb", h->perturb) || !need_f("visc", h->visc) ||
        !need_f("ambient_fx", h->F[0]) || !need_f("ambient_fy", h->F[1]) || !need_f("ambient_fz", h->F[2]) ||
        !need_i("periods_x", h->periodic[0]) || !need_i("periods_y", h->periodic[1]) ||
        !need_i("periods_z", h->periodic[2]) || !need_i("gpusPerThread", h->gpus_per_thread))
        return h->fail(DG_ERR_CONFIG, e);
    // extension keys
    const std::string prec = cf.opt_string("precision", "fp64");
    if (prec == "fp64") h->prec = DG_PREC_FP64;
    else if (prec == "fp32") h->prec = DG_PREC_FP32;
    else if (prec == "fp16") h->prec = DG_PREC_FP16;
    else if (prec == "bf16") h->prec = DG_PREC_BF16;
    else return h->fail(DG_ERR_CONFIG, "config key 'precision': expected fp64, fp32, fp16 or bf16, got '" + prec + "'");
    const std::string mesh = cf.opt_string("mesh", "uniform");
    if (mesh == "uniform") h->mesh = 0;
    else if (mesh == "tanh") h->mesh = 1;
    else if (mesh == "file") h->mesh = 2;
    else return h->fail(DG_ERR_CONFIG, "config key 'mesh': expected uniform, tanh or file, got '" + mesh + "'");
    if (!cf.opt_double("mesh_alpha", 0.85, h->mesh_alpha, e)) return h->fail(DG_ERR_CONFIG, e);
    // the stretched-mesh channel holds its width in double precision (a -r8
    // parameter, src/fortran/channel/src/dugks.cuf:18); the mesh and its upper
    // ghost use that value rather than the std::stof-rounded one
    if (!cf.opt_double("xwidth", h->xwidth, h->xwidth_d, e)) return h->fail(DG_ERR_CONFIG, e);
    if (!cf.opt_double("tg_u0", 0.1, h->tg_u0, e)) return h->fail(DG_ERR_CONFIG, e);
    h->mesh_file = cf.opt_string("mesh_file", "mesh.txt");
    const std::string rounding = cf.opt_string("rounding", "stochastic");
    if (rounding == "stochastic") h->stochastic = 1;
    else if (rounding == "nearest") h->stochastic = 0;
    else return h->fail(DG_ERR_CONFIG, "config key 'rounding': expected stochastic or nearest, got '" + rounding + "'");
    const std::string recon = cf.opt_string("recon", "trilinear");
    if (recon == "trilinear") h->recon = 0;
    else if (recon == "gradient") h->recon = 1;
    else return h->fail(DG_ERR_CONFIG, "config key 'recon': expected trilinear or gradient, got '" + recon + "'");

    // validation the reference does not do (src/checks.cu:17-19 asserts only)
    if (h->nx < 3 || h->ny < 1 || h->nz < 1) return h->fail(DG_ERR_SHAPE, "grid must have nx>=3, ny>=1, nz>=1");
    if ((long long)h->nx * h->ny * h->nz > (1LL << 31)) return h->fail(DG_ERR_SHAPE, "grid larger than 2^31 cells");
    if (h->periodic[1] == 0) return h->fail(DG_ERR_UNSUPPORTED, "wall BC is not supported in y-direction");
    if (h->periodic[2] == 0) return h->fail(DG_ERR_UNSUPPORTED, "wall BC is not supported in z-direction");
    if (h->gpus_per_thread < 1) return h->fail(DG_ERR_CONFIG, "gpusPerThread must be >= 1");
    if (h->noutput2 < 1 || h->ndump < 1) return h->fail(DG_ERR_CONFIG, "noutput2 and ndump must be >= 1");
    if (!(h->visc > 0)) return h->fail(DG_ERR_CONFIG, "visc must be > 0");
    if (!(h->cfl > 0) || !(h->xwidth > 0) || !(h->ywidth > 0) || !(h->zwidth > 0))
        return h->fail(DG_ERR_CONFIG, "CFL and the widths must be > 0");
    if (h->mesh != 0 && h->periodic[0]) return h->fail(DG_ERR_CONFIG, "a stretched mesh needs walls in x (periods_x=0)");
    return DG_OK;
}

// tanh-stretched faces (src/fortran/channel/run/mesh.py:21-25) or a mesh file
// of nx+1 face positions; centres, widths and mirrored ghosts as
// src/fortran/channel/src/dugks.cuf:114-121.
int build_mesh(dg_ctx *h)
{
    const int nx = h->nx;
    h->xf.assign(nx + 1, 0.0);
    if (h->mesh == 1) {
        const double a = h->mesh_alpha, L = h->xwidth_d;
        if (!(a > 0 && a < 1)) return h->fail(DG_ERR_CONFIG, "mesh_alpha must lie in (0, 1)");
        for (int k = 0; k <= nx; ++k) {
            const double eta = -1. + 2. * ((k + 0) - 0.0) / nx;
            h->xf[k] = L / (2. * a) * std::tanh(eta * 0.5 * (std::log(1. + a) - std::log(1. - a))) + 0.5 * L;
        }
    } else if (h->mesh == 2) {
        std::string path = h->mesh_file;
        if (!path.empty() && path[0] != '/') path = h->workdir + "/" + path;
        std::ifstream in(path);
        if (!in) return h->fail(DG_ERR_IO, "cannot open mesh file '" + path + "'");
        for (int k = 0; k <= nx; ++k)
            if (!(in >> h->xf[k])) return h->fail(DG_ERR_IO, "mesh file '" + path + "' has fewer than nx+1 values");
    } else {
        for (int k = 0; k <= nx; ++k) h->xf[k] = double(float(h->xwidth)) / nx * k;
    }
    h->xc.assign(nx + 2, 0.0);
    h->dxx.assign(nx + 2, 0.0);
    for (int i = 1; i <= nx; ++i) {
        h->xc[i] = 0.5 * (h->xf[i] + h->xf[i - 1]);
        h->dxx[i] = h->xf[i] - h->xf[i - 1];
        if (!(h->dxx[i] > 0)) return h->fail(DG_ERR_CONFIG, "mesh faces must increase strictly");
    }
    h->xc[0] = -h->xc[1];
    h->xc[nx + 1] = 2 * (h->mesh ? h->xwidth_d : h->xwidth) - h->xc[nx];
    h->dxx[0] = h->dxx[1];
    h->dxx[nx + 1] = h->dxx[nx];
    return DG_OK;
}

// ---------------------------------------------------------------------------
// parameter blocks
// ---------------------------------------------------------------------------
// Uniform lerp weights of the y and z directions, in the reference's real R:
// transverse |hdt/dy|, |hdt/dz| (src/dugks.cu:769-770) and the y / z face
// normal fractions (dy/2 - hdt c_y)/dy, (dz/2 - hdt c_z)/dz (828, 871).
template <class R>
struct YZWeights {
    R ty, tz, yn[19], zn[19];
    explicit YZWeights(const RefCoef<R> &c)
    {
        ty = std::fabs((-c.hdt * 1) / c.dy);
        tz = std::fabs((-c.hdt * 1) / c.dz);
        for (int p = 0; p < 19; ++p) {
            yn[p] = (c.dy / 2. - c.hdt * dg::cy(p)) / c.dy;
            zn[p] = (c.dz / 2. - c.hdt * dg::cz(p)) / c.dz;
        }
    }
};

// T-typed tables (x-face normal weights, transverse x weights, corner weights,
// dt/dxx, perturbation factors)
template <class T, class R>
void make_tables(const dg_ctx *h, const RefCoef<R> &c, std::vector<T> &xw, std::vector<T> &txw, std::vector<T> &cxu,
                 std::vector<T> &px, std::vector<T> &py, std::vector<T> &pz, std::vector<T> &cxuf, std::vector<T> &cw,
                 std::vector<T> &gw)
{
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const bool st = h->mesh != 0;
    const R hdt = c.hdt, dx = c.dx;
    // population-major rows [2p + (0: 1-w, 1: w)][column], so that lanes of a warp
    // (consecutive columns) read consecutive words
    const size_t xs = size_t(nx + 2);
    xw.assign(xs * 38, T(0));
    txw.assign(xs * 38, T(0));
    cxu.assign(nx + 2, T(0));
    for (int p = 1; p < 19; ++p) {
        const int cxp = dg::cx(p);
        for (int I = 0; I <= nx; ++I) {
            R m;
            if (!st) {
                const R mx1 = (dx / 2. - hdt * cxp) / dx;  // src/dugks.cu:768
                m = I == 0 ? R(1 - mx1) : mx1;             // face 0 of cell 1 uses mx0 = 1-mx1 (772)
            } else {
                // src/fortran/channel/src/dugks.cuf:541 (mx1) and 546 (mx0)
                if (I == 0) {
                    const R d1 = R(h->dxx[1]), d0 = R(h->dxx[0]);
                    m = (d1 / 2 + hdt * cxp) / (R(0.5) * d1 + R(0.5) * d0);
                } else {
                    const R di = R(h->dxx[I]), dn = R(h->dxx[I + 1]);
                    m = (di / 2 - hdt * cxp) / (R(0.5) * di + R(0.5) * dn);
                }
            }
            xw[size_t(2 * p) * xs + I] = T(R(1 - m));
            xw[size_t(2 * p + 1) * xs + I] = T(m);
        }
        if (cxp != 0) {
            for (int gi = 1; gi <= nx; ++gi) {
                R t;
                if (!st)
                    t = std::fabs((-hdt * cxp) / dx);  // src/dugks.cu:827 with fabs at 850
                else
                    t = std::fabs((-hdt * cxp) / (R(0.5) * R(h->dxx[gi]) + R(0.5) * R(h->dxx[gi - cxp])));  // dugks.cuf:595
                txw[size_t(2 * p) * xs + gi] = T(R(1 - t));
                txw[size_t(2 * p + 1) * xs + gi] = T(t);
            }
        }
    }
    // gradient reconstruction on a stretched x mesh (recon=gradient, mesh !=
    // uniform), rows of GW_* per column, computed in double from the mesh:
    //   x face I (between cells I and I+1): the face value is the linear
    //   interpolation of the two cell values to the face, weight lam_I =
    //   (dxx_I/2) / (xc_{I+1} - xc_I) on cell I+1, and the normal derivative is
    //   their difference over xc_{I+1} - xc_I;
    //   y and z faces at column i: the x derivative of the face-averaged values
    //   is the three-point central difference on the non-uniform centres
    //   xc_{i-1}, xc_i, xc_{i+1} (exact for quadratics).
    // On a uniform mesh these are 1/2, 1/dx and (-1/(2dx), 0, 1/(2dx)): the
    // reference's calc_fx (src/dugks.cu:421-649).
    gw.assign(xs * dg::GW_ROWS, T(0));
    if (st) {
        for (int I = 0; I <= nx; ++I) {
            const double d = h->xc[I + 1] - h->xc[I];
            gw[size_t(dg::GW_LAM) * xs + I] = T(0.5 * h->dxx[I] / d);
            gw[size_t(dg::GW_IDX) * xs + I] = T(1.0 / d);
        }
        for (int i = 1; i <= nx; ++i) {
            const double hm = h->xc[i] - h->xc[i - 1], hp = h->xc[i + 1] - h->xc[i];
            gw[size_t(dg::GW_WM) * xs + i] = T(-hp / (hm * (hp + hm)));
            gw[size_t(dg::GW_W0) * xs + i] = T((hp - hm) / (hp * hm));
            gw[size_t(dg::GW_WP) * xs + i] = T(hm / (hp * (hp + hm)));
        }
    }
    // corner weights: products of the lerp weights as T values, evaluated in
    // double (exact for the FP32 tables' float factors)
    cw.assign(xs * dg::CW_ROWS, T(0));
    {
        const YZWeights<R> yz(c);
        const double tyo = double(T(R(1 - yz.ty))), tym = double(T(yz.ty));
        const double tzo = double(T(R(1 - yz.tz))), tzm = double(T(yz.tz));
        auto put = [&](int row, int col, double w) { cw[size_t(row) * xs + col] = T(w); };
        for (int I = 0; I <= nx; ++I) {
            for (int cl = 1; cl <= 3; ++cl) {
                const double om = double(xw[size_t(2 * cl) * xs + I]), m = double(xw[size_t(2 * cl + 1) * xs + I]);
                const int y = dg::CW_XY + 4 * (cl - 1), z = dg::CW_XZ + 4 * (cl - 1);
                put(y, I, tyo * om); put(y + 1, I, tyo * m); put(y + 2, I, tym * om); put(y + 3, I, tym * m);
                put(z, I, tzo * om); put(z + 1, I, tzo * m); put(z + 2, I, tzm * om); put(z + 3, I, tzm * m);
                if (cl == 3) {
                    const double a[4] = {tzo * tyo, tzo * tym, tzm * tyo, tzm * tym};
                    for (int q = 0; q < 4; ++q) {
                        put(dg::CW_XYZ + 2 * q, I, a[q] * om);
                        put(dg::CW_XYZ + 2 * q + 1, I, a[q] * m);
                    }
                }
            }
        }
        for (int gi = 1; gi <= nx; ++gi) {
            for (int p = 1; p < 19; ++p) {
                if (dg::cx(p) == 0) continue;
                const int cl = dg::xrep(p);
                const double txo = double(txw[size_t(2 * cl) * xs + gi]), txm = double(txw[size_t(2 * cl + 1) * xs + gi]);
                const double yo = double(T(R(1 - yz.yn[p]))), ym = double(T(yz.yn[p]));
                const double zo = double(T(R(1 - yz.zn[p]))), zm = double(T(yz.zn[p]));
                if (dg::cz(p) == 0) {  // y face, 4 corners (rows A, B x columns i, i - cx)
                    const int r = dg::CW_Y4 + 4 * dg::slot4y(p);
                    put(r, gi, yo * txo); put(r + 1, gi, yo * txm); put(r + 2, gi, ym * txo); put(r + 3, gi, ym * txm);
                } else {               // y face, 8 corners (c_y = 0): planes k, k - cz
                    const int r = dg::CW_Y8 + 8 * (cl - 1);
                    put(r, gi, tzo * yo * txo); put(r + 1, gi, tzo * yo * txm);
                    put(r + 2, gi, tzo * ym * txo); put(r + 3, gi, tzo * ym * txm);
                    put(r + 4, gi, tzm * yo * txo); put(r + 5, gi, tzm * yo * txm);
                    put(r + 6, gi, tzm * ym * txo); put(r + 7, gi, tzm * ym * txm);
                }
                if (dg::cy(p) == 0) {  // z face, 4 corners (planes A, B x columns i, i - cx)
                    const int r = dg::CW_Z4 + 4 * dg::slot4z(p);
                    put(r, gi, zo * txo); put(r + 1, gi, zo * txm); put(r + 2, gi, zm * txo); put(r + 3, gi, zm * txm);
                } else {               // z face, 8 corners (c_z = 0): rows j, j - cy
                    const int r = dg::CW_Z8 + 8 * (cl - 1);
                    put(r, gi, zo * tyo * txo); put(r + 1, gi, zo * tyo * txm);
                    put(r + 2, gi, zo * tym * txo); put(r + 3, gi, zo * tym * txm);
                    put(r + 4, gi, zm * tyo * txo); put(r + 5, gi, zm * tyo * txm);
                    put(r + 6, gi, zm * tym * txo); put(r + 7, gi, zm * tym * txm);
                }
            }
        }
    }
    cxuf.assign(nx + 2, T(0));
    for (int gi = 0; gi <= nx + 1; ++gi) {
        const R cu = st ? R(c.dt / R(h->dxx[gi])) : R(c.dt / c.dx);  // dugks.cuf:833
        cxu[gi] = T(cu);
        cxuf[gi] = T(c.fw1 * cu);
    }
    // perturbation forcing factors, src/dugks.cu:1101-1119
    const double pi = 3.141592653589793, pi2 = pi * 2;
    const double beta = 3, gamma = 2, zoffset = 0;
    px.assign(size_t(nx + 2) * 3, T(0));
    py.assign(size_t(ny + 2) * 3, T(0));
    pz.assign(size_t(nz + 2) * 3, T(0));
    for (int i = 0; i <= nx + 1; ++i) {
        if (3 < i && i < h->nx / 4 + 2) {
            const double xx = pi2 * (i - 3) * double(c.dx) / (double(R(h->xwidth)) / 4.);
            px[3 * i + 0] = T(1 - std::cos(xx));
            px[3 * i + 1] = T(std::sin(xx));
            px[3 * i + 2] = T(1);
        }
    }
    for (int j = 0; j <= ny + 1; ++j) {
        const double yy = pi2 * (j - 0.5) * double(c.dy) / double(R(h->ywidth));
        py[3 * j + 0] = T(std::cos(beta * yy));
        py[3 * j + 1] = T(std::sin(beta * yy));
    }
    for (int k = 0; k <= nz + 1; ++k) {
        const double zz = pi2 * ((k - 0.5) * double(c.dz) + zoffset) / double(R(h->zwidth));
        pz[3 * k + 0] = T(std::cos(gamma * zz));
        pz[3 * k + 1] = T(std::sin(gamma * zz));
    }
}

template <class T, class S, class R>
StepParams<T, S> make_params(const dg_ctx *h, const RefCoef<R> &c)
{
    StepParams<T, S> P;
    std::memset(&P, 0, sizeof(P));
    P.nx = h->nx; P.ny = h->ny; P.nz = h->nz; P.pitch = h->pitch; P.ps = h->ps;
    P.pitch_b = h->pitch_b; P.ps_b = h->ps_b;
    P.periodic_x = h->periodic[0];
    P.perturb = h->perturb;
    P.force_on = (c.F[0] != 0 || c.F[1] != 0 || c.F[2] != 0) ? 1 : 0;
    {
        const int nnz = (c.F[0] != 0) + (c.F[1] != 0) + (c.F[2] != 0);
        P.fax = nnz > 1 ? -1 : (c.F[1] != 0 ? 1 : (c.F[2] != 0 ? 2 : 0));
    }
    P.hdt = T(c.hdt); P.bw1 = T(c.bw1); P.bw2 = T(c.bw2); P.bw0x3 = T(R(3) * c.bw0);
    P.fw1 = T(c.fw1); P.fw2 = T(c.fw2); P.fw0x3 = T(R(3) * c.fw0);
    for (int a = 0; a < 3; ++a) {
        P.F[a] = T(c.F[a]);
        P.hF[a] = T(R(0.5 * c.hdt) * c.F[a]);  // 0.5*p->hdt*hp->ambient_f (src/dugks.cu:698)
    }
    const YZWeights<R> yz(c);
    for (int p = 0; p < 19; ++p) {
        const R cf = R(dg::cx(p)) * c.F[0] + R(dg::cy(p)) * c.F[1] + R(dg::cz(p)) * c.F[2];
        P.Kb[p] = T(R(3) * c.bw0 * cf);
        P.Kf[p] = T(R(3) * c.fw0 * cf);
        P.yn_m[p] = T(yz.yn[p]); P.yn_om[p] = T(R(1 - yz.yn[p]));
        P.zn_m[p] = T(yz.zn[p]); P.zn_om[p] = T(R(1 - yz.zn[p]));
    }
    P.ty_m = T(yz.ty); P.ty_om = T(R(1 - yz.ty));
    P.tz_m = T(yz.tz); P.tz_om = T(R(1 - yz.tz));
    // uniform corner weights of the y faces with c_x = 0 != c_z (rows j, j+1 at
    // planes k, k - cz) and of the z faces with c_x = 0 != c_y (planes k, k+1 at
    // rows j, j - cy), for face_tri_cw
    for (int p = 1; p < 19; ++p) {
        if (dg::cx(p) != 0) continue;
        const double yo = double(P.yn_om[p]), ym = double(P.yn_m[p]), zo = double(P.zn_om[p]), zm = double(P.zn_m[p]);
        const double tyo = double(P.ty_om), tym = double(P.ty_m), tzo = double(P.tz_om), tzm = double(P.tz_m);
        if (dg::cz(p) != 0) {
            P.ycw[p][0] = T(tzo * yo); P.ycw[p][1] = T(tzo * ym); P.ycw[p][2] = T(tzm * yo); P.ycw[p][3] = T(tzm * ym);
        }
        if (dg::cy(p) != 0) {
            P.zcw[p][0] = T(zo * tyo); P.zcw[p][1] = T(zo * tym); P.zcw[p][2] = T(zm * tyo); P.zcw[p][3] = T(zm * tym);
        }
    }
    P.cyu = T(c.dt / c.dy);
    P.czu = T(c.dt / c.dz);
    P.bwF = T(c.bw2 * c.hdt + c.bw0);
    if (P.fax >= 0) {
        // the values of the tables at a population with c = +1 on the force axis
        const R Fa = c.F[P.fax];
        P.Fa = T(Fa);
        P.hFa = T(R(0.5 * c.hdt) * Fa);
        P.Kba = T(R(3) * c.bw0 * Fa);
        P.Kfa = T(R(3) * c.fw0 * Fa / c.fw1);
    }
    P.fw2s = T(c.fw2 / c.fw1);
    P.fw0x3s = T(R(3) * c.fw0 / c.fw1);
    for (int p = 0; p < 19; ++p) {
        const R cf = R(dg::cx(p)) * c.F[0] + R(dg::cy(p)) * c.F[1] + R(dg::cz(p)) * c.F[2];
        P.Kfs[p] = T(R(3) * c.fw0 * cf / c.fw1);
    }
    P.cyuf = T(c.fw1 * (c.dt / c.dy));
    P.czuf = T(c.fw1 * (c.dt / c.dz));
    P.g_idx = T(R(1) / c.dx); P.g_idy = T(R(1) / c.dy); P.g_idz = T(R(1) / c.dz);
    P.g_i2dx = T(R(1) / (2 * c.dx)); P.g_i2dy = T(R(1) / (2 * c.dy)); P.g_i2dz = T(R(1) / (2 * c.dz));
    if (h->mesh != 0) {
        const int nx = h->nx;
        P.q0 = T((h->xc[2] - h->xc[0]) / (h->xc[2] - h->xc[1]));                  // dugks.cuf:368
        P.q1 = T((h->xc[nx + 1] - h->xc[nx - 1]) / (h->xc[nx] - h->xc[nx - 1]));  // dugks.cuf:372
    } else {
        P.q0 = T(2);
        P.q1 = T(2);
    }
    const char *base = static_cast<const char *>(h->tab);
    P.xw = reinterpret_cast<const T *>(base + h->tab_off[0]);
    P.xws = h->nx + 2;
    P.txw = reinterpret_cast<const T *>(base + h->tab_off[1]);
    P.cxu = reinterpret_cast<const T *>(base + h->tab_off[2]);
    P.cxuf = reinterpret_cast<const T *>(base + h->tab_off[6]);
    P.cw = reinterpret_cast<const T *>(base + h->tab_off[7]);
    P.gw = reinterpret_cast<const T *>(base + h->tab_off[8]);
    P.grad_st = (h->recon == 1 && h->mesh != 0) ? 1 : 0;
    P.err = h->dev_err;
    P.pert_x = reinterpret_cast<const T *>(base + h->tab_off[3]);
    P.pert_y = reinterpret_cast<const T *>(base + h->tab_off[4]);
    P.pert_z = reinterpret_cast<const T *>(base + h->tab_off[5]);
    return P;
}

template <class T, class S>
void set_codec(const dg_ctx *, Codec<T, S> &) {}
template <>
void set_codec<float, __half>(const dg_ctx *h, Codec<float, __half> &c)
{
    for (int p = 0; p < 19; ++p) {
        c.w[p] = h->dev_w[p]; c.s[p] = h->dev_s[p]; c.is[p] = 1.0f / h->dev_s[p];
    }
}
template <>
void set_codec<float, __nv_bfloat16>(const dg_ctx *h, Codec<float, __nv_bfloat16> &c)
{
    for (int p = 0; p < 19; ++p) {
        c.w[p] = h->dev_w[p]; c.s[p] = h->dev_s[p]; c.is[p] = 1.0f / h->dev_s[p];
    }
}

// per-step stochastic-rounding seed of the 16-bit forms (other forms: nothing)
template <class T, class S>
void set_round_seed(const dg_ctx *, Codec<T, S> &, int) {}
template <>
void set_round_seed<float, __nv_bfloat16>(const dg_ctx *h, Codec<float, __nv_bfloat16> &c, int istep)
{
    c.sr_seed = h->stochastic ? (mix32(unsigned(istep)) | 1u) : 0u;
}
template <>
void set_round_seed<float, __half>(const dg_ctx *h, Codec<float, __half> &c, int istep)
{
    c.sr_seed = h->stochastic ? (mix32(unsigned(istep)) | 1u) : 0u;
}

template <class T, class S>
StepParams<T, S> params_for(const dg_ctx *h, int istep)
{
    StepParams<T, S> P;
    if (std::is_same<T, double>::value)
        P = make_params<T, S>(h, h->c64);
    else
        P = make_params<T, S>(h, h->c32);
    set_codec<T, S>(h, P.codec);
    P.ffield = static_cast<const T *>(h->ffield);
    P.ffaxis = h->ffaxis;
    if (h->perturb) {
        // per-step amplitudes, src/dugks.cu:1101-1108
        const double pi = 3.141592653589793, pi2 = pi * 2;
        const double beta = 3, Tpd = 2000, gamma = 2, Re_tau = 180;
        const double visc = std::is_same<T, double>::value ? h->c64.visc : double(h->c32.visc);
        const double dt = std::is_same<T, double>::value ? h->c64.dt : double(h->c32.dt);
        const double xwidth = double(float(h->xwidth)), ywidth = double(float(h->ywidth)), zwidth = double(float(h->zwidth));
        const double ustar = 2 * Re_tau * visc / xwidth;
        const double FF = 2 * std::pow(ustar, 2) / xwidth;
        const double A0 = 5 * 40.0 / h->nx * beta * std::sin(pi2 * istep * dt / Tpd);
        P.pert_ax = T(0.5 * FF * A0 * xwidth / 4);
        P.pert_ay = T(0.5 * FF * A0 * ywidth / gamma);
        P.pert_az = T(A0 * zwidth / beta);
        P.pert_FF = T(FF);
    }
    return P;
}

// ---------------------------------------------------------------------------
// per-form dispatch
// ---------------------------------------------------------------------------
constexpr int kGraphSteps = 8;

// Steps whose launch parameters are the same every step (no per-step
// perturbation amplitudes, no per-step rounding seed) can be replayed from a
// captured graph: kGraphSteps steps cost one graph launch instead of
// 3 * kGraphSteps kernel launches, which matters for small grids.
template <class T, class S>
bool graph_eligible(const dg_ctx *h)
{
    if (h->perturb) return false;
    if ((std::is_same<S, __nv_bfloat16>::value || std::is_same<S, __half>::value) && h->stochastic) return false;
    return true;
}

template <class T, class S>
int ensure_step_graph(dg_ctx *h, const StepParams<T, S> &P)
{
    using K = Kern<T, S>;
    if (h->step_graph) return DG_OK;
    if (!h->cap_stream) CK(cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking), "stream create");
    S *f = static_cast<S *>(h->f);
    S *fb = static_cast<S *>(h->fb);
    CK(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    cudaError_t le = cudaSuccess;
    for (int s = 0; s < kGraphSteps && le == cudaSuccess; ++s) {
        le = K::fbar(f, fb, P, h->cap_stream);
        if (le == cudaSuccess) le = K::flux(fb, f, f, P, h->recon, h->have_tmap ? &h->tmap : nullptr, h->cap_stream);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return h->cuda_fail(le != cudaSuccess ? le : ce, "step graph capture");
    }
    const cudaError_t ie = cudaGraphInstantiate(&h->step_graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        h->step_graph = nullptr;
        return h->cuda_fail(ie, "step graph instantiate");
    }
    return DG_OK;
}

// n steps; with `ev` (2n+1 recorded events) the launches are bracketed by
// CUDA events on the handle's stream for per-kernel timing.  Without events,
// whole groups of kGraphSteps steps replay the captured step graph where the
// parameters allow (same kernels, same arguments: identical results).
template <class T, class S>
int step_form(dg_ctx *h, int istep0, int n, cudaEvent_t *ev)
{
    using K = Kern<T, S>;
    S *f = static_cast<S *>(h->f);
    S *fb = static_cast<S *>(h->fb);
    StepParams<T, S> P = params_for<T, S>(h, istep0);
    int s = 0;
    if (!ev && n >= 2 * kGraphSteps && graph_eligible<T, S>(h)) {
        const int rc = ensure_step_graph<T, S>(h, P);
        if (rc) return rc;
        for (; s + kGraphSteps <= n; s += kGraphSteps) CK(cudaGraphLaunch(h->step_graph, h->stream), "graph launch");
    }
    if (ev) CK(cudaEventRecord(ev[0], h->stream), "event record");
    for (; s < n; ++s) {
        if (h->perturb && s > 0) P = params_for<T, S>(h, istep0 + s);
        set_round_seed<T, S>(h, P.codec, istep0 + s);
        CK(K::fbar(f, fb, P, h->stream), "stage (a) launch");
        if (ev) CK(cudaEventRecord(ev[2 * s + 1], h->stream), "event record");
        CK(K::flux(fb, f, f, P, h->recon, h->have_tmap ? &h->tmap : nullptr, h->stream), "flux launch");
        if (ev) CK(cudaEventRecord(ev[2 * s + 2], h->stream), "event record");
    }
    h->macro_valid = false;
    return DG_OK;
}

// n steps from the state at src into the state at dst (device arrays in the
// engine's SoA layout): the first step reads src and writes dst, the others
// update dst in place.  The handle's own state is src or dst only when the
// caller passes it.
template <class T, class S>
int step_between_form(dg_ctx *h, int istep0, int n, const void *src, void *dst)
{
    using K = Kern<T, S>;
    const S *fi = static_cast<const S *>(src);
    S *fo = static_cast<S *>(dst);
    S *fb = static_cast<S *>(h->fb);
    StepParams<T, S> P = params_for<T, S>(h, istep0);
    for (int s = 0; s < n; ++s) {
        if (h->perturb && s > 0) P = params_for<T, S>(h, istep0 + s);
        set_round_seed<T, S>(h, P.codec, istep0 + s);
        const S *in = s == 0 ? fi : fo;
        CK(K::fbar(in, fb, P, h->stream), "stage (a) launch");
        CK(K::flux(fb, in, fo, P, h->recon, h->have_tmap ? &h->tmap : nullptr, h->stream), "flux launch");
    }
    if (fo == h->f) h->macro_valid = false;
    return DG_OK;
}

// Device staging of a dump-order double array (host transfers of the state):
// f-bar-plus when it is large enough (the FP64 form: every step rewrites it,
// so between steps it is free), else a temporary allocation (*owned = true).
double *state_staging(dg_ctx *h, size_t bytes, bool *owned)
{
    *owned = false;
    if (h->fb && size_t(h->ps_b) * 19 * storage_bytes(h->prec) >= bytes) return static_cast<double *>(h->fb);
    double *tmp = nullptr;
    if (cudaMalloc(&tmp, bytes) != cudaSuccess) return nullptr;
    *owned = true;
    return tmp;
}

template <class T, class S>
int set_state_form(dg_ctx *h, const double *host_dump)
{
    using K = Kern<T, S>;
    const size_t n = h->ncell() * 19;
    bool owned = false;
    double *tmp = state_staging(h, n * sizeof(double), &owned);
    if (!tmp) return h->fail(DG_ERR_CUDA, "cudaMalloc (state upload staging) failed");
    cudaError_t e = cudaMemcpyAsync(tmp, host_dump, n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = K::aos_to_soa(tmp, static_cast<S *>(h->f), params_for<T, S>(h, 0), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (owned) cudaFree(tmp);
    if (e != cudaSuccess) return h->cuda_fail(e, "state upload");
    h->macro_valid = false;
    return DG_OK;
}

template <class T, class S>
int get_state_form(dg_ctx *h, double *host_dump)
{
    using K = Kern<T, S>;
    const size_t n = h->ncell() * 19;
    bool owned = false;
    double *tmp = state_staging(h, n * sizeof(double), &owned);
    if (!tmp) return h->fail(DG_ERR_CUDA, "cudaMalloc (state download staging) failed");
    cudaError_t e = K::soa_to_aos(static_cast<const S *>(h->f), tmp, params_for<T, S>(h, 0), h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_dump, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (owned) cudaFree(tmp);
    if (e != cudaSuccess) return h->cuda_fail(e, "state download");
    return DG_OK;
}

template <class T, class S>
int macro_form(dg_ctx *h)
{
    using K = Kern<T, S>;
    const size_t g = h->ghosted();
    if (!h->macro) {
        CK(cudaMalloc(&h->macro, 4 * g * sizeof(double)), "cudaMalloc (macro arrays)");
        CK(cudaMemsetAsync(h->macro, 0, 4 * g * sizeof(double), h->stream), "cudaMemset (macro arrays)");
    }
    CK(K::macro(static_cast<const S *>(h->f), params_for<T, S>(h, 0), h->hdt(), h->F, h->macro, h->macro + g,
                         h->macro + 2 * g, h->macro + 3 * g, h->stream),
       "macro launch");
    h->macro_valid = true;
    return DG_OK;
}

int ensure_scratch(dg_ctx *h, size_t bytes)
{
    if (h->scratch_bytes >= bytes) return DG_OK;
    if (h->scratch) cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_bytes = 0;
    CK(cudaMalloc(&h->scratch, bytes), "cudaMalloc (reduction scratch)");
    h->scratch_bytes = bytes;
    return DG_OK;
}

int stats_blocks(const dg_ctx *h)
{
    const int rows = h->ny * h->nz;
    return rows < 608 ? rows : 608;
}

template <class T, class S>
int stats_form(dg_ctx *h, std::vector<double> &total)
{
    using K = Kern<T, S>;
    const int nb = stats_blocks(h);
    const size_t part = size_t(nb) * h->nx * NSTAT;
    int rc = ensure_scratch(h, (part + size_t(h->nx) * NSTAT) * sizeof(double));
    if (rc) return rc;
    double *partial = h->scratch, *tot = h->scratch + part;
    CK(K::stats_partials(static_cast<const S *>(h->f), params_for<T, S>(h, 0), h->hdt(), h->F, partial, nb,
                                  h->stream),
       "statistics launch");
    CK(launch_stats_reduce(partial, nb, h->nx, tot, h->stream), "statistics reduce launch");
    total.assign(size_t(h->nx) * NSTAT, 0.0);
    CK(cudaMemcpyAsync(total.data(), tot, total.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
       "statistics copy");
    CK(cudaStreamSynchronize(h->stream), "statistics sync");
    return DG_OK;
}

// one statistics pass into the device running sums (no host transfer)
template <class T, class S>
int accumulate_form(dg_ctx *h)
{
    using K = Kern<T, S>;
    const int nb = stats_blocks(h);
    const size_t part = size_t(nb) * h->nx * NSTAT;
    int rc = ensure_scratch(h, (part + size_t(h->nx) * NSTAT) * sizeof(double));
    if (rc) return rc;
    if (!h->acc) {
        CK(cudaMalloc(&h->acc, size_t(h->nx) * 10 * sizeof(double)), "cudaMalloc (statistics accumulator)");
        CK(cudaMemsetAsync(h->acc, 0, size_t(h->nx) * 10 * sizeof(double), h->stream), "cudaMemset (accumulator)");
        h->acc_count = 0;
    }
    double *partial = h->scratch, *tot = h->scratch + part;
    CK(K::stats_partials(static_cast<const S *>(h->f), params_for<T, S>(h, 0), h->hdt(), h->F, partial, nb, h->stream),
       "statistics launch");
    CK(launch_stats_reduce(partial, nb, h->nx, tot, h->stream), "statistics reduce launch");
    stats_accumulate_kernel<<<(h->nx * 10 + 127) / 128, 128, 0, h->stream>>>(tot, h->nx, h->acc);
    CK(cudaGetLastError(), "accumulate launch");
    h->acc_count++;
    return DG_OK;
}

template <class T, class S>
int moments_form(dg_ctx *h, double *out4)
{
    using K = Kern<T, S>;
    const int nb = 608;
    int rc = ensure_scratch(h, size_t(nb) * 4 * sizeof(double));
    if (rc) return rc;
    CK(K::moments_partials(static_cast<const S *>(h->f), params_for<T, S>(h, 0), h->scratch, nb, h->stream),
       "moments launch");
    std::vector<double> part(size_t(nb) * 4);
    CK(cudaMemcpyAsync(part.data(), h->scratch, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
       "moments copy");
    CK(cudaStreamSynchronize(h->stream), "moments sync");
    for (int m = 0; m < 4; ++m) out4[m] = 0;
    for (int b = 0; b < nb; ++b)
        for (int m = 0; m < 4; ++m) out4[m] += part[size_t(b) * 4 + m];
    return DG_OK;
}

template <class T, class S>
int adjoint_form(dg_ctx *h, int istep, const void *f_n, const void *lam_next, void *lam_out)
{
    using K = Kern<T, S>;
    if (!std::is_same<T, S>::value) return h->fail(DG_ERR_UNSUPPORTED, "the adjoint exists for the fp64 and fp32 forms");
    if (h->recon != 0) return h->fail(DG_ERR_UNSUPPORTED, "the adjoint exists for the trilinear reconstruction");
    if (!h->adj) {
        // 19 adjoint values and one dJ/dF (force-field face term) per face, the
        // wall-ghost sums (2 * 19 per row and plane) and the transposed-stencil
        // sums (19 per cell)
        const long long n = adj_nface(0, h->nx, h->ny, h->nz) + 2 * adj_nface(1, h->nx, h->ny, h->nz);
        const long long ng = 2LL * NPOP * h->ny * h->nz;
        const long long nm = (long long)NPOP * h->ncell();
        CK(cudaMalloc(&h->adj, (size_t(n) * (NPOP + 1) + size_t(ng) + size_t(nm)) * sizeof(T)),
           "cudaMalloc (adjoint scratch)");
    }
    if (h->ffield && !h->dphi) {
        CK(cudaMalloc(&h->dphi, h->ncell() * sizeof(double)), "cudaMalloc (field gradient)");
        CK(cudaMemsetAsync(h->dphi, 0, h->ncell() * sizeof(double), h->stream), "cudaMemset (field gradient)");
    }
    CK(K::adjoint(static_cast<const S *>(f_n), static_cast<S *>(h->fb), static_cast<const S *>(lam_next),
                  static_cast<S *>(lam_out), static_cast<T *>(h->adj), params_for<T, S>(h, istep),
                  h->ffield ? h->dphi : nullptr, h->have_tmap ? &h->tmap_adj : nullptr, h->stream),
       "adjoint launch");
    h->macro_valid = false;
    return DG_OK;
}

#define DISPATCH(h, fn, ...)                                                             \
    ((h)->prec == DG_PREC_FP64   ? fn<double, double>((h), ##__VA_ARGS__)                \
     : (h)->prec == DG_PREC_FP32 ? fn<float, float>((h), ##__VA_ARGS__)                  \
     : (h)->prec == DG_PREC_FP16 ? fn<float, __half>((h), ##__VA_ARGS__)                 \
                                 : fn<float, __nv_bfloat16>((h), ##__VA_ARGS__))

// ---------------------------------------------------------------------------
// spectral statistics of a periodic box (src/fortran/dhit/src/stat.f90:5-205)
// ---------------------------------------------------------------------------
// cuFFT is loaded on first use, so that the library itself does not depend on it.
struct CufftLib {
    decltype(&cufftPlan3d) plan3d = nullptr;
    decltype(&cufftExecZ2Z) z2z = nullptr;
    decltype(&cufftSetStream) set_stream = nullptr;
    decltype(&cufftDestroy) destroy = nullptr;
    std::string err;
};

const CufftLib &cufft_lib()
{
    static const CufftLib lib = [] {
        CufftLib l;
        void *so = nullptr;
        for (const char *name : {"libcufft.so.12", "libcufft.so", "/usr/local/cuda/lib64/libcufft.so.12"})
            if (!so) so = dlopen(name, RTLD_NOW | RTLD_LOCAL);
        if (!so) {
            const char *e = dlerror();
            l.err = std::string("cannot load cuFFT: ") + (e ? e : "unknown error");
            return l;
        }
        l.plan3d = reinterpret_cast<decltype(l.plan3d)>(dlsym(so, "cufftPlan3d"));
        l.z2z = reinterpret_cast<decltype(l.z2z)>(dlsym(so, "cufftExecZ2Z"));
        l.set_stream = reinterpret_cast<decltype(l.set_stream)>(dlsym(so, "cufftSetStream"));
        l.destroy = reinterpret_cast<decltype(l.destroy)>(dlsym(so, "cufftDestroy"));
        if (!l.plan3d || !l.z2z || !l.set_stream || !l.destroy) l.err = "cuFFT lacks an entry point";
        return l;
    }();
    return lib;
}

}  // namespace

void dg_ctx::release_spec_plan()
{
    if (spec_have_plan && cufft_lib().destroy) cufft_lib().destroy(cufftHandle(spec_plan));
    spec_have_plan = false;
}

namespace {

constexpr int kSpecBlocks = 608;  // blocks of the grid-stride reductions (fixed: deterministic sums)

// Values of dg_spectral_stats, in this order.
enum SpecVal { SV_TE, SV_ETOTAL, SV_EDISS0, SV_EDISS, SV_ETA, SV_VK, SV_TK, SV_UPRM, SV_TMSE, SV_RETMS, SV_XL,
               SV_KMXETA, SV_SKEW, SV_FLAT, SV_COUNT };

// Buffers, shell lists and plan on first use.
int spec_setup(dg_ctx *h)
{
    const CufftLib &L = cufft_lib();
    if (!L.err.empty()) return h->fail(DG_ERR_UNSUPPORTED, L.err);
    const long long n = (long long)h->ncell();
    if (n >= (1LL << 31)) return h->fail(DG_ERR_UNSUPPORTED, "spectral statistics: more than 2^31 cells");
    if (!h->spec) {
        // shells wn = nint(|f|) of the signed integer frequencies (stat.f90:142-151), each shell's
        // modes in ascending order
        std::vector<int> bin(static_cast<size_t>(n));
        int nb = 0;
        for (int k = 0; k < h->nz; ++k)
            for (int j = 0; j < h->ny; ++j)
                for (int i = 0; i < h->nx; ++i) {
                    const double fx = spec_freq(i, h->nx), fy = spec_freq(j, h->ny), fz = spec_freq(k, h->nz);
                    const int wn = int(std::lround(std::sqrt(fx * fx + fy * fy + fz * fz)));
                    bin[(size_t(k) * h->ny + j) * h->nx + i] = wn;
                    nb = std::max(nb, wn + 1);
                }
        std::vector<int> off(static_cast<size_t>(nb) + 1, 0), order(static_cast<size_t>(n));
        for (long long t = 0; t < n; ++t) ++off[size_t(bin[size_t(t)]) + 1];
        for (int b = 0; b < nb; ++b) off[size_t(b) + 1] += off[size_t(b)];
        std::vector<int> fill(off.begin(), off.end() - 1);
        for (long long t = 0; t < n; ++t) order[size_t(fill[size_t(bin[size_t(t)])]++)] = int(t);
        const size_t bytes = size_t(n) * (3 * sizeof(double2) + 2 * sizeof(double)) +
                             size_t(kSpecBlocks) * 3 * sizeof(double) + size_t(nb) * 2 * sizeof(double);
        CK(cudaMalloc(&h->spec, bytes), "cudaMalloc (spectral statistics)");
        CK(cudaMalloc(&h->spec_order, size_t(n) * sizeof(int)), "cudaMalloc (spectral shells)");
        CK(cudaMalloc(&h->spec_off, (size_t(nb) + 1) * sizeof(int)), "cudaMalloc (spectral shells)");
        CK(cudaMemcpy(h->spec_order, order.data(), size_t(n) * sizeof(int), cudaMemcpyHostToDevice), "shell upload");
        CK(cudaMemcpy(h->spec_off, off.data(), (size_t(nb) + 1) * sizeof(int), cudaMemcpyHostToDevice),
           "shell upload");
        h->spec_nbins = nb;
    }
    if (!h->spec_have_plan) {
        cufftHandle plan;
        // row-major dims, x fastest: the reference's fftw_plan_dft_3d(nz, ny, nx, ...) (dft.f90:28-34)
        if (L.plan3d(&plan, h->nz, h->ny, h->nx, CUFFT_Z2Z) != CUFFT_SUCCESS)
            return h->fail(DG_ERR_CUDA, "cufftPlan3d failed");
        h->spec_plan = int(plan);
        h->spec_have_plan = true;
    }
    if (L.set_stream(cufftHandle(h->spec_plan), h->stream) != CUFFT_SUCCESS)
        return h->fail(DG_ERR_CUDA, "cufftSetStream failed");
    return DG_OK;
}

template <class T, class S>
int spectral_form(dg_ctx *h, double *vals, std::vector<double> *shells)
{
    int rc = spec_setup(h);
    if (rc) return rc;
    const CufftLib &L = cufft_lib();
    const long long n = (long long)h->ncell();
    double2 *U = static_cast<double2 *>(h->spec), *V = U + n, *W = V + n;
    double *ET = reinterpret_cast<double *>(W + n), *ETS = ET + n, *part = ETS + n, *sh = part + kSpecBlocks * 3;
    StepParams<T, S> P = params_for<T, S>(h, 0);
    const cufftHandle plan = cufftHandle(h->spec_plan);

    spec_velocity_kernel<T, S><<<kSpecBlocks, 256, 0, h->stream>>>(static_cast<const S *>(h->f), P, U, V, W, part);
    CK(cudaGetLastError(), "spectral velocity launch");
    std::vector<double> hp(size_t(kSpecBlocks) * 3);
    CK(cudaMemcpyAsync(hp.data(), part, kSpecBlocks * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
       "spectral copy");
    CK(cudaStreamSynchronize(h->stream), "spectral sync");
    double ke2 = 0;
    for (int b = 0; b < kSpecBlocks; ++b) ke2 += hp[size_t(b)];
    for (double2 *X : {U, V, W})
        if (L.z2z(plan, reinterpret_cast<cufftDoubleComplex *>(X), reinterpret_cast<cufftDoubleComplex *>(X),
                  CUFFT_FORWARD) != CUFFT_SUCCESS)
            return h->fail(DG_ERR_CUDA, "cufftExecZ2Z (forward) failed");
    // the reference's constants: pi = 3.14159 in single precision (stat.f90:28), widths and
    // viscosity as parsed (float)
    const double pi = double(3.14159f), L0 = h->xwidth, nu = h->visc;
    spec_modes_kernel<<<kSpecBlocks, 256, 0, h->stream>>>(U, V, W, ET, ETS, h->nx, h->ny, h->nz, 1.0 / double(n),
                                                          2 * pi / L0, 2 * nu);
    CK(cudaGetLastError(), "spectral modes launch");
    spec_shell_kernel<<<h->spec_nbins, 256, 0, h->stream>>>(ET, ETS, h->spec_order, h->spec_off, sh);
    CK(cudaGetLastError(), "spectral shells launch");
    for (double2 *X : {U, V, W})
        if (L.z2z(plan, reinterpret_cast<cufftDoubleComplex *>(X), reinterpret_cast<cufftDoubleComplex *>(X),
                  CUFFT_INVERSE) != CUFFT_SUCCESS)
            return h->fail(DG_ERR_CUDA, "cufftExecZ2Z (inverse) failed");
    spec_deriv_moments_kernel<<<kSpecBlocks, 256, 0, h->stream>>>(U, V, W, n, part);
    CK(cudaGetLastError(), "spectral derivative launch");
    std::vector<double> hs(size_t(h->spec_nbins) * 2);
    CK(cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
       "spectral copy");
    CK(cudaMemcpyAsync(hs.data(), sh, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
       "spectral copy");
    CK(cudaStreamSynchronize(h->stream), "spectral sync");
    double m2 = 0, m3 = 0, m4 = 0;
    for (int b = 0; b < kSpecBlocks; ++b) {
        m2 += hp[size_t(b) * 3];
        m3 += hp[size_t(b) * 3 + 1];
        m4 += hp[size_t(b) * 3 + 2];
    }
    double etotal = 0, ediss = 0;
    if (shells) shells->assign(size_t(h->spec_nbins), 0.0);
    for (int b = 0; b < h->spec_nbins; ++b) {
        etotal += hs[size_t(b) * 2];
        ediss += hs[size_t(b) * 2 + 1];
        if (shells) (*shells)[size_t(b)] = hs[size_t(b) * 2];
    }
    // stat.f90:157-168 and 186-190
    const double nn = double(n), dx = L0 / h->nx, cw = L0, cwh = cw / 2;
    vals[SV_TE] = 0.5 * ke2 / nn;
    vals[SV_ETOTAL] = etotal;
    vals[SV_EDISS0] = ediss;
    vals[SV_EDISS] = 0.0;
    vals[SV_ETA] = std::pow(nu * nu * nu / ediss, 0.25);
    vals[SV_VK] = std::pow(nu * ediss, 0.25);
    vals[SV_TK] = std::sqrt(nu / ediss);
    vals[SV_UPRM] = std::sqrt(2.0 / 3.0 * etotal);
    vals[SV_TMSE] = std::sqrt(15 * nu * vals[SV_UPRM] * vals[SV_UPRM] / ediss);
    vals[SV_RETMS] = vals[SV_UPRM] * vals[SV_TMSE] / nu;
    vals[SV_XL] = vals[SV_UPRM] * vals[SV_UPRM] * vals[SV_UPRM] / ediss;
    vals[SV_KMXETA] = (cwh - 1.5 * dx) * (2 * pi) / cw * vals[SV_ETA];
    const double bottom = m2 / (3 * nn), top3 = m3 / (3 * nn), top4 = m4 / (3 * nn);
    vals[SV_SKEW] = top3 / std::pow(bottom, 1.5);
    vals[SV_FLAT] = top4 / (bottom * bottom);
    return DG_OK;
}

// ---------------------------------------------------------------------------
// allocation and initial condition
// ---------------------------------------------------------------------------
template <class T>
int upload_tables(dg_ctx *h)
{
    std::vector<T> xw, txw, cxu, px, py, pz, cxuf, cw, gw;
    if (h->prec == DG_PREC_FP64)
        make_tables<T, double>(h, h->c64, xw, txw, cxu, px, py, pz, cxuf, cw, gw);
    else
        make_tables<T, float>(h, h->c32, xw, txw, cxu, px, py, pz, cxuf, cw, gw);
    const std::vector<T> *parts[9] = {&xw, &txw, &cxu, &px, &py, &pz, &cxuf, &cw, &gw};
    size_t off = 0;
    for (int t = 0; t < 9; ++t) {
        h->tab_off[t] = off;
        off += (parts[t]->size() * sizeof(T) + 255) / 256 * 256;
    }
    CK(cudaMalloc(&h->tab, off), "cudaMalloc (tables)");
    for (int t = 0; t < 9; ++t)
        CK(cudaMemcpy(static_cast<char *>(h->tab) + h->tab_off[t], parts[t]->data(), parts[t]->size() * sizeof(T),
                      cudaMemcpyHostToDevice),
           "table upload");
    return DG_OK;
}

template <class T, class S>
int make_tmap_form(dg_ctx *h)
{
    using K = Kern<T, S>;
    if (!K::uses_tma()) return DG_OK;
    const S *fb = static_cast<const S *>(h->fb);
    int r = K::make_tmap(fb, h->nx, h->ny, h->nz, h->pitch_b, h->ps_b, TileCfg<T, S>::W + 1, &h->tmap);
    if (!r) r = K::make_tmap(fb, h->nx, h->ny, h->nz, h->pitch_b, h->ps_b, AdjCfg<T, S>::W + 2, &h->tmap_adj);
    if (r) return h->fail(DG_ERR_CUDA, "cuTensorMapEncodeTiled failed for the f-bar-plus tensor map (" + std::to_string(r) + ")");
    h->have_tmap = true;
    return DG_OK;
}

int allocate(dg_ctx *h)
{
    const size_t sb = storage_bytes(h->prec);
    const int align = int(128 / sb);
    h->pitch = (h->nx + align - 1) / align * align;
    const long long plane = (long long)h->pitch * h->ny * h->nz;
    const long long a256 = 256 / (long long)sb;
    h->ps = (plane + a256 - 1) / a256 * a256;
    h->pitch_b = (h->nx + 2 + align - 1) / align * align;
    const long long plane_b = (long long)h->pitch_b * (h->ny + 2) * (h->nz + 2);
    h->ps_b = (plane_b + a256 - 1) / a256 * a256;
    const size_t bytes = size_t(h->ps) * 19 * sb, bytes_b = size_t(h->ps_b) * 19 * sb;
    CK(cudaMalloc(&h->f, bytes), "cudaMalloc (f)");
    CK(cudaMalloc(&h->fb, bytes_b), "cudaMalloc (fb)");
    CK(cudaMemset(h->f, 0, bytes), "cudaMemset (f)");
    CK(cudaMemset(h->fb, 0, bytes_b), "cudaMemset (fb)");
    CK(cudaMalloc(&h->dev_err, sizeof(int)), "cudaMalloc (error flag)");
    CK(cudaMemset(h->dev_err, 0, sizeof(int)), "cudaMemset (error flag)");
    int rc = h->prec == DG_PREC_FP64 ? upload_tables<double>(h) : upload_tables<float>(h);
    if (rc) return rc;
    return DISPATCH(h, make_tmap_form);
}

// host equilibrium, src/dugks.cu:304-309
double feq_host(int p, double r, double u, double v, double w)
{
    const double RT = 1. / 3.;
    const double tp = p == 0 ? 1.0 / 3.0 : (p <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
    const double eu = (dg::cx(p) * u + dg::cy(p) * v + dg::cz(p) * w) / RT;
    const double uv = (u * u + v * v + w * w) / RT;
    return tp * r * (1.0 + eu + 0.5 * (eu * eu - uv));
}

// Initial state in dump order.  tg_eq / channel: src/dugks.cu:222-259; the
// tg_eq amplitude is the reference's 0.1 unless the extension key tg_u0 gives
// another (it scales both the velocity and the density correction).
// channel_turb (extension): laminar Poiseuille profile of bulk velocity
// `ub` along the forcing axis plus seeded uniform perturbations and near-wall
// streaks, f = feq(1, u).
int initial_state(dg_ctx *h, const ConfigFile &cf, std::vector<double> &f)
{
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    f.assign(h->ncell() * 19, 0.0);
    const double pi = 3.141592653589793, pi2 = pi * 2;
    const double dx = h->c64.dx, dy = h->c64.dy, dz = h->c64.dz;
    const double xwidth = double(float(h->xwidth)), ywidth = double(float(h->ywidth)), zwidth = double(float(h->zwidth));
    const double RT = 1. / 3.;
    std::string e;
    double ub = 0.1, re_tau = 180, amp = 0.1, streak = 0.05;
    int seed = 0, m = 4;
    if (h->casename == "channel_turb") {
        if (!cf.opt_double("ub", 0.1, ub, e) || !cf.opt_double("re_tau", 180, re_tau, e) ||
            !cf.opt_double("pert_amp", 0.1, amp, e) || !cf.opt_double("streak_amp", 0.05, streak, e) ||
            !cf.opt_int("seed", 0, seed, e) || !cf.opt_int("streak_m", 4, m, e))
            return h->fail(DG_ERR_CONFIG, e);
        if (h->periodic[0]) return h->fail(DG_ERR_CONFIG, "case=channel_turb needs walls in x (periods_x=0)");
    } else if (h->casename != "tg_eq" && h->casename != "channel") {
        return h->fail(DG_ERR_CONFIG, "ERROR: Unknown case '" + h->casename + "' (use tg_eq, channel, channel_turb, or restart=1)");
    }
    // streamwise axis: the largest ambient force component (z in the reference orientation)
    int sa = 2;
    if (std::fabs(h->F[0]) > std::fabs(h->F[sa])) sa = 0;
    if (std::fabs(h->F[1]) > std::fabs(h->F[sa])) sa = 1;
    const double H = 0.5 * xwidth;
    for (int k = 1; k <= nz; ++k) {
        const double z = (k - 0.5) * dz;
        for (int j = 1; j <= ny; ++j) {
            const double y = (j - 0.5) * dy;
            for (int i = 1; i <= nx; ++i) {
                const double x = h->mesh ? h->xc[i] : (i - 0.5) * dx;
                double rho = 1, u[3] = {0, 0, 0};
                if (h->casename == "tg_eq") {
                    const double vs = h->tg_u0;
                    rho = 1.0 + 1.0 * vs * vs / 16 * (std::cos(2 * pi2 / xwidth * x) + std::cos(2 * pi2 / ywidth * y)) *
                                    (std::cos(2 * pi2 / zwidth * z) + 2) / RT;
                    u[0] = vs * std::sin(pi2 / xwidth * x) * std::cos(pi2 / ywidth * y) * std::cos(pi2 / zwidth * z);
                    u[1] = -vs * std::cos(pi2 / xwidth * x) * std::sin(pi2 / ywidth * y) * std::cos(pi2 / zwidth * z);
                    u[2] = 0;
                } else if (h->casename == "channel") {
                    u[2] = 0.1;
                } else {
                    const size_t cell = (size_t(k - 1) * ny + (j - 1)) * nx + (i - 1);
                    const double eta = x / xwidth;
                    u[sa] = 6.0 * ub * eta * (1 - eta);  // bulk ub
                    for (int a = 0; a < 3; ++a) u[a] += amp * ub * rng_sym(uint64_t(seed), cell, a);
                    const double wall = std::min(x, xwidth - x);
                    const double yplus_scale = re_tau / H;
                    const double et = wall * yplus_scale / 10.0;
                    const int span = sa == 2 ? 1 : 2;
                    const double sc = span == 1 ? y / ywidth : z / zwidth;
                    u[sa] += streak * ub * std::sin(pi2 * m * sc) * et * std::exp(1 - et);
                }
                const size_t cell = (size_t(k - 1) * ny + (j - 1)) * nx + (i - 1);
                for (int p = 0; p < 19; ++p) f[cell * 19 + p] = feq_host(p, rho, u[0], u[1], u[2]);
            }
        }
    }
    return DG_OK;
}

// Deviation scales of the 16-bit forms: s_p = w_p * max(1e-3, max|f_p - w_p|/w_p)
// over the initial state, which keeps typical deviations in the normal range
// of FP16 (relative precision of a floating format does not depend on s_p).
void choose_dev_scales(dg_ctx *h, const std::vector<double> &f)
{
    for (int p = 0; p < 19; ++p) {
        const double w = p == 0 ? 1.0 / 3.0 : (p <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
        double mx = 1e-3;
        for (size_t c = 0; c < h->ncell(); ++c) mx = std::max(mx, std::fabs(f[c * 19 + p] - w) / w);
        h->dev_w[p] = float(w);
        h->dev_s[p] = float(w * mx);
    }
}

int read_dump_file(dg_ctx *h, int step, std::vector<double> &f)
{
    char name[32];
    std::snprintf(name, sizeof(name), "ddf%8.8d.dat", step);
    const std::string path = h->workdir + "/" + name;
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in) return h->fail(DG_ERR_IO, "cannot open dump '" + path + "'");
    const size_t width = h->prec == DG_PREC_FP64 ? 8 : 4;
    const size_t want = h->ncell() * 19 * width;
    const size_t have = size_t(in.tellg());
    if (have != want) {
        std::ostringstream os;
        os << "dump '" << path << "' has " << have << " bytes, expected " << want << " (19*nx*ny*nz reals of "
           << width << " bytes)";
        return h->fail(DG_ERR_IO, os.str());
    }
    in.seekg(0);
    f.resize(h->ncell() * 19);
    if (width == 8) {
        in.read(reinterpret_cast<char *>(f.data()), std::streamsize(want));
    } else {
        std::vector<float> tmp(f.size());
        in.read(reinterpret_cast<char *>(tmp.data()), std::streamsize(want));
        for (size_t q = 0; q < f.size(); ++q) f[q] = tmp[q];
    }
    if (!in) return h->fail(DG_ERR_IO, "short read from '" + path + "'");
    return DG_OK;
}

int check_finite(dg_ctx *h, const std::vector<double> &f)
{
    for (double v : f)
        if (!std::isfinite(v)) return h->fail(DG_ERR_NUMERIC, "initial state contains NaN or Inf");
    return DG_OK;
}

int create_common(dg_ctx *h, const ConfigFile &cf)
{
    int rc = load_config(h, cf);
    if (rc) return rc;
    rc = build_mesh(h);
    if (rc) return rc;
    const bool st = h->mesh != 0;
    h->c64 = ref_coef<double>(h->visc, h->cfl, h->xwidth, h->ywidth, h->zwidth, h->nx, h->ny, h->nz, h->F, st, h->dxx[1]);
    h->c32 = ref_coef<float>(h->visc, h->cfl, h->xwidth, h->ywidth, h->zwidth, h->nx, h->ny, h->nz, h->F, st, h->dxx[1]);
    if (st) {
        // the transverse-x shift must stay inside the neighbouring cell
        for (int i = 1; i <= h->nx; ++i)
            if (h->c64.hdt > 0.5 * h->dxx[i] + 1e-15)
                return h->fail(DG_ERR_CONFIG, "time step too large for the smallest stretched cell (CFL)");
    }
    // everything that can fail on the host runs before the first CUDA call
    std::vector<double> f0;
    if (h->restart) {
        rc = read_dump_file(h, h->nrestart, f0);
    } else {
        rc = initial_state(h, cf, f0);
    }
    if (rc) return rc;
    rc = check_finite(h, f0);
    if (rc) return rc;
    CK(cudaGetDevice(&h->device), "cudaGetDevice");
    for (int p = 0; p < 19; ++p) {
        h->dev_w[p] = float(p == 0 ? 1.0 / 3.0 : (p <= 6 ? 1.0 / 18.0 : 1.0 / 36.0));
        h->dev_s[p] = h->dev_w[p];
    }
    if (h->prec == DG_PREC_FP16 || h->prec == DG_PREC_BF16) choose_dev_scales(h, f0);
    rc = allocate(h);
    if (rc) return rc;
    return DISPATCH(h, set_state_form, f0.data());
}

std::string dirname_of(const std::string &p)
{
    const auto s = p.find_last_of('/');
    if (s == std::string::npos) return ".";
    if (s == 0) return "/";
    return p.substr(0, s);
}

}  // namespace

namespace dg {
__global__ void stats_reduce_kernel(const double *__restrict__ partial, int nblocks, int nx, double *__restrict__ total)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    double acc[NSTAT];
    stats_combine_blocks(partial, nblocks, nx, i, acc);
    for (int s = 0; s < NSTAT; ++s) total[size_t(i) * NSTAT + s] = acc[s];
}

cudaError_t launch_stats_reduce(const double *partial, int nblocks, int nx, double *total, cudaStream_t st)
{
    stats_reduce_kernel<<<(nx + 127) / 128, 128, 0, st>>>(partial, nblocks, nx, total);
    return cudaGetLastError();
}

// acc[i][s] += total[i][s] for the 10 sums (rho, u, v, w, uw, uv, vw, uu, vv, ww)
__global__ void stats_accumulate_kernel(const double *__restrict__ total, int nx, double *__restrict__ acc)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nx * 10) return;
    const int i = q / 10, s = q % 10;
    acc[q] += total[size_t(i) * NSTAT + s];
}
}  // namespace dg

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

static int create_impl(const ConfigFile &cf, const std::string &workdir, dg_t **out)
{
    if (!out) {
        g_create_error = "NULL output handle pointer";
        return DG_ERR_ARG;
    }
    *out = nullptr;
    std::unique_ptr<dg_ctx> h(new (std::nothrow) dg_ctx());
    if (!h) {
        g_create_error = "out of host memory";
        return DG_ERR_ARG;
    }
    h->workdir = workdir;
    const int rc = create_common(h.get(), cf);
    if (rc) {
        g_create_error = h->err;
        return rc;
    }
    *out = h.release();
    return DG_OK;
}

int dg_create(const char *config_path, dg_t **out)
{
    if (!config_path) {
        g_create_error = "NULL config path";
        return DG_ERR_ARG;
    }
    ConfigFile cf;
    std::string e;
    if (!cf.load_file(config_path, e)) {
        g_create_error = e;
        if (out) *out = nullptr;
        return DG_ERR_IO;
    }
    return create_impl(cf, dirname_of(config_path), out);
}

int dg_create_from_text(const char *config_text, const char *workdir, dg_t **out)
{
    if (!config_text) {
        g_create_error = "NULL config text";
        return DG_ERR_ARG;
    }
    ConfigFile cf;
    cf.load_text(config_text);
    return create_impl(cf, workdir ? workdir : ".", out);
}

int dg_destroy(dg_t *h)
{
    if (!h) return DG_ERR_ARG;
    delete h;
    return DG_OK;
}

const char *dg_last_error(const dg_t *h)
{
    if (!h) return g_create_error.c_str();
    return h->err.c_str();
}

int dg_get_info(const dg_t *h, dg_info_t *info)
{
    if (!h || !info) return DG_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    info->nx = h->nx; info->ny = h->ny; info->nz = h->nz;
    info->pitch = h->pitch; info->pop_stride = h->ps;
    info->precision = h->prec;
    for (int a = 0; a < 3; ++a) info->periodic[a] = h->periodic[a];
    info->mesh = h->mesh; info->recon = h->recon; info->perturb = h->perturb;
    info->istep0 = h->istep0; info->nsteps = h->nsteps; info->noutput2 = h->noutput2;
    info->ndump = h->ndump; info->restart = h->restart; info->nrestart = h->nrestart;
    const bool d = h->prec == DG_PREC_FP64;
    info->dx = d ? h->c64.dx : h->c32.dx;
    info->dy = d ? h->c64.dy : h->c32.dy;
    info->dz = d ? h->c64.dz : h->c32.dz;
    info->dt = d ? h->c64.dt : h->c32.dt;
    info->visc = d ? h->c64.visc : h->c32.visc;
    info->tau = d ? h->c64.tau : h->c32.tau;
    info->xwidth = h->xwidth; info->ywidth = h->ywidth; info->zwidth = h->zwidth;
    for (int a = 0; a < 3; ++a) info->ambient[a] = h->F[a];
    info->bw0 = d ? h->c64.bw0 : h->c32.bw0;
    info->bw1 = d ? h->c64.bw1 : h->c32.bw1;
    info->bw2 = d ? h->c64.bw2 : h->c32.bw2;
    info->fw0 = d ? h->c64.fw0 : h->c32.fw0;
    info->fw1 = d ? h->c64.fw1 : h->c32.fw1;
    info->fw2 = d ? h->c64.fw2 : h->c32.fw2;
    // two-pass structure: stage (a) reads f, writes fb; the flux pass reads fb once, reads and writes f
    info->hbm_bytes_per_cell = 95.0 * double(storage_bytes(h->prec));
    return DG_OK;
}

int dg_set_stream(dg_t *h, void *cuda_stream)
{
    if (!h) return DG_ERR_ARG;
    h->stream = static_cast<cudaStream_t>(cuda_stream);
    return DG_OK;
}

int dg_run(dg_t *h, int istep0, int nsteps)
{
    if (!h) return DG_ERR_ARG;
    if (nsteps < 0) return h->fail(DG_ERR_ARG, "nsteps < 0");
    if (nsteps == 0) return DG_OK;
    return DISPATCH(h, step_form, istep0, nsteps, (cudaEvent_t *)nullptr);
}

int dg_run_between(dg_t *h, int istep0, int nsteps, const void *src, void *dst)
{
    if (!h) return DG_ERR_ARG;
    if (nsteps < 0) return h->fail(DG_ERR_ARG, "nsteps < 0");
    if (nsteps == 0) return DG_OK;
    if (!src) src = h->f;
    if (!dst) dst = h->f;
    const size_t sb = size_t(h->ps) * 19 * storage_bytes(h->prec);
    const char *lo = static_cast<const char *>(dst), *fb = static_cast<const char *>(h->fb);
    if (lo < fb + size_t(h->ps_b) * 19 * storage_bytes(h->prec) && fb < lo + sb)
        return h->fail(DG_ERR_ARG, "dg_run_between: the destination overlaps f-bar-plus");
    const char *si = static_cast<const char *>(src);
    if (si != lo && si < lo + sb && lo < si + sb)
        return h->fail(DG_ERR_ARG, "dg_run_between: source and destination overlap without being equal");
    return DISPATCH(h, step_between_form, istep0, nsteps, src, dst);
}

int dg_run_profiled(dg_t *h, int istep0, int nsteps, double *kernel_ms)
{
    if (!h || !kernel_ms) return DG_ERR_ARG;
    if (nsteps <= 0) return h->fail(DG_ERR_ARG, "nsteps <= 0");
    std::vector<cudaEvent_t> ev(size_t(2 * nsteps + 1), nullptr);
    int rc = DG_OK;
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) rc = h->fail(DG_ERR_CUDA, "cudaEventCreate");
    if (!rc) rc = DISPATCH(h, step_form, istep0, nsteps, ev.data());
    if (!rc && cudaEventSynchronize(ev.back()) != cudaSuccess) rc = h->fail(DG_ERR_CUDA, "event synchronize");
    kernel_ms[0] = kernel_ms[1] = 0;
    for (int s = 0; !rc && s < nsteps; ++s) {
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, ev[2 * s], ev[2 * s + 1]);
        cudaEventElapsedTime(&b, ev[2 * s + 1], ev[2 * s + 2]);
        kernel_ms[0] += a;
        kernel_ms[1] += b;
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    return rc;
}

int dg_step(dg_t *h, int istep) { return dg_run(h, istep, 1); }

int dg_sync(dg_t *h)
{
    if (!h) return DG_ERR_ARG;
    CK(cudaStreamSynchronize(h->stream), "stream synchronize");
    CK(cudaGetLastError(), "pending CUDA error");
    int flag = 0;
    CK(cudaMemcpy(&flag, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag read");
    if (flag) {
        cudaMemset(h->dev_err, 0, sizeof(int));
        return h->fail(DG_ERR_CUDA, "a bounded device wait (the TMA pipeline of a flux or adjoint kernel) timed out");
    }
    return DG_OK;
}

int dg_selftest_wait_timeout(dg_t *h, int limit, long long *waited_cycles)
{
    if (!h || limit < 1 || limit > (1 << 22)) return DG_ERR_ARG;
    int rc = ensure_scratch(h, sizeof(long long));
    if (rc) return rc;
    long long *cyc = reinterpret_cast<long long *>(h->scratch);
    CK(dg::launch_wait_timeout_selftest(h->dev_err, limit, cyc, h->stream), "wait time-out self-test launch");
    long long c = 0;
    CK(cudaMemcpyAsync(&c, cyc, sizeof(c), cudaMemcpyDeviceToHost, h->stream), "wait time-out self-test read");
    CK(cudaStreamSynchronize(h->stream), "wait time-out self-test");
    if (waited_cycles) *waited_cycles = c;
    return DG_OK;
}

int dg_upload_macro(dg_t *h)
{
    if (!h) return DG_ERR_ARG;
    return DISPATCH(h, macro_form);
}

int dg_copy_vel(dg_t *h, double *rho, double *ux, double *uy, double *uz)
{
    if (!h) return DG_ERR_ARG;
    if (!h->macro_valid) {
        const int rc = dg_upload_macro(h);
        if (rc) return rc;
    }
    const size_t g = h->ghosted();
    double *dst[4] = {rho, ux, uy, uz};
    for (int a = 0; a < 4; ++a)
        if (dst[a])
            CK(cudaMemcpyAsync(dst[a], h->macro + a * g, g * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
               "copy_vel");
    CK(cudaStreamSynchronize(h->stream), "copy_vel sync");
    return DG_OK;
}

int dg_stats_values(dg_t *h, double *diag12, double *prof9)
{
    if (!h) return DG_ERR_ARG;
    std::vector<double> tot;
    const int rc = DISPATCH(h, stats_form, tot);
    if (rc) return rc;
    const int nx = h->nx;
    const double nyz = double(h->ny * h->nz), n = double(h->nx * h->ny * h->nz);
    double sum[4] = {0, 0, 0, 0}, mn[4], mx[4], bad = 0;
    for (int a = 0; a < 4; ++a) { mn[a] = 99999; mx[a] = -99999; }  // src/output.cu:232-233
    for (int i = 0; i < nx; ++i) {
        const double *t = &tot[size_t(i) * NSTAT];
        for (int a = 0; a < 4; ++a) {
            sum[a] += t[a];
            if (t[10 + a] < mn[a]) mn[a] = t[10 + a];
            if (t[14 + a] > mx[a]) mx[a] = t[14 + a];
        }
        bad += t[18];
        if (prof9) {
            const double ua = t[1] / nyz, va = t[2] / nyz, wa = t[3] / nyz;
            double *o = prof9 + 9 * size_t(i);
            o[0] = ua; o[1] = va; o[2] = wa;
            o[3] = t[4] / nyz - ua * wa;
            o[4] = t[5] / nyz - ua * va;
            o[5] = t[6] / nyz - va * wa;
            o[6] = t[7] / nyz - ua * ua;
            o[7] = t[8] / nyz - va * va;
            o[8] = t[9] / nyz - wa * wa;
        }
    }
    if (diag12) {
        for (int a = 0; a < 4; ++a) {
            diag12[a] = sum[a] / n;
            diag12[4 + a] = mn[a];
            diag12[8 + a] = mx[a];
        }
    }
    if (bad > 0) return h->fail(DG_ERR_NUMERIC, "state contains NaN or Inf");
    return DG_OK;
}

int dg_stats(dg_t *h, int step)
{
    if (!h) return DG_ERR_ARG;
    std::vector<double> diag(12), prof(size_t(h->nx) * 9);
    const int rc = dg_stats_values(h, diag.data(), prof.data());
    if (rc && rc != DG_ERR_NUMERIC) return rc;
    const std::string dpath = h->workdir + "/diag.dat";
    FILE *file = std::fopen(dpath.c_str(), "a");
    if (!file) return h->fail(DG_ERR_IO, "cannot append '" + dpath + "'");
    std::fprintf(file, "%8.8d  % 7.7e % 7.7e % 7.7e % 7.7e  % 7.7e % 7.7e % 7.7e % 7.7e  % 7.7e % 7.7e % 7.7e % 7.7e\n",
                 step, diag[0], diag[1], diag[2], diag[3], diag[4], diag[5], diag[6], diag[7], diag[8], diag[9],
                 diag[10], diag[11]);
    std::fclose(file);
    const std::string ppath = h->workdir + "/profiles-2.dat";
    file = std::fopen(ppath.c_str(), "a");
    if (!file) return h->fail(DG_ERR_IO, "cannot append '" + ppath + "'");
    std::fprintf(file, "%8.8d\n", step);
    for (int i = 0; i < h->nx; ++i) {
        const double *o = &prof[size_t(i) * 9];
        std::fprintf(file, "% 7.7e % 7.7e % 7.7e   % 7.7e % 7.7e % 7.7e   % 7.7e % 7.7e % 7.7e \n", o[0], o[1], o[2],
                     o[3], o[4], o[5], o[6], o[7], o[8]);
    }
    std::fclose(file);
    return rc;
}

int dg_spectral_stats(dg_t *h, double *vals14, double *spectrum, int nbins)
{
    if (!h || nbins < 0 || (nbins > 0 && !spectrum)) return DG_ERR_ARG;
    if (!h->periodic[0]) return h->fail(DG_ERR_UNSUPPORTED, "spectral statistics need a periodic box (periods_x=1)");
    double v[SV_COUNT];
    std::vector<double> sh;
    const int rc = DISPATCH(h, spectral_form, v, &sh);
    if (rc) return rc;
    if (vals14) std::memcpy(vals14, v, sizeof(v));
    for (int b = 0; b < nbins; ++b) spectrum[b] = b < int(sh.size()) ? sh[size_t(b)] : 0.0;
    return DG_OK;
}

int dg_output_spectral(dg_t *h, int step)
{
    if (!h) return DG_ERR_ARG;
    if (!h->periodic[0]) return h->fail(DG_ERR_UNSUPPORTED, "spectral statistics need a periodic box (periods_x=1)");
    double v[SV_COUNT];
    std::vector<double> sh;
    const int rc = DISPATCH(h, spectral_form, v, &sh);
    if (rc) return rc;
    const double dt = h->prec == DG_PREC_FP64 ? h->c64.dt : double(h->c32.dt), t = step * dt;
    auto append = [&](const char *name) -> FILE * { return std::fopen((h->workdir + "/" + name).c_str(), "a"); };
    FILE *fp = append("KE.dat");  // (I6.6,1X,F12.5,1X,1pe16.9)
    if (!fp) return h->fail(DG_ERR_IO, "cannot append KE.dat");
    std::fprintf(fp, "%06d %12.5f %16.9E\n", step, t, v[SV_TE]);
    std::fclose(fp);
    fp = append("stat_te.dat");  // (I7,1X,F16.8,1X,1pe15.6)
    if (!fp) return h->fail(DG_ERR_IO, "cannot append stat_te.dat");
    std::fprintf(fp, "%7d %16.8f %15.6E\n", step, t, v[SV_TE]);
    std::fclose(fp);
    fp = append("stat_te_spectral.dat");  // (I7,1X,F16.8,1X,3(1pe15.6,1X),8(1pe15.6,1X))
    if (!fp) return h->fail(DG_ERR_IO, "cannot append stat_te_spectral.dat");
    std::fprintf(fp, "%7d %16.8f ", step, t);
    for (int q = SV_ETOTAL; q <= SV_KMXETA; ++q) std::fprintf(fp, "%15.6E ", v[q]);
    std::fprintf(fp, "\n");
    std::fclose(fp);
    char name[32];
    std::snprintf(name, sizeof(name), "spe%9.9d.dat", step);  // (I4,1X,1pe15.6), shells 0..nx
    fp = std::fopen((h->workdir + "/" + name).c_str(), "w");
    if (!fp) return h->fail(DG_ERR_IO, std::string("cannot write ") + name);
    for (int b = 0; b <= h->nx; ++b) std::fprintf(fp, "%4d %15.6E\n", b, b < int(sh.size()) ? sh[size_t(b)] : 0.0);
    std::fclose(fp);
    fp = append("skew-flat.dat");  // (I7,1X,1pe15.6,1X,1pe15.6,1X,1pe15.6)
    if (!fp) return h->fail(DG_ERR_IO, "cannot append skew-flat.dat");
    std::fprintf(fp, "%7d %15.6E %15.6E %15.6E\n", step, t, v[SV_SKEW], v[SV_FLAT]);
    std::fclose(fp);
    return DG_OK;
}

int dg_output_2d(dg_t *h, int step)
{
    if (!h) return DG_ERR_ARG;
    int rc = dg_upload_macro(h);
    if (rc) return rc;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const size_t g = h->ghosted();
    std::vector<double> m(4 * g);
    rc = dg_copy_vel(h, m.data(), m.data() + g, m.data() + 2 * g, m.data() + 3 * g);
    if (rc) return rc;
    // gathered global arrays, src/parallel.cu:260-272
    auto at = [&](int a, int i, int j, int k) { return m[a * g + (size_t(k + 1) * (ny + 2) + (j + 1)) * (nx + 2) + (i + 1)]; };
    const double dx = h->prec == DG_PREC_FP64 ? h->c64.dx : h->c32.dx;
    const double dy = h->prec == DG_PREC_FP64 ? h->c64.dy : h->c32.dy;
    const double dz = h->prec == DG_PREC_FP64 ? h->c64.dz : h->c32.dz;
    auto xpos = [&](int i) { return h->mesh ? h->xc[i + 1] : (i + 0.5) * dx; };
    // src/output.cu:152-218
    const char *tags[3] = {"s2X", "s2Y", "s2Z"};
    for (int s = 0; s < 3; ++s) {
        char name[32];
        std::snprintf(name, sizeof(name), "%s%8.8d.tec", tags[s], step);
        std::ofstream file(h->workdir + "/" + name);
        if (!file) return h->fail(DG_ERR_IO, std::string("cannot write ") + name);
        file << "TITLE = \"Example: Simple 2D-Slice Data\"" << std::endl;
        file << "VARIABLES = \"X\", \"Y\", \"Z\", \"RHO\", \"UX\", \"UY\", \"UZ\"" << std::endl;
        if (s == 0) file << "ZONE I=" << 1 << ", J=" << ny << ", K=" << nz << " F=POINT" << std::endl;
        if (s == 1) file << "ZONE I=" << nx << ", J=" << 1 << ", K=" << nz << " F=POINT" << std::endl;
        if (s == 2) file << "ZONE I=" << nx << ", J=" << ny << ", K=" << 1 << " F=POINT" << std::endl;
        auto row = [&](int i, int j, int k) {
            file << xpos(i) << " " << (j + 0.5) * dy << " " << (k + 0.5) * dz << " " << at(0, i, j, k) << " "
                 << at(1, i, j, k) << " " << at(2, i, j, k) << " " << at(3, i, j, k) << std::endl;
        };
        if (s == 0)
            for (int k = 0; k < nz; k++)
                for (int j = 0; j < ny; j++) row(nx / 2, j, k);
        if (s == 1)
            for (int k = 0; k < nz; k++)
                for (int i = 0; i < nx; i++) row(i, ny / 2, k);
        if (s == 2)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) row(i, j, nz / 2);
    }
    return dg_stats(h, step);
}

int dg_get_state(dg_t *h, double *f_dump_order)
{
    if (!h || !f_dump_order) return DG_ERR_ARG;
    return DISPATCH(h, get_state_form, f_dump_order);
}

int dg_set_state(dg_t *h, const double *f_dump_order)
{
    if (!h || !f_dump_order) return DG_ERR_ARG;
    return DISPATCH(h, set_state_form, f_dump_order);
}

int dg_copy_ddf(dg_t *h, double *f_ghosted)
{
    if (!h || !f_ghosted) return DG_ERR_ARG;
    std::vector<double> tmp(h->ncell() * 19);
    const int rc = dg_get_state(h, tmp.data());
    if (rc) return rc;
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    std::memset(f_ghosted, 0, h->ghosted() * 19 * sizeof(double));
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t s = ((size_t(k) * ny + j) * nx + i) * 19;
                const size_t d = ((size_t(k + 1) * (ny + 2) + (j + 1)) * (nx + 2) + (i + 1)) * 19;
                std::memcpy(f_ghosted + d, tmp.data() + s, 19 * sizeof(double));
            }
    return DG_OK;
}

int dg_dump(dg_t *h, int step)
{
    if (!h) return DG_ERR_ARG;
    std::vector<double> f(h->ncell() * 19);
    int rc = dg_get_state(h, f.data());
    if (rc) return rc;
    char name[32];
    std::snprintf(name, sizeof(name), "ddf%8.8d.dat", step);
    const std::string path = h->workdir + "/" + name;
    std::ofstream out(path, std::ios::binary);
    if (!out) return h->fail(DG_ERR_IO, "cannot write '" + path + "'");
    if (h->prec == DG_PREC_FP64) {
        out.write(reinterpret_cast<const char *>(f.data()), std::streamsize(f.size() * sizeof(double)));
    } else {
        std::vector<float> g(f.begin(), f.end());
        out.write(reinterpret_cast<const char *>(g.data()), std::streamsize(g.size() * sizeof(float)));
    }
    if (!out) return h->fail(DG_ERR_IO, "short write to '" + path + "'");
    return DG_OK;
}

int dg_read_dump(dg_t *h, int step)
{
    if (!h) return DG_ERR_ARG;
    std::vector<double> f;
    int rc = read_dump_file(h, step, f);
    if (rc) return rc;
    rc = check_finite(h, f);
    if (rc) return rc;
    return dg_set_state(h, f.data());
}

const void *dg_device_ptr(const dg_t *h, int which)
{
    if (!h) return nullptr;
    const size_t g = h->ghosted();
    switch (which) {
    case DG_BUF_F: return h->f;
    case DG_BUF_FB: return h->fb;
    case DG_BUF_RHO: return h->macro;
    case DG_BUF_UX: return h->macro ? h->macro + g : nullptr;
    case DG_BUF_UY: return h->macro ? h->macro + 2 * g : nullptr;
    case DG_BUF_UZ: return h->macro ? h->macro + 3 * g : nullptr;
    }
    return nullptr;
}

int dg_adjoint_step(dg_t *h, int istep, const void *f_n, const void *lam_next, void *lam_out)
{
    if (!h || !f_n || !lam_next || !lam_out) return DG_ERR_ARG;
    if (f_n == h->fb || lam_next == h->fb || lam_out == h->fb || f_n == lam_out)
        return h->fail(DG_ERR_ARG, "adjoint buffers must not alias f-bar-plus or each other (lam_out may equal lam_next)");
    return DISPATCH(h, adjoint_form, istep, f_n, lam_next, lam_out);
}

int dg_run_store(dg_t *h, int istep0, int n, void *states, long long stride_bytes)
{
    if (!h || n < 0 || (n > 0 && !states)) return DG_ERR_ARG;
    const long long sb = (long long)h->ps * 19 * (long long)storage_bytes(h->prec);
    if (n > 1 && stride_bytes < sb) return h->fail(DG_ERR_ARG, "dg_run_store: stride smaller than one state");
    char *base = static_cast<char *>(states);
    for (int s = 0; s < n; ++s) {
        if (base + s * stride_bytes == h->fb) return h->fail(DG_ERR_ARG, "dg_run_store: a state slot aliases f-bar-plus");
        int rc = dg_get_state_device(h, base + s * stride_bytes);
        if (!rc && s + 1 < n) rc = dg_step(h, istep0 + s);
        if (rc) return rc;
    }
    return DG_OK;
}

int dg_adjoint_run(dg_t *h, int istep0, int n, const void *states, long long stride_bytes, void *lam)
{
    if (!h || n < 0 || (n > 0 && (!states || !lam))) return DG_ERR_ARG;
    const long long sb = (long long)h->ps * 19 * (long long)storage_bytes(h->prec);
    if (n > 1 && stride_bytes < sb) return h->fail(DG_ERR_ARG, "dg_adjoint_run: stride smaller than one state");
    const char *base = static_cast<const char *>(states);
    const char *lo = base, *hi = base + (n - 1) * stride_bytes + sb, *l = static_cast<const char *>(lam);
    if (n > 0 && l + sb > lo && l < hi) return h->fail(DG_ERR_ARG, "dg_adjoint_run: lam overlaps the states");
    for (int s = n - 1; s >= 0; --s) {
        const int rc = dg_adjoint_step(h, istep0 + s, base + s * stride_bytes, lam, lam);
        if (rc) return rc;
    }
    return DG_OK;
}

int dg_set_force_field(dg_t *h, int axis, const double *phi)
{
    if (!h) return DG_ERR_ARG;
    h->drop_graph();  // the captured steps hold the field pointer and axis
    if (!phi) {
        if (h->ffield) CK(cudaFree(h->ffield), "cudaFree (force field)");
        h->ffield = nullptr;
        return DG_OK;
    }
    if (axis < 0 || axis > 2) return h->fail(DG_ERR_ARG, "force-field axis must be 0 (x), 1 (y) or 2 (z)");
    if (h->perturb) return h->fail(DG_ERR_UNSUPPORTED, "a force field cannot be combined with perturb=1");
    const size_t es = h->prec == DG_PREC_FP64 ? sizeof(double) : sizeof(float);
    const size_t n = size_t(h->pitch) * h->ny * h->nz;
    std::vector<char> buf(n * es, 0);
    for (int k = 0; k < h->nz; ++k)
        for (int j = 0; j < h->ny; ++j)
            for (int i = 0; i < h->nx; ++i) {
                const double v = phi[(size_t(k) * h->ny + j) * h->nx + i];
                if (!std::isfinite(v)) return h->fail(DG_ERR_NUMERIC, "force field holds a non-finite value");
                const size_t c = (size_t(k) * h->ny + j) * h->pitch + i;
                if (es == sizeof(double)) reinterpret_cast<double *>(buf.data())[c] = v;
                else reinterpret_cast<float *>(buf.data())[c] = float(v);
            }
    if (!h->ffield) CK(cudaMalloc(&h->ffield, buf.size()), "cudaMalloc (force field)");
    // synchronous: the host buffer is released on return and earlier steps may still read the old field
    CK(cudaStreamSynchronize(h->stream), "force-field sync");
    CK(cudaMemcpy(h->ffield, buf.data(), buf.size(), cudaMemcpyHostToDevice), "force-field copy");
    h->ffaxis = axis;
    return DG_OK;
}

int dg_field_grad(dg_t *h, double *dphi, int reset)
{
    if (!h) return DG_ERR_ARG;
    if (dphi) {
        if (h->dphi) {
            CK(cudaMemcpyAsync(dphi, h->dphi, h->ncell() * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
               "field-gradient copy");
            CK(cudaStreamSynchronize(h->stream), "field-gradient sync");
        } else {
            std::fill(dphi, dphi + h->ncell(), 0.0);
        }
    }
    if (reset && h->dphi)
        CK(cudaMemsetAsync(h->dphi, 0, h->ncell() * sizeof(double), h->stream), "cudaMemset (field gradient)");
    return DG_OK;
}

int dg_get_state_device(dg_t *h, void *dst)
{
    if (!h || !dst) return DG_ERR_ARG;
    CK(cudaMemcpyAsync(dst, h->f, size_t(h->ps) * 19 * storage_bytes(h->prec), cudaMemcpyDeviceToDevice, h->stream),
       "state copy (device)");
    return DG_OK;
}

int dg_set_state_device(dg_t *h, const void *src)
{
    if (!h || !src) return DG_ERR_ARG;
    CK(cudaMemcpyAsync(h->f, src, size_t(h->ps) * 19 * storage_bytes(h->prec), cudaMemcpyDeviceToDevice, h->stream),
       "state copy (device)");
    h->macro_valid = false;
    return DG_OK;
}

int dg_stats_accumulate(dg_t *h)
{
    if (!h) return DG_ERR_ARG;
    return DISPATCH(h, accumulate_form);
}

int dg_stats_accumulated(dg_t *h, double *prof9, long long *count)
{
    if (!h) return DG_ERR_ARG;
    if (count) *count = h->acc_count;
    if (!prof9) return DG_OK;
    const int nx = h->nx;
    std::vector<double> a(size_t(nx) * 10, 0.0);
    if (h->acc) {
        CK(cudaMemcpyAsync(a.data(), h->acc, a.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
           "accumulator copy");
        CK(cudaStreamSynchronize(h->stream), "accumulator sync");
    }
    const double n = double(h->ny) * h->nz * double(h->acc_count > 0 ? h->acc_count : 1);
    for (int i = 0; i < nx; ++i) {
        const double *t = &a[size_t(i) * 10];
        const double ua = t[1] / n, va = t[2] / n, wa = t[3] / n;
        double *o = prof9 + 9 * size_t(i);
        o[0] = ua; o[1] = va; o[2] = wa;
        o[3] = t[4] / n - ua * wa;
        o[4] = t[5] / n - ua * va;
        o[5] = t[6] / n - va * wa;
        o[6] = t[7] / n - ua * ua;
        o[7] = t[8] / n - va * va;
        o[8] = t[9] / n - wa * wa;
    }
    return DG_OK;
}

int dg_stats_reset(dg_t *h)
{
    if (!h) return DG_ERR_ARG;
    if (h->acc) CK(cudaMemsetAsync(h->acc, 0, size_t(h->nx) * 10 * sizeof(double), h->stream), "cudaMemset (accumulator)");
    h->acc_count = 0;
    return DG_OK;
}

int dg_get_mesh(const dg_t *h, double *xc, double *dxx)
{
    if (!h) return DG_ERR_ARG;
    for (int i = 0; i <= h->nx + 1; ++i) {
        if (xc) xc[i] = h->mesh ? h->xc[i] : (i - 0.5) * (h->prec == DG_PREC_FP64 ? h->c64.dx : double(h->c32.dx));
        if (dxx) dxx[i] = h->mesh ? h->dxx[i] : (h->prec == DG_PREC_FP64 ? h->c64.dx : double(h->c32.dx));
    }
    return DG_OK;
}

int dg_moments(dg_t *h, double *mass_mom4)
{
    if (!h || !mass_mom4) return DG_ERR_ARG;
    return DISPATCH(h, moments_form, mass_mom4);
}

}  // extern "C"
