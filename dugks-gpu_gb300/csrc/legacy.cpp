// Legacy names of the reference's solver interface (src/dugks.h:1-9) over the
// handle API, so that a driver written against them -- the reference's own
// src/main.cu among them -- links unchanged.  Compiled twice: real = double
// (libdugks_legacy.so) and, with -DPREC4, real = float
// (libdugks_legacy_prec4.so, an fp32 engine unless config.txt names another
// precision).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dugks_gb300.h"
#include "../../include/dugks_legacy.h"

typedef dugks_legacy_real real;

real *h_rho = nullptr, *h_ux = nullptr, *h_uy = nullptr, *h_uz = nullptr;
real *h_f = nullptr;

namespace {

dg_t *g_engine = nullptr;
dg_info_t g_info;
[[maybe_unused]] std::vector<double> g_tmp;  // double staging of the copies when real is float

[[noreturn]] void die(const char *what, int rc)
{
    std::printf("ERROR: %s failed (status %d): %s\n", what, rc, dg_last_error(g_engine));
    std::fflush(stdout);
    std::exit(1);
}

void check(int rc, const char *what)
{
    if (rc != DG_OK) die(what, rc);
}

size_t ghosted_cells()
{
    return size_t(g_info.nx + 2) * (g_info.ny + 2) * (g_info.nz + 2);
}

void need_engine(const char *what)
{
    if (!g_engine) {
        std::printf("ERROR: %s called before init_dugks\n", what);
        std::fflush(stdout);
        std::exit(1);
    }
}

// dst (real) <- src (double), n values
[[maybe_unused]] void store(real *dst, const double *src, size_t n)
{
    for (size_t q = 0; q < n; ++q) dst[q] = real(src[q]);
}

}  // namespace

void init_dugks(void)
{
    if (g_engine) return;
    // src/config.h:21 reads config.txt from the working directory
    std::ifstream in("config.txt");
    if (!in) {
        std::printf("ERROR: cannot open config.txt\n");
        std::fflush(stdout);
        std::exit(1);
    }
    std::stringstream text;
    text << in.rdbuf();
    std::string cfg = text.str();
#ifdef PREC4
    // the PREC4 build computes in float: an fp32 engine unless the file chooses
    // (the first occurrence of a key wins, so an appended default never overrides)
    cfg += "\nprecision=fp32\n";
#endif
    const int rc = dg_create_from_text(cfg.c_str(), ".", &g_engine);
    if (rc != DG_OK) {
        std::printf("ERROR: init_dugks: status %d: %s\n", rc, dg_last_error(nullptr));
        std::fflush(stdout);
        std::exit(1);
    }
    check(dg_get_info(g_engine, &g_info), "dg_get_info");
    const size_t n = ghosted_cells();
    h_rho = new real[n]();
    h_ux = new real[n]();
    h_uy = new real[n]();
    h_uz = new real[n]();
    h_f = new real[n * 19]();
}

void dugks_step(int step)
{
    need_engine("dugks_step");
    check(dg_step(g_engine, step), "dugks_step");
    check(dg_sync(g_engine), "dugks_step");
}

void upload_macro()
{
    need_engine("upload_macro");
    check(dg_upload_macro(g_engine), "upload_macro");
}

void copy_vel(void)
{
    need_engine("copy_vel");
    const size_t n = ghosted_cells();
#ifdef PREC4
    g_tmp.resize(4 * n);
    check(dg_copy_vel(g_engine, g_tmp.data(), g_tmp.data() + n, g_tmp.data() + 2 * n, g_tmp.data() + 3 * n),
          "copy_vel");
    store(h_rho, g_tmp.data(), n);
    store(h_ux, g_tmp.data() + n, n);
    store(h_uy, g_tmp.data() + 2 * n, n);
    store(h_uz, g_tmp.data() + 3 * n, n);
#else
    (void)n;
    check(dg_copy_vel(g_engine, h_rho, h_ux, h_uy, h_uz), "copy_vel");
#endif
}

void copy_ddf(void)
{
    need_engine("copy_ddf");
#ifdef PREC4
    const size_t n = ghosted_cells() * 19;
    g_tmp.resize(n);
    check(dg_copy_ddf(g_engine, g_tmp.data()), "copy_ddf");
    store(h_f, g_tmp.data(), n);
#else
    check(dg_copy_ddf(g_engine, h_f), "copy_ddf");
#endif
}
