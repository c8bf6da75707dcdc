// A driver written against the reference's solver interface, linked against
// libdugks_legacy.so (or, with -DPREC4, libdugks_legacy_prec4.so): the call
// sequence of src/main.cu:16-43 -- init_dugks, then dugks_step every step,
// upload_macro + copy_vel at output steps and copy_ddf + a dump at dump steps.
// The dump is written as src/output.cu:22-41 writes it (the interior of h_f,
// cell by cell k-major, 19 reals each, raw); at output steps the ghosted
// macro arrays h_rho, h_ux, h_uy, h_uz go raw to macro%08d.dat.
//   legacy_main NX NY NZ ISTEP0 NSTEPS NOUTPUT2 NDUMP
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dugks_legacy.h"

typedef dugks_legacy_real real;

static void write_raw(const char *prefix, int step, const real *p, size_t n)
{
    char name[64];
    std::snprintf(name, sizeof(name), "%s%8.8d.dat", prefix, step);
    FILE *fp = std::fopen(name, "wb");
    if (!fp || std::fwrite(p, sizeof(real), n, fp) != n) std::exit(3);
    std::fclose(fp);
}

int main(int argc, char **argv)
{
    if (argc != 8) return 2;
    const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
    const int istep0 = std::atoi(argv[4]), nsteps = std::atoi(argv[5]);
    const int noutput2 = std::atoi(argv[6]), ndump = std::atoi(argv[7]);
    const size_t ng = size_t(nx + 2) * (ny + 2) * (nz + 2);
    init_dugks();
    std::vector<real> fg(size_t(nx) * ny * nz * 19), mac(4 * ng);
    for (int istep = istep0; istep <= istep0 + nsteps - 1; istep++) {
        dugks_step(istep);
        if (istep == istep0 || istep % noutput2 == 0) {
            upload_macro();
            copy_vel();
            const real *src[4] = {h_rho, h_ux, h_uy, h_uz};
            for (int a = 0; a < 4; ++a)
                for (size_t q = 0; q < ng; ++q) mac[a * ng + q] = src[a][q];
            write_raw("macro", istep, mac.data(), mac.size());
        }
        if (istep % ndump == 0) {
            copy_ddf();
            for (int k = 0; k < nz; k++)
                for (int j = 0; j < ny; j++)
                    for (int i = 0; i < nx; i++)
                        for (int p = 0; p < 19; p++)
                            fg[((size_t(k) * ny + j) * nx + i) * 19 + p] =
                                h_f[((size_t(k + 1) * (ny + 2) + j + 1) * (nx + 2) + i + 1) * 19 + p];
            write_raw("ddf", istep, fg.data(), fg.size());
        }
    }
    return 0;
}
