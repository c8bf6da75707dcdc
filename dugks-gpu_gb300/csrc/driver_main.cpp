// Host driver with the reference's time loop (src/main.cu:14-56): reads
// ./config.txt (or the path given as argv[1]), runs istep0 .. istep0+nsteps-1,
// writes the statistics and slices at istep==istep0 or istep%noutput2==0 and
// a dump at istep%ndump==0, and prints the main-loop wall time.
//
//   dugks_gb300 [config.txt] [--quiet]
//
// --quiet drops the per-step "istep = N" line (src/main.cu:27-29).
#include <chrono>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <iostream>

#include "dugks_gb300.h"

int main(int argc, char **argv)
{
    const char *cfg = "config.txt";
    bool quiet = false;
    for (int a = 1; a < argc; ++a) {
        if (std::strcmp(argv[a], "--quiet") == 0) quiet = true;
        else cfg = argv[a];
    }
    dg_t *h = nullptr;
    int rc = dg_create(cfg, &h);
    if (rc) {
        std::cerr << "ERROR: " << dg_last_error(nullptr) << " (status " << rc << ")" << std::endl;
        return 1;
    }
    dg_info_t info;
    dg_get_info(h, &info);
    const auto t0 = std::chrono::steady_clock::now();
    for (int istep = info.istep0; istep <= info.istep0 + info.nsteps - 1; istep++) {
        if (!quiet) std::cout << "istep = " << std::setw(8) << istep << std::endl;
        rc = dg_step(h, istep);
        if (!rc && (istep == info.istep0 || istep % info.noutput2 == 0)) rc = dg_output_2d(h, istep);
        if (!rc && istep % info.ndump == 0) rc = dg_dump(h, istep);
        if (rc) {
            std::cerr << "ERROR at step " << istep << ": " << dg_last_error(h) << " (status " << rc << ")" << std::endl;
            dg_destroy(h);
            return 1;
        }
    }
    rc = dg_sync(h);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc) std::cerr << "ERROR: " << dg_last_error(h) << std::endl;
    std::cout << "Main loop time: " << secs << " seconds." << std::endl;
    dg_destroy(h);
    return rc ? 1 : 0;
}
