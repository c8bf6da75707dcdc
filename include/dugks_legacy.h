/*
 * Legacy names of the reference's solver interface, for drivers written
 * against it (Kairzhan/DUGKS-GPU src/dugks.h:1-9, driven by src/main.cu:16-43).
 *
 * libdugks_legacy.so (real = double) and libdugks_legacy_prec4.so (real =
 * float, the reference's PREC4 build) export exactly these symbols, with the
 * reference's C++ linkage, on top of the handle API of dugks_gb300.h, so that
 * the reference's own src/main.cu, src/output.cu, src/parallel.cu,
 * src/numerics.cu, src/cuda.cu and src/checks.cu link against them unchanged in
 * place of src/dugks.cu.  The library holds one engine handle.
 *
 * Behaviour kept from the reference because the signatures return nothing:
 * the configuration is config.txt in the working directory (src/config.h:21),
 * and a failure prints "ERROR: <message>" and ends the process with exit(1),
 * where the reference exits or crashes.  dugks_step returns after the step has
 * finished on the GPU (the reference ends it with cudaDeviceSynchronize).
 */
#ifndef DUGKS_LEGACY_H
#define DUGKS_LEGACY_H

#ifdef PREC4
typedef float dugks_legacy_real;
#else
typedef double dugks_legacy_real;
#endif

/* Host mirrors, allocated by init_dugks (src/dugks.cu:204-209):
 *   h_rho, h_ux, h_uy, h_uz  (lx+2)(ly+2)(lz+2) values, ghosted, index
 *                            (k*(ly+2) + j)*(lx+2) + i; filled by copy_vel
 *   h_f                      19*(lx+2)(ly+2)(lz+2) values, ghosted AoS, index
 *                            ((k*(ly+2) + j)*(lx+2) + i)*19 + p; filled by copy_ddf
 * Ghost entries are zero. */
extern dugks_legacy_real *h_rho, *h_ux, *h_uy, *h_uz;
extern dugks_legacy_real *h_f;

/* Replaces init_dugks (src/dugks.cu:95-302): reads config.txt, builds the
 * engine (initial state or restart dump) and allocates the host mirrors. */
void init_dugks(void);
/* Replaces dugks_step (src/dugks.cu:322-391): one DUGKS step, synchronous. */
void dugks_step(int step);
/* Replaces copy_vel (src/dugks.cu:393-405): macro fields into h_rho..h_uz
 * (upload_macro first, as the reference's driver does). */
void copy_vel(void);
/* Replaces copy_ddf (src/dugks.cu:407-416): f-tilde into h_f. */
void copy_ddf(void);
/* Replaces upload_macro (src/dugks.cu:311-320): rho and u = j/rho + hdt*F on the device. */
void upload_macro();

#endif
