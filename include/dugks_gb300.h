/*
 * dugks_gb300 -- C ABI of the GB300-native D3Q19 DUGKS time-step engine.
 *
 * A handle-based replacement for the reference's module-global solver
 * interface (Kairzhan/DUGKS-GPU src/dugks.h:1-9, src/output.h:1-5).  Plain
 * pointers and sizes only; every call returns an int status (DG_OK == 0,
 * negative on error) and never exits the process.  One handle per host
 * thread; a handle owns all of its device memory and frees it in
 * dg_destroy().
 *
 * Host-side arrays exchanged through this interface are always double,
 * whatever the engine's storage precision.  Layouts:
 *   - "ghosted AoS" (the reference's h_f, src/dugks.cu:15-17):
 *       f[((k*(ny+2)+j)*(nx+2)+i)*19+ip], 0<=i<nx+2 ...
 *   - "dump order" (ddf%08d.dat, src/output.cu:22-41):
 *       f[((k*ny+j)*nx+i)*19+ip], interior cells only
 *   - "ghosted scalar" (h_rho, h_ux ..., src/dugks.cu:204-207):
 *       a[(k*(ny+2)+j)*(nx+2)+i]
 */
#ifndef DUGKS_GB300_H
#define DUGKS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dg_ctx dg_t;

/* status codes */
#define DG_OK 0
#define DG_ERR_CONFIG (-1)      /* missing / malformed config key */
#define DG_ERR_IO (-2)          /* file missing, short or oversized */
#define DG_ERR_SHAPE (-3)       /* grid sizes / buffer sizes inconsistent */
#define DG_ERR_CUDA (-4)        /* a CUDA runtime call or launch failed */
#define DG_ERR_NUMERIC (-5)     /* NaN / Inf detected in the state */
#define DG_ERR_ARG (-6)         /* NULL handle or pointer, bad enum */
#define DG_ERR_UNSUPPORTED (-7) /* boundary / option the engine does not implement */

/* storage / arithmetic forms (config key `precision`) */
#define DG_PREC_FP64 0          /* FP64 storage and arithmetic (parity mode) */
#define DG_PREC_FP32 1          /* FP32 storage and arithmetic */
#define DG_PREC_FP16 2          /* FP16 deviation storage, FP32 arithmetic */
#define DG_PREC_BF16 3          /* BF16 deviation storage, FP32 arithmetic */

/* device buffers exposed read-only (dg_device_ptr) */
#define DG_BUF_F 0              /* f-tilde, structure of arrays */
#define DG_BUF_FB 1             /* f-bar-plus, structure of arrays with x ghost columns 0, nx+1; scratch
                                 * of every step and of the host state transfers (dg_set_state,
                                 * dg_get_state, dg_copy_ddf, dg_dump), which may overwrite it; the
                                 * fp16 / bf16 forms between walls do not store its x ghost columns */
#define DG_BUF_RHO 2            /* ghosted scalar macro arrays (after dg_upload_macro) */
#define DG_BUF_UX 3
#define DG_BUF_UY 4
#define DG_BUF_UZ 5

typedef struct {
    int nx, ny, nz;             /* interior cells */
    int pitch;                  /* x pitch of the device SoA arrays, elements */
    long long pop_stride;       /* elements between populations in the device SoA arrays */
    int precision;              /* DG_PREC_* */
    int periodic[3];            /* periods_x/y/z */
    int mesh;                   /* 0 uniform, 1 tanh-stretched x, 2 x faces from a mesh file */
    int recon;                  /* 0 trilinear, 1 central-difference gradient */
    int perturb;                /* calc_perturb_force active */
    int istep0, nsteps, noutput2, ndump, restart, nrestart;
    double dx, dy, dz, dt, visc, tau;
    double xwidth, ywidth, zwidth;
    double ambient[3];
    double bw0, bw1, bw2, fw0, fw1, fw2;
    double hbm_bytes_per_cell;  /* algorithmic HBM bytes per cell update of one step */
} dg_info_t;

/* --- lifetime ---------------------------------------------------------- */

/* Reads a reference config.txt (same keys and std::stof / std::stoi parsing,
 * src/numerics.cu:62-106, src/parallel.cu:95-97, src/cuda.cu:17), allocates
 * the device state and sets the initial condition of `case` or, with
 * restart=1, reads ddf<nrestart>.dat from the config file's directory.
 * Replaces Numerics::init_numerics + init_parallel + init_cuda + init_dugks
 * (src/main.cu:16-20, src/dugks.cu:95-302). */
int dg_create(const char *config_path, dg_t **out);

/* Same, from config text; dumps / statistics files go to `workdir`. */
int dg_create_from_text(const char *config_text, const char *workdir, dg_t **out);

/* Frees everything the handle owns. */
int dg_destroy(dg_t *h);

/* Message of the last failing call on this handle (or of the last failing
 * dg_create* when h is NULL). */
const char *dg_last_error(const dg_t *h);

int dg_get_info(const dg_t *h, dg_info_t *info);

/* Caller-supplied stream (a cudaStream_t); 0 = legacy default stream. */
int dg_set_stream(dg_t *h, void *cuda_stream);

/* --- time stepping ----------------------------------------------------- */

/* One DUGKS step (stage a, ghost fill, stages b-e), asynchronous on the
 * handle's stream.  Replaces dugks_step(int) (src/dugks.cu:322-391). */
int dg_step(dg_t *h, int istep);

/* Steps istep0 .. istep0+nsteps-1 back to back, asynchronous. */
int dg_run(dg_t *h, int istep0, int nsteps);

/* Steps istep0 .. istep0+nsteps-1 from the state at src into the state at
 * dst, asynchronous (no counterpart in the reference; for checkpointed
 * reversals, which step from a stored state without copying it in first):
 * src and dst are device arrays in the engine's SoA state layout
 * (19*pop_stride values of the storage type, like dg_device_ptr(h,
 * DG_BUF_F)), NULL meaning the handle's own state.  The first step reads src
 * and writes dst, the others update dst in place; src stays unchanged unless
 * it equals dst, and the handle's own state changes only when it is dst.
 * DG_ERR_ARG when dst overlaps f-bar-plus or src and dst overlap partly. */
int dg_run_between(dg_t *h, int istep0, int nsteps, const void *src, void *dst);

/* dg_run with every launch bracketed by CUDA events on the handle's stream;
 * waits for completion and returns the summed milliseconds of the stage (a)
 * launches in kernel_ms[0] and of the flux launches in kernel_ms[1]. */
int dg_run_profiled(dg_t *h, int istep0, int nsteps, double *kernel_ms);

/* Waits for the handle's stream and reports any pending CUDA error, and
 * DG_ERR_CUDA when a kernel gave up a bounded device wait (the TMA pipelines
 * of the flux and adjoint kernels poll their mbarriers a bounded number of
 * times, then raise a device flag and finish instead of hanging).  Reading the
 * flag clears it. */
int dg_sync(dg_t *h);

/* Self-test of that time-out path (no counterpart in the reference): one
 * kernel waits `limit` polls (1 .. 2^22; the pipelines use 2^18) on an mbarrier that nothing arrives
 * at -- no copy is issued, nothing is in flight -- raises the handle's device
 * flag and returns.  Synchronous; the SM cycles spent waiting go to
 * *waited_cycles (may be NULL).  The next dg_sync returns DG_ERR_CUDA and the
 * handle stays usable. */
int dg_selftest_wait_timeout(dg_t *h, int limit, long long *waited_cycles);

/* --- macroscopic output and statistics --------------------------------- */

/* rho, u = j/rho + hdt*F on device (src/dugks.cu:311-320, 1021-1064). */
int dg_upload_macro(dg_t *h);

/* Copies the macro arrays to host, ghosted scalar layout; any pointer may be
 * NULL (src/dugks.cu:393-405 copy_vel). */
int dg_copy_vel(dg_t *h, double *rho, double *ux, double *uy, double *uz);

/* diag.dat values (mean rho,u,v,w; min ...; max ...) and the 9 x nx
 * profiles-2.dat values of src/output.cu:223-334, reduced on the device in
 * FP64 from the current state (calls dg_upload_macro). */
int dg_stats_values(dg_t *h, double *diag12, double *prof9);

/* Appends diag.dat and profiles-2.dat in the working directory with the
 * reference's formats (src/output.cu:261-333). */
int dg_stats(dg_t *h, int step);

/* dg_stats plus the Tecplot slices s2X/s2Y/s2Z%08d.tec of
 * src/output.cu:152-218 (output_2d, src/output.cu:118-147). */
int dg_output_2d(dg_t *h, int step);

/* Spectral statistics of a periodic box: the statistics of the reference's
 * Fortran decaying-turbulence code (src/fortran/dhit/src/stat.f90:5-205) from
 * the current state, u = j/rho (src/fortran/dhit/src/main.cuf:86-103), on
 * the device with cuFFT (loaded on first use), in FP64.  vals14 (may be
 * NULL): kinetic energy 0.5<|u|^2>, spectral energy, dissipation, 0 (the
 * reference's ediss_total), Kolmogorov length, velocity and time, u', Taylor
 * microscale, Taylor Reynolds number, large-eddy length, kmax*eta, skewness
 * and flatness of the longitudinal derivatives.  spectrum (may be NULL):
 * shell energies E(k), k = 0 .. nbins-1 (zero past the last shell).  Needs
 * periods_x=1 (DG_ERR_UNSUPPORTED otherwise). */
int dg_spectral_stats(dg_t *h, double *vals14, double *spectrum, int nbins);

/* dg_spectral_stats written as the reference writes it for step `step`:
 * KE.dat (main.cuf:114-116), stat_te.dat, stat_te_spectral.dat, skew-flat.dat
 * (appended) and spe%09d.dat (stat.f90:60-62, 170-182, 192-194). */
int dg_output_spectral(dg_t *h, int step);

/* Time-averaged statistics (an extension; the reference writes instantaneous
 * profiles only): dg_stats_accumulate adds the current per-x plane sums of
 * u, v, w and their products into FP64 device accumulators;
 * dg_stats_accumulated returns the averages over all accumulated samples in
 * the profiles-2.dat layout (9 values per x index: means, covariances
 * <uw>', <uv>', <vw>', variances) and the sample count; dg_stats_reset clears. */
int dg_stats_accumulate(dg_t *h);
int dg_stats_accumulated(dg_t *h, double *prof9, long long *count);
int dg_stats_reset(dg_t *h);

/* --- state and checkpoint I/O ------------------------------------------ */

/* Full ghosted AoS copy of f-tilde (src/dugks.cu:407-416 copy_ddf); ghost
 * entries are written as 0. */
int dg_copy_ddf(dg_t *h, double *f_ghosted);

/* Interior state in dump order (get) / load it (set). */
int dg_get_state(dg_t *h, double *f_dump_order);
int dg_set_state(dg_t *h, const double *f_dump_order);

/* ddf%08d.dat in the working directory: raw native-endian reals of the
 * engine's dump width (8 B for fp64, 4 B otherwise), dump order, no header
 * (src/output.cu:22-89). */
int dg_dump(dg_t *h, int step);
int dg_read_dump(dg_t *h, int step);

/* Read-only device pointer of one of the DG_BUF_* buffers. */
const void *dg_device_ptr(const dg_t *h, int which);

/* --- harness hooks (used by the adjoint verification harness) ---------- */

/* Total mass, x/y/z momentum of the current state in FP64. */
int dg_moments(dg_t *h, double *mass_mom4);

/* Device-to-device copy of the state in the engine's own SoA layout
 * (19 * pop_stride elements of the storage type, see dg_info_t), on the
 * handle's stream. */
int dg_get_state_device(dg_t *h, void *dst);
int dg_set_state_device(dg_t *h, const void *src);

/* Hand-written adjoint of step `istep` (no counterpart in the reference):
 * lam_out = (dS/df)^T lam_next at the state f_n, all three device arrays in
 * the engine's SoA layout (fp64 and fp32 forms).  Recomputes f-bar-plus of
 * f_n; lam_out may equal lam_next.  Asynchronous on the handle's stream. */
int dg_adjoint_step(dg_t *h, int istep, const void *f_n, const void *lam_next, void *lam_out);

/* Batched forms of the adjoint harness's inner loops (no counterpart in the
 * reference), asynchronous on the handle's stream:
 * dg_run_store records in states[s] (s = 0 .. n-1, slots stride_bytes apart,
 * each one state in the engine's SoA layout) the state from which step
 * istep0 + s starts, advancing the engine's state by the n - 1 steps in
 * between; dg_adjoint_run applies the adjoint steps istep0 + n - 1 down to
 * istep0 to lam in place, step istep0 + s at states[s]. */
int dg_run_store(dg_t *h, int istep0, int n, void *states, long long stride_bytes);
int dg_adjoint_run(dg_t *h, int istep0, int n, const void *states, long long stride_bytes, void *lam);

/* Body-force field (no counterpart in the reference; the control variable
 * of the adjoint drag-reduction harness): F(cell) = ambient + phi(cell) e_axis
 * in stage (a), and on a face the mean of phi over its two cells (the one
 * interior cell on a wall face).  phi: host array of nx*ny*nz doubles in dump
 * order (i fastest); NULL removes the field.  Not combinable with perturb=1.
 * Synchronises the handle's stream. */
int dg_set_force_field(dg_t *h, int axis, const double *phi);

/* dJ/dphi accumulated by dg_adjoint_step over the steps run while a field was
 * set (no counterpart in the reference).  dphi: host array of nx*ny*nz
 * doubles, dump order, may be NULL; reset != 0 zeroes the accumulator after
 * the copy. */
int dg_field_grad(dg_t *h, double *dphi, int reset);

/* Cell centres and widths along x, nx+2 entries each (index 0 and nx+1 are
 * the mirrored ghosts of src/fortran/channel/src/dugks.cuf:118-121); either
 * pointer may be NULL. */
int dg_get_mesh(const dg_t *h, double *xc, double *dxx);

/* --- allocation-free statistics (no counterpart in the reference) ------ */

/* Largest nx accepted by dg_stats_values_noalloc. */
#define DG_NOALLOC_MAX_NX 512

/* The statistics of dg_stats_values (diag.dat and profiles-2.dat values) for
 * callers that cannot allocate device memory at the point where they need
 * them: host programs whose own allocator owns all device memory and forbids
 * later cudaMalloc calls, and callers whose memory budget the state arrays
 * have already spent.  This entry point allocates nothing; its
 * scratch is a fixed array in the library's device image (about 5 MB, present
 * on every GPU that loads the library until the process exits).
 *   f      FP64 state in device memory in the engine's SoA layout, e.g.
 *          dg_device_ptr(h, DG_BUF_F) of an fp64 engine, with nx <=
 *          DG_NOALLOC_MAX_NX and pitch / pop_stride as in dg_info_t
 *   hdt, fx, fy, fz   the velocity shift hdt*F of the macro output
 *   out    device array of 12 + 9*nx + 1 doubles: the 12 diag values, the
 *          nx x 9 profile values, then the number of cells with a non-finite
 *          moment (dg_stats_values returns DG_ERR_NUMERIC for such a state;
 *          here the caller reads the count)
 * Only FP64 data is valid input: the pointer carries no type, and the state of
 * an fp32 or 16-bit engine gives meaningless numbers.
 * Asynchronous on `stream` (a cudaStream_t; 0 = legacy default stream).
 * The first call on a device looks up the scratch array's device address with
 * that device current; make that first call before any stream capture.  All
 * calls share the one scratch array and each overwrites it completely: calls
 * whose kernels can overlap on the GPU race on it and must be ordered by the
 * caller.  nx beyond the maximum returns DG_ERR_SHAPE; the message of the
 * last failure is dg_noalloc_last_error(). */
int dg_stats_values_noalloc(const double *f, int nx, int ny, int nz, int pitch, long long pop_stride,
                            double hdt, double fx, double fy, double fz, double *out, void *stream);
/* Message of the last failing dg_stats_values_noalloc call made by the
 * calling host thread (the message buffer is per thread). */
const char *dg_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
