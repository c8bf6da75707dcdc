/*
 * Oracle interface: a CPU restatement of the reference DUGKS step
 * (Kairzhan/DUGKS-GPU src/dugks.cu and src/fortran/channel/src/dugks.cuf).
 *
 * TEST INFRASTRUCTURE ONLY -- used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py as the checker; never part of the product.
 */
#ifndef DUGKS_ORACLE_H
#define DUGKS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;      /* interior cells (single rank: lx=nx, ...) */
    int periodic_x;      /* periods_x; 0 = bounce-back walls on the x faces */
    int mesh;            /* 0 uniform (CUDA-C formulas), 1 stretched x (Fortran channel formulas) */
    int recon;           /* 0 trilinear (calc_fx_tri), 1 central-difference gradient (calc_fx) */
    int face_force;      /* 0 ambient force on every face (f2ruvwh), 1 Fortran channel (y faces only) */
    int perturb;         /* calc_perturb_force in stage (a) */
    double dx, dy, dz, dt;
    double visc;
    double xwidth, ywidth, zwidth;
    double Fx, Fy, Fz;   /* ambient force */
    const double *xc;    /* nx+2 cell centres incl. mirrored ghosts (mesh==1) */
    const double *dxx;   /* nx+2 cell widths incl. ghosts (mesh==1) */
} oracle_cfg;

int oracle_coefficients_f64(const oracle_cfg *c, double *out13);
int oracle_init_f64(const oracle_cfg *c, int kind, double *f);
int oracle_init_case_f64(const oracle_cfg *c, int kind, const double *par, double *f);
int oracle_fbar_f64(const oracle_cfg *c, const double *f, double *fb, int step, int nthreads);
int oracle_run_f64(const oracle_cfg *c, double *f, int istep0, int nsteps, int nthreads);
int oracle_macro_f64(const oracle_cfg *c, const double *f, double *rho, double *ux, double *uy, double *uz);
int oracle_stats_f64(int nx, int ny, int nz, const double *rhg, const double *uxg, const double *uyg,
                     const double *uzg, double *diag, double *prof);

int oracle_coefficients_f32(const oracle_cfg *c, double *out13);
int oracle_init_f32(const oracle_cfg *c, int kind, float *f);
int oracle_init_case_f32(const oracle_cfg *c, int kind, const double *par, float *f);
int oracle_fbar_f32(const oracle_cfg *c, const float *f, float *fb, int step, int nthreads);
int oracle_run_f32(const oracle_cfg *c, float *f, int istep0, int nsteps, int nthreads);
int oracle_macro_f32(const oracle_cfg *c, const float *f, float *rho, float *ux, float *uy, float *uz);
int oracle_stats_f32(int nx, int ny, int nz, const float *rhg, const float *uxg, const float *uyg,
                     const float *uzg, double *diag, double *prof);

int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
