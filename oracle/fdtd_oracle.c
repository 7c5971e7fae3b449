/*
 * fdtd_oracle.c -- CPU oracle for the Yee-grid FDTD step of ptaskUnitTest/graphfdtd.cpp.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference leg may load it.
 * The shipped library (ptask_gb300) never links or calls anything here.
 *
 * What it restates (reference file:line, paths inside rossbach/ptask):
 *   oracle_ref_f32      fdtd_cpu                    ptaskUnitTest/graphfdtd.cpp:314-340
 *                       with the six field updates  graphfdtd.cpp:185-312
 *                       (Hx 185-201, Hy 204-221, Hz 223-240, Ex 243-264, Ey 267-288, Ez 291-312)
 *                       Scalar vacuum coefficients Dt/mu0 and Dt/eps0, FP32, same operation order,
 *                       out-of-place update (the reference news a fresh array per update; here two
 *                       buffers per field are swapped, which computes identical values).
 *   oracle_ext_f32      the same scheme with per-cell coefficients (Ca, Cb for E, Da, Db for H) and
 *                       a soft Ez point source added after the E update.  Not in the reference; it
 *                       reduces bit-for-bit to oracle_ref_f32 when Ca=Da=1, Cb=fl(Dt/eps0),
 *                       Db=fl(Dt/mu0) and the source is off (pinned by tests).
 *   oracle_ext_f64      FP64 twin of oracle_ext_f32 (inputs widened once), for the "error vs FP64"
 *                       figure.
 *   oracle_field_task_f32  one per-field task (graphfdtd.cpp:185-312), out of place, for the test
 *                       host-task library.
 *   oracle_problem_generate  the benchmark's seeded problem generator (vacuum cavity with the
 *                       reference's constants, graphfdtd.cpp:1357-1381, plus dielectric boxes, a
 *                       Courant-number time step and a Gaussian source), restated independently of
 *                       the product library so that the CPU baseline needs nothing from it.  Tests
 *                       pin it bit for bit to ptk_problem_generate.
 *
 * Layouts are the reference's (Simple3DArray.h:33): element (i,j,k) of an array with extents
 * (d1,d2,d3) sits at i + j*d1 + k*d1*d2; the six fields have extents
 *   Hx(Nx+1,Ny,Nz) Hy(Nx,Ny+1,Nz) Hz(Nx,Ny,Nz+1) Ex(Nx,Ny+1,Nz+1) Ey(Nx+1,Ny,Nz+1) Ez(Nx+1,Ny+1,Nz)
 * (graphfdtd.cpp:68-86).  Coefficient arrays are per cell, extents (Nx,Ny,Nz); a field node outside
 * the cell range (the i=Nx, j=Ny, k=Nz faces) uses the nearest cell (index clamped).
 *
 * Must be compiled with -ffp-contract=off so that no multiply-add is fused: every operation is
 * rounded separately, as in the reference built for x86-64 SSE.  Loops over k are split across
 * OpenMP threads when built with -fopenmp; each output element is computed independently, so the
 * result is bit-identical for any thread count.
 */
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

typedef struct oracle_params {   /* same layout as FDTD_PARAMS, graphfdtd.h:6-19 */
    int Nx, Ny, Nz;
    float Cx, Cy, Cz, eps0, mu0, c0, Dt;
} oracle_params;

#define IDX(i, j, k, d1, d2) ((size_t)(i) + (size_t)(j) * (size_t)(d1) + (size_t)(k) * (size_t)(d1) * (size_t)(d2))

static size_t field_count(int f, int Nx, int Ny, int Nz)
{
    switch (f) {
    case 0: return (size_t)(Nx + 1) * Ny * Nz;          /* Hx */
    case 1: return (size_t)Nx * (Ny + 1) * Nz;          /* Hy */
    case 2: return (size_t)Nx * Ny * (Nz + 1);          /* Hz */
    case 3: return (size_t)Nx * (Ny + 1) * (Nz + 1);    /* Ex */
    case 4: return (size_t)(Nx + 1) * Ny * (Nz + 1);    /* Ey */
    default: return (size_t)(Nx + 1) * (Ny + 1) * Nz;   /* Ez */
    }
}

size_t oracle_field_count(int f, int Nx, int Ny, int Nz) { return field_count(f, Nx, Ny, Nz); }

static inline int clampi(int v, int hi) { return v < hi ? v : hi - 1; }

/* ------------------------------------------------------------------------------------------ */
/* FP32 / FP64 generic body.  T is the arithmetic type; scalar coefficients are expressed as   */
/* uniform arrays by the caller when coef == NULL (reference mode).                             */
/* ------------------------------------------------------------------------------------------ */

#define DEFINE_STEPPER(NAME, T)                                                                     \
static void NAME(T *Hx, T *Hy, T *Hz, T *Ex, T *Ey, T *Ez,                                          \
                 T *nHx, T *nHy, T *nHz, T *nEx, T *nEy, T *nEz,                                    \
                 const T *Ca, const T *Cb, const T *Da, const T *Db,                                \
                 T ca_s, T cb_s, T da_s, T db_s,                                                    \
                 int Nx, int Ny, int Nz, T Cx, T Cy, T Cz,                                          \
                 long src, T srcval)                                                                \
{                                                                                                   \
    /* ---- H half step: graphfdtd.cpp:185-240 (reads old E) ---- */                                \
    int i, j, k;                                                                                    \
    _Pragma("omp parallel for private(i, j) schedule(static)")                                      \
    for (k = 0; k < Nz; ++k)                                                                        \
        for (j = 0; j < Ny; ++j)                                                                    \
            for (i = 0; i <= Nx; ++i) {                                                             \
                size_t c = IDX(clampi(i, Nx), j, k, Nx, Ny);                                        \
                T da = Da ? Da[c] : da_s, db = Db ? Db[c] : db_s;                                   \
                T curl = (Ey[IDX(i, j, k + 1, Nx + 1, Ny)] - Ey[IDX(i, j, k, Nx + 1, Ny)]) * Cz     \
                       - (Ez[IDX(i, j + 1, k, Nx + 1, Ny + 1)] - Ez[IDX(i, j, k, Nx + 1, Ny + 1)]) * Cy; \
                size_t o = IDX(i, j, k, Nx + 1, Ny);                                                \
                nHx[o] = da * Hx[o] + db * curl;                                                    \
            }                                                                                       \
    _Pragma("omp parallel for private(i, j) schedule(static)")                                      \
    for (k = 0; k < Nz; ++k)                                                                        \
        for (j = 0; j <= Ny; ++j)                                                                   \
            for (i = 0; i < Nx; ++i) {                                                              \
                size_t c = IDX(i, clampi(j, Ny), k, Nx, Ny);                                        \
                T da = Da ? Da[c] : da_s, db = Db ? Db[c] : db_s;                                   \
                T curl = (Ez[IDX(i + 1, j, k, Nx + 1, Ny + 1)] - Ez[IDX(i, j, k, Nx + 1, Ny + 1)]) * Cx \
                       - (Ex[IDX(i, j, k + 1, Nx, Ny + 1)] - Ex[IDX(i, j, k, Nx, Ny + 1)]) * Cz;    \
                size_t o = IDX(i, j, k, Nx, Ny + 1);                                                \
                nHy[o] = da * Hy[o] + db * curl;                                                    \
            }                                                                                       \
    _Pragma("omp parallel for private(i, j) schedule(static)")                                      \
    for (k = 0; k <= Nz; ++k)                                                                       \
        for (j = 0; j < Ny; ++j)                                                                    \
            for (i = 0; i < Nx; ++i) {                                                              \
                size_t c = IDX(i, j, clampi(k, Nz), Nx, Ny);                                        \
                T da = Da ? Da[c] : da_s, db = Db ? Db[c] : db_s;                                   \
                T curl = (Ex[IDX(i, j + 1, k, Nx, Ny + 1)] - Ex[IDX(i, j, k, Nx, Ny + 1)]) * Cy     \
                       - (Ey[IDX(i + 1, j, k, Nx + 1, Ny)] - Ey[IDX(i, j, k, Nx + 1, Ny)]) * Cx;    \
                size_t o = IDX(i, j, k, Nx, Ny);                                                    \
                nHz[o] = da * Hz[o] + db * curl;                                                    \
            }                                                                                       \
    /* ---- E half step: graphfdtd.cpp:243-312 (reads new H); faces copied ---- */                 \
    _Pragma("omp parallel for private(i, j) schedule(static)")                                      \
    for (k = 0; k <= Nz; ++k)                                                                       \
        for (j = 0; j <= Ny; ++j)                                                                   \
            for (i = 0; i < Nx; ++i) {                                                              \
                size_t o = IDX(i, j, k, Nx, Ny + 1);                                                \
                if (j < 1 || k < 1 || j > Ny - 1 || k > Nz - 1) { nEx[o] = Ex[o]; continue; }      \
                size_t c = IDX(i, j, k, Nx, Ny);                                                    \
                T ca = Ca ? Ca[c] : ca_s, cb = Cb ? Cb[c] : cb_s;                                   \
                T curl = (nHz[IDX(i, j, k, Nx, Ny)] - nHz[IDX(i, j - 1, k, Nx, Ny)]) * Cy           \
                       - (nHy[IDX(i, j, k, Nx, Ny + 1)] - nHy[IDX(i, j, k - 1, Nx, Ny + 1)]) * Cz;  \
                nEx[o] = ca * Ex[o] + cb * curl;                                                    \
            }                                                                                       \
    _Pragma("omp parallel for private(i, j) schedule(static)")                                      \
    for (k = 0; k <= Nz; ++k)                                                                       \
        for (j = 0; j < Ny; ++j)                                                                    \
            for (i = 0; i <= Nx; ++i) {                                                             \
                size_t o = IDX(i, j, k, Nx + 1, Ny);                                                \
                if (i < 1 || k < 1 || i > Nx - 1 || k > Nz - 1) { nEy[o] = Ey[o]; continue; }      \
                size_t c = IDX(i, j, k, Nx, Ny);                                                    \
                T ca = Ca ? Ca[c] : ca_s, cb = Cb ? Cb[c] : cb_s;                                   \
                T curl = (nHx[IDX(i, j, k, Nx + 1, Ny)] - nHx[IDX(i, j, k - 1, Nx + 1, Ny)]) * Cz   \
                       - (nHz[IDX(i, j, k, Nx, Ny)] - nHz[IDX(i - 1, j, k, Nx, Ny)]) * Cx;          \
                nEy[o] = ca * Ey[o] + cb * curl;                                                    \
            }                                                                                       \
    _Pragma("omp parallel for private(i, j) schedule(static)")                                      \
    for (k = 0; k < Nz; ++k)                                                                        \
        for (j = 0; j <= Ny; ++j)                                                                   \
            for (i = 0; i <= Nx; ++i) {                                                             \
                size_t o = IDX(i, j, k, Nx + 1, Ny + 1);                                            \
                if (i < 1 || j < 1 || i > Nx - 1 || j > Ny - 1) { nEz[o] = Ez[o]; continue; }      \
                size_t c = IDX(i, j, k, Nx, Ny);                                                    \
                T ca = Ca ? Ca[c] : ca_s, cb = Cb ? Cb[c] : cb_s;                                   \
                T curl = (nHy[IDX(i, j, k, Nx, Ny + 1)] - nHy[IDX(i - 1, j, k, Nx, Ny + 1)]) * Cx   \
                       - (nHx[IDX(i, j, k, Nx + 1, Ny)] - nHx[IDX(i, j - 1, k, Nx + 1, Ny)]) * Cy;  \
                nEz[o] = ca * Ez[o] + cb * curl;                                                    \
            }                                                                                       \
    if (src >= 0) nEz[src] = nEz[src] + srcval;                                                     \
}

DEFINE_STEPPER(step_f32, float)
DEFINE_STEPPER(step_f64, double)

/* Swap the caller's six arrays through scratch copies for T steps.  The arrays are updated in
 * place: on return they hold the fields after T steps. */
#define DEFINE_DRIVER(NAME, T, STEP)                                                                \
static int NAME(T *f[6], const T *Ca, const T *Cb, const T *Da, const T *Db,                        \
                T ca_s, T cb_s, T da_s, T db_s, int Nx, int Ny, int Nz, T Cx, T Cy, T Cz,           \
                int steps, int si, int sj, int sk, const float *wave, int nwave)                    \
{                                                                                                   \
    T *g[6];                                                                                        \
    int q, n;                                                                                       \
    long src = -1;                                                                                  \
    if (Nx < 1 || Ny < 1 || Nz < 1 || steps < 0) return 1;                                          \
    if (wave && si >= 0) src = (long)IDX(si, sj, sk, Nx + 1, Ny + 1);                               \
    for (q = 0; q < 6; ++q) {                                                                       \
        g[q] = (T *)malloc(field_count(q, Nx, Ny, Nz) * sizeof(T));                                 \
        if (!g[q]) { while (q--) free(g[q]); return 2; }                                            \
    }                                                                                               \
    for (n = 0; n < steps; ++n) {                                                                   \
        T sv = (src >= 0 && n < nwave) ? (T)wave[n] : (T)0;                                         \
        STEP(f[0], f[1], f[2], f[3], f[4], f[5], g[0], g[1], g[2], g[3], g[4], g[5],                \
             Ca, Cb, Da, Db, ca_s, cb_s, da_s, db_s, Nx, Ny, Nz, Cx, Cy, Cz,                        \
             (src >= 0 && n < nwave) ? src : -1, sv);                                               \
        for (q = 0; q < 6; ++q) { T *t = f[q]; f[q] = g[q]; g[q] = t; }                             \
    }                                                                                               \
    /* after an odd number of swaps the results live in the scratch arrays: copy back */            \
    if (steps & 1)                                                                                  \
        for (q = 0; q < 6; ++q) {                                                                   \
            memcpy(g[q], f[q], field_count(q, Nx, Ny, Nz) * sizeof(T));                             \
            T *t = f[q]; f[q] = g[q]; g[q] = t;                                                     \
        }                                                                                           \
    for (q = 0; q < 6; ++q) free(g[q]);                                                             \
    return 0;                                                                                       \
}

DEFINE_DRIVER(drive_f32, float, step_f32)
DEFINE_DRIVER(drive_f64, double, step_f64)

/* Reference mode: fdtd_cpu (graphfdtd.cpp:314-340) on the six arrays in place. */
int oracle_ref_f32(float *Hx, float *Hy, float *Hz, float *Ex, float *Ey, float *Ez,
                   int steps, const oracle_params *p)
{
    float *f[6] = {Hx, Hy, Hz, Ex, Ey, Ez};
    float ch = p->Dt / p->mu0;     /* (params.Dt/params.mu0), graphfdtd.cpp:198 */
    float ce = p->Dt / p->eps0;    /* (params.Dt/params.eps0), graphfdtd.cpp:260 */
    return drive_f32(f, NULL, NULL, NULL, NULL, 1.0f, ce, 1.0f, ch, p->Nx, p->Ny, p->Nz,
                     p->Cx, p->Cy, p->Cz, steps, -1, 0, 0, NULL, 0);
}

/* Extended mode, FP32: per-cell coefficients and an optional soft Ez source at (si,sj,sk)
 * (si < 0 disables it); wave[n] is added to Ez after the E update of step n. */
int oracle_ext_f32(float *Hx, float *Hy, float *Hz, float *Ex, float *Ey, float *Ez,
                   const float *Ca, const float *Cb, const float *Da, const float *Db,
                   int steps, const oracle_params *p, int si, int sj, int sk,
                   const float *wave, int nwave)
{
    float *f[6] = {Hx, Hy, Hz, Ex, Ey, Ez};
    return drive_f32(f, Ca, Cb, Da, Db, 0, 0, 0, 0, p->Nx, p->Ny, p->Nz, p->Cx, p->Cy, p->Cz,
                     steps, si, sj, sk, wave, nwave);
}

/* Extended mode, FP64: FP32 inputs are widened once; results are written to the double arrays
 * out[0..5] (which need not be initialised). */
int oracle_ext_f64(const float *const in[6], double *const out[6],
                   const float *Ca, const float *Cb, const float *Da, const float *Db,
                   int steps, const oracle_params *p, int si, int sj, int sk,
                   const float *wave, int nwave)
{
    int Nx = p->Nx, Ny = p->Ny, Nz = p->Nz, q, rc;
    size_t ncell = (size_t)Nx * Ny * Nz, n;
    double *f[6], *c[4] = {0, 0, 0, 0};
    const float *cs[4] = {Ca, Cb, Da, Db};
    for (q = 0; q < 6; ++q) {
        size_t m = field_count(q, Nx, Ny, Nz);
        f[q] = out[q];
        for (n = 0; n < m; ++n) f[q][n] = (double)in[q][n];
    }
    for (q = 0; q < 4; ++q) {
        c[q] = (double *)malloc(ncell * sizeof(double));
        if (!c[q]) { while (q--) free(c[q]); return 2; }
        for (n = 0; n < ncell; ++n) c[q][n] = (double)cs[q][n];
    }
    rc = drive_f64(f, c[0], c[1], c[2], c[3], 0, 0, 0, 0, Nx, Ny, Nz, (double)p->Cx,
                   (double)p->Cy, (double)p->Cz, steps, si, sj, sk, wave, nwave);
    for (q = 0; q < 4; ++q) free(c[q]);
    return rc;
}

/* One per-field task of the reference graph, out-of-place: field f (0..5 = Hx..Ez) with the inputs
 * of its task in the reference's port order (graphfdtd.cpp:458-597):
 *   Hx: (Hx, Ey, Ez)  Hy: (Hy, Ex, Ez)  Hz: (Hz, Ex, Ey)  Ex: (Ex, Hy, Hz)  Ey: (Ey, Hx, Hz)  Ez: (Ez, Hx, Hy)
 * Restates fdtd_Hx..EzComputation_cpu (graphfdtd.cpp:185-312) with the scalar vacuum coefficients,
 * the same expressions as step_f32 above (H: 1*H + (Dt/mu0)*curl, E: 1*E + (Dt/eps0)*curl, E faces
 * copied).  Used by the test host-task library to run the reference graph on the host. */
int oracle_field_task_f32(int f, const float *a, const float *b, const float *c, const oracle_params *p,
                          float *out)
{
    const int Nx = p->Nx, Ny = p->Ny, Nz = p->Nz;
    const float Cx = p->Cx, Cy = p->Cy, Cz = p->Cz;
    const float ch = p->Dt / p->mu0, ce = p->Dt / p->eps0, one = 1.0f;
    int i, j, k;
    if (Nx < 1 || Ny < 1 || Nz < 1 || f < 0 || f > 5) return 1;
    switch (f) {
    case 0:   /* Hx from Ey, Ez */
        for (k = 0; k < Nz; ++k) for (j = 0; j < Ny; ++j) for (i = 0; i <= Nx; ++i) {
            float curl = (b[IDX(i, j, k + 1, Nx + 1, Ny)] - b[IDX(i, j, k, Nx + 1, Ny)]) * Cz
                       - (c[IDX(i, j + 1, k, Nx + 1, Ny + 1)] - c[IDX(i, j, k, Nx + 1, Ny + 1)]) * Cy;
            size_t o = IDX(i, j, k, Nx + 1, Ny);
            out[o] = one * a[o] + ch * curl;
        }
        break;
    case 1:   /* Hy from Ex, Ez */
        for (k = 0; k < Nz; ++k) for (j = 0; j <= Ny; ++j) for (i = 0; i < Nx; ++i) {
            float curl = (c[IDX(i + 1, j, k, Nx + 1, Ny + 1)] - c[IDX(i, j, k, Nx + 1, Ny + 1)]) * Cx
                       - (b[IDX(i, j, k + 1, Nx, Ny + 1)] - b[IDX(i, j, k, Nx, Ny + 1)]) * Cz;
            size_t o = IDX(i, j, k, Nx, Ny + 1);
            out[o] = one * a[o] + ch * curl;
        }
        break;
    case 2:   /* Hz from Ex, Ey */
        for (k = 0; k <= Nz; ++k) for (j = 0; j < Ny; ++j) for (i = 0; i < Nx; ++i) {
            float curl = (b[IDX(i, j + 1, k, Nx, Ny + 1)] - b[IDX(i, j, k, Nx, Ny + 1)]) * Cy
                       - (c[IDX(i + 1, j, k, Nx + 1, Ny)] - c[IDX(i, j, k, Nx + 1, Ny)]) * Cx;
            size_t o = IDX(i, j, k, Nx, Ny);
            out[o] = one * a[o] + ch * curl;
        }
        break;
    case 3:   /* Ex from Hy, Hz */
        for (k = 0; k <= Nz; ++k) for (j = 0; j <= Ny; ++j) for (i = 0; i < Nx; ++i) {
            size_t o = IDX(i, j, k, Nx, Ny + 1);
            if (j < 1 || k < 1 || j > Ny - 1 || k > Nz - 1) { out[o] = a[o]; continue; }
            float curl = (c[IDX(i, j, k, Nx, Ny)] - c[IDX(i, j - 1, k, Nx, Ny)]) * Cy
                       - (b[IDX(i, j, k, Nx, Ny + 1)] - b[IDX(i, j, k - 1, Nx, Ny + 1)]) * Cz;
            out[o] = one * a[o] + ce * curl;
        }
        break;
    case 4:   /* Ey from Hx, Hz */
        for (k = 0; k <= Nz; ++k) for (j = 0; j < Ny; ++j) for (i = 0; i <= Nx; ++i) {
            size_t o = IDX(i, j, k, Nx + 1, Ny);
            if (i < 1 || k < 1 || i > Nx - 1 || k > Nz - 1) { out[o] = a[o]; continue; }
            float curl = (b[IDX(i, j, k, Nx + 1, Ny)] - b[IDX(i, j, k - 1, Nx + 1, Ny)]) * Cz
                       - (c[IDX(i, j, k, Nx, Ny)] - c[IDX(i - 1, j, k, Nx, Ny)]) * Cx;
            out[o] = one * a[o] + ce * curl;
        }
        break;
    default:  /* Ez from Hx, Hy */
        for (k = 0; k < Nz; ++k) for (j = 0; j <= Ny; ++j) for (i = 0; i <= Nx; ++i) {
            size_t o = IDX(i, j, k, Nx + 1, Ny + 1);
            if (i < 1 || j < 1 || i > Nx - 1 || j > Ny - 1) { out[o] = a[o]; continue; }
            float curl = (c[IDX(i, j, k, Nx, Ny + 1)] - c[IDX(i - 1, j, k, Nx, Ny + 1)]) * Cx
                       - (b[IDX(i, j, k, Nx + 1, Ny)] - b[IDX(i, j - 1, k, Nx + 1, Ny)]) * Cy;
            out[o] = one * a[o] + ce * curl;
        }
        break;
    }
    return 0;
}

/* Threads the OpenMP runtime will use (1 when built without OpenMP). */
int oracle_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------------------ */
/* Seeded problem generator.  Same description and the same numbers as ptk_problem_generate:   */
/* a splitmix64 stream draws the boxes (edges, positions, eps_r) and the source position; the  */
/* vacuum constants are the reference's cavity (graphfdtd.cpp:1357-1361).  Every expression is */
/* evaluated in the type and order the description below gives, so the arrays are bit-equal.   */
/* ------------------------------------------------------------------------------------------ */
#include <math.h>

typedef struct oracle_problem_desc {   /* same layout as ptk_problem_desc */
    int Nx, Ny, Nz;
    int n_boxes;
    float eps_min, eps_max;
    int box_min, box_max;
    float courant;
    int steps;
    int source_mode;    /* 0 none, 1 centre, 2 seeded interior node */
    uint64_t seed;
} oracle_problem_desc;

static uint64_t sm64_next(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* uniform double in [0, 1) from the top 53 bits */
static double sm64_u01(uint64_t *s) { return (double)(sm64_next(s) >> 11) * (1.0 / 9007199254740992.0); }

/* uniform integer in [a, b] */
static int sm64_range(uint64_t *s, int a, int b)
{
    int v;
    if (b <= a) return a;
    v = a + (int)(sm64_u01(s) * (double)(b - a + 1));
    return v > b ? b : v;
}

int oracle_problem_generate(const oracle_problem_desc *d, oracle_params *p, float *Ca, float *Cb, float *Da,
                            float *Db, int *si, int *sj, int *sk, float *wave)
{
    const float Lx = 0.05f, Ly = 0.04f, Lz = 0.03f, pi = 3.1415f;
    uint64_t s;
    int b, a, n, Nx, Ny, Nz, i = -1, j = -1, k = -1;
    size_t c, ncell;
    float *epsr;
    double cx, cy, cz;
    if (!d || !p || d->Nx < 1 || d->Ny < 1 || d->Nz < 1 || d->steps < 0 || d->n_boxes < 0) return 1;
    Nx = d->Nx; Ny = d->Ny; Nz = d->Nz;
    p->Nx = Nx; p->Ny = Ny; p->Nz = Nz;
    p->Cx = (float)Nx / Lx;
    p->Cy = (float)Ny / Ly;
    p->Cz = (float)Nz / Lz;
    p->eps0 = 8.8541878e-12f;
    p->mu0 = 4e-7f * pi;
    p->c0 = 299792458.0f;
    cx = p->Cx; cy = p->Cy; cz = p->Cz;
    p->Dt = (float)((double)d->courant / ((double)p->c0 * sqrt(cx * cx + cy * cy + cz * cz)));

    ncell = (size_t)Nx * Ny * Nz;
    epsr = (float *)malloc(ncell * sizeof(float));
    if (!epsr) return 2;
    for (c = 0; c < ncell; ++c) epsr[c] = 1.0f;
    s = d->seed;
    for (b = 0; b < d->n_boxes; ++b) {   /* later boxes overwrite earlier ones */
        const int N[3] = {Nx, Ny, Nz};
        int lo[3], hi[3], x, y, z;
        float e;
        for (a = 0; a < 3; ++a) {
            int size = sm64_range(&s, d->box_min, d->box_max);
            if (size < 1) size = 1;
            if (size > N[a]) size = N[a];
            lo[a] = sm64_range(&s, 0, N[a] - size);
            hi[a] = lo[a] + size;
        }
        e = (float)(d->eps_min + (double)(d->eps_max - d->eps_min) * sm64_u01(&s));
        for (z = lo[2]; z < hi[2]; ++z)
            for (y = lo[1]; y < hi[1]; ++y)
                for (x = lo[0]; x < hi[0]; ++x) epsr[IDX(x, y, z, Nx, Ny)] = e;
    }
    if (d->source_mode != 0 && Nx >= 2 && Ny >= 2) {
        if (d->source_mode == 1) {
            i = Nx / 2; j = Ny / 2; k = Nz / 2;
        } else {
            i = sm64_range(&s, 1, Nx - 1);
            j = sm64_range(&s, 1, Ny - 1);
            k = sm64_range(&s, 0, Nz - 1);
        }
    }
    if (si) *si = i;
    if (sj) *sj = j;
    if (sk) *sk = k;
    {
        const float ch = p->Dt / p->mu0;
        for (c = 0; c < ncell; ++c) {
            if (Ca) Ca[c] = 1.0f;
            if (Cb) Cb[c] = p->Dt / (p->eps0 * epsr[c]);
            if (Da) Da[c] = 1.0f;
            if (Db) Db[c] = ch;
        }
    }
    free(epsr);
    if (wave) {   /* Gaussian pulse exp(-((n - t0)/tw)^2), tw = steps/8 clamped to [2, 20], t0 = 3 tw */
        double tw = d->steps / 8.0, t0;
        if (tw > 20.0) tw = 20.0;
        if (tw < 2.0) tw = 2.0;
        t0 = 3.0 * tw;
        for (n = 0; n < d->steps; ++n) {
            const double x = ((double)n - t0) / tw;
            wave[n] = (i >= 0) ? (float)exp(-x * x) : 0.0f;
        }
    }
    return 0;
}
