// ref_shim.cpp -- C entry points over the reference's own CPU FDTD functions (test infrastructure).
// Links against the reference's fdtd_cpu / fdtd_cpu_multiple_inputs (graphfdtd.cpp:314-391),
// compiled unmodified by oracle/Makefile.  Used only by tests/ and bench.py's reference arm.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include "Simple3DArray.h"
#include "graphfdtd.h"

typedef CSimple3DArray<float> A3;
void fdtd_cpu(A3 *&Hx, A3 *&Hy, A3 *&Hz, A3 *&Ex, A3 *&Ey, A3 *&Ez, int numIterations, FDTD_PARAMS params);
void fdtd_cpu_multiple_inputs(A3 *&Hx, A3 *&Hy, A3 *&Hz, A3 *&Ex, A3 *&Ey, A3 *&Ez, int numIterations,
                              int numBlocks, FDTD_PARAMS params);

static void extents(int f, int Nx, int Ny, int Nz, int e[3])
{
    e[0] = Nx + ((f == 0 || f == 4 || f == 5) ? 1 : 0);
    e[1] = Ny + ((f == 1 || f == 3 || f == 5) ? 1 : 0);
    e[2] = Nz + ((f == 2 || f == 3 || f == 4) ? 1 : 0);
}

static int run(float *f[6], int steps, int blocks, const FDTD_PARAMS *p)
{
    A3 *a[6];
    for (int q = 0; q < 6; ++q) {
        int e[3];
        extents(q, p->Nx, p->Ny, p->Nz, e);
        a[q] = new A3(e[0], e[1], e[2]);
        memcpy(a[q]->cells(), f[q], sizeof(float) * a[q]->arraysize());
    }
    if (blocks <= 0)
        fdtd_cpu(a[0], a[1], a[2], a[3], a[4], a[5], steps, *p);
    else
        fdtd_cpu_multiple_inputs(a[0], a[1], a[2], a[3], a[4], a[5], steps, blocks, *p);
    for (int q = 0; q < 6; ++q) {
        memcpy(f[q], a[q]->cells(), sizeof(float) * a[q]->arraysize());
        delete a[q];
    }
    return 0;
}

extern "C" int ref_fdtd_cpu(float *Hx, float *Hy, float *Hz, float *Ex, float *Ey, float *Ez, int steps,
                            const FDTD_PARAMS *p)
{
    float *f[6] = {Hx, Hy, Hz, Ex, Ey, Ez};
    return run(f, steps, 0, p);
}

extern "C" int ref_fdtd_cpu_multiple_inputs(float *Hx, float *Hy, float *Hz, float *Ex, float *Ey,
                                            float *Ez, int steps, int blocks, const FDTD_PARAMS *p)
{
    float *f[6] = {Hx, Hy, Hz, Ex, Ey, Ez};
    return run(f, steps, blocks, p);
}

#ifdef REF_MAIN
// ref_fdtd_main Nx Ny Nz steps : time fdtd_cpu on zero fields with the reference's constants.
int main(int argc, char **argv)
{
    if (argc < 5) { fprintf(stderr, "usage: %s Nx Ny Nz steps\n", argv[0]); return 2; }
    int Nx = atoi(argv[1]), Ny = atoi(argv[2]), Nz = atoi(argv[3]), T = atoi(argv[4]);
    FDTD_PARAMS p;
    float Lx = 0.05f, Ly = 0.04f, Lz = 0.03f;
    p.Nx = Nx; p.Ny = Ny; p.Nz = Nz; p.Cx = Nx / Lx; p.Cy = Ny / Ly; p.Cz = Nz / Lz;
    p.eps0 = 8.8541878e-12f; p.mu0 = 4e-7f * 3.1415f; p.c0 = 299792458.0f; p.Dt = 1e-13f;
    float *f[6];
    for (int q = 0; q < 6; ++q) {
        int e[3];
        extents(q, Nx, Ny, Nz, e);
        f[q] = (float *)calloc((size_t)e[0] * e[1] * e[2], sizeof(float));
    }
    auto t0 = std::chrono::steady_clock::now();
    run(f, T, 0, &p);
    double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("%.6f\n", s);
    return 0;
}
#endif
