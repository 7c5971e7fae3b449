// problem.cpp -- seeded synthetic FDTD problems (host code, plain C++).
//
// The reference builds one problem: a vacuum cavity Lx=.05, Ly=.04, Lz=.03 with random initial
// fields and Courant number about 0.01 (ptaskUnitTest/graphfdtd.cpp:1357-1381, inputs from
// configure_raw_array :106-126).  The benchmark workloads extend it with axis-aligned dielectric
// boxes, Courant 0.5 and a Gaussian soft source.  Everything here is a pure function of the seed
// (splitmix64 stream), so the same arrays come out on x86-64 and aarch64.
//
// Must be compiled with -ffp-contract=off: Cb = Dt/(eps0*eps_r) is formed with separately rounded
// FP32 operations so that a vacuum cell gets exactly the reference's fl(Dt/eps0).  The device-side
// generator (k_generate_coefs in fdtd_batch.cu) evaluates the same expression from the same boxes.
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "ptk_problem.h"

#include <exception>
#include <new>

// No C++ exception unwinds into a C caller of the entry point below.
#define PTK_PROBLEM_CATCH_ALL                              \
    catch (const std::bad_alloc &) { return PTK_ERR_NOMEM; } \
    catch (...) { return PTK_ERR_STATE; }

namespace {

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // Uniform integer in [a, b].
    int range(int a, int b)
    {
        if (b <= a) return a;
        int v = a + (int)(u01() * (double)(b - a + 1));
        return v > b ? b : v;
    }
};

const float kLx = 0.05f, kLy = 0.04f, kLz = 0.03f;   // cavity size, graphfdtd.cpp:1357

void base_params(int Nx, int Ny, int Nz, ptk_fdtd_params *p)
{
    const float pi = 3.1415f;                          // graphfdtd.cpp:1359
    p->Nx = Nx;
    p->Ny = Ny;
    p->Nz = Nz;
    p->Cx = (float)Nx / kLx;
    p->Cy = (float)Ny / kLy;
    p->Cz = (float)Nz / kLz;
    p->eps0 = 8.8541878e-12f;
    p->mu0 = 4e-7f * pi;
    p->c0 = 299792458.0f;
}

}  // namespace

namespace ptk {

int problem_plan(const ptk_problem_desc *d, ptk_fdtd_params *p, std::vector<BoxSpec> *boxes, int *si, int *sj,
                 int *sk, std::vector<float> *wave)
{
    if (!d || !p || d->Nx < 1 || d->Ny < 1 || d->Nz < 1 || d->steps < 0 || d->n_boxes < 0) return PTK_ERR_INVALID;
    const int Nx = d->Nx, Ny = d->Ny, Nz = d->Nz;
    base_params(Nx, Ny, Nz, p);
    const double cx = p->Cx, cy = p->Cy, cz = p->Cz;
    p->Dt = (float)((double)d->courant / ((double)p->c0 * std::sqrt(cx * cx + cy * cy + cz * cz)));

    Rng r{d->seed};
    if (boxes) boxes->clear();
    for (int b = 0; b < d->n_boxes; ++b) {
        const int N[3] = {Nx, Ny, Nz};
        BoxSpec bx;
        for (int a = 0; a < 3; ++a) {
            int size = r.range(d->box_min, d->box_max);
            if (size < 1) size = 1;
            if (size > N[a]) size = N[a];
            bx.lo[a] = r.range(0, N[a] - size);
            bx.hi[a] = bx.lo[a] + size;
        }
        bx.epsr = (float)(d->eps_min + (double)(d->eps_max - d->eps_min) * r.u01());
        if (boxes) boxes->push_back(bx);
    }
    int i = -1, j = -1, k = -1;
    if (d->source_mode != 0 && Nx >= 2 && Ny >= 2) {
        if (d->source_mode == 1) {
            i = Nx / 2; j = Ny / 2; k = Nz / 2;
        } else {
            i = r.range(1, Nx - 1);
            j = r.range(1, Ny - 1);
            k = r.range(0, Nz - 1);
        }
    }
    if (si) *si = i;
    if (sj) *sj = j;
    if (sk) *sk = k;
    if (wave) {
        // Gaussian pulse exp(-((n - t0)/tw)^2), tw in steps, t0 = 3 tw.
        wave->assign((size_t)d->steps, 0.0f);
        double tw = d->steps / 8.0;
        if (tw > 20.0) tw = 20.0;
        if (tw < 2.0) tw = 2.0;
        const double t0 = 3.0 * tw;
        for (int n = 0; n < d->steps; ++n) {
            const double a = ((double)n - t0) / tw;
            (*wave)[(size_t)n] = (i >= 0) ? (float)std::exp(-a * a) : 0.0f;
        }
    }
    return PTK_OK;
}

}  // namespace ptk

extern "C" {

int ptk_reference_params(int Nx, int Ny, int Nz, ptk_fdtd_params *p)
{
    if (!p || Nx < 1 || Ny < 1 || Nz < 1) return PTK_ERR_INVALID;
    base_params(Nx, Ny, Nz, p);
    const float nrm = std::sqrt((Nx / kLx * Nx / kLx) + (Ny / kLy * Ny / kLy) + (Nz / kLz * Nz / kLz)) * 100;
    p->Dt = 1.0f / (p->c0 * nrm);
    return PTK_OK;
}

int ptk_fill_uniform(float *dst, size_t n, float scale, uint64_t seed)
{
    if (!dst && n) return PTK_ERR_INVALID;
    Rng r{seed};
    for (size_t q = 0; q < n; ++q) dst[q] = (float)(r.u01() * (double)scale);
    return PTK_OK;
}

int ptk_problem_generate(const ptk_problem_desc *d, ptk_fdtd_params *p, float *Ca, float *Cb, float *Da,
                         float *Db, int *si, int *sj, int *sk, float *wave)
try {
    std::vector<ptk::BoxSpec> boxes;
    std::vector<float> w;
    int rc = ptk::problem_plan(d, p, &boxes, si, sj, sk, &w);
    if (rc) return rc;
    const int Nx = d->Nx, Ny = d->Ny, Nz = d->Nz;
    const size_t ncell = (size_t)Nx * Ny * Nz;
    std::vector<float> epsr(ncell, 1.0f);
    for (const ptk::BoxSpec &b : boxes)   // later boxes overwrite earlier ones
        for (int k = b.lo[2]; k < b.hi[2]; ++k)
            for (int j = b.lo[1]; j < b.hi[1]; ++j)
                for (int i = b.lo[0]; i < b.hi[0]; ++i) epsr[(size_t)i + (size_t)Nx * j + (size_t)Nx * Ny * k] = b.epsr;
    const float ch = p->Dt / p->mu0;
    for (size_t c = 0; c < ncell; ++c) {
        if (Ca) Ca[c] = 1.0f;
        if (Cb) Cb[c] = p->Dt / (p->eps0 * epsr[c]);
        if (Da) Da[c] = 1.0f;
        if (Db) Db[c] = ch;
    }
    if (wave)
        for (size_t n = 0; n < w.size(); ++n) wave[n] = w[n];
    return PTK_OK;
} PTK_PROBLEM_CATCH_ALL

}  // extern "C"
