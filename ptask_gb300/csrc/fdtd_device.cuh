// fdtd_device.cuh -- device helpers shared by the fused-step kernels (fdtd_kernels.cu, fdtd_step_bulk.cu).
#pragma once

#include "ptk_internal.h"

namespace ptk {

// d*h + c*((a1-a0)*s1 - (b1-b0)*s2), each operation rounded separately.
static __device__ __forceinline__ float yee(float d, float h, float c, float a1, float a0, float s1,
                                     float b1, float b0, float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(__fmul_rn(d, h), __fmul_rn(c, curl));
}

// ---------------------------------------------------------------------------------------------
// Face work of one instance: the H nodes outside the cell block [0,Nx)x[0,Ny)x[0,Nz), i.e. Hx on
// i=Nx, Hy on j=Ny and Hz on k=Nz.  They depend only on E nodes of the PEC walls (which never
// change) and on themselves, so they can be updated by any CTA of the same launch.
// ---------------------------------------------------------------------------------------------
static __device__ void yee_faces(const InstDesc *__restrict__ D, int par, int ftile, int cells_per_tile)
{
    const int nx = D->nx, ny = D->ny, nz = D->nz, pitch = D->pitch;
    const long long plane = D->plane;
    const float *__restrict__ Hx = D->buf[par][0];
    const float *__restrict__ Hy = D->buf[par][1];
    const float *__restrict__ Hz = D->buf[par][2];
    const float *__restrict__ Ex = D->buf[par][3];
    const float *__restrict__ Ey = D->buf[par][4];
    const float *__restrict__ Ez = D->buf[par][5];
    float *__restrict__ oHx = D->buf[par ^ 1][0];
    float *__restrict__ oHy = D->buf[par ^ 1][1];
    float *__restrict__ oHz = D->buf[par ^ 1][2];
    const float *__restrict__ Da = D->coef[2];
    const float *__restrict__ Db = D->coef[3];
    const float cx = D->cx, cy = D->cy, cz = D->cz;
    const long long A = (long long)ny * nz, B = (long long)nx * nz, C = (long long)nx * ny;
    const long long q0 = (long long)ftile * cells_per_tile;
    const long long q1 = min(q0 + cells_per_tile, A + B + C);
    const int nthr = blockDim.x * blockDim.y;
    for (long long q = q0 + threadIdx.y * blockDim.x + threadIdx.x; q < q1; q += nthr) {
        if (q < A) {                       // Hx at i = Nx
            const int j = (int)(q % ny), k = (int)(q / ny);
            const long long o = nx + (long long)pitch * j + plane * k;
            oHx[o] = yee(__ldg(Da + o), __ldg(Hx + o), __ldg(Db + o), __ldg(Ey + o + plane),
                         __ldg(Ey + o), cz, __ldg(Ez + o + pitch), __ldg(Ez + o), cy);
        } else if (q < A + B) {            // Hy at j = Ny
            const long long r = q - A;
            const int i = (int)(r % nx), k = (int)(r / nx);
            const long long o = i + (long long)pitch * ny + plane * k;
            oHy[o] = yee(__ldg(Da + o), __ldg(Hy + o), __ldg(Db + o), __ldg(Ez + o + 1), __ldg(Ez + o),
                         cx, __ldg(Ex + o + plane), __ldg(Ex + o), cz);
        } else {                           // Hz at k = Nz
            const long long r = q - A - B;
            const int i = (int)(r % nx), j = (int)(r / nx);
            const long long o = i + (long long)pitch * j + plane * nz;
            oHz[o] = yee(__ldg(Da + o), __ldg(Hz + o), __ldg(Db + o), __ldg(Ex + o + pitch),
                         __ldg(Ex + o), cy, __ldg(Ey + o + 1), __ldg(Ey + o), cx);
        }
    }
}

}  // namespace ptk
