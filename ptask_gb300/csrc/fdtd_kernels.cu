// fdtd_kernels.cu -- sm_103a kernels for the Yee-grid FDTD task graph.
//
// The update equations are those of the reference's six field tasks
// (ptaskUnitTest/graphfdtd.cpp:185-312, HLSL twins ptaskUnitTest/fdtdKernels/{Hx..Ez}Comp.hlsl),
// generalised to per-cell coefficients:
//   H' = Da*H + Db*curl(E)            (reference: Da = 1, Db = Dt/mu0)
//   E' = Ca*E + Cb*curl(H')           (reference: Ca = 1, Cb = Dt/eps0), PEC faces copied through.
// Every floating-point operation is issued with an explicit round-to-nearest intrinsic so that no
// multiply-add is contracted; with Ca = Da = 1 the results are bit-identical to the reference's
// FP32 host code.
//
// Kernels here:
//   k_yee_step<BY>   fused H+E step over a work list of tiles of one or many instances (padded
//                    layout); the hot kernel.  Bandwidth bound: 64 algorithmic bytes per cell.
//   k_field_ref      the reference's per-field task kernels (dense layout), one field per launch.
//   k_h_half/k_e_half  the three H (or E) tasks of one step fused in one launch (dense layout).
//   k_pack_* / k_unpack_field   reference layout <-> padded layout.
#include "ptk_internal.h"

#include <cstdio>

namespace ptk {

#define FULL_MASK 0xffffffffu

// d*h + c*((a1-a0)*s1 - (b1-b0)*s2), each operation rounded separately.
__device__ __forceinline__ float yee(float d, float h, float c, float a1, float a0, float s1,
                                     float b1, float b0, float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(__fmul_rn(d, h), __fmul_rn(c, curl));
}

// h + c*((a1-a0)*s1 - (b1-b0)*s2): the reference's scalar form (graphfdtd.cpp:198 and siblings).
__device__ __forceinline__ float yee_ref(float h, float c, float a1, float a0, float s1, float b1,
                                         float b0, float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(h, __fmul_rn(c, curl));
}

struct F4 {
    float v[4];
};

__device__ __forceinline__ F4 ld4(const float *__restrict__ p)
{
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    F4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
}

__device__ __forceinline__ F4 zero4()
{
    F4 r;
    r.v[0] = r.v[1] = r.v[2] = r.v[3] = 0.f;
    return r;
}

// Store the first `n` (1..4) elements of v at p; a full aligned vector store when n == 4.
__device__ __forceinline__ void st4(float *p, const F4 &v, int n)
{
    if (n >= 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (e < n) p[e] = v.v[e];
    }
}

__device__ __forceinline__ float4 as_f4(const F4 &v) { return make_float4(v.v[0], v.v[1], v.v[2], v.v[3]); }
__device__ __forceinline__ F4 from_f4(const float4 &t)
{
    F4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
}

// ---------------------------------------------------------------------------------------------
// Face work of one instance: the H nodes outside the cell block [0,Nx)x[0,Ny)x[0,Nz), i.e. Hx on
// i=Nx, Hy on j=Ny and Hz on k=Nz.  They depend only on E nodes of the PEC walls (which never
// change) and on themselves, so they can be updated by any CTA of the same launch.
// ---------------------------------------------------------------------------------------------
__device__ void yee_faces(const InstDesc *__restrict__ D, int par, int ftile, int cells_per_tile)
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

// ---------------------------------------------------------------------------------------------
// Fused Yee step.  One CTA owns a main tile of 128 (x) by BY (y) cells and a range of z planes
// [k0, k1); it streams the planes in order, keeping the previous plane's new Hx, Hy and the next
// plane's Ex, Ey in registers (sliding window), so every array element is read from HBM once per
// step.  Thread (lane, ty): ty = 1..BY own row y0+ty-1, 4 consecutive x cells per lane (128-bit
// loads and stores); ty = 0 is a halo row y0-1 that only recomputes new Hx, Hz for the E update of
// row y0.  In-plane neighbours: x+1 / x-1 through warp shuffles (lane 31 / lane 0 fetch the one
// cell beyond the tile), y+1 / y-1 through shared memory.  A tile that starts at k0 > 0 first
// recomputes new Hx, Hy on plane k0-1 ("warm" plane, no stores).
// Work list: blockIdx.x indexes the concatenated tiles of all instances (tile0 = prefix sums);
// each instance's main tiles are followed by its face tiles.
// ---------------------------------------------------------------------------------------------
template <int BY>
__global__ void __launch_bounds__(32 * (BY + 1), BY <= 4 ? 4 : (BY <= 8 ? 2 : 1))
k_yee_step(const InstDesc *__restrict__ insts, const int *__restrict__ tile0, int ninst, int s_off,
           int total_tiles)
{
    __shared__ float4 sEx[BY + 1][32];
    __shared__ float4 sEz[BY + 1][32];
    __shared__ float4 sHx[BY + 1][32];
    __shared__ float4 sHz[BY + 1][32];

    // Persistent form: a CTA takes tiles blockIdx.x, blockIdx.x + gridDim.x, ...  Shared memory is
    // safe to reuse across tiles: every plane ends with a barrier after the last read of sEx/sEz,
    // and sHx/sHz are first written after the next tile's first barrier.
    for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
    int lo = 0, hi = ninst;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(tile0 + mid) <= t) lo = mid; else hi = mid;
    }
    const InstDesc *__restrict__ D = insts + lo;
    if (s_off >= D->steps_left) continue;
    const int lt = t - __ldg(tile0 + lo);
    const int step = D->step + s_off;
    const int par = step & 1;
    const int nmain = D->tiles_x * D->tiles_y * D->tiles_z;
    if (lt >= nmain) {
        yee_faces(D, par, lt - nmain, 32 * (BY + 1) * kFaceCellsPerThread);
        continue;
    }

    const int nx = D->nx, ny = D->ny, nz = D->nz, pitch = D->pitch, kc = D->kc;
    const long long plane = D->plane;
    const float cx = D->cx, cy = D->cy, cz = D->cz;
    const float *__restrict__ Hx = D->buf[par][0];
    const float *__restrict__ Hy = D->buf[par][1];
    const float *__restrict__ Hz = D->buf[par][2];
    const float *__restrict__ Ex = D->buf[par][3];
    const float *__restrict__ Ey = D->buf[par][4];
    const float *__restrict__ Ez = D->buf[par][5];
    float *__restrict__ oHx = D->buf[par ^ 1][0];
    float *__restrict__ oHy = D->buf[par ^ 1][1];
    float *__restrict__ oHz = D->buf[par ^ 1][2];
    float *__restrict__ oEx = D->buf[par ^ 1][3];
    float *__restrict__ oEy = D->buf[par ^ 1][4];
    float *__restrict__ oEz = D->buf[par ^ 1][5];
    const float *__restrict__ Ca = D->coef[0];
    const float *__restrict__ Cb = D->coef[1];
    const float *__restrict__ Da = D->coef[2];
    const float *__restrict__ Db = D->coef[3];
    const long long src = D->src;
    const float srcv = (src >= 0 && step < D->nwave) ? __ldg(D->wave + step) : 0.f;

    int r = lt;
    const int xt = r % D->tiles_x; r /= D->tiles_x;
    const int yt = r % D->tiles_y;
    const int zt = r / D->tiles_y;
    const int x0 = xt * kTileX, y0 = yt * BY;
    const int k0 = zt * kc, k1 = min(k0 + kc, nz);
    const int kstart = k0 > 0 ? k0 - 1 : k0;

    const int lane = threadIdx.x, ty = threadIdx.y;
    const int i = x0 + 4 * lane;
    const int j = y0 + ty - 1;
    const bool halo = (ty == 0);
    const bool xin = (i <= nx);               // vector holds at least one node of the row
    const bool jrow = (j >= 0 && j < ny);     // a row of cells (or a valid halo row)
    const bool jshare = (!halo && j == ny);   // the wall row: only lends Ex, Ez to row Ny-1
    const int nout = min(4, nx - i);          // cells of this vector inside [0, Nx)
    const bool xl = (lane == 31) && (x0 + kTileX <= nx);   // one node beyond the tile exists
    const bool hcol = (!halo) && (lane == 0) && (x0 > 0) && jrow;   // lane 0 recomputes x0-1

    // Offsets are formed only for rows that exist (j >= 0).
    long long off = (long long)i + (long long)pitch * (j < 0 ? 0 : j) + plane * kstart;

    F4 ex0 = zero4(), ey0 = zero4();   // Ex(k), Ey(k)
    F4 hxp = zero4(), hyp = zero4();   // new Hx, Hy on plane k-1
    if (!halo && xin) {
        if (jrow || jshare) ex0 = ld4(Ex + off);
        if (jrow) ey0 = ld4(Ey + off);
    }

    for (int k = kstart; k < k1; ++k, off += plane) {
        const bool warm = (k < k0);
        F4 hx = zero4(), hy = zero4(), hz = zero4(), ez = zero4(), ex1 = zero4(), ey1 = zero4();
        F4 da = zero4(), db = zero4(), ca = zero4(), cb = zero4();
        F4 exj1 = zero4(), ezj1 = zero4();
        float ez_l = 0.f, ey_l = 0.f;                                  // lane 31: x0+128
        float hy_h = 0.f, hz_h = 0.f, ez_h = 0.f, ex_h0 = 0.f, ex_h1 = 0.f, ex_hj = 0.f,
              ey_h = 0.f, da_h = 0.f, db_h = 0.f;                        // lane 0: x0-1

        // ---- loads ----------------------------------------------------------------------
        if (halo) {
            if (!warm && jrow && xin) {
                hx = ld4(Hx + off); hz = ld4(Hz + off); ez = ld4(Ez + off);
                ex0 = ld4(Ex + off); ey0 = ld4(Ey + off); ey1 = ld4(Ey + off + plane);
                da = ld4(Da + off); db = ld4(Db + off);
                if (xl) ey_l = __ldg(Ey + off + 4);
            }
        } else if (jrow && xin) {
            hx = ld4(Hx + off); hy = ld4(Hy + off); ez = ld4(Ez + off);
            ex1 = ld4(Ex + off + plane); ey1 = ld4(Ey + off + plane);
            da = ld4(Da + off); db = ld4(Db + off);
            if (!warm) { hz = ld4(Hz + off); ca = ld4(Ca + off); cb = ld4(Cb + off); }
            if (ty == BY) { exj1 = ld4(Ex + off + pitch); ezj1 = ld4(Ez + off + pitch); }
            if (xl) { ez_l = __ldg(Ez + off + 4); ey_l = __ldg(Ey + off + 4); }
            if (hcol && !warm) {
                const long long oh = off - 1;
                hy_h = __ldg(Hy + oh); hz_h = __ldg(Hz + oh); ez_h = __ldg(Ez + oh);
                ex_h0 = __ldg(Ex + oh); ex_h1 = __ldg(Ex + oh + plane); ex_hj = __ldg(Ex + oh + pitch);
                ey_h = __ldg(Ey + oh); da_h = __ldg(Da + oh); db_h = __ldg(Db + oh);
            }
        } else if (jshare && xin) {
            ex0 = ld4(Ex + off); ez = ld4(Ez + off);
        }

        // ---- share Ex, Ez of each row with the row above (its y+1 neighbour) -----------------
        sEx[ty][lane] = as_f4(ex0);
        sEz[ty][lane] = as_f4(ez);
        __syncthreads();
        if (ty < BY) {
            exj1 = from_f4(sEx[ty + 1][lane]);
            ezj1 = from_f4(sEz[ty + 1][lane]);
        }

        // ---- x+1 neighbours through shuffles ----------------------------------------------
        float ez_n = __shfl_down_sync(FULL_MASK, ez.v[0], 1);
        float ey_n = __shfl_down_sync(FULL_MASK, ey0.v[0], 1);
        if (lane == 31) { ez_n = ez_l; ey_n = ey_l; }

        // ---- new H on plane k ---------------------------------------------------------------
        F4 hxn, hyn, hzn;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float ez_ip = e < 3 ? ez.v[e + 1] : ez_n;
            const float ey_ip = e < 3 ? ey0.v[e + 1] : ey_n;
            hxn.v[e] = yee(da.v[e], hx.v[e], db.v[e], ey1.v[e], ey0.v[e], cz, ezj1.v[e], ez.v[e], cy);
            hyn.v[e] = yee(da.v[e], hy.v[e], db.v[e], ez_ip, ez.v[e], cx, ex1.v[e], ex0.v[e], cz);
            hzn.v[e] = yee(da.v[e], hz.v[e], db.v[e], exj1.v[e], ex0.v[e], cy, ey_ip, ey0.v[e], cx);
        }
        // halo column x0-1 (lane 0 of the cell rows): new Hy, Hz
        float hyh = 0.f, hzh = 0.f;
        if (hcol && !warm) {
            hyh = yee(da_h, hy_h, db_h, ez.v[0], ez_h, cx, ex_h1, ex_h0, cz);
            hzh = yee(da_h, hz_h, db_h, ex_hj, ex_h0, cy, ey0.v[0], ey_h, cx);
        }

        if (!warm) {
            sHx[ty][lane] = as_f4(hxn);
            sHz[ty][lane] = as_f4(hzn);
        }
        __syncthreads();

        // ---- x-1 neighbours of new Hy, Hz ---------------------------------------------------
        float hy_p = __shfl_up_sync(FULL_MASK, hyn.v[3], 1);
        float hz_p = __shfl_up_sync(FULL_MASK, hzn.v[3], 1);
        if (lane == 0) { hy_p = hyh; hz_p = hzh; }

        if (!halo && jrow && xin) {
            if (!warm) {
                const F4 hxj = from_f4(sHx[ty - 1][lane]);   // new Hx at j-1
                const F4 hzj = from_f4(sHz[ty - 1][lane]);   // new Hz at j-1
                F4 exn, eyn, ezn;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int x = i + e;
                    const float hy_im = e > 0 ? hyn.v[e - 1] : hy_p;
                    const float hz_im = e > 0 ? hzn.v[e - 1] : hz_p;
                    exn.v[e] = (j >= 1 && k >= 1)
                        ? yee(ca.v[e], ex0.v[e], cb.v[e], hzn.v[e], hzj.v[e], cy, hyn.v[e], hyp.v[e], cz)
                        : ex0.v[e];
                    eyn.v[e] = (x >= 1 && k >= 1)
                        ? yee(ca.v[e], ey0.v[e], cb.v[e], hxn.v[e], hxp.v[e], cz, hzn.v[e], hz_im, cx)
                        : ey0.v[e];
                    ezn.v[e] = (x >= 1 && j >= 1)
                        ? yee(ca.v[e], ez.v[e], cb.v[e], hyn.v[e], hy_im, cx, hxn.v[e], hxj.v[e], cy)
                        : ez.v[e];
                }
                if (src >= 0) {
                    const long long dsrc = src - off;
                    if (dsrc >= 0 && dsrc < 4) {
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (e == (int)dsrc) ezn.v[e] = __fadd_rn(ezn.v[e], srcv);
                    }
                }
                if (nout > 0) {
                    st4(oHx + off, hxn, nout); st4(oHy + off, hyn, nout); st4(oHz + off, hzn, nout);
                    st4(oEx + off, exn, nout); st4(oEy + off, eyn, nout); st4(oEz + off, ezn, nout);
                }
            }
            hxp = hxn;
            hyp = hyn;
            ex0 = ex1;
            ey0 = ey1;
        }
    }
    }   // tile loop
}

__global__ void k_advance(InstDesc *insts, int ninst, int nsteps)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ninst) return;
    InstDesc &d = insts[q];
    const int n = min(nsteps, d.steps_left);
    if (n > 0) {
        d.step += n;
        d.steps_left -= n;
    }
}

int face_tile_cells(int by) { return 32 * (by + 1) * kFaceCellsPerThread; }

void plan_tiles(InstDesc &d, int by, int kc)
{
    const int kcc = (kc <= 0 || kc > d.nz) ? d.nz : kc;
    d.kc = kcc;
    d.tiles_x = (d.nx + kTileX - 1) / kTileX;
    d.tiles_y = (d.ny + by - 1) / by;
    d.tiles_z = (d.nz + kcc - 1) / kcc;
    const long long fc = (long long)d.ny * d.nz + (long long)d.nx * d.nz + (long long)d.nx * d.ny;
    const int per = face_tile_cells(by);
    d.face_tiles = (int)((fc + per - 1) / per);
}

int launch_yee_step_grid(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles,
                         int s_offset, int by, int grid, cudaStream_t s)
{
    if (total_tiles <= 0) return PTK_OK;
    const int g = (grid <= 0 || grid > total_tiles) ? total_tiles : grid;
    switch (by) {
    case 4: k_yee_step<4><<<g, dim3(32, 5), 0, s>>>(d_insts, d_tile0, ninst, s_offset, total_tiles); break;
    case 8: k_yee_step<8><<<g, dim3(32, 9), 0, s>>>(d_insts, d_tile0, ninst, s_offset, total_tiles); break;
    case 16: k_yee_step<16><<<g, dim3(32, 17), 0, s>>>(d_insts, d_tile0, ninst, s_offset, total_tiles); break;
    default: return set_error(PTK_ERR_INVALID, "tile rows must be 4, 8 or 16 (got %d)", by);
    }
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int launch_yee_step(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles,
                    int s_offset, int by, cudaStream_t s)
{
    return launch_yee_step_grid(d_insts, d_tile0, ninst, total_tiles, s_offset, by, 0, s);
}

int yee_resident_ctas(int by)
{
    int per_sm = 0;
    cudaError_t e = cudaSuccess;
    switch (by) {
    case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_yee_step<4>, 32 * 5, 0); break;
    case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_yee_step<8>, 32 * 9, 0); break;
    case 16: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_yee_step<16>, 32 * 17, 0); break;
    default: return 0;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * sm_count();
}

int launch_advance(InstDesc *d_insts, int ninst, int nsteps, cudaStream_t s)
{
    if (ninst <= 0) return PTK_OK;
    k_advance<<<(ninst + 127) / 128, 128, 0, s>>>(d_insts, ninst, nsteps);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

// ---------------------------------------------------------------------------------------------
// Layout conversion.
// ---------------------------------------------------------------------------------------------
__global__ void k_pack_field(const float *__restrict__ src, int ex, int ey, int ez, int pitch,
                             long long plane, float *__restrict__ d0, float *__restrict__ d1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= ex) return;
    const float v = src[i + (long long)ex * j + (long long)ex * ey * k];
    const long long o = i + (long long)pitch * j + plane * k;
    d0[o] = v;
    if (d1) d1[o] = v;
}

__global__ void k_unpack_field(const float *__restrict__ src, int ex, int ey, int ez, int pitch,
                               long long plane, float *__restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= ex) return;
    dst[i + (long long)ex * j + (long long)ex * ey * k] = src[i + (long long)pitch * j + plane * k];
}

// Per-cell (Nx,Ny,Nz) array to padded nodes (Nx+1,Ny+1,Nz+1); wall nodes take the nearest cell.
__global__ void k_pack_coef(const float *__restrict__ src, int nx, int ny, int nz, int pitch,
                            long long plane, float *__restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i > nx) return;
    const int ci = min(i, nx - 1), cj = min(j, ny - 1), ck = min(k, nz - 1);
    dst[i + (long long)pitch * j + plane * k] = src[ci + (long long)nx * cj + (long long)nx * ny * ck];
}

__global__ void k_fill(float *__restrict__ dst, long long n, float v)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x)
        dst[q] = v;
}

int launch_pack_field(const float *src, int ex, int ey, int ez, const Layout &L, float *dst0,
                      float *dst1, cudaStream_t s)
{
    dim3 grid((ex + 127) / 128, ey, ez);
    k_pack_field<<<grid, 128, 0, s>>>(src, ex, ey, ez, L.pitch, L.plane, dst0, dst1);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int launch_unpack_field(const float *src, int ex, int ey, int ez, const Layout &L, float *dst,
                        cudaStream_t s)
{
    dim3 grid((ex + 127) / 128, ey, ez);
    k_unpack_field<<<grid, 128, 0, s>>>(src, ex, ey, ez, L.pitch, L.plane, dst);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int launch_pack_coef(const float *src, const Layout &L, float *dst, cudaStream_t s)
{
    dim3 grid((L.nx + 1 + 127) / 128, L.ny + 1, L.nz + 1);
    k_pack_coef<<<grid, 128, 0, s>>>(src, L.nx, L.ny, L.nz, L.pitch, L.plane, dst);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int launch_fill(float *dst, long long n, float v, cudaStream_t s)
{
    if (n <= 0) return PTK_OK;
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_fill<<<(int)blocks, 256, 0, s>>>(dst, n, v);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

// ---------------------------------------------------------------------------------------------
// The reference's six task kernels over dense arrays, one output field per launch.  Thread (i,j,k)
// of the output extents computes exactly the expression of fdtd_<F>Computation_cpu.
// ---------------------------------------------------------------------------------------------
__global__ void k_field_ref(int field, const float *__restrict__ a, const float *__restrict__ b,
                            const float *__restrict__ c, ptk_fdtd_params p, float *__restrict__ out)
{
    const int Nx = p.Nx, Ny = p.Ny, Nz = p.Nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const float ch = __fdiv_rn(p.Dt, p.mu0);
    const float ce = __fdiv_rn(p.Dt, p.eps0);
#define D3(ii, jj, kk, d1, d2) ((long long)(ii) + (long long)(d1) * (jj) + (long long)(d1) * (d2) * (kk))
    switch (field) {
    case PTK_HX: {   // a=Hx(Nx+1,Ny,Nz) b=Ey(Nx+1,Ny,Nz+1) c=Ez(Nx+1,Ny+1,Nz)
        if (i > Nx) return;
        const long long o = D3(i, j, k, Nx + 1, Ny);
        out[o] = yee_ref(a[o], ch, b[D3(i, j, k + 1, Nx + 1, Ny)], b[D3(i, j, k, Nx + 1, Ny)], p.Cz,
                         c[D3(i, j + 1, k, Nx + 1, Ny + 1)], c[D3(i, j, k, Nx + 1, Ny + 1)], p.Cy);
        break;
    }
    case PTK_HY: {   // a=Hy(Nx,Ny+1,Nz) b=Ex(Nx,Ny+1,Nz+1) c=Ez(Nx+1,Ny+1,Nz)
        if (i >= Nx) return;
        const long long o = D3(i, j, k, Nx, Ny + 1);
        out[o] = yee_ref(a[o], ch, c[D3(i + 1, j, k, Nx + 1, Ny + 1)], c[D3(i, j, k, Nx + 1, Ny + 1)], p.Cx,
                         b[D3(i, j, k + 1, Nx, Ny + 1)], b[D3(i, j, k, Nx, Ny + 1)], p.Cz);
        break;
    }
    case PTK_HZ: {   // a=Hz(Nx,Ny,Nz+1) b=Ex(Nx,Ny+1,Nz+1) c=Ey(Nx+1,Ny,Nz+1)
        if (i >= Nx) return;
        const long long o = D3(i, j, k, Nx, Ny);
        out[o] = yee_ref(a[o], ch, b[D3(i, j + 1, k, Nx, Ny + 1)], b[D3(i, j, k, Nx, Ny + 1)], p.Cy,
                         c[D3(i + 1, j, k, Nx + 1, Ny)], c[D3(i, j, k, Nx + 1, Ny)], p.Cx);
        break;
    }
    case PTK_EX: {   // a=Ex(Nx,Ny+1,Nz+1) b=Hy(Nx,Ny+1,Nz) c=Hz(Nx,Ny,Nz+1)
        if (i >= Nx) return;
        const long long o = D3(i, j, k, Nx, Ny + 1);
        if (j < 1 || k < 1 || j > Ny - 1 || k > Nz - 1) { out[o] = a[o]; return; }
        out[o] = yee_ref(a[o], ce, c[D3(i, j, k, Nx, Ny)], c[D3(i, j - 1, k, Nx, Ny)], p.Cy,
                         b[D3(i, j, k, Nx, Ny + 1)], b[D3(i, j, k - 1, Nx, Ny + 1)], p.Cz);
        break;
    }
    case PTK_EY: {   // a=Ey(Nx+1,Ny,Nz+1) b=Hx(Nx+1,Ny,Nz) c=Hz(Nx,Ny,Nz+1)
        if (i > Nx) return;
        const long long o = D3(i, j, k, Nx + 1, Ny);
        if (i < 1 || k < 1 || i > Nx - 1 || k > Nz - 1) { out[o] = a[o]; return; }
        out[o] = yee_ref(a[o], ce, b[D3(i, j, k, Nx + 1, Ny)], b[D3(i, j, k - 1, Nx + 1, Ny)], p.Cz,
                         c[D3(i, j, k, Nx, Ny)], c[D3(i - 1, j, k, Nx, Ny)], p.Cx);
        break;
    }
    default: {       // PTK_EZ: a=Ez(Nx+1,Ny+1,Nz) b=Hx(Nx+1,Ny,Nz) c=Hy(Nx,Ny+1,Nz)
        if (i > Nx) return;
        const long long o = D3(i, j, k, Nx + 1, Ny + 1);
        if (i < 1 || j < 1 || i > Nx - 1 || j > Ny - 1) { out[o] = a[o]; return; }
        out[o] = yee_ref(a[o], ce, c[D3(i, j, k, Nx, Ny + 1)], c[D3(i - 1, j, k, Nx, Ny + 1)], p.Cx,
                         b[D3(i, j, k, Nx + 1, Ny)], b[D3(i, j - 1, k, Nx + 1, Ny)], p.Cy);
        break;
    }
    }
}

void field_extents(int f, int nx, int ny, int nz, int *ex, int *ey, int *ez)
{
    *ex = nx + ((f == PTK_HX || f == PTK_EY || f == PTK_EZ) ? 1 : 0);
    *ey = ny + ((f == PTK_HY || f == PTK_EX || f == PTK_EZ) ? 1 : 0);
    *ez = nz + ((f == PTK_HZ || f == PTK_EX || f == PTK_EY) ? 1 : 0);
}

int launch_field_ref(int field, const float *in0, const float *in1, const float *in2,
                     const ptk_fdtd_params &p, float *out, cudaStream_t s)
{
    int ex, ey, ez;
    field_extents(field, p.Nx, p.Ny, p.Nz, &ex, &ey, &ez);
    dim3 grid((ex + 127) / 128, ey, ez);
    k_field_ref<<<grid, 128, 0, s>>>(field, in0, in1, in2, p, out);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

// Three H (or E) tasks of one step in one launch over the node box (Nx+1,Ny+1,Nz+1).
__global__ void k_h_half(const float *__restrict__ Hx, const float *__restrict__ Hy,
                         const float *__restrict__ Hz, const float *__restrict__ Ex,
                         const float *__restrict__ Ey, const float *__restrict__ Ez,
                         ptk_fdtd_params p, float *__restrict__ oHx, float *__restrict__ oHy,
                         float *__restrict__ oHz)
{
    const int Nx = p.Nx, Ny = p.Ny, Nz = p.Nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const float ch = __fdiv_rn(p.Dt, p.mu0);
    if (i <= Nx && j < Ny && k < Nz) {
        const long long o = D3(i, j, k, Nx + 1, Ny);
        oHx[o] = yee_ref(Hx[o], ch, Ey[D3(i, j, k + 1, Nx + 1, Ny)], Ey[D3(i, j, k, Nx + 1, Ny)], p.Cz,
                         Ez[D3(i, j + 1, k, Nx + 1, Ny + 1)], Ez[D3(i, j, k, Nx + 1, Ny + 1)], p.Cy);
    }
    if (i < Nx && j <= Ny && k < Nz) {
        const long long o = D3(i, j, k, Nx, Ny + 1);
        oHy[o] = yee_ref(Hy[o], ch, Ez[D3(i + 1, j, k, Nx + 1, Ny + 1)], Ez[D3(i, j, k, Nx + 1, Ny + 1)], p.Cx,
                         Ex[D3(i, j, k + 1, Nx, Ny + 1)], Ex[D3(i, j, k, Nx, Ny + 1)], p.Cz);
    }
    if (i < Nx && j < Ny && k <= Nz) {
        const long long o = D3(i, j, k, Nx, Ny);
        oHz[o] = yee_ref(Hz[o], ch, Ex[D3(i, j + 1, k, Nx, Ny + 1)], Ex[D3(i, j, k, Nx, Ny + 1)], p.Cy,
                         Ey[D3(i + 1, j, k, Nx + 1, Ny)], Ey[D3(i, j, k, Nx + 1, Ny)], p.Cx);
    }
}

__global__ void k_e_half(const float *__restrict__ Ex, const float *__restrict__ Ey,
                         const float *__restrict__ Ez, const float *__restrict__ Hx,
                         const float *__restrict__ Hy, const float *__restrict__ Hz,
                         ptk_fdtd_params p, float *__restrict__ oEx, float *__restrict__ oEy,
                         float *__restrict__ oEz)
{
    const int Nx = p.Nx, Ny = p.Ny, Nz = p.Nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    const float ce = __fdiv_rn(p.Dt, p.eps0);
    if (i < Nx && j <= Ny && k <= Nz) {
        const long long o = D3(i, j, k, Nx, Ny + 1);
        oEx[o] = (j < 1 || k < 1 || j > Ny - 1 || k > Nz - 1)
            ? Ex[o]
            : yee_ref(Ex[o], ce, Hz[D3(i, j, k, Nx, Ny)], Hz[D3(i, j - 1, k, Nx, Ny)], p.Cy,
                      Hy[D3(i, j, k, Nx, Ny + 1)], Hy[D3(i, j, k - 1, Nx, Ny + 1)], p.Cz);
    }
    if (i <= Nx && j < Ny && k <= Nz) {
        const long long o = D3(i, j, k, Nx + 1, Ny);
        oEy[o] = (i < 1 || k < 1 || i > Nx - 1 || k > Nz - 1)
            ? Ey[o]
            : yee_ref(Ey[o], ce, Hx[D3(i, j, k, Nx + 1, Ny)], Hx[D3(i, j, k - 1, Nx + 1, Ny)], p.Cz,
                      Hz[D3(i, j, k, Nx, Ny)], Hz[D3(i - 1, j, k, Nx, Ny)], p.Cx);
    }
    if (i <= Nx && j <= Ny && k < Nz) {
        const long long o = D3(i, j, k, Nx + 1, Ny + 1);
        oEz[o] = (i < 1 || j < 1 || i > Nx - 1 || j > Ny - 1)
            ? Ez[o]
            : yee_ref(Ez[o], ce, Hy[D3(i, j, k, Nx, Ny + 1)], Hy[D3(i - 1, j, k, Nx, Ny + 1)], p.Cx,
                      Hx[D3(i, j, k, Nx + 1, Ny)], Hx[D3(i, j - 1, k, Nx + 1, Ny)], p.Cy);
    }
}
#undef D3

int launch_h_half(const float *const in[6], float *const out[3], const ptk_fdtd_params &p,
                  cudaStream_t s)
{
    dim3 grid((p.Nx + 1 + 127) / 128, p.Ny + 1, p.Nz + 1);
    k_h_half<<<grid, 128, 0, s>>>(in[0], in[1], in[2], in[3], in[4], in[5], p, out[0], out[1], out[2]);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int launch_e_half(const float *const e_in[3], const float *const h_new[3], float *const out[3],
                  const ptk_fdtd_params &p, cudaStream_t s)
{
    dim3 grid((p.Nx + 1 + 127) / 128, p.Ny + 1, p.Nz + 1);
    k_e_half<<<grid, 128, 0, s>>>(e_in[0], e_in[1], e_in[2], h_new[0], h_new[1], h_new[2], p,
                                  out[0], out[1], out[2]);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

}  // namespace ptk
