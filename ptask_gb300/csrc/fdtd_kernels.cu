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
#include "fdtd_device.cuh"

#include <cstdio>

namespace ptk {

#define FULL_MASK 0xffffffffu

// h + c*((a1-a0)*s1 - (b1-b0)*s2): the reference's scalar form (graphfdtd.cpp:198 and siblings).
__device__ __forceinline__ float yee_ref(float h, float c, float a1, float a0, float s1, float b1,
                                         float b0, float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(h, __fmul_rn(c, curl));
}

// V consecutive x cells held by one thread (V = 1, 2, 4: 32-, 64- or 128-bit accesses).
template <int V>
struct __align__(4 * V) Vec {
    float v[V];
};

template <int V>
__device__ __forceinline__ Vec<V> ldv(const float *__restrict__ p)
{
    Vec<V> r;
    if constexpr (V == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else if constexpr (V == 2) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        r.v[0] = t.x; r.v[1] = t.y;
    } else {
        r.v[0] = __ldg(p);
    }
    return r;
}

template <int V>
__device__ __forceinline__ Vec<V> zerov()
{
    Vec<V> r;
#pragma unroll
    for (int e = 0; e < V; ++e) r.v[e] = 0.f;
    return r;
}

// Store the first `n` (1..V) elements of v at p; one aligned vector store when n == V.
template <int V>
__device__ __forceinline__ void stv(float *p, const Vec<V> &v, int n)
{
    if (n >= V) {
        if constexpr (V == 4) *reinterpret_cast<float4 *>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
        else if constexpr (V == 2) *reinterpret_cast<float2 *>(p) = make_float2(v.v[0], v.v[1]);
        else p[0] = v.v[0];
    } else {
#pragma unroll
        for (int e = 0; e < V; ++e)
            if (e < n) p[e] = v.v[e];
    }
}

// ---------------------------------------------------------------------------------------------
// Fused Yee step.  One CTA owns a main tile of 32*V (x) by BY (y) cells and a range of z planes
// [k0, k1); it streams the planes in order, keeping the previous plane's new Hx, Hy and the next
// plane's Ex, Ey in registers (sliding window), so every array element is read from HBM once per
// step.  Thread (lane, ty): ty = 1..BY own row y0+ty-1, V consecutive x cells per lane (V*32-bit
// loads and stores); ty = 0 is a halo row y0-1 that only recomputes new Hx, Hz for the E update of
// row y0.  In-plane neighbours: x+1 / x-1 through warp shuffles (lane 31 / lane 0 fetch the one
// cell beyond the tile), y+1 / y-1 through shared memory.  A tile that starts at k0 > 0 first
// recomputes new Hx, Hy on plane k0-1 ("warm" plane, no stores).
// Work list: blockIdx.x indexes the concatenated tiles of all instances (tile0 = prefix sums);
// each instance's main tiles are followed by its face tiles.  Every instance of a launch must have
// been planned with vec == V.
// ---------------------------------------------------------------------------------------------
template <int BY, int V>
__global__ void __launch_bounds__(32 * (BY + 1), BY <= 4 ? 4 : (BY <= 8 ? 2 : 1))
k_yee_step(const InstDesc *__restrict__ insts, const int *__restrict__ tile0, int ninst, int s_off,
           int total_tiles)
{
    constexpr int TX = 32 * V;
    __shared__ Vec<V> sEx[BY + 1][32];
    __shared__ Vec<V> sEz[BY + 1][32];
    __shared__ Vec<V> sHx[BY + 1][32];
    __shared__ Vec<V> sHz[BY + 1][32];

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
    const int x0 = xt * TX, y0 = yt * BY;
    const int k0 = zt * kc, k1 = min(k0 + kc, nz);
    const int kstart = k0 > 0 ? k0 - 1 : k0;

    const int lane = threadIdx.x, ty = threadIdx.y;
    const int i = x0 + V * lane;
    const int j = y0 + ty - 1;
    const bool halo = (ty == 0);
    const bool xin = (i <= nx);               // vector holds at least one node of the row
    const bool jrow = (j >= 0 && j < ny);     // a row of cells (or a valid halo row)
    const bool jshare = (!halo && j == ny);   // the wall row: only lends Ex, Ez to row Ny-1
    const int nout = min(V, nx - i);          // cells of this vector inside [0, Nx)
    const bool xl = (lane == 31) && (x0 + TX <= nx);   // one node beyond the tile exists
    const bool hcol = (!halo) && (lane == 0) && (x0 > 0) && jrow;   // lane 0 recomputes x0-1

    // Offsets are formed only for rows that exist (j >= 0).
    long long off = (long long)i + (long long)pitch * (j < 0 ? 0 : j) + plane * kstart;

    Vec<V> ex0 = zerov<V>(), ey0 = zerov<V>();   // Ex(k), Ey(k)
    Vec<V> hxp = zerov<V>(), hyp = zerov<V>();   // new Hx, Hy on plane k-1
    if (!halo && xin) {
        if (jrow || jshare) ex0 = ldv<V>(Ex + off);
        if (jrow) ey0 = ldv<V>(Ey + off);
    }

    for (int k = kstart; k < k1; ++k, off += plane) {
        const bool warm = (k < k0);
        Vec<V> hx = zerov<V>(), hy = zerov<V>(), hz = zerov<V>(), ez = zerov<V>(), ex1 = zerov<V>(), ey1 = zerov<V>();
        Vec<V> da = zerov<V>(), db = zerov<V>(), ca = zerov<V>(), cb = zerov<V>();
        Vec<V> exj1 = zerov<V>(), ezj1 = zerov<V>();
        float ez_l = 0.f, ey_l = 0.f;                                  // lane 31: x0+TX
        float hy_h = 0.f, hz_h = 0.f, ez_h = 0.f, ex_h0 = 0.f, ex_h1 = 0.f, ex_hj = 0.f,
              ey_h = 0.f, da_h = 0.f, db_h = 0.f;                        // lane 0: x0-1

        // ---- loads ----------------------------------------------------------------------
        if (halo) {
            if (!warm && jrow && xin) {
                hx = ldv<V>(Hx + off); hz = ldv<V>(Hz + off); ez = ldv<V>(Ez + off);
                ex0 = ldv<V>(Ex + off); ey0 = ldv<V>(Ey + off); ey1 = ldv<V>(Ey + off + plane);
                da = ldv<V>(Da + off); db = ldv<V>(Db + off);
                if (xl) ey_l = __ldg(Ey + off + V);
            }
        } else if (jrow && xin) {
            hx = ldv<V>(Hx + off); hy = ldv<V>(Hy + off); ez = ldv<V>(Ez + off);
            ex1 = ldv<V>(Ex + off + plane); ey1 = ldv<V>(Ey + off + plane);
            da = ldv<V>(Da + off); db = ldv<V>(Db + off);
            if (!warm) { hz = ldv<V>(Hz + off); ca = ldv<V>(Ca + off); cb = ldv<V>(Cb + off); }
            if (ty == BY) { exj1 = ldv<V>(Ex + off + pitch); ezj1 = ldv<V>(Ez + off + pitch); }
            if (xl) { ez_l = __ldg(Ez + off + V); ey_l = __ldg(Ey + off + V); }
            if (hcol && !warm) {
                const long long oh = off - 1;
                hy_h = __ldg(Hy + oh); hz_h = __ldg(Hz + oh); ez_h = __ldg(Ez + oh);
                ex_h0 = __ldg(Ex + oh); ex_h1 = __ldg(Ex + oh + plane); ex_hj = __ldg(Ex + oh + pitch);
                ey_h = __ldg(Ey + oh); da_h = __ldg(Da + oh); db_h = __ldg(Db + oh);
            }
        } else if (jshare && xin) {
            ex0 = ldv<V>(Ex + off); ez = ldv<V>(Ez + off);
        }

        // ---- share Ex, Ez of each row with the row above (its y+1 neighbour) -----------------
        sEx[ty][lane] = ex0;
        sEz[ty][lane] = ez;
        __syncthreads();
        if (ty < BY) {
            exj1 = sEx[ty + 1][lane];
            ezj1 = sEz[ty + 1][lane];
        }

        // ---- x+1 neighbours through shuffles ----------------------------------------------
        float ez_n = __shfl_down_sync(FULL_MASK, ez.v[0], 1);
        float ey_n = __shfl_down_sync(FULL_MASK, ey0.v[0], 1);
        if (lane == 31) { ez_n = ez_l; ey_n = ey_l; }

        // ---- new H on plane k ---------------------------------------------------------------
        Vec<V> hxn, hyn, hzn;
#pragma unroll
        for (int e = 0; e < V; ++e) {
            const float ez_ip = e < V - 1 ? ez.v[e + 1] : ez_n;
            const float ey_ip = e < V - 1 ? ey0.v[e + 1] : ey_n;
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
            sHx[ty][lane] = hxn;
            sHz[ty][lane] = hzn;
        }
        __syncthreads();

        // ---- x-1 neighbours of new Hy, Hz ---------------------------------------------------
        float hy_p = __shfl_up_sync(FULL_MASK, hyn.v[V - 1], 1);
        float hz_p = __shfl_up_sync(FULL_MASK, hzn.v[V - 1], 1);
        if (lane == 0) { hy_p = hyh; hz_p = hzh; }

        if (!halo && jrow && xin) {
            if (!warm) {
                const Vec<V> hxj = sHx[ty - 1][lane];   // new Hx at j-1
                const Vec<V> hzj = sHz[ty - 1][lane];   // new Hz at j-1
                Vec<V> exn, eyn, ezn;
#pragma unroll
                for (int e = 0; e < V; ++e) {
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
                    if (dsrc >= 0 && dsrc < V) {
#pragma unroll
                        for (int e = 0; e < V; ++e)
                            if (e == (int)dsrc) ezn.v[e] = __fadd_rn(ezn.v[e], srcv);
                    }
                }
                if (nout > 0) {
                    stv<V>(oHx + off, hxn, nout); stv<V>(oHy + off, hyn, nout); stv<V>(oHz + off, hzn, nout);
                    stv<V>(oEx + off, exn, nout); stv<V>(oEy + off, eyn, nout); stv<V>(oEz + off, ezn, nout);
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

void plan_tiles(InstDesc &d, int by, int kc, int vec)
{
    const int kcc = (kc <= 0 || kc > d.nz) ? d.nz : kc;
    const int tx = 32 * vec;
    d.vec = vec;
    d.kc = kcc;
    d.tiles_x = (d.nx + tx - 1) / tx;
    d.tiles_y = (d.ny + by - 1) / by;
    d.tiles_z = (d.nz + kcc - 1) / kcc;
    const long long fc = (long long)d.ny * d.nz + (long long)d.nx * d.nz + (long long)d.nx * d.ny;
    const int per = face_tile_cells(by);
    d.face_tiles = (int)((fc + per - 1) / per);
}

void plan_tiles(InstDesc &d, int by, int kc) { plan_tiles(d, by, kc, 4); }

int balanced_depths(int nx, int ny, int nz, int by, int vec, int resident, int *out, int n)
{
    if (resident <= 0 || n <= 0 || by <= 0 || vec <= 0) return 0;
    const long long cols = (long long)((nx + 32 * vec - 1) / (32 * vec)) * ((ny + by - 1) / by);
    std::vector<std::pair<long long, int>> c;
    for (int tz = 1; tz <= nz; ++tz) {
        const int kc = (nz + tz - 1) / tz;
        if ((nz + kc - 1) / kc != tz) continue;   // same depth as a smaller tz
        if (kc < 4) break;
        const long long waves = (cols * tz + resident - 1) / resident;
        c.push_back({waves * (kc + (tz > 1 ? 1 : 0) + 2), kc >= nz ? 0 : kc});
    }
    std::stable_sort(c.begin(), c.end(),
                     [](const std::pair<long long, int> &a, const std::pair<long long, int> &b) { return a.first < b.first; });
    int k = 0;
    for (const auto &e : c) {
        if (k == n) break;
        out[k++] = e.second;
    }
    return k;
}

int leftover_depths(int nx, int ny, int nz, int by, int vec, int resident, int *out, int n)
{
    if (resident <= 0 || n <= 0 || by <= 0 || vec <= 0) return 0;
    const long long cols = (long long)((nx + 32 * vec - 1) / (32 * vec)) * ((ny + by - 1) / by);
    const long long layers = resident / cols, extra = resident - layers * cols;
    if (layers < 1 || extra < 1) return 0;
    const long long rounds = (cols + extra - 1) / extra;   // leftover tiles per extra CTA
    int k = 0;
    for (int kc = 4; kc < nz && k < n; ++kc) {
        const long long rest = nz - layers * kc;
        if (rest <= 0) break;
        if (rest >= kc) continue;   // a full further layer, not a leftover
        if (rounds * (rest + 2) <= kc + 1) out[k++] = kc;
    }
    return k;
}

template <int BY, int V>
static void launch_by_v(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                        int g, cudaStream_t s)
{
    k_yee_step<BY, V><<<g, dim3(32, BY + 1), 0, s>>>(d_insts, d_tile0, ninst, s_offset, total_tiles);
}

int launch_yee_step_v(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                      int by, int vec, int grid, cudaStream_t s)
{
    if (total_tiles <= 0) return PTK_OK;
    const int g = (grid <= 0 || grid > total_tiles) ? total_tiles : grid;
#define PTK_CASE(B, W)                                                                       \
    if (by == B && vec == W) {                                                               \
        launch_by_v<B, W>(d_insts, d_tile0, ninst, total_tiles, s_offset, g, s);             \
        PTK_CUDA_TRY(cudaGetLastError());                                                    \
        count_launches(1);                                                                   \
        return PTK_OK;                                                                       \
    }
    PTK_CASE(4, 1) PTK_CASE(4, 2) PTK_CASE(4, 4)
    PTK_CASE(8, 1) PTK_CASE(8, 2) PTK_CASE(8, 4)
    PTK_CASE(16, 1) PTK_CASE(16, 2) PTK_CASE(16, 4)
#undef PTK_CASE
    return set_error(PTK_ERR_INVALID, "tile rows must be 4, 8 or 16 and cells per thread 1, 2 or 4 (got %d, %d)",
                     by, vec);
}

int launch_yee_step_grid(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles,
                         int s_offset, int by, int grid, cudaStream_t s)
{
    return launch_yee_step_v(d_insts, d_tile0, ninst, total_tiles, s_offset, by, 4, grid, s);
}

int launch_yee_step(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles,
                    int s_offset, int by, cudaStream_t s)
{
    return launch_yee_step_v(d_insts, d_tile0, ninst, total_tiles, s_offset, by, 4, 0, s);
}

int yee_resident_ctas(int by, int vec)
{
    int per_sm = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define PTK_OCC(B, W)                                                                               \
    if (by == B && vec == W)                                                                        \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_yee_step<B, W>, 32 * (B + 1), 0);
    PTK_OCC(4, 1) PTK_OCC(4, 2) PTK_OCC(4, 4)
    PTK_OCC(8, 1) PTK_OCC(8, 2) PTK_OCC(8, 4)
    PTK_OCC(16, 1) PTK_OCC(16, 2) PTK_OCC(16, 4)
#undef PTK_OCC
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * sm_count();
}

int yee_resident_ctas(int by) { return yee_resident_ctas(by, 4); }

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
