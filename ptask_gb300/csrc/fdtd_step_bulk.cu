// fdtd_step_bulk.cu -- the fused Yee step with its operands staged by the TMA engine.
//
// Same arithmetic, work list and results as k_yee_step (fdtd_kernels.cu), different data
// movement.  For every z plane of a W x BY tile (W = 128: a warp per row; W = 64 for 7 and 23 rows:
// a warp per two half rows), the rows of the ten arrays that the plane needs (own rows plus the
// y-1 / y+1 halo rows, W+8 floats wide to cover the x-1 / x+1 halo) arrive in shared memory as one
// TMA tensor copy per array (cp.async.bulk.tensor.3d, box (W+8) x rows x 1): ten copies per plane,
// issued by ten lanes of one warp.  Boxes that hang over the grid's edges are
// filled with zeros by the TMA unit.  Planes are loaded ahead into a ring of S stages, each guarded
// by an mbarrier whose transaction count is the bytes in flight, so the number of bytes in flight
// does not depend on registers or occupancy.  Compute reads only shared memory; results leave with
// 128-bit stores.  One block barrier per plane: new Hx, Hz rows are exchanged through a
// double-buffered shared array, and a stage is refilled only after the barrier that follows its
// last reader.
//
// With a material index (MAT instantiations) the four coefficient boxes of a plane become one box
// of one-byte material ids (160 bytes wide, rows of the tile and its y-1 halo row), and each
// thread looks its cells' (Ca, Cb, Da, Db) up in the instance's table of at most 256 entries,
// copied into shared memory when a CTA starts a tile of another instance: 49 bytes of HBM traffic
// per cell update instead of 64, same values, same results.
//
// Tensor maps (one per array and parity: 6 fields x 2, 4 coefficients, the material index) are
// encoded on the host (cuTensorMapEncodeTiled through the runtime's driver entry point) into
// device memory; the issuing lane acquire-fences a map before its first use in a tile.
//
// Waits on an mbarrier are bounded; on expiry the kernel raises *err (results of that launch are
// then invalid and the host reports PTK_ERR_TIMEOUT).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "fdtd_device.cuh"
#include "fdtd_tma.cuh"

namespace ptk {

namespace {

using namespace tma;

// Tile width W (cells): 128 (a warp per row, 4 cells per lane) or 64 (a warp per two rows, 16
// lanes per row).  A staged float row covers x0-4 .. x0+W+3 and a material-index row x0-16 ..
// x0+W+15, so that both start and end on 16-byte boundaries.
template <int W>
__host__ __device__ constexpr int row_w() { return W + 8; }
template <int W>
__host__ __device__ constexpr int row_b8() { return W + 32; }
template <int W>
__host__ __device__ constexpr int lanes_per_row() { return W / 4; }
template <int W>
__host__ __device__ constexpr int rows_per_warp() { return 32 / lanes_per_row<W>(); }
// Rows that go with a tile width: 7- and 23-row tiles are 64 cells wide (four and twelve warps),
// all others 128.
__host__ __device__ constexpr int width_of(int by) { return (by == 7 || by == 23) ? 64 : 128; }
// CTAs per SM the instantiation is compiled for: four-warp CTAs (7 rows) run three to an SM, each
// with its own plane barrier; the others one.
__host__ __device__ constexpr int ctas_per_sm(int by) { return by == 7 ? 3 : 1; }
constexpr int kMapMat = 16;     // tensor map of the material index in an instance's set

// Arrays in stage order and the frame rows r (j = y0 - 1 + r) each one needs.  With per-cell
// coefficient arrays the stage holds Ca, Cb, Da, Db; with a material index (MAT) one byte per
// node (rows 0..BY) replaces all four and the values come from a table in shared memory.
enum { A_HX, A_HY, A_HZ, A_EX, A_EY, A_EZ, A_CA, A_CB, A_DA, A_DB };
constexpr int A_MT = 6;

template <bool MAT>
__host__ __device__ constexpr int n_arrays() { return MAT ? 7 : 10; }
template <bool MAT>
__host__ __device__ constexpr bool is_u8(int a) { return MAT && a == A_MT; }
template <bool MAT>
__host__ __device__ constexpr int row_lo(int a) { return (a == A_HY || (!MAT && (a == A_CA || a == A_CB))) ? 1 : 0; }
template <int BY>
__host__ __device__ constexpr int row_hi(int a) { return (a == A_EX || a == A_EZ) ? BY + 2 : BY + 1; }
template <int BY, bool MAT>
__host__ __device__ constexpr int rows_of(int a) { return row_hi<BY>(a) - row_lo<MAT>(a); }
template <bool MAT, int W = 128>
__host__ __device__ constexpr int row_bytes(int a) { return is_u8<MAT>(a) ? row_b8<W>() : row_w<W>() * 4; }
// Each array's region in a stage starts on a 128-byte boundary (TMA destination alignment).
template <int BY, bool MAT, int W = width_of(BY)>
__host__ __device__ constexpr int region_bytes(int a) { return (rows_of<BY, MAT>(a) * row_bytes<MAT, W>(a) + 127) / 128 * 128; }
template <int BY, bool MAT>
__host__ __device__ constexpr int region_off(int a)
{
    int o = 0;
    for (int q = 0; q < a; ++q) o += region_bytes<BY, MAT>(q);
    return o;
}
template <int BY, bool MAT>
__host__ __device__ constexpr size_t stage_bytes() { return (size_t)region_off<BY, MAT>(n_arrays<MAT>()); }
template <int BY, bool MAT>
__host__ __device__ constexpr uint32_t box_bytes(int a) { return (uint32_t)(rows_of<BY, MAT>(a) * row_bytes<MAT, width_of(BY)>(a)); }
template <int BY, bool MAT>
__host__ __device__ constexpr uint32_t plane_tx_bytes()
{
    uint32_t t = 0;
    for (int a = 0; a < n_arrays<MAT>(); ++a) t += box_bytes<BY, MAT>(a);
    return t;
}
// Threads of a CTA: one per 4 cells of the tile's BY rows and its y-1 halo row.
template <int BY>
__host__ __device__ constexpr int warps_of() { return (BY + 1) / rows_per_warp<width_of(BY)>(); }
template <int BY>
__host__ __device__ constexpr size_t xchg_bytes() { return (size_t)2 * 2 * (BY + 1) * lanes_per_row<width_of(BY)>() * sizeof(float4); }
// [S stages][H exchange][material table (MAT)][S mbarriers][tile slot][next tile (LAZY)]
constexpr size_t kTileBytes = 64;
template <int BY, int S, bool MAT, bool LAZY = false>
__host__ __device__ constexpr size_t smem_bytes()
{
    return S * stage_bytes<BY, MAT>() + xchg_bytes<BY>() + (MAT ? kTabBytes : 0) + S * 8 + 16 + (LAZY ? kTileBytes : 0);
}

// Map of array a for field parity par in an instance's map set.
template <bool MAT>
__device__ __forceinline__ const CUtensorMap *map_of(const CUtensorMap *set, int a, int par)
{
    return a < 6 ? set + par * 6 + a : (MAT ? set + kMapMat : set + 12 + (a - 6));
}

// Issue plane k of the tile into stage buffer `st` (called by the 32 lanes of one warp; lane a
// issues array a's box).
template <int BY, bool MAT>
__device__ __forceinline__ void issue_plane(const CUtensorMap *set, int par, int x0, int y0, int k, bool next_only,
                                            unsigned char *st, uint64_t *bar, int lane)
{
    if (lane == 0)
        mbar_expect_tx(bar, next_only ? box_bytes<BY, MAT>(A_EX) + box_bytes<BY, MAT>(A_EY) : plane_tx_bytes<BY, MAT>());
    __syncwarp();
    if (lane < n_arrays<MAT>() && (!next_only || lane == A_EX || lane == A_EY))
        tma_load_3d(st + region_off<BY, MAT>(lane), map_of<MAT>(set, lane, par), is_u8<MAT>(lane) ? x0 - 16 : x0 - 4,
                    y0 - 1 + row_lo<MAT>(lane), k, bar);
}

template <int BY, bool MAT>
__device__ __forceinline__ const float *row_ptr(const unsigned char *st, int a, int r)
{
    return reinterpret_cast<const float *>(st + region_off<BY, MAT>(a)) + (size_t)(r - row_lo<MAT>(a)) * row_w<width_of(BY)>();
}

// Material-index row of frame row r; byte 16 + c is the node at x0 + c.
template <int BY>
__device__ __forceinline__ const unsigned char *row_mat(const unsigned char *st, int r)
{
    return st + region_off<BY, true>(A_MT) + (size_t)r * row_b8<width_of(BY)>();
}

}  // namespace

// One main tile of an instance: where it lies and the z-planes it streams (kstart .. k1; plane
// kstart is the warm plane when k0 > 0, plane k1 is read as "next" only).
struct Tile {
    const InstDesc *D;
    const CUtensorMap *maps;
    int par, x0, y0, k0, k1, kstart, nplanes;
};

// Tile t of the concatenated main-tile lists; false when its instance has no step left.
template <int BY>
__device__ __forceinline__ bool tile_at(int t, const InstDesc *__restrict__ insts, const int *__restrict__ tile0,
                                        int ninst, int s_off, Tile &T)
{
    int lo = 0, hi = ninst;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(tile0 + mid) <= t) lo = mid; else hi = mid;
    }
    const InstDesc *D = insts + lo;
    if (s_off >= D->steps_left) return false;
    int r0 = t - __ldg(tile0 + lo);
    const int xt = r0 % D->tiles_x;
    r0 /= D->tiles_x;
    const int yt = r0 % D->tiles_y;
    const int zt = r0 / D->tiles_y;
    T.x0 = xt * width_of(BY);
    T.y0 = yt * BY;
    T.k0 = zt * D->kc;
    T.k1 = min(T.k0 + D->kc, D->nz);
    T.D = D;
    T.maps = reinterpret_cast<const CUtensorMap *>(D->tma);
    T.par = (D->step + s_off) & 1;
    T.kstart = T.k0 > 0 ? T.k0 - 1 : T.k0;
    T.nplanes = T.k1 - T.kstart + 1;
    return true;
}

// The tile lists hold main tiles only: the H nodes of the i = Nx, j = Ny, k = Nz faces are advanced
// by k_yee_faces_steps.  A CTA streams its tiles' planes through one continuous ring: it knows its
// next tile while it works on the current one, and once the current tile's planes are all in
// flight the refills continue with the next tile's, so a tile starts without a pipeline fill.
//
// When the next tile is claimed from the work counter: EAGER (LAZY false) as soon as the current
// one starts, which keeps the claim's latency (an atomic, a search over the instances) off the
// plane loop of the many shallow tiles of a served mix; LAZY just before the ring reaches the next
// tile's first plane, so that CTAs that run ahead take the remaining tiles.  The single-instance
// solver uses LAZY: its grids can then be cut into layers that occupy all but a few resident CTAs
// plus a thin last layer that those few work through meanwhile (an eager CTA would claim a
// last-layer tile at the start and run it after its own layer tile).
template <int BY, int S, bool MAT, bool LAZY = false>
__global__ void __launch_bounds__(32 * warps_of<BY>(), ctas_per_sm(BY))
k_yee_step_bulk(const InstDesc *__restrict__ insts, const int *__restrict__ tile0, int ninst, int s_off,
                int total_tiles, int *err, int *work)
{
    constexpr size_t SB = stage_bytes<BY, MAT>();
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *stages = smem;
    constexpr int LW = lanes_per_row<width_of(BY)>();   // lanes per tile row
    constexpr int RPW = rows_per_warp<width_of(BY)>();   // tile rows per warp
    static_assert((BY + 1) % RPW == 0, "a warp holds whole rows of the frame");
    float4 *xchg = reinterpret_cast<float4 *>(smem + S * SB);   // [2 buf][2 arr][BY+1][LW]
    float4 *tab = reinterpret_cast<float4 *>(smem + S * SB + xchg_bytes<BY>());   // MAT: (Ca, Cb, Da, Db)[256]
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * SB + xchg_bytes<BY>() + (MAT ? kTabBytes : 0));
    int *slot = reinterpret_cast<int *>(bars + S);   // next tile, handed to the whole CTA
    // LAZY: the claimed tile's descriptor; only warp 0 reads it (to issue its planes) until it
    // becomes the current tile, so it holds no registers in the plane loop.
    Tile *sT1 = reinterpret_cast<Tile *>(bars + S + 2);
    const void *tab_src = nullptr;                   // instance whose table is loaded (MAT)

    const int lane = threadIdx.x, ty = threadIdx.y;
    if (smem_u32(smem) & 127u) {   // TMA destinations need 128-byte alignment: refuse, do not fault
        if (ty == 0 && lane == 0) atomicOr(err, 2);
        return;
    }
    if (ty == 0 && lane == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // Tiles: the first one is blockIdx.x; later ones are static (t + gridDim.x) or, with a work
    // counter (zeroed before the launch), taken in list order as CTAs free up.  All threads take
    // every branch below together, so the barriers in `advance` are reached by all.
    auto advance = [&](int t) -> int {
        if (!work) return t + (int)gridDim.x;
        __syncthreads();
        if (ty == 0 && lane == 0) *slot = (int)gridDim.x + atomicAdd(work + s_off, 1);
        __syncthreads();
        return *slot;
    };
    auto fetch = [&](int &t, Tile &T) -> bool {   // first live tile at or after t
        while (t < total_tiles) {
            if (tile_at<BY>(t, insts, tile0, ninst, s_off, T)) return true;
            t = advance(t);
        }
        return false;
    };

    int t = blockIdx.x, t1 = total_tiles;
    Tile T0{}, T1{};
    bool have0 = fetch(t, T0), have1 = false, asked1 = false;
    if constexpr (!LAZY) {
        if (have0) {
            t1 = advance(t);
            have1 = fetch(t1, T1);
        }
    }
    auto next_tile = [&]() -> const Tile & {
        if constexpr (LAZY) return *sT1; else return T1;
    };
    // Ring positions: the planes of this CTA's tiles in order; plane j of the current tile is
    // position gbase + j.  Positions below `issued` are in flight or consumed.
    unsigned gbase = 0, issued = 0;
    bool acq0 = false, acq1 = false;   // tensor maps of T0 / T1 acquire-fenced by warp 0
    bool failed = false;
    // Issue every position below `limit` that belongs to the current or the next tile (warp 0).
    auto top_up = [&](unsigned limit) {
        while (issued < limit) {
            const unsigned p = issued;
            if (p < gbase + (unsigned)T0.nplanes) {
                if (!acq0) {
                    if (lane < n_arrays<MAT>()) tma_acquire(map_of<MAT>(T0.maps, lane, T0.par));
                    acq0 = true;
                }
                const int j = (int)(p - gbase);
                issue_plane<BY, MAT>(T0.maps, T0.par, T0.x0, T0.y0, T0.kstart + j, T0.kstart + j == T0.k1,
                                     stages + (size_t)(p % S) * SB, &bars[p % S], lane);
            } else if (have1 && p < gbase + (unsigned)(T0.nplanes + next_tile().nplanes)) {
                const Tile &T1 = next_tile();
                if (!acq1) {
                    if (lane < n_arrays<MAT>()) tma_acquire(map_of<MAT>(T1.maps, lane, T1.par));
                    acq1 = true;
                }
                const int j = (int)(p - gbase) - T0.nplanes;
                issue_plane<BY, MAT>(T1.maps, T1.par, T1.x0, T1.y0, T1.kstart + j, T1.kstart + j == T1.k1,
                                     stages + (size_t)(p % S) * SB, &bars[p % S], lane);
            } else {
                break;
            }
            ++issued;
        }
    };

    while (have0) {
        const InstDesc *__restrict__ D = T0.D;
        if constexpr (MAT) {
            // The previous tile ended with a block barrier: nobody reads the old table any more.
            if (D->mat_tab != tab_src) {
                const float4 *src_tab = reinterpret_cast<const float4 *>(D->mat_tab);
                for (int m = ty * 32 + lane; m < D->nmat; m += 32 * warps_of<BY>()) tab[m] = __ldg(src_tab + m);
                tab_src = D->mat_tab;
                __syncthreads();
            }
        }
        if (ty == 0) top_up(gbase + S);

        const int nx = D->nx, ny = D->ny, pitch = D->pitch;
        const long long plane = D->plane;
        const float cx = D->cx, cy = D->cy, cz = D->cz;
        const int par = T0.par, x0 = T0.x0, y0 = T0.y0, k0 = T0.k0, k1 = T0.k1, kstart = T0.kstart;
        const int step = D->step + s_off;
        float *__restrict__ oHx = D->buf[par ^ 1][0];
        float *__restrict__ oHy = D->buf[par ^ 1][1];
        float *__restrict__ oHz = D->buf[par ^ 1][2];
        float *__restrict__ oEx = D->buf[par ^ 1][3];
        float *__restrict__ oEy = D->buf[par ^ 1][4];
        float *__restrict__ oEz = D->buf[par ^ 1][5];
        const long long src = D->src;
        const float srcv = (src >= 0 && step < D->nwave) ? __ldg(D->wave + step) : 0.f;

        const int lx = lane % LW;         // this thread's 4 cells in its row
        const int r = ty * RPW + lane / LW;   // frame row of this thread
        const int i = x0 + 4 * lx;
        const int j = y0 + r - 1;
        const bool halo = (r == 0);
        const bool xin = (i <= nx);
        const bool jrow = (j >= 0 && j < ny);
        const int nout = min(4, nx - i);
        const bool hcol = (!halo) && (lx == 0) && (x0 > 0) && jrow;
        const int xl = 4 + 4 * lx;        // local x of this thread's first cell in a staged row
        long long off = (long long)i + (long long)pitch * (j < 0 ? 0 : j) + plane * kstart;

        float4 hxp = make_float4(0, 0, 0, 0), hyp = make_float4(0, 0, 0, 0);

        for (int k = kstart; k < k1; ++k, off += plane) {
            const int q = k - kstart;
            const unsigned Gc = gbase + q, Gn = Gc + 1;
            const unsigned char *cur = stages + (size_t)(Gc % S) * SB;
            const unsigned char *nxt = stages + (size_t)(Gn % S) * SB;
            if (!failed) {
                // Within a tile, plane q's stage was waited for as "next" in iteration q-1, and it is
                // refilled only after this iteration's barrier.
                bool ok = q > 0 || mbar_wait(&bars[Gc % S], (Gc / S) & 1);
                ok = ok && mbar_wait(&bars[Gn % S], (Gn / S) & 1);
                if (!ok) {
                    failed = true;
                    atomicOr(err, 1);
                }
            }
            const bool warm = (k < k0);
            float4 hx = make_float4(0, 0, 0, 0), hy = hx, hz = hx, ez = hx, ex0 = hx, ey0 = hx, ex1 = hx, ey1 = hx;
            float4 exj1 = hx, ezj1 = hx, da = hx, db = hx, ca = hx, cb = hx;
            float ez_l = 0.f, ey_l = 0.f;
            const bool act = xin && (halo ? (jrow && !warm) : jrow);
            if (act) {
                hx = ld4s(row_ptr<BY, MAT>(cur, A_HX, r) + xl);
                ez = ld4s(row_ptr<BY, MAT>(cur, A_EZ, r) + xl);
                ex0 = ld4s(row_ptr<BY, MAT>(cur, A_EX, r) + xl);
                ey0 = ld4s(row_ptr<BY, MAT>(cur, A_EY, r) + xl);
                ey1 = ld4s(row_ptr<BY, MAT>(nxt, A_EY, r) + xl);
                exj1 = ld4s(row_ptr<BY, MAT>(cur, A_EX, r + 1) + xl);
                ezj1 = ld4s(row_ptr<BY, MAT>(cur, A_EZ, r + 1) + xl);
                hz = ld4s(row_ptr<BY, MAT>(cur, A_HZ, r) + xl);
                if constexpr (MAT) {
                    // four material ids, one per cell, then their (Ca, Cb, Da, Db) from the table
                    const uint32_t ids = *reinterpret_cast<const uint32_t *>(row_mat<BY>(cur, r) + 16 + 4 * lx);
                    const float4 m0 = tab[ids & 255u], m1 = tab[(ids >> 8) & 255u];
                    const float4 m2 = tab[(ids >> 16) & 255u], m3 = tab[ids >> 24];
                    ca = make_float4(m0.x, m1.x, m2.x, m3.x);
                    cb = make_float4(m0.y, m1.y, m2.y, m3.y);
                    da = make_float4(m0.z, m1.z, m2.z, m3.z);
                    db = make_float4(m0.w, m1.w, m2.w, m3.w);
                } else {
                    da = ld4s(row_ptr<BY, MAT>(cur, A_DA, r) + xl);
                    db = ld4s(row_ptr<BY, MAT>(cur, A_DB, r) + xl);
                }
                if (!halo) {
                    hy = ld4s(row_ptr<BY, MAT>(cur, A_HY, r) + xl);
                    ex1 = ld4s(row_ptr<BY, MAT>(nxt, A_EX, r) + xl);
                    if constexpr (!MAT) {
                        ca = ld4s(row_ptr<BY, MAT>(cur, A_CA, r) + xl);
                        cb = ld4s(row_ptr<BY, MAT>(cur, A_CB, r) + xl);
                    }
                }
                if (lx == LW - 1) {
                    ez_l = row_ptr<BY, MAT>(cur, A_EZ, r)[xl + 4];
                    ey_l = row_ptr<BY, MAT>(cur, A_EY, r)[xl + 4];
                }
            }
            // x+1 neighbours (shuffles within each row's LW lanes)
            float ez_n = __shfl_down_sync(0xffffffffu, ez.x, 1, LW);
            float ey_n = __shfl_down_sync(0xffffffffu, ey0.x, 1, LW);
            if (lx == LW - 1) { ez_n = ez_l; ey_n = ey_l; }
            const float ezv[4] = {ez.x, ez.y, ez.z, ez.w}, eyv[4] = {ey0.x, ey0.y, ey0.z, ey0.w};
            const float ez_ip[4] = {ez.y, ez.z, ez.w, ez_n}, ey_ip[4] = {ey0.y, ey0.z, ey0.w, ey_n};
            const float hxv[4] = {hx.x, hx.y, hx.z, hx.w}, hyv[4] = {hy.x, hy.y, hy.z, hy.w};
            const float hzv[4] = {hz.x, hz.y, hz.z, hz.w};
            const float ex0v[4] = {ex0.x, ex0.y, ex0.z, ex0.w}, ex1v[4] = {ex1.x, ex1.y, ex1.z, ex1.w};
            const float ey1v[4] = {ey1.x, ey1.y, ey1.z, ey1.w};
            const float exjv[4] = {exj1.x, exj1.y, exj1.z, exj1.w}, ezjv[4] = {ezj1.x, ezj1.y, ezj1.z, ezj1.w};
            const float dav[4] = {da.x, da.y, da.z, da.w}, dbv[4] = {db.x, db.y, db.z, db.w};
            // In 128-wide tiles a warp is one row: a warp whose row lies outside the instance (past Ny
            // in the last tile of a column, or the halo row of a warm plane) has no H to compute and
            // skips the arithmetic instead of running it on zeros, leaving the SM's issue slots to the
            // warps with cells.  (64-wide tiles keep the unconditional form, measured faster there.)
            float hxn[4] = {0.f, 0.f, 0.f, 0.f}, hyn[4] = {0.f, 0.f, 0.f, 0.f}, hzn[4] = {0.f, 0.f, 0.f, 0.f};
            if (LW != 32 || __any_sync(0xffffffffu, act)) {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    hxn[e] = yee_b(dav[e], hxv[e], dbv[e], ey1v[e], eyv[e], cz, ezjv[e], ezv[e], cy);
                    hyn[e] = yee_b(dav[e], hyv[e], dbv[e], ez_ip[e], ezv[e], cx, ex1v[e], ex0v[e], cz);
                    hzn[e] = yee_b(dav[e], hzv[e], dbv[e], exjv[e], ex0v[e], cy, ey_ip[e], eyv[e], cx);
                }
            }
            float hyh = 0.f, hzh = 0.f;   // halo column x0-1
            if (hcol && !warm) {
                const float *Hy = row_ptr<BY, MAT>(cur, A_HY, r), *Hz = row_ptr<BY, MAT>(cur, A_HZ, r);
                const float *Ez = row_ptr<BY, MAT>(cur, A_EZ, r), *Ex = row_ptr<BY, MAT>(cur, A_EX, r);
                const float *Exn = row_ptr<BY, MAT>(nxt, A_EX, r), *Exj = row_ptr<BY, MAT>(cur, A_EX, r + 1);
                const float *Ey = row_ptr<BY, MAT>(cur, A_EY, r);
                float dah, dbh;   // coefficients of node x0-1
                if constexpr (MAT) {
                    const float4 mh = tab[row_mat<BY>(cur, r)[15]];
                    dah = mh.z;
                    dbh = mh.w;
                } else {
                    dah = row_ptr<BY, MAT>(cur, A_DA, r)[3];
                    dbh = row_ptr<BY, MAT>(cur, A_DB, r)[3];
                }
                hyh = yee_b(dah, Hy[3], dbh, ez.x, Ez[3], cx, Exn[3], Ex[3], cz);
                hzh = yee_b(dah, Hz[3], dbh, Exj[3], Ex[3], cy, ey0.x, Ey[3], cx);
            }
            float4 *sH = xchg + (size_t)(q & 1) * 2 * (BY + 1) * LW;   // [arr][row][x lane]
            if (!warm) {
                sH[r * LW + lx] = make_float4(hxn[0], hxn[1], hxn[2], hxn[3]);
                sH[(BY + 1) * LW + r * LW + lx] = make_float4(hzn[0], hzn[1], hzn[2], hzn[3]);
            }
            __syncthreads();
            if constexpr (LAZY) {
                // the refill below reaches the next tile's first plane from q = nplanes - S on
                if (!asked1 && q == max(0, T0.nplanes - S)) {
                    t1 = advance(t);
                    Tile Tn;
                    have1 = fetch(t1, Tn);
                    if (ty == 0 && lane == 0 && have1) *sT1 = Tn;
                    __syncwarp();   // warp 0 reads it in the refill below
                    asked1 = true;
                }
            }
            // Plane k's stage was read (as "next") before the previous barrier and (as "current")
            // before this one, and nothing after this barrier reads a stage: refill it now (with a
            // plane of the next tile once this tile's planes are all in flight).
            if (ty == 0) top_up(gbase + q + 1 + S);
            float hy_p = __shfl_up_sync(0xffffffffu, hyn[3], 1, LW);
            float hz_p = __shfl_up_sync(0xffffffffu, hzn[3], 1, LW);
            if (lx == 0) { hy_p = hyh; hz_p = hzh; }
            if (!halo && jrow && xin) {
                if (!warm) {
                    const float4 hxj4 = sH[(r - 1) * LW + lx];
                    const float4 hzj4 = sH[(BY + 1) * LW + (r - 1) * LW + lx];
                    const float hxj[4] = {hxj4.x, hxj4.y, hxj4.z, hxj4.w}, hzj[4] = {hzj4.x, hzj4.y, hzj4.z, hzj4.w};
                    const float cav[4] = {ca.x, ca.y, ca.z, ca.w}, cbv[4] = {cb.x, cb.y, cb.z, cb.w};
                    const float hxpv[4] = {hxp.x, hxp.y, hxp.z, hxp.w}, hypv[4] = {hyp.x, hyp.y, hyp.z, hyp.w};
                    float exn[4], eyn[4], ezn[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int x = i + e;
                        const float hy_im = e > 0 ? hyn[e - 1] : hy_p;
                        const float hz_im = e > 0 ? hzn[e - 1] : hz_p;
                        exn[e] = (j >= 1 && k >= 1)
                            ? yee_b(cav[e], ex0v[e], cbv[e], hzn[e], hzj[e], cy, hyn[e], hypv[e], cz) : ex0v[e];
                        eyn[e] = (x >= 1 && k >= 1)
                            ? yee_b(cav[e], eyv[e], cbv[e], hxn[e], hxpv[e], cz, hzn[e], hz_im, cx) : eyv[e];
                        ezn[e] = (x >= 1 && j >= 1)
                            ? yee_b(cav[e], ezv[e], cbv[e], hyn[e], hy_im, cx, hxn[e], hxj[e], cy) : ezv[e];
                    }
                    if (src >= 0) {
                        const long long dsrc = src - off;
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (dsrc == e) ezn[e] = __fadd_rn(ezn[e], srcv);
                    }
                    if (nout >= 4) {
                        *reinterpret_cast<float4 *>(oHx + off) = make_float4(hxn[0], hxn[1], hxn[2], hxn[3]);
                        *reinterpret_cast<float4 *>(oHy + off) = make_float4(hyn[0], hyn[1], hyn[2], hyn[3]);
                        *reinterpret_cast<float4 *>(oHz + off) = make_float4(hzn[0], hzn[1], hzn[2], hzn[3]);
                        *reinterpret_cast<float4 *>(oEx + off) = make_float4(exn[0], exn[1], exn[2], exn[3]);
                        *reinterpret_cast<float4 *>(oEy + off) = make_float4(eyn[0], eyn[1], eyn[2], eyn[3]);
                        *reinterpret_cast<float4 *>(oEz + off) = make_float4(ezn[0], ezn[1], ezn[2], ezn[3]);
                    } else {
                        for (int e = 0; e < nout; ++e) {
                            oHx[off + e] = hxn[e]; oHy[off + e] = hyn[e]; oHz[off + e] = hzn[e];
                            oEx[off + e] = exn[e]; oEy[off + e] = eyn[e]; oEz[off + e] = ezn[e];
                        }
                    }
                }
                hxp = make_float4(hxn[0], hxn[1], hxn[2], hxn[3]);
                hyp = make_float4(hyn[0], hyn[1], hyn[2], hyn[3]);
            }
        }
        gbase += (unsigned)T0.nplanes;
        // The stages of this tile are refilled only after the barriers of the planes that follow
        // them, which every thread reaches after finishing this tile.
        __syncthreads();
        if constexpr (LAZY) {
            if (!asked1) {   // not reached: the plane loop claims it (q = nplanes - S <= nplanes - 2)
                t1 = advance(t);
                Tile Tn;
                have1 = fetch(t1, Tn);
                if (ty == 0 && lane == 0 && have1) *sT1 = Tn;
                __syncthreads();
            }
            if (have1) T0 = *sT1;   // written before this tile's last barrier
            have0 = have1;
            acq0 = acq1;
            acq1 = false;
            have1 = false;
            asked1 = false;
            if (have0) t = t1;
        } else {
            T0 = T1;
            have0 = have1;
            acq0 = acq1;
            acq1 = false;
            have1 = false;
            if (have0) {
                t = t1;
                t1 = advance(t);
                have1 = fetch(t1, T1);
            }
        }
    }
    // Every issued plane has normally been waited for.  If a wait expired, let the copies still
    // in flight land (bounded) before this CTA's shared memory is released.
    if (ty == 0 && lane == 0)
        for (unsigned G = issued > (unsigned)S ? issued - S : 0u; G < issued; ++G) mbar_wait(&bars[G % S], (G / S) & 1);
}

// The H nodes outside the cell block (Hx at i = Nx, Hy at j = Ny, Hz at k = Nz) for `len` steps
// from step offset s_off.  Their update reads only E nodes on the PEC walls, which never change,
// and no other node's update reads them, so each evolves alone: H <- Da*H + Db*curl with a fixed
// curl, the same operations in the same order as one step at a time.  Thread per face node over
// all instances (face0: prefix of the instances' face-node counts); the result is written to the
// buffer of the parity the instance's step counter has after its steps in this range.
__global__ void k_yee_faces_steps(const InstDesc *__restrict__ insts, const long long *__restrict__ face0,
                                  int ninst, int s_off, int len)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= __ldg(face0 + ninst)) return;
    int lo = 0, hi = ninst;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(face0 + mid) <= g) lo = mid; else hi = mid;
    }
    const InstDesc *__restrict__ D = insts + lo;
    const int n = min(len, D->steps_left - s_off);
    if (n <= 0) return;
    const int nx = D->nx, ny = D->ny, nz = D->nz, pitch = D->pitch;
    const long long plane = D->plane;
    const int p0 = (D->step + s_off) & 1;
    const float *__restrict__ Ex = D->buf[p0][3];
    const float *__restrict__ Ey = D->buf[p0][4];
    const float *__restrict__ Ez = D->buf[p0][5];
    const long long A = (long long)ny * nz, B = (long long)nx * nz;
    const long long q = g - __ldg(face0 + lo);
    long long o;
    int f;
    float a1, a0, s1, b1, b0, s2;
    if (q < A) {                       // Hx at i = Nx: (Ey(k+1) - Ey(k)) Cz - (Ez(j+1) - Ez(j)) Cy
        const int j = (int)(q % ny), k = (int)(q / ny);
        o = nx + (long long)pitch * j + plane * k;
        f = 0;
        a1 = Ey[o + plane]; a0 = Ey[o]; s1 = D->cz; b1 = Ez[o + pitch]; b0 = Ez[o]; s2 = D->cy;
    } else if (q < A + B) {            // Hy at j = Ny: (Ez(i+1) - Ez(i)) Cx - (Ex(k+1) - Ex(k)) Cz
        const long long r = q - A;
        const int i = (int)(r % nx), k = (int)(r / nx);
        o = i + (long long)pitch * ny + plane * k;
        f = 1;
        a1 = Ez[o + 1]; a0 = Ez[o]; s1 = D->cx; b1 = Ex[o + plane]; b0 = Ex[o]; s2 = D->cz;
    } else {                           // Hz at k = Nz: (Ex(j+1) - Ex(j)) Cy - (Ey(i+1) - Ey(i)) Cx
        const long long r = q - A - B;
        const int i = (int)(r % nx), j = (int)(r / nx);
        o = i + (long long)pitch * j + plane * nz;
        f = 2;
        a1 = Ex[o + pitch]; a0 = Ex[o]; s1 = D->cy; b1 = Ey[o + 1]; b0 = Ey[o]; s2 = D->cx;
    }
    const float da = D->coef[2][o], db = D->coef[3][o];
    float h = D->buf[p0][f][o];
    for (int s = 0; s < n; ++s) h = yee_b(da, h, db, a1, a0, s1, b1, b0, s2);
    D->buf[(p0 + n) & 1][f][o] = h;
}

int launch_yee_faces_steps(const InstDesc *d_insts, const long long *d_face0, int ninst, long long total_faces,
                           int s_offset, int len, cudaStream_t s)
{
    if (total_faces <= 0 || len <= 0) return PTK_OK;
    const long long blocks = (total_faces + 255) / 256;
    k_yee_faces_steps<<<(unsigned)blocks, 256, 0, s>>>(d_insts, d_face0, ninst, s_offset, len);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

long long face_nodes(int nx, int ny, int nz) { return (long long)ny * nz + (long long)nx * nz + (long long)nx * ny; }

// Opt the instantiation into its dynamic shared memory (once per process; repeating it is harmless).
template <int BY, int S, bool MAT, bool LAZY>
static int prepare_bulk()
{
    static bool attr_set = false;
    if (!attr_set) {
        PTK_CUDA_TRY(cudaFuncSetAttribute(k_yee_step_bulk<BY, S, MAT, LAZY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem_bytes<BY, S, MAT, LAZY>()));
        // all of the unified L1 / shared storage as shared memory, so small rings can co-reside
        PTK_CUDA_TRY(cudaFuncSetAttribute(k_yee_step_bulk<BY, S, MAT, LAZY>,
                                          cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        attr_set = true;
    }
    return PTK_OK;
}

template <int BY, int S, bool MAT, bool LAZY>
static int resident_bulk()
{
    if (prepare_bulk<BY, S, MAT, LAZY>()) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_yee_step_bulk<BY, S, MAT, LAZY>, 32 * warps_of<BY>(),
                                                      smem_bytes<BY, S, MAT, LAZY>()) != cudaSuccess)
        return 0;
    return per_sm * std::max(1, sm_count());
}

template <int BY, int S, bool MAT, bool LAZY>
static int launch_bulk(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                       int grid, int *err, int *work, cudaStream_t s)
{
    const size_t smem = smem_bytes<BY, S, MAT, LAZY>();
    int rc = prepare_bulk<BY, S, MAT, LAZY>();
    if (rc) return rc;
    const int g = (grid <= 0 || grid > total_tiles) ? total_tiles : grid;
    k_yee_step_bulk<BY, S, MAT, LAZY><<<g, dim3(32, warps_of<BY>()), smem, s>>>(d_insts, d_tile0, ninst, s_offset,
                                                                                total_tiles, err, work);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

// Instantiated shapes (rows, ring stages).  Rings of at least 2 stages: plane q waits for the stage
// of plane q+1 before its barrier, and the stage of plane q+1 is issued after the barrier of plane
// q+1-S, so q+1-S <= q-1.  The material-index stages are smaller, so deeper rings fit.  The
// material-index shapes also come with the late next-tile claim (the solver's form).
#define PTK_DENSE_SHAPES(X) X(4, 2, false) X(4, 3, false) X(4, 4, false) X(4, 5, false) \
    X(8, 2, false) X(8, 3, false) X(8, 4, false) X(10, 3, false) X(11, 3, false)
#define PTK_MAT_SHAPES(X) X(4, 2, true) X(4, 3, true) X(4, 4, true) X(4, 5, true) X(4, 6, true) \
    X(8, 2, true) X(8, 3, true) X(8, 4, true) X(8, 5, true) X(8, 6, true) \
    X(10, 4, true) X(10, 5, true) X(11, 4, true) X(23, 3, true) X(23, 4, true) \
    X(7, 3, true) X(7, 4, true)

int launch_yee_step_bulk(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                         int by, int stages, int grid, int *err, cudaStream_t s, int *work, bool mat, bool lazy)
{
    if (total_tiles <= 0) return PTK_OK;
    if (lazy && mat) {
#define PTK_BULK_L(B, S, M)                                                                           \
    if (by == B && stages == S && mat == M)                                                           \
        return launch_bulk<B, S, M, true>(d_insts, d_tile0, ninst, total_tiles, s_offset, grid, err, work, s);
        PTK_MAT_SHAPES(PTK_BULK_L)
#undef PTK_BULK_L
    }
#define PTK_BULK(B, S, M)                                                                               \
    if (by == B && stages == S && mat == M)                                                             \
        return launch_bulk<B, S, M, false>(d_insts, d_tile0, ninst, total_tiles, s_offset, grid, err, work, s);
    PTK_DENSE_SHAPES(PTK_BULK) PTK_MAT_SHAPES(PTK_BULK)
#undef PTK_BULK
    return set_error(PTK_ERR_INVALID, "no staged kernel for %d rows x %d stages%s", by, stages,
                     mat ? " with a material index" : "");
}

int yee_bulk_tile_vec(int by) { return width_of(by) / 32; }

size_t yee_bulk_smem_bytes(int by, int stages, bool mat)
{
#define PTK_SM(B, S, M) \
    if (by == B && stages == S && mat == M) return smem_bytes<B, S, M, false>();
    PTK_DENSE_SHAPES(PTK_SM) PTK_MAT_SHAPES(PTK_SM)
#undef PTK_SM
    return 0;
}

int yee_bulk_resident_ctas(int by, int stages, bool mat)
{
#define PTK_RES(B, S, M) \
    if (by == B && stages == S && mat == M) return resident_bulk<B, S, M, false>();
    PTK_DENSE_SHAPES(PTK_RES) PTK_MAT_SHAPES(PTK_RES)
#undef PTK_RES
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Self-test of the bounded wait: an mbarrier armed for transactions that never arrive.
// ---------------------------------------------------------------------------------------------
__global__ void k_wait_expiry_probe(int *err)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);   // the phase needs 16 bytes that no copy brings
    __syncthreads();
    if (!mbar_wait(&bar, 0) && threadIdx.x == 0) atomicOr(err, 1);
}

}  // namespace ptk

extern "C" int ptk_selftest_wait_expiry(int *error_word, float *elapsed_ms)
{
    using namespace ptk;
    clear_error();
    int rc = ensure_init();
    if (rc) return rc;
    cudaStream_t st = default_stream();
    int *d_err = nullptr;
    rc = pool_alloc(sizeof(int), st, (void **)&d_err);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(d_err, 0, sizeof(int), st);
    cudaEventRecord(e0, st);
    k_wait_expiry_probe<<<1, 32, 0, st>>>(d_err);
    const cudaError_t le = cudaGetLastError();
    count_launches(1);
    cudaEventRecord(e1, st);
    int h = 0;
    cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t se = cudaStreamSynchronize(st);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pool_free(d_err, st);
    if (le != cudaSuccess || se != cudaSuccess)
        return set_error(PTK_ERR_CUDA, "wait-expiry probe failed: %s", cudaGetErrorString(le != cudaSuccess ? le : se));
    if (error_word) *error_word = h;
    if (elapsed_ms) *elapsed_ms = ms;
    if (h) return set_error(PTK_ERR_TIMEOUT, "bounded wait expired after %.1f ms (error word %d)", ms, h);
    return set_error(PTK_ERR_STATE, "the probe's wait completed, but no transaction could complete it");
}

namespace ptk {

// ---------------------------------------------------------------------------------------------
// Tensor maps.
// ---------------------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

template <int BY>
static int encode_set(const InstDesc &d, CUtensorMap *out)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return set_error(PTK_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[3] = {(cuuint64_t)d.pitch, (cuuint64_t)d.ny + 1, (cuuint64_t)d.nz + 1};
    const cuuint64_t strides[2] = {(cuuint64_t)d.pitch * 4, (cuuint64_t)d.plane * 4};
    const cuuint64_t strides8[2] = {(cuuint64_t)d.pitch, (cuuint64_t)d.plane};
    const cuuint32_t estr[3] = {1, 1, 1};
    // maps 0..11: the fields of both parities; 12..15: Ca, Cb, Da, Db; 16: the material index
    for (int m = 0; m < 17; ++m) {
        if (m == kMapMat && !d.mat) break;
        const bool u8 = m == kMapMat;
        const int a = m < 12 ? m % 6 : (u8 ? A_MT : 6 + (m - 12));
        void *base = m < 12 ? (void *)d.buf[m / 6][m % 6] : u8 ? (void *)d.mat : (void *)d.coef[m - 12];
        const cuuint32_t box[3] = {(cuuint32_t)(u8 ? row_b8<width_of(BY)>() : row_w<width_of(BY)>()),
                                   (cuuint32_t)(u8 ? rows_of<BY, true>(a) : rows_of<BY, false>(a)), 1};
        CUresult r = enc(&out[m], u8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims,
                         u8 ? strides8 : strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return set_error(PTK_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for map %d", (int)r, m);
    }
    return PTK_OK;
}

int encode_tma_set(const InstDesc &d, int by, void *host_out)
{
    CUtensorMap *out = static_cast<CUtensorMap *>(host_out);
    if (by == 4) return encode_set<4>(d, out);
    if (by == 8) return encode_set<8>(d, out);
    if (by == 10) return encode_set<10>(d, out);
    if (by == 11) return encode_set<11>(d, out);
    if (by == 23) return encode_set<23>(d, out);
    if (by == 7) return encode_set<7>(d, out);
    return set_error(PTK_ERR_INVALID, "no staged kernel for %d rows", by);
}

}  // namespace ptk
