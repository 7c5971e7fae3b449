// fdtd_step_bulk.cu -- the fused Yee step with its operands staged by the TMA engine.
//
// Same arithmetic, tiles, work list and results as k_yee_step (fdtd_kernels.cu), different data
// movement.  For every z plane of a 128 x BY tile, the rows of all ten arrays that the plane needs
// (own rows plus the y-1 / y+1 halo rows, 136 floats wide to cover the x-1 / x+1 halo with 16-byte
// aligned copies) are fetched into shared memory by one-dimensional bulk asynchronous copies
// (cp.async.bulk ... mbarrier::complete_tx::bytes).  Planes are loaded S-1 ahead into a ring of S
// stages, each guarded by an mbarrier whose transaction count is the bytes in flight, so the number
// of bytes in flight no longer depends on registers or occupancy: the SM keeps whole planes
// streaming while its warps compute.  Compute reads only shared memory; results are written with
// 128-bit stores.  One block barrier per plane: new Hx, Hz rows are exchanged through a
// double-buffered shared array, and a stage is refilled only after the barrier that follows its
// last reader.
//
// Waits on an mbarrier are bounded; on expiry the kernel raises *err and stops using the stage
// (results of that launch are then invalid and the host reports PTK_ERR_TIMEOUT).
#include "fdtd_device.cuh"

namespace ptk {

namespace {

constexpr int kRowW = 136;      // staged row: x0-4 .. x0+131 (16-byte aligned ends)
constexpr int kWaitLimit = 1 << 22;

// Arrays in stage order and the frame rows r (j = y0 - 1 + r) each one needs.
enum { A_HX, A_HY, A_HZ, A_EX, A_EY, A_EZ, A_CA, A_CB, A_DA, A_DB, A_N };

__host__ __device__ constexpr int row_lo(int a) { return (a == A_HY || a == A_CA || a == A_CB) ? 1 : 0; }
template <int BY>
__host__ __device__ constexpr int row_hi(int a) { return (a == A_EX || a == A_EZ) ? BY + 2 : BY + 1; }
template <int BY>
__host__ __device__ constexpr int row_off(int a)   // first row of array a inside a stage
{
    int o = 0;
    for (int q = 0; q < a; ++q) o += row_hi<BY>(q) - row_lo(q);
    return o;
}
template <int BY>
__host__ __device__ constexpr int stage_rows() { return row_off<BY>(A_N); }
template <int BY>
__host__ __device__ constexpr size_t stage_bytes() { return (size_t)stage_rows<BY>() * kRowW * sizeof(float); }
template <int BY>
__host__ __device__ constexpr size_t xchg_bytes() { return (size_t)2 * 2 * (BY + 1) * 32 * sizeof(float4); }
template <int BY, int S>
__host__ __device__ constexpr size_t smem_bytes() { return S * stage_bytes<BY>() + xchg_bytes<BY>() + S * 8; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ float4 ld4s(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ float yee_b(float d, float h, float c, float a1, float a0, float s1, float b1, float b0,
                                       float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(__fmul_rn(d, h), __fmul_rn(c, curl));
}

struct TileGeom {
    const float *src[A_N];   // plane-0 base of each array (fields of the current parity)
    long long plane;
    int pitch, ny, x0, y0, xs, xe;   // staged x range [xs, xe) in global floats
};

// Issue the copies of plane k into stage buffer `st` (called by the 32 lanes of one warp).
template <int BY>
__device__ __forceinline__ void issue_plane(const TileGeom &g, int k, bool next_only, float *st, uint64_t *bar,
                                            int lane)
{
    const uint32_t row_bytes = (uint32_t)(g.xe - g.xs) * 4u;
    const int dx = g.xs - (g.x0 - 4);   // destination offset inside a staged row (floats)
    // count the rows first so that the transaction count is registered before any copy lands
    uint32_t rows = 0;
#pragma unroll
    for (int a = 0; a < A_N; ++a) {
        if (next_only && a != A_EX && a != A_EY) continue;
        for (int r = row_lo(a); r < row_hi<BY>(a); ++r) {
            const int j = g.y0 - 1 + r;
            if (j >= 0 && j <= g.ny) ++rows;
        }
    }
    if (lane == 0) mbar_expect_tx(bar, rows * row_bytes);
    __syncwarp();
    int n = 0;
#pragma unroll
    for (int a = 0; a < A_N; ++a) {
        if (next_only && a != A_EX && a != A_EY) continue;
        for (int r = row_lo(a); r < row_hi<BY>(a); ++r) {
            const int j = g.y0 - 1 + r;
            if (j < 0 || j > g.ny) continue;
            if ((n++ & 31) != lane) continue;
            const float *src = g.src[a] + g.xs + (long long)g.pitch * j + g.plane * k;
            float *dst = st + (size_t)(row_off<BY>(a) + r - row_lo(a)) * kRowW + dx;
            bulk_g2s(dst, src, row_bytes, bar);
        }
    }
}

template <int BY>
__device__ __forceinline__ const float *row_ptr(const float *st, int a, int r)
{
    return st + (size_t)(row_off<BY>(a) + r - row_lo(a)) * kRowW;
}

}  // namespace

template <int BY, int S>
__global__ void __launch_bounds__(32 * (BY + 1), 1)
k_yee_step_bulk(const InstDesc *__restrict__ insts, const int *__restrict__ tile0, int ninst, int s_off,
                int total_tiles, int *err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    float *stages = reinterpret_cast<float *>(smem);
    float4 *xchg = reinterpret_cast<float4 *>(smem + S * stage_bytes<BY>());   // [2 buf][2 arr][BY+1][32]
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * stage_bytes<BY>() + xchg_bytes<BY>());

    const int lane = threadIdx.x, ty = threadIdx.y;
    if (ty == 0 && lane == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    unsigned gbase = 0;     // planes loaded by this CTA before the current tile
    bool failed = false;

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
        float *__restrict__ oHx = D->buf[par ^ 1][0];
        float *__restrict__ oHy = D->buf[par ^ 1][1];
        float *__restrict__ oHz = D->buf[par ^ 1][2];
        float *__restrict__ oEx = D->buf[par ^ 1][3];
        float *__restrict__ oEy = D->buf[par ^ 1][4];
        float *__restrict__ oEz = D->buf[par ^ 1][5];
        const long long src = D->src;
        const float srcv = (src >= 0 && step < D->nwave) ? __ldg(D->wave + step) : 0.f;

        int r0 = lt;
        const int xt = r0 % D->tiles_x; r0 /= D->tiles_x;
        const int yt = r0 % D->tiles_y;
        const int zt = r0 / D->tiles_y;
        TileGeom g;
        for (int f = 0; f < 6; ++f) g.src[f] = D->buf[par][f];
        for (int c = 0; c < 4; ++c) g.src[6 + c] = D->coef[c];
        g.plane = plane;
        g.pitch = pitch;
        g.ny = ny;
        g.x0 = xt * 128;
        g.y0 = yt * BY;
        g.xs = max(g.x0 - 4, 0);
        g.xe = min(g.x0 + 132, pitch);
        const int x0 = g.x0, y0 = g.y0;
        const int k0 = zt * kc, k1 = min(k0 + kc, nz);
        const int kstart = k0 > 0 ? k0 - 1 : k0;
        const int nplanes = k1 - kstart + 1;   // planes kstart..k1 (k1 is read as "next" only)

        // prologue: the first S planes
        if (ty == 0) {
            for (int q = 0; q < S && q < nplanes; ++q) {
                const unsigned G = gbase + q;
                issue_plane<BY>(g, kstart + q, kstart + q == k1, stages + (size_t)(G % S) * (stage_bytes<BY>() / 4),
                                &bars[G % S], lane);
            }
        }

        const int i = x0 + 4 * lane;
        const int r = ty;                 // frame row of this thread
        const int j = y0 + ty - 1;
        const bool halo = (ty == 0);
        const bool xin = (i <= nx);
        const bool jrow = (j >= 0 && j < ny);
        const int nout = min(4, nx - i);
        const bool hcol = (!halo) && (lane == 0) && (x0 > 0) && jrow;
        const int xl = 4 + 4 * lane;      // local x of this thread's first cell in a staged row
        long long off = (long long)i + (long long)pitch * (j < 0 ? 0 : j) + plane * kstart;

        float4 hxp = make_float4(0, 0, 0, 0), hyp = make_float4(0, 0, 0, 0);

        for (int k = kstart; k < k1; ++k, off += plane) {
            const int q = k - kstart;
            const unsigned Gc = gbase + q, Gn = Gc + 1;
            const float *cur = stages + (size_t)(Gc % S) * (stage_bytes<BY>() / 4);
            const float *nxt = stages + (size_t)(Gn % S) * (stage_bytes<BY>() / 4);
            if (!failed) {
                bool ok = mbar_wait(&bars[Gc % S], (Gc / S) & 1);
                ok = ok && mbar_wait(&bars[Gn % S], (Gn / S) & 1);
                if (!ok) {
                    failed = true;
                    atomicOr(err, 1);
                }
            }
            const bool warm = (k < k0);
            float4 hx = make_float4(0, 0, 0, 0), hy = hx, hz = hx, ez = hx, ex0 = hx, ey0 = hx, ex1 = hx, ey1 = hx;
            float4 exj1 = hx, ezj1 = hx, da = hx, db = hx;
            float ez_l = 0.f, ey_l = 0.f;
            const bool act = xin && (halo ? (jrow && !warm) : jrow);
            if (act) {
                hx = ld4s(row_ptr<BY>(cur, A_HX, r) + xl);
                ez = ld4s(row_ptr<BY>(cur, A_EZ, r) + xl);
                ex0 = ld4s(row_ptr<BY>(cur, A_EX, r) + xl);
                ey0 = ld4s(row_ptr<BY>(cur, A_EY, r) + xl);
                ey1 = ld4s(row_ptr<BY>(nxt, A_EY, r) + xl);
                exj1 = ld4s(row_ptr<BY>(cur, A_EX, r + 1) + xl);
                ezj1 = ld4s(row_ptr<BY>(cur, A_EZ, r + 1) + xl);
                da = ld4s(row_ptr<BY>(cur, A_DA, r) + xl);
                db = ld4s(row_ptr<BY>(cur, A_DB, r) + xl);
                hz = ld4s(row_ptr<BY>(cur, A_HZ, r) + xl);
                if (!halo) {
                    hy = ld4s(row_ptr<BY>(cur, A_HY, r) + xl);
                    ex1 = ld4s(row_ptr<BY>(nxt, A_EX, r) + xl);
                }
                if (lane == 31) {
                    ez_l = row_ptr<BY>(cur, A_EZ, r)[xl + 4];
                    ey_l = row_ptr<BY>(cur, A_EY, r)[xl + 4];
                }
            }
            // x+1 neighbours
            float ez_n = __shfl_down_sync(0xffffffffu, ez.x, 1);
            float ey_n = __shfl_down_sync(0xffffffffu, ey0.x, 1);
            if (lane == 31) { ez_n = ez_l; ey_n = ey_l; }
            const float ezv[4] = {ez.x, ez.y, ez.z, ez.w}, eyv[4] = {ey0.x, ey0.y, ey0.z, ey0.w};
            const float ez_ip[4] = {ez.y, ez.z, ez.w, ez_n}, ey_ip[4] = {ey0.y, ey0.z, ey0.w, ey_n};
            const float hxv[4] = {hx.x, hx.y, hx.z, hx.w}, hyv[4] = {hy.x, hy.y, hy.z, hy.w};
            const float hzv[4] = {hz.x, hz.y, hz.z, hz.w};
            const float ex0v[4] = {ex0.x, ex0.y, ex0.z, ex0.w}, ex1v[4] = {ex1.x, ex1.y, ex1.z, ex1.w};
            const float ey1v[4] = {ey1.x, ey1.y, ey1.z, ey1.w};
            const float exjv[4] = {exj1.x, exj1.y, exj1.z, exj1.w}, ezjv[4] = {ezj1.x, ezj1.y, ezj1.z, ezj1.w};
            const float dav[4] = {da.x, da.y, da.z, da.w}, dbv[4] = {db.x, db.y, db.z, db.w};
            float hxn[4], hyn[4], hzn[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                hxn[e] = yee_b(dav[e], hxv[e], dbv[e], ey1v[e], eyv[e], cz, ezjv[e], ezv[e], cy);
                hyn[e] = yee_b(dav[e], hyv[e], dbv[e], ez_ip[e], ezv[e], cx, ex1v[e], ex0v[e], cz);
                hzn[e] = yee_b(dav[e], hzv[e], dbv[e], exjv[e], ex0v[e], cy, ey_ip[e], eyv[e], cx);
            }
            float hyh = 0.f, hzh = 0.f;   // halo column x0-1
            if (hcol && !warm) {
                const float *Hy = row_ptr<BY>(cur, A_HY, r), *Hz = row_ptr<BY>(cur, A_HZ, r);
                const float *Ez = row_ptr<BY>(cur, A_EZ, r), *Ex = row_ptr<BY>(cur, A_EX, r);
                const float *Exn = row_ptr<BY>(nxt, A_EX, r), *Exj = row_ptr<BY>(cur, A_EX, r + 1);
                const float *Ey = row_ptr<BY>(cur, A_EY, r), *Da = row_ptr<BY>(cur, A_DA, r);
                const float *Db = row_ptr<BY>(cur, A_DB, r);
                hyh = yee_b(Da[3], Hy[3], Db[3], ez.x, Ez[3], cx, Exn[3], Ex[3], cz);
                hzh = yee_b(Da[3], Hz[3], Db[3], Exj[3], Ex[3], cy, ey0.x, Ey[3], cx);
            }
            float4 *sH = xchg + (size_t)(q & 1) * 2 * (BY + 1) * 32;   // [arr][row][lane]
            if (!warm) {
                sH[ty * 32 + lane] = make_float4(hxn[0], hxn[1], hxn[2], hxn[3]);
                sH[(BY + 1) * 32 + ty * 32 + lane] = make_float4(hzn[0], hzn[1], hzn[2], hzn[3]);
            }
            __syncthreads();
            // every reader of the stage of plane k-1 has passed the barrier: refill it
            if (ty == 0 && q >= 1 && q - 1 + S < nplanes) {
                const unsigned G = gbase + q - 1 + S;
                issue_plane<BY>(g, kstart + q - 1 + S, kstart + q - 1 + S == k1,
                                stages + (size_t)(G % S) * (stage_bytes<BY>() / 4), &bars[G % S], lane);
            }
            float hy_p = __shfl_up_sync(0xffffffffu, hyn[3], 1);
            float hz_p = __shfl_up_sync(0xffffffffu, hzn[3], 1);
            if (lane == 0) { hy_p = hyh; hz_p = hzh; }
            if (!halo && jrow && xin) {
                if (!warm) {
                    const float4 hxj4 = sH[(ty - 1) * 32 + lane];
                    const float4 hzj4 = sH[(BY + 1) * 32 + (ty - 1) * 32 + lane];
                    const float hxj[4] = {hxj4.x, hxj4.y, hxj4.z, hxj4.w}, hzj[4] = {hzj4.x, hzj4.y, hzj4.z, hzj4.w};
                    const float4 ca4 = ld4s(row_ptr<BY>(cur, A_CA, r) + xl), cb4 = ld4s(row_ptr<BY>(cur, A_CB, r) + xl);
                    const float cav[4] = {ca4.x, ca4.y, ca4.z, ca4.w}, cbv[4] = {cb4.x, cb4.y, cb4.z, cb4.w};
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
        gbase += (unsigned)nplanes;
        // The last plane's stage buffers are refilled by the next tile only after its first
        // barrier, which every thread reaches after finishing this tile.
        __syncthreads();
    }
    // Every issued plane has normally been waited for.  If a wait expired, let the copies still
    // in flight land (bounded) before this CTA's shared memory is released.
    if (ty == 0 && lane == 0)
        for (unsigned G = gbase > (unsigned)S ? gbase - S : 0u; G < gbase; ++G) mbar_wait(&bars[G % S], (G / S) & 1);
}

template <int BY, int S>
static int launch_bulk(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                       int grid, int *err, cudaStream_t s)
{
    static bool attr_set = false;
    const size_t smem = smem_bytes<BY, S>();
    if (!attr_set) {
        PTK_CUDA_TRY(cudaFuncSetAttribute(k_yee_step_bulk<BY, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        attr_set = true;
    }
    const int g = (grid <= 0 || grid > total_tiles) ? total_tiles : grid;
    k_yee_step_bulk<BY, S><<<g, dim3(32, BY + 1), smem, s>>>(d_insts, d_tile0, ninst, s_offset, total_tiles, err);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

// Rings of at least 3 stages: plane q waits for the stage of plane q+1 before its barrier, and a
// stage is refilled only after the barrier of the plane that follows its last reader, so the stage
// of plane q+1 must have been issued no later than plane q-1 (q+1-S+1 <= q-1).
int launch_yee_step_bulk(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                         int by, int stages, int grid, int *err, cudaStream_t s)
{
    if (total_tiles <= 0) return PTK_OK;
#define PTK_BULK(B, S)                                                                                  \
    if (by == B && stages == S)                                                                         \
        return launch_bulk<B, S>(d_insts, d_tile0, ninst, total_tiles, s_offset, grid, err, s);
    PTK_BULK(4, 3) PTK_BULK(4, 4) PTK_BULK(4, 5)
    PTK_BULK(8, 3) PTK_BULK(8, 4)
#undef PTK_BULK
    return set_error(PTK_ERR_INVALID, "no staged kernel for %d rows x %d stages", by, stages);
}

size_t yee_bulk_smem_bytes(int by, int stages)
{
#define PTK_SM(B, S) \
    if (by == B && stages == S) return smem_bytes<B, S>();
    PTK_SM(4, 3) PTK_SM(4, 4) PTK_SM(4, 5)
    PTK_SM(8, 3) PTK_SM(8, 4)
#undef PTK_SM
    return 0;
}

}  // namespace ptk
