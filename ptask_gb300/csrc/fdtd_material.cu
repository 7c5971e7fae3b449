// fdtd_material.cu -- per-node material index of an instance's coefficient arrays.
//
// FDTD problems are built from a few materials, so the four per-cell coefficient arrays (Ca, Cb,
// Da, Db: 16 bytes per node) hold few distinct tuples.  The staged step kernel can read a one-byte
// material id per node and the tuple from a table instead (49 bytes of traffic per cell update
// instead of 64).  This file finds the distinct tuples on the device:
//
//   1. k_mat_insert: every node's tuple (compared bit for bit) goes into an open-addressing hash
//      table of kSlots slots; lanes of a warp holding the same tuple insert it once.  A slot is
//      claimed with atomicCAS, filled, then published; readers of a claimed slot wait for the
//      publication with a bounded poll (on expiry an error word is raised and the index is not
//      used).
//   2. k_mat_compact: one thread numbers the occupied slots in slot order and writes the table.
//   3. k_mat_index: every node looks its tuple up and stores the id.
//
// More than kMaxMaterials distinct tuples (or a raised error word) leaves the index unused: the
// caller keeps the per-cell arrays.  The values in the table are the arrays' own bits, so results
// are identical either way.
#include "ptk_internal.h"

namespace ptk {

namespace {

constexpr int kSlots = 1024;
constexpr int kPollLimit = 1 << 20;

struct MatScratch {
    unsigned state[kSlots];   // 0 empty, 1 being filled, 2 published
    uint4 key[kSlots];
    int id[kSlots];
    int count;                // distinct tuples inserted
    int err;                  // 1: a poll expired, 2: the table filled up
    int nmat;                 // result: number of materials, 0 = index unusable
};

__device__ __forceinline__ unsigned mix(uint4 k)
{
    unsigned h = k.x * 0x9E3779B1u;
    h = (h ^ k.y) * 0x85EBCA77u;
    h = (h ^ k.z) * 0xC2B2AE3Du;
    h = (h ^ k.w) * 0x27D4EB2Fu;
    return h ^ (h >> 15);
}

__device__ __forceinline__ uint4 tuple_at(const float *const *c, long long o)
{
    return make_uint4(__float_as_uint(__ldg(c[0] + o)), __float_as_uint(__ldg(c[1] + o)),
                      __float_as_uint(__ldg(c[2] + o)), __float_as_uint(__ldg(c[3] + o)));
}

__device__ __forceinline__ bool same(uint4 a, uint4 b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

__device__ uint4 read_key(const MatScratch *S, int h)
{
    const volatile unsigned *k = reinterpret_cast<const volatile unsigned *>(&S->key[h]);
    return make_uint4(k[0], k[1], k[2], k[3]);
}

__device__ void insert(MatScratch *S, uint4 key)
{
    unsigned h = mix(key) & (kSlots - 1);
    for (int probe = 0; probe < kSlots; ++probe, h = (h + 1) & (kSlots - 1)) {
        // Most nodes repeat a tuple that is already published: check with a plain read first, so
        // that only new tuples contend for a slot with an atomic.
        if (reinterpret_cast<volatile unsigned *>(S->state)[h] == 2u) {
            __threadfence();
            if (same(read_key(S, h), key)) return;
            continue;
        }
        const unsigned st = atomicCAS(&S->state[h], 0u, 1u);
        if (st == 0u) {
            S->key[h] = key;
            __threadfence();
            atomicExch(&S->state[h], 2u);
            atomicAdd(&S->count, 1);
            return;
        }
        int it = 0;
        while (reinterpret_cast<volatile unsigned *>(S->state)[h] != 2u && ++it < kPollLimit) {
        }
        if (it >= kPollLimit) {
            atomicOr(&S->err, 1);
            return;
        }
        __threadfence();
        if (same(read_key(S, h), key)) return;
    }
    atomicOr(&S->err, 2);
}

// Node q of the (nx+1) x (ny+1) x (nz+1) node grid (row padding is not part of the problem).
struct Nodes {
    int nx, ny, pitch;
    long long plane, n;
    __device__ long long offset(long long q) const
    {
        const int i = (int)(q % (nx + 1));
        q /= nx + 1;
        const int j = (int)(q % (ny + 1));
        return i + (long long)pitch * j + plane * (q / (ny + 1));
    }
};

__global__ void k_mat_insert(const float *Ca, const float *Cb, const float *Da, const float *Db, Nodes N,
                             MatScratch *S)
{
    const float *c[4] = {Ca, Cb, Da, Db};
    const long long stride = (long long)gridDim.x * blockDim.x;
    uint4 last = make_uint4(0, 0, 0, 0);   // the tuple this thread inserted last (already in the table)
    bool have_last = false;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < N.n; q += stride) {
        const uint4 key = tuple_at(c, N.offset(q));
        // lanes with the same tuple (all four words equal) let their lowest lane insert it
        const unsigned act = __activemask();
        const unsigned m = __match_any_sync(act, key.x) & __match_any_sync(act, key.y) &
                           __match_any_sync(act, key.z) & __match_any_sync(act, key.w);
        if ((threadIdx.x & 31) == __ffs(m) - 1 && !(have_last && same(key, last))) {
            insert(S, key);
            last = key;
            have_last = true;
        }
    }
}

__global__ void k_mat_compact(MatScratch *S, float4 *tab)
{
    int n = 0;
    for (int h = 0; h < kSlots; ++h) {
        if (S->state[h] != 2u) continue;
        if (n < kMaxMaterials) {
            const uint4 k = S->key[h];
            tab[n] = make_float4(__uint_as_float(k.x), __uint_as_float(k.y), __uint_as_float(k.z), __uint_as_float(k.w));
        }
        S->id[h] = n++;
    }
    S->nmat = (S->err || n > kMaxMaterials || n != S->count) ? 0 : n;
}

__global__ void k_mat_index(const float *Ca, const float *Cb, const float *Da, const float *Db, Nodes N,
                            const MatScratch *S, unsigned char *mat)
{
    if (S->nmat == 0) return;
    const float *c[4] = {Ca, Cb, Da, Db};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < N.n; q += stride) {
        const long long o = N.offset(q);
        const uint4 key = tuple_at(c, o);
        unsigned h = mix(key) & (kSlots - 1);
        for (int probe = 0; probe < kSlots; ++probe, h = (h + 1) & (kSlots - 1))
            if (S->state[h] == 2u && same(S->key[h], key)) {
                mat[o] = (unsigned char)S->id[h];
                break;
            }
    }
}

}  // namespace

int build_material_index(const float *const coef[4], const Layout &L, unsigned char *mat, float *tab, int *nmat,
                         cudaStream_t s)
{
    PTK_CHECK_ARG(coef && mat && tab && nmat, "NULL argument");
    *nmat = 0;
    MatScratch *S = nullptr;
    int rc = pool_alloc(sizeof(MatScratch), s, (void **)&S);
    if (rc) return rc;
    PTK_CUDA_TRY(cudaMemsetAsync(S, 0, sizeof(MatScratch), s));
    Nodes N{L.nx, L.ny, L.pitch, L.plane, (long long)(L.nx + 1) * (L.ny + 1) * (L.nz + 1)};
    const int grid = (int)std::min<long long>((N.n + 255) / 256, 8LL * std::max(1, sm_count()));
    k_mat_insert<<<grid, 256, 0, s>>>(coef[0], coef[1], coef[2], coef[3], N, S);
    k_mat_compact<<<1, 1, 0, s>>>(S, reinterpret_cast<float4 *>(tab));
    k_mat_index<<<grid, 256, 0, s>>>(coef[0], coef[1], coef[2], coef[3], N, S, mat);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(3);
    int h = 0;
    PTK_CUDA_TRY(cudaMemcpyAsync(&h, &S->nmat, sizeof(int), cudaMemcpyDeviceToHost, s));
    PTK_CUDA_TRY(cudaStreamSynchronize(s));
    pool_free(S, s);
    *nmat = h;
    return PTK_OK;
}

}  // namespace ptk
