// fdtd_batch.cu -- batched and served FDTD: many device-resident instances of uneven size advanced
// together by the fused step kernel, with continuous admission by HBM budget.
//
// One time step of every active instance is ONE launch of the step kernel (the TMA-staged
// k_yee_step_bulk with a material index by default, the register kernel k_yee_step on request) over
// the concatenated tile lists of all instances: a persistent grid of resident CTAs takes tiles from
// a counter.  Chunks of steps are replayed as captured CUDA graphs (at most kMaxGraphs kept).
// Instances finish at their own step counts: their tiles go idle inside the chunk in which they
// finish and they leave the batch at the chunk boundary, where newly arrived requests are admitted
// if they fit the HBM budget.  Request problems are generated on the device (coefficients and the
// material index from the seeded box list), so admission moves only the waveform and the tensor
// maps over the host link.
//
// The host keeps one chunk queued ahead: while chunk i runs it admits, rebuilds the work list into
// the other half of a double-buffered pinned staging area and launches chunk i+1, with chunk i's
// finishers retired (fixed-order FP64 checksums, frees) in stream order between them; only then
// does it wait for chunk i.  Each instance's arrays are one device block; an admission that fits
// the budget but finds no free block waits for retirements instead of failing.
//
// The reference has no batching: it pipelines numBlocks copies of one problem through one graph
// (graphfdtd.cpp:1076-1097) and dispatches every task of every copy separately.
#include "ptk_internal.h"
#include "ptk_problem.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

namespace ptk {

constexpr int kMaxBoxes = 64;

struct BoxArgs {
    int n;
    int lo[kMaxBoxes][3];
    int hi[kMaxBoxes][3];
    float epsr[kMaxBoxes];
};

// Padded coefficients of a generated problem: the device twin of ptk_problem_generate (same boxes,
// same FP32 expressions Cb = Dt/(eps0*eps_r), Db = Dt/mu0; wall nodes take the nearest cell).  With
// `mat`, also the material index: 0 for vacuum, b + 1 inside box b (the last box listed wins).
__global__ void k_generate_coefs(BoxArgs boxes, int nx, int ny, int nz, int pitch, long long plane, float dt,
                                 float eps0, float mu0, float *Ca, float *Cb, float *Da, float *Db,
                                 unsigned char *mat)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i > nx) return;
    const int ci = min(i, nx - 1), cj = min(j, ny - 1), ck = min(k, nz - 1);
    float e = 1.0f;
    int id = 0;
    for (int b = boxes.n - 1; b >= 0; --b)
        if (ci >= boxes.lo[b][0] && ci < boxes.hi[b][0] && cj >= boxes.lo[b][1] && cj < boxes.hi[b][1] &&
            ck >= boxes.lo[b][2] && ck < boxes.hi[b][2]) {
            e = boxes.epsr[b];
            id = b + 1;
            break;
        }
    const long long o = i + (long long)pitch * j + plane * k;
    Ca[o] = 1.0f;
    Cb[o] = __fdiv_rn(dt, __fmul_rn(eps0, e));
    Da[o] = 1.0f;
    Db[o] = __fdiv_rn(dt, mu0);
    if (mat) mat[o] = (unsigned char)id;
}

// The material table of a generated problem: entry 0 vacuum, entry b + 1 box b, with the
// coefficient expressions of k_generate_coefs.
__global__ void k_generate_table(BoxArgs boxes, float dt, float eps0, float mu0, float4 *tab)
{
    const int t = threadIdx.x;
    if (t > boxes.n) return;
    const float e = t == 0 ? 1.0f : boxes.epsr[t - 1];
    tab[t] = make_float4(1.0f, __fdiv_rn(dt, __fmul_rn(eps0, e)), 1.0f, __fdiv_rn(dt, mu0));
}

// Sum of each valid field element (FP64; order of accumulation not fixed, for reporting only).
// FP64 sums of an instance's six result fields in two launches with a fixed summation order (the
// same request gives the same checksum bits every time): blocks sum strided rows into partials,
// then one warp per field adds the partials.
constexpr int kSumBlocks = 96;   // partial sums per field
struct SumArgs {
    const float *f[6];
    int ex[6], ey[6], ez[6];
    int pitch;
    long long plane;
};

__global__ void __launch_bounds__(256) k_checksum_partial(SumArgs a, double *__restrict__ part)
{
    __shared__ double warp_sum[8];
    const int f = blockIdx.y;
    const int ex = a.ex[f], ey = a.ey[f], rows = a.ey[f] * a.ez[f];
    const float *__restrict__ p = a.f[f];
    double v = 0.0;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const float *__restrict__ row = p + (long long)a.pitch * (r % ey) + a.plane * (r / ey);
        for (int i = threadIdx.x; i < ex; i += blockDim.x) v += (double)row[i];
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < 8; ++w) b += warp_sum[w];
        part[f * gridDim.x + blockIdx.x] = b;
    }
}

__global__ void k_checksum_final(const double *__restrict__ part, int nb, double *__restrict__ out)
{
    const int f = threadIdx.y, lane = threadIdx.x;
    double v = 0.0;
    for (int b = lane; b < nb; b += 32) v += part[f * nb + b];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[f] = v;
}

struct Inst {
    long long ticket = -1;
    ptk_problem_desc desc{};
    ptk_fdtd_params p{};
    Layout L{};
    float *buf[2][6] = {};
    float *coef[4] = {};
    float *wave = nullptr;
    void *tma = nullptr;        // tensor maps of the staged kernel
    unsigned char *mat = nullptr;   // material index (staged kernel)
    float *mat_tab = nullptr;
    int nmat = 0;
    int nwave = 0;
    long long src = -1;
    int steps_total = 0, done = 0;
    size_t bytes = 0;
    double t_arrival = 0, t_admit = -1, t_finish = -1;
    double t_arrival_run = 0;   // arrival on the run's clock (scaled trace time)
    double *d_sum = nullptr;
    double checksum[6] = {};
    std::vector<float> result[6];
    bool finished = false;
    void *block = nullptr;      // the one device allocation holding all of the above arrays
};

// An instance's arrays live in one device allocation (few, large blocks keep the pool's free space
// usable when thousands of requests of different sizes come and go): byte offsets, each array
// 256-byte aligned.
struct InstBlock {
    size_t field[2][6], coef[4], mat, sum, tma, tab, wave, total;
};

InstBlock block_layout(const Layout &L, int nwave)
{
    InstBlock b{};
    size_t o = 0;
    auto take = [&o](size_t bytes) {
        const size_t at = o;
        o += (bytes + 255) / 256 * 256;
        return at;
    };
    const size_t a = (size_t)L.total * sizeof(float);
    for (int p = 0; p < 2; ++p)
        for (int f = 0; f < 6; ++f) b.field[p][f] = take(a);
    for (int c = 0; c < 4; ++c) b.coef[c] = take(a);
    b.mat = take((size_t)L.total);
    b.sum = take(6 * sizeof(double));
    b.tma = take(kTmaSetBytes);
    b.tab = take((size_t)kMaxMaterials * 4 * sizeof(float));
    b.wave = take((size_t)std::max(nwave, 1) * sizeof(float));
    b.total = o;
    return b;
}

size_t instance_bytes(const Layout &L, int nwave) { return block_layout(L, nwave).total; }

}  // namespace ptk

using namespace ptk;

struct ptk_server {
    ptk_server_config cfg{};
    cudaStream_t st = nullptr;
    std::vector<Inst *> all;        // every submitted request, by ticket
    std::vector<Inst *> active;     // admitted, running
    size_t used = 0, peak_bytes = 0;
    int peak_active = 0;
    // device work list; its pinned host staging is double-buffered by `par` (below)
    InstDesc *d_desc = nullptr;
    int *d_tile0 = nullptr;
    InstDesc *h_desc[2] = {};
    int *h_tile0[2] = {};
    long long *d_face0 = nullptr;   // staged kernel: prefix sums of the instances' face nodes
    long long *h_face0[2] = {};
    long long total_faces = 0;
    int cap = 0;
    int total_tiles = 0;
    int vec = 4;                    // x cells per thread of the current work list
    int rows = 8, stages = 4;       // step kernel: tile rows; staged ring planes (0 = register kernel)
    int *d_err = nullptr;           // raised by the staged kernel if a bounded wait expires
    int *d_work = nullptr;          // staged kernel's tile counters, one per step of a chunk
    int depth_cap = 0;              // staged kernel: deepest z chunk of the current work list
    int resident = 1;               // CTAs of the step kernel that fit on the GPU at once
    double *d_part = nullptr;       // checksum partials (6 x kSumBlocks)
    // Pipelining: a chunk is queued while the previous one runs.  Chunk slot b (= `par` when it was
    // launched) owns the pinned error-word copy, the checksum landing slots of its finishers and its
    // events; the host staging of parity b (work list, admission uploads) is reused two chunks later.
    int par = 0;
    int *h_err = nullptr;           // pinned, two slots
    double *h_sums[2] = {};
    int sums_cap[2] = {};
    unsigned char *h_up[2] = {};    // pinned admission uploads (tensor maps, waveforms)
    size_t up_used[2] = {};
    struct Flight {
        bool on = false;
        std::vector<Inst *> gone;   // instances that finish with this chunk (retired behind it)
        cudaGraphExec_t exec = nullptr;   // the chunk graph it replays
    } flight[2];
    bool dirty = true;
    bool admit_blocked = false;     // the pool could not place a request: wait for retirements
    std::map<std::tuple<int, int, int, int, long long>, cudaGraphExec_t> graphs;
    long long chunks = 0, launches = 0, captures = 0, admit_waits = 0;
    double wall_s = 0, cell_updates = 0;
    double chunk_dev_s = 0, admit_s = 0, retire_s = 0, sched_s = 0;   // where wall_s went
    cudaEvent_t ev_start[2] = {}, ev_end[2] = {};   // around each chunk replay, per slot
    cudaEvent_t ev_ret[2] = {};                      // after the slot's retirement copies
    std::mutex mu;
};

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int grow_worklist(ptk_server *s, int n)
{
    if (n <= s->cap) return PTK_OK;
    int cap = std::max(n, 2 * s->cap);
    if (s->d_desc) {
        cudaStreamSynchronize(s->st);   // queued chunks read the old lists and staging
        pool_free(s->d_desc, s->st);
        pool_free(s->d_tile0, s->st);
        pool_free(s->d_face0, s->st);
        for (int b = 0; b < 2; ++b) {
            cudaFreeHost(s->h_desc[b]);
            cudaFreeHost(s->h_tile0[b]);
            cudaFreeHost(s->h_face0[b]);
            s->h_desc[b] = nullptr;
            s->h_tile0[b] = nullptr;
            s->h_face0[b] = nullptr;
        }
    }
    int rc = pool_alloc(sizeof(InstDesc) * cap, s->st, (void **)&s->d_desc);
    if (!rc) rc = pool_alloc(sizeof(int) * (cap + 1), s->st, (void **)&s->d_tile0);
    if (!rc) rc = pool_alloc(sizeof(long long) * (cap + 1), s->st, (void **)&s->d_face0);
    if (rc) return rc;
    for (int b = 0; b < 2; ++b) {
        PTK_CUDA_TRY(cudaMallocHost(&s->h_desc[b], sizeof(InstDesc) * cap));
        PTK_CUDA_TRY(cudaMallocHost(&s->h_tile0[b], sizeof(int) * (cap + 1)));
        PTK_CUDA_TRY(cudaMallocHost(&s->h_face0[b], sizeof(long long) * (cap + 1)));
    }
    s->cap = cap;
    for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
    return PTK_OK;
}

// Tile depth (0 = whole) of an instance nz planes deep under a cap: near-equal chunks of at most
// `cap` planes.  The register kernel keeps the short chunks it was tuned with.
int depth_for_cap(int nz, int cap)
{
    if (nz <= cap) return 0;
    const int parts = (nz + cap - 1) / cap;
    return (nz + parts - 1) / parts;
}

int instance_depth(const ptk_server *s, int nz)
{
    if (!s->stages) return nz > 48 ? 16 : 0;
    return depth_for_cap(nz, s->depth_cap);
}

// Deepest cap (planes per staged tile) that still gives the work list eight tiles per resident CTA:
// deep tiles pay the pipeline fill and the warm plane rarely, but one small instance alone needs
// shallow tiles to occupy the GPU, and a mix of instances balances its last wave better with more,
// shorter tiles (on the 64-instance mix eight per CTA beat four, sixteen and thirty-two).
int choose_depth_cap(const ptk_server *s)
{
    static const int caps[] = {192, 128, 96, 64, 48, 32, 24, 16, 12, 8};
    const long long want = 8LL * s->resident;
    for (int cap : caps) {
        long long tiles = 0;
        for (const Inst *in : s->active) {
            const int d = depth_for_cap(in->L.nz, cap);
            const int kc = d ? d : in->L.nz;
            tiles += (long long)((in->L.nx + 32 * s->vec - 1) / (32 * s->vec)) * ((in->L.ny + s->rows - 1) / s->rows) *
                     ((in->L.nz + kc - 1) / kc);
        }
        if (tiles >= want) return cap;
    }
    return 8;
}

InstDesc instance_desc(const ptk_server *s, const Inst *in)
{
    InstDesc d{};
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 6; ++f) d.buf[b][f] = in->buf[b][f];
    for (int c = 0; c < 4; ++c) d.coef[c] = in->coef[c];
    d.wave = in->wave;
    d.plane = in->L.plane;
    d.nx = in->L.nx; d.ny = in->L.ny; d.nz = in->L.nz; d.pitch = in->L.pitch;
    d.cx = in->p.Cx; d.cy = in->p.Cy; d.cz = in->p.Cz;
    d.src = in->nwave ? in->src : -1;
    d.nwave = in->nwave;
    d.step = in->done;
    d.steps_left = in->steps_total - in->done;
    d.tma = in->tma;
    if (s->stages) {
        d.mat = in->mat;
        d.mat_tab = in->mat_tab;
        d.nmat = in->nmat;
    }
    plan_tiles(d, s->rows, instance_depth(s, in->L.nz), s->vec);
    if (s->stages) d.face_tiles = 0;   // faces: launch_yee_faces_steps, once per chunk
    return d;
}

constexpr size_t kUpBytes = 4u << 20;   // each half of the pinned admission-upload arena

// Host-to-device copy through the pinned upload arena of parity `par`, so that it is queued without
// waiting for the chunks ahead of it.  A half is reused two chunks later, when the chunk that its
// copies preceded has completed.  Uploads larger than a half are copied after the queue drains.
int stage_upload(ptk_server *s, void *dst, const void *src, size_t bytes)
{
    const size_t need = (bytes + 63) & ~(size_t)63;
    if (need > kUpBytes) {
        PTK_CUDA_TRY(cudaStreamSynchronize(s->st));
        PTK_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
        return PTK_OK;
    }
    if (!s->h_up[0]) {
        for (int b = 0; b < 2; ++b) PTK_CUDA_TRY(cudaMallocHost(&s->h_up[b], kUpBytes));
    }
    size_t &used = s->up_used[s->par];
    if (used + need > kUpBytes) {   // full: let every queued copy from either half run
        PTK_CUDA_TRY(cudaStreamSynchronize(s->st));
        s->up_used[0] = s->up_used[1] = 0;
    }
    unsigned char *p = s->h_up[s->par] + used;
    memcpy(p, src, bytes);
    used += need;
    PTK_CUDA_TRY(cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, s->st));
    return PTK_OK;
}

int admit(ptk_server *s, Inst *in)
{
    std::vector<BoxSpec> boxes;
    std::vector<float> wave;
    int si, sj, sk;
    int rc = problem_plan(&in->desc, &in->p, &boxes, &si, &sj, &sk, &wave);
    if (rc) return set_error(rc, "bad request descriptor");
    if ((int)boxes.size() > kMaxBoxes) return set_error(PTK_ERR_INVALID, "at most %d boxes per request", kMaxBoxes);
    in->L = make_layout(in->p.Nx, in->p.Ny, in->p.Nz);
    in->steps_total = in->desc.steps;
    const size_t bytes = (size_t)in->L.total * sizeof(float);
    cudaStream_t st = s->st;
    in->nwave = (si >= 0 && !wave.empty()) ? (int)wave.size() : 0;
    // One allocation, the first device operation: if it fails nothing needs undoing.
    const InstBlock lay = block_layout(in->L, in->nwave);
    rc = pool_alloc(lay.total, st, &in->block);
    if (rc) return rc;
    char *base = static_cast<char *>(in->block);
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 6; ++f) in->buf[b][f] = reinterpret_cast<float *>(base + lay.field[b][f]);
    for (int c = 0; c < 4; ++c) in->coef[c] = reinterpret_cast<float *>(base + lay.coef[c]);
    in->d_sum = reinterpret_cast<double *>(base + lay.sum);
    if (s->stages) {
        in->tma = base + lay.tma;
        in->mat = reinterpret_cast<unsigned char *>(base + lay.mat);
        in->mat_tab = reinterpret_cast<float *>(base + lay.tab);
    }
    if (in->nwave) in->wave = reinterpret_cast<float *>(base + lay.wave);
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 6; ++f) PTK_CUDA_TRY(cudaMemsetAsync(in->buf[b][f], 0, bytes, st));
    if (in->mat) PTK_CUDA_TRY(cudaMemsetAsync(in->mat, 0, (size_t)in->L.total, st));
    BoxArgs ba{};
    ba.n = (int)boxes.size();
    for (int b = 0; b < ba.n; ++b) {
        for (int a = 0; a < 3; ++a) {
            ba.lo[b][a] = boxes[b].lo[a];
            ba.hi[b][a] = boxes[b].hi[a];
        }
        ba.epsr[b] = boxes[b].epsr;
    }
    dim3 grid((in->L.nx + 1 + 127) / 128, in->L.ny + 1, in->L.nz + 1);
    k_generate_coefs<<<grid, 128, 0, st>>>(ba, in->L.nx, in->L.ny, in->L.nz, in->L.pitch, in->L.plane, in->p.Dt,
                                           in->p.eps0, in->p.mu0, in->coef[0], in->coef[1], in->coef[2], in->coef[3],
                                           in->mat);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    if (in->mat) {
        k_generate_table<<<1, 128, 0, st>>>(ba, in->p.Dt, in->p.eps0, in->p.mu0, reinterpret_cast<float4 *>(in->mat_tab));
        PTK_CUDA_TRY(cudaGetLastError());
        count_launches(1);
        in->nmat = ba.n + 1;
    }
    if (in->nwave) {
        rc = stage_upload(s, in->wave, wave.data(), wave.size() * sizeof(float));
        if (rc) return rc;
        in->src = (long long)si + (long long)in->L.pitch * sj + in->L.plane * sk;
    }
    if (s->stages) {
        // The arrays never move while the instance lives: its tensor maps are encoded once.
        alignas(64) unsigned char maps[kTmaSetBytes];
        rc = encode_tma_set(instance_desc(s, in), s->rows, maps);
        if (rc) return rc;
        rc = stage_upload(s, in->tma, maps, kTmaSetBytes);
        if (rc) return rc;
    }
    in->bytes = instance_bytes(in->L, in->nwave);
    s->used += in->bytes;
    s->peak_bytes = std::max(s->peak_bytes, s->used);
    s->active.push_back(in);
    s->peak_active = std::max(s->peak_active, (int)s->active.size());
    s->dirty = true;
    return PTK_OK;
}

void release(ptk_server *s, Inst *in)
{
    pool_free(in->block, s->st);
    in->block = nullptr;
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 6; ++f) in->buf[b][f] = nullptr;
    for (int c = 0; c < 4; ++c) in->coef[c] = nullptr;
    in->wave = nullptr;
    in->d_sum = nullptr;
    in->tma = nullptr;
    in->mat = nullptr;
    in->mat_tab = nullptr;
    s->used -= in->bytes;
}

int rebuild_worklist(ptk_server *s)
{
    const int n = (int)s->active.size();
    int rc = grow_worklist(s, n);
    if (rc) return rc;
    // Staging of parity `par`: its last copies fed the chunk before the previous one, which has
    // completed (the run loop lands every chunk before launching the next-but-one).
    InstDesc *h_desc = s->h_desc[s->par];
    int *h_tile0 = s->h_tile0[s->par];
    long long *h_face0 = s->h_face0[s->par];
    // Register kernel: 128-wide tiles (4 cells per thread); narrower ones keep more lanes busy on
    // small grids but hold fewer bytes in flight per thread, and measured slower on the batched
    // workload.  The staged kernel's width goes with its rows (set at creation).
    if (!s->stages) s->vec = 4;
    if (s->stages) {
        s->depth_cap = choose_depth_cap(s);
        // longest tiles first, so that the dynamic tile queue ends with short ones
        std::stable_sort(s->active.begin(), s->active.end(), [s](const Inst *a, const Inst *b) {
            const int da = instance_depth(s, a->L.nz), db = instance_depth(s, b->L.nz);
            return (da ? da : a->L.nz) > (db ? db : b->L.nz);
        });
    }
    int tiles = 0;
    long long faces = 0;
    for (int q = 0; q < n; ++q) {
        const InstDesc d = instance_desc(s, s->active[q]);
        h_desc[q] = d;
        h_face0[q] = faces;
        faces += face_nodes(d.nx, d.ny, d.nz);
        h_tile0[q] = tiles;
        tiles += d.tiles_x * d.tiles_y * d.tiles_z + d.face_tiles;
    }
    h_tile0[n] = tiles;
    s->total_tiles = tiles;
    h_face0[n] = faces;
    s->total_faces = s->stages ? faces : 0;
    if (n) {   // queued behind the running chunk, which reads the old lists
        PTK_CUDA_TRY(cudaMemcpyAsync(s->d_desc, h_desc, sizeof(InstDesc) * n, cudaMemcpyHostToDevice, s->st));
        PTK_CUDA_TRY(cudaMemcpyAsync(s->d_tile0, h_tile0, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s->st));
        PTK_CUDA_TRY(cudaMemcpyAsync(s->d_face0, h_face0, sizeof(long long) * (n + 1), cudaMemcpyHostToDevice,
                                     s->st));
    }
    s->dirty = false;
    return PTK_OK;
}

constexpr size_t kMaxGraphs = 256;   // chunk graphs kept for reuse

int chunk_graph(ptk_server *s, int len, int grid, cudaGraphExec_t *out)
{
    const int n = (int)s->active.size();
    auto key = std::make_tuple(len, n, s->total_tiles, (grid * 8 + s->vec) * 8 + s->stages, s->total_faces);
    auto it = s->graphs.find(key);
    if (it != s->graphs.end()) {
        *out = it->second;
        return PTK_OK;
    }
    cudaStream_t cap;
    PTK_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    PTK_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    int rc = PTK_OK;
    if (s->stages && cudaMemsetAsync(s->d_work, 0, sizeof(int) * len, cap) != cudaSuccess)
        rc = set_error(PTK_ERR_CUDA, "chunk capture: counter reset failed");
    else if (s->stages)
        count_launches(1);
    if (!rc && s->stages) rc = launch_yee_faces_steps(s->d_desc, s->d_face0, n, s->total_faces, 0, len, cap);
    for (int q = 0; q < len && !rc; ++q)
        rc = s->stages ? launch_yee_step_bulk(s->d_desc, s->d_tile0, n, s->total_tiles, q, s->rows, s->stages, grid,
                                              s->d_err, cap, s->d_work, true)
                       : launch_yee_step_v(s->d_desc, s->d_tile0, n, s->total_tiles, q, s->rows, s->vec, grid, cap);
    if (!rc) rc = launch_advance(s->d_desc, n, len, cap);
    set_capturing(false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return set_error(PTK_ERR_CUDA, "chunk capture: %s", cudaGetErrorString(e));
    cudaGraphExec_t ex;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(PTK_ERR_CUDA, "chunk instantiate: %s", cudaGetErrorString(e));
    // Bounded cache: under a changing request mix most work lists never repeat.  Evict all but the
    // graph of the chunk that may still be queued or running (slot par ^ 1; slot par has landed).
    if (s->graphs.size() >= kMaxGraphs) {
        const cudaGraphExec_t busy = s->flight[s->par ^ 1].on ? s->flight[s->par ^ 1].exec : nullptr;
        for (auto it = s->graphs.begin(); it != s->graphs.end();) {
            if (it->second == busy) {
                ++it;
            } else {
                cudaGraphExecDestroy(it->second);
                it = s->graphs.erase(it);
            }
        }
    }
    s->graphs[key] = ex;
    ++s->captures;
    *out = ex;
    return PTK_OK;
}

// A finished instance's checksums (and, with keep_results, its result fields) are enqueued, and
// its arrays freed (also on failure), in stream order; the checksums land in the pinned slot
// h_slot, valid after the next synchronisation of the server's stream (retire_finish).
int retire_copies(ptk_server *s, Inst *in, double *h_slot)
{
    const int par = in->done & 1;
    SumArgs a{};
    for (int f = 0; f < 6; ++f) {
        a.f[f] = in->buf[par][f];
        field_extents(f, in->L.nx, in->L.ny, in->L.nz, &a.ex[f], &a.ey[f], &a.ez[f]);
    }
    a.pitch = in->L.pitch;
    a.plane = in->L.plane;
    k_checksum_partial<<<dim3(kSumBlocks, 6), 256, 0, s->st>>>(a, s->d_part);
    k_checksum_final<<<1, dim3(32, 6), 0, s->st>>>(s->d_part, kSumBlocks, in->d_sum);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(2);
    PTK_CUDA_TRY(cudaMemcpyAsync(h_slot, in->d_sum, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    if (s->cfg.keep_results) {
        for (int f = 0; f < 6; ++f) {
            in->result[f].resize((size_t)a.ex[f] * a.ey[f] * a.ez[f]);
            float *stage = nullptr;
            int rc = pool_alloc(in->result[f].size() * sizeof(float), s->st, (void **)&stage);
            if (rc) return rc;
            rc = launch_unpack_field(in->buf[par][f], a.ex[f], a.ey[f], a.ez[f], in->L, stage, s->st);
            if (rc) return rc;
            PTK_CUDA_TRY(cudaMemcpyAsync(in->result[f].data(), stage, in->result[f].size() * sizeof(float),
                                         cudaMemcpyDeviceToHost, s->st));
            pool_free(stage, s->st);
        }
    }
    return PTK_OK;
}

int retire_enqueue(ptk_server *s, Inst *in, double *h_slot)
{
    const int rc = retire_copies(s, in, h_slot);
    release(s, in);
    return rc;
}

// After the stream has been synchronised: the instance's checksums are in h_slot.
void retire_finish(ptk_server *s, Inst *in, const double *h_slot, double t)
{
    for (int f = 0; f < 6; ++f) in->checksum[f] = h_slot[f];
    in->t_finish = t;
    in->finished = true;
    s->cell_updates += (double)in->L.nx * in->L.ny * in->L.nz * in->steps_total;
}

}  // namespace

extern "C" {

int ptk_server_create(const ptk_server_config *cfg, ptk_server **out)
try {
    clear_error();
    PTK_CHECK_ARG(cfg && out, "NULL argument");
    int rc = ensure_init();
    if (rc) return rc;
    auto *s = new ptk_server();
    s->cfg = *cfg;
    if (s->cfg.max_active <= 0) s->cfg.max_active = 1 << 20;
    if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 32;
    // default rows: 11 for the staged kernel (twelve warps per CTA; measured best), 8 otherwise
    if (s->cfg.tile_rows == 0) s->cfg.tile_rows = s->cfg.stages >= 0 ? 11 : 8;
    const bool staged_rows = s->cfg.stages >= 0 && (s->cfg.tile_rows == 7 || s->cfg.tile_rows == 10 ||
                                                    s->cfg.tile_rows == 11 || s->cfg.tile_rows == 23);
    if (s->cfg.tile_rows != 4 && s->cfg.tile_rows != 8 && s->cfg.tile_rows != 16 && !staged_rows) s->cfg.tile_rows = 8;
    s->rows = s->cfg.tile_rows;
    if (s->cfg.stages < 0) {
        s->stages = 0;
    } else if (s->cfg.stages == 0) {
        if (s->rows == 16) s->rows = 8;
        s->stages = s->rows == 4 ? 3 : 4;
        s->vec = yee_bulk_tile_vec(s->rows);
    } else {
        s->stages = s->cfg.stages;
        s->vec = yee_bulk_tile_vec(s->rows);
        if (yee_bulk_smem_bytes(s->rows, s->stages, true) == 0) {
            delete s;
            return set_error(PTK_ERR_INVALID, "no staged kernel for %d rows with %d stages", cfg->tile_rows,
                             cfg->stages);
        }
    }
    if (pool_alloc(sizeof(double) * 6 * kSumBlocks, default_stream(), (void **)&s->d_part)) {
        delete s;
        return set_error(PTK_ERR_NOMEM, "server checksum partials allocation failed");
    }
    if (s->stages && (pool_alloc(sizeof(int), default_stream(), (void **)&s->d_err) ||
                      pool_alloc(sizeof(int) * s->cfg.chunk_steps, default_stream(), (void **)&s->d_work) ||
                      cudaMallocHost(&s->h_err, 2 * sizeof(int)) != cudaSuccess ||
                      cudaMemsetAsync(s->d_err, 0, sizeof(int), default_stream()) != cudaSuccess ||
                      cudaStreamSynchronize(default_stream()) != cudaSuccess)) {
        if (s->d_err) pool_free(s->d_err, default_stream());
        if (s->d_work) pool_free(s->d_work, default_stream());
        if (s->h_err) cudaFreeHost(s->h_err);
        pool_free(s->d_part, default_stream());
        delete s;
        return set_error(PTK_ERR_CUDA, "server error word allocation failed");
    }
    if (s->h_err) s->h_err[0] = s->h_err[1] = 0;
    if (s->cfg.hbm_budget_bytes == 0) {
        size_t f = 0, t = 0;
        cudaMemGetInfo(&f, &t);
        s->cfg.hbm_budget_bytes = f / 10 * 8;
    }
    bool ok = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) == cudaSuccess;
    for (int b = 0; b < 2 && ok; ++b)
        ok = cudaEventCreate(&s->ev_start[b]) == cudaSuccess && cudaEventCreate(&s->ev_end[b]) == cudaSuccess &&
             cudaEventCreateWithFlags(&s->ev_ret[b], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        for (int b = 0; b < 2; ++b)
            for (cudaEvent_t e : {s->ev_start[b], s->ev_end[b], s->ev_ret[b]})
                if (e) cudaEventDestroy(e);
        if (s->st) cudaStreamDestroy(s->st);
        if (s->d_err) pool_free(s->d_err, default_stream());
        if (s->d_work) pool_free(s->d_work, default_stream());
        if (s->h_err) cudaFreeHost(s->h_err);
        pool_free(s->d_part, default_stream());
        delete s;
        return set_error(PTK_ERR_CUDA, "stream creation failed");
    }
    *out = s;
    return PTK_OK;
} PTK_CATCH_ALL

int ptk_server_submit(ptk_server *s, const ptk_problem_desc *d, double arrival_s, long long *ticket)
try {
    PTK_CHECK_ARG(s && d, "NULL argument");
    PTK_CHECK_ARG(d->Nx >= 1 && d->Ny >= 1 && d->Nz >= 1 && d->steps >= 1, "bad request %dx%dx%d x %d steps",
                  d->Nx, d->Ny, d->Nz, d->steps);
    PTK_CHECK_ARG(d->n_boxes <= kMaxBoxes, "at most %d boxes per request", kMaxBoxes);
    const Layout L = make_layout(d->Nx, d->Ny, d->Nz);
    const size_t need = instance_bytes(L, d->steps);
    if (need > s->cfg.hbm_budget_bytes)
        return set_error(PTK_ERR_BUDGET, "request needs %zu bytes, more than the whole HBM budget (%zu)", need,
                         s->cfg.hbm_budget_bytes);
    std::lock_guard<std::mutex> lk(s->mu);
    Inst *in = new Inst();
    in->ticket = (long long)s->all.size();
    in->desc = *d;
    in->t_arrival = arrival_s;
    s->all.push_back(in);
    if (ticket) *ticket = in->ticket;
    return PTK_OK;
} PTK_CATCH_ALL

int ptk_server_run(ptk_server *s, double time_scale)
try {
    clear_error();
    PTK_CHECK_ARG(s, "NULL server");
    std::lock_guard<std::mutex> lk(s->mu);
    // admission order = arrival order (stable for ties)
    std::vector<Inst *> order;
    for (Inst *in : s->all)
        if (!in->finished && in->t_admit < 0) order.push_back(in);
    std::stable_sort(order.begin(), order.end(), [](Inst *a, Inst *b) { return a->t_arrival < b->t_arrival; });
    for (Inst *in : order) in->t_arrival_run = time_scale > 0 ? in->t_arrival * time_scale : 0.0;
    const double t0 = now_s();
    size_t nxt = 0;
    int grid_cap[5] = {0, 0, 0, 0, 0};   // resident CTAs of the step kernel per vec (1, 2, 4)
    for (int v : {1, 2, 4})
        grid_cap[v] = std::max(1, s->stages ? yee_bulk_resident_ctas(s->rows, s->stages, true)
                                            : yee_resident_ctas(s->rows, v));
    s->resident = grid_cap[s->vec];
    auto clock = [&] { return (now_s() - t0); };
    auto arrived = [&](Inst *in, double t) { return time_scale <= 0 || in->t_arrival * time_scale <= t; };
    // Wait for the chunk of slot b and its retirement copies; complete its finishers.
    auto land = [&](int b) -> int {
        ptk_server::Flight &F = s->flight[b];
        if (!F.on) return PTK_OK;
        F.on = false;
        if (cudaEventSynchronize(s->ev_ret[b]) != cudaSuccess)
            return set_error(PTK_ERR_CUDA, "chunk failed: %s", cudaGetErrorString(cudaGetLastError()));
        if (s->stages && s->h_err[b])
            return set_error(PTK_ERR_TIMEOUT, "staged step kernel: a bounded wait expired (error word %d)",
                             s->h_err[b]);
        float ms = 0;
        if (cudaEventElapsedTime(&ms, s->ev_start[b], s->ev_end[b]) == cudaSuccess) s->chunk_dev_s += ms * 1e-3;
        const double t = clock();
        for (size_t q = 0; q < F.gone.size(); ++q) retire_finish(s, F.gone[q], s->h_sums[b] + 6 * q, t);
        F.gone.clear();
        return PTK_OK;
    };
    int rc = PTK_OK;
    // One chunk is queued behind the running one: the host admits, rebuilds the work list and
    // launches chunk i+1 (with chunk i's finishers retired in stream order between them), then
    // waits for chunk i.
    while (rc == PTK_OK && (nxt < order.size() || !s->active.empty())) {
        double t = clock();
        s->up_used[s->par] = 0;   // this half's copies preceded a chunk that has landed
        // admit arrived requests, FIFO, while they fit the budget and the slot limit
        while (nxt < order.size() && !s->admit_blocked && arrived(order[nxt], t) &&
               (int)s->active.size() < s->cfg.max_active) {
            Inst *in = order[nxt];
            const size_t need = instance_bytes(make_layout(in->desc.Nx, in->desc.Ny, in->desc.Nz), in->desc.steps);
            if (s->used + need > s->cfg.hbm_budget_bytes) break;
            in->t_admit = t;
            const double ta = now_s();
            rc = admit(s, in);
            s->admit_s += now_s() - ta;
            if (rc == PTK_ERR_NOMEM && (!s->active.empty() || s->flight[0].on || s->flight[1].on)) {
                // Within the budget but the pool has no block that fits right now: back-pressure,
                // not a failure.  Try again once running requests have retired and freed theirs.
                clear_error();
                rc = PTK_OK;
                in->t_admit = -1;
                s->admit_blocked = true;
                ++s->admit_waits;
                break;
            }
            if (rc) break;
            ++nxt;
        }
        if (rc) break;
        if (s->active.empty()) {
            // nothing to run: complete what is queued, then wait for the next arrival
            rc = land(s->par ^ 1);
            if (!rc) rc = land(s->par);
            if (rc) break;
            if (cudaStreamSynchronize(s->st) != cudaSuccess) {
                rc = set_error(PTK_ERR_CUDA, "stream failed: %s", cudaGetErrorString(cudaGetLastError()));
                break;
            }
            s->up_used[0] = s->up_used[1] = 0;
            if (s->admit_blocked) {   // everything has retired and its memory is free: try again
                s->admit_blocked = false;
                continue;
            }
            if (nxt < order.size()) {
                const double wait = order[nxt]->t_arrival * time_scale - clock();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            }
            continue;
        }
        const double ts = now_s();
        if (s->dirty) rc = rebuild_worklist(s);
        if (rc) break;
        int left_min = 1 << 30;
        for (Inst *in : s->active) left_min = std::min(left_min, in->steps_total - in->done);
        // chunk length: the configured chunk, shortened so that the first finisher leaves promptly
        const int len = std::max(1, std::min(s->cfg.chunk_steps, left_min));
        const int grid = s->cfg.persistent ? std::min(grid_cap[s->vec], s->total_tiles) : 0;
        cudaGraphExec_t ex;
        rc = chunk_graph(s, len, grid, &ex);
        if (rc) break;
        s->sched_s += now_s() - ts;
        const int b = s->par;
        if (cudaEventRecord(s->ev_start[b], s->st) != cudaSuccess || cudaGraphLaunch(ex, s->st) != cudaSuccess ||
            cudaEventRecord(s->ev_end[b], s->st) != cudaSuccess) {
            rc = set_error(PTK_ERR_CUDA, "chunk launch failed");
            break;
        }
        s->flight[b].exec = ex;
        // kernels in the chunk graph: the steps, the step-counter advance and (staged) the faces
        const int kernels = len + 1 + (s->stages && s->total_faces > 0 ? 1 : 0);
        count_graph_launch(kernels);
        s->launches += kernels;
        ++s->chunks;
        if (s->stages &&
            cudaMemcpyAsync(s->h_err + b, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st) != cudaSuccess) {
            rc = set_error(PTK_ERR_CUDA, "error word copy failed");
            break;
        }
        // This chunk's finishers: checksums (and results) and frees queued behind it.
        const double tr = now_s();
        std::vector<Inst *> still, gone;
        for (Inst *in : s->active) {
            in->done += std::min(len, in->steps_total - in->done);
            (in->done >= in->steps_total ? gone : still).push_back(in);
        }
        s->active.swap(still);
        if (!gone.empty()) {
            if ((int)gone.size() > s->sums_cap[b]) {
                // slot b's landing slots were read when slot b last landed
                if (s->h_sums[b]) cudaFreeHost(s->h_sums[b]);
                s->h_sums[b] = nullptr;
                s->sums_cap[b] = 0;
                if (cudaMallocHost(&s->h_sums[b], sizeof(double) * 6 * gone.size()) != cudaSuccess) {
                    for (Inst *in : gone) release(s, in);
                    rc = set_error(PTK_ERR_NOMEM, "pinned checksum slots");
                    break;
                }
                s->sums_cap[b] = (int)gone.size();
            }
            for (size_t q = 0; q < gone.size(); ++q) {
                if (!rc) rc = retire_enqueue(s, gone[q], s->h_sums[b] + 6 * q);
                else release(s, gone[q]);
            }
            if (rc) break;
            s->dirty = true;
            s->admit_blocked = false;   // memory was freed: admission may try again
        }
        if (cudaEventRecord(s->ev_ret[b], s->st) != cudaSuccess) {
            rc = set_error(PTK_ERR_CUDA, "event record failed");
            break;
        }
        s->flight[b].on = true;
        s->flight[b].gone.swap(gone);
        s->retire_s += now_s() - tr;
        // the previous chunk ran while this one was prepared
        rc = land(b ^ 1);
        s->par = b ^ 1;
    }
    if (rc == PTK_OK) rc = land(s->par ^ 1);
    if (rc == PTK_OK) rc = land(s->par);
    if (rc != PTK_OK) cudaStreamSynchronize(s->st);
    s->wall_s += clock();
    return rc;
} PTK_CATCH_ALL

int ptk_server_request(ptk_server *s, long long ticket, ptk_request_info *info)
{
    PTK_CHECK_ARG(s && info, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);   // waits for a run in progress
    if (ticket < 0 || ticket >= (long long)s->all.size()) return set_error(PTK_ERR_NOTFOUND, "no ticket %lld", ticket);
    Inst *in = s->all[(size_t)ticket];
    info->ticket = ticket;
    info->Nx = in->desc.Nx;
    info->Ny = in->desc.Ny;
    info->Nz = in->desc.Nz;
    info->steps = in->desc.steps;
    info->arrival_s = in->t_arrival;
    info->admit_s = in->t_admit;
    info->finish_s = in->t_finish;
    info->done = in->finished ? 1 : 0;
    for (int f = 0; f < 6; ++f) info->checksum[f] = in->checksum[f];
    return PTK_OK;
}

int ptk_server_fetch(ptk_server *s, long long ticket, float *const fields[6])
try {
    PTK_CHECK_ARG(s && fields, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket < 0 || ticket >= (long long)s->all.size()) return set_error(PTK_ERR_NOTFOUND, "no ticket %lld", ticket);
    Inst *in = s->all[(size_t)ticket];
    if (!in->finished) return set_error(PTK_ERR_STATE, "request %lld has not finished", ticket);
    if (in->result[0].empty()) return set_error(PTK_ERR_STATE, "server was created without keep_results");
    for (int f = 0; f < 6; ++f) memcpy(fields[f], in->result[f].data(), in->result[f].size() * sizeof(float));
    return PTK_OK;
} PTK_CATCH_ALL

int ptk_server_stats_get(ptk_server *s, ptk_server_stats *st)
try {
    PTK_CHECK_ARG(s && st, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> lat;
    for (Inst *in : s->all)
        if (in->finished) lat.push_back(in->t_finish - in->t_arrival_run);
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) {
        if (lat.empty()) return 0.0;
        size_t i = (size_t)std::ceil(q * lat.size()) - 1;
        return lat[std::min(i, lat.size() - 1)];
    };
    memset(st, 0, sizeof *st);
    st->submitted = (long long)s->all.size();
    st->completed = (long long)lat.size();
    st->wall_s = s->wall_s;
    st->solves_per_s = s->wall_s > 0 ? lat.size() / s->wall_s : 0;
    st->p50_latency_s = pct(0.50);
    st->p99_latency_s = pct(0.99);
    double sum = 0;
    for (double v : lat) sum += v;
    st->mean_latency_s = lat.empty() ? 0 : sum / lat.size();
    st->cell_updates = s->cell_updates;
    st->mcells_per_s = s->wall_s > 0 ? s->cell_updates / s->wall_s / 1e6 : 0;
    st->chunks = s->chunks;
    st->kernel_launches = s->launches;
    st->peak_active = s->peak_active;
    st->peak_bytes = s->peak_bytes;
    st->chunk_device_s = s->chunk_dev_s;
    st->admit_s = s->admit_s;
    st->retire_s = s->retire_s;
    st->schedule_s = s->sched_s;
    st->graph_captures = s->captures;
    st->admit_waits = s->admit_waits;
    return PTK_OK;
} PTK_CATCH_ALL

int ptk_server_destroy(ptk_server *s)
{
    if (!s) return PTK_OK;
    cudaStreamSynchronize(s->st);
    for (Inst *in : s->active) release(s, in);
    for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
    if (s->d_desc) pool_free(s->d_desc, s->st);
    if (s->d_tile0) pool_free(s->d_tile0, s->st);
    if (s->d_face0) pool_free(s->d_face0, s->st);
    for (int b = 0; b < 2; ++b) {
        if (s->h_desc[b]) cudaFreeHost(s->h_desc[b]);
        if (s->h_tile0[b]) cudaFreeHost(s->h_tile0[b]);
        if (s->h_face0[b]) cudaFreeHost(s->h_face0[b]);
        if (s->h_sums[b]) cudaFreeHost(s->h_sums[b]);
        if (s->h_up[b]) cudaFreeHost(s->h_up[b]);
    }
    if (s->d_err) pool_free(s->d_err, s->st);
    if (s->d_work) pool_free(s->d_work, s->st);
    if (s->h_err) cudaFreeHost(s->h_err);
    if (s->d_part) pool_free(s->d_part, s->st);
    cudaStreamSynchronize(s->st);
    cudaStreamDestroy(s->st);
    for (int b = 0; b < 2; ++b)
        for (cudaEvent_t e : {s->ev_start[b], s->ev_end[b], s->ev_ret[b]})
            if (e) cudaEventDestroy(e);
    for (Inst *in : s->all) delete in;
    delete s;
    return PTK_OK;
}

}  // extern "C"
