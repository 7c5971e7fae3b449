// fdtd_solver.cu -- device-resident FDTD instance with CUDA-graph replay of the fused step.
//
// A solver owns, in HBM: two buffers of each of the six fields (ping-pong), the four coefficient
// arrays, the source waveform and a one-entry work list (InstDesc + tile prefix).  A run of T steps
// replays a captured graph of L fused-step launches followed by one "advance" launch that moves the
// instance's step counter, so the only host work per L steps is one cudaGraphLaunch.  This is the
// scheduler's execution of an iterated FDTD cycle: the per-task dispatch of the reference
// (ptask/task.cpp:3822-3900 -> ptask/cutask.cpp:634-705, six launches per step with host-side
// readiness checks) becomes one replayed graph.
#include "ptk_internal.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace ptk {

__global__ void k_store_desc(InstDesc *dst, InstDesc v) { *dst = v; }

__global__ void k_store_tile0(int *dst, int a, int b)
{
    dst[0] = a;
    dst[1] = b;
}

static int store_desc(InstDesc *d_dst, const InstDesc &v, cudaStream_t s)
{
    k_store_desc<<<1, 1, 0, s>>>(d_dst, v);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

// x cells per thread for a row of nx cells: the widest tile that keeps most lanes busy.
int default_vec(int nx)
{
    if (nx >= 96) return 4;
    if (nx >= 40) return 2;
    return 1;
}

// Default tile shape: rows of 8, z depth chosen so the grid holds several waves of CTAs.
static void default_tiles(int nx, int ny, int nz, int *by, int *kc, int *vec)
{
    *by = 8;
    *vec = default_vec(nx);
    const int tx = 32 * *vec;
    const long long cols = (long long)((nx + tx - 1) / tx) * ((ny + 7) / 8);
    const long long want = 4LL * std::max(1, sm_count()) * 2;   // ~4 waves at 2 CTAs per SM
    long long zc = (want + cols - 1) / std::max(1LL, cols);
    int k = (int)((nz + zc - 1) / std::max(1LL, zc));
    if (k < 16) k = 16;
    if (k >= nz) k = 0;
    *kc = k;
}

struct GraphKey {
    int len, by, kc, vec, stages;
    bool operator<(const GraphKey &o) const
    {
        return std::tie(len, by, kc, vec, stages) < std::tie(o.len, o.by, o.kc, o.vec, o.stages);
    }
};

}  // namespace ptk

using namespace ptk;

struct ptk_solver {
    ptk_fdtd_params p;
    Layout L;
    float *buf[2][6] = {};
    float *coef[4] = {};
    float *wave = nullptr;
    int nwave = 0;
    long long src = -1;
    int step = 0;              // host mirror of the device step counter
    int by = 0, kc = 0, vec = 4, stages = 0;
    int *d_err = nullptr;      // raised by the staged kernel if a bounded wait expires
    void *d_tma = nullptr;     // tensor maps of the staged kernel (encoded for tma_by rows)
    int tma_by = 0;
    unsigned char *mat = nullptr;   // material index of the coefficients (one byte per node)
    float *mat_tab = nullptr;       // its table, kMaxMaterials x (Ca, Cb, Da, Db)
    int nmat = 0;                   // materials in the table; 0 = per-cell arrays only
    bool mat_enabled = true;
    long long *d_face0 = nullptr;   // {0, face nodes}: the staged path advances faces per chunk
    long long faces = 0;
    int *d_work = nullptr;          // staged path: tile counters, one per step of a chunk
    int total_tiles = 0;
    InstDesc *d_desc = nullptr;
    int *d_tile0 = nullptr;
    cudaStream_t cap = nullptr;   // capture stream
    std::map<GraphKey, cudaGraphExec_t> graphs;
    long long last_launches = 0;
    std::mutex mu;
};

namespace ptk {

// The staged kernel reads the material index when the coefficients have one and an instantiation
// of the shape exists; otherwise the per-cell arrays, with the shape clamped to a dense one (10- and
// 11-row tiles have only a 3-plane ring with the per-cell arrays; 5 and 6 planes exist only with
// the index).
static bool use_mat(const ptk_solver *s)
{
    return s->stages > 0 && s->mat_enabled && s->nmat > 0 && yee_bulk_smem_bytes(s->by, s->stages, true) > 0;
}

struct RunShape {
    int by, stages;
    bool mat;
};

static RunShape run_shape(const ptk_solver *s)
{
    if (s->stages <= 0) return {s->by, 0, false};
    if (use_mat(s)) return {s->by, s->stages, true};
    if (yee_bulk_smem_bytes(s->by, s->stages, false) > 0) return {s->by, s->stages, false};
    // same rows with the 3-plane ring the per-cell arrays leave room for (10 and 11 rows), else 4
    if (yee_bulk_smem_bytes(s->by, 3, false) > 0) return {s->by, 3, false};
    return {s->by >= 8 ? 8 : 4, 4, false};
}

static int rebuild_material(ptk_solver *s, cudaStream_t st)
{
    s->nmat = 0;
    if (!s->mat_enabled) return PTK_OK;
    const float *const c[4] = {s->coef[0], s->coef[1], s->coef[2], s->coef[3]};
    return build_material_index(c, s->L, s->mat, s->mat_tab, &s->nmat, st);
}

static InstDesc host_desc(const ptk_solver *s, int steps_left)
{
    InstDesc d{};
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 6; ++f) d.buf[b][f] = s->buf[b][f];
    for (int c = 0; c < 4; ++c) d.coef[c] = s->coef[c];
    d.wave = s->wave;
    d.plane = s->L.plane;
    d.nx = s->L.nx; d.ny = s->L.ny; d.nz = s->L.nz; d.pitch = s->L.pitch;
    d.cx = s->p.Cx; d.cy = s->p.Cy; d.cz = s->p.Cz;
    d.src = s->nwave > 0 ? s->src : -1;
    d.nwave = s->nwave;
    d.step = s->step;
    d.steps_left = steps_left;
    const RunShape rs = run_shape(s);
    if (rs.mat) {
        d.mat = s->mat;
        d.mat_tab = s->mat_tab;
        d.nmat = s->nmat;
    }
    plan_tiles(d, rs.by, s->kc, rs.stages > 0 ? yee_bulk_tile_vec(rs.by) : s->vec);
    if (rs.stages > 0) d.face_tiles = 0;   // faces: launch_yee_faces_steps, once per chunk
    return d;
}


static int solver_sync_desc(ptk_solver *s, int steps_left, cudaStream_t st)
{
    InstDesc d = host_desc(s, steps_left);
    s->total_tiles = d.tiles_x * d.tiles_y * d.tiles_z + d.face_tiles;
    const RunShape rs = run_shape(s);
    if (rs.stages > 0) {
        if (s->tma_by != rs.by) {
            // The arrays never move, so the maps change only with the tile rows.
            alignas(64) unsigned char maps[kTmaSetBytes];
            InstDesc e = d;
            e.mat = s->mat;   // the index map is always encoded; the kernel variant decides its use
            int rc = encode_tma_set(e, rs.by, maps);
            if (rc) return rc;
            PTK_CUDA_TRY(cudaStreamSynchronize(st));
            PTK_CUDA_TRY(cudaMemcpy(s->d_tma, maps, kTmaSetBytes, cudaMemcpyHostToDevice));
            s->tma_by = rs.by;
        }
        d.tma = s->d_tma;
    }
    int rc = store_desc(s->d_desc, d, st);
    if (rc) return rc;
    k_store_tile0<<<1, 1, 0, st>>>(s->d_tile0, 0, s->total_tiles);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

static void drop_graphs(ptk_solver *s)
{
    for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
}

// Graph of `len` fused steps + one advance for this solver's current tile shape.
static int solver_graph(ptk_solver *s, int len, cudaGraphExec_t *out)
{
    const RunShape rs = run_shape(s);
    GraphKey key{len, rs.by, s->kc, s->vec, rs.stages * 2 + (rs.mat ? 1 : 0)};
    auto it = s->graphs.find(key);
    if (it != s->graphs.end()) {
        *out = it->second;
        return PTK_OK;
    }
    if (!s->cap) PTK_CUDA_TRY(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
    // The staged kernel runs as a persistent grid of resident CTAs taking tiles from a counter, so
    // a CTA streams several tiles through one ring and the last wave is balanced.
    const int grid = rs.stages > 0 ? yee_bulk_resident_ctas(rs.by, rs.stages, rs.mat) : 0;
    PTK_CUDA_TRY(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    int rc = PTK_OK;
    if (rs.stages > 0) {
        if (cudaMemsetAsync(s->d_work, 0, sizeof(int) * len, s->cap) != cudaSuccess)
            rc = set_error(PTK_ERR_CUDA, "tile counter reset failed");
        else
            count_launches(1);
    }
    for (int q = 0; q < len && rc == PTK_OK; ++q)
        rc = rs.stages > 0
                 ? launch_yee_step_bulk(s->d_desc, s->d_tile0, 1, s->total_tiles, q, rs.by, rs.stages, grid, s->d_err,
                                        s->cap, s->d_work, rs.mat, /*lazy=*/true)
                 : launch_yee_step_v(s->d_desc, s->d_tile0, 1, s->total_tiles, q, s->by, s->vec, 0, s->cap);
    if (rc == PTK_OK && rs.stages > 0) rc = launch_yee_faces_steps(s->d_desc, s->d_face0, 1, s->faces, 0, len, s->cap);
    if (rc == PTK_OK) rc = launch_advance(s->d_desc, 1, len, s->cap);
    set_capturing(false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->cap, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return set_error(PTK_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(PTK_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    s->graphs[key] = ex;
    *out = ex;
    return PTK_OK;
}

static constexpr int kChunk = 32;   // fused steps per replayed graph

int solver_run(ptk_solver *s, int steps, cudaStream_t st)
{
    if (steps < 0) return set_error(PTK_ERR_INVALID, "negative step count");
    s->last_launches = 0;
    if (steps == 0) return PTK_OK;
    int rc = solver_sync_desc(s, steps, st);
    if (rc) return rc;
    int left = steps;
    while (left > 0) {
        const int len = left >= kChunk ? kChunk : left;
        cudaGraphExec_t ex;
        rc = solver_graph(s, len, &ex);
        if (rc) return rc;
        PTK_CUDA_TRY(cudaGraphLaunch(ex, st));
        count_graph_launch(len + 1);
        s->last_launches += len + 1;
        left -= len;
    }
    s->step += steps;
    return PTK_OK;
}

static size_t field_bytes(int f, const ptk_fdtd_params &p)
{
    int ex, ey, ez;
    field_extents(f, p.Nx, p.Ny, p.Nz, &ex, &ey, &ez);
    return (size_t)ex * ey * ez * sizeof(float);
}

}  // namespace ptk

static inline cudaStream_t S(void *s) { return s ? (cudaStream_t)s : default_stream(); }

static int validate_params(const ptk_fdtd_params *p)
{
    PTK_CHECK_ARG(p, "params is NULL");
    PTK_CHECK_ARG(p->Nx >= 1 && p->Ny >= 1 && p->Nz >= 1, "grid %dx%dx%d must be at least 1x1x1",
                  p->Nx, p->Ny, p->Nz);
    PTK_CHECK_ARG((long long)p->Nx * p->Ny * p->Nz <= (1LL << 33), "grid too large");
    return PTK_OK;
}

extern "C" {

int ptk_solver_create(const ptk_fdtd_params *p, ptk_solver **out)
try {
    clear_error();
    int rc = validate_params(p);
    if (rc) return rc;
    PTK_CHECK_ARG(out, "out is NULL");
    rc = ensure_init();
    if (rc) return rc;
    ptk_solver *s = new ptk_solver();
    s->p = *p;
    s->L = make_layout(p->Nx, p->Ny, p->Nz);
    default_tiles(p->Nx, p->Ny, p->Nz, &s->by, &s->kc, &s->vec);
    cudaStream_t st = default_stream();
    const size_t bytes = (size_t)s->L.total * sizeof(float);
    for (int b = 0; b < 2 && rc == PTK_OK; ++b)
        for (int f = 0; f < 6 && rc == PTK_OK; ++f) rc = pool_alloc(bytes, st, (void **)&s->buf[b][f]);
    for (int c = 0; c < 4 && rc == PTK_OK; ++c) rc = pool_alloc(bytes, st, (void **)&s->coef[c]);
    if (rc == PTK_OK) rc = pool_alloc(sizeof(InstDesc), st, (void **)&s->d_desc);
    if (rc == PTK_OK) rc = pool_alloc(2 * sizeof(int), st, (void **)&s->d_tile0);
    if (rc == PTK_OK) rc = pool_alloc(sizeof(int), st, (void **)&s->d_err);
    if (rc == PTK_OK) rc = pool_alloc(kTmaSetBytes, st, &s->d_tma);
    if (rc == PTK_OK) rc = pool_alloc((size_t)s->L.total, st, (void **)&s->mat);
    if (rc == PTK_OK) rc = pool_alloc(sizeof(float) * 4 * kMaxMaterials, st, (void **)&s->mat_tab);
    if (rc == PTK_OK) cudaMemsetAsync(s->mat, 0, (size_t)s->L.total, st);
    if (rc == PTK_OK) rc = pool_alloc(2 * sizeof(long long), st, (void **)&s->d_face0);
    if (rc == PTK_OK) rc = pool_alloc(sizeof(int) * kChunk, st, (void **)&s->d_work);
    if (rc == PTK_OK) {
        s->faces = face_nodes(p->Nx, p->Ny, p->Nz);
        const long long f0[2] = {0, s->faces};   // pageable: staged before the call returns
        if (cudaMemcpyAsync(s->d_face0, f0, sizeof f0, cudaMemcpyHostToDevice, st) != cudaSuccess)
            rc = set_error(PTK_ERR_CUDA, "face prefix upload failed");
    }
    if (rc == PTK_OK && ((uintptr_t)s->d_tma & 63))
        rc = set_error(PTK_ERR_CUDA, "tensor-map buffer is not 64-byte aligned");
    if (rc == PTK_OK) cudaMemsetAsync(s->d_err, 0, sizeof(int), st);
    if (rc) {
        ptk_solver_destroy(s);
        return rc;
    }
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 6; ++f) cudaMemsetAsync(s->buf[b][f], 0, bytes, st);
    for (int c = 0; c < 4; ++c) cudaMemsetAsync(s->coef[c], 0, bytes, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        ptk_solver_destroy(s);
        return set_error(PTK_ERR_CUDA, "solver initialisation failed");
    }
    rc = ptk_solver_set_vacuum(s, nullptr);
    if (rc) {
        ptk_solver_destroy(s);
        return rc;
    }
    *out = s;
    return PTK_OK;
} PTK_CATCH_ALL

int ptk_solver_destroy(ptk_solver *s)
{
    if (!s) return PTK_OK;
    cudaStream_t st = default_stream();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        drop_graphs(s);
        for (int b = 0; b < 2; ++b)
            for (int f = 0; f < 6; ++f) pool_free(s->buf[b][f], st);
        for (int c = 0; c < 4; ++c) pool_free(s->coef[c], st);
        pool_free(s->wave, st);
        pool_free(s->d_desc, st);
        pool_free(s->d_tile0, st);
        pool_free(s->d_err, st);
        pool_free(s->d_tma, st);
        pool_free(s->mat, st);
        pool_free(s->mat_tab, st);
        pool_free(s->d_face0, st);
        pool_free(s->d_work, st);
        if (s->cap) cudaStreamDestroy(s->cap);
    }
    cudaStreamSynchronize(st);
    delete s;
    return PTK_OK;
}

int ptk_solver_set_fields(ptk_solver *s, const float *const f[6], int where, void *stream)
{
    clear_error();
    PTK_CHECK_ARG(s && f, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    cudaStream_t st = S(stream);
    for (int q = 0; q < 6; ++q) {
        PTK_CHECK_ARG(f[q], "field %d is NULL", q);
        int ex, ey, ez;
        field_extents(q, s->p.Nx, s->p.Ny, s->p.Nz, &ex, &ey, &ez);
        const float *src = f[q];
        float *stage = nullptr;
        if (where == PTK_HOST) {
            int rc = pool_alloc(field_bytes(q, s->p), st, (void **)&stage);
            if (rc) return rc;
            PTK_CUDA_TRY(cudaMemcpyAsync(stage, f[q], field_bytes(q, s->p), cudaMemcpyHostToDevice, st));
            src = stage;
        }
        int rc = launch_pack_field(src, ex, ey, ez, s->L, s->buf[0][q], s->buf[1][q], st);
        if (stage) pool_free(stage, st);
        if (rc) return rc;
    }
    return PTK_OK;
}

int ptk_solver_get_fields(ptk_solver *s, float *const f[6], int where, void *stream)
{
    clear_error();
    PTK_CHECK_ARG(s && f, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    cudaStream_t st = S(stream);
    const int par = s->step & 1;
    for (int q = 0; q < 6; ++q) {
        PTK_CHECK_ARG(f[q], "field %d is NULL", q);
        int ex, ey, ez;
        field_extents(q, s->p.Nx, s->p.Ny, s->p.Nz, &ex, &ey, &ez);
        float *dst = f[q];
        float *stage = nullptr;
        if (where == PTK_HOST) {
            int rc = pool_alloc(field_bytes(q, s->p), st, (void **)&stage);
            if (rc) return rc;
            dst = stage;
        }
        int rc = launch_unpack_field(s->buf[par][q], ex, ey, ez, s->L, dst, st);
        if (rc) return rc;
        if (stage) {
            PTK_CUDA_TRY(cudaMemcpyAsync(f[q], stage, field_bytes(q, s->p), cudaMemcpyDeviceToHost, st));
            pool_free(stage, st);
        }
    }
    if (where == PTK_HOST) {
        PTK_CUDA_TRY(cudaStreamSynchronize(st));
        int err = 0;
        PTK_CUDA_TRY(cudaMemcpy(&err, s->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err)
            return set_error(PTK_ERR_TIMEOUT, "a bounded wait of the staged step kernel expired; the fields are invalid");
    }
    return PTK_OK;
}

int ptk_solver_set_coefficients(ptk_solver *s, const float *Ca, const float *Cb, const float *Da,
                                const float *Db, int where, void *stream)
{
    clear_error();
    PTK_CHECK_ARG(s && Ca && Cb && Da && Db, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    cudaStream_t st = S(stream);
    const float *src[4] = {Ca, Cb, Da, Db};
    const size_t bytes = (size_t)s->p.Nx * s->p.Ny * s->p.Nz * sizeof(float);
    for (int c = 0; c < 4; ++c) {
        const float *a = src[c];
        float *stage = nullptr;
        if (where == PTK_HOST) {
            int rc = pool_alloc(bytes, st, (void **)&stage);
            if (rc) return rc;
            PTK_CUDA_TRY(cudaMemcpyAsync(stage, src[c], bytes, cudaMemcpyHostToDevice, st));
            a = stage;
        }
        int rc = launch_pack_coef(a, s->L, s->coef[c], st);
        if (stage) pool_free(stage, st);
        if (rc) return rc;
    }
    return rebuild_material(s, st);
}

int ptk_solver_set_vacuum(ptk_solver *s, void *stream)
{
    PTK_CHECK_ARG(s, "NULL solver");
    cudaStream_t st = S(stream);
    // Scalar coefficients of the reference: (params.Dt/params.eps0), (params.Dt/params.mu0) in FP32.
    const float ce = s->p.Dt / s->p.eps0;
    const float ch = s->p.Dt / s->p.mu0;
    const float v[4] = {1.0f, ce, 1.0f, ch};
    for (int c = 0; c < 4; ++c) {
        int rc = launch_fill(s->coef[c], s->L.total, v[c], st);
        if (rc) return rc;
    }
    return rebuild_material(s, st);
}

int ptk_solver_set_source(ptk_solver *s, int i, int j, int k, const float *wave, int nwave, int where,
                          void *stream)
{
    clear_error();
    PTK_CHECK_ARG(s, "NULL solver");
    std::lock_guard<std::mutex> lk(s->mu);
    cudaStream_t st = S(stream);
    if (nwave <= 0 || !wave) {
        s->nwave = 0;
        s->src = -1;
        return PTK_OK;
    }
    PTK_CHECK_ARG(i >= 1 && i < s->p.Nx && j >= 1 && j < s->p.Ny && k >= 0 && k < s->p.Nz,
                  "source node (%d,%d,%d) must be an interior Ez node of a %dx%dx%d grid", i, j, k,
                  s->p.Nx, s->p.Ny, s->p.Nz);
    if (s->wave) pool_free(s->wave, st);
    s->wave = nullptr;
    int rc = pool_alloc((size_t)nwave * sizeof(float), st, (void **)&s->wave);
    if (rc) return rc;
    PTK_CUDA_TRY(cudaMemcpyAsync(s->wave, wave, (size_t)nwave * sizeof(float),
                                 where == PTK_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    s->nwave = nwave;
    s->src = (long long)i + (long long)s->L.pitch * j + s->L.plane * k;
    return PTK_OK;
}

int ptk_solver_reset_clock(ptk_solver *s, void *stream)
{
    PTK_CHECK_ARG(s, "NULL solver");
    (void)stream;
    std::lock_guard<std::mutex> lk(s->mu);
    // The parity of the current field buffer is tied to the step counter; keep it and only
    // rebase the waveform index by storing the offset in the host mirror.
    if (s->step & 1) {
        // Swap buffer roles so that step 0 reads the buffer that holds the current fields.  The
        // staged kernel's tensor maps name the buffers by parity: encode them again.
        for (int f = 0; f < 6; ++f) std::swap(s->buf[0][f], s->buf[1][f]);
        s->tma_by = 0;
    }
    s->step = 0;
    return PTK_OK;
}

int ptk_solver_set_tiles(ptk_solver *s, const ptk_tile_config *cfg)
{
    PTK_CHECK_ARG(s && cfg, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    int by = cfg->by, kc = cfg->kc, vec = cfg->vec;
    if (by == 0 && kc == 0) {
        int dv = 4;
        default_tiles(s->p.Nx, s->p.Ny, s->p.Nz, &by, &kc, &dv);
        if (vec == 0) vec = dv;
    }
    const int stages = cfg->stages;
    if (stages > 0) vec = yee_bulk_tile_vec(by);
    if (vec == 0) vec = default_vec(s->p.Nx);
    PTK_CHECK_ARG(by == 4 || by == 8 || by == 16 || (stages > 0 && (by == 7 || by == 10 || by == 11 || by == 23)),
                  "tile rows must be 4, 8 or 16, or 7, 10, 11 or 23 with a staged ring (got %d)", by);
    PTK_CHECK_ARG(vec == 1 || vec == 2 || vec == 4, "cells per thread must be 1, 2 or 4 (got %d)", vec);
    PTK_CHECK_ARG(stages == 0 || yee_bulk_smem_bytes(by, stages, false) > 0 || yee_bulk_smem_bytes(by, stages, true) > 0,
                  "no staged kernel for %d rows with %d stages", by, stages);
    PTK_CHECK_ARG(kc >= 0, "tile depth must be >= 0");
    if (kc >= s->p.Nz) kc = 0;
    s->by = by;
    s->kc = kc;
    s->vec = vec;
    s->stages = stages;
    return PTK_OK;
}

int ptk_solver_use_material_index(ptk_solver *s, int enable, void *stream)
{
    clear_error();
    PTK_CHECK_ARG(s, "NULL solver");
    std::lock_guard<std::mutex> lk(s->mu);
    s->mat_enabled = enable != 0;
    return rebuild_material(s, S(stream));
}

int ptk_solver_material_count(const ptk_solver *s, int *nmat)
{
    PTK_CHECK_ARG(s && nmat, "NULL argument");
    *nmat = s->mat_enabled ? s->nmat : 0;
    return PTK_OK;
}

int ptk_solver_kernel(const ptk_solver *s, int *stages, int *material_index)
{
    PTK_CHECK_ARG(s && stages && material_index, "NULL argument");
    const RunShape rs = run_shape(s);
    *stages = rs.stages;
    *material_index = rs.mat ? 1 : 0;
    return PTK_OK;
}

int ptk_solver_get_tiles(const ptk_solver *s, ptk_tile_config *cfg)
{
    PTK_CHECK_ARG(s && cfg, "NULL argument");
    cfg->by = s->by;
    cfg->kc = s->kc;
    cfg->vec = s->vec;
    cfg->stages = s->stages;
    return PTK_OK;
}

int ptk_solver_run(ptk_solver *s, int steps, void *stream)
try {
    clear_error();
    PTK_CHECK_ARG(s, "NULL solver");
    std::lock_guard<std::mutex> lk(s->mu);
    return solver_run(s, steps, S(stream));
} PTK_CATCH_ALL

int ptk_solver_bytes(const ptk_solver *s, size_t *bytes)
{
    PTK_CHECK_ARG(s && bytes, "NULL argument");
    *bytes = (size_t)s->L.total * sizeof(float) * 16 + (size_t)s->nwave * sizeof(float);
    return PTK_OK;
}

int ptk_solver_last_launches(const ptk_solver *s, long long *launches)
{
    PTK_CHECK_ARG(s && launches, "NULL argument");
    *launches = s->last_launches;
    return PTK_OK;
}

int ptk_fdtd_solve(const ptk_fdtd_params *p, float *const fields[6], const float *Ca, const float *Cb,
                   const float *Da, const float *Db, int si, int sj, int sk, const float *wave,
                   int nwave, int steps, float *ms)
try {
    clear_error();
    ptk_solver *s = nullptr;
    int rc = ptk_solver_create(p, &s);
    if (rc) return rc;
    cudaStream_t st = default_stream();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    rc = ptk_solver_set_fields(s, fields, PTK_HOST, st);
    if (!rc && Ca) rc = ptk_solver_set_coefficients(s, Ca, Cb, Da, Db, PTK_HOST, st);
    if (!rc && wave && nwave > 0) rc = ptk_solver_set_source(s, si, sj, sk, wave, nwave, PTK_HOST, st);
    if (!rc) rc = ptk_solver_run(s, steps, st);
    if (!rc) rc = ptk_solver_get_fields(s, fields, PTK_HOST, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    if (ms) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ptk_solver_destroy(s);
    return rc;
} PTK_CATCH_ALL

int ptk_launch_field_update(int field, const float *in0, const float *in1, const float *in2,
                            const ptk_fdtd_params *p, float *out, void *stream)
{
    clear_error();
    int rc = validate_params(p);
    if (rc) return rc;
    PTK_CHECK_ARG(field >= 0 && field < 6, "field id %d out of range", field);
    PTK_CHECK_ARG(in0 && in1 && in2 && out, "NULL buffer");
    rc = ensure_init();
    if (rc) return rc;
    return launch_field_ref(field, in0, in1, in2, *p, out, S(stream));
}

int ptk_launch_h_half_step(const float *const in[6], float *const out_h[3], const ptk_fdtd_params *p,
                           void *stream)
{
    clear_error();
    int rc = validate_params(p);
    if (rc) return rc;
    PTK_CHECK_ARG(in && out_h, "NULL buffer");
    rc = ensure_init();
    if (rc) return rc;
    return launch_h_half(in, out_h, *p, S(stream));
}

int ptk_launch_e_half_step(const float *const e_in[3], const float *const h_new[3],
                           float *const out_e[3], const ptk_fdtd_params *p, void *stream)
{
    clear_error();
    int rc = validate_params(p);
    if (rc) return rc;
    PTK_CHECK_ARG(e_in && h_new && out_e, "NULL buffer");
    rc = ensure_init();
    if (rc) return rc;
    return launch_e_half(e_in, h_new, out_e, *p, S(stream));
}

// --------------------------------------------------------------------------------------------
// Autotuner: time candidate (rows, depth) shapes on a scratch solver of the requested size.
// --------------------------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, std::pair<ptk_tile_config, float>> g_tune_cache;

int ptk_autotune_tiles(int Nx, int Ny, int Nz, ptk_tile_config *best, float *best_ms)
try {
    clear_error();
    PTK_CHECK_ARG(best, "NULL argument");
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find({Nx, Ny, Nz});
        if (it != g_tune_cache.end()) {
            *best = it->second.first;
            if (best_ms) *best_ms = it->second.second;
            return PTK_OK;
        }
    }
    ptk_fdtd_params p{};
    int rc = ptk_reference_params(Nx, Ny, Nz, &p);
    if (rc) return rc;
    ptk_solver *s = nullptr;
    rc = ptk_solver_create(&p, &s);
    if (rc) return rc;
    cudaStream_t st = default_stream();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int rows[3] = {4, 8, 16};
    const int depths[6] = {8, 16, 32, 64, 128, 0};
    const long long cells = (long long)Nx * Ny * Nz;
    const int steps = (int)std::max(4LL, std::min(64LL, 400000000LL / std::max(1LL, cells)));
    float best_t = 1e30f;
    ptk_tile_config bc{8, 0, default_vec(Nx), 0};
    std::vector<ptk_tile_config> cands;
    // Fixed depths plus the two that fill whole waves of resident CTAs best for each kernel.
    auto add = [&](int by, int vec, int stages, int resident) {
        std::vector<int> ks;
        for (int kc : depths)
            if (!(stages > 0 && kc == 8)) ks.push_back(kc);
        int bal[4];
        int nb = balanced_depths(Nx, Ny, Nz, by, vec, resident, bal, 2);
        if (stages > 0) nb += leftover_depths(Nx, Ny, Nz, by, vec, resident, bal + nb, 2);
        for (int q = 0; q < nb; ++q)
            if (std::find(ks.begin(), ks.end(), bal[q]) == ks.end()) ks.push_back(bal[q]);
        for (int kc : ks)
            if (kc == 0 || kc < Nz) cands.push_back({by, kc, vec, stages});
    };
    for (int vec : {1, 2, 4})
        for (int by : rows) {
            if (32 * vec > 2 * std::max(Nx, 32)) continue;   // tiles far wider than the grid
            add(by, vec, 0, yee_resident_ctas(by, vec));
        }
    // Staged shapes: timed on vacuum coefficients, i.e. with the material index where the shape has it.
    const int staged[17][2] = {{4, 2}, {4, 3}, {4, 4}, {4, 5}, {4, 6}, {8, 2}, {8, 3}, {8, 4}, {8, 5}, {8, 6},
                               {10, 4}, {10, 5}, {11, 4}, {23, 3}, {23, 4}, {7, 3}, {7, 4}};
    for (const auto &bs : staged) {
        const bool m = yee_bulk_smem_bytes(bs[0], bs[1], true) > 0;
        add(bs[0], yee_bulk_tile_vec(bs[0]), bs[1], yee_bulk_resident_ctas(bs[0], bs[1], m));
    }
    // ms per step of one shape over n steps after a 2-step warm-up (< 0: the shape does not run)
    auto time_shape = [&](const ptk_tile_config &c, int n) -> float {
        if (ptk_solver_set_tiles(s, &c)) return -1.f;
        if (ptk_solver_run(s, 2, st)) return -2.f;
        cudaEventRecord(e0, st);
        if (ptk_solver_run(s, n, st)) return -2.f;
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms / n;
    };
    // First pass: every candidate, briefly.  Second pass: the closest few again over longer runs,
    // twice in alternating order, since shapes within a few per cent of each other trade places
    // in short timings.
    std::vector<std::pair<float, ptk_tile_config>> timed;
    for (const ptk_tile_config &c : cands) {
        const float ms = time_shape(c, steps);
        if (ms == -2.f) { rc = PTK_ERR_CUDA; break; }
        if (ms > 0) timed.push_back({ms, c});
    }
    if (!rc && !timed.empty()) {
        std::stable_sort(timed.begin(), timed.end(),
                         [](const std::pair<float, ptk_tile_config> &a, const std::pair<float, ptk_tile_config> &b) {
                             return a.first < b.first;
                         });
        std::vector<std::pair<float, ptk_tile_config>> top;
        for (const auto &e : timed)
            if (top.size() < 4 && e.first <= timed[0].first * 1.05f) top.push_back({0.f, e.second});
        for (int pass = 0; pass < 2 && !rc && top.size() > 1; ++pass)
            for (size_t q = 0; q < top.size() && !rc; ++q) {
                auto &e = top[pass ? top.size() - 1 - q : q];
                const float ms = time_shape(e.second, std::max(8 * steps, 128));
                if (ms < 0) rc = PTK_ERR_CUDA; else e.first += ms;
            }
        if (top.size() == 1) top[0].first = 2 * timed[0].first;
        for (const auto &e : top)
            if (e.first / 2 < best_t) {
                best_t = e.first / 2;
                bc = e.second;
            }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ptk_solver_destroy(s);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[{Nx, Ny, Nz}] = {bc, best_t};
    }
    *best = bc;
    if (best_ms) *best_ms = best_t;
    return PTK_OK;
} PTK_CATCH_ALL

int ptk_default_tiles(int Nx, int Ny, int Nz, ptk_tile_config *cfg)
try {
    clear_error();
    PTK_CHECK_ARG(cfg, "NULL argument");
    PTK_CHECK_ARG(Nx >= 1 && Ny >= 1 && Nz >= 1, "grid %dx%dx%d must be at least 1x1x1", Nx, Ny, Nz);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find({Nx, Ny, Nz});
        if (it != g_tune_cache.end()) {
            *cfg = it->second.first;
            return PTK_OK;
        }
    }
    int rc = ensure_init();
    if (rc) return rc;
    const int by = 11, stages = 4, vec = yee_bulk_tile_vec(by);
    int kc = 0;
    balanced_depths(Nx, Ny, Nz, by, vec, yee_bulk_resident_ctas(by, stages, true), &kc, 1);
    *cfg = {by, kc, vec, stages};
    return PTK_OK;
} PTK_CATCH_ALL

}  // extern "C"
