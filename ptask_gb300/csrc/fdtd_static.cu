// fdtd_static.cu -- an FDTD solve that allocates no device memory.
//
// Who this is for: callers that must not have a library allocate GPU memory behind their back.  A
// plugin or solver component inside a larger application often gets all of its device memory from
// the host application's own arena, sized against a budget; a private cudaMalloc bypasses that
// accounting and can fail once the arena holds the rest of the GPU.  A latency-critical loop cannot
// take cudaMalloc / cudaFree either: they may synchronise the device and their latency is unbounded.
// ptk_fdtd_solve_static serves both: the caller passes its six fields and coefficients in device
// memory, and every intermediate the fused step kernel needs (the padded ping-pong fields, padded
// coefficients, the instance descriptor and the one-entry work list) lives in one file-scope
// __device__ array of fixed size.  It calls no cudaMalloc, cudaFree or other allocating routine.
//
// Costs and rules, for the user:
//   * Every GPU that loads this library holds kStaticScratchBytes (48 MiB) of device memory until
//     the process exits (the array is part of the module image).  Cubes up to 89^3 fit (padded
//     nodes roundup(Nx+1,32) * (Ny+1) * (Nz+1) up to 786,424); larger grids are rejected.
//   * The array's device address is looked up once per device (cudaGetSymbolAddress) by the first
//     call on that device, with that device current, and kept for the life of the process: make
//     that first call before any stream capture, and do not call again on a device after
//     cudaDeviceReset (the kept address would name freed memory).
//   * All calls share the one array and it keeps the previous call's contents: the regions a call
//     uses are cleared at its start.  Calls whose GPU work overlaps (different streams, no ordering)
//     race on the array; serialise them.
#include "ptk_internal.h"

#include <map>
#include <mutex>

namespace ptk {

// 48 MiB: 16 padded arrays and a 512-byte header, i.e. grids whose padded node count
// (roundup(Nx+1,32) * (Ny+1) * (Nz+1)) is at most 786,424: cubes up to 89^3, or e.g. 96x64x48.
constexpr size_t kStaticScratchBytes = 48ull << 20;
constexpr size_t kStaticAlign = 256;

static __device__ __align__(256) unsigned char g_fdtd_static_scratch[kStaticScratchBytes];

namespace {

std::mutex g_static_mu;
std::map<int, void *> g_static_addr;   // device ordinal -> device address of the scratch array

// Device address of the scratch array on the current device.  In host code the array's name is a
// host-side stand-in, so the address must come from the runtime.
int static_scratch(void **out)
{
    int dev = -1;
    PTK_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_static_mu);
    auto it = g_static_addr.find(dev);
    if (it != g_static_addr.end()) {
        *out = it->second;
        return PTK_OK;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_fdtd_static_scratch);
    if (e != cudaSuccess || !p)
        return set_error(PTK_ERR_CUDA, "cudaGetSymbolAddress of the static FDTD scratch failed on device %d: %s",
                         dev, cudaGetErrorString(e));
    g_static_addr[dev] = p;
    *out = p;
    return PTK_OK;
}

size_t align_up(size_t v) { return (v + kStaticAlign - 1) / kStaticAlign * kStaticAlign; }

__global__ void k_static_desc(InstDesc *dst, InstDesc v, int *tile0, int total)
{
    *dst = v;
    tile0[0] = 0;
    tile0[1] = total;
}

}  // namespace
}  // namespace ptk

using namespace ptk;

extern "C" {

size_t ptk_fdtd_static_scratch_bytes(void) { return kStaticScratchBytes; }

int ptk_fdtd_solve_static(const ptk_fdtd_params *p, float *const fields[6], const float *Ca, const float *Cb,
                          const float *Da, const float *Db, int si, int sj, int sk, const float *wave, int nwave,
                          int steps, void *stream)
{
    clear_error();
    PTK_CHECK_ARG(p && fields, "NULL argument");
    PTK_CHECK_ARG(p->Nx >= 1 && p->Ny >= 1 && p->Nz >= 1, "grid %dx%dx%d must be at least 1x1x1", p->Nx, p->Ny,
                  p->Nz);
    PTK_CHECK_ARG(steps >= 0, "negative step count");
    for (int q = 0; q < 6; ++q) PTK_CHECK_ARG(fields[q], "field %d is NULL", q);
    const bool vacuum = !Ca && !Cb && !Da && !Db;
    PTK_CHECK_ARG(vacuum || (Ca && Cb && Da && Db), "give all four coefficient arrays or none");
    const bool has_src = wave && nwave > 0;
    if (has_src)
        PTK_CHECK_ARG(si >= 1 && si < p->Nx && sj >= 1 && sj < p->Ny && sk >= 0 && sk < p->Nz,
                      "source node (%d,%d,%d) must be an interior Ez node", si, sj, sk);

    const Layout L = make_layout(p->Nx, p->Ny, p->Nz);
    const size_t arr = align_up((size_t)L.total * sizeof(float));
    const size_t head = 2 * kStaticAlign;   // InstDesc, then the tile prefix
    const size_t need = head + 16 * arr;
    if (need > kStaticScratchBytes)
        return set_error(PTK_ERR_BUDGET,
                         "grid %dx%dx%d needs %zu bytes of scratch; ptk_fdtd_solve_static is limited to %zu bytes "
                         "(padded node count roundup(Nx+1,32)*(Ny+1)*(Nz+1) up to about %zu); use the solver API",
                         p->Nx, p->Ny, p->Nz, need, kStaticScratchBytes, (kStaticScratchBytes - head) / 64);

    void *base = nullptr;
    int rc = static_scratch(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;   // NULL: the device's default stream
    unsigned char *b = (unsigned char *)base;
    InstDesc *d_desc = (InstDesc *)b;
    int *d_tile0 = (int *)(b + kStaticAlign);
    float *arrays[16];
    for (int q = 0; q < 16; ++q) arrays[q] = (float *)(b + head + (size_t)q * arr);

    // The scratch keeps the previous call's contents: clear everything this call uses.
    PTK_CUDA_TRY(cudaMemsetAsync(b, 0, need, st));

    InstDesc d{};
    for (int q = 0; q < 6; ++q) {
        d.buf[0][q] = arrays[q];
        d.buf[1][q] = arrays[6 + q];
    }
    for (int c = 0; c < 4; ++c) d.coef[c] = arrays[12 + c];
    d.wave = has_src ? wave : nullptr;
    d.plane = L.plane;
    d.nx = L.nx; d.ny = L.ny; d.nz = L.nz; d.pitch = L.pitch;
    d.cx = p->Cx; d.cy = p->Cy; d.cz = p->Cz;
    d.src = has_src ? ((long long)si + (long long)L.pitch * sj + L.plane * sk) : -1;
    d.nwave = has_src ? nwave : 0;
    d.step = 0;
    d.steps_left = steps;
    const int by = 8;
    plan_tiles(d, by, 16);
    const int total = d.tiles_x * d.tiles_y * d.tiles_z + d.face_tiles;
    k_static_desc<<<1, 1, 0, st>>>(d_desc, d, d_tile0, total);
    PTK_CUDA_TRY(cudaGetLastError());

    for (int q = 0; q < 6; ++q) {
        int ex, ey, ez;
        field_extents(q, p->Nx, p->Ny, p->Nz, &ex, &ey, &ez);
        rc = launch_pack_field(fields[q], ex, ey, ez, L, arrays[q], arrays[6 + q], st);
        if (rc) return rc;
    }
    if (vacuum) {
        const float v[4] = {1.0f, p->Dt / p->eps0, 1.0f, p->Dt / p->mu0};
        for (int c = 0; c < 4; ++c) {
            rc = launch_fill(arrays[12 + c], L.total, v[c], st);
            if (rc) return rc;
        }
    } else {
        const float *src[4] = {Ca, Cb, Da, Db};
        for (int c = 0; c < 4; ++c) {
            rc = launch_pack_coef(src[c], L, arrays[12 + c], st);
            if (rc) return rc;
        }
    }
    for (int s = 0; s < steps; ++s) {
        rc = launch_yee_step(d_desc, d_tile0, 1, total, s, by, st);
        if (rc) return rc;
    }
    const int par = steps & 1;
    for (int q = 0; q < 6; ++q) {
        int ex, ey, ez;
        field_extents(q, p->Nx, p->Ny, p->Nz, &ex, &ey, &ez);
        rc = launch_unpack_field(arrays[par * 6 + q], ex, ey, ez, L, fields[q], st);
        if (rc) return rc;
    }
    return PTK_OK;
}

}  // extern "C"
