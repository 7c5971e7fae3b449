// ptk_internal.h -- declarations shared by the CUDA translation units of libptask_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ptask_gb300.h"

namespace ptk {

// ---------------------------------------------------------------------------------------------
// Error reporting: every C entry point funnels failures through set_error, which stores a
// thread-local message for ptk_last_error() and returns the code.
// ---------------------------------------------------------------------------------------------
int set_error(int code, const char *fmt, ...);

// Handlers of the C entry points' function-try-blocks: no C++ exception (a host allocation that
// throws std::bad_alloc, say) unwinds into a C caller; it becomes a status and ptk_last_error().
#define PTK_CATCH_ALL                                                                                  \
    catch (const std::bad_alloc &) { return ptk::set_error(PTK_ERR_NOMEM, "host allocation failed"); } \
    catch (const std::exception &e) { return ptk::set_error(PTK_ERR_STATE, "unexpected error: %s", e.what()); } \
    catch (...) { return ptk::set_error(PTK_ERR_STATE, "unexpected error"); }
void clear_error();

#define PTK_CUDA_TRY(expr)                                                                        \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess)                                                                    \
            return ::ptk::set_error(PTK_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,                 \
                                    cudaGetErrorString(_e), __FILE__, __LINE__);                  \
    } while (0)

#define PTK_CHECK_ARG(cond, ...)                                                                  \
    do {                                                                                          \
        if (!(cond)) return ::ptk::set_error(PTK_ERR_INVALID, __VA_ARGS__);                      \
    } while (0)

// Ensure the runtime is initialised on the current thread (device selected).
int ensure_init();
cudaStream_t default_stream();
int sm_count();

// Stream-ordered device pool (BlockPool replacement).
int pool_alloc(size_t bytes, cudaStream_t s, void **p);
int pool_free(void *p, cudaStream_t s);

// ---------------------------------------------------------------------------------------------
// Padded HBM layout of one FDTD instance.
//   node (i,j,k), 0<=i<=Nx, 0<=j<=Ny, 0<=k<=Nz, lives at i + pitch*j + plane*k with
//   pitch = roundup(Nx+1, 32) floats (rows start on 128-byte boundaries) and plane = pitch*(Ny+1).
// All six fields and the four coefficient arrays share this indexing, so one offset addresses
// every operand of a cell.  Fields are double-buffered (ping-pong); E nodes on the PEC walls are
// never rewritten with new values, so both buffers keep them from the upload onwards.
// ---------------------------------------------------------------------------------------------
struct Layout {
    int nx, ny, nz;
    int pitch;
    long long plane;
    long long total;   // floats per array (plane * (nz+1))
};
Layout make_layout(int nx, int ny, int nz);

// Device-side descriptor of one instance, read by the step kernel.
struct InstDesc {
    float *buf[2][6];          // ping-pong fields: Hx Hy Hz Ex Ey Ez
    const float *coef[4];      // Ca Cb Da Db (padded, face nodes replicate the nearest cell)
    const float *wave;         // source waveform, indexed by absolute step
    long long plane;
    int nx, ny, nz, pitch;
    float cx, cy, cz;
    long long src;             // padded index of the Ez source node, -1 = none
    int nwave;
    int step;                  // absolute index of the first step of the current chunk
    int steps_left;            // steps still to run at the start of the current chunk
    int tiles_x, tiles_y, tiles_z, face_tiles;
    int kc;                    // z-planes per main tile
    int vec;                   // x cells per thread: main tiles are 32*vec cells wide
    const void *tma;           // staged kernel only: tensor maps (6 fields x 2 parities, 4 coefs, index)
    const unsigned char *mat;  // material index (padded layout, one byte per node), or null
    const float *mat_tab;      // its table: nmat entries of (Ca, Cb, Da, Db)
    int nmat;
};

// Bytes of one instance's tensor-map set (17 CUtensorMap of 128 bytes; 64-byte alignment).
constexpr size_t kTmaSetBytes = 17 * 128;
// Material table entries (one-byte ids).
constexpr int kMaxMaterials = 256;

// Per-node material index of an instance's padded coefficient arrays (Ca, Cb, Da, Db): the
// distinct tuples of the nodes (i <= Nx, j <= Ny, k <= Nz; row padding excluded) are gathered on
// the device; if there are at most kMaxMaterials of them, `mat` (L.total bytes, padding left as
// is) receives each node's id and `tab` (kMaxMaterials x 4 floats) the tuples, and *nmat their
// count; otherwise *nmat = 0 and nothing else is written.  Synchronises `s`.
int build_material_index(const float *const coef[4], const Layout &L, unsigned char *mat, float *tab, int *nmat,
                         cudaStream_t s);
// Encode the tensor maps of `d`'s arrays for the staged kernel with `by` tile rows into host
// memory (kTmaSetBytes).
int encode_tma_set(const InstDesc &d, int by, void *host_out);

constexpr int kFaceCellsPerThread = 4;

// Work-list geometry for an instance under tile rows `by`, depth `kc` and `vec` x cells per thread
// (the three-argument form plans 128-wide tiles, vec = 4).
void plan_tiles(InstDesc &d, int by, int kc, int vec);
void plan_tiles(InstDesc &d, int by, int kc);
int face_tile_cells(int by);

// Launchers (asynchronous on `s`).
int launch_yee_step(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles,
                    int s_offset, int by, cudaStream_t s);
// Same, with `grid` CTAs looping over the tiles (0: one CTA per tile).
int launch_yee_step_grid(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles,
                         int s_offset, int by, int grid, cudaStream_t s);
// Same, for tiles planned with `vec` x cells per thread.
int launch_yee_step_v(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                      int by, int vec, int grid, cudaStream_t s);
// The staged variant (operands brought into shared memory by TMA tensor copies, `stages` planes
// in a ring; 128-wide tiles, vec == 4; every instance's `tma` set encoded for `by`).  *err is
// raised if a bounded wait expires.  With `work` (one zeroed counter per step offset), CTAs past
// the first wave take tiles in list order as they free up instead of a static stride.  With `mat`
// every instance carries a material index (and its map) and the coefficients come from its table.
// With `lazy` (material-index shapes), each CTA claims its next tile from `work` just before the
// ring needs it instead of when the current one starts (the single-instance solver's form).
int launch_yee_step_bulk(const InstDesc *d_insts, const int *d_tile0, int ninst, int total_tiles, int s_offset,
                         int by, int stages, int grid, int *err, cudaStream_t s, int *work = nullptr,
                         bool mat = false, bool lazy = false);
// The face H nodes (Hx at i = Nx, Hy at j = Ny, Hz at k = Nz) of every instance advanced by `len`
// steps from step offset s_offset in one launch; the staged kernel's tile lists leave them out
// (descriptors planned with face_tiles = 0).  d_face0: ninst + 1 prefix sums of face_nodes().
int launch_yee_faces_steps(const InstDesc *d_insts, const long long *d_face0, int ninst, long long total_faces,
                           int s_offset, int len, cudaStream_t s);
long long face_nodes(int nx, int ny, int nz);
// Cells per thread of the tile width that goes with `by` staged rows (plan_tiles' vec): 23-row
// tiles are 64 cells wide (2), all others 128 (4).
int yee_bulk_tile_vec(int by);
// Shared memory of a staged instantiation (0: no such kernel).
size_t yee_bulk_smem_bytes(int by, int stages, bool mat = false);
// CTAs of the staged kernel that fit on the whole GPU at once (0: no such kernel).
int yee_bulk_resident_ctas(int by, int stages, bool mat = false);
// Z depths (at most `n`, best first) whose tile count fills whole waves of `resident` CTAs with the
// least work per CTA: each CTA's cost is its planes plus the warm plane and the pipeline fill.
int balanced_depths(int nx, int ny, int nz, int by, int vec, int resident, int *out, int n);
// Z depths (at most `n`, shallowest first) that fill `resident` CTAs with whole layers of tiles
// and leave a thin last layer: the CTAs beyond those layers work through the last layer's tiles
// while the layers run, so every layer tile is shallower than one depth covering the grid.
int leftover_depths(int nx, int ny, int nz, int by, int vec, int resident, int *out, int n);
// CTAs of the step kernel with `by` rows (and `vec`) that fit on the whole GPU at once.
int yee_resident_ctas(int by);
int yee_resident_ctas(int by, int vec);
int launch_advance(InstDesc *d_insts, int ninst, int nsteps, cudaStream_t s);
int launch_pack_field(const float *src, int ex, int ey, int ez, const Layout &L, float *dst0,
                      float *dst1, cudaStream_t s);
int launch_unpack_field(const float *src, int ex, int ey, int ez, const Layout &L, float *dst,
                        cudaStream_t s);
int launch_pack_coef(const float *src, const Layout &L, float *dst, cudaStream_t s);
int launch_fill(float *dst, long long n, float v, cudaStream_t s);
int launch_field_ref(int field, const float *in0, const float *in1, const float *in2,
                     const ptk_fdtd_params &p, float *out, cudaStream_t s);
int launch_h_half(const float *const in[6], float *const out[3], const ptk_fdtd_params &p,
                  cudaStream_t s);
int launch_e_half(const float *const e_in[3], const float *const h_new[3], float *const out[3],
                  const ptk_fdtd_params &p, cudaStream_t s);

// Extents of field f (0..5) in the reference layout.
void field_extents(int f, int nx, int ny, int nz, int *ex, int *ey, int *ez);

// Kernel launch counter (all launches issued by this library, graph nodes counted per replay).
void count_launches(long long n);
void count_graph_launch(long long nodes);
void set_capturing(bool on);
long long launches_issued();

}  // namespace ptk
