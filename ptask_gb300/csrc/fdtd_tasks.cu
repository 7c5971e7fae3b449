// fdtd_tasks.cu -- the two half-step task kernels of the cyclic FDTD graph, over dense
// reference-layout blocks, plus CUDA-graph capture entry points used by the PTask scheduler.
//
// Both half steps are safe in place: a new H value depends only on the old H value of the same
// node and on E; a new E value only on the old E value of the same node and on H.  The cyclic graph
// therefore circulates one datablock per field through in-out ports, with no allocation per step
// (the reference allocates a new output block per task dispatch, OutputPort.cpp:536).
#include "ptk_internal.h"

namespace ptk {

__device__ __forceinline__ float yee_c(float d, float h, float c, float a1, float a0, float s1, float b1,
                                       float b0, float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(__fmul_rn(d, h), __fmul_rn(c, curl));
}

#define D3(ii, jj, kk, d1, d2) ((long long)(ii) + (long long)(d1) * (jj) + (long long)(d1) * (d2) * (kk))

// Cell index of node (i,j,k) for per-cell coefficient arrays (Nx,Ny,Nz): wall nodes use the
// nearest cell.
__device__ __forceinline__ long long cell(int i, int j, int k, int Nx, int Ny, int Nz)
{
    return D3(min(i, Nx - 1), min(j, Ny - 1), min(k, Nz - 1), Nx, Ny);
}

__global__ void k_h_step_coef(float *__restrict__ Hx, float *__restrict__ Hy, float *__restrict__ Hz,
                              const float *__restrict__ Ex, const float *__restrict__ Ey,
                              const float *__restrict__ Ez, const float *__restrict__ Da,
                              const float *__restrict__ Db, ptk_fdtd_params p)
{
    const int Nx = p.Nx, Ny = p.Ny, Nz = p.Nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i <= Nx && j < Ny && k < Nz) {
        const long long o = D3(i, j, k, Nx + 1, Ny), c = cell(i, j, k, Nx, Ny, Nz);
        Hx[o] = yee_c(Da[c], Hx[o], Db[c], Ey[D3(i, j, k + 1, Nx + 1, Ny)], Ey[D3(i, j, k, Nx + 1, Ny)], p.Cz,
                      Ez[D3(i, j + 1, k, Nx + 1, Ny + 1)], Ez[D3(i, j, k, Nx + 1, Ny + 1)], p.Cy);
    }
    if (i < Nx && j <= Ny && k < Nz) {
        const long long o = D3(i, j, k, Nx, Ny + 1), c = cell(i, j, k, Nx, Ny, Nz);
        Hy[o] = yee_c(Da[c], Hy[o], Db[c], Ez[D3(i + 1, j, k, Nx + 1, Ny + 1)], Ez[D3(i, j, k, Nx + 1, Ny + 1)],
                      p.Cx, Ex[D3(i, j, k + 1, Nx, Ny + 1)], Ex[D3(i, j, k, Nx, Ny + 1)], p.Cz);
    }
    if (i < Nx && j < Ny && k <= Nz) {
        const long long o = D3(i, j, k, Nx, Ny), c = cell(i, j, k, Nx, Ny, Nz);
        Hz[o] = yee_c(Da[c], Hz[o], Db[c], Ex[D3(i, j + 1, k, Nx, Ny + 1)], Ex[D3(i, j, k, Nx, Ny + 1)], p.Cy,
                      Ey[D3(i + 1, j, k, Nx + 1, Ny)], Ey[D3(i, j, k, Nx + 1, Ny)], p.Cx);
    }
}

__global__ void k_e_step_coef(float *__restrict__ Ex, float *__restrict__ Ey, float *__restrict__ Ez,
                              const float *__restrict__ Hx, const float *__restrict__ Hy,
                              const float *__restrict__ Hz, const float *__restrict__ Ca,
                              const float *__restrict__ Cb, ptk_fdtd_params p, long long src,
                              const float *__restrict__ wave, int nwave, int *__restrict__ counter)
{
    const int Nx = p.Nx, Ny = p.Ny, Nz = p.Nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i < Nx && j >= 1 && j <= Ny - 1 && k >= 1 && k <= Nz - 1) {
        const long long o = D3(i, j, k, Nx, Ny + 1), c = D3(i, j, k, Nx, Ny);
        Ex[o] = yee_c(Ca[c], Ex[o], Cb[c], Hz[D3(i, j, k, Nx, Ny)], Hz[D3(i, j - 1, k, Nx, Ny)], p.Cy,
                      Hy[D3(i, j, k, Nx, Ny + 1)], Hy[D3(i, j, k - 1, Nx, Ny + 1)], p.Cz);
    }
    if (i >= 1 && i <= Nx - 1 && j < Ny && k >= 1 && k <= Nz - 1) {
        const long long o = D3(i, j, k, Nx + 1, Ny), c = D3(i, j, k, Nx, Ny);
        Ey[o] = yee_c(Ca[c], Ey[o], Cb[c], Hx[D3(i, j, k, Nx + 1, Ny)], Hx[D3(i, j, k - 1, Nx + 1, Ny)], p.Cz,
                      Hz[D3(i, j, k, Nx, Ny)], Hz[D3(i - 1, j, k, Nx, Ny)], p.Cx);
    }
    if (i >= 1 && i <= Nx - 1 && j >= 1 && j <= Ny - 1 && k < Nz) {
        const long long o = D3(i, j, k, Nx + 1, Ny + 1), c = D3(i, j, k, Nx, Ny);
        float v = yee_c(Ca[c], Ez[o], Cb[c], Hy[D3(i, j, k, Nx, Ny + 1)], Hy[D3(i - 1, j, k, Nx, Ny + 1)], p.Cx,
                        Hx[D3(i, j, k, Nx + 1, Ny)], Hx[D3(i, j - 1, k, Nx + 1, Ny)], p.Cy);
        if (o == src && counter) {
            // Only this thread touches the counter, so the read-modify-write needs no atomics.
            const int n = *counter;
            if (n < nwave) v = __fadd_rn(v, wave[n]);
            *counter = n + 1;
        }
        Ez[o] = v;
    }
}
#undef D3

}  // namespace ptk

using namespace ptk;

static inline cudaStream_t S(void *s) { return s ? (cudaStream_t)s : default_stream(); }

extern "C" {

int ptk_launch_h_step_coef(float *const h[3], const float *const e[3], const float *Da, const float *Db,
                           const ptk_fdtd_params *p, void *stream)
{
    PTK_CHECK_ARG(h && e && Da && Db && p, "NULL argument");
    PTK_CHECK_ARG(p->Nx >= 1 && p->Ny >= 1 && p->Nz >= 1, "bad grid");
    int rc = ensure_init();
    if (rc) return rc;
    dim3 grid((p->Nx + 1 + 127) / 128, p->Ny + 1, p->Nz + 1);
    k_h_step_coef<<<grid, 128, 0, S(stream)>>>(h[0], h[1], h[2], e[0], e[1], e[2], Da, Db, *p);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int ptk_launch_e_step_coef(float *const e[3], const float *const h[3], const float *Ca, const float *Cb,
                           const ptk_fdtd_params *p, int si, int sj, int sk, const float *wave, int nwave,
                           int *step_counter, void *stream)
{
    PTK_CHECK_ARG(e && h && Ca && Cb && p, "NULL argument");
    PTK_CHECK_ARG(p->Nx >= 1 && p->Ny >= 1 && p->Nz >= 1, "bad grid");
    int rc = ensure_init();
    if (rc) return rc;
    long long src = -1;
    if (wave && nwave > 0 && step_counter) {
        PTK_CHECK_ARG(si >= 1 && si < p->Nx && sj >= 1 && sj < p->Ny && sk >= 0 && sk < p->Nz,
                      "source node (%d,%d,%d) must be an interior Ez node", si, sj, sk);
        src = (long long)si + (long long)(p->Nx + 1) * sj + (long long)(p->Nx + 1) * (p->Ny + 1) * sk;
    }
    dim3 grid((p->Nx + 1 + 127) / 128, p->Ny + 1, p->Nz + 1);
    k_e_step_coef<<<grid, 128, 0, S(stream)>>>(e[0], e[1], e[2], h[0], h[1], h[2], Ca, Cb, *p, src, wave,
                                                nwave, src >= 0 ? step_counter : nullptr);
    PTK_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return PTK_OK;
}

int ptk_capture_begin(void *stream)
{
    PTK_CHECK_ARG(stream, "capture needs an explicit stream");
    PTK_CUDA_TRY(cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    return PTK_OK;
}

int ptk_capture_end(void *stream, void **graph_exec)
{
    PTK_CHECK_ARG(stream && graph_exec, "NULL argument");
    set_capturing(false);
    cudaGraph_t g = nullptr;
    PTK_CUDA_TRY(cudaStreamEndCapture((cudaStream_t)stream, &g));
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(PTK_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    *graph_exec = ex;
    return PTK_OK;
}

int ptk_graph_exec_launch(void *graph_exec, void *stream, long long kernel_nodes)
{
    PTK_CHECK_ARG(graph_exec, "NULL graph");
    PTK_CUDA_TRY(cudaGraphLaunch((cudaGraphExec_t)graph_exec, S(stream)));
    count_graph_launch(kernel_nodes);
    return PTK_OK;
}

int ptk_graph_exec_destroy(void *graph_exec)
{
    if (!graph_exec) return PTK_OK;
    PTK_CUDA_TRY(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec));
    return PTK_OK;
}

}  // extern "C"
