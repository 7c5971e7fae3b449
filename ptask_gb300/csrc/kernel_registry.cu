// kernel_registry.cu -- registry of the native sm_103a task kernels.
//
// The reference resolves a task's kernel by JIT-compiling a PTX file (Runtime::GetCompiledKernel,
// ptask/PTaskRuntime.h:540 -> CUAccelerator::Compile, ptask/cuaccelerator.cpp:1324-1450) and the
// FDTD graph asks for entries of "fdtdMain.compute_10.ptx" (ptaskUnitTest/graphfdtd.cpp:469).  Here
// every kernel is linked into the library; a (file, entry) pair resolves by entry name only.
#include "ptk_internal.h"

#include <cstring>

namespace {

struct KernelInfo {
    const char *entry;
    int n_in, n_out, const_bytes;
};

// Ids are positions in this table.
const KernelInfo kKernels[] = {
    {"HxComputation", 3, 1, (int)sizeof(ptk_fdtd_params)},   // graphfdtd.cpp:478
    {"HyComputation", 3, 1, (int)sizeof(ptk_fdtd_params)},   // :503
    {"HzComputation", 3, 1, (int)sizeof(ptk_fdtd_params)},   // :526
    {"ExComputation", 3, 1, (int)sizeof(ptk_fdtd_params)},   // :550
    {"EyComputation", 3, 1, (int)sizeof(ptk_fdtd_params)},   // :573
    {"EzComputation", 3, 1, (int)sizeof(ptk_fdtd_params)},   // :596
    {"HStep", 6, 3, (int)sizeof(ptk_fdtd_params)},           // the three H tasks in one launch
    {"EStep", 6, 3, (int)sizeof(ptk_fdtd_params)},           // the three E tasks in one launch
    // Cyclic-graph half steps, in place, per-cell coefficients:
    //   FDTDHStep(Hx,Hy,Hz,Ex,Ey,Ez, Da,Db, FDTD_PARAMS)
    //   FDTDEStep(Ex,Ey,Ez,Hx,Hy,Hz, Ca,Cb, FDTD_PARAMS, SOURCE{i,j,k,n}, wave)
    {"FDTDHStep", 8, 6, (int)sizeof(ptk_fdtd_params)},
    {"FDTDEStep", 9, 6, (int)sizeof(ptk_fdtd_params) + 16},
};
const int kNumKernels = (int)(sizeof(kKernels) / sizeof(kKernels[0]));

bool ends_with(const char *s, const char *suf)
{
    const size_t a = strlen(s), b = strlen(suf);
    return a >= b && strcmp(s + a - b, suf) == 0;
}

}  // namespace

extern "C" {

int ptk_can_execute_kernel(const char *file)
{
    // CUDA kernel files (.ptx / .cu / .cubin names) are served by linked native kernels; graphics
    // (.hlsl) and OpenCL (.cl) kernels are not supported.
    if (!file) return 0;
    return (ends_with(file, ".ptx") || ends_with(file, ".cu") || ends_with(file, ".cubin")) ? 1 : 0;
}

int ptk_kernel_lookup(const char *file, const char *entry, int *kernel_id)
{
    (void)file;
    if (!entry || !kernel_id) return ptk::set_error(PTK_ERR_INVALID, "NULL argument");
    for (int q = 0; q < kNumKernels; ++q)
        if (strcmp(entry, kKernels[q].entry) == 0) {
            *kernel_id = q;
            return PTK_OK;
        }
    return ptk::set_error(PTK_ERR_NOTFOUND, "no native kernel registered for entry '%s'", entry);
}

int ptk_kernel_signature(int kernel_id, int *n_inputs, int *n_outputs, int *const_bytes)
{
    if (kernel_id < 0 || kernel_id >= kNumKernels)
        return ptk::set_error(PTK_ERR_NOTFOUND, "kernel id %d not registered", kernel_id);
    if (n_inputs) *n_inputs = kKernels[kernel_id].n_in;
    if (n_outputs) *n_outputs = kKernels[kernel_id].n_out;
    if (const_bytes) *const_bytes = kKernels[kernel_id].const_bytes;
    return PTK_OK;
}

}  // extern "C"
