/*
 * fdtd_dephosttasks.c -- TEST INFRASTRUCTURE: host tasks that use the GPU as a dependent
 * accelerator (ptask/hosttask.h:33-144).  Each entry point receives the three field inputs and the
 * output as device pointers (bound to the dependent device) and FDTD_PARAMS as a host pointer, and
 * runs the per-field update (graphfdtd.cpp:185-312) on the GPU through the product's C ABI
 * (ptk_launch_field_update).  Built twice by the tests: by default with the LPFNDEPHOSTTASKEX form
 * (a DEPENDENTCONTEXT with the stream to order the work on), with -DPTK_LEGACY_FORM with the
 * LPFNDEPHOSTTASK form (no stream: the launch goes to the library's own stream and the runtime waits
 * for the device around the call).  An entry point that finds an argument bound where it does not
 * expect it launches nothing, so the graph's result is wrong and the test fails.
 */
#include "ptask_gb300.h"

/* Same member order and types as DEPENDENTCONTEXT (include/ptask/ptask_core.h). */
typedef struct {
    unsigned cbDependentContext, nArguments, nDependentAccelerators, uiReserved0;
    void **ppArguments;
    void **ppDatablocks;
    int *pbIsDependentBinding;
    void **pvDeviceBindings;
    void **pDependentDevices;
    void **pStreams;
    char *lpszTaskName;
} dep_context;

static void run(int f, unsigned n, void **a, const int *dep, unsigned ndeps, void *stream)
{
    if (n != 5 || ndeps != 1 || !dep[0] || !dep[1] || !dep[2] || dep[3] || !dep[4]) return;
    ptk_launch_field_update(f, (const float *)a[0], (const float *)a[1], (const float *)a[2],
                            (const ptk_fdtd_params *)a[3], (float *)a[4], stream);
}

#ifdef PTK_LEGACY_FORM
#define ENTRY(NAME, F)                                                                               \
    void NAME(unsigned n, void **a, int *dep, void **bindings, unsigned ndeps, void **deps)         \
    {                                                                                                \
        (void)bindings;                                                                              \
        (void)deps;                                                                                  \
        run(F, n, a, dep, ndeps, 0);                                                                 \
    }
#else
#define ENTRY(NAME, F)                                                                               \
    void NAME(dep_context *c)                                                                        \
    {                                                                                                \
        if (c->cbDependentContext != sizeof(dep_context)) return;                                    \
        run(F, c->nArguments, c->ppArguments, c->pbIsDependentBinding, c->nDependentAccelerators,    \
            c->pStreams[0]);                                                                         \
    }
#endif

ENTRY(HxComputation, PTK_HX)
ENTRY(HyComputation, PTK_HY)
ENTRY(HzComputation, PTK_HZ)
ENTRY(ExComputation, PTK_EX)
ENTRY(EyComputation, PTK_EY)
ENTRY(EzComputation, PTK_EZ)
