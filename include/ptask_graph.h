/*
 * ptask_graph.h -- C ABI of the PTask FDTD graph (libptask_rt.so).
 *
 * These entry points build and drive the FDTD task graph through the PTask-compatible C++ runtime
 * (include/ptask/ptaskapi.h): Runtime::GetDatablockTemplate / CreatePort / Graph::AddTask /
 * AddInputChannel / AddInternalChannel / AddOutputChannel / Run, GraphInputChannel::Push,
 * GraphOutputChannel::Pull and Datablock::GetDataPointer, exactly as the reference's driver does
 * (ptaskUnitTest/graphfdtd.cpp:1008-1167).  They exist so that non-C++ callers (Python through ctypes,
 * any FFI) can run the graph with host buffers.  Plain C types only.
 *
 * Graph forms (`mode`):
 *   PTK_GRAPH_CYCLIC_FUSED     H-step and E-step tasks in a loop driven by an MF_GENERAL_ITERATOR meta
 *                              port (pattern of ptaskUnitTest/iteration.cpp:197-435); the scheduler
 *                              lowers the whole loop to the fused Yee-step kernel replayed as CUDA graphs.
 *   PTK_GRAPH_CYCLIC_CAPTURED  the same graph; the loop body (two half-step kernels) is captured once
 *                              as a CUDA graph and replayed.
 *   PTK_GRAPH_CYCLIC_TASKWISE  the same graph dispatched task by task (no loop lowering).
 *   PTK_GRAPH_UNROLLED         the reference's own structure: six per-field tasks per step, `steps`
 *                              steps unrolled (graphfdtd.cpp:448-739); scalar vacuum coefficients only.
 */
#ifndef PTASK_GRAPH_H
#define PTASK_GRAPH_H

#include "ptask_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PTK_GRAPH_CYCLIC_FUSED = 0,
    PTK_GRAPH_CYCLIC_CAPTURED = 1,
    PTK_GRAPH_CYCLIC_TASKWISE = 2,
    PTK_GRAPH_UNROLLED = 3
};

typedef struct ptk_fdtd_graph ptk_fdtd_graph;

typedef struct ptk_graph_stats {
    unsigned long long dispatches;        /* task dispatches executed one by one */
    unsigned long long kernel_launches;   /* kernels enqueued (lowered loops included) */
    unsigned long long cycles_lowered;    /* general-iteration loops run as a whole */
    unsigned long long cycle_iterations;  /* iterations inside lowered loops */
    unsigned long long graph_replays;     /* CUDA-graph launches of lowered loops */
    float last_cycle_ms;                  /* device time of the last lowered loop */
    float last_solve_ms;                  /* host wall time of the last ptk_fdtd_graph_solve */
    unsigned long long host_dispatches;   /* of the dispatches, host tasks */
} ptk_graph_stats;

/* Build the FDTD graph for grid p (Graph construction of graphfdtd.cpp:448-739, or its cyclic form)
 * and start it (Graph::Run, ptask/graph.h:216).  `unrolled_steps` is the number of unrolled steps
 * for PTK_GRAPH_UNROLLED and ignored otherwise. */
int ptk_fdtd_graph_create(const ptk_fdtd_params *p, int mode, int unrolled_steps, ptk_fdtd_graph **out);

/* The unrolled graph with host tasks (hosttask.h:28-31): the tasks of every field whose bit is set
 * in `host_fields` (bit f = field f, PTK_HX..PTK_EZ) run the entry points HxComputation ..
 * EzComputation of the shared library `library` ("x.so", or a reference-style "x.dll" name, looked up
 * as x.dll, x.so and libx.so), called as void f(unsigned n, void **args) with args = (in0, in1, in2,
 * &FDTD_PARAMS, out) as host pointers; the other fields' tasks run on the GPU.  Blocks move between
 * host and device as the tasks that read them need.  PTK_ERR_NOTFOUND: library or entry missing. */
int ptk_fdtd_graph_create_host(const ptk_fdtd_params *p, int unrolled_steps, const char *library,
                               unsigned host_fields, ptk_fdtd_graph **out);

/* The same graph with host tasks that use the GPU as a dependent accelerator (hosttask.h:33-144,
 * task.h:768 BindDependentAcceleratorClass, port.h:1185 BindDependentAccelerator): each host task is
 * bound to the CUDA class, and its three field inputs and its output to the dependent device, so
 * the entry point receives device pointers for them and a host pointer for FDTD_PARAMS.
 * with_streams = 0: entry points have the LPFNDEPHOSTTASK form
 *   void f(unsigned n, void **args, int *is_dependent, void **device_bindings, unsigned ndeps, void **deps)
 * and the runtime waits for the device before and after each call;
 * with_streams = 1: entry points have the LPFNDEPHOSTTASKEX form void f(DEPENDENTCONTEXT *) and order
 * their work on pStreams[0] (a cudaStream_t), with no host wait.  PTK_ERR_NOTFOUND: library or entry
 * missing. */
int ptk_fdtd_graph_create_dephost(const ptk_fdtd_params *p, int unrolled_steps, const char *library,
                                  unsigned host_fields, int with_streams, ptk_fdtd_graph **out);

/* Push the sticky inputs: per-cell coefficients (Nx*Ny*Nz floats each; all NULL = scalar vacuum
 * coefficients Dt/eps0, Dt/mu0 as in the reference) and the soft Ez source (si<0 or wave NULL = none). */
int ptk_fdtd_graph_set_problem(ptk_fdtd_graph *g, const float *Ca, const float *Cb, const float *Da,
                               const float *Db, int si, int sj, int sk, const float *wave, int nwave);

/* Push the six fields (host, reference layout) and the iteration count, pull the six results into
 * the same arrays (GraphInputChannel::Push / GraphOutputChannel::Pull, graphfdtd.cpp:1074-1127).
 * For PTK_GRAPH_UNROLLED, `steps` must equal the unrolled step count. */
int ptk_fdtd_graph_solve(ptk_fdtd_graph *g, float *const fields[6], int steps);

/* Push `instances` copies of the six fields back to back and pull every result (the reference's
 * numBlocks pipelining, graphfdtd.cpp:1076-1127); results[i*6+f] receives instance i, field f. */
int ptk_fdtd_graph_solve_many(ptk_fdtd_graph *g, float *const fields[6], int instances,
                              float *const results[], int steps);

int ptk_fdtd_graph_stats(const ptk_fdtd_graph *g, ptk_graph_stats *st);
/* Graph::WriteDOTFile (ptask/graph.h:884). */
int ptk_fdtd_graph_write_dot(ptk_fdtd_graph *g, const char *path);
/* Graph::Stop, Teardown, DestroyGraph (ptask/graph.h:234, :242, :122). */
int ptk_fdtd_graph_destroy(ptk_fdtd_graph *g);

/* ---- graph files (Graph::Serialize / Graph::Deserialize, ptask/graph.h:1545, :1561) ----------
 * The file holds the graph's structure in the reference's XML layout (ptask/XMLWriter.cpp,
 * XMLReader.cpp): templates, kernels, tasks and ports, channels and configuration actions. */

/* Write the running graph's structure.  PTK_ERR_STATE if the file cannot be written. */
int ptk_fdtd_graph_save(ptk_fdtd_graph *g, const char *path);

/* Build and start an FDTD graph from a file written by ptk_fdtd_graph_save or by the reference's
 * Graph::Serialize.  The file decides the structure (unrolled per-field tasks or the cyclic pair);
 * for a cyclic file `mode` chooses the lowering (FUSED, CAPTURED or TASKWISE) and
 * PTK_GRAPH_UNROLLED is rejected.  `p` supplies FDTD_PARAMS, which a graph file does not hold; the
 * field templates in the file must match its grid.  Boundary channels are found by the template and
 * variable binding of their ports.  PTK_ERR_STATE: unreadable or malformed file;
 * PTK_ERR_INVALID: not an FDTD graph for this grid. */
int ptk_fdtd_graph_load(const ptk_fdtd_params *p, int mode, const char *path, ptk_fdtd_graph **out);

/* Write the structure of the graph ptk_fdtd_graph_create would build, without starting it (no
 * device needed). */
int ptk_fdtd_graph_export(const ptk_fdtd_params *p, int mode, int unrolled_steps, const char *path);

/* Read any graph file into a new graph and write it out again (no device needed): the output
 * equals the input for files written by this runtime. */
int ptk_graph_xml_roundtrip(const char *in_path, const char *out_path);

#ifdef __cplusplus
}
#endif
#endif
