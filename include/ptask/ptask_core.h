// ptask_core.h -- the PTask object model of the GB300 runtime: templates, datablocks, ports,
// channels, tasks and graphs.  The public headers named after the reference's (graph.h, task.h,
// channel.h, datablock.h, ...) include this file, so code written against ptask/ptaskapi.h compiles
// against it unchanged.
//
// Execution model (GB300-first, not the reference's):
//   * One scheduler thread per running graph (or the caller's thread in single-threaded mode) finds
//     ready tasks and dispatches them.  A dispatch binds device views of its input blocks, takes
//     output blocks from the device pool, and enqueues the task's native sm_103a kernel on the
//     graph's CUDA stream through the C ABI (include/ptask_gb300.h).  Nothing waits on the GPU
//     between dispatches: ordering is stream order.  (Reference: one runner thread per task,
//     Task::Execute/Dispatch task.cpp:1596/3822, Scheduler.cpp:4551, one CUstream per task.)
//   * Datablocks live in HBM; a host view is made only for AllocateDatablock's initial data and on
//     GetDataPointer / EAGER output materialisation.  (Reference: MSI coherence over memory spaces,
//     datablock.cpp:2235.)
//   * Iteration: when a MF_GENERAL_ITERATOR loop (MetaPort.cpp:927-1011) can be run as a whole, the
//     scheduler lowers the loop body to a CUDA graph and replays it (or to a registered fused
//     lowering, e.g. the Yee step solver) instead of dispatching task by task.
#ifndef PTASK_GB300_CORE_H
#define PTASK_GB300_CORE_H

#include <atomic>
#include <condition_variable>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "primitive_types.h"

namespace PTask {

class Graph;
class Task;
class Port;
class Channel;
class Datablock;
class DatablockTemplate;
class CompiledKernel;
class Accelerator;
struct CyclePlan;

// Recursive lock with the reference's Lock/Unlock interface (ptask/Lockable.h:56-66).
class Lockable {
public:
    virtual ~Lockable() {}
    int Lock()
    {
        m_lock.lock();
        return ++m_depth;
    }
    int Unlock()
    {
        int d = --m_depth;
        m_lock.unlock();
        return d;
    }
    BOOL LockIsHeld() { return m_depth > 0; }

protected:
    std::recursive_mutex m_lock;
    std::atomic<int> m_depth{0};
};

// ---------------------------------------------------------------------------------------------
class DatablockTemplate : public Lockable {
public:
    DatablockTemplate(const char *name, UINT stride, UINT x, UINT y, UINT z, bool record, bool raw);
    DatablockTemplate(const char *name, UINT stride, PTASK_PARM_TYPE type);
    const char *GetTemplateName() { return m_name.c_str(); }
    UINT GetStride() { return m_stride; }
    UINT GetXElementCount() { return m_dims[0]; }
    UINT GetYElementCount() { return m_dims[1]; }
    UINT GetZElementCount() { return m_dims[2]; }
    UINT GetDatablockByteCount() { return m_stride * m_dims[0] * m_dims[1] * m_dims[2]; }
    PTASK_PARM_TYPE GetParameterBaseType() { return m_parm; }
    BOOL DescribesScalarParameter() { return m_parm != PTPARM_BUFFER && m_parm != PTPARM_NONE; }
    BOOL IsRecordStream() { return m_record; }
    BOOL IsByteAddressable() { return m_raw; }

private:
    std::string m_name;
    UINT m_stride;
    UINT m_dims[3];
    PTASK_PARM_TYPE m_parm;
    bool m_record, m_raw;
};

// ---------------------------------------------------------------------------------------------
// A reference-counted block of data.  The device copy is authoritative once a kernel has written
// it; the host copy (pinned) is made valid on demand.
class Datablock : public Lockable {
public:
    Datablock(DatablockTemplate *t, size_t bytes, CONTROLSIGNAL sig);
    virtual ~Datablock();

    long AddRef();
    long Release();
    long RefCount() { return m_refs.load(); }

    // Host view.  bWriteable invalidates the device copy.  (datablock.h:1544)
    void *GetDataPointer(BOOL bWriteable, BOOL bSynchronizeBufferView = TRUE);
    UINT GetDataBufferLogicalSizeBytes() { return (UINT)m_bytes; }
    UINT GetDataBufferAllocatedSizeBytes() { return (UINT)m_bytes; }
    DatablockTemplate *GetTemplate() { return m_template; }
    CONTROLSIGNAL GetControlSignals() { return m_signals; }
    BOOL TestControlSignal(CONTROLSIGNAL s) { return TESTSIGNAL(m_signals, s); }
    void SetControlSignal(CONTROLSIGNAL s) { m_signals |= s; }
    void ClearControlSignal(CONTROLSIGNAL s) { m_signals &= ~s; }
    void ClearAllControlSignals() { m_signals = DBCTLC_NONE; }
    void SetRecordCount(UINT n) { m_records = n; }
    UINT GetRecordCount() { return m_records; }
    UINT GetDBUID() { return m_uid; }
    BOOL IsScalarParameter() { return m_template && m_template->DescribesScalarParameter(); }

    // ---- runtime side (not part of the reference API) ----
    void *DeviceView(void *stream, bool for_write, bool keep_contents);   // device pointer, valid on `stream`
    void DeviceWritten(void *stream);                                      // a kernel on `stream` wrote it
    void StartHostMaterialization(void *stream);                           // EAGER: async D2H
    // Whole-block copies straight between caller memory (pinned or not) and the device view, with
    // no host view in between: for blocks that live on the device (pushed fields, pulled results).
    void UploadFrom(const void *src);     // pageable src: reusable on return; pinned: once consumed
    void DownloadTo(void *dst);           // from the host view if it is (being) materialised
    const void *HostBytes();                                               // host copy without syncing (params)
    size_t Bytes() const { return m_bytes; }

private:
    void ensure_host_alloc();
    void sync_host();

    DatablockTemplate *m_template;
    size_t m_bytes;
    std::atomic<long> m_refs{1};
    CONTROLSIGNAL m_signals;
    UINT m_records = 0;
    UINT m_uid;
    void *m_host = nullptr;        // pinned
    void *m_dev = nullptr;         // pool
    void *m_dev_stream = nullptr;  // stream the device copy was last written on
    void *m_event = nullptr;       // recorded after the last device write / pending D2H
    bool m_host_valid = false;
    bool m_dev_valid = false;
    bool m_d2h_pending = false;
};

// ---------------------------------------------------------------------------------------------
class Port : public Lockable {
public:
    Port(PORTTYPE t, DatablockTemplate *tmpl, UINT uid, const char *name, int param_idx, int inout_idx);
    virtual ~Port();
    PORTTYPE GetPortType() { return m_type; }
    DatablockTemplate *GetTemplate() { return m_template; }
    const char *GetVariableBinding() { return m_name.c_str(); }
    UINT GetUID() { return m_uid; }
    Task *GetTask() { return m_task; }
    UINT GetFormalParameterIndex() { return (UINT)m_param_idx; }
    int GetInOutRoutingIndex() { return m_inout_idx; }
    BOOL IsInOutParameter() { return m_inout_idx >= 0; }
    BOOL IsSticky() { return m_type == STICKY_PORT; }
    // Dependent-accelerator binding (port.h:1185-1248): the block bound to this port of a host task
    // is materialised in the memory space of the task's dependent accelerator (a device pointer)
    // instead of host memory.  nIndex picks one of the task's dependent accelerators.
    void BindDependentAccelerator(ACCELERATOR_CLASS cls, int nIndex)
    {
        m_dep_class = cls;
        m_dep_index = nIndex;
    }
    BOOL HasDependentAcceleratorBinding() { return m_dep_class != ACCELERATOR_CLASS_UNKNOWN; }
    int GetDependentAcceleratorIndex() { return m_dep_index; }
    ACCELERATOR_CLASS GetDependentAcceleratorClass() { return m_dep_class; }
    void SetMetaFunction(METAFUNCTION f) { m_meta = f; }
    METAFUNCTION GetMetaFunction() { return m_meta; }
    void SetSticky(BOOL b) { m_sticky_flag = b; }
    BOOL IsOccupied();
    UINT GetChannelCount() { return (UINT)(m_type == OUTPUT_PORT ? m_out.size() : m_in.size()); }
    // Position in the port array passed to Graph::AddTask (port.h GetOriginalIndex/SetOriginalIndex).
    UINT GetOriginalIndex() { return m_orig_idx; }
    void SetOriginalIndex(UINT i) { m_orig_idx = i; }
    Channel *GetChannel(UINT i);

    // ---- runtime side ----
    ACCELERATOR_CLASS m_dep_class = ACCELERATOR_CLASS_UNKNOWN;   // dependent binding, if any
    int m_dep_index = -1;
    std::vector<Channel *> m_in;         // channels feeding an input-side port
    std::vector<Channel *> m_out;        // channels fed by an output port
    std::vector<Port *> m_ctl_targets;   // control propagation (BindControlPropagationPort)
    Datablock *m_sticky = nullptr;       // retained block of a sticky port
    Port *m_inout_partner = nullptr;     // output port that forwards this input's block
    Task *m_task = nullptr;

private:
    PORTTYPE m_type;
    DatablockTemplate *m_template;
    UINT m_uid;
    std::string m_name;
    int m_param_idx;
    int m_inout_idx;
    METAFUNCTION m_meta = MF_NONE;
    BOOL m_sticky_flag = FALSE;
    UINT m_orig_idx = 0;
};

class InputPort : public Port {
public:
    using Port::Port;
};
class OutputPort : public Port {
public:
    using Port::Port;
};
class StickyPort : public Port {
public:
    using Port::Port;
};
class MetaPort : public Port {
public:
    using Port::Port;
};
class InitializerPort : public Port {
public:
    using Port::Port;
};

// ---------------------------------------------------------------------------------------------
class Channel : public Lockable {
public:
    Channel(Graph *g, CHANNELTYPE t, Port *src, Port *dst, const char *name, BOOL is_switch);
    virtual ~Channel();
    // Push blocks until there is capacity (or the timeout in ms expires). (channel.h:379)
    virtual BOOL Push(Datablock *pBlock, DWORD dwTimeout = 0xFFFFFFFF);
    // Pull blocks until a block is available (or the timeout expires, returning NULL). (channel.h:353)
    virtual Datablock *Pull(DWORD dwTimeout = 0xFFFFFFFF);
    Datablock *Peek();
    BOOL IsReady();
    UINT GetQueueDepth();
    UINT GetCapacity() { return m_capacity; }
    void SetCapacity(UINT n) { m_capacity = n; }
    void SetNoDraw() { m_draw = false; }
    bool ShouldDraw() { return m_draw; }
    void SetViewMaterializationPolicy(VIEWMATERIALIZATIONPOLICY p) { m_view = p; }
    VIEWMATERIALIZATIONPOLICY GetViewMaterializationPolicy() { return m_view; }
    void SetPredicationType(CHANNELENDPOINTTYPE e, CHANNELPREDICATE p, BOOL bCanonical = TRUE);
    CHANNELPREDICATE GetPredicationType(CHANNELENDPOINTTYPE e) { return m_pred[e]; }
    CHANNELTYPE GetType() { return m_type; }
    const char *GetName() { return m_name.c_str(); }
    Port *GetBoundPort(CHANNELENDPOINTTYPE e) { return e == CE_SRC ? m_src : m_dst; }
    DatablockTemplate *GetTemplate();
    BOOL IsSwitchChannel() { return m_switch; }
    void SetTimeout(DWORD ms) { m_timeout = ms; }

    // ---- runtime side ----
    bool PassesPredicate(CHANNELENDPOINTTYPE e, Datablock *b);
    bool Enqueue(Datablock *b, DWORD timeout_ms);   // producer side (adds a reference)
    Datablock *Dequeue();                           // consumer side (transfers the reference)
    void Drain();

protected:
    Graph *m_graph;
    CHANNELTYPE m_type;
    Port *m_src, *m_dst;
    std::string m_name;
    BOOL m_switch;
    std::deque<Datablock *> m_q;
    UINT m_capacity;
    bool m_draw = true;
    VIEWMATERIALIZATIONPOLICY m_view = VIEWMATERIALIZATIONPOLICY_ON_DEMAND;
    CHANNELPREDICATE m_pred[2] = {CGATEFN_NONE, CGATEFN_NONE};
    DWORD m_timeout = 0xFFFFFFFF;
    std::condition_variable_any m_cv;
};

class GraphInputChannel : public Channel {
public:
    using Channel::Channel;
};
class GraphOutputChannel : public Channel {
public:
    using Channel::Channel;
};
class InternalChannel : public Channel {
public:
    using Channel::Channel;
};
class InitializerChannel : public Channel {
public:
    using Channel::Channel;
};
class MultiChannel : public Channel {
public:
    using Channel::Channel;
};

// ---------------------------------------------------------------------------------------------
// Host-task entry point (hosttask.h:28-31): called with the task's formal parameters as host
// pointers, in parameter-index order.  (__stdcall has no meaning on the platforms this runs on.)
typedef void (*LPFNHOSTTASK)(UINT nArguments, void **ppArguments);

// Host tasks that use a dependent accelerator (hosttask.h:45-144).  Arguments bound to ports with a
// dependent binding are device pointers (pbIsDependentBinding[i] TRUE, pvDeviceBindings[i] the
// device's ordinal as a pointer-sized integer); the others are host pointers.  pDeps / the
// context's pDependentDevices list the dependent devices (one: the runtime's GPU).
typedef void (*LPFNDEPHOSTTASK)(UINT nArguments, void **ppArguments, BOOL *pbIsDependentBinding,
                                void **pvDeviceBindings, UINT nDeps, void **pDeps);

// Descriptor form, chosen when the task asked for platform-specific objects
// (BindDependentAcceleratorClass(..., bRequestDependentPSObjects = TRUE)).  Same member order and
// types as the reference's DEPENDENTCONTEXT, so entry points written for it read it unchanged;
// pStreams[0] is the CUDA stream (cudaStream_t) the task's work must be ordered on.
typedef struct _dependent_context_t {
    UINT cbDependentContext;       // sizeof(DEPENDENTCONTEXT)
    UINT nArguments;
    UINT nDependentAccelerators;
    UINT uiReserved0;
    void **ppArguments;
    Datablock **ppDatablocks;      // the block behind each argument
    BOOL *pbIsDependentBinding;
    void **pvDeviceBindings;
    void **pDependentDevices;
    void **pStreams;
    char *lpszTaskName;
} DEPENDENTCONTEXT, *LPDEPENDENTCONTEXT;
typedef void (*LPFNDEPHOSTTASKEX)(LPDEPENDENTCONTEXT);

// A (file, entry) pair resolved to a linked native kernel, or to a host function exported by a
// shared library (CompiledKernel.h; hostaccelerator.cpp:328-380 for the host case).
class CompiledKernel {
public:
    CompiledKernel(const char *file, const char *entry, int id) : m_file(file), m_entry(entry), m_id(id) {}
    CompiledKernel(const char *file, const char *entry, LPFNHOSTTASK fn)
        : m_file(file), m_entry(entry), m_id(-1), m_host(fn) {}
    const char *GetSourceFile() { return m_file.c_str(); }
    const char *GetOperation() { return m_entry.c_str(); }
    int NativeId() const { return m_id; }
    bool IsHost() const { return m_host != nullptr; }
    LPFNHOSTTASK HostFunction() const { return m_host; }

private:
    std::string m_file, m_entry;
    int m_id;
    LPFNHOSTTASK m_host = nullptr;
};

// ---------------------------------------------------------------------------------------------
class Task : public Lockable {
public:
    Task(Graph *g, CompiledKernel *k, const char *name);
    virtual ~Task();
    void SetComputeGeometry(int x = 1, int y = 1, int z = 1);
    void SetBlockAndGridSize(PTASKDIM3 grid, PTASKDIM3 block);
    const char *GetTaskName() { return m_name.c_str(); }
    ACCELERATOR_CLASS GetAcceleratorClass()
    {
        return m_kernel && m_kernel->IsHost() ? ACCELERATOR_CLASS_HOST : ACCELERATOR_CLASS_CUDA;
    }
    // Dependent accelerators of a host task (task.h:768-800): the scheduler gives the task an
    // accelerator of class `cls` besides the host.  With bRequestDependentPSObjects the entry point
    // has the LPFNDEPHOSTTASKEX form and receives streams; otherwise LPFNDEPHOSTTASK.  Only the
    // CUDA class, one instance, is supported (one GPU per runtime); anything else fails.
    BOOL BindDependentAcceleratorClass(ACCELERATOR_CLASS cls, int nRequiredInstances, BOOL bRequestDependentPSObjects);
    int GetDependentBindingClassCount() { return m_dep_class == ACCELERATOR_CLASS_UNKNOWN ? 0 : 1; }
    BOOL HasDependentAcceleratorBindings() { return GetDependentBindingClassCount() > 0; }
    BOOL DependentBindingsRequirePSObjects() { return m_dep_ps; }
    ACCELERATOR_CLASS GetDependentAcceleratorClass(int) { return m_dep_class; }
    Graph *GetGraph() { return m_graph; }
    CompiledKernel *GetCompiledKernel() { return m_kernel; }
    UINT GetInputPortCount() { return (UINT)m_inputs.size(); }
    UINT GetOutputPortCount() { return (UINT)m_outputs.size(); }
    Port *GetInputPort(UINT i) { return i < m_inputs.size() ? m_inputs[i] : nullptr; }
    Port *GetOutputPort(UINT i) { return i < m_outputs.size() ? m_outputs[i] : nullptr; }
    UINT64 GetDispatchCount() { return m_dispatches; }

    // ---- runtime side ----
    std::vector<Port *> m_inputs;
    std::vector<Port *> m_outputs;
    PTASKDIM3 m_geom, m_grid, m_block;
    bool m_geom_set = false;
    bool m_explicit_launch = false;
    UINT64 m_dispatches = 0;
    // MF_GENERAL_ITERATOR state of a meta port on this task
    Datablock *m_iter_block = nullptr;
    UINT m_iter_max = 0, m_iter_count = 0;
    void *m_step_counter = nullptr;   // device int used by kernels that index a waveform by step
    CyclePlan *m_loop_top = nullptr;     // this task heads a general-iteration loop
    CyclePlan *m_loop_bottom = nullptr;  // this task owns the loop's MF_GENERAL_ITERATOR port
    ACCELERATOR_CLASS m_dep_class = ACCELERATOR_CLASS_UNKNOWN;   // dependent accelerator class
    BOOL m_dep_ps = FALSE;               // entry point wants DEPENDENTCONTEXT (streams)

private:
    Graph *m_graph;
    CompiledKernel *m_kernel;
    std::string m_name;
};

// ---------------------------------------------------------------------------------------------
struct GraphStats {
    UINT64 dispatches = 0;         // task dispatches executed one by one
    UINT64 host_dispatches = 0;    // of which host tasks (entry points of a shared library)
    UINT64 kernel_launches = 0;    // kernels enqueued by dispatches
    UINT64 cycles_lowered = 0;     // iteration loops run as a captured / fused whole
    UINT64 cycle_iterations = 0;   // iterations executed inside lowered loops
    UINT64 graph_replays = 0;      // CUDA graph launches issued for lowered loops
    float last_cycle_ms = 0;       // device time of the last lowered loop (CUDA events)
    UINT last_cycle_iterations = 0;
};

class Graph : public Lockable {
public:
    Graph(const char *name = nullptr);
    virtual ~Graph();
    static BOOL DestroyGraph(Graph *pGraph, BOOL bGCSweep = FALSE);

    Task *AddTask(CompiledKernel *pKernel, UINT uiInputPortCount, Port **pvInputPorts,
                  UINT uiOutputPortCount, Port **pvOutputPorts, const char *lpszTaskName);
    GraphInputChannel *AddInputChannel(Port *pDestinationPort, const char *lpszChannelName = nullptr,
                                       BOOL bSwitchChannel = FALSE, Port *pTriggerPort = nullptr,
                                       CONTROLSIGNAL luiTriggerSignal = DBCTLC_NONE);
    GraphOutputChannel *AddOutputChannel(Port *pSourcePort, const char *lpszChannelName = nullptr,
                                         Port *pTriggerPort = nullptr,
                                         CONTROLSIGNAL luiTriggerSignal = DBCTLC_NONE);
    InternalChannel *AddInternalChannel(Port *pSourcePort, Port *pDestinationPort,
                                        const char *lpszChannelName = nullptr, BOOL bSwitchChannel = FALSE);
    void Run(BOOL bSingleThreaded = FALSE);
    void Stop();
    void Teardown();
    BOOL IsRunning();
    GRAPHSTATE GetState() { return m_state; }
    void WriteDOTFile(const char *lpszFileName, BOOL bPresentationMode = FALSE, BOOL bShowSchedulerPartitions = FALSE);
    void BindControlPropagationPort(Port *pInputPort, Port *pOutputPort);
    void BindControlPropagationChannel(Port *pInputPort, Channel *pControlledChannel);
    void BindIterationScope(Port *pMetaPort, Port *pScopedPort);
    void BindDescriptorPort(Port *pDescribedPort, Port *pDescriberPort, DESCRIPTORFUNC func = DF_SIZE);
    void BindControlPort(Port *pController, Port *pGatedPort, BOOL bInitiallyOpen = FALSE);
    PTRESULT CheckGraphSemantics(BOOL bVerbose = TRUE, BOOL bFixErrors = TRUE);
    const char *GetName() { return m_name.c_str(); }
    Channel *GetChannel(const char *lpszChannelName);
    Task *GetTask(const char *lpszTaskName);
    // Graph structure to / from an XML file in the reference's format (graph.h:1545, :1561;
    // XMLWriter.cpp, XMLReader.cpp).  Deserialize builds into an empty graph.
    void Serialize(const char *filename);
    void Deserialize(const char *filename);
    // GB300 extension: why the last Serialize / Deserialize failed ("" after a success).
    const char *GetSerializationError() { return m_xml_error.c_str(); }

    // ---- GB300 extensions ----
    // Lower MF_GENERAL_ITERATOR loops to a captured CUDA graph / registered fused kernel (default on).
    void SetCycleLowering(BOOL b) { m_lower_cycles = b; }
    void SetCycleFusion(BOOL b) { m_fuse_cycles = b; }
    GraphStats GetStats();
    void *GetStream() { return m_stream; }
    // Block until every dispatched kernel of this graph has finished.
    void Synchronize();

    // ---- runtime side ----
    void Signal();                 // a channel changed: wake the scheduler
    // Bindings kept for serialization (the FDTD path does not act on them).
    struct ControlPortBinding { Port *controller, *gated; BOOL open; };
    struct DescriptorBinding { Port *described, *describer; DESCRIPTORFUNC func; };
    std::vector<std::pair<Port *, Channel *>> m_ctl_channels;   // BindControlPropagationChannel
    std::vector<std::pair<Port *, Port *>> m_iter_scopes;       // BindIterationScope
    std::vector<DescriptorBinding> m_descriptors;               // BindDescriptorPort
    std::vector<ControlPortBinding> m_control_ports;            // BindControlPort
    std::vector<Task *> m_tasks;
    std::vector<Channel *> m_channels;
    std::vector<Port *> m_ports;
    std::recursive_mutex m_sched_mu;

private:
    friend struct CyclePlan;
    void scheduler_loop();
    bool schedule_once();          // dispatch every ready task once; true if anything ran
    bool task_ready(Task *t);
    void dispatch(Task *t);
    bool try_lower_cycle(Task *top);
    void finalize();
    void push_outputs(Port *out, Datablock *b);

    std::string m_name;
    GRAPHSTATE m_state = PTGS_INITIALIZING;
    bool m_single = false;
    bool m_scheduling = false;
    bool m_lower_cycles = true;
    bool m_fuse_cycles = true;
    std::thread m_thread;
    std::atomic<bool> m_stop{false};
    std::mutex m_wake_mu;
    std::condition_variable m_wake;
    UINT64 m_signals = 0;
    void *m_stream = nullptr;
    GraphStats m_stats;
    std::vector<std::unique_ptr<CyclePlan>> m_plans;
    bool m_finalized = false;
    std::string m_xml_error;
};

// Host copy of `bytes`, split over the host cores when it is large (one core moves a few tens of
// GB/s; the fields of one FDTD solve are about a gigabyte).  Used for datablock initial data and
// for Pull results.
void HostCopy(void *dst, const void *src, size_t bytes);

// ---------------------------------------------------------------------------------------------
// The single CUDA accelerator this runtime drives (accelerator.h).
class Accelerator {
public:
    ACCELERATOR_CLASS GetClass() { return ACCELERATOR_CLASS_CUDA; }
    const char *GetDeviceName();
    UINT GetCoreCount();
    size_t GetGlobalMemorySize();
};

}  // namespace PTask

#endif
