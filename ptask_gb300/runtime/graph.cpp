// graph.cpp -- ports, channels, tasks and the graph scheduler of the GB300 PTask runtime.
//
// Semantics kept from the reference: channel queues with capacity (channel.cpp:1125 Push, :523
// Pull), predicated channels (CGATEFN_*, channel.cpp:1619), sticky ports that retain their last
// block (StickyPort.cpp:96), in-out ports that forward the input block to an output port after the
// dispatch (CreatePort's nInOutParmOutputIndex), MF_GENERAL_ITERATOR meta ports that count
// dispatches and mark the last one with DBCTLC_ENDITERATION on the ports bound by
// BindControlPropagationPort (MetaPort.cpp:927-1011), and MF_SIMPLE_ITERATOR (MetaPort.cpp:887-916).
//
// What is different: one scheduler thread per graph enqueues kernels on one CUDA stream (no host
// synchronisation between dispatches), and a general-iteration loop whose whole input is present is
// lowered: the loop body is captured once as a CUDA graph and replayed N times, or, for the FDTD
// H-step/E-step pair, run by the fused Yee-step solver (one kernel per step, 64 B per cell).
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <fstream>

#include "PTaskRuntime.h"
#include "ptask_gb300.h"

namespace PTask {

void *runtime_io_stream();
void *acquire_stream();
void release_stream(void *s);

// ---------------------------------------------------------------------------------------------
// Ports
// ---------------------------------------------------------------------------------------------
Port::Port(PORTTYPE t, DatablockTemplate *tmpl, UINT uid, const char *name, int pi, int io)
    : m_type(t), m_template(tmpl), m_uid(uid), m_name(name ? name : ""), m_param_idx(pi), m_inout_idx(io)
{
}

Port::~Port()
{
    if (m_sticky) m_sticky->Release();
}

BOOL Port::IsOccupied()
{
    for (Channel *c : m_in)
        if (c->GetQueueDepth()) return TRUE;
    return m_sticky != nullptr;
}

Channel *Port::GetChannel(UINT i)
{
    auto &v = (m_type == OUTPUT_PORT) ? m_out : m_in;
    return i < v.size() ? v[i] : nullptr;
}

// ---------------------------------------------------------------------------------------------
// Channels
// ---------------------------------------------------------------------------------------------
Channel::Channel(Graph *g, CHANNELTYPE t, Port *src, Port *dst, const char *name, BOOL sw)
    : m_graph(g), m_type(t), m_src(src), m_dst(dst), m_name(name ? name : ""), m_switch(sw),
      m_capacity((UINT)Runtime::GetDefaultChannelCapacity())
{
}

Channel::~Channel() { Drain(); }

void Channel::Drain()
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    for (Datablock *b : m_q) b->Release();
    m_q.clear();
}

DatablockTemplate *Channel::GetTemplate()
{
    if (m_dst) return m_dst->GetTemplate();
    return m_src ? m_src->GetTemplate() : nullptr;
}

void Channel::SetPredicationType(CHANNELENDPOINTTYPE e, CHANNELPREDICATE p, BOOL) { m_pred[e] = p; }

bool Channel::PassesPredicate(CHANNELENDPOINTTYPE e, Datablock *b)
{
    const CONTROLSIGNAL s = b->GetControlSignals();
    switch (m_pred[e]) {
    case CGATEFN_NONE: return true;
    case CGATEFN_CLOSE_ON_EOF: return !TESTSIGNAL(s, DBCTLC_EOF);
    case CGATEFN_OPEN_ON_EOF: return TESTSIGNAL(s, DBCTLC_EOF);
    case CGATEFN_OPEN_ON_BEGINITERATION: return TESTSIGNAL(s, DBCTLC_BEGINITERATION);
    case CGATEFN_CLOSE_ON_BEGINITERATION: return !TESTSIGNAL(s, DBCTLC_BEGINITERATION);
    case CGATEFN_OPEN_ON_ENDITERATION: return TESTSIGNAL(s, DBCTLC_ENDITERATION);
    case CGATEFN_CLOSE_ON_ENDITERATION: return !TESTSIGNAL(s, DBCTLC_ENDITERATION);
    case CGATEFN_DEVNULL: return false;
    case CGATEFN_CLOSE_ON_BOF: return !TESTSIGNAL(s, DBCTLC_BOF);
    case CGATEFN_OPEN_ON_BOF: return TESTSIGNAL(s, DBCTLC_BOF);
    default: return true;
    }
}

bool Channel::Enqueue(Datablock *b, DWORD timeout_ms)
{
    std::unique_lock<std::recursive_mutex> lk(m_lock);
    if (!PassesPredicate(CE_SRC, b)) return true;   // gated: the block does not enter this channel
    if (m_type == CT_GRAPH_INPUT && m_capacity > 0) {
        auto full = [&] { return m_q.size() >= m_capacity; };
        if (full()) {
            if (timeout_ms == 0xFFFFFFFF) {
                m_cv.wait(lk, [&] { return !full(); });
            } else if (!m_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !full(); })) {
                return false;
            }
        }
    }
    b->AddRef();
    m_q.push_back(b);
    if (m_type == CT_GRAPH_OUTPUT && m_view == VIEWMATERIALIZATIONPOLICY_EAGER && m_graph)
        b->StartHostMaterialization(m_graph->GetStream());
    m_cv.notify_all();
    lk.unlock();
    if (m_graph) m_graph->Signal();
    return true;
}

Datablock *Channel::Dequeue()
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    while (!m_q.empty()) {
        Datablock *b = m_q.front();
        m_q.pop_front();
        m_cv.notify_all();
        if (PassesPredicate(CE_DST, b)) return b;
        b->Release();
    }
    return nullptr;
}

BOOL Channel::Push(Datablock *b, DWORD timeout)
{
    if (!b) return FALSE;
    return Enqueue(b, timeout) ? TRUE : FALSE;
}

Datablock *Channel::Pull(DWORD timeout)
{
    auto ready = [&] { return !m_q.empty(); };
    {
        std::unique_lock<std::recursive_mutex> lk(m_lock);
        if (!ready()) {
            if (m_graph) {
                lk.unlock();
                m_graph->Signal();
                lk.lock();
            }
            if (timeout == 0xFFFFFFFF) {
                m_cv.wait(lk, ready);
            } else if (!m_cv.wait_for(lk, std::chrono::milliseconds(timeout), ready)) {
                return nullptr;
            }
        }
    }
    Datablock *b = Dequeue();
    if (m_graph) m_graph->Signal();
    return b;
}

Datablock *Channel::Peek()
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    return m_q.empty() ? nullptr : m_q.front();
}

BOOL Channel::IsReady()
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    return m_q.empty() ? FALSE : TRUE;
}

UINT Channel::GetQueueDepth()
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    return (UINT)m_q.size();
}

// ---------------------------------------------------------------------------------------------
// Tasks
// ---------------------------------------------------------------------------------------------
Task::Task(Graph *g, CompiledKernel *k, const char *name) : m_graph(g), m_kernel(k), m_name(name ? name : "") {}

Task::~Task()
{
    if (m_iter_block) m_iter_block->Release();
    if (m_step_counter) ptk_mem_free(m_step_counter, m_graph ? m_graph->GetStream() : nullptr);
}

void Task::SetComputeGeometry(int x, int y, int z)
{
    m_geom = PTASKDIM3(x, y, z);
    m_geom_set = true;
}

BOOL Task::BindDependentAcceleratorClass(ACCELERATOR_CLASS cls, int nRequiredInstances, BOOL bRequestDependentPSObjects)
{
    if (!m_kernel || !m_kernel->IsHost()) {
        Runtime::HandleError("task %s: dependent accelerators are bound to host tasks only", GetTaskName());
        return FALSE;
    }
    if (cls != ACCELERATOR_CLASS_CUDA || nRequiredInstances != 1) {
        Runtime::HandleError("task %s: dependent accelerator class %d x %d is not available (one CUDA device)",
                             GetTaskName(), (int)cls, nRequiredInstances);
        return FALSE;
    }
    m_dep_class = cls;
    m_dep_ps = bRequestDependentPSObjects;
    return TRUE;
}

void Task::SetBlockAndGridSize(PTASKDIM3 grid, PTASKDIM3 block)
{
    // Recorded for inspection; native kernels choose their own launch shape.
    m_grid = grid;
    m_block = block;
    m_explicit_launch = true;
}

// ---------------------------------------------------------------------------------------------
// Kernel adapters: formal parameters (ports with a parameter index, in index order) to C-ABI calls.
// ---------------------------------------------------------------------------------------------
struct Formal {
    Port *port;
    Datablock *block;
    void *dev;          // device pointer for buffers
    const void *host;   // host bytes for by-value constants
};

static bool is_scalar(Datablock *b) { return b && b->IsScalarParameter(); }

static int launch_native(Task *t, std::vector<Formal> &f, void *stream)
{
    const char *op = t->GetCompiledKernel()->GetOperation();
    auto dev = [&](size_t i) -> float * { return i < f.size() ? (float *)f[i].dev : nullptr; };
    auto params = [&](size_t i) -> const ptk_fdtd_params * {
        return i < f.size() ? (const ptk_fdtd_params *)f[i].host : nullptr;
    };
    static const char *field_ops[6] = {"HxComputation", "HyComputation", "HzComputation",
                                       "ExComputation", "EyComputation", "EzComputation"};
    for (int q = 0; q < 6; ++q)
        if (strcmp(op, field_ops[q]) == 0) {
            // (in0, in1, in2, FDTD_PARAMS, out): graphfdtd.cpp:398-436
            if (f.size() != 5 || !params(3)) return PTK_ERR_INVALID;
            return ptk_launch_field_update(q, dev(0), dev(1), dev(2), params(3), dev(4), stream);
        }
    if (strcmp(op, "FDTDHStep") == 0) {
        // (Hx, Hy, Hz, Ex, Ey, Ez, Da, Db, FDTD_PARAMS)
        if (f.size() < 9 || !params(8)) return PTK_ERR_INVALID;
        float *h[3] = {dev(0), dev(1), dev(2)};
        const float *e[3] = {dev(3), dev(4), dev(5)};
        return ptk_launch_h_step_coef(h, e, dev(6), dev(7), params(8), stream);
    }
    if (strcmp(op, "FDTDEStep") == 0) {
        // (Ex, Ey, Ez, Hx, Hy, Hz, Ca, Cb, FDTD_PARAMS, SOURCE{i,j,k,n}, wave)
        if (f.size() < 9 || !params(8)) return PTK_ERR_INVALID;
        float *e[3] = {dev(0), dev(1), dev(2)};
        const float *h[3] = {dev(3), dev(4), dev(5)};
        int si = -1, sj = -1, sk = -1, n = 0;
        const float *wave = nullptr;
        if (f.size() >= 11 && f[9].host) {
            const int *s = (const int *)f[9].host;
            si = s[0]; sj = s[1]; sk = s[2]; n = s[3];
            wave = dev(10);
        }
        if (n > 0 && !t->m_step_counter) {
            ptk_mem_alloc(sizeof(int), stream, &t->m_step_counter);
            ptk_memset(t->m_step_counter, 0, sizeof(int), stream);
        }
        return ptk_launch_e_step_coef(e, h, dev(6), dev(7), params(8), si, sj, sk, wave, n,
                                      n > 0 ? (int *)t->m_step_counter : nullptr, stream);
    }
    return PTK_ERR_NOTFOUND;
}

// ---------------------------------------------------------------------------------------------
// Lowered general-iteration loops.
// ---------------------------------------------------------------------------------------------
struct CyclePlan {
    Task *top = nullptr;      // task whose inputs come back around the loop
    Task *bottom = nullptr;   // task with the MF_GENERAL_ITERATOR meta port
    Port *meta = nullptr;
    bool entered = false;     // a loop instance is running task by task
    bool fused_kind = false;  // FDTDHStep -> FDTDEStep: can run on the fused Yee solver
    // captured replay
    void *exec = nullptr;
    std::vector<void *> exec_key;
    // fused solver
    ptk_solver *solver = nullptr;
    ptk_fdtd_params solver_params{};
    std::vector<UINT> coef_key;
    float last_ms = 0;
    void *ev0 = nullptr, *ev1 = nullptr;

    ~CyclePlan()
    {
        if (exec) ptk_graph_exec_destroy(exec);
        if (solver) ptk_solver_destroy(solver);
        if (ev0) ptk_event_destroy(ev0);
        if (ev1) ptk_event_destroy(ev1);
    }
};

// ---------------------------------------------------------------------------------------------
// Graph
// ---------------------------------------------------------------------------------------------
Graph::Graph(const char *name) : m_name(name ? name : "graph") {}

Graph::~Graph()
{
    Stop();
    Teardown();
}

BOOL Graph::DestroyGraph(Graph *g, BOOL)
{
    delete g;
    return TRUE;
}

Task *Graph::AddTask(CompiledKernel *k, UINT nin, Port **in, UINT nout, Port **out, const char *name)
{
    if (!k) {
        Runtime::HandleError("Graph::AddTask(%s): NULL kernel", name ? name : "");
        return nullptr;
    }
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    Task *t = new Task(this, k, name);
    for (UINT i = 0; i < nin; ++i) {
        in[i]->m_task = t;
        in[i]->SetOriginalIndex(i);
        t->m_inputs.push_back(in[i]);
        m_ports.push_back(in[i]);
    }
    for (UINT i = 0; i < nout; ++i) {
        out[i]->m_task = t;
        out[i]->SetOriginalIndex(i);
        t->m_outputs.push_back(out[i]);
        m_ports.push_back(out[i]);
    }
    for (Port *p : t->m_inputs)
        if (p->GetInOutRoutingIndex() >= 0 && p->GetInOutRoutingIndex() < (int)nout)
            p->m_inout_partner = out[p->GetInOutRoutingIndex()];
    m_tasks.push_back(t);
    return t;
}

GraphInputChannel *Graph::AddInputChannel(Port *dst, const char *name, BOOL sw, Port *, CONTROLSIGNAL)
{
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    auto *c = new GraphInputChannel(this, CT_GRAPH_INPUT, nullptr, dst, name, sw);
    dst->m_in.push_back(c);
    m_channels.push_back(c);
    return c;
}

GraphOutputChannel *Graph::AddOutputChannel(Port *src, const char *name, Port *, CONTROLSIGNAL)
{
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    auto *c = new GraphOutputChannel(this, CT_GRAPH_OUTPUT, src, nullptr, name, FALSE);
    c->SetCapacity(0);
    src->m_out.push_back(c);
    m_channels.push_back(c);
    return c;
}

InternalChannel *Graph::AddInternalChannel(Port *src, Port *dst, const char *name, BOOL sw)
{
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    auto *c = new InternalChannel(this, CT_INTERNAL, src, dst, name, sw);
    c->SetCapacity(0);
    src->m_out.push_back(c);
    dst->m_in.push_back(c);
    m_channels.push_back(c);
    return c;
}

void Graph::BindControlPropagationPort(Port *in, Port *out)
{
    if (in && out) in->m_ctl_targets.push_back(out);
}

void Graph::BindControlPropagationChannel(Port *in, Channel *c)
{
    if (in && c) m_ctl_channels.push_back({in, c});
}
void Graph::BindIterationScope(Port *meta, Port *scoped)
{
    if (meta && scoped) m_iter_scopes.push_back({meta, scoped});
}
void Graph::BindDescriptorPort(Port *described, Port *describer, DESCRIPTORFUNC f)
{
    if (described && describer) m_descriptors.push_back({described, describer, f});
}
void Graph::BindControlPort(Port *controller, Port *gated, BOOL open)
{
    if (controller && gated) m_control_ports.push_back({controller, gated, open});
}

Channel *Graph::GetChannel(const char *name)
{
    for (Channel *c : m_channels)
        if (name && !strcmp(c->GetName(), name)) return c;
    return nullptr;
}

Task *Graph::GetTask(const char *name)
{
    for (Task *t : m_tasks)
        if (name && !strcmp(t->GetTaskName(), name)) return t;
    return nullptr;
}

PTRESULT Graph::CheckGraphSemantics(BOOL verbose, BOOL)
{
    PTRESULT r = PTASK_OK;
    for (Task *t : m_tasks) {
        for (Port *p : t->m_inputs)
            if (p->m_in.empty() && p->GetPortType() != INITIALIZER_PORT) {
                if (verbose) Runtime::Warning(std::string("unbound input port ") + p->GetVariableBinding() +
                                              " on task " + t->GetTaskName());
                r = PTASK_WARNING_GRAPH_MALFORMED;
            }
        for (Port *p : t->m_outputs)
            if (p->m_out.empty()) {
                if (verbose) Runtime::Warning(std::string("unbound output port ") + p->GetVariableBinding() +
                                              " on task " + t->GetTaskName());
                r = PTASK_WARNING_GRAPH_MALFORMED;
            }
    }
    return r;
}

void Graph::WriteDOTFile(const char *file, BOOL, BOOL)
{
    std::ofstream o(file ? file : "graph.dot");
    o << "digraph " << '"' << m_name << '"' << " {\n  rankdir=TB;\n";
    for (Task *t : m_tasks)
        o << "  \"" << t->GetTaskName() << "\" [shape=box,label=\"" << t->GetTaskName() << "\\n"
          << t->GetCompiledKernel()->GetOperation() << "\"];\n";
    for (Channel *c : m_channels) {
        if (!c->ShouldDraw()) continue;
        Port *s = c->GetBoundPort(CE_SRC), *d = c->GetBoundPort(CE_DST);
        std::string src = s && s->GetTask() ? s->GetTask()->GetTaskName() : std::string("in:") + c->GetName();
        std::string dst = d && d->GetTask() ? d->GetTask()->GetTaskName() : std::string("out:") + c->GetName();
        if (!s) o << "  \"" << src << "\" [shape=ellipse];\n";
        if (!d) o << "  \"" << dst << "\" [shape=ellipse];\n";
        o << "  \"" << src << "\" -> \"" << dst << "\" [label=\"" << c->GetName() << "\"";
        if (c->GetPredicationType(CE_SRC) != CGATEFN_NONE) o << ",style=dashed";
        o << "];\n";
    }
    o << "}\n";
}

void Graph::Signal()
{
    {
        std::lock_guard<std::mutex> lk(m_wake_mu);
        ++m_signals;
    }
    m_wake.notify_all();
    if (m_single && m_state == PTGS_RUNNING && !m_scheduling) {
        // Single-threaded mode: the caller's thread runs the scheduler (never re-entered from a
        // dispatch that pushes its outputs).
        std::unique_lock<std::recursive_mutex> lk(m_sched_mu, std::try_to_lock);
        if (lk.owns_lock())
            while (schedule_once()) {
            }
    }
}

BOOL Graph::IsRunning() { return m_state == PTGS_RUNNING; }

void Graph::finalize()
{
    if (m_finalized) return;
    m_finalized = true;
    // Find general-iteration loops: bottom task owns an MF_GENERAL_ITERATOR meta port; the back
    // channels are bottom outputs gated CLOSE_ON_ENDITERATION; their destination task is the top.
    for (Task *b : m_tasks) {
        for (Port *p : b->m_inputs) {
            if (p->GetPortType() != META_PORT || p->GetMetaFunction() != MF_GENERAL_ITERATOR) continue;
            Task *top = nullptr;
            bool ok = true;
            for (Port *o : b->m_outputs)
                for (Channel *c : o->m_out)
                    if (c->GetType() == CT_INTERNAL && c->GetPredicationType(CE_SRC) == CGATEFN_CLOSE_ON_ENDITERATION) {
                        Task *d = c->GetBoundPort(CE_DST)->GetTask();
                        if (top && d != top) ok = false;
                        top = d;
                    }
            if (!ok || !top) continue;
            // host tasks run where they are: only loops of native kernels are lowered to the GPU
            if (top->GetCompiledKernel()->IsHost() || b->GetCompiledKernel()->IsHost()) continue;
            auto plan = std::make_unique<CyclePlan>();
            plan->top = top;
            plan->bottom = b;
            plan->meta = p;
            plan->fused_kind = top != b && strcmp(top->GetCompiledKernel()->GetOperation(), "FDTDHStep") == 0 &&
                               strcmp(b->GetCompiledKernel()->GetOperation(), "FDTDEStep") == 0;
            top->m_loop_top = plan.get();
            b->m_loop_bottom = plan.get();
            m_plans.push_back(std::move(plan));
        }
    }
}

void Graph::Run(BOOL single)
{
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    if (m_state == PTGS_RUNNING) return;
    if (!Runtime::IsInitialized()) Runtime::Initialize();
    if (!m_stream) m_stream = acquire_stream();
    if (!m_stream) {
        Runtime::HandleError("Graph::Run: %s", ptk_last_error());
        return;
    }
    finalize();
    m_single = single ? true : false;
    m_stop = false;
    m_state = PTGS_RUNNING;
    if (!m_single) m_thread = std::thread([this] { scheduler_loop(); });
}

void Graph::scheduler_loop()
{
    UINT64 seen = 0;
    while (!m_stop) {
        bool progressed;
        {
            std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
            progressed = schedule_once();
        }
        if (progressed) continue;
        std::unique_lock<std::mutex> lk(m_wake_mu);
        m_wake.wait_for(lk, std::chrono::milliseconds(50), [&] { return m_stop || m_signals != seen; });
        seen = m_signals;
    }
}

void Graph::Stop()
{
    if (m_state != PTGS_RUNNING) return;
    m_stop = true;
    m_wake.notify_all();
    if (m_thread.joinable()) m_thread.join();
    if (m_stream) ptk_stream_sync(m_stream);
    m_state = PTGS_QUIESCING;
}

void Graph::Synchronize()
{
    if (m_stream) ptk_stream_sync(m_stream);
}

void Graph::Teardown()
{
    Stop();
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    if (m_state == PTGS_TEARDOWNCOMPLETE) return;
    m_state = PTGS_TEARINGDOWN;
    if (m_stream) ptk_stream_sync(m_stream);
    m_plans.clear();
    for (Channel *c : m_channels) delete c;
    m_channels.clear();
    for (Task *t : m_tasks) delete t;
    m_tasks.clear();
    std::set<Port *> uniq(m_ports.begin(), m_ports.end());
    for (Port *p : uniq) delete p;
    m_ports.clear();
    if (m_stream) {
        // Blocks the application still holds free their device memory on this stream later, so the
        // stream goes back to the runtime's pool instead of being destroyed.
        release_stream(m_stream);
        m_stream = nullptr;
    }
    m_state = PTGS_TEARDOWNCOMPLETE;
}

GraphStats Graph::GetStats()
{
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    return m_stats;
}

// Which input channels of port p the scheduler may draw from now.  For the top task of a loop, a
// port fed both by entry (switch) channels and by back channels takes a new instance only from the
// entry channels while no loop instance is in flight, and only from the back channels while one is
// (the role of switch channels in the reference's iteration graphs, iteration.cpp:355-366).
static bool may_draw(Task *t, Port *p, Channel *c)
{
    if (!t->m_loop_top) return true;
    bool has_switch = false, has_back = false;
    for (Channel *x : p->m_in) (x->IsSwitchChannel() ? has_switch : has_back) = true;
    if (!(has_switch && has_back)) return true;
    return t->m_loop_top->entered ? !c->IsSwitchChannel() : c->IsSwitchChannel() != FALSE;
}

static Datablock *take_for(Task *t, Port *p)
{
    for (Channel *c : p->m_in)
        if (may_draw(t, p, c) && c->GetQueueDepth()) {
            Datablock *b = c->Dequeue();
            if (b) return b;
        }
    return nullptr;
}

bool Graph::task_ready(Task *t)
{
    // With loop lowering on, the head of a loop does not start an instance task by task before the
    // loop's iteration count has arrived: once it has, the whole loop is lowered at once.
    if (t->m_loop_top && m_lower_cycles && !t->m_loop_top->entered) {
        bool count = false;
        for (Channel *c : t->m_loop_top->meta->m_in)
            if (c->GetQueueDepth()) count = true;
        if (!count) return false;
    }
    for (Port *p : t->m_inputs) {
        switch (p->GetPortType()) {
        case INPUT_PORT: {
            bool any = false;
            for (Channel *c : p->m_in)
                if (may_draw(t, p, c) && c->GetQueueDepth()) { any = true; break; }
            if (!any) return false;
            break;
        }
        case STICKY_PORT: {
            if (p->m_sticky) break;
            bool any = false;
            for (Channel *c : p->m_in)
                if (c->GetQueueDepth()) { any = true; break; }
            if (!any) return false;
            break;
        }
        case META_PORT: {
            if (p->GetMetaFunction() == MF_GENERAL_ITERATOR && t->m_iter_block) break;
            bool any = false;
            for (Channel *c : p->m_in)
                if (c->GetQueueDepth()) { any = true; break; }
            if (!any) return false;
            break;
        }
        default: break;
        }
    }
    return true;
}

static Datablock *take(Port *p)
{
    for (Channel *c : p->m_in)
        if (c->GetQueueDepth()) {
            Datablock *b = c->Dequeue();
            if (b) return b;
        }
    return nullptr;
}

static UINT int_value(Datablock *b)
{
    const void *h = b->HostBytes();
    return h ? *(const UINT *)h : 0;
}

void Graph::push_outputs(Port *out, Datablock *b)
{
    for (Channel *c : out->m_out) c->Enqueue(b, 0xFFFFFFFF);
}

void Graph::dispatch(Task *t)
{
    std::vector<Datablock *> owned;             // references this dispatch holds
    std::vector<Datablock *> in(t->m_inputs.size(), nullptr);
    UINT repeat = 1;
    bool last_iteration = false, general = false;
    Port *meta = nullptr;
    for (size_t q = 0; q < t->m_inputs.size(); ++q) {
        Port *p = t->m_inputs[q];
        switch (p->GetPortType()) {
        case INPUT_PORT:
            in[q] = take_for(t, p);
            owned.push_back(in[q]);
            break;
        case STICKY_PORT: {
            Datablock *nb = nullptr;
            for (Channel *c : p->m_in)
                if (c->GetQueueDepth()) nb = c->Dequeue();
            if (nb) {
                if (p->m_sticky) p->m_sticky->Release();
                p->m_sticky = nb;
            }
            in[q] = p->m_sticky;
            break;
        }
        case META_PORT:
            meta = p;
            if (p->GetMetaFunction() == MF_GENERAL_ITERATOR) {
                general = true;
                if (!t->m_iter_block) {
                    t->m_iter_block = take(p);
                    t->m_iter_max = int_value(t->m_iter_block);
                    t->m_iter_count = 0;
                    if (t->m_iter_max == 0)
                        Runtime::HandleError("%s: PTask cannot handle iteration max of 0 (task %s)", __FUNCTION__,
                                             t->GetTaskName());
                    if (t->m_step_counter) ptk_memset(t->m_step_counter, 0, sizeof(int), m_stream);
                }
                last_iteration = ++t->m_iter_count >= t->m_iter_max;
            } else if (p->GetMetaFunction() == MF_SIMPLE_ITERATOR) {
                Datablock *b = take(p);
                repeat = b ? int_value(b) : 1;
                if (b) b->Release();
            } else {
                Datablock *b = take(p);
                if (b) b->Release();
            }
            break;
        default: break;
        }
    }

    // Output blocks: the forwarded input of an in-out port, or a fresh device block.
    std::vector<Datablock *> out(t->m_outputs.size(), nullptr);
    for (size_t q = 0; q < t->m_inputs.size(); ++q) {
        Port *p = t->m_inputs[q];
        int r = p->GetInOutRoutingIndex();
        if (r >= 0 && r < (int)out.size()) out[r] = in[q];
    }
    for (size_t r = 0; r < out.size(); ++r)
        if (!out[r]) {
            DatablockTemplate *tm = t->m_outputs[r]->GetTemplate();
            out[r] = new Datablock(tm, tm ? tm->GetDatablockByteCount() : 0, DBCTLC_NONE);
            owned.push_back(out[r]);
        }

    // Formal parameters in index order: device views for a native kernel, host views for a host
    // task (whose writes leave the host copy as the only valid one).  A host task with a dependent
    // CUDA accelerator gets device views on the ports bound to it (port.h:1185) and host views on
    // the others (hosttask.cpp:380-405).
    const bool host = t->GetCompiledKernel()->IsHost();
    const bool dep = host && t->HasDependentAcceleratorBindings();
    auto on_device = [&](Port *p) { return !host || (dep && p->HasDependentAcceleratorBinding()); };
    std::vector<std::pair<int, Formal>> formals;
    for (size_t q = 0; q < t->m_inputs.size(); ++q) {
        Port *p = t->m_inputs[q];
        if (p->GetPortType() == META_PORT || p->GetFormalParameterIndex() == (UINT)-1) continue;
        Formal f{p, in[q], nullptr, nullptr};
        if (in[q]) {
            if (is_scalar(in[q])) f.host = in[q]->HostBytes();
            else if (!on_device(p)) f.host = in[q]->GetDataPointer(p->IsInOutParameter(), TRUE);
            else f.dev = in[q]->DeviceView(m_stream, p->IsInOutParameter(), true);
        }
        formals.push_back({(int)p->GetFormalParameterIndex(), f});
    }
    for (size_t r = 0; r < t->m_outputs.size(); ++r) {
        Port *p = t->m_outputs[r];
        if (p->GetFormalParameterIndex() == (UINT)-1) continue;
        Formal f{p, out[r], nullptr, nullptr};
        if (!on_device(p)) f.host = out[r]->GetDataPointer(TRUE, FALSE);
        else f.dev = out[r]->DeviceView(m_stream, true, false);
        formals.push_back({(int)p->GetFormalParameterIndex(), f});
    }
    std::stable_sort(formals.begin(), formals.end(),
                     [](const std::pair<int, Formal> &a, const std::pair<int, Formal> &b) { return a.first < b.first; });
    std::vector<Formal> fv;
    for (auto &pf : formals) fv.push_back(pf.second);

    if (host) {
        // Host task (hosttask.cpp:305-340): the arguments are the formal parameters 0..n-1 as host
        // pointers (device pointers where bound to the dependent accelerator); the entry point runs
        // once per point of the task's geometry.
        std::vector<void *> args;
        std::vector<BOOL> is_dep;
        std::vector<void *> dev_of;
        std::vector<Datablock *> blocks;
        int ordinal = 0;
        if (dep && ptk_device_ordinal(&ordinal) != PTK_OK)
            Runtime::HandleError("dispatch of host task %s: no dependent device: %s", t->GetTaskName(), ptk_last_error());
        void *device = reinterpret_cast<void *>((intptr_t)ordinal);
        for (size_t i = 0; i < formals.size(); ++i) {
            if (formals[i].first != (int)i) {
                Runtime::HandleError("dispatch of host task %s: no formal parameter %zu", t->GetTaskName(), i);
                args.clear();
                break;
            }
            const Formal &f = formals[i].second;
            const bool d = f.dev != nullptr;
            args.push_back(d ? f.dev : const_cast<void *>(f.host));
            is_dep.push_back(d ? TRUE : FALSE);
            dev_of.push_back(d ? device : nullptr);
            blocks.push_back(f.block);
        }
        const UINT reps = repeat * std::max(1, t->m_geom.x) * std::max(1, t->m_geom.y) * std::max(1, t->m_geom.z);
        if (args.size() == formals.size()) {
            void *fn = reinterpret_cast<void *>(t->GetCompiledKernel()->HostFunction());
            if (!dep) {
                for (UINT n = 0; n < reps; ++n) t->GetCompiledKernel()->HostFunction()((UINT)args.size(), args.data());
            } else if (t->DependentBindingsRequirePSObjects()) {
                // LPFNDEPHOSTTASKEX (hosttask.cpp:520-560): the task orders its work on pStreams[0],
                // this graph's stream, after the views above; no host wait.
                void *deps[1] = {device};
                void *streams[1] = {m_stream};
                DEPENDENTCONTEXT c{};
                c.cbDependentContext = sizeof(DEPENDENTCONTEXT);
                c.nArguments = (UINT)args.size();
                c.nDependentAccelerators = 1;
                c.ppArguments = args.data();
                c.ppDatablocks = blocks.data();
                c.pbIsDependentBinding = is_dep.data();
                c.pvDeviceBindings = dev_of.data();
                c.pDependentDevices = deps;
                c.pStreams = streams;
                c.lpszTaskName = const_cast<char *>(t->GetTaskName());
                for (UINT n = 0; n < reps; ++n) reinterpret_cast<LPFNDEPHOSTTASKEX>(fn)(&c);
            } else {
                // LPFNDEPHOSTTASK (hosttask.cpp:405-430): no stream is handed over, so the views
                // are complete before the call and the task's device work is waited for after it.
                void *deps[1] = {device};
                if (ptk_stream_sync(m_stream) != PTK_OK)
                    Runtime::HandleError("dispatch of host task %s: inputs not ready: %s", t->GetTaskName(),
                                         ptk_last_error());
                for (UINT n = 0; n < reps; ++n)
                    reinterpret_cast<LPFNDEPHOSTTASK>(fn)((UINT)args.size(), args.data(), is_dep.data(), dev_of.data(),
                                                          1, deps);
                if (ptk_device_sync() != PTK_OK)
                    Runtime::HandleError("host task %s: its device work failed: %s", t->GetTaskName(), ptk_last_error());
            }
        }
        ++m_stats.host_dispatches;
    } else {
        for (UINT n = 0; n < repeat; ++n) {
            int rc = launch_native(t, fv, m_stream);
            if (rc != PTK_OK) {
                Runtime::HandleError("dispatch of task %s (%s) failed: %s", t->GetTaskName(),
                                     t->GetCompiledKernel()->GetOperation(), ptk_last_error());
                break;
            }
            ++m_stats.kernel_launches;
        }
    }
    ++t->m_dispatches;
    ++m_stats.dispatches;

    // Blocks written on the device get a completion event (a host task's host writes are already
    // complete; a dependent host task's device writes are ordered on this stream, or waited for).
    if (!host || dep) {
        for (size_t q = 0; q < t->m_inputs.size(); ++q)
            if (t->m_inputs[q]->IsInOutParameter() && in[q] && !is_scalar(in[q]) && on_device(t->m_inputs[q]))
                in[q]->DeviceWritten(m_stream);
        for (size_t r = 0; r < out.size(); ++r)
            if (t->m_outputs[r]->GetFormalParameterIndex() != (UINT)-1 && on_device(t->m_outputs[r]))
                out[r]->DeviceWritten(m_stream);
    }

    // Control propagation of the general iterator.
    if (general && meta) {
        for (Port *o : meta->m_ctl_targets) {
            for (size_t r = 0; r < t->m_outputs.size(); ++r)
                if (t->m_outputs[r] == o) {
                    if (last_iteration) out[r]->SetControlSignal(DBCTLC_ENDITERATION);
                    else out[r]->ClearControlSignal(DBCTLC_ENDITERATION);
                }
        }
    }
    if (t->m_loop_top) t->m_loop_top->entered = true;   // an instance is now inside the loop
    if (general && last_iteration && t->m_loop_bottom) t->m_loop_bottom->entered = false;
    for (size_t r = 0; r < out.size(); ++r) push_outputs(t->m_outputs[r], out[r]);
    if (general && last_iteration) {
        for (size_t r = 0; r < out.size(); ++r) out[r]->ClearControlSignal(DBCTLC_ENDITERATION);
        t->m_iter_block->Release();
        t->m_iter_block = nullptr;
        t->m_iter_count = t->m_iter_max = 0;
    }
    for (Datablock *b : owned)
        if (b) b->Release();
}

// Run a whole general-iteration loop at once when its inputs are all present.
bool Graph::try_lower_cycle(Task *top)
{
    if (!m_lower_cycles) return false;
    CyclePlan *plan = nullptr;
    for (auto &p : m_plans)
        if (p->top == top) plan = p.get();
    if (!plan) return false;
    Task *bot = plan->bottom;
    if (bot->m_iter_block || plan->entered) return false;                 // a loop is already running task by task
    if (!task_ready(top)) return false;
    // The meta port must hold the iteration count; every other bottom input must come from the top
    // (in flight: none queued) or be sticky.
    bool count_ready = false;
    for (Channel *c : plan->meta->m_in)
        if (c->GetQueueDepth()) count_ready = true;
    if (!count_ready) return false;
    for (Port *p : bot->m_inputs) {
        if (p == plan->meta) continue;
        if (p->GetPortType() == STICKY_PORT) {
            if (!p->m_sticky) {
                bool any = false;
                for (Channel *c : p->m_in)
                    if (c->GetQueueDepth()) any = true;
                if (!any) return false;
            }
            continue;
        }
        for (Channel *c : p->m_in)
            if (c->GetQueueDepth()) return false;
        // must be fed by the top task
        bool from_top = false;
        for (Channel *c : p->m_in)
            if (c->GetBoundPort(CE_SRC) && c->GetBoundPort(CE_SRC)->GetTask() == top) from_top = true;
        if (!from_top) return false;
    }
    if (top != bot && plan->fused_kind == false) {
        // Generic lowering needs every top output consumed only by the bottom (one iteration = top; bottom).
        for (Port *o : top->m_outputs)
            for (Channel *c : o->m_out)
                if (!c->GetBoundPort(CE_DST) || c->GetBoundPort(CE_DST)->GetTask() != bot) return false;
    }

    // ---- take the loop inputs ----
    auto refresh_sticky = [](Port *p) {
        Datablock *nb = nullptr;
        for (Channel *c : p->m_in)
            if (c->GetQueueDepth()) nb = c->Dequeue();
        if (nb) {
            if (p->m_sticky) p->m_sticky->Release();
            p->m_sticky = nb;
        }
    };
    for (Port *p : top->m_inputs)
        if (p->GetPortType() == STICKY_PORT) refresh_sticky(p);
    for (Port *p : bot->m_inputs)
        if (p->GetPortType() == STICKY_PORT) refresh_sticky(p);
    Datablock *count_block = take(plan->meta);
    const UINT N = count_block ? int_value(count_block) : 0;
    if (N == 0) {
        Runtime::HandleError("%s: PTask cannot handle iteration max of 0 (task %s)", __FUNCTION__, bot->GetTaskName());
        if (count_block) count_block->Release();
        return true;
    }
    std::vector<Datablock *> entry(top->m_inputs.size(), nullptr);
    for (size_t q = 0; q < top->m_inputs.size(); ++q) {
        Port *p = top->m_inputs[q];
        if (p->GetPortType() == INPUT_PORT) entry[q] = take_for(top, p);
        else if (p->GetPortType() == STICKY_PORT) entry[q] = p->m_sticky;
    }
    auto find_input = [](Task *t, int formal) -> Port * {
        for (Port *p : t->m_inputs)
            if (p->GetPortType() != META_PORT && (int)p->GetFormalParameterIndex() == formal) return p;
        return nullptr;
    };
    auto block_of = [&](Task *t, int formal) -> Datablock * {
        Port *p = find_input(t, formal);
        if (!p) return nullptr;
        if (p->GetPortType() == STICKY_PORT) return p->m_sticky;
        for (size_t q = 0; q < top->m_inputs.size(); ++q)
            if (top->m_inputs[q] == p) return entry[q];
        return nullptr;
    };

    if (!plan->ev0) {
        ptk_event_create(&plan->ev0);
        ptk_event_create(&plan->ev1);
    }
    int rc = PTK_OK;
    std::vector<Datablock *> fields;   // the blocks that circulate, in top formal order 0..5
    ptk_event_record(plan->ev0, m_stream);

    if (plan->fused_kind && m_fuse_cycles) {
        // FDTDHStep(Hx,Hy,Hz,Ex,Ey,Ez,Da,Db,P) -> FDTDEStep(Ex,Ey,Ez,Hx,Hy,Hz,Ca,Cb,P,SRC,wave)
        for (int q = 0; q < 6; ++q) fields.push_back(block_of(top, q));
        Datablock *pb = block_of(top, 8);
        const ptk_fdtd_params *P = pb ? (const ptk_fdtd_params *)pb->HostBytes() : nullptr;
        Datablock *Da = block_of(top, 6), *Db = block_of(top, 7);
        Port *caP = find_input(bot, 6), *cbP = find_input(bot, 7), *srcP = find_input(bot, 9), *wvP = find_input(bot, 10);
        Datablock *Ca = caP ? caP->m_sticky : nullptr, *Cb = cbP ? cbP->m_sticky : nullptr;
        Datablock *Src = srcP ? srcP->m_sticky : nullptr, *Wave = wvP ? wvP->m_sticky : nullptr;
        for (Datablock *b : fields)
            if (!b) rc = PTK_ERR_INVALID;
        if (!P || !Da || !Db || !Ca || !Cb) rc = PTK_ERR_INVALID;
        if (rc == PTK_OK) {
            if (!plan->solver || memcmp(&plan->solver_params, P, sizeof *P) != 0) {
                if (plan->solver) ptk_solver_destroy(plan->solver);
                plan->solver = nullptr;
                rc = ptk_solver_create(P, &plan->solver);
                plan->solver_params = *P;
                plan->coef_key.clear();
                if (rc == PTK_OK) {
                    // the autotuner's shape if this process tuned the grid, else the default
                    // staged shape: a graph built for one request must not pay for a tuning pass
                    ptk_tile_config tiles{0, 0, 0, 0};
                    if (ptk_default_tiles(P->Nx, P->Ny, P->Nz, &tiles) == PTK_OK)
                        ptk_solver_set_tiles(plan->solver, &tiles);
                }
            }
        }
        if (rc == PTK_OK) {
            std::vector<UINT> key = {Ca->GetDBUID(), Cb->GetDBUID(), Da->GetDBUID(), Db->GetDBUID(),
                                     Src ? Src->GetDBUID() : 0u, Wave ? Wave->GetDBUID() : 0u};
            if (key != plan->coef_key) {
                rc = ptk_solver_set_coefficients(plan->solver, (float *)Ca->DeviceView(m_stream, false, true),
                                                 (float *)Cb->DeviceView(m_stream, false, true),
                                                 (float *)Da->DeviceView(m_stream, false, true),
                                                 (float *)Db->DeviceView(m_stream, false, true), PTK_DEVICE, m_stream);
                int si = -1, sj = -1, sk = -1, n = 0;
                if (Src) {
                    const int *s = (const int *)Src->HostBytes();
                    si = s[0]; sj = s[1]; sk = s[2]; n = s[3];
                }
                if (rc == PTK_OK)
                    rc = ptk_solver_set_source(plan->solver, si, sj, sk,
                                               (n > 0 && Wave) ? (float *)Wave->DeviceView(m_stream, false, true) : nullptr,
                                               n, PTK_DEVICE, m_stream);
                if (rc == PTK_OK) plan->coef_key = key;
            }
        }
        if (rc == PTK_OK) {
            float *dev[6];
            for (int q = 0; q < 6; ++q) dev[q] = (float *)fields[q]->DeviceView(m_stream, true, true);
            rc = ptk_solver_set_fields(plan->solver, dev, PTK_DEVICE, m_stream);
            if (rc == PTK_OK) rc = ptk_solver_reset_clock(plan->solver, m_stream);
            if (rc == PTK_OK) rc = ptk_solver_run(plan->solver, (int)N, m_stream);
            if (rc == PTK_OK) rc = ptk_solver_get_fields(plan->solver, dev, PTK_DEVICE, m_stream);
            long long l = 0;
            ptk_solver_last_launches(plan->solver, &l);
            m_stats.kernel_launches += (UINT64)l;
            m_stats.graph_replays += (UINT64)(N + 31) / 32;
        }
    } else {
        // Generic: capture [top; bottom] once for these blocks, replay N times.
        std::vector<Formal> ftop, fbot;
        std::vector<void *> key;
        auto bind = [&](Task *t, std::vector<Formal> &fv) {
            std::vector<std::pair<int, Formal>> fs;
            for (Port *p : t->m_inputs) {
                if (p->GetPortType() == META_PORT || p->GetFormalParameterIndex() == (UINT)-1) continue;
                Datablock *b = nullptr;
                if (p->GetPortType() == STICKY_PORT) b = p->m_sticky;
                else if (t == top) b = block_of(top, (int)p->GetFormalParameterIndex());
                else {
                    // bottom input fed by the top: the top's forwarded block for that channel
                    for (Channel *c : p->m_in) {
                        Port *src = c->GetBoundPort(CE_SRC);
                        if (!src || src->GetTask() != top) continue;
                        for (size_t q = 0; q < top->m_inputs.size(); ++q)
                            if (top->m_inputs[q]->m_inout_partner == src) b = entry[q];
                    }
                }
                Formal f{p, b, nullptr, nullptr};
                if (b) {
                    if (is_scalar(b)) f.host = b->HostBytes();
                    else f.dev = b->DeviceView(m_stream, p->IsInOutParameter(), true);
                }
                key.push_back(f.dev ? f.dev : (void *)f.host);
                fs.push_back({(int)p->GetFormalParameterIndex(), f});
            }
            std::stable_sort(fs.begin(), fs.end(), [](const std::pair<int, Formal> &a, const std::pair<int, Formal> &b) {
                return a.first < b.first;
            });
            for (auto &x : fs) fv.push_back(x.second);
        };
        bind(top, ftop);
        if (bot != top) bind(bot, fbot);
        for (size_t q = 0; q < top->m_inputs.size(); ++q)
            if (top->m_inputs[q]->GetPortType() == INPUT_PORT) fields.push_back(entry[q]);
        if (bot->m_step_counter) ptk_memset(bot->m_step_counter, 0, sizeof(int), m_stream);
        else if (top->m_step_counter) ptk_memset(top->m_step_counter, 0, sizeof(int), m_stream);
        // The E-step kernel allocates its step counter on first use: do one eager iteration outside
        // the capture so that allocation never happens inside it.
        UINT done = 0;
        if (!plan->exec || key != plan->exec_key) {
            rc = launch_native(top, ftop, m_stream);
            if (rc == PTK_OK && bot != top) rc = launch_native(bot, fbot, m_stream);
            done = 1;
            if (plan->exec) ptk_graph_exec_destroy(plan->exec);
            plan->exec = nullptr;
            if (rc == PTK_OK && N > 1) {
                rc = ptk_capture_begin(m_stream);
                if (rc == PTK_OK) {
                    int r1 = launch_native(top, ftop, m_stream);
                    int r2 = (bot != top) ? launch_native(bot, fbot, m_stream) : PTK_OK;
                    rc = ptk_capture_end(m_stream, &plan->exec);
                    if (r1 != PTK_OK) rc = r1;
                    if (r2 != PTK_OK) rc = r2;
                }
                plan->exec_key = key;
            }
        }
        const long long nodes = (bot != top) ? 2 : 1;
        for (UINT n = done; n < N && rc == PTK_OK; ++n) {
            rc = ptk_graph_exec_launch(plan->exec, m_stream, nodes);
            ++m_stats.graph_replays;
        }
        m_stats.kernel_launches += (UINT64)N * (UINT64)nodes;
    }
    ptk_event_record(plan->ev1, m_stream);
    if (rc != PTK_OK) {
        Runtime::HandleError("lowered loop %s -> %s failed: %s", top->GetTaskName(), bot->GetTaskName(), ptk_last_error());
    }
    for (Datablock *b : fields)
        if (b) b->DeviceWritten(m_stream);
    ++m_stats.cycles_lowered;
    m_stats.cycle_iterations += N;
    top->m_dispatches += N;
    bot->m_dispatches += N;

    // ---- emit the loop's results from the bottom task with DBCTLC_ENDITERATION ----
    std::vector<Datablock *> outs(bot->m_outputs.size(), nullptr);
    for (size_t r = 0; r < bot->m_outputs.size(); ++r) {
        for (Port *p : bot->m_inputs) {
            if (p->GetInOutRoutingIndex() != (int)r) continue;
            // the block behind bottom input p is the top's forwarded entry block
            for (Channel *c : p->m_in) {
                Port *src = c->GetBoundPort(CE_SRC);
                if (!src || src->GetTask() != top) continue;
                for (size_t q = 0; q < top->m_inputs.size(); ++q)
                    if (top->m_inputs[q]->m_inout_partner == src) outs[r] = entry[q];
            }
            if (!outs[r] && bot == top) {
                for (size_t q = 0; q < top->m_inputs.size(); ++q)
                    if (top->m_inputs[q] == p) outs[r] = entry[q];
            }
        }
    }
    for (size_t r = 0; r < outs.size(); ++r) {
        if (!outs[r]) continue;
        bool ctl = std::find(plan->meta->m_ctl_targets.begin(), plan->meta->m_ctl_targets.end(),
                             bot->m_outputs[r]) != plan->meta->m_ctl_targets.end();
        if (ctl) outs[r]->SetControlSignal(DBCTLC_ENDITERATION);
        push_outputs(bot->m_outputs[r], outs[r]);
        if (ctl) outs[r]->ClearControlSignal(DBCTLC_ENDITERATION);
    }
    for (size_t q = 0; q < top->m_inputs.size(); ++q)
        if (top->m_inputs[q]->GetPortType() == INPUT_PORT && entry[q]) entry[q]->Release();
    if (count_block) count_block->Release();
    ptk_event_sync(plan->ev1);
    ptk_event_elapsed_ms(plan->ev0, plan->ev1, &plan->last_ms);
    m_stats.last_cycle_ms = plan->last_ms;
    m_stats.last_cycle_iterations = N;
    return true;
}

bool Graph::schedule_once()
{
    struct Flag {
        bool &f;
        explicit Flag(bool &x) : f(x) { f = true; }
        ~Flag() { f = false; }
    } guard(m_scheduling);
    bool any = false;
    for (Task *t : m_tasks) {
        if (m_stop) break;
        if (try_lower_cycle(t)) {
            any = true;
            continue;
        }
        if (task_ready(t)) {
            dispatch(t);
            any = true;
        }
    }
    return any;
}

}  // namespace PTask
