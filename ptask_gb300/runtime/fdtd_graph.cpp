// fdtd_graph.cpp -- the FDTD task graph built on the PTask API, and its C ABI (ptask_graph.h).
//
// Two structures:
//   * unrolled: the reference's graph (ptaskUnitTest/graphfdtd.cpp:448-739): per step six tasks
//     HxComputation..EzComputation with three input ports, a sticky "Config" port and one output
//     port each; H outputs feed the E tasks of the same step; every output feeds the next step.
//   * cyclic: two tasks in a loop (pattern of ptaskUnitTest/iteration.cpp:197-435).  FDTDHStep takes
//     the six fields through in-out ports and updates H in place; FDTDEStep updates E in place and
//     carries the MF_GENERAL_ITERATOR meta port; its outputs return to FDTDHStep through back channels
//     gated CGATEFN_CLOSE_ON_ENDITERATION, and leave the graph through output channels gated
//     CGATEFN_OPEN_ON_ENDITERATION.
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "ptaskapi.h"
#include "ptask_graph.h"

using namespace PTask;

namespace {

const char *kFieldNames[6] = {"Hx", "Hy", "Hz", "Ex", "Ey", "Ez"};
const char *kTemplateNames[6] = {"HxSize", "HySize", "HzSize", "ExSize", "EySize", "EzSize"};

void extents(int f, int Nx, int Ny, int Nz, UINT e[3])
{
    e[0] = Nx + ((f == 0 || f == 4 || f == 5) ? 1 : 0);
    e[1] = Ny + ((f == 1 || f == 3 || f == 5) ? 1 : 0);
    e[2] = Nz + ((f == 2 || f == 3 || f == 4) ? 1 : 0);
}

struct SourceDesc {
    int i, j, k, n;
};

}  // namespace

struct ptk_fdtd_graph {
    ptk_fdtd_params p{};
    int mode = 0;
    int unrolled_steps = 0;
    Graph *g = nullptr;
    DatablockTemplate *field_t[6] = {};
    DatablockTemplate *param_t = nullptr, *coef_t = nullptr, *src_t = nullptr, *iter_t = nullptr;
    std::vector<GraphInputChannel *> field_in[6];   // every channel a field block is pushed into
    GraphOutputChannel *field_out[6] = {};
    std::vector<GraphInputChannel *> param_in;      // sticky FDTD_PARAMS channels
    GraphInputChannel *coef_in[4] = {};             // Ca, Cb, Da, Db (cyclic)
    GraphInputChannel *src_in = nullptr, *wave_in = nullptr, *iter_in = nullptr;
    bool problem_set = false;
    float last_solve_ms = 0;
    UINT uid = 0;
    std::string host_library;   // unrolled graph: tasks of the fields in host_fields are host tasks
    unsigned host_fields = 0;
    int dep_form = 0;           // host tasks with the GPU as dependent accelerator: 1 LPFNDEPHOSTTASK, 2 ...EX
};

namespace {

// ---- unrolled graph: graphfdtd.cpp:448-739 -------------------------------------------------
Task *field_task(ptk_fdtd_graph *G, const char *kernel, const char *task, int out_field, const int in_fields[3],
                 Port **in, Port **out)
{
    const bool host = (G->host_fields >> out_field) & 1u;
    CompiledKernel *k = Runtime::GetCompiledKernel(host ? G->host_library.c_str() : "fdtdMain.compute_10.ptx", kernel);
    if (!k) return nullptr;
    for (int q = 0; q < 3; ++q)
        in[q] = Runtime::CreatePort(INPUT_PORT, G->field_t[in_fields[q]], G->uid++, kFieldNames[in_fields[q]], q);
    in[3] = Runtime::CreatePort(STICKY_PORT, G->param_t, G->uid++, "Config", 3);
    out[0] = Runtime::CreatePort(OUTPUT_PORT, G->field_t[out_field], G->uid++, kFieldNames[out_field], 4);
    Task *t = G->g->AddTask(k, 4, in, 1, out, task);
    UINT e[3];
    extents(out_field, G->p.Nx, G->p.Ny, G->p.Nz, e);
    // A host task's geometry is the number of times its entry point runs (hosttask.cpp:330-338):
    // once, since the entry point updates the whole field.
    if (host) t->SetComputeGeometry(1, 1, 1);
    if (host && G->dep_form) {
        // the field blocks live on the dependent GPU; FDTD_PARAMS stays a host value
        if (!t->BindDependentAcceleratorClass(ACCELERATOR_CLASS_CUDA, 1, G->dep_form == 2 ? TRUE : FALSE)) return nullptr;
        for (int q = 0; q < 3; ++q) in[q]->BindDependentAccelerator(ACCELERATOR_CLASS_CUDA, 0);
        out[0]->BindDependentAccelerator(ACCELERATOR_CLASS_CUDA, 0);
    }
    else t->SetComputeGeometry((int)e[0], (int)e[1], (int)e[2]);
    return t;
}

bool build_unrolled(ptk_fdtd_graph *G, int steps)
{
    static const char *kernels[6] = {"HxComputation", "HyComputation", "HzComputation",
                                     "ExComputation", "EyComputation", "EzComputation"};
    // inputs of each field task, as graphfdtd.cpp:458-597 wires them
    static const int ins[6][3] = {{0, 4, 5}, {1, 3, 5}, {2, 3, 4}, {3, 1, 2}, {4, 0, 2}, {5, 0, 1}};
    Port *prev[6] = {};
    for (int s = 1; s <= steps; ++s) {
        Port *in[6][4], *out[6][1];
        for (int f = 0; f < 6; ++f) {
            std::string name = std::string(kFieldNames[f]) + "ComTask_" + std::to_string(s);
            if (!field_task(G, kernels[f], name.c_str(), f, ins[f], in[f], out[f])) return false;
            G->param_in.push_back(G->g->AddInputChannel(in[f][3], ("ConstParam" + name).c_str()));
        }
        // H outputs feed the E tasks of the same step (graphfdtd.cpp:606-615)
        for (int e = 3; e < 6; ++e)
            for (int q = 1; q < 3; ++q) {
                int h = ins[e][q];
                G->g->AddInternalChannel(out[h][0], in[e][q],
                                         (std::string(kFieldNames[h]) + "To" + kFieldNames[e] + "_" + std::to_string(s)).c_str());
            }
        for (int f = 0; f < 6; ++f) {
            // inputs taken from outside this step: own field, and E fields for the H tasks
            for (int q = 0; q < 3; ++q) {
                if (f >= 3 && q > 0) continue;   // already wired from this step's H tasks
                int src = ins[f][q];
                std::string cname = std::string(kFieldNames[f]) + "Comp" + kFieldNames[src] + "Input_" + std::to_string(s);
                if (s == 1) G->field_in[src].push_back(G->g->AddInputChannel(in[f][q], cname.c_str()));
                else G->g->AddInternalChannel(prev[src], in[f][q], cname.c_str());
            }
        }
        for (int f = 0; f < 6; ++f) prev[f] = out[f][0];
        if (s == steps)
            for (int f = 0; f < 6; ++f) {
                G->field_out[f] = G->g->AddOutputChannel(out[f][0], (std::string(kFieldNames[f]) + "Output").c_str());
                G->field_out[f]->SetViewMaterializationPolicy(VIEWMATERIALIZATIONPOLICY_EAGER);
            }
    }
    for (GraphInputChannel *c : G->param_in) c->SetNoDraw();
    return true;
}

// ---- cyclic graph -----------------------------------------------------------------------------
void build_cyclic(ptk_fdtd_graph *G)
{
    Port *hin[9], *hout[6], *ein[12], *eout[6];
    for (int q = 0; q < 6; ++q)
        hin[q] = Runtime::CreatePort(INPUT_PORT, G->field_t[q], G->uid++, kFieldNames[q], q, q);
    hin[6] = Runtime::CreatePort(STICKY_PORT, G->coef_t, G->uid++, "Da", 6);
    hin[7] = Runtime::CreatePort(STICKY_PORT, G->coef_t, G->uid++, "Db", 7);
    hin[8] = Runtime::CreatePort(STICKY_PORT, G->param_t, G->uid++, "Config", 8);
    for (int q = 0; q < 6; ++q) hout[q] = Runtime::CreatePort(OUTPUT_PORT, G->field_t[q], G->uid++, kFieldNames[q]);
    // E-step formal order: Ex Ey Ez Hx Hy Hz (fields 3,4,5,0,1,2)
    static const int eorder[6] = {3, 4, 5, 0, 1, 2};
    for (int q = 0; q < 6; ++q)
        ein[q] = Runtime::CreatePort(INPUT_PORT, G->field_t[eorder[q]], G->uid++, kFieldNames[eorder[q]], q, q);
    ein[6] = Runtime::CreatePort(STICKY_PORT, G->coef_t, G->uid++, "Ca", 6);
    ein[7] = Runtime::CreatePort(STICKY_PORT, G->coef_t, G->uid++, "Cb", 7);
    ein[8] = Runtime::CreatePort(STICKY_PORT, G->param_t, G->uid++, "Config", 8);
    ein[9] = Runtime::CreatePort(STICKY_PORT, G->src_t, G->uid++, "Source", 9);
    DatablockTemplate *wave_t = Runtime::GetDatablockTemplate("fdtdwave", sizeof(float), PTPARM_BUFFER);
    ein[10] = Runtime::CreatePort(STICKY_PORT, wave_t, G->uid++, "Wave", 10);
    ein[11] = Runtime::CreatePort(META_PORT, G->iter_t, G->uid++, "Iterations");
    ein[11]->SetMetaFunction(MF_GENERAL_ITERATOR);
    for (int q = 0; q < 6; ++q) eout[q] = Runtime::CreatePort(OUTPUT_PORT, G->field_t[eorder[q]], G->uid++, kFieldNames[eorder[q]]);

    Task *ht = G->g->AddTask(Runtime::GetCompiledKernel("fdtd_gb300", "FDTDHStep"), 9, hin, 6, hout, "HStep");
    Task *et = G->g->AddTask(Runtime::GetCompiledKernel("fdtd_gb300", "FDTDEStep"), 12, ein, 6, eout, "EStep");
    ht->SetComputeGeometry(G->p.Nx + 1, G->p.Ny + 1, G->p.Nz + 1);
    et->SetComputeGeometry(G->p.Nx + 1, G->p.Ny + 1, G->p.Nz + 1);

    for (int q = 0; q < 6; ++q)
        G->field_in[q].push_back(G->g->AddInputChannel(hin[q], (std::string(kFieldNames[q]) + "Input").c_str(), TRUE));
    G->coef_in[2] = G->g->AddInputChannel(hin[6], "DaInput");
    G->coef_in[3] = G->g->AddInputChannel(hin[7], "DbInput");
    G->param_in.push_back(G->g->AddInputChannel(hin[8], "ConfigH"));
    G->coef_in[0] = G->g->AddInputChannel(ein[6], "CaInput");
    G->coef_in[1] = G->g->AddInputChannel(ein[7], "CbInput");
    G->param_in.push_back(G->g->AddInputChannel(ein[8], "ConfigE"));
    G->src_in = G->g->AddInputChannel(ein[9], "SourceInput");
    G->wave_in = G->g->AddInputChannel(ein[10], "WaveInput");
    G->iter_in = G->g->AddInputChannel(ein[11], "IterationCount");
    // H-step forwards all six fields to the E-step.
    for (int q = 0; q < 6; ++q) {
        int f = eorder[q];
        G->g->AddInternalChannel(hout[f], ein[q], (std::string(kFieldNames[f]) + "HToE").c_str());
    }
    // Back channels and outputs of the loop.
    for (int q = 0; q < 6; ++q) {
        int f = eorder[q];
        InternalChannel *back = G->g->AddInternalChannel(eout[q], hin[f], (std::string(kFieldNames[f]) + "Back").c_str(), FALSE);
        back->SetPredicationType(CE_SRC, CGATEFN_CLOSE_ON_ENDITERATION);
        G->field_out[f] = G->g->AddOutputChannel(eout[q], (std::string(kFieldNames[f]) + "Output").c_str());
        G->field_out[f]->SetPredicationType(CE_SRC, CGATEFN_OPEN_ON_ENDITERATION);
        G->field_out[f]->SetViewMaterializationPolicy(VIEWMATERIALIZATIONPOLICY_EAGER);
        G->g->BindControlPropagationPort(ein[11], eout[q]);
    }
    G->param_in[0]->SetNoDraw();
    G->param_in[1]->SetNoDraw();
}

int push_copy(GraphInputChannel *c, DatablockTemplate *t, const void *data, size_t bytes)
{
    Datablock *b = Runtime::AllocateDatablock(t, const_cast<void *>(data), (UINT)bytes, c);
    if (!b) return PTK_ERR_NOMEM;
    BOOL ok = c->Push(b);
    b->Release();
    return ok ? PTK_OK : PTK_ERR_TIMEOUT;
}

// Wrapper with the FDTD templates of `p` and an empty graph (no device work).
ptk_fdtd_graph *new_graph(const ptk_fdtd_params *p, int mode, int unrolled_steps)
{
    auto *G = new ptk_fdtd_graph();
    G->p = *p;
    G->mode = mode;
    G->unrolled_steps = unrolled_steps;
    for (int f = 0; f < 6; ++f) {
        UINT e[3];
        extents(f, p->Nx, p->Ny, p->Nz, e);
        G->field_t[f] = Runtime::GetDatablockTemplate(kTemplateNames[f], sizeof(float), e[0], e[1], e[2]);
    }
    G->param_t = Runtime::GetDatablockTemplate("fdtdparms", sizeof(ptk_fdtd_params), PTPARM_BYVALSTRUCT);
    G->coef_t = Runtime::GetDatablockTemplate("CellCoef", sizeof(float), p->Nx, p->Ny, p->Nz);
    G->src_t = Runtime::GetDatablockTemplate("fdtdsource", sizeof(SourceDesc), PTPARM_BYVALSTRUCT);
    G->iter_t = Runtime::GetDatablockTemplate("dbiter", sizeof(int), PTPARM_INT);
    G->g = new Graph(mode == PTK_GRAPH_UNROLLED ? "graphfdtd_unrolled" : "graphfdtd_cyclic");
    return G;
}

// Lowering choice, Run, and the FDTD_PARAMS block shared by every sticky Config port
// (graphfdtd.cpp:1099-1104).
void start(ptk_fdtd_graph *G)
{
    G->g->SetCycleLowering(G->mode != PTK_GRAPH_CYCLIC_TASKWISE);
    G->g->SetCycleFusion(G->mode == PTK_GRAPH_CYCLIC_FUSED);
    G->g->Run(FALSE);
    Datablock *cp = Runtime::AllocateDatablock(G->param_t, (void *)&G->p, sizeof(G->p), nullptr);
    for (GraphInputChannel *c : G->param_in) c->Push(cp);
    cp->Release();
}

// Find the FDTD graph's boundary channels in a graph read from a file.  Channels are recognised by
// the template and variable binding of the port they feed or drain, not by name: the reference's
// driver names its channels differently (graphfdtd.cpp:617-700) from this runtime's builder.
int bind_loaded(ptk_fdtd_graph *G, int mode)
{
    int cyclic = 0, unrolled = 0;
    for (Task *t : G->g->m_tasks) {
        const std::string op = t->GetCompiledKernel()->GetOperation();
        if (op == "FDTDHStep" || op == "FDTDEStep") ++cyclic;
        else if (op.size() > 11 && op.compare(op.size() - 11, 11, "Computation") == 0) ++unrolled;
        else return PTK_ERR_INVALID;
    }
    if ((cyclic == 0) == (unrolled == 0) || unrolled % 6 || (cyclic && cyclic != 2)) return PTK_ERR_INVALID;
    if (unrolled) {
        G->mode = PTK_GRAPH_UNROLLED;
        G->unrolled_steps = unrolled / 6;
    } else {
        if (mode == PTK_GRAPH_UNROLLED) return PTK_ERR_INVALID;
        G->mode = mode;
    }
    auto field_of = [&](DatablockTemplate *t) {
        for (int f = 0; f < 6; ++f)
            if (t && !strcmp(t->GetTemplateName(), kTemplateNames[f])) return f;
        return -1;
    };
    for (Channel *c : G->g->m_channels) {
        if (c->GetType() == CT_GRAPH_INPUT) {
            Port *d = c->GetBoundPort(CE_DST);
            DatablockTemplate *t = d->GetTemplate();
            const std::string tn = t ? t->GetTemplateName() : "", vb = d->GetVariableBinding();
            auto *in = static_cast<GraphInputChannel *>(c);
            const int f = field_of(t);
            if (f >= 0) {
                if (t->GetXElementCount() != G->field_t[f]->GetXElementCount() ||
                    t->GetYElementCount() != G->field_t[f]->GetYElementCount() ||
                    t->GetZElementCount() != G->field_t[f]->GetZElementCount())
                    return PTK_ERR_INVALID;   // the file was written for another grid
                G->field_in[f].push_back(in);
            } else if (tn == "fdtdparms") {
                G->param_in.push_back(in);
            } else if (tn == "CellCoef") {
                static const char *names[4] = {"Ca", "Cb", "Da", "Db"};
                int q = 0;
                while (q < 4 && vb != names[q]) ++q;
                if (q == 4) return PTK_ERR_INVALID;
                G->coef_in[q] = in;
            } else if (tn == "fdtdsource") {
                G->src_in = in;
            } else if (tn == "fdtdwave") {
                G->wave_in = in;
            } else if (tn == "dbiter") {
                G->iter_in = in;
            } else {
                return PTK_ERR_INVALID;
            }
        } else if (c->GetType() == CT_GRAPH_OUTPUT) {
            const int f = field_of(c->GetBoundPort(CE_SRC)->GetTemplate());
            if (f < 0 || G->field_out[f]) return PTK_ERR_INVALID;
            G->field_out[f] = static_cast<GraphOutputChannel *>(c);
        }
    }
    for (int f = 0; f < 6; ++f)
        if (G->field_in[f].empty() || !G->field_out[f]) return PTK_ERR_INVALID;
    if (G->param_in.empty()) return PTK_ERR_INVALID;
    if (G->mode != PTK_GRAPH_UNROLLED &&
        (!G->coef_in[0] || !G->coef_in[1] || !G->coef_in[2] || !G->coef_in[3] || !G->src_in || !G->wave_in ||
         !G->iter_in))
        return PTK_ERR_INVALID;
    return PTK_OK;
}

}  // namespace

// No C++ exception unwinds into a C caller of the entry points below.
#define PTK_GRAPH_CATCH_ALL                                \
    catch (const std::bad_alloc &) { return PTK_ERR_NOMEM; } \
    catch (...) { return PTK_ERR_STATE; }

extern "C" {

int ptk_fdtd_graph_create(const ptk_fdtd_params *p, int mode, int unrolled_steps, ptk_fdtd_graph **out)
try {
    if (!p || !out || p->Nx < 1 || p->Ny < 1 || p->Nz < 1 || mode < 0 || mode > 3) return PTK_ERR_INVALID;
    if (mode == PTK_GRAPH_UNROLLED && unrolled_steps < 1) return PTK_ERR_INVALID;
    Runtime::SetExitOnRuntimeFailure(FALSE);
    if (PTFAILED(Runtime::Initialize())) return PTK_ERR_CUDA;
    ptk_fdtd_graph *G = new_graph(p, mode, unrolled_steps);
    if (mode == PTK_GRAPH_UNROLLED) build_unrolled(G, unrolled_steps);
    else build_cyclic(G);
    start(G);
    *out = G;
    return PTK_OK;
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_create_host(const ptk_fdtd_params *p, int unrolled_steps, const char *library,
                               unsigned host_fields, ptk_fdtd_graph **out)
try {
    if (!p || !out || !library || p->Nx < 1 || p->Ny < 1 || p->Nz < 1 || unrolled_steps < 1 || host_fields > 0x3Fu)
        return PTK_ERR_INVALID;
    Runtime::SetExitOnRuntimeFailure(FALSE);
    if (PTFAILED(Runtime::Initialize())) return PTK_ERR_CUDA;
    ptk_fdtd_graph *G = new_graph(p, PTK_GRAPH_UNROLLED, unrolled_steps);
    G->host_library = library;
    G->host_fields = host_fields;
    if (!build_unrolled(G, unrolled_steps)) {
        Graph::DestroyGraph(G->g);
        delete G;
        return PTK_ERR_NOTFOUND;
    }
    start(G);
    *out = G;
    return PTK_OK;
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_create_dephost(const ptk_fdtd_params *p, int unrolled_steps, const char *library,
                                  unsigned host_fields, int with_streams, ptk_fdtd_graph **out)
try {
    if (!p || !out || !library || p->Nx < 1 || p->Ny < 1 || p->Nz < 1 || unrolled_steps < 1 || host_fields > 0x3Fu ||
        with_streams < 0 || with_streams > 1)
        return PTK_ERR_INVALID;
    Runtime::SetExitOnRuntimeFailure(FALSE);
    if (PTFAILED(Runtime::Initialize())) return PTK_ERR_CUDA;
    ptk_fdtd_graph *G = new_graph(p, PTK_GRAPH_UNROLLED, unrolled_steps);
    G->host_library = library;
    G->host_fields = host_fields;
    G->dep_form = with_streams ? 2 : 1;
    if (!build_unrolled(G, unrolled_steps)) {
        Graph::DestroyGraph(G->g);
        delete G;
        return PTK_ERR_NOTFOUND;
    }
    start(G);
    *out = G;
    return PTK_OK;
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_export(const ptk_fdtd_params *p, int mode, int unrolled_steps, const char *path)
try {
    if (!p || !path || p->Nx < 1 || p->Ny < 1 || p->Nz < 1 || mode < 0 || mode > 3) return PTK_ERR_INVALID;
    if (mode == PTK_GRAPH_UNROLLED && unrolled_steps < 1) return PTK_ERR_INVALID;
    Runtime::SetExitOnRuntimeFailure(FALSE);
    ptk_fdtd_graph *G = new_graph(p, mode, unrolled_steps);
    if (mode == PTK_GRAPH_UNROLLED) build_unrolled(G, unrolled_steps);
    else build_cyclic(G);
    G->g->Serialize(path);
    const int rc = *G->g->GetSerializationError() ? PTK_ERR_STATE : PTK_OK;
    Graph::DestroyGraph(G->g);
    delete G;
    return rc;
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_save(ptk_fdtd_graph *G, const char *path)
try {
    if (!G || !path) return PTK_ERR_INVALID;
    G->g->Serialize(path);
    return *G->g->GetSerializationError() ? PTK_ERR_STATE : PTK_OK;
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_load(const ptk_fdtd_params *p, int mode, const char *path, ptk_fdtd_graph **out)
try {
    if (!p || !path || !out || p->Nx < 1 || p->Ny < 1 || p->Nz < 1 || mode < 0 || mode > 3) return PTK_ERR_INVALID;
    Runtime::SetExitOnRuntimeFailure(FALSE);
    if (PTFAILED(Runtime::Initialize())) return PTK_ERR_CUDA;
    ptk_fdtd_graph *G = new_graph(p, mode, 0);
    G->g->Deserialize(path);
    int rc = *G->g->GetSerializationError() ? PTK_ERR_STATE : bind_loaded(G, mode);
    if (rc) {
        Graph::DestroyGraph(G->g);
        delete G;
        return rc;
    }
    start(G);
    *out = G;
    return PTK_OK;
} PTK_GRAPH_CATCH_ALL

int ptk_graph_xml_roundtrip(const char *in_path, const char *out_path)
try {
    if (!in_path || !out_path) return PTK_ERR_INVALID;
    Runtime::SetExitOnRuntimeFailure(FALSE);
    Graph *g = new Graph("roundtrip");
    g->Deserialize(in_path);
    int rc = *g->GetSerializationError() ? PTK_ERR_STATE : PTK_OK;
    if (!rc) {
        g->Serialize(out_path);
        if (*g->GetSerializationError()) rc = PTK_ERR_STATE;
    }
    Graph::DestroyGraph(g);
    return rc;
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_set_problem(ptk_fdtd_graph *G, const float *Ca, const float *Cb, const float *Da, const float *Db,
                               int si, int sj, int sk, const float *wave, int nwave)
try {
    if (!G) return PTK_ERR_INVALID;
    if (G->mode == PTK_GRAPH_UNROLLED) {
        // The reference's tasks use the scalar coefficients of FDTD_PARAMS and have no source.
        if (Ca || Cb || Da || Db || (wave && si >= 0)) return PTK_ERR_INVALID;
        G->problem_set = true;
        return PTK_OK;
    }
    const size_t n = (size_t)G->p.Nx * G->p.Ny * G->p.Nz;
    std::vector<float> v[4];
    const float *c[4] = {Ca, Cb, Da, Db};
    if (!Ca || !Cb || !Da || !Db) {
        const float ce = G->p.Dt / G->p.eps0, ch = G->p.Dt / G->p.mu0;
        const float val[4] = {1.0f, ce, 1.0f, ch};
        for (int q = 0; q < 4; ++q) {
            v[q].assign(n, val[q]);
            c[q] = v[q].data();
        }
    }
    for (int q = 0; q < 4; ++q) {
        // The coefficients are read on the device only (the H and E step kernels of the cyclic
        // graph): like the fields, they go straight from the caller's array to the block's device
        // view, with no copy into a host view first.
        Datablock *b = Runtime::AllocateDatablock(G->coef_t, nullptr, 0, G->coef_in[q]);
        if (!b) return PTK_ERR_NOMEM;
        b->UploadFrom(c[q]);
        const BOOL ok = G->coef_in[q]->Push(b);
        b->Release();
        if (!ok) return PTK_ERR_TIMEOUT;
    }
    SourceDesc sd{-1, -1, -1, 0};
    if (wave && nwave > 0 && si >= 0) {
        if (si < 1 || si >= G->p.Nx || sj < 1 || sj >= G->p.Ny || sk < 0 || sk >= G->p.Nz) return PTK_ERR_INVALID;
        sd = SourceDesc{si, sj, sk, nwave};
    }
    int rc = push_copy(G->src_in, G->src_t, &sd, sizeof sd);
    if (rc) return rc;
    float zero = 0.0f;
    DatablockTemplate *wt = Runtime::GetDatablockTemplate("fdtdwave", sizeof(float), (UINT)(sd.n > 0 ? sd.n : 1), 1, 1);
    rc = push_copy(G->wave_in, wt, sd.n > 0 ? (const void *)wave : &zero, (size_t)(sd.n > 0 ? sd.n : 1) * sizeof(float));
    if (rc) return rc;
    G->problem_set = true;
    return PTK_OK;
} PTK_GRAPH_CATCH_ALL

static int solve_impl(ptk_fdtd_graph *G, float *const fields[6], int instances, float *const results[], int steps)
{
    if (!G || !fields || instances < 1 || steps < 1) return PTK_ERR_INVALID;
    if (G->mode == PTK_GRAPH_UNROLLED && steps != G->unrolled_steps) return PTK_ERR_INVALID;
    if (!G->problem_set) {
        int rc = ptk_fdtd_graph_set_problem(G, nullptr, nullptr, nullptr, nullptr, -1, -1, -1, nullptr, 0);
        if (rc) return rc;
    }
    auto t0 = std::chrono::steady_clock::now();
    size_t bytes[6];
    for (int f = 0; f < 6; ++f) bytes[f] = G->field_t[f]->GetDatablockByteCount();
    for (int inst = 0; inst < instances; ++inst) {
        for (int f = 0; f < 6; ++f) {
            // One block per field, pushed into every channel that reads it (graphfdtd.cpp:1078-1096).
            // The fields are read on the device only: they go straight to the block's device view.
            Datablock *b = Runtime::AllocateDatablock(G->field_t[f], nullptr, 0, G->field_in[f][0]);
            if (!b) return PTK_ERR_NOMEM;
            b->UploadFrom(fields[f]);
            for (GraphInputChannel *c : G->field_in[f]) c->Push(b);
            b->Release();
        }
        if (G->mode != PTK_GRAPH_UNROLLED) {
            int it = steps;
            int rc = push_copy(G->iter_in, G->iter_t, &it, sizeof it);
            if (rc) return rc;
        }
    }
    for (int inst = 0; inst < instances; ++inst)
        for (int f = 0; f < 6; ++f) {
            Datablock *b = G->field_out[f]->Pull();
            if (!b) return PTK_ERR_TIMEOUT;
            b->DownloadTo(results ? results[inst * 6 + f] : fields[f]);
            b->Release();
        }
    G->last_solve_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return PTK_OK;
}

int ptk_fdtd_graph_solve(ptk_fdtd_graph *G, float *const fields[6], int steps)
try {
    return solve_impl(G, fields, 1, nullptr, steps);
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_solve_many(ptk_fdtd_graph *G, float *const fields[6], int instances, float *const results[],
                              int steps)
try {
    if (!results) return PTK_ERR_INVALID;
    return solve_impl(G, fields, instances, results, steps);
} PTK_GRAPH_CATCH_ALL

int ptk_fdtd_graph_stats(const ptk_fdtd_graph *G, ptk_graph_stats *st)
{
    if (!G || !st) return PTK_ERR_INVALID;
    GraphStats s = G->g->GetStats();
    st->dispatches = s.dispatches;
    st->host_dispatches = s.host_dispatches;
    st->kernel_launches = s.kernel_launches;
    st->cycles_lowered = s.cycles_lowered;
    st->cycle_iterations = s.cycle_iterations;
    st->graph_replays = s.graph_replays;
    st->last_cycle_ms = s.last_cycle_ms;
    st->last_solve_ms = G->last_solve_ms;
    return PTK_OK;
}

int ptk_fdtd_graph_write_dot(ptk_fdtd_graph *G, const char *path)
{
    if (!G || !path) return PTK_ERR_INVALID;
    G->g->WriteDOTFile(path, FALSE);
    return PTK_OK;
}

int ptk_fdtd_graph_destroy(ptk_fdtd_graph *G)
{
    if (!G) return PTK_OK;
    G->g->Stop();
    G->g->Teardown();
    Graph::DestroyGraph(G->g);
    delete G;
    return PTK_OK;
}

}  // extern "C"
