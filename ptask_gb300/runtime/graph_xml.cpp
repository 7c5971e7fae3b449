// graph_xml.cpp -- Graph::Serialize / Graph::Deserialize: a graph's structure as an XML file.
//
// The document has the reference's layout (ptask/XMLWriter.cpp:124-588, read back in the order of
// ptask/XMLReader.cpp:383-1083): <Graph> holds <DatablockTemplates>, <CompiledKernels>, <Tasks>
// (each with its <InputPorts> and <OutputPorts>), <Channels> (ports referenced by UniqueID) and
// <Actions>, the configuration calls made after construction (Recorder.cpp: SetComputeGeometry,
// SetBlockAndGridSize, SetPredicationType, BindControlPropagationPort, BindControlPropagationChannel,
// BindIterationScope, BindDescriptorPort, BindControlPort).  Element names, order and enum values
// are the reference's, so a graph file written by the reference loads here.  Only the structure is
// stored: datablocks and executions in flight are not.
//
// Differences: the reference records actions in a process-wide recorder as they are called; here
// they are derived from each graph's own state when it is written.  Some state the reference never
// writes is needed to run the cyclic FDTD graph after loading it, so four more action kinds follow
// the reference's: SetMetaFunction (MF_GENERAL_ITERATOR ports), SetSwitchChannel, SetChannelCapacity
// (only where it differs from a new channel's) and SetViewMaterializationPolicy, plus SetNoDraw.  A
// reference reader rejects files that contain them; graphs that use none of that state do not.
// The reader tolerates the XML declaration, comments and whitespace the reference's writer emits.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "PTaskRuntime.h"

namespace PTask {

namespace {

// ---------------------------------------------------------------------------------------------
// Writer
// ---------------------------------------------------------------------------------------------
class XmlOut {
public:
    XmlOut() { m_s << "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n"; }
    void start(const char *n)
    {
        indent();
        m_s << '<' << n << ">\n";
        m_open.push_back(n);
    }
    void end()
    {
        const std::string n = m_open.back();
        m_open.pop_back();
        indent();
        m_s << "</" << n << ">\n";
    }
    void comment(const char *c)
    {
        indent();
        m_s << "<!--" << c << "-->\n";
    }
    void text(const char *n, const std::string &v)
    {
        indent();
        m_s << '<' << n << '>' << escape(v) << "</" << n << ">\n";
    }
    void num(const char *n, long long v) { text(n, std::to_string(v)); }
    void flag(const char *n, bool v) { text(n, v ? "true" : "false"); }
    std::string str() const { return m_s.str(); }

private:
    void indent()
    {
        for (size_t i = 0; i < m_open.size(); ++i) m_s << "  ";
    }
    static std::string escape(const std::string &v)
    {
        std::string o;
        for (char c : v) {
            switch (c) {
            case '&': o += "&amp;"; break;
            case '<': o += "&lt;"; break;
            case '>': o += "&gt;"; break;
            case '"': o += "&quot;"; break;
            default: o += c;
            }
        }
        return o;
    }
    std::ostringstream m_s;
    std::vector<std::string> m_open;
};

// ---------------------------------------------------------------------------------------------
// Reader: a small DOM of element names, text and children
// ---------------------------------------------------------------------------------------------
struct XNode {
    std::string name, text;
    std::vector<XNode> kids;

    const XNode *child(const char *n) const
    {
        for (const XNode &k : kids)
            if (k.name == n) return &k;
        return nullptr;
    }
};

class XmlIn {
public:
    explicit XmlIn(const std::string &s) : m_s(s) {}

    bool parse(XNode &root)
    {
        skip_misc();
        if (!element(root)) return false;
        skip_misc();
        if (m_p != m_s.size()) return fail("content after the root element");
        return true;
    }
    const std::string &error() const { return m_err; }

private:
    bool fail(const char *what)
    {
        if (m_err.empty()) m_err = std::string(what) + " at byte " + std::to_string(m_p);
        return false;
    }
    bool starts(const char *t) const { return m_s.compare(m_p, strlen(t), t) == 0; }
    bool skip_past(const char *t)
    {
        size_t q = m_s.find(t, m_p);
        if (q == std::string::npos) return fail("unterminated markup");
        m_p = q + strlen(t);
        return true;
    }
    void skip_ws()
    {
        while (m_p < m_s.size() && isspace((unsigned char)m_s[m_p])) ++m_p;
    }
    // whitespace, the XML declaration / processing instructions, comments, a DOCTYPE
    void skip_misc()
    {
        for (;;) {
            skip_ws();
            if (starts("<?")) {
                if (!skip_past("?>")) return;
            } else if (starts("<!--")) {
                if (!skip_past("-->")) return;
            } else if (starts("<!")) {
                if (!skip_past(">")) return;
            } else {
                return;
            }
        }
    }
    std::string name()
    {
        size_t b = m_p;
        while (m_p < m_s.size() && !isspace((unsigned char)m_s[m_p]) && m_s[m_p] != '>' && m_s[m_p] != '/') ++m_p;
        return m_s.substr(b, m_p - b);
    }
    static std::string unescape(const std::string &t)
    {
        std::string o;
        for (size_t i = 0; i < t.size(); ++i) {
            if (t[i] != '&') {
                o += t[i];
                continue;
            }
            static const struct { const char *ent; char c; } ents[] = {
                {"&amp;", '&'}, {"&lt;", '<'}, {"&gt;", '>'}, {"&quot;", '"'}, {"&apos;", '\''}};
            bool done = false;
            for (const auto &e : ents)
                if (t.compare(i, strlen(e.ent), e.ent) == 0) {
                    o += e.c;
                    i += strlen(e.ent) - 1;
                    done = true;
                    break;
                }
            if (!done) o += '&';
        }
        return o;
    }
    static std::string trim(const std::string &t)
    {
        size_t b = 0, e = t.size();
        while (b < e && isspace((unsigned char)t[b])) ++b;
        while (e > b && isspace((unsigned char)t[e - 1])) --e;
        return t.substr(b, e - b);
    }
    bool element(XNode &n)
    {
        if (!starts("<")) return fail("expected an element");
        ++m_p;
        n.name = name();
        if (n.name.empty()) return fail("empty element name");
        size_t gt = m_s.find('>', m_p);   // attributes are not used by the format: skipped
        if (gt == std::string::npos) return fail("unterminated start tag");
        const bool empty = gt > 0 && m_s[gt - 1] == '/';
        m_p = gt + 1;
        if (empty) return true;
        std::string raw;
        for (;;) {
            if (m_p >= m_s.size()) return fail("unterminated element");
            if (starts("<!--")) {
                if (!skip_past("-->")) return false;
            } else if (starts("<![CDATA[")) {
                size_t q = m_s.find("]]>", m_p);
                if (q == std::string::npos) return fail("unterminated CDATA");
                raw += m_s.substr(m_p + 9, q - m_p - 9);
                m_p = q + 3;
            } else if (starts("</")) {
                m_p += 2;
                if (name() != n.name) return fail("mismatched end tag");
                skip_ws();
                if (!starts(">")) return fail("unterminated end tag");
                ++m_p;
                n.text = trim(unescape(raw));
                return true;
            } else if (starts("<")) {
                n.kids.emplace_back();
                if (!element(n.kids.back())) return false;
            } else {
                size_t q = m_s.find('<', m_p);
                if (q == std::string::npos) return fail("unterminated text");
                raw += m_s.substr(m_p, q - m_p);
                m_p = q;
            }
        }
    }

    const std::string &m_s;
    size_t m_p = 0;
    std::string m_err;
};

struct LoadError {
    std::string what;
};

const XNode &need(const XNode &n, const char *c)
{
    const XNode *k = n.child(c);
    if (!k) throw LoadError{std::string("<") + n.name + "> has no <" + c + ">"};
    return *k;
}
std::string str_of(const XNode &n, const char *c) { return need(n, c).text; }
long long int_of(const XNode &n, const char *c)
{
    const std::string &t = need(n, c).text;
    errno = 0;
    char *end = nullptr;
    long long v = strtoll(t.c_str(), &end, 10);
    if (t.empty() || *end || errno) throw LoadError{"<" + std::string(c) + "> is not an integer: '" + t + "'"};
    return v;
}
bool bool_of(const XNode &n, const char *c)
{
    std::string t = need(n, c).text;
    for (char &ch : t) ch = (char)tolower((unsigned char)ch);
    if (t == "true" || t == "1") return true;
    if (t == "false" || t == "0") return false;
    throw LoadError{"<" + std::string(c) + "> is not a boolean: '" + t + "'"};
}
// Elements named `c` under `n` in document order (the count element is a cross-check).
std::vector<const XNode *> list_of(const XNode &n, const char *c)
{
    std::vector<const XNode *> v;
    for (const XNode &k : n.kids)
        if (k.name == c) v.push_back(&k);
    if (const XNode *cnt = n.child("Count")) {
        char *end = nullptr;
        long long want = strtoll(cnt->text.c_str(), &end, 10);
        if (want != (long long)v.size())
            throw LoadError{"<" + n.name + "> Count " + cnt->text + " but " + std::to_string(v.size()) + " <" + c + ">"};
    }
    return v;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
void Graph::Serialize(const char *filename)
{
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    m_xml_error.clear();
    std::vector<DatablockTemplate *> templates;
    std::set<DatablockTemplate *> seen_t;
    std::vector<CompiledKernel *> kernels;
    for (Task *t : m_tasks) {
        for (auto *ports : {&t->m_inputs, &t->m_outputs})
            for (Port *p : *ports)
                if (p->GetTemplate() && seen_t.insert(p->GetTemplate()).second) templates.push_back(p->GetTemplate());
        if (std::find(kernels.begin(), kernels.end(), t->GetCompiledKernel()) == kernels.end())
            kernels.push_back(t->GetCompiledKernel());
    }
    XmlOut w;
    w.start("Graph");
    w.comment("  DatablockTemplates  ");
    w.start("DatablockTemplates");
    w.num("Count", (long long)templates.size());
    for (DatablockTemplate *t : templates) {
        w.start("DatablockTemplate");
        w.text("Name", t->GetTemplateName());
        w.num("Stride", t->GetStride());
        w.num("ParamType", (int)t->GetParameterBaseType());
        w.num("ElementsX", t->GetXElementCount());
        w.num("ElementsY", t->GetYElementCount());
        w.num("ElementsZ", t->GetZElementCount());
        w.flag("IsRecordStream", t->IsRecordStream());
        w.flag("IsByteAddressable", t->IsByteAddressable());
        w.end();
    }
    w.end();
    w.comment("  CompiledKernels  ");
    w.comment("  (KernelID is internal to this serialization. Used to associate each Task with its CompiledKernel)  ");
    w.start("CompiledKernels");
    w.num("Count", (long long)kernels.size());
    for (size_t i = 0; i < kernels.size(); ++i) {
        w.start("CompiledKernel");
        w.num("KernelID", (long long)i);
        w.text("SourceFile", kernels[i]->GetSourceFile());
        w.text("Operation", kernels[i]->GetOperation());
        w.end();
    }
    w.end();
    auto port = [&](Port *p) {
        w.start("Port");
        w.num("UniqueID", p->GetUID());
        w.num("OriginalIndex", p->GetOriginalIndex());
        w.num("Type", (int)p->GetPortType());
        w.text("DatablockTemplate", p->GetTemplate() ? p->GetTemplate()->GetTemplateName() : "");
        w.text("VariableBinding", p->GetVariableBinding());
        w.num("ParameterIndex", p->GetFormalParameterIndex());
        w.num("InOutIndex", p->GetInOutRoutingIndex());
        w.end();
    };
    w.comment("  Tasks  ");
    w.start("Tasks");
    w.num("Count", (long long)m_tasks.size());
    for (Task *t : m_tasks) {
        w.start("Task");
        w.text("Name", t->GetTaskName());
        w.num("KernelID", (long long)(std::find(kernels.begin(), kernels.end(), t->GetCompiledKernel()) - kernels.begin()));
        w.num("AcceleratorClass", (int)t->GetAcceleratorClass());
        w.start("InputPorts");
        w.num("Count", (long long)t->m_inputs.size());
        for (Port *p : t->m_inputs) port(p);
        w.end();
        w.start("OutputPorts");
        w.num("Count", (long long)t->m_outputs.size());
        for (Port *p : t->m_outputs) port(p);
        w.end();
        w.end();
    }
    w.end();
    w.comment("  Channels  ");
    w.comment("  (Ports are referenced by their UniqueID)  ");
    w.start("Channels");
    w.num("Count", (long long)m_channels.size());
    for (Channel *c : m_channels) {
        w.start("Channel");
        w.text("Name", c->GetName());
        w.num("Type", (int)c->GetType());
        Port *s = c->GetBoundPort(CE_SRC), *d = c->GetBoundPort(CE_DST);
        w.num("SourcePort", s ? (long long)s->GetUID() : -1LL);
        w.num("DestinationPort", d ? (long long)d->GetUID() : -1LL);
        w.end();
    }
    w.end();

    // Actions: the configuration calls, regenerated from this graph's state.
    std::vector<std::function<void()>> acts;
    auto action = [&](const char *name, std::function<void()> body) {
        acts.push_back([&w, name, body] {
            w.start("Action");
            w.text("ActionName", name);
            body();
            w.end();
        });
    };
    for (Task *t : m_tasks) {
        if (t->m_geom_set)
            action("SetComputeGeometry", [&w, t] {
                w.text("TaskName", t->GetTaskName());
                w.num("PreferredXDim", t->m_geom.x);
                w.num("PreferredYDim", t->m_geom.y);
                w.num("PreferredZDim", t->m_geom.z);
            });
        if (t->m_explicit_launch)
            action("SetBlockAndGridSize", [&w, t] {
                w.text("TaskName", t->GetTaskName());
                w.num("BlockXDim", t->m_block.x);
                w.num("BlockYDim", t->m_block.y);
                w.num("BlockZDim", t->m_block.z);
                w.num("GridXDim", t->m_grid.x);
                w.num("GridYDim", t->m_grid.y);
                w.num("GridZDim", t->m_grid.z);
            });
    }
    for (Channel *c : m_channels)
        for (CHANNELENDPOINTTYPE e : {CE_SRC, CE_DST})
            if (c->GetPredicationType(e) != CGATEFN_NONE)
                action("SetPredicationType", [&w, c, e] {
                    w.text("ChannelName", c->GetName());
                    w.num("EndpointType", (int)e);
                    w.num("CanonicalPredicate", (int)c->GetPredicationType(e));
                });
    for (Port *p : m_ports)
        for (Port *o : p->m_ctl_targets)
            action("BindControlPropagationPort", [&w, p, o] {
                w.num("InputPort", p->GetUID());
                w.num("OutputPort", o->GetUID());
            });
    for (auto &b : m_ctl_channels)
        action("BindControlPropagationChannel", [&w, b] {
            w.num("InputPort", b.first->GetUID());
            w.text("ControlledChannel", b.second->GetName());
        });
    for (auto &b : m_iter_scopes)
        action("BindIterationScope", [&w, b] {
            w.num("MetaPort", b.first->GetUID());
            w.num("ScopedPort", b.second->GetUID());
        });
    for (auto &b : m_descriptors)
        action("BindDescriptorPort", [&w, b] {
            w.num("DescribedPort", b.described->GetUID());
            w.num("DescriberPort", b.describer->GetUID());
            w.num("DescriptorFunction", (int)b.func);
        });
    for (auto &b : m_control_ports)
        action("BindControlPort", [&w, b] {
            w.num("ControllerPort", b.controller->GetUID());
            w.num("GatedPort", b.gated->GetUID());
            w.flag("InitiallyOpen", b.open != FALSE);
        });
    // state the reference does not write (see the file comment)
    for (Port *p : m_ports)
        if (p->GetMetaFunction() != MF_NONE)
            action("SetMetaFunction", [&w, p] {
                w.num("Port", p->GetUID());
                w.num("MetaFunction", (int)p->GetMetaFunction());
            });
    const UINT cap_in = (UINT)Runtime::GetDefaultChannelCapacity();
    for (Channel *c : m_channels) {
        if (c->IsSwitchChannel()) action("SetSwitchChannel", [&w, c] { w.text("ChannelName", c->GetName()); });
        const UINT dflt = c->GetType() == CT_GRAPH_INPUT ? cap_in : 0;
        if (c->GetCapacity() != dflt)
            action("SetChannelCapacity", [&w, c] {
                w.text("ChannelName", c->GetName());
                w.num("Capacity", c->GetCapacity());
            });
        if (c->GetViewMaterializationPolicy() != VIEWMATERIALIZATIONPOLICY_ON_DEMAND)
            action("SetViewMaterializationPolicy", [&w, c] {
                w.text("ChannelName", c->GetName());
                w.num("Policy", (int)c->GetViewMaterializationPolicy());
            });
        if (!c->ShouldDraw()) action("SetNoDraw", [&w, c] { w.text("ChannelName", c->GetName()); });
    }
    w.start("Actions");
    w.num("Count", (long long)acts.size());
    for (auto &a : acts) a();
    w.end();
    w.end();

    std::ofstream f(filename ? filename : "", std::ios::binary | std::ios::trunc);
    if (!f) {
        m_xml_error = std::string("cannot open ") + (filename ? filename : "(null)") + " for writing";
        Runtime::HandleError("Graph::Serialize(%s): %s", GetName(), m_xml_error.c_str());
        return;
    }
    const std::string s = w.str();
    f.write(s.data(), (std::streamsize)s.size());
    if (!f) {
        m_xml_error = std::string("write to ") + filename + " failed";
        Runtime::HandleError("Graph::Serialize(%s): %s", GetName(), m_xml_error.c_str());
    }
}

// ---------------------------------------------------------------------------------------------
void Graph::Deserialize(const char *filename)
{
    m_xml_error.clear();
    std::ifstream f(filename ? filename : "", std::ios::binary);
    if (!f) {
        m_xml_error = std::string("cannot open ") + (filename ? filename : "(null)");
        Runtime::HandleError("Graph::Deserialize: %s", m_xml_error.c_str());
        return;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string doc = ss.str();
    XNode root;
    XmlIn in(doc);
    if (!in.parse(root)) {
        m_xml_error = "malformed XML: " + in.error();
        Runtime::HandleError("Graph::Deserialize(%s): %s", filename, m_xml_error.c_str());
        return;
    }
    std::lock_guard<std::recursive_mutex> lk(m_sched_mu);
    if (!m_tasks.empty() || !m_channels.empty()) {
        m_xml_error = "the graph is not empty";
        Runtime::HandleError("Graph::Deserialize(%s): %s", filename, m_xml_error.c_str());
        return;
    }
    try {
        if (root.name != "Graph") throw LoadError{"root element is <" + root.name + ">, not <Graph>"};
        std::set<std::string> switches;
        const XNode &actions = need(root, "Actions");
        for (const XNode *a : list_of(actions, "Action"))
            if (str_of(*a, "ActionName") == "SetSwitchChannel") switches.insert(str_of(*a, "ChannelName"));

        std::map<std::string, DatablockTemplate *> tmap;
        for (const XNode *t : list_of(need(root, "DatablockTemplates"), "DatablockTemplate")) {
            const std::string name = str_of(*t, "Name");
            const UINT stride = (UINT)int_of(*t, "Stride");
            const PTASK_PARM_TYPE pt = (PTASK_PARM_TYPE)int_of(*t, "ParamType");
            DatablockTemplate *d =
                pt == PTPARM_NONE
                    ? Runtime::GetDatablockTemplate(name.c_str(), stride, (UINT)int_of(*t, "ElementsX"),
                                                    (UINT)int_of(*t, "ElementsY"), (UINT)int_of(*t, "ElementsZ"),
                                                    bool_of(*t, "IsRecordStream"), bool_of(*t, "IsByteAddressable"))
                    : Runtime::GetDatablockTemplate(name.c_str(), stride, pt);
            if (!d) throw LoadError{"template " + name + " could not be created"};
            tmap[name] = d;
        }
        std::map<long long, CompiledKernel *> kmap;
        for (const XNode *k : list_of(need(root, "CompiledKernels"), "CompiledKernel")) {
            const std::string file = str_of(*k, "SourceFile"), op = str_of(*k, "Operation");
            CompiledKernel *ck = Runtime::GetCompiledKernel(file.c_str(), op.c_str());
            if (!ck) throw LoadError{"no kernel for " + file + ":" + op};
            kmap[int_of(*k, "KernelID")] = ck;
        }
        std::map<UINT, Port *> pmap;
        auto read_ports = [&](const XNode &grp, std::vector<Port *> &out) {
            std::vector<const XNode *> ps = list_of(grp, "Port");
            out.assign(ps.size(), nullptr);
            for (const XNode *p : ps) {
                const UINT uid = (UINT)int_of(*p, "UniqueID");
                const long long idx = int_of(*p, "OriginalIndex");
                if (idx < 0 || idx >= (long long)ps.size() || out[(size_t)idx])
                    throw LoadError{"port " + std::to_string(uid) + ": bad OriginalIndex"};
                const std::string tname = str_of(*p, "DatablockTemplate");
                auto ti = tmap.find(tname);
                if (ti == tmap.end()) throw LoadError{"port " + std::to_string(uid) + ": unknown template " + tname};
                const std::string binding = str_of(*p, "VariableBinding");
                Port *port = Runtime::CreatePort((PORTTYPE)int_of(*p, "Type"), ti->second, uid, binding.c_str(),
                                                 (UINT)int_of(*p, "ParameterIndex"), (UINT)int_of(*p, "InOutIndex"));
                if (!port) throw LoadError{"port " + std::to_string(uid) + " could not be created"};
                port->SetOriginalIndex((UINT)idx);
                if (!pmap.emplace(uid, port).second) throw LoadError{"duplicate port UniqueID " + std::to_string(uid)};
                out[(size_t)idx] = port;
            }
        };
        for (const XNode *t : list_of(need(root, "Tasks"), "Task")) {
            const std::string name = str_of(*t, "Name");
            auto ki = kmap.find(int_of(*t, "KernelID"));
            if (ki == kmap.end()) throw LoadError{"task " + name + ": unknown KernelID"};
            const long long cls = int_of(*t, "AcceleratorClass");
            const long long have = ki->second->IsHost() ? (long long)ACCELERATOR_CLASS_HOST : (long long)ACCELERATOR_CLASS_CUDA;
            if (cls != have)
                throw LoadError{"task " + name + ": accelerator class " + std::to_string(cls) + " but its kernel is " +
                                (ki->second->IsHost() ? "a host task" : "a CUDA kernel")};
            std::vector<Port *> ins, outs;
            read_ports(need(*t, "InputPorts"), ins);
            read_ports(need(*t, "OutputPorts"), outs);
            if (!AddTask(ki->second, (UINT)ins.size(), ins.data(), (UINT)outs.size(), outs.data(), name.c_str()))
                throw LoadError{"task " + name + " could not be added"};
        }
        auto port_of = [&](long long uid, const std::string &ch) -> Port * {
            auto it = pmap.find((UINT)uid);
            if (it == pmap.end()) throw LoadError{"channel " + ch + ": unknown port " + std::to_string(uid)};
            return it->second;
        };
        for (const XNode *c : list_of(need(root, "Channels"), "Channel")) {
            const std::string name = str_of(*c, "Name");
            if (name.rfind("BindDescriptorPort_Channel_", 0) == 0) continue;   // made by BindDescriptorPort
            const BOOL sw = switches.count(name) ? TRUE : FALSE;
            switch ((CHANNELTYPE)int_of(*c, "Type")) {
            case CT_GRAPH_INPUT: AddInputChannel(port_of(int_of(*c, "DestinationPort"), name), name.c_str(), sw); break;
            case CT_GRAPH_OUTPUT: AddOutputChannel(port_of(int_of(*c, "SourcePort"), name), name.c_str()); break;
            case CT_INTERNAL:
                AddInternalChannel(port_of(int_of(*c, "SourcePort"), name), port_of(int_of(*c, "DestinationPort"), name),
                                   name.c_str(), sw);
                break;
            default: throw LoadError{"channel " + name + ": unsupported channel type"};
            }
        }
        auto chan = [&](const XNode &a, const char *el) -> Channel * {
            const std::string n = str_of(a, el);
            Channel *c = GetChannel(n.c_str());
            if (!c) throw LoadError{"action refers to unknown channel " + n};
            return c;
        };
        auto task = [&](const XNode &a) -> Task * {
            const std::string n = str_of(a, "TaskName");
            Task *t = GetTask(n.c_str());
            if (!t) throw LoadError{"action refers to unknown task " + n};
            return t;
        };
        for (const XNode *a : list_of(actions, "Action")) {
            const std::string n = str_of(*a, "ActionName");
            if (n == "SetComputeGeometry") {
                task(*a)->SetComputeGeometry((int)int_of(*a, "PreferredXDim"), (int)int_of(*a, "PreferredYDim"),
                                             (int)int_of(*a, "PreferredZDim"));
            } else if (n == "SetBlockAndGridSize") {
                task(*a)->SetBlockAndGridSize(
                    PTASKDIM3((int)int_of(*a, "GridXDim"), (int)int_of(*a, "GridYDim"), (int)int_of(*a, "GridZDim")),
                    PTASKDIM3((int)int_of(*a, "BlockXDim"), (int)int_of(*a, "BlockYDim"), (int)int_of(*a, "BlockZDim")));
            } else if (n == "SetPredicationType") {
                chan(*a, "ChannelName")->SetPredicationType((CHANNELENDPOINTTYPE)int_of(*a, "EndpointType"),
                                                            (CHANNELPREDICATE)int_of(*a, "CanonicalPredicate"));
            } else if (n == "BindControlPropagationPort") {
                BindControlPropagationPort(port_of(int_of(*a, "InputPort"), n), port_of(int_of(*a, "OutputPort"), n));
            } else if (n == "BindControlPropagationChannel") {
                BindControlPropagationChannel(port_of(int_of(*a, "InputPort"), n), chan(*a, "ControlledChannel"));
            } else if (n == "BindIterationScope") {
                BindIterationScope(port_of(int_of(*a, "MetaPort"), n), port_of(int_of(*a, "ScopedPort"), n));
            } else if (n == "BindDescriptorPort") {
                BindDescriptorPort(port_of(int_of(*a, "DescribedPort"), n), port_of(int_of(*a, "DescriberPort"), n),
                                   (DESCRIPTORFUNC)int_of(*a, "DescriptorFunction"));
            } else if (n == "BindControlPort") {
                BindControlPort(port_of(int_of(*a, "ControllerPort"), n), port_of(int_of(*a, "GatedPort"), n),
                                bool_of(*a, "InitiallyOpen") ? TRUE : FALSE);
            } else if (n == "SetMetaFunction") {
                port_of(int_of(*a, "Port"), n)->SetMetaFunction((METAFUNCTION)int_of(*a, "MetaFunction"));
            } else if (n == "SetSwitchChannel") {
                // applied when the channel was created
            } else if (n == "SetChannelCapacity") {
                chan(*a, "ChannelName")->SetCapacity((UINT)int_of(*a, "Capacity"));
            } else if (n == "SetViewMaterializationPolicy") {
                chan(*a, "ChannelName")->SetViewMaterializationPolicy((VIEWMATERIALIZATIONPOLICY)int_of(*a, "Policy"));
            } else if (n == "SetNoDraw") {
                chan(*a, "ChannelName")->SetNoDraw();
            } else {
                throw LoadError{"unknown action " + n};
            }
        }
    } catch (const LoadError &e) {
        m_xml_error = e.what;
        Runtime::HandleError("Graph::Deserialize(%s): %s", filename, e.what.c_str());
    }
}

}  // namespace PTask
