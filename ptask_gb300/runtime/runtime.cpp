// runtime.cpp -- PTask::Runtime entry points, datablock templates, datablocks and kernel
// resolution for the GB300 runtime.  Device work goes through the C ABI of libptask_gb300.so.
#include <dlfcn.h>

#include <algorithm>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "PTaskRuntime.h"
#include "ptask_gb300.h"

namespace PTask {

namespace {

struct Config {
    BOOL use_cuda = TRUE, use_opencl = FALSE, use_dx = FALSE, use_host = TRUE;   // PTaskRuntime.cpp:2298
    BOOL verbose = FALSE;
    int channel_capacity = 4;             // DEFAULT_CHANNEL_CAPACITY, PTaskRuntime.cpp:79
    SCHEDULINGMODE sched = SCHEDMODE_DATADRIVEN;
    THREADPOOLPOLICY tpp = TPP_AUTOMATIC;
    int max_concurrency = 1;
    BOOL exit_on_failure = TRUE;          // PTaskRuntime.cpp:192
    DWORD watchdog_ms = 5000;
};

Config g_cfg;
std::mutex g_mu;
bool g_init = false;
std::map<std::string, DatablockTemplate *> g_templates;
std::map<std::string, CompiledKernel *> g_kernels;
std::atomic<UINT> g_block_uid{1};
void *g_io_stream = nullptr;
Accelerator g_accel;

void vlog(FILE *f, const char *prefix, const char *fmt, va_list ap)
{
    fputs(prefix, f);
    vfprintf(f, fmt, ap);
    size_t n = strlen(fmt);
    if (n == 0 || fmt[n - 1] != '\n') fputc('\n', f);
    fflush(f);
}

}  // namespace

void *runtime_io_stream() { return g_io_stream; }

// Streams handed to graphs; kept for the life of the process because blocks may be freed on them
// after their graph is gone.
static std::mutex g_stream_mu;
static std::vector<void *> g_free_streams;

void *acquire_stream()
{
    std::lock_guard<std::mutex> lk(g_stream_mu);
    if (!g_free_streams.empty()) {
        void *s = g_free_streams.back();
        g_free_streams.pop_back();
        return s;
    }
    void *s = nullptr;
    return ptk_stream_create(&s) == PTK_OK ? s : nullptr;
}

void release_stream(void *s)
{
    if (!s) return;
    ptk_stream_sync(s);
    std::lock_guard<std::mutex> lk(g_stream_mu);
    g_free_streams.push_back(s);
}

const char *ControlSignalString(CONTROLSIGNAL s)
{
    static const char *names[] = {"DBCTLC_NONE", "DBCTLC_BOF", "DBCTLC_EOF", "DBCTLC_BEGINITERATION",
                                  "DBCTLC_ENDITERATION", "DBCTLC_ERR", "DBCTLC_DEVNULL"};
    if (!s) return names[0];
    for (int i = 0; i < 6; ++i)
        if (s & (1ull << i)) return names[i + 1];
    return "DBCTLC_UNKNOWN";
}

const char *ViewPolicyString(VIEWMATERIALIZATIONPOLICY p)
{
    return p == VIEWMATERIALIZATIONPOLICY_EAGER ? "VIEWMATERIALIZATIONPOLICY_EAGER"
                                                : "VIEWMATERIALIZATIONPOLICY_ON_DEMAND";
}

// ---------------------------------------------------------------------------------------------
DatablockTemplate::DatablockTemplate(const char *name, UINT stride, UINT x, UINT y, UINT z, bool record,
                                     bool raw)
    : m_name(name ? name : ""), m_stride(stride), m_dims{x, y, z}, m_parm(PTPARM_NONE), m_record(record),
      m_raw(raw)
{
}

DatablockTemplate::DatablockTemplate(const char *name, UINT stride, PTASK_PARM_TYPE type)
    : m_name(name ? name : ""), m_stride(stride), m_dims{1, 1, 1}, m_parm(type), m_record(false), m_raw(false)
{
}

// ---------------------------------------------------------------------------------------------
Datablock::Datablock(DatablockTemplate *t, size_t bytes, CONTROLSIGNAL sig)
    : m_template(t), m_bytes(bytes), m_signals(sig), m_uid(g_block_uid.fetch_add(1))
{
}

Datablock::~Datablock()
{
    if (m_event) {
        ptk_event_sync(m_event);
        ptk_event_destroy(m_event);
    }
    if (m_dev) ptk_mem_free(m_dev, m_dev_stream);
    if (m_host) ptk_host_free(m_host);
}

long Datablock::AddRef() { return ++m_refs; }

long Datablock::Release()
{
    long r = --m_refs;
    if (r == 0) delete this;
    return r;
}

void Datablock::ensure_host_alloc()
{
    if (!m_host) {
        if (ptk_host_alloc(m_bytes ? m_bytes : 16, &m_host) != PTK_OK)
            Runtime::HandleError("%s: pinned host allocation of %zu bytes failed: %s", __FUNCTION__, m_bytes,
                                 ptk_last_error());
    }
}

void Datablock::sync_host()
{
    if (m_host_valid) return;
    if (m_d2h_pending) {
        ptk_event_sync(m_event);
        m_d2h_pending = false;
        m_host_valid = true;
        return;
    }
    if (!m_dev_valid) {
        ensure_host_alloc();
        memset(m_host, 0, m_bytes);
        m_host_valid = true;
        return;
    }
    ensure_host_alloc();
    void *io = runtime_io_stream();
    if (m_event) ptk_stream_wait_event(io, m_event);
    if (ptk_memcpy_d2h(m_host, m_dev, m_bytes, io) != PTK_OK || ptk_stream_sync(io) != PTK_OK)
        Runtime::HandleError("%s: device-to-host copy failed: %s", __FUNCTION__, ptk_last_error());
    m_host_valid = true;
}

void *Datablock::GetDataPointer(BOOL bWriteable, BOOL bSynchronizeBufferView)
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    if (bSynchronizeBufferView) sync_host();
    ensure_host_alloc();
    if (m_event && m_dev_valid && !m_d2h_pending) ptk_event_sync(m_event);   // pending H2D reads m_host
    if (bWriteable) {
        // The caller writes the host view: it becomes the only valid copy.
        if (m_d2h_pending) ptk_event_sync(m_event);
        m_d2h_pending = false;
        m_host_valid = true;
        m_dev_valid = false;
    }
    return m_host;
}

const void *Datablock::HostBytes()
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    sync_host();
    return m_host;
}

void *Datablock::DeviceView(void *stream, bool for_write, bool keep_contents)
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    if (!m_dev) {
        if (ptk_mem_alloc(m_bytes ? m_bytes : 16, stream, &m_dev) != PTK_OK) {
            Runtime::HandleError("%s: device allocation of %zu bytes failed: %s", __FUNCTION__, m_bytes,
                                 ptk_last_error());
            return nullptr;
        }
        m_dev_stream = stream;
    }
    if (m_dev_stream != stream && m_event) ptk_stream_wait_event(stream, m_event);
    if (keep_contents && !m_dev_valid) {
        if (m_host_valid) {
            ptk_memcpy_h2d(m_dev, m_host, m_bytes, stream);
            if (!m_event) ptk_event_create(&m_event);
            ptk_event_record(m_event, stream);
        } else {
            ptk_memset(m_dev, 0, m_bytes, stream);
        }
    }
    m_dev_valid = true;
    m_dev_stream = stream;
    if (for_write) {
        m_host_valid = false;
        m_d2h_pending = false;
    }
    return m_dev;
}

void Datablock::DeviceWritten(void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    if (!m_event) ptk_event_create(&m_event);
    ptk_event_record(m_event, stream);
    m_dev_valid = true;
    m_host_valid = false;
    m_d2h_pending = false;
}

void Datablock::UploadFrom(const void *src)
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    void *io = runtime_io_stream();
    if (!m_dev) {
        if (ptk_mem_alloc(m_bytes ? m_bytes : 16, io, &m_dev) != PTK_OK) {
            Runtime::HandleError("%s: device allocation of %zu bytes failed: %s", __FUNCTION__, m_bytes,
                                 ptk_last_error());
            return;
        }
        m_dev_stream = io;
    }
    if (m_dev_stream != io && m_event) ptk_stream_wait_event(io, m_event);
    // A pageable source is staged by the driver before the call returns; a pinned one is read by
    // the copy engine, so the event below is what a caller reusing it would wait for.
    if (ptk_memcpy_h2d(m_dev, src, m_bytes, io) != PTK_OK) {
        Runtime::HandleError("%s: host-to-device copy failed: %s", __FUNCTION__, ptk_last_error());
        return;
    }
    if (!m_event) ptk_event_create(&m_event);
    ptk_event_record(m_event, io);
    m_dev_stream = io;
    m_dev_valid = true;
    m_host_valid = false;
    m_d2h_pending = false;
}

void Datablock::DownloadTo(void *dst)
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    if (m_d2h_pending) {
        ptk_event_sync(m_event);
        m_d2h_pending = false;
        m_host_valid = true;
    }
    if (m_host_valid) {
        HostCopy(dst, m_host, m_bytes);
        return;
    }
    if (!m_dev_valid) {
        memset(dst, 0, m_bytes);
        return;
    }
    void *io = runtime_io_stream();
    if (m_event) ptk_stream_wait_event(io, m_event);
    if (ptk_memcpy_d2h(dst, m_dev, m_bytes, io) != PTK_OK || ptk_stream_sync(io) != PTK_OK)
        Runtime::HandleError("%s: device-to-host copy failed: %s", __FUNCTION__, ptk_last_error());
}

void Datablock::StartHostMaterialization(void *stream)
{
    std::lock_guard<std::recursive_mutex> lk(m_lock);
    if (m_host_valid || !m_dev_valid || m_d2h_pending) return;
    ensure_host_alloc();
    ptk_memcpy_d2h(m_host, m_dev, m_bytes, stream);
    if (!m_event) ptk_event_create(&m_event);
    ptk_event_record(m_event, stream);
    m_d2h_pending = true;
}

// ---------------------------------------------------------------------------------------------
const char *Accelerator::GetDeviceName()
{
    static char name[256] = {0};
    if (!name[0]) ptk_device_info(name, sizeof name, nullptr, nullptr, nullptr);
    return name;
}

UINT Accelerator::GetCoreCount()
{
    int sms = 0;
    ptk_device_info(nullptr, 0, &sms, nullptr, nullptr);
    return (UINT)sms;
}

size_t Accelerator::GetGlobalMemorySize()
{
    size_t t = 0;
    ptk_device_info(nullptr, 0, nullptr, &t, nullptr);
    return t;
}

void HostCopy(void *dst, const void *src, size_t bytes)
{
    constexpr size_t kPiece = (size_t)4 << 20;
    if (bytes < 4 * kPiece) {
        memcpy(dst, src, bytes);
        return;
    }
    const long long n = (long long)((bytes + kPiece - 1) / kPiece);
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < n; ++c) {
        const size_t o = (size_t)c * kPiece;
        memcpy(static_cast<char *>(dst) + o, static_cast<const char *>(src) + o, std::min(kPiece, bytes - o));
    }
}

namespace Runtime {

PTRESULT Initialize()
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_init) return PTASK_OK;
    if (!g_cfg.use_cuda) {
        MandatoryInform("PTask::Runtime::Initialize: only the CUDA backend exists in this runtime\n");
        return PTASK_ERR_INVALID_PARAMETER;
    }
    if (ptk_runtime_init(0) != PTK_OK) {
        ErrorMessage(std::string("PTask::Runtime::Initialize: ") + ptk_last_error());
        return PTASK_ERR_UNINITIALIZED;
    }
    if (ptk_stream_create(&g_io_stream) != PTK_OK) return PTASK_ERR;
    g_init = true;
    return PTASK_OK;
}

PTRESULT Terminate()
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_init) return PTASK_OK;
    ptk_stream_sync(g_io_stream);
    ptk_stream_destroy(g_io_stream);
    g_io_stream = nullptr;
    std::set<DatablockTemplate *> uniq;
    for (auto &kv : g_templates) uniq.insert(kv.second);
    for (DatablockTemplate *t : uniq) delete t;
    g_templates.clear();
    for (auto &kv : g_kernels) delete kv.second;
    g_kernels.clear();
    ptk_runtime_shutdown();
    g_init = false;
    return PTASK_OK;
}

BOOL IsInitialized() { return g_init; }

DatablockTemplate *GetDatablockTemplate(const char *name, unsigned int stride, unsigned int x, unsigned int y,
                                        unsigned int z, bool rec, bool raw)
{
    // A template is identified by its name and shape: graphs of different sizes that reuse a name
    // (every FDTD graph calls its field templates "HxSize" ...) get distinct templates.
    std::lock_guard<std::mutex> lk(g_mu);
    std::string key = std::string(name ? name : "") + "#" + std::to_string(stride) + "," + std::to_string(x) +
                      "," + std::to_string(y) + "," + std::to_string(z) + (rec ? "r" : "") + (raw ? "b" : "");
    auto it = g_templates.find(key);
    if (it != g_templates.end()) return it->second;
    auto *t = new DatablockTemplate(name, stride, x, y, z, rec, raw);
    g_templates[key] = t;
    g_templates[name ? name : ""] = t;   // latest template of this name, for lookup by name
    return t;
}

DatablockTemplate *GetDatablockTemplate(const char *name, unsigned int stride, PTASK_PARM_TYPE type)
{
    std::lock_guard<std::mutex> lk(g_mu);
    std::string key = name ? name : "";
    auto it = g_templates.find(key);
    if (it != g_templates.end()) return it->second;
    auto *t = new DatablockTemplate(name, stride, type);
    g_templates[key] = t;
    return t;
}

DatablockTemplate *GetDatablockTemplate(const char *name)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_templates.find(name ? name : "");
    return it == g_templates.end() ? nullptr : it->second;
}

Port *CreatePort(PORTTYPE type, DatablockTemplate *t, UINT uid, const char *binding, UINT param_idx,
                 UINT inout_idx)
{
    int pi = (param_idx == (UINT)-1) ? -1 : (int)param_idx;
    int io = (inout_idx == (UINT)-1) ? -1 : (int)inout_idx;
    switch (type) {
    case INPUT_PORT: return new InputPort(type, t, uid, binding, pi, io);
    case OUTPUT_PORT: return new OutputPort(type, t, uid, binding, pi, io);
    case STICKY_PORT: return new StickyPort(type, t, uid, binding, pi, io);
    case META_PORT: return new MetaPort(type, t, uid, binding, pi, io);
    case INITIALIZER_PORT: return new InitializerPort(type, t, uid, binding, pi, io);
    }
    HandleError("%s: unknown port type %d", __FUNCTION__, (int)type);
    return nullptr;
}

// Size and init-data semantics follow the reference (datablock.cpp:350-360, 2665-2700): the block
// is sized by a fixed-dimension template; init data shorter than the block is repeated to fill it,
// longer init data is truncated.  cbInitData is a byte count.
Datablock *AllocateDatablock(DatablockTemplate *t, void *init, UINT cb, Channel *dest, BUFFERACCESSFLAGS flags,
                             CONTROLSIGNAL ctl)
{
    (void)dest;
    (void)flags;
    if (init && cb == 0) {
        printf("AllocateDatablock::non-null init buffer requires non-zero byte count!\n");
        return nullptr;
    }
    if (!init && cb != 0) {
        printf("AllocateDatablock::null init buffer requires zero byte count!\n");
        return nullptr;
    }
    size_t bytes = t ? (size_t)t->GetDatablockByteCount() : (size_t)cb;
    if (t && t->GetParameterBaseType() != PTPARM_BUFFER && t->GetParameterBaseType() != PTPARM_NONE)
        bytes = t->GetStride();
    auto *b = new Datablock(t, bytes, ctl);
    if (init) {
        char *h = (char *)b->GetDataPointer(TRUE, FALSE);
        if (cb >= bytes) {
            HostCopy(h, init, bytes);
        } else {
            for (size_t i = 0; i < bytes; i += cb) memcpy(h + i, init, std::min<size_t>(cb, bytes - i));
        }
    }
    return b;
}

Datablock *AllocateDatablock(DatablockTemplate *t, void *init, UINT cb, BUFFERACCESSFLAGS flags, CONTROLSIGNAL ctl)
{
    return AllocateDatablock(t, init, cb, nullptr, flags, ctl);
}

// A kernel file that names a shared library holds host tasks: "x.so", or the reference's "x.dll",
// which is looked up as x.dll, x.so and libx.so in the same directory.
static bool is_host_library(const std::string &f)
{
    auto ends = [&](const char *e) { return f.size() >= strlen(e) && f.compare(f.size() - strlen(e), strlen(e), e) == 0; };
    return ends(".dll") || ends(".so") || f.find(".so.") != std::string::npos;
}

static void *open_host_library(const std::string &f, std::string &why)
{
    std::vector<std::string> names{f};
    if (f.size() > 4 && f.compare(f.size() - 4, 4, ".dll") == 0) {
        const size_t slash = f.find_last_of('/');
        const std::string dir = slash == std::string::npos ? "" : f.substr(0, slash + 1);
        const std::string stem = f.substr(dir.size(), f.size() - dir.size() - 4);
        names.push_back(dir + stem + ".so");
        names.push_back(dir + "lib" + stem + ".so");
    }
    for (const std::string &n : names) {
        // a bare name would make dlopen search the system paths: look in the current directory
        const std::string path = n.find('/') == std::string::npos ? "./" + n : n;
        if (void *h = dlopen(path.c_str(), RTLD_NOW | RTLD_LOCAL)) return h;
        const char *e = dlerror();
        why = e ? e : "dlopen failed";
    }
    return nullptr;
}

CompiledKernel *GetCompiledKernel(const char *file, const char *op, char *out, int outsz, int, int, int)
{
    std::lock_guard<std::mutex> lk(g_mu);
    std::string key = std::string(file ? file : "") + "|" + (op ? op : "");
    auto it = g_kernels.find(key);
    if (it != g_kernels.end()) return it->second;
    if (file && op && is_host_library(file)) {
        // Host task: the entry point of a shared library (hostaccelerator.cpp:328-380).
        std::string why = "host tasks are disabled (SetUseHost)";
        void *h = g_cfg.use_host ? open_host_library(file, why) : nullptr;
        void *fn = h ? dlsym(h, op) : nullptr;
        if (h && !fn) why = std::string("no entry point ") + op + " in " + file;
        if (!fn) {
            if (out && outsz > 0) snprintf(out, (size_t)outsz, "%s", why.c_str());
            return nullptr;
        }
        auto *k = new CompiledKernel(file, op, reinterpret_cast<LPFNHOSTTASK>(fn));
        g_kernels[key] = k;
        if (out && outsz > 0) out[0] = 0;
        return k;
    }
    int id = -1;
    if (ptk_kernel_lookup(file, op, &id) != PTK_OK) {
        if (out && outsz > 0) snprintf(out, (size_t)outsz, "%s", ptk_last_error());
        return nullptr;
    }
    auto *k = new CompiledKernel(file ? file : "", op, id);
    g_kernels[key] = k;
    if (out && outsz > 0) out[0] = 0;
    return k;
}

BOOL CanExecuteKernel(const char *file)
{
    if (file && is_host_library(file)) return g_cfg.use_host;   // the host accelerator always exists
    return (g_cfg.use_cuda && ptk_can_execute_kernel(file)) ? TRUE : FALSE;
}

void SetUseCUDA(BOOL b) { g_cfg.use_cuda = b; }
BOOL GetUseCUDA() { return g_cfg.use_cuda; }
void SetUseOpenCL(BOOL b) { g_cfg.use_opencl = b; }
BOOL GetUseOpenCL() { return g_cfg.use_opencl; }
void SetUseDirectX(BOOL b) { g_cfg.use_dx = b; }
BOOL GetUseDirectX() { return g_cfg.use_dx; }
void SetUseHost(BOOL b) { g_cfg.use_host = b; }
BOOL GetUseHost() { return g_cfg.use_host; }
void SetVerbose(BOOL b) { g_cfg.verbose = b; }
BOOL GetVerbose() { return g_cfg.verbose; }
void SetDefaultChannelCapacity(int n) { g_cfg.channel_capacity = n; }
int GetDefaultChannelCapacity() { return g_cfg.channel_capacity; }
void SetSchedulingMode(SCHEDULINGMODE m) { g_cfg.sched = m; }
SCHEDULINGMODE GetSchedulingMode() { return g_cfg.sched; }
void SetThreadPoolPolicy(THREADPOOLPOLICY p) { g_cfg.tpp = p; }
THREADPOOLPOLICY GetThreadPoolPolicy() { return g_cfg.tpp; }
void SetMaximumConcurrency(int n) { g_cfg.max_concurrency = n; }
int GetMaximumConcurrency() { return g_cfg.max_concurrency; }
void SetExitOnRuntimeFailure(BOOL b) { g_cfg.exit_on_failure = b; }
BOOL GetExitOnRuntimeFailure() { return g_cfg.exit_on_failure; }
void SetDispatchWatchdogThreshold(DWORD ms) { g_cfg.watchdog_ms = ms; }
DWORD GetDispatchWatchdogThreshold() { return g_cfg.watchdog_ms; }

BOOL HandleError(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vlog(stderr, "PTask runtime error: ", fmt, ap);
    va_end(ap);
    if (g_cfg.exit_on_failure) exit(1);
    return FALSE;
}

BOOL HandleError(const std::string &s) { return HandleError("%s", s.c_str()); }

BOOL MandatoryInform(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stdout, fmt, ap);
    va_end(ap);
    fflush(stdout);
    return TRUE;
}

void Inform(const char *fmt, ...)
{
    if (!g_cfg.verbose) return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stdout, fmt, ap);
    va_end(ap);
}

void Inform(const std::string &s)
{
    if (g_cfg.verbose) fputs(s.c_str(), stdout);
}

void Warning(const char *s, UINT) { fprintf(stderr, "PTask warning: %s\n", s); }
void Warning(const std::string &s, UINT l) { Warning(s.c_str(), l); }
void ErrorMessage(const char *s, UINT) { fprintf(stderr, "PTask error: %s\n", s); }
void ErrorMessage(const std::string &s, UINT l) { ErrorMessage(s.c_str(), l); }

void Trace(const char *fmt, ...)
{
    if (!g_cfg.verbose) return;
    va_list ap;
    va_start(ap, fmt);
    vlog(stderr, "trace: ", fmt, ap);
    va_end(ap);
}

Accelerator *GetAccelerator() { return &g_accel; }

}  // namespace Runtime
}  // namespace PTask
