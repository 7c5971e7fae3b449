// runtime_core.cu -- device selection, error reporting, stream-ordered memory pool, streams and
// events behind the C ABI.  Replaces the CUDA accelerator / buffer / async-context layer of the
// reference (ptask/cuaccelerator.cpp, ptask/PCUBuffer.cpp, ptask/CUAsyncContext.cpp) and its block
// pools (ptask/BlockPool.cpp): one device, one default non-blocking stream, cudaMallocAsync pool.
#include "ptk_internal.h"

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>

namespace ptk {

static thread_local std::string t_error;
static std::mutex g_init_mu;
static bool g_inited = false;
static int g_device = 0;
static int g_sms = 0;
static cudaStream_t g_stream = nullptr;
static cudaMemPool_t g_pool = nullptr;
static std::atomic<long long> g_launches{0};
static std::atomic<long long> g_trims{0};   // pool trims after a failed allocation

int set_error(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_error = buf;
    return code;
}

void clear_error() { t_error.clear(); }

static thread_local int t_capturing = 0;

void set_capturing(bool on) { t_capturing += on ? 1 : -1; }

void count_launches(long long n)
{
    // Launches recorded into a CUDA graph are counted when the graph is replayed.
    if (t_capturing) return;
    g_launches.fetch_add(n, std::memory_order_relaxed);
}

void count_graph_launch(long long nodes) { g_launches.fetch_add(nodes, std::memory_order_relaxed); }

long long launches_issued() { return g_launches.load(std::memory_order_relaxed); }

static int init_locked(int device)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return set_error(PTK_ERR_CUDA, "no CUDA device available (%s)",
                         e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0");
    if (device < 0 || device >= n)
        return set_error(PTK_ERR_INVALID, "device %d out of range (have %d)", device, n);
    PTK_CUDA_TRY(cudaSetDevice(device));
    PTK_CUDA_TRY(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, device));
    PTK_CUDA_TRY(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
    PTK_CUDA_TRY(cudaDeviceGetDefaultMemPool(&g_pool, device));
    uint64_t keep = UINT64_MAX;   // keep freed blocks cached in the pool (no trim between steps)
    PTK_CUDA_TRY(cudaMemPoolSetAttribute(g_pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_device = device;
    g_inited = true;
    return PTK_OK;
}

int ensure_init()
{
    if (g_inited) {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != g_device) cudaSetDevice(g_device);
        return PTK_OK;
    }
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_inited) return PTK_OK;
    return init_locked(0);
}

cudaStream_t default_stream() { return g_stream; }
int sm_count() { return g_sms; }

int pool_alloc(size_t bytes, cudaStream_t s, void **p)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (bytes == 0) bytes = 16;
    cudaStream_t st = s ? s : g_stream;
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, g_pool, st);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (e == cudaErrorMemoryAllocation && cudaStreamIsCapturing(st, &cs) == cudaSuccess &&
        cs == cudaStreamCaptureStatusNone) {
        // Freed blocks stay cached in the pool (no trim between steps).  When the cached blocks of
        // many different sizes leave none that fits, let the frees queued so far run, give the
        // unused cache back to the driver and try once more.
        cudaGetLastError();
        cudaDeviceSynchronize();
        cudaMemPoolTrimTo(g_pool, 0);
        g_trims.fetch_add(1, std::memory_order_relaxed);
        e = cudaMallocFromPoolAsync(p, bytes, g_pool, st);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(PTK_ERR_NOMEM, "device allocation of %zu bytes failed: %s", bytes,
                         cudaGetErrorString(e));
    }
    return PTK_OK;
}

int pool_free(void *p, cudaStream_t s)
{
    if (!p) return PTK_OK;
    PTK_CUDA_TRY(cudaFreeAsync(p, s ? s : g_stream));
    return PTK_OK;
}

Layout make_layout(int nx, int ny, int nz)
{
    Layout L;
    L.nx = nx; L.ny = ny; L.nz = nz;
    L.pitch = ((nx + 1) + 31) / 32 * 32;
    L.plane = (long long)L.pitch * (ny + 1);
    L.total = L.plane * (nz + 1);
    return L;
}

}  // namespace ptk

using namespace ptk;

static inline cudaStream_t S(void *s) { return s ? (cudaStream_t)s : default_stream(); }

extern "C" {

const char *ptk_last_error(void) { return t_error.c_str(); }

int ptk_runtime_init(int device)
{
    clear_error();
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_inited) {
        if (device != g_device)
            return set_error(PTK_ERR_STATE, "runtime already initialised on device %d", g_device);
        return PTK_OK;
    }
    return init_locked(device);
}

int ptk_runtime_shutdown(void)
{
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (!g_inited) return PTK_OK;
    cudaStreamSynchronize(g_stream);
    cudaDeviceSynchronize();
    if (g_pool) cudaMemPoolTrimTo(g_pool, 0);
    return PTK_OK;   // the stream and pool live until process exit (other threads may hold them)
}

int ptk_device_info(char *name, int name_len, int *sms, size_t *total, size_t *free_b)
{
    int rc = ensure_init();
    if (rc) return rc;
    cudaDeviceProp prop;
    PTK_CUDA_TRY(cudaGetDeviceProperties(&prop, g_device));
    if (name && name_len > 0) {
        strncpy(name, prop.name, (size_t)name_len - 1);
        name[name_len - 1] = 0;
    }
    if (sms) *sms = prop.multiProcessorCount;
    size_t f = 0, t = 0;
    PTK_CUDA_TRY(cudaMemGetInfo(&f, &t));
    if (total) *total = t;
    if (free_b) *free_b = f;
    return PTK_OK;
}

int ptk_mem_alloc(size_t bytes, void *stream, void **dptr)
{
    PTK_CHECK_ARG(dptr, "dptr is NULL");
    return pool_alloc(bytes, S(stream), dptr);
}

int ptk_mem_free(void *dptr, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return pool_free(dptr, S(stream));
}

// Pinned host memory: the driver page-locks every allocation, milliseconds for the tens of
// megabytes of one field, and a graph pushes and pulls fresh datablocks every solve.  Freed buffers
// are therefore kept by exact size and handed out again (the host half of the reference's block
// pools, ptask/BlockPool.cpp); at most kHostCacheBytes are held, the rest is returned to the driver.
// Callers free a buffer only after their copies from or into it have completed.
namespace {
constexpr size_t kHostCacheBytes = (size_t)4 << 30;
std::mutex g_host_mu;
std::multimap<size_t, void *> g_host_cache;      // free buffers by size
std::unordered_map<void *, size_t> g_host_size;  // every buffer handed out or cached
size_t g_host_cached = 0;
}  // namespace

int ptk_host_alloc(size_t bytes, void **hptr)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CHECK_ARG(hptr, "hptr is NULL");
    if (!bytes) bytes = 16;
    {
        std::lock_guard<std::mutex> lk(g_host_mu);
        auto it = g_host_cache.find(bytes);
        if (it != g_host_cache.end()) {
            *hptr = it->second;
            g_host_cache.erase(it);
            g_host_cached -= bytes;
            return PTK_OK;
        }
    }
    PTK_CUDA_TRY(cudaMallocHost(hptr, bytes));
    std::lock_guard<std::mutex> lk(g_host_mu);
    g_host_size[*hptr] = bytes;
    return PTK_OK;
}

int ptk_host_free(void *hptr)
{
    if (!hptr) return PTK_OK;
    {
        std::lock_guard<std::mutex> lk(g_host_mu);
        auto it = g_host_size.find(hptr);
        if (it != g_host_size.end()) {
            const size_t b = it->second;
            if (g_host_cached + b <= kHostCacheBytes) {
                g_host_cache.emplace(b, hptr);
                g_host_cached += b;
                return PTK_OK;
            }
            g_host_size.erase(it);
        }
    }
    PTK_CUDA_TRY(cudaFreeHost(hptr));
    return PTK_OK;
}

int ptk_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, S(stream)));
    return PTK_OK;
}

int ptk_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, S(stream)));
    return PTK_OK;
}

int ptk_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, S(stream)));
    return PTK_OK;
}

int ptk_memset(void *dst, int value, size_t bytes, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CUDA_TRY(cudaMemsetAsync(dst, value, bytes, S(stream)));
    return PTK_OK;
}

int ptk_stream_create(void **stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    cudaStream_t s;
    PTK_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = s;
    return PTK_OK;
}

int ptk_stream_destroy(void *stream)
{
    if (!stream) return PTK_OK;
    PTK_CUDA_TRY(cudaStreamDestroy((cudaStream_t)stream));
    return PTK_OK;
}

int ptk_stream_sync(void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CUDA_TRY(cudaStreamSynchronize(S(stream)));
    return PTK_OK;
}

int ptk_device_sync(void)
{
    int rc = ensure_init();
    if (rc) return rc;
    PTK_CUDA_TRY(cudaDeviceSynchronize());
    return PTK_OK;
}

int ptk_device_ordinal(int *device)
{
    if (!device) return set_error(PTK_ERR_INVALID, "NULL argument");
    int rc = ensure_init();
    if (rc) return rc;
    *device = g_device;
    return PTK_OK;
}

int ptk_event_create(void **event)
{
    int rc = ensure_init();
    if (rc) return rc;
    cudaEvent_t e;
    PTK_CUDA_TRY(cudaEventCreate(&e));
    *event = e;
    return PTK_OK;
}

int ptk_event_destroy(void *event)
{
    if (!event) return PTK_OK;
    PTK_CUDA_TRY(cudaEventDestroy((cudaEvent_t)event));
    return PTK_OK;
}

int ptk_event_record(void *event, void *stream)
{
    PTK_CUDA_TRY(cudaEventRecord((cudaEvent_t)event, S(stream)));
    return PTK_OK;
}

int ptk_event_sync(void *event)
{
    PTK_CUDA_TRY(cudaEventSynchronize((cudaEvent_t)event));
    return PTK_OK;
}

int ptk_event_query(void *event)
{
    cudaError_t e = cudaEventQuery((cudaEvent_t)event);
    if (e == cudaSuccess) return PTK_OK;
    if (e == cudaErrorNotReady) {
        cudaGetLastError();
        return PTK_ERR_STATE;
    }
    return set_error(PTK_ERR_CUDA, "cudaEventQuery: %s", cudaGetErrorString(e));
}

int ptk_stream_wait_event(void *stream, void *event)
{
    PTK_CUDA_TRY(cudaStreamWaitEvent(S(stream), (cudaEvent_t)event, 0));
    return PTK_OK;
}

int ptk_event_elapsed_ms(void *start, void *stop, float *ms)
{
    PTK_CUDA_TRY(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop));
    return PTK_OK;
}

int ptk_pool_stats(size_t *reserved, size_t *used)
{
    int rc = ensure_init();
    if (rc) return rc;
    uint64_t r = 0, u = 0;
    PTK_CUDA_TRY(cudaMemPoolGetAttribute(g_pool, cudaMemPoolAttrReservedMemCurrent, &r));
    PTK_CUDA_TRY(cudaMemPoolGetAttribute(g_pool, cudaMemPoolAttrUsedMemCurrent, &u));
    if (reserved) *reserved = (size_t)r;
    if (used) *used = (size_t)u;
    return PTK_OK;
}

long long ptk_launch_count(void) { return launches_issued(); }

long long ptk_pool_trim_count(void) { return ptk::g_trims.load(std::memory_order_relaxed); }

}  // extern "C"
