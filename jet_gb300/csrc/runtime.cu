// Error reporting and device queries of the jetgpu C-ABI.
#include <mutex>
#include <string>
#include <unordered_map>

#include "common.cuh"

namespace jetgpu {

namespace {
thread_local std::string g_last_error;
std::mutex g_sm_mutex;
int g_sm_count[64] = {0};
} // namespace

int SetError(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

void ClearError() { g_last_error.clear(); }

int CheckLaunch(const char *what)
{
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess)
        return SetError(JETGPU_ERR_CUDA,
                        std::string(what) + ": " + cudaGetErrorString(err));
    return JETGPU_OK;
}

int SmCount()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return 152;
    std::lock_guard<std::mutex> lock(g_sm_mutex);
    if (g_sm_count[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                cudaSuccess ||
            n <= 0)
            n = 152;
        g_sm_count[dev] = n;
    }
    return g_sm_count[dev];
}

bool TcAvailable()
{
    int dev = 0, major = 0, minor = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return false;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    // The tensor-core kernels are compiled for sm_103a only.
    return major == 10 && minor == 3;
}

} // namespace jetgpu

extern "C" {

const char *jetgpu_last_error(void) { return jetgpu::g_last_error.c_str(); }

int jetgpu_version(void) { return JETGPU_ABI_VERSION; }

int jetgpu_get_device(int *device)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(device != nullptr, "null device pointer");
    JETGPU_CUDA_TRY(cudaGetDevice(device));
    return JETGPU_OK;
}

int jetgpu_set_device(int device)
{
    jetgpu::ClearError();
    int count = 0;
    JETGPU_CUDA_TRY(cudaGetDeviceCount(&count));
    JETGPU_REQUIRE(device >= 0 && device < count && device < 64, "device out of range");
    JETGPU_CUDA_TRY(cudaSetDevice(device));
    return JETGPU_OK;
}

int jetgpu_device_info(int *sm_count, int *cc_major, int *cc_minor)
{
    jetgpu::ClearError();
    int dev = 0;
    JETGPU_CUDA_TRY(cudaGetDevice(&dev));
    if (sm_count)
        JETGPU_CUDA_TRY(cudaDeviceGetAttribute(
            sm_count, cudaDevAttrMultiProcessorCount, dev));
    if (cc_major)
        JETGPU_CUDA_TRY(cudaDeviceGetAttribute(
            cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    if (cc_minor)
        JETGPU_CUDA_TRY(cudaDeviceGetAttribute(
            cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    return JETGPU_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Memory, streams and graphs.
// Device memory comes from the device's stream-ordered memory pool
// (cudaMallocAsync on the library stream) with its release threshold raised so
// freed blocks stay cached for reuse instead of returning to the driver.
// ---------------------------------------------------------------------------
namespace jetgpu {
// jetgpu_malloc accounting for jetgpu_set_pool_limit.
std::mutex g_pool_mutex;
size_t g_pool_limit = 0;
size_t g_pool_in_use = 0;
std::unordered_map<void *, size_t> g_pool_sizes;

namespace {
std::mutex g_stream_mutex;
cudaStream_t g_streams[64] = {nullptr};
bool g_pool_configured[64] = {false};

int CurrentDevice()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return 0;
    return dev;
}
} // namespace

cudaStream_t LibraryStream()
{
    const int dev = CurrentDevice();
    std::lock_guard<std::mutex> lock(g_stream_mutex);
    if (g_streams[dev] == nullptr) {
        cudaStream_t s = nullptr;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
            return nullptr;
        g_streams[dev] = s;
    }
    if (!g_pool_configured[dev]) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t threshold = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        }
        g_pool_configured[dev] = true;
    }
    return g_streams[dev];
}

} // namespace jetgpu

extern "C" {

void *jetgpu_default_stream(void) { return (void *)jetgpu::LibraryStream(); }

int jetgpu_malloc(size_t bytes, void **ptr)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(ptr != nullptr, "null output pointer");
    *ptr = nullptr;
    if (bytes == 0)
        return JETGPU_OK;
    const size_t rounded = (bytes + 255) / 256 * 256;
    {
        std::lock_guard<std::mutex> lock(jetgpu::g_pool_mutex);
        if (jetgpu::g_pool_limit != 0 && jetgpu::g_pool_in_use + rounded > jetgpu::g_pool_limit)
            return jetgpu::SetError(JETGPU_ERR_MEMORY,
                                    "device memory limit of " +
                                        std::to_string(jetgpu::g_pool_limit) + " bytes reached (" +
                                        std::to_string(jetgpu::g_pool_in_use) + " in use, " +
                                        std::to_string(rounded) + " requested)");
    }
    cudaStream_t s = jetgpu::LibraryStream();
    JETGPU_CUDA_TRY(cudaMallocAsync(ptr, rounded, s));
    std::lock_guard<std::mutex> lock(jetgpu::g_pool_mutex);
    jetgpu::g_pool_sizes[*ptr] = rounded;
    jetgpu::g_pool_in_use += rounded;
    return JETGPU_OK;
}

int jetgpu_free(void *ptr)
{
    jetgpu::ClearError();
    if (ptr == nullptr)
        return JETGPU_OK;
    JETGPU_CUDA_TRY(cudaFreeAsync(ptr, jetgpu::LibraryStream()));
    std::lock_guard<std::mutex> lock(jetgpu::g_pool_mutex);
    auto it = jetgpu::g_pool_sizes.find(ptr);
    if (it != jetgpu::g_pool_sizes.end()) {
        jetgpu::g_pool_in_use -= it->second;
        jetgpu::g_pool_sizes.erase(it);
    }
    return JETGPU_OK;
}

int jetgpu_set_pool_limit(size_t bytes)
{
    jetgpu::ClearError();
    std::lock_guard<std::mutex> lock(jetgpu::g_pool_mutex);
    jetgpu::g_pool_limit = bytes;
    return JETGPU_OK;
}

size_t jetgpu_pool_bytes_in_use(void)
{
    std::lock_guard<std::mutex> lock(jetgpu::g_pool_mutex);
    return jetgpu::g_pool_in_use;
}

void jetgpu_range_push(const char *name) { nvtxRangePushA(name ? name : "jetgpu"); }

void jetgpu_range_pop(void) { nvtxRangePop(); }

int jetgpu_release_cached(void)
{
    jetgpu::ClearError();
    cudaMemPool_t pool;
    JETGPU_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, jetgpu::CurrentDevice()));
    JETGPU_CUDA_TRY(cudaStreamSynchronize(jetgpu::LibraryStream()));
    JETGPU_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
    return JETGPU_OK;
}

int jetgpu_memory_stats(size_t *in_use, size_t *cached, size_t *peak_in_use)
{
    jetgpu::ClearError();
    cudaMemPool_t pool;
    JETGPU_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, jetgpu::CurrentDevice()));
    uint64_t used = 0, reserved = 0, high = 0;
    JETGPU_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
    JETGPU_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved));
    JETGPU_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high));
    if (in_use)
        *in_use = used;
    if (cached)
        *cached = reserved > used ? reserved - used : 0;
    if (peak_in_use)
        *peak_in_use = high;
    return JETGPU_OK;
}

int jetgpu_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream)
{
    jetgpu::ClearError();
    if (bytes == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(dst != nullptr && src != nullptr, "null pointer");
    cudaMemcpyKind k = kind == 0   ? cudaMemcpyHostToDevice
                       : kind == 1 ? cudaMemcpyDeviceToHost
                       : kind == 2 ? cudaMemcpyDeviceToDevice
                                   : cudaMemcpyDefault;
    JETGPU_REQUIRE(kind >= 0 && kind <= 2, "bad copy kind");
    JETGPU_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, k, jetgpu::AsStream(stream)));
    return JETGPU_OK;
}

int jetgpu_memset_zero(void *dst, size_t bytes, void *stream)
{
    jetgpu::ClearError();
    if (bytes == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(dst != nullptr, "null pointer");
    JETGPU_CUDA_TRY(cudaMemsetAsync(dst, 0, bytes, jetgpu::AsStream(stream)));
    return JETGPU_OK;
}

int jetgpu_stream_synchronize(void *stream)
{
    jetgpu::ClearError();
    JETGPU_CUDA_TRY(cudaStreamSynchronize(jetgpu::AsStream(stream)));
    return JETGPU_OK;
}

int jetgpu_graph_begin(void *stream)
{
    jetgpu::ClearError();
    JETGPU_CUDA_TRY(cudaStreamBeginCapture(jetgpu::AsStream(stream),
                                           cudaStreamCaptureModeThreadLocal));
    return JETGPU_OK;
}

int jetgpu_graph_end(void *stream, void **graph_exec)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(graph_exec != nullptr, "null output pointer");
    cudaGraph_t graph = nullptr;
    JETGPU_CUDA_TRY(cudaStreamEndCapture(jetgpu::AsStream(stream), &graph));
    cudaGraphExec_t exec = nullptr;
    cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess)
        return jetgpu::SetError(JETGPU_ERR_CUDA, std::string("cudaGraphInstantiate: ") +
                                                     cudaGetErrorString(err));
    *graph_exec = (void *)exec;
    return JETGPU_OK;
}

int jetgpu_graph_launch(void *graph_exec, void *stream)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(graph_exec != nullptr, "null graph");
    JETGPU_CUDA_TRY(cudaGraphLaunch((cudaGraphExec_t)graph_exec, jetgpu::AsStream(stream)));
    return JETGPU_OK;
}

int jetgpu_graph_destroy(void *graph_exec)
{
    jetgpu::ClearError();
    if (graph_exec)
        JETGPU_CUDA_TRY(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec));
    return JETGPU_OK;
}

int jetgpu_event_create(void **event)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(event != nullptr, "null output pointer");
    cudaEvent_t e = nullptr;
    JETGPU_CUDA_TRY(cudaEventCreate(&e));
    *event = (void *)e;
    return JETGPU_OK;
}

int jetgpu_event_record(void *event, void *stream)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(event != nullptr, "null event");
    JETGPU_CUDA_TRY(cudaEventRecord((cudaEvent_t)event, jetgpu::AsStream(stream)));
    return JETGPU_OK;
}

int jetgpu_event_elapsed_ms(void *start, void *end, float *ms)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(start != nullptr && end != nullptr && ms != nullptr, "null pointer");
    JETGPU_CUDA_TRY(cudaEventSynchronize((cudaEvent_t)end));
    JETGPU_CUDA_TRY(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)end));
    return JETGPU_OK;
}

int jetgpu_event_destroy(void *event)
{
    jetgpu::ClearError();
    if (event)
        JETGPU_CUDA_TRY(cudaEventDestroy((cudaEvent_t)event));
    return JETGPU_OK;
}

} // extern "C"
