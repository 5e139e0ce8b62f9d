// Error reporting and device queries of the jetgpu C-ABI.
#include <mutex>
#include <string>

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
