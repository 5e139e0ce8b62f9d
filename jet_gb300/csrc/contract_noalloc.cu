// Allocation-free variant of jetgpu_contract.
//
// Some callers of this library cannot allocate device memory at the moment
// they contract: code that runs while a stream is being captured into a CUDA
// graph (cudaMalloc is not a legal call during capture and breaks it), hosts
// that hand the GPU to this library under a fixed memory budget owned by their
// own allocator (JNI/cgo services, embedded runtimes) and latency-sensitive
// loops where a cudaMalloc or cudaFree would synchronise the device. For them,
// jetgpu_contract_noalloc takes its scratch from one file-scope device array
// of kScratchBytes instead of a caller-provided workspace.
//
// The array belongs to the module: every GPU that loads the library holds it
// until the process exits. Host code must not hand the array's symbol to a
// kernel (on the host it is only a stand-in, not a device address); the
// device address is looked up once per device with cudaGetSymbolAddress and
// cached.
#include <mutex>
#include <string>

#include "common.cuh"

namespace jetgpu {
namespace {

constexpr size_t kScratchBytes = size_t(32) << 20; // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_contract_scratch[kScratchBytes];

std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_contract_scratch on the current device, looked up on
// first use with that device current.
int ScratchAddress(void **out)
{
    int dev = 0;
    JETGPU_CUDA_TRY(cudaGetDevice(&dev));
    JETGPU_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_contract_scratch);
        if (err != cudaSuccess || p == nullptr)
            return SetError(JETGPU_ERR_CUDA,
                            std::string("cudaGetSymbolAddress(scratch): ") +
                                cudaGetErrorString(err));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return JETGPU_OK;
}

} // namespace
} // namespace jetgpu

extern "C" {

size_t jetgpu_contract_noalloc_max_scratch(void) { return jetgpu::kScratchBytes; }

int jetgpu_contract_noalloc(const void *A, int a_rank, const uint64_t *a_shape,
                            const int32_t *a_perm, const void *B, int b_rank,
                            const uint64_t *b_shape, const int32_t *b_perm, void *C,
                            uint64_t m, uint64_t n, uint64_t k, int dtype, int precision,
                            int algo, int scale_a, int scale_b, void *stream)
{
    jetgpu::ClearError();
    const size_t need = jetgpu_contract_workspace_size(a_rank, a_shape, a_perm, b_rank, b_shape,
                                                       b_perm, m, n, k, dtype, precision);
    if (need > jetgpu::kScratchBytes)
        return jetgpu::SetError(
            JETGPU_ERR_WORKSPACE,
            "jetgpu_contract_noalloc: this contraction needs " + std::to_string(need) +
                " bytes of scratch, more than the " + std::to_string(jetgpu::kScratchBytes) +
                " bytes the allocation-free entry point holds; use jetgpu_contract with a "
                "caller-provided workspace");
    void *scratch = nullptr;
    if (need > 0) {
        const int rc = jetgpu::ScratchAddress(&scratch);
        if (rc != JETGPU_OK)
            return rc;
    }
    // Every scratch byte the contraction reads is written earlier in the same
    // call (split planes, transposed operands, partial sums), so nothing has
    // to be cleared between calls.
    return jetgpu_contract(A, a_rank, a_shape, a_perm, B, b_rank, b_shape, b_perm, C, m, n, k,
                           dtype, precision, algo, scale_a, scale_b, scratch,
                           need > 0 ? jetgpu::kScratchBytes : 0, stream);
}

} // extern "C"
