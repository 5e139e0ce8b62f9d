// Grouped launch of small contractions: several independent (batched)
// products C[b] = A[b] B[b] in one kernel.
//
// The reference runs every path step as its own ContractTensors call
// (Tensor.hpp:708-752: two transposes, then one BLAS call). For the many small
// slice-dependent steps of a sliced network that is one to three launches per
// step, each too small to fill the GPU. Here a run of such steps that do not
// read each other's outputs goes into one launch.
// Each operand is read through offset tables instead of a transpose pass:
// element (b, i, j) of the product's view of A is A[a_bat[b] + a_row[i] +
// a_col[j]], so any permutation of the operand's axes and any placement of
// the batch axes is absorbed into the load. C is written packed, batch x m x
// n, row-major, as jetgpu_contract_batched writes it.
//
// CTA tiles are 32 x 32 outputs of one (task, batch item); 256 threads, each
// accumulating 2 x 2 complex outputs in the element type (FP32 or FP64 FMA,
// the plain form's arithmetic) over k slices of 32 staged in shared memory.
#include "common.cuh"

namespace jetgpu {
namespace {

constexpr int kGT = 32;       // output tile edge
constexpr int kGK = 32;       // k slice
constexpr int kMaxTasks = 256; // tasks per launch
constexpr int kGThreads = 256; // threads per CTA: one per task in the tile prefix scan
static_assert(kGThreads == kMaxTasks, "the prefix scan reads one task per thread");

template <typename T> struct V2;
template <> struct V2<float> {
    using type = float2;
};
template <> struct V2<double> {
    using type = double2;
};

template <typename T>
__global__ void __launch_bounds__(kGThreads)
    group_contract_kernel(const jetgpu_group_task *__restrict__ tasks, int n_tasks,
                          uint64_t total_tiles)
{
    using V = typename V2<T>::type;
    __shared__ uint64_t first_tile[kMaxTasks + 1];
    __shared__ V As[kGK][kGT + 1];
    __shared__ V Bs[kGK][kGT + 1];
    // First tile of every task: thread t reads task t's tile count, then a
    // block-wide inclusive scan (kMaxTasks = blockDim.x = 256: 8 rounds).
    // One thread walking the tasks took 0.13 us a task, 30 us for 184.
    {
        const int tid = threadIdx.x;
        uint64_t mine = 0;
        if (tid < n_tasks) {
            const jetgpu_group_task &q = tasks[tid];
            mine = q.batch * ((q.m + kGT - 1) / kGT) * ((q.n + kGT - 1) / kGT);
        }
        first_tile[tid + 1] = mine;
        if (tid == 0)
            first_tile[0] = 0;
        __syncthreads();
        for (int off = 1; off < kMaxTasks; off <<= 1) {
            const uint64_t add = tid >= off ? first_tile[tid + 1 - off] : 0;
            __syncthreads();
            first_tile[tid + 1] += add;
            __syncthreads();
        }
    }
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16; // 2 x 2 outputs each
    int t = 0; // this CTA's tiles come in increasing order: the task only advances
    for (uint64_t g = blockIdx.x; g < total_tiles; g += gridDim.x) {
        while (t + 1 < n_tasks && first_tile[t + 1] <= g)
            ++t;
        const jetgpu_group_task &q = tasks[t];
        const uint64_t local = g - first_tile[t];
        const uint64_t tiles_n = (q.n + kGT - 1) / kGT;
        const uint64_t tiles_mn = ((q.m + kGT - 1) / kGT) * tiles_n;
        const uint64_t b = local / tiles_mn;
        const uint64_t r = local - b * tiles_mn;
        const uint64_t m0 = (r / tiles_n) * kGT, n0 = (r % tiles_n) * kGT;
        const V *A = static_cast<const V *>(q.A) + q.a_bat[b];
        const V *B = static_cast<const V *>(q.B) + q.b_bat[b];
        V acc[2][2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j)
                acc[i][j] = V{0, 0};
        for (uint64_t k0 = 0; k0 < q.k; k0 += kGK) {
            // 32 x 32 of A (rows m0.., k k0..) and of B (k k0.., cols n0..):
            // 4 elements of each per thread, consecutive threads along k for A
            // and along n for B.
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int idx = threadIdx.x + 256 * e;
                const int rr = idx / kGK, cc = idx % kGK;
                const uint64_t gi = m0 + rr, gk = k0 + cc;
                As[cc][rr] = (gi < q.m && gk < q.k) ? A[q.a_row[gi] + q.a_col[gk]] : V{0, 0};
                const uint64_t gk2 = k0 + rr, gj = n0 + cc;
                Bs[rr][cc] = (gk2 < q.k && gj < q.n) ? B[q.b_row[gk2] + q.b_col[gj]] : V{0, 0};
            }
            __syncthreads();
#pragma unroll 8
            for (int kk = 0; kk < kGK; ++kk) {
                const V a0 = As[kk][ty], a1 = As[kk][ty + 16];
                const V b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
                const V av[2] = {a0, a1}, bv[2] = {b0, b1};
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        acc[i][j].x = fma(av[i].x, bv[j].x, acc[i][j].x);
                        acc[i][j].x = fma(-av[i].y, bv[j].y, acc[i][j].x);
                        acc[i][j].y = fma(av[i].x, bv[j].y, acc[i][j].y);
                        acc[i][j].y = fma(av[i].y, bv[j].x, acc[i][j].y);
                    }
            }
            __syncthreads();
        }
        V *C = static_cast<V *>(q.C) + b * q.m * q.n;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const uint64_t gi = m0 + ty + 16 * i, gj = n0 + tx + 16 * j;
                if (gi < q.m && gj < q.n)
                    C[gi * q.n + gj] = acc[i][j];
            }
    }
}

} // namespace
} // namespace jetgpu

using namespace jetgpu;

extern "C" {

uint64_t jetgpu_group_tiles(uint64_t batch, uint64_t m, uint64_t n)
{
    return batch * ((m + kGT - 1) / kGT) * ((n + kGT - 1) / kGT);
}

int jetgpu_contract_group(const jetgpu_group_task *tasks, int n_tasks, uint64_t total_tiles,
                          int dtype, void *stream)
{
    NvtxRange range("jetgpu_contract_group");
    ClearError();
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    JETGPU_REQUIRE(n_tasks >= 0 && n_tasks <= kMaxTasks, "at most 256 tasks per group");
    if (n_tasks == 0 || total_tiles == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(tasks != nullptr, "null task table");
    const unsigned grid = GridFor(total_tiles, 8);
    cudaStream_t st = AsStream(stream);
    if (dtype == JETGPU_C64)
        group_contract_kernel<float><<<grid, kGThreads, 0, st>>>(tasks, n_tasks, total_tiles);
    else
        group_contract_kernel<double><<<grid, kGThreads, 0, st>>>(tasks, n_tasks, total_tiles);
    return CheckLaunch("group_contract_kernel");
}

} // extern "C"
