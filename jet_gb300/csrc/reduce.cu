// Element-wise and reduction kernels: AddTensors, Conj, the FP64 cross-slice
// sum, device SliceIndex and the max-exponent query.
#include <vector>

#include "common.cuh"

namespace jetgpu {
namespace {

constexpr int kThreads = 256;

template <typename V>
__global__ void add_kernel(const V *__restrict__ a, const V *__restrict__ b,
                           V *__restrict__ c, uint64_t n)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        V x = a[i], y = b[i];
        c[i] = V{x.x + y.x, x.y + y.y};
    }
}

template <typename V>
__global__ void conj_kernel(const V *__restrict__ a, V *__restrict__ c, uint64_t n)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        V x = a[i];
        c[i] = V{x.x, -x.y};
    }
}

// size >= kThreads: one thread per element, slices summed in order.
template <typename V>
__global__ void slice_sum_wide(const V *__restrict__ r, double2 *__restrict__ out,
                               uint64_t n_slices, uint64_t size, int accumulate)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size;
         i += (uint64_t)gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        if (accumulate) {
            re = out[i].x;
            im = out[i].y;
        }
        for (uint64_t s = 0; s < n_slices; ++s) {
            V v = r[s * size + i];
            re += (double)v.x;
            im += (double)v.y;
        }
        out[i] = make_double2(re, im);
    }
}

// Small outputs (amplitudes): one CTA per element; threads stride over the
// slices, then a fixed-shape tree reduction (deterministic).
template <typename V>
__global__ void slice_sum_narrow(const V *__restrict__ r, double2 *__restrict__ out,
                                 uint64_t n_slices, uint64_t size, int accumulate)
{
    __shared__ double sre[kThreads], sim[kThreads];
    for (uint64_t i = blockIdx.x; i < size; i += gridDim.x) {
        double re = 0, im = 0;
        for (uint64_t s = threadIdx.x; s < n_slices; s += blockDim.x) {
            V v = r[s * size + i];
            re += (double)v.x;
            im += (double)v.y;
        }
        sre[threadIdx.x] = re;
        sim[threadIdx.x] = im;
        __syncthreads();
        for (int w = kThreads / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) {
                sre[threadIdx.x] += sre[threadIdx.x + w];
                sim[threadIdx.x] += sim[threadIdx.x + w];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            double2 prev = accumulate ? out[i] : make_double2(0, 0);
            out[i] = make_double2(prev.x + sre[0], prev.y + sim[0]);
        }
        __syncthreads();
    }
}

constexpr int kMaxRank = 64;

struct SliceParams {
    int free_rank;
    uint64_t free_dims[kMaxRank];
    uint64_t free_strides[kMaxRank];
    int n_axes;
    uint64_t fixed_stride[kMaxRank];  // input stride of each sliced axis
    uint64_t fixed_dim[kMaxRank];     // its dimension
    uint64_t value_stride[kMaxRank];  // divisor of the global slice value
    uint64_t out_size;
    uint64_t first_value;
    uint64_t total;                   // n_values * out_size
};

template <typename E>
__global__ void slice_gather_kernel(const __grid_constant__ SliceParams p,
                                    const E *__restrict__ in, E *__restrict__ out,
                                    const uint64_t *__restrict__ first_dev)
{
    // The first slice value comes from the parameters or, for launches that a
    // captured graph replays over successive chunks, from device memory.
    const uint64_t first = first_dev ? *first_dev : p.first_value;
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
         idx < p.total; idx += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = idx / p.out_size;
        uint64_t o = idx - s * p.out_size;
        const uint64_t v = first + s;
        uint64_t src = 0;
        for (int j = 0; j < p.n_axes; ++j)
            src += ((v / p.value_stride[j]) % p.fixed_dim[j]) * p.fixed_stride[j];
        for (int j = p.free_rank - 1; j >= 0; --j) {
            const uint64_t d = p.free_dims[j];
            const uint64_t q = o / d;
            src += (o - q * d) * p.free_strides[j];
            o = q;
        }
        out[idx] = in[src];
    }
}

// Adjoint of slice_gather_kernel for one slice value: full[src] += sliced[o]
// at the same positions. Within one value every o has its own src, so the
// read-modify-write needs no atomics and the result is deterministic.
template <typename E, typename R>
__global__ void slice_scatter_add_kernel(const __grid_constant__ SliceParams p,
                                         const E *__restrict__ sliced, E *__restrict__ full)
{
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < p.total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = p.first_value;
        uint64_t o = idx;
        uint64_t dst = 0;
        for (int j = 0; j < p.n_axes; ++j)
            dst += ((v / p.value_stride[j]) % p.fixed_dim[j]) * p.fixed_stride[j];
        for (int j = p.free_rank - 1; j >= 0; --j) {
            const uint64_t d = p.free_dims[j];
            const uint64_t q = o / d;
            dst += (o - q * d) * p.free_strides[j];
            o = q;
        }
        const E g = sliced[idx];
        E f = full[dst];
        f.x = (R)(f.x + g.x);
        f.y = (R)(f.y + g.y);
        full[dst] = f;
    }
}

__global__ void init_exp_kernel(int *e) { *e = kExpZero; }

__global__ void counter_add_kernel(uint64_t *c, uint64_t delta) { *c += delta; }

// Max exponent of operand blockIdx.y (x0 or x1) into e[blockIdx.y]; e must
// start below -1000 (the 0x80 byte fill), so all-zero operands give -1000.
// An operand whose hint (h0 / h1, may be null) already holds its exponent
// (>= -1000: recorded by the kernel that produced it) is not read: its hint
// is copied.
template <typename V, typename U>
__global__ void max_exp_kernel(const V *__restrict__ x0, uint64_t n0, const V *__restrict__ x1,
                               uint64_t n1, int *e, const int *h0, const int *h1)
{
    const V *__restrict__ x = blockIdx.y ? x1 : x0;
    const uint64_t n = blockIdx.y ? n1 : n0;
    const int *h = blockIdx.y ? h1 : h0;
    e += blockIdx.y;
    if (h != nullptr) {
        const int known = *h;
        if (known >= kExpZero) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                atomicMax(e, known);
            return;
        }
    }
    U best = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        V v = x[i];
        U a, b;
        if constexpr (sizeof(U) == 4) {
            a = (U)(__float_as_uint((float)v.x) & 0x7fffffffu);
            b = (U)(__float_as_uint((float)v.y) & 0x7fffffffu);
        }
        else {
            a = (U)((unsigned long long)__double_as_longlong((double)v.x) &
                    0x7fffffffffffffffull);
            b = (U)((unsigned long long)__double_as_longlong((double)v.y) &
                    0x7fffffffffffffffull);
        }
        best = max(best, max(a, b));
    }
    // Exponent of the largest magnitude (finite values; bit patterns of
    // non-negative floats order like the values).
    int ex;
    if (best == 0) {
        ex = kExpZero;
    }
    else if constexpr (sizeof(U) == 4) {
        const int biased = (int)((best >> 23) & 0xff);
        ex = biased == 0 ? -127 : biased - 127;
    }
    else {
        const int biased = (int)((best >> 52) & 0x7ff);
        ex = biased == 0 ? -1023 : biased - 1023;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(e, ex);
}

} // namespace
} // namespace jetgpu

using namespace jetgpu;

extern "C" {

int jetgpu_add(const void *A, const void *B, void *C, uint64_t size, int dtype,
               void *stream)
{
    ClearError();
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    if (size == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(A && B && C, "null pointer");
    unsigned grid = GridFor((size + kThreads - 1) / kThreads, 8);
    if (dtype == JETGPU_C64)
        add_kernel<float2><<<grid, kThreads, 0, AsStream(stream)>>>(
            (const float2 *)A, (const float2 *)B, (float2 *)C, size);
    else
        add_kernel<double2><<<grid, kThreads, 0, AsStream(stream)>>>(
            (const double2 *)A, (const double2 *)B, (double2 *)C, size);
    return CheckLaunch("add_kernel");
}

int jetgpu_conj(const void *in, void *out, uint64_t size, int dtype, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    if (size == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in && out, "null pointer");
    unsigned grid = GridFor((size + kThreads - 1) / kThreads, 8);
    if (dtype == JETGPU_C64)
        conj_kernel<float2><<<grid, kThreads, 0, AsStream(stream)>>>(
            (const float2 *)in, (float2 *)out, size);
    else
        conj_kernel<double2><<<grid, kThreads, 0, AsStream(stream)>>>(
            (const double2 *)in, (double2 *)out, size);
    return CheckLaunch("conj_kernel");
}

int jetgpu_slice_sum_f64(const void *results, uint64_t n_slices, uint64_t size,
                         int dtype, void *out, int accumulate, void *stream)
{
    NvtxRange range("jetgpu_slice_sum_f64");
    ClearError();
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    if (size == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(out != nullptr, "null output");
    if (n_slices == 0 && accumulate)
        return JETGPU_OK;
    JETGPU_REQUIRE(n_slices == 0 || results != nullptr, "null results");
    cudaStream_t st = AsStream(stream);
    if (size >= kThreads) {
        unsigned grid = GridFor((size + kThreads - 1) / kThreads, 8);
        if (dtype == JETGPU_C64)
            slice_sum_wide<float2><<<grid, kThreads, 0, st>>>(
                (const float2 *)results, (double2 *)out, n_slices, size, accumulate);
        else
            slice_sum_wide<double2><<<grid, kThreads, 0, st>>>(
                (const double2 *)results, (double2 *)out, n_slices, size, accumulate);
    }
    else {
        unsigned grid = (unsigned)size;
        if (dtype == JETGPU_C64)
            slice_sum_narrow<float2><<<grid, kThreads, 0, st>>>(
                (const float2 *)results, (double2 *)out, n_slices, size, accumulate);
        else
            slice_sum_narrow<double2><<<grid, kThreads, 0, st>>>(
                (const double2 *)results, (double2 *)out, n_slices, size, accumulate);
    }
    return CheckLaunch("slice_sum");
}

static int SliceGatherImpl(const void *in, int rank, const uint64_t *shape, int n_axes,
                           const int32_t *axes, const uint64_t *value_strides,
                           uint64_t first_value, const uint64_t *first_dev, uint64_t n_values,
                           void *out, int dtype, void *stream, bool scatter_add = false);

int jetgpu_slice_gather(const void *in, int rank, const uint64_t *shape,
                        int n_axes, const int32_t *axes,
                        const uint64_t *value_strides, uint64_t first_value,
                        uint64_t n_values, void *out, int dtype, void *stream)
{
    return SliceGatherImpl(in, rank, shape, n_axes, axes, value_strides, first_value, nullptr,
                           n_values, out, dtype, stream);
}

int jetgpu_slice_gather_at(const void *in, int rank, const uint64_t *shape, int n_axes,
                           const int32_t *axes, const uint64_t *value_strides,
                           const uint64_t *first_value_dev, uint64_t n_values, void *out,
                           int dtype, void *stream)
{
    JETGPU_REQUIRE(first_value_dev != nullptr, "null first-value pointer");
    return SliceGatherImpl(in, rank, shape, n_axes, axes, value_strides, 0, first_value_dev,
                           n_values, out, dtype, stream);
}

int jetgpu_slice_scatter_add(const void *sliced, int rank, const uint64_t *shape, int n_axes,
                             const int32_t *axes, const uint64_t *value_strides, uint64_t value,
                             void *full, int dtype, void *stream)
{
    return SliceGatherImpl(sliced, rank, shape, n_axes, axes, value_strides, value, nullptr, 1,
                           full, dtype, stream, true);
}

int jetgpu_counter_add(uint64_t *counter_dev, uint64_t delta, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(counter_dev != nullptr, "null counter");
    counter_add_kernel<<<1, 1, 0, AsStream(stream)>>>(counter_dev, delta);
    return CheckLaunch("counter_add_kernel");
}

static int SliceGatherImpl(const void *in, int rank, const uint64_t *shape, int n_axes,
                           const int32_t *axes, const uint64_t *value_strides,
                           uint64_t first_value, const uint64_t *first_dev, uint64_t n_values,
                           void *out, int dtype, void *stream, bool scatter_add)
{
    ClearError();
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    JETGPU_REQUIRE(rank >= 0 && rank <= kMaxRank, "rank out of range");
    JETGPU_REQUIRE(n_axes >= 0 && n_axes <= rank, "bad number of sliced axes");
    std::vector<uint64_t> stride(rank, 1);
    for (int i = rank - 2; i >= 0; --i)
        stride[i] = stride[i + 1] * shape[i + 1];
    std::vector<char> fixed(rank, 0);
    static thread_local SliceParams p;
    p.n_axes = n_axes;
    for (int j = 0; j < n_axes; ++j) {
        JETGPU_REQUIRE(axes[j] >= 0 && axes[j] < rank && !fixed[axes[j]],
                       "bad sliced axis");
        JETGPU_REQUIRE(value_strides[j] >= 1, "bad value stride");
        fixed[axes[j]] = 1;
        p.fixed_stride[j] = stride[axes[j]];
        p.fixed_dim[j] = shape[axes[j]];
        p.value_stride[j] = value_strides[j];
    }
    p.free_rank = 0;
    p.out_size = 1;
    for (int i = 0; i < rank; ++i)
        if (!fixed[i]) {
            p.free_dims[p.free_rank] = shape[i];
            p.free_strides[p.free_rank] = stride[i];
            ++p.free_rank;
            p.out_size *= shape[i];
        }
    p.first_value = first_value;
    p.total = p.out_size * n_values;
    if (p.total == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in && out, "null pointer");
    unsigned grid = GridFor((p.total + kThreads - 1) / kThreads, 8);
    if (scatter_add) {
        // `in` is the sliced tensor, `out` the full one it is added into.
        if (dtype == JETGPU_C64)
            slice_scatter_add_kernel<float2, float><<<grid, kThreads, 0, AsStream(stream)>>>(
                p, (const float2 *)in, (float2 *)out);
        else
            slice_scatter_add_kernel<double2, double><<<grid, kThreads, 0, AsStream(stream)>>>(
                p, (const double2 *)in, (double2 *)out);
        return CheckLaunch("slice_scatter_add_kernel");
    }
    if (dtype == JETGPU_C64)
        slice_gather_kernel<uint2><<<grid, kThreads, 0, AsStream(stream)>>>(
            p, (const uint2 *)in, (uint2 *)out, first_dev);
    else
        slice_gather_kernel<uint4><<<grid, kThreads, 0, AsStream(stream)>>>(
            p, (const uint4 *)in, (uint4 *)out, first_dev);
    return CheckLaunch("slice_gather_kernel");
}

int jetgpu_max_exponent(const void *x, uint64_t size, int dtype, int *exp_dev,
                        void *stream)
{
    ClearError();
    return MaxExponent(x, size, dtype, exp_dev, AsStream(stream));
}

} // extern "C"

namespace jetgpu {

int MaxExponent(const void *x, uint64_t size, int dtype, int *exp_dev, cudaStream_t st)
{
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    JETGPU_REQUIRE(exp_dev != nullptr, "null exponent pointer");
    if (size == 0) {
        init_exp_kernel<<<1, 1, 0, st>>>(exp_dev);
        return CheckLaunch("init_exp_kernel");
    }
    return MaxExponent2(x, size, x, 0, dtype, exp_dev, st, 1);
}

// Both operands' max exponents (e[0] of x0, e[1] of x1) with one fill and one
// launch; `operands` = 1 computes e[0] only. Empty operands leave their word
// at the fill value (below any exponent).
int MaxExponent2(const void *x0, uint64_t n0, const void *x1, uint64_t n1, int dtype, int *e,
                 cudaStream_t st, int operands, const int *hint0, const int *hint1)
{
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    JETGPU_REQUIRE(e != nullptr, "null exponent pointer");
    JETGPU_REQUIRE((n0 == 0 || x0 != nullptr) && (n1 == 0 || x1 != nullptr), "null input");
    JETGPU_CUDA_TRY(cudaMemsetAsync(e, 0x80, sizeof(int) * operands, st));
    const uint64_t n = n0 > n1 ? n0 : n1;
    const dim3 grid(GridFor((n + kThreads - 1) / kThreads, 8), (unsigned)operands);
    if (dtype == JETGPU_C64)
        max_exp_kernel<float2, uint32_t><<<grid, kThreads, 0, st>>>(
            (const float2 *)x0, n0, (const float2 *)x1, n1, e, hint0, hint1);
    else
        max_exp_kernel<double2, unsigned long long><<<grid, kThreads, 0, st>>>(
            (const double2 *)x0, n0, (const double2 *)x1, n1, e, hint0, hint1);
    return CheckLaunch("max_exp_kernel");
}

} // namespace jetgpu
