// Plain-arithmetic complex products (the "plain FP32" form and complex128).
//
// Replaces TensorHelpers::MultiplyTensorData (include/jet/TensorHelpers.hpp:
// 128-168), which dispatches row-major CBLAS cgemm/zgemm (m, n > 1),
// cgemv (right labels empty), cgemv^T (left labels empty) and cdotu (both
// empty) with alpha = 1, beta = 0. Here:
//  * gemm_kernel: 128x64 (complex64) / 64x64 (complex128) CTA tiles, 8-deep
//    k slices staged in shared memory with register double buffering, each
//    thread accumulating an 8x4 (4x4) block of complex outputs with 4 FMAs
//    per complex multiply-add.
//  * gemv_rows_kernel (n == 1) / gemv_cols_kernel (m == 1, also DOTU): split
//    over k into partial sums, reduced in a fixed order by reduce_partials
//    (deterministic).
#include "common.cuh"

namespace jetgpu {
namespace {

template <typename T> struct C2;
template <> struct C2<float> {
    using type = float2;
};
template <> struct C2<double> {
    using type = double2;
};

template <typename T> struct GemmCfg;
template <> struct GemmCfg<float> {
    static constexpr int TM = 8; // rows per thread
};
template <> struct GemmCfg<double> {
    static constexpr int TM = 4;
};

constexpr int kBK = 8;
constexpr int kTN = 4;
constexpr int kTX = 16, kTY = 16; // 256 threads

template <typename T>
__global__ void __launch_bounds__(256)
    gemm_kernel(const typename C2<T>::type *__restrict__ A,
                const typename C2<T>::type *__restrict__ B,
                typename C2<T>::type *__restrict__ C, int64_t M, int64_t N,
                int64_t K, T scale, int64_t sa, int64_t sb)
{
    using V = typename C2<T>::type;
    constexpr int TM = GemmCfg<T>::TM;
    // Batch b = blockIdx.z: operand strides sa, sb (0 = shared), C packed.
    A += (int64_t)blockIdx.z * sa;
    B += (int64_t)blockIdx.z * sb;
    C += (int64_t)blockIdx.z * M * N;
    constexpr int BM = TM * kTY;
    constexpr int BN = kTN * kTX;
    constexpr int A_PER = BM * kBK / 256; // A elements loaded per thread
    constexpr int B_PER = BN * kBK / 256;

    __shared__ V As[2][kBK][BM + 1];
    __shared__ V Bs[2][kBK][BN];

    const int tid = threadIdx.x;
    const int tx = tid % kTX, ty = tid / kTX;
    const int64_t m0 = (int64_t)blockIdx.y * BM;
    const int64_t n0 = (int64_t)blockIdx.x * BN;

    V acc[TM][kTN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < kTN; ++j)
            acc[i][j] = V{0, 0};

    V ra[A_PER], rb[B_PER];
    auto load_tiles = [&](int64_t k0) {
#pragma unroll
        for (int q = 0; q < A_PER; ++q) {
            int row = tid / kBK + q * (256 / kBK);
            int col = tid % kBK;
            int64_t gm = m0 + row, gk = k0 + col;
            ra[q] = (gm < M && gk < K) ? A[gm * K + gk] : V{0, 0};
        }
#pragma unroll
        for (int q = 0; q < B_PER; ++q) {
            int row = tid / BN + q * (256 / BN);
            int col = tid % BN;
            int64_t gk = k0 + row, gn = n0 + col;
            rb[q] = (gk < K && gn < N) ? B[gk * N + gn] : V{0, 0};
        }
    };
    auto store_tiles = [&](int buf) {
#pragma unroll
        for (int q = 0; q < A_PER; ++q) {
            int row = tid / kBK + q * (256 / kBK);
            int col = tid % kBK;
            As[buf][col][row] = ra[q];
        }
#pragma unroll
        for (int q = 0; q < B_PER; ++q) {
            int row = tid / BN + q * (256 / BN);
            int col = tid % BN;
            Bs[buf][row][col] = rb[q];
        }
    };

    const int64_t ktiles = (K + kBK - 1) / kBK;
    if (ktiles > 0) {
        load_tiles(0);
        store_tiles(0);
    }
    __syncthreads();
    for (int64_t kt = 0; kt < ktiles; ++kt) {
        const int buf = kt & 1;
        const bool more = kt + 1 < ktiles;
        if (more)
            load_tiles((kt + 1) * kBK);
#pragma unroll
        for (int k = 0; k < kBK; ++k) {
            V a[TM], b[kTN];
#pragma unroll
            for (int i = 0; i < TM; ++i)
                a[i] = As[buf][k][ty + kTY * i];
#pragma unroll
            for (int j = 0; j < kTN; ++j)
                b[j] = Bs[buf][k][tx + kTX * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < kTN; ++j) {
                    acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
                    acc[i][j].x = fma(-a[i].y, b[j].y, acc[i][j].x);
                    acc[i][j].y = fma(a[i].x, b[j].y, acc[i][j].y);
                    acc[i][j].y = fma(a[i].y, b[j].x, acc[i][j].y);
                }
        }
        if (more)
            store_tiles(buf ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        int64_t gm = m0 + ty + kTY * i;
        if (gm >= M)
            continue;
#pragma unroll
        for (int j = 0; j < kTN; ++j) {
            int64_t gn = n0 + tx + kTX * j;
            if (gn < N)
                C[gm * N + gn] = V{acc[i][j].x * scale, acc[i][j].y * scale};
        }
    }
}

// Compensated (Kahan) running sum: vector-shaped products reduce long k
// ranges in one thread, where plain FP32 accumulation would lose ~log2(k)
// bits; the extra adds are free in these bandwidth-bound kernels.
template <typename T> struct KahanSum {
    T s = 0, c = 0;
    __device__ __forceinline__ void add(T x)
    {
        const T y = x - c;
        const T t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// y[m] (+ partial s) = sum_{k in chunk s} A[m, k] x[k]; one warp per row.
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_rows_kernel(const typename C2<T>::type *__restrict__ A,
                     const typename C2<T>::type *__restrict__ x,
                     typename C2<T>::type *__restrict__ out, int64_t M,
                     int64_t K, int64_t kchunk, T scale)
{
    using V = typename C2<T>::type;
    const int lane = threadIdx.x & 31;
    const int64_t m = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int64_t s = blockIdx.y;
    if (m >= M)
        return;
    const int64_t k_begin = s * kchunk;
    const int64_t k_end = min(K, k_begin + kchunk);
    KahanSum<T> sr, si;
    for (int64_t k = k_begin + lane; k < k_end; k += 32) {
        V a = A[m * K + k], b = x[k];
        sr.add(fma(a.x, b.x, -a.y * b.y));
        si.add(fma(a.x, b.y, a.y * b.x));
    }
    T re = sr.s, im = si.s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0)
        out[s * M + m] = V{re * scale, im * scale};
}

// y[n] (+ partial s) = sum_{k in chunk s} x[k] B[k, n]; one thread per column.
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_cols_kernel(const typename C2<T>::type *__restrict__ x,
                     const typename C2<T>::type *__restrict__ B,
                     typename C2<T>::type *__restrict__ out, int64_t N,
                     int64_t K, int64_t kchunk, T scale)
{
    using V = typename C2<T>::type;
    const int64_t s = blockIdx.y;
    const int64_t k_begin = s * kchunk;
    const int64_t k_end = min(K, k_begin + kchunk);
    if (N == 1) {
        // Dot product: the block reduces its k chunk.
        KahanSum<T> sr, si;
        for (int64_t k = k_begin + threadIdx.x; k < k_end; k += blockDim.x) {
            V a = x[k], b = B[k];
            sr.add(fma(a.x, b.x, -a.y * b.y));
            si.add(fma(a.x, b.y, a.y * b.x));
        }
        T re = sr.s, im = si.s;
        __shared__ T sre[256], sim[256];
        sre[threadIdx.x] = re;
        sim[threadIdx.x] = im;
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) {
                sre[threadIdx.x] += sre[threadIdx.x + w];
                sim[threadIdx.x] += sim[threadIdx.x + w];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0)
            out[s] = V{sre[0] * scale, sim[0] * scale};
        return;
    }
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N)
        return;
    KahanSum<T> sr, si;
    for (int64_t k = k_begin; k < k_end; ++k) {
        V a = x[k], b = B[k * N + n];
        sr.add(fma(a.x, b.x, -a.y * b.y));
        si.add(fma(a.x, b.y, a.y * b.x));
    }
    out[s * N + n] = V{sr.s * scale, si.s * scale};
}

// Batched vector products: row r of batch b (n == 1) or column c of batch b
// (m == 1); operand strides sa, sb (0 = shared).
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_rows_batched(const typename C2<T>::type *__restrict__ A,
                      const typename C2<T>::type *__restrict__ x,
                      typename C2<T>::type *__restrict__ out, int64_t batch, int64_t M,
                      int64_t K, int64_t sa, int64_t sb, T scale)
{
    using V = typename C2<T>::type;
    const int lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (row >= batch * M)
        return;
    const int64_t b = row / M, m = row - b * M;
    const V *a = A + b * sa + m * K;
    const V *v = x + b * sb;
    KahanSum<T> sr, si;
    for (int64_t k = lane; k < K; k += 32) {
        V p = a[k], q = v[k];
        sr.add(fma(p.x, q.x, -p.y * q.y));
        si.add(fma(p.x, q.y, p.y * q.x));
    }
    T re = sr.s, im = si.s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0)
        out[row] = V{re * scale, im * scale};
}

template <typename T>
__global__ void __launch_bounds__(256)
    gemv_cols_batched(const typename C2<T>::type *__restrict__ x,
                      const typename C2<T>::type *__restrict__ B,
                      typename C2<T>::type *__restrict__ out, int64_t batch, int64_t N,
                      int64_t K, int64_t sa, int64_t sb, T scale)
{
    using V = typename C2<T>::type;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= batch * N)
        return;
    const int64_t b = idx / N, n = idx - b * N;
    const V *v = x + b * sa;
    const V *bb = B + b * sb + n;
    KahanSum<T> sr, si;
    for (int64_t k = 0; k < K; ++k) {
        V p = v[k], q = bb[k * N];
        sr.add(fma(p.x, q.x, -p.y * q.y));
        si.add(fma(p.x, q.y, p.y * q.x));
    }
    out[idx] = V{sr.s * scale, si.s * scale};
}

template <typename T>
__global__ void reduce_partials(const typename C2<T>::type *__restrict__ part,
                                typename C2<T>::type *__restrict__ out,
                                int64_t len, int64_t S)
{
    using V = typename C2<T>::type;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
        T re = 0, im = 0;
        for (int64_t s = 0; s < S; ++s) {
            V v = part[s * len + i];
            re += v.x;
            im += v.y;
        }
        out[i] = V{re, im};
    }
}

template <typename T>
__global__ void fill_zero(typename C2<T>::type *out, int64_t len)
{
    using V = typename C2<T>::type;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = V{0, 0};
}

// Split-k factor for the vector kernels: enough CTAs to fill the GPU, with at
// least 4096 k per chunk.
int64_t SplitK(int64_t blocks_per_split, int64_t K)
{
    int64_t target = (int64_t)SmCount() * 4;
    int64_t s = blocks_per_split >= target ? 1 : target / blocks_per_split;
    int64_t max_s = (K + 4095) / 4096;
    if (s > max_s)
        s = max_s;
    return s < 1 ? 1 : s;
}

template <typename T>
size_t VectorWorkspace(int64_t m, int64_t n, int64_t k)
{
    using V = typename C2<T>::type;
    if (m > 1 && n > 1)
        return 0;
    int64_t len = n == 1 ? m : n;
    int64_t blocks = n == 1 ? (m + 7) / 8 : (n == 1 ? 1 : (n + 255) / 256);
    if (m == 1 && n == 1)
        blocks = 1;
    int64_t S = SplitK(blocks, k);
    return S > 1 ? (size_t)(S * len) * sizeof(V) : 0;
}

template <typename T>
int MultiplyT(const void *Av, const void *Bv, void *Cv, int64_t M, int64_t N,
              int64_t K, int scale_exp, void *ws, size_t ws_bytes,
              cudaStream_t stream)
{
    using V = typename C2<T>::type;
    const V *A = (const V *)Av;
    const V *B = (const V *)Bv;
    V *C = (V *)Cv;
    const T scale = (T)ldexp(1.0, scale_exp);
    if (M == 0 || N == 0)
        return JETGPU_OK;
    if (K == 0) {
        fill_zero<T><<<GridFor((M * N + 255) / 256, 4), 256, 0, stream>>>(
            C, M * N);
        return CheckLaunch("fill_zero");
    }
    if (M > 1 && N > 1) {
        constexpr int BM = GemmCfg<T>::TM * kTY;
        constexpr int BN = kTN * kTX;
        dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM));
        JETGPU_REQUIRE(grid.y <= 65535u, "m too large for one launch");
        gemm_kernel<T><<<grid, 256, 0, stream>>>(A, B, C, M, N, K, scale, 0, 0);
        return CheckLaunch("gemm_kernel");
    }
    // Split over k only when the caller supplied room for the partial sums.
    const size_t need = VectorWorkspace<T>(M, N, K);
    const bool split = need > 0 && ws != nullptr && ws_bytes >= need;
    if (N == 1 && M > 1) {
        int64_t blocks = (M + 7) / 8;
        int64_t S = split ? SplitK(blocks, K) : 1;
        int64_t kchunk = (K + S - 1) / S;
        V *dst = S > 1 ? (V *)ws : C;
        gemv_rows_kernel<T><<<dim3((unsigned)blocks, (unsigned)S), 256, 0,
                              stream>>>(A, B, dst, M, K, kchunk, scale);
        int rc = CheckLaunch("gemv_rows_kernel");
        if (rc || S == 1)
            return rc;
        reduce_partials<T><<<GridFor((M + 255) / 256, 4), 256, 0, stream>>>(
            dst, C, M, S);
        return CheckLaunch("reduce_partials");
    }
    // M == 1 (GEMV^T, or DOTU when N == 1).
    int64_t blocks = N == 1 ? 1 : (N + 255) / 256;
    int64_t S = split ? SplitK(blocks, K) : 1;
    int64_t kchunk = (K + S - 1) / S;
    V *dst = S > 1 ? (V *)ws : C;
    gemv_cols_kernel<T><<<dim3((unsigned)blocks, (unsigned)S), 256, 0,
                          stream>>>(A, B, dst, N, K, kchunk, scale);
    int rc = CheckLaunch("gemv_cols_kernel");
    if (rc || S == 1)
        return rc;
    reduce_partials<T><<<GridFor((N + 255) / 256, 4), 256, 0, stream>>>(
        dst, C, N, S);
    return CheckLaunch("reduce_partials");
}

template <typename T>
int MultiplyBatchedT(const void *Av, const void *Bv, void *Cv, int64_t batch, int64_t sa,
                     int64_t sb, int64_t M, int64_t N, int64_t K, int scale_exp,
                     cudaStream_t stream)
{
    using V = typename C2<T>::type;
    const V *A = (const V *)Av;
    const V *B = (const V *)Bv;
    V *C = (V *)Cv;
    const T scale = (T)ldexp(1.0, scale_exp);
    if (M == 0 || N == 0 || batch == 0)
        return JETGPU_OK;
    if (K == 0) {
        fill_zero<T><<<GridFor((batch * M * N + 255) / 256, 4), 256, 0, stream>>>(C, batch * M * N);
        return CheckLaunch("fill_zero");
    }
    if (M > 1 && N > 1) {
        constexpr int BM = GemmCfg<T>::TM * kTY;
        constexpr int BN = kTN * kTX;
        dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM), (unsigned)batch);
        JETGPU_REQUIRE(grid.y <= 65535u && grid.z <= 65535u, "batched product too large");
        gemm_kernel<T><<<grid, 256, 0, stream>>>(A, B, C, M, N, K, scale, sa, sb);
        return CheckLaunch("gemm_kernel (batched)");
    }
    if (N == 1) {
        const int64_t rows = batch * M;
        gemv_rows_batched<T><<<(unsigned)((rows + 7) / 8), 256, 0, stream>>>(A, B, C, batch, M, K,
                                                                            sa, sb, scale);
        return CheckLaunch("gemv_rows_batched");
    }
    const int64_t cols = batch * N;
    gemv_cols_batched<T><<<(unsigned)((cols + 255) / 256), 256, 0, stream>>>(A, B, C, batch, N,
                                                                            K, sa, sb, scale);
    return CheckLaunch("gemv_cols_batched");
}

} // namespace

int MultiplyPlainBatched(const void *A, const void *B, void *C, uint64_t batch, uint64_t sa,
                         uint64_t sb, uint64_t m, uint64_t n, uint64_t k, int dtype,
                         int scale_exp, cudaStream_t stream)
{
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    if (dtype == JETGPU_C128)
        return MultiplyBatchedT<double>(A, B, C, (int64_t)batch, (int64_t)sa, (int64_t)sb,
                                        (int64_t)m, (int64_t)n, (int64_t)k, scale_exp, stream);
    return MultiplyBatchedT<float>(A, B, C, (int64_t)batch, (int64_t)sa, (int64_t)sb, (int64_t)m,
                                   (int64_t)n, (int64_t)k, scale_exp, stream);
}

size_t MultiplyPlainWorkspace(uint64_t m, uint64_t n, uint64_t k, int dtype)
{
    return dtype == JETGPU_C128 ? VectorWorkspace<double>(m, n, k)
                                : VectorWorkspace<float>(m, n, k);
}

int MultiplyPlain(const void *A, const void *B, void *C, uint64_t m,
                  uint64_t n, uint64_t k, int dtype, int scale_exp,
                  void *workspace, size_t ws_bytes, cudaStream_t stream)
{
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    if (m * n > 0)
        JETGPU_REQUIRE(C != nullptr, "null output");
    if (m * n * k > 0)
        JETGPU_REQUIRE(A != nullptr && B != nullptr, "null operand");
    if (dtype == JETGPU_C128)
        return MultiplyT<double>(A, B, C, (int64_t)m, (int64_t)n, (int64_t)k,
                                 scale_exp, workspace, ws_bytes, stream);
    return MultiplyT<float>(A, B, C, (int64_t)m, (int64_t)n, (int64_t)k,
                            scale_exp, workspace, ws_bytes, stream);
}

} // namespace jetgpu
