// Plain-arithmetic complex products (the "plain FP32" form and complex128).
//
// Replaces TensorHelpers::MultiplyTensorData (include/jet/TensorHelpers.hpp:
// 128-168), which dispatches row-major CBLAS cgemm/zgemm (m, n > 1),
// cgemv (right labels empty), cgemv^T (left labels empty) and cdotu (both
// empty) with alpha = 1, beta = 0. Here:
//  * gemm_kernel: 128x64 (complex64) / 64x64 (complex128) CTA tiles (32x64
//    when M <= 32), 8-deep
//    k slices staged in shared memory with register double buffering, each
//    thread accumulating an 8x4 (4x4) block of complex outputs with 4 FMAs
//    per complex multiply-add. Products whose tiles would leave SMs idle
//    split k into partial sums in the workspace (GemmSplits), reduced in a
//    fixed order.
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

template <typename T, int TM>
__global__ void __launch_bounds__(256)
    gemm_kernel(const typename C2<T>::type *__restrict__ A,
                const typename C2<T>::type *__restrict__ B,
                typename C2<T>::type *__restrict__ C, int64_t M, int64_t N,
                int64_t K, T scale, int64_t sa, int64_t sb, int splits, int64_t kchunk)
{
    using V = typename C2<T>::type;
    // blockIdx.z = b * splits + s: batch b (operand strides sa, sb, 0 =
    // shared; C packed) and k range s (splits > 1: [s kchunk, (s + 1)
    // kchunk), partial sums to C + (s * batch + b) * M * N, reduced later).
    const int64_t s = (int64_t)blockIdx.z % splits;
    const int64_t bz = (int64_t)blockIdx.z / splits;
    const int64_t batch = (int64_t)gridDim.z / splits;
    A += bz * sa;
    B += bz * sb;
    C += (s * batch + bz) * M * N;
    const int64_t lda = K; // A's row length
    const int64_t k_begin = s * kchunk;
    const int64_t k_end = min(K, k_begin + kchunk);
    A += k_begin;
    B += k_begin * N;
    K = k_end > k_begin ? k_end - k_begin : 0; // this split's k range
    constexpr int BM = TM * kTY;
    constexpr int BN = kTN * kTX;
    constexpr int A_PER = BM * kBK / 256; // A elements loaded per thread
    constexpr int B_PER = BN * kBK / 256;

    __shared__ V As[2][kBK][BM + 1];
    __shared__ V Bs[2][kBK][BN];

    const int tid = threadIdx.x;
    const int tx = tid % kTX, ty = tid / kTX;
    // Tiles in row-major order over one grid dimension (N tiles fastest), so
    // M may exceed 65535 tiles (2^23 rows).
    const int64_t tiles_n = (N + BN - 1) / BN;
    const int64_t m0 = ((int64_t)blockIdx.x / tiles_n) * BM;
    const int64_t n0 = ((int64_t)blockIdx.x % tiles_n) * BN;

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
            ra[q] = (gm < M && gk < K) ? A[gm * lda + gk] : V{0, 0};
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

// y[b, m] (+ partial s) = sum_{k in chunk s} A_b[m, k] x_b[k]. A CTA of 8
// warps covers `rows` rows (8, 4, 2 or 1) with 8 / rows warps per row, which
// interleave the row's k chunk, so few rows still keep every warp streaming.
// Batch b = blockIdx.z (operand strides sa, sb; 0 = shared). Partial s of row
// (b, m) lands at out[(s * batch + b) * M + m].
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_rows_kernel(const typename C2<T>::type *__restrict__ A,
                     const typename C2<T>::type *__restrict__ x,
                     typename C2<T>::type *__restrict__ out, int64_t M,
                     int64_t K, int64_t kchunk, T scale, int64_t sa, int64_t sb, int rows)
{
    using V = typename C2<T>::type;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wpr = 8 / rows; // warps per row
    const int part = warp % wpr;
    const int64_t m = (int64_t)blockIdx.x * rows + warp / wpr;
    const int64_t s = blockIdx.y;
    const int64_t b = blockIdx.z;
    A += b * sa;
    x += b * sb;
    out += (s * gridDim.z + b) * M;
    const int64_t k_begin = s * kchunk;
    const int64_t k_end = min(K, k_begin + kchunk);
    KahanSum<T> sr, si;
    if (m < M) {
        // Four products per compensated add: four loads in flight per thread
        // and a quarter of the compensation work (the sum of four products
        // carries one rounding of the plain FMA chain).
        const int64_t step = wpr * 32;
        int64_t k = k_begin + part * 32 + lane;
        for (; k + 3 * step < k_end; k += 4 * step) {
            V a[4], xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = A[m * K + k + u * step];
                xv[u] = x[k + u * step];
            }
            T re = a[0].x * xv[0].x - a[0].y * xv[0].y;
            T im = a[0].x * xv[0].y + a[0].y * xv[0].x;
#pragma unroll
            for (int u = 1; u < 4; ++u) {
                re = fma(a[u].x, xv[u].x, fma(-a[u].y, xv[u].y, re));
                im = fma(a[u].x, xv[u].y, fma(a[u].y, xv[u].x, im));
            }
            sr.add(re);
            si.add(im);
        }
        for (; k < k_end; k += step) {
            V a = A[m * K + k], b = x[k];
            sr.add(fma(a.x, b.x, -a.y * b.y));
            si.add(fma(a.x, b.y, a.y * b.x));
        }
    }
    T re = sr.s, im = si.s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    __shared__ T wre[8], wim[8];
    if (lane == 0) {
        wre[warp] = re;
        wim[warp] = im;
    }
    __syncthreads();
    if (lane == 0 && part == 0 && m < M) {
        for (int w = 1; w < wpr; ++w) { // fixed order: deterministic
            re += wre[warp + w];
            im += wim[warp + w];
        }
        out[m] = V{re * scale, im * scale};
    }
}

// y[b, n] (+ partial s) = sum_{k in chunk s} x_b[k] B_b[k, n]. A CTA of 256
// threads covers `cols` columns (a power of two up to 256) with 256 / cols
// threads per column, which interleave the k chunk: thread t takes column
// t % cols and rows k = t / cols (mod 256 / cols), so consecutive threads read
// consecutive elements of B's rows. `cols` = 1 is the dot product. Batch b =
// blockIdx.z (strides sa, sb; 0 = shared). Partial s of column (b, n) lands at
// out[(s * batch + b) * N + n].
template <typename T>
__global__ void __launch_bounds__(256)
    gemv_cols_kernel(const typename C2<T>::type *__restrict__ x,
                     const typename C2<T>::type *__restrict__ B,
                     typename C2<T>::type *__restrict__ out, int64_t N,
                     int64_t K, int64_t kchunk, T scale, int64_t sa, int64_t sb, int cols)
{
    using V = typename C2<T>::type;
    const int64_t s = blockIdx.y;
    const int64_t b = blockIdx.z;
    const int tk_count = 256 / cols;
    const int tn = threadIdx.x % cols;
    const int tk = threadIdx.x / cols;
    const int64_t n = (int64_t)blockIdx.x * cols + tn;
    const int64_t k_begin = s * kchunk;
    const int64_t k_end = min(K, k_begin + kchunk);
    x += b * sa;
    B += b * sb;
    out += (s * gridDim.z + b) * N;
    KahanSum<T> sr, si;
    if (n < N) {
        // Four products per compensated add (see gemv_rows_kernel).
        int64_t k = k_begin + tk;
        for (; k + 3 * (int64_t)tk_count < k_end; k += 4 * (int64_t)tk_count) {
            V a[4], v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = x[k + u * tk_count];
                v[u] = B[(k + u * tk_count) * N + n];
            }
            T re = a[0].x * v[0].x - a[0].y * v[0].y;
            T im = a[0].x * v[0].y + a[0].y * v[0].x;
#pragma unroll
            for (int u = 1; u < 4; ++u) {
                re = fma(a[u].x, v[u].x, fma(-a[u].y, v[u].y, re));
                im = fma(a[u].x, v[u].y, fma(a[u].y, v[u].x, im));
            }
            sr.add(re);
            si.add(im);
        }
        for (; k < k_end; k += tk_count) {
            V a = x[k], v = B[k * N + n];
            sr.add(fma(a.x, v.x, -a.y * v.y));
            si.add(fma(a.x, v.y, a.y * v.x));
        }
    }
    if (tk_count == 1) {
        if (n < N)
            out[n] = V{sr.s * scale, si.s * scale};
        return;
    }
    __shared__ T pre[256], pim[256];
    pre[threadIdx.x] = sr.s;
    pim[threadIdx.x] = si.s;
    __syncthreads();
    if (tk == 0 && n < N) {
        T re = 0, im = 0;
        for (int j = 0; j < tk_count; ++j) { // fixed order: deterministic
            re += pre[j * cols + tn];
            im += pim[j * cols + tn];
        }
        out[n] = V{re * scale, im * scale};
    }
}

// Products with a small output and a long k: M <= 16 and N <= 32, or M <= 32
// and N <= 16, with k >= 2048 -- steps that close two large tensors down to a
// few values, such as the 16 x 32 x 2^21 step of the reference's m10 network,
// where gemm_kernel's 32 x 64 tile is three quarters empty and streams 8 k per
// pass with few loads in flight (1.06 ms, 0.76 TB/s). Here one CTA per
// (k range, batch item):
//  * the A (MT x KC, stored k-major under an XOR swizzle) and B (KC x NT)
//    tiles of the range come in by cp.async, double-buffered, elements past
//    M, N or the range zero-filled; KC = 32 (complex64) or 16 (complex128),
//    so each warp has four (two) k per tile between barriers;
//  * the 8 warps split every tile, each lane accumulating an
//    (MT / 4) x (NT / 8) block, so each warp covers the whole output;
//  * the warps' sums are added in warp order in shared memory and the k
//    ranges' in the workspace by reduce_partials: a fixed order.
template <typename V> __device__ __forceinline__ void CpAsyncElem(V *smem, const V *src, bool valid)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
    const int n = valid ? (int)sizeof(V) : 0; // 0: zero-fill, nothing read
    if constexpr (sizeof(V) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(n)
                     : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n)
                     : "memory");
}

template <typename T, int MT, int NT>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1)
    gemm_small_kernel(const typename C2<T>::type *__restrict__ A,
                      const typename C2<T>::type *__restrict__ B,
                      typename C2<T>::type *__restrict__ C, int64_t M, int64_t N, int64_t K,
                      T scale, int64_t sa, int64_t sb, int64_t kchunk)
{
    using V = typename C2<T>::type;
    constexpr int TR = MT / 4, TC = NT / 8;
    constexpr int kSmallKC = sizeof(T) == 4 ? 32 : 16;
    constexpr int NS = 2; // stages (three measured 5 % slower: occupancy, not latency, binds)
    __shared__ __align__(16) V As[NS][kSmallKC * MT];
    __shared__ __align__(16) V Bs[NS][kSmallKC][NT];
    __shared__ V red[MT * NT];
    const int64_t s = blockIdx.x, bz = blockIdx.z, batch = gridDim.z;
    A += bz * sa;
    B += bz * sb;
    C += (s * batch + bz) * M * N;
    const int64_t k_begin = s * kchunk;
    const int64_t k_end = min(K, k_begin + kchunk);
    const int64_t tiles = k_end > k_begin ? (k_end - k_begin + kSmallKC - 1) / kSmallKC : 0;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rg = lane >> 3, cg = lane & 7;

    auto load = [&](int st, int64_t t) {
        const int64_t k0 = k_begin + t * kSmallKC;
        for (int e = tid; e < MT * kSmallKC; e += 256) {
            const int i = e / kSmallKC, kk = e % kSmallKC;
            const bool ok = i < M && k0 + kk < k_end;
            CpAsyncElem(&As[st][kk * MT + (i ^ (kk & (MT - 1)))], ok ? A + i * K + k0 + kk : A,
                        ok);
        }
        for (int e = tid; e < kSmallKC * NT; e += 256) {
            const int kk = e / NT, j = e % NT;
            const bool ok = j < N && k0 + kk < k_end;
            CpAsyncElem(&Bs[st][kk][j], ok ? B + (k0 + kk) * N + j : B, ok);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    V acc[TR][TC];
#pragma unroll
    for (int r = 0; r < TR; ++r)
#pragma unroll
        for (int c = 0; c < TC; ++c)
            acc[r][c] = V{0, 0};
    // Every iteration commits one group (empty past the last tile), so
    // wait_group NS - 1 always means "tile t has landed".
    for (int q = 0; q < NS - 1; ++q) {
        if (q < tiles)
            load(q, q);
        else
            asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int64_t t = 0; t < tiles; ++t) {
        const int st = (int)(t % NS);
        if (t + NS - 1 < tiles)
            load((int)((t + NS - 1) % NS), t + NS - 1);
        else
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group %0;\n" ::"n"(NS - 1) : "memory");
        __syncthreads();
#pragma unroll
        for (int kk = warp; kk < kSmallKC; kk += 8) {
            V a[TR], b[TC];
#pragma unroll
            for (int r = 0; r < TR; ++r)
                a[r] = As[st][kk * MT + ((rg * TR + r) ^ (kk & (MT - 1)))];
#pragma unroll
            for (int c = 0; c < TC; ++c)
                b[c] = Bs[st][kk][cg * TC + c];
#pragma unroll
            for (int r = 0; r < TR; ++r)
#pragma unroll
                for (int c = 0; c < TC; ++c) {
                    acc[r][c].x = fma(a[r].x, b[c].x, acc[r][c].x);
                    acc[r][c].x = fma(-a[r].y, b[c].y, acc[r][c].x);
                    acc[r][c].y = fma(a[r].x, b[c].y, acc[r][c].y);
                    acc[r][c].y = fma(a[r].y, b[c].x, acc[r][c].y);
                }
        }
        __syncthreads(); // the next load reuses this stage
    }
    for (int w = 0; w < 8; ++w) {
        if (warp == w) {
#pragma unroll
            for (int r = 0; r < TR; ++r)
#pragma unroll
                for (int c = 0; c < TC; ++c) {
                    V &o = red[(rg * TR + r) * NT + cg * TC + c];
                    if (w == 0)
                        o = acc[r][c];
                    else
                        o = V{o.x + acc[r][c].x, o.y + acc[r][c].y};
                }
        }
        __syncthreads();
    }
    for (int64_t e = tid; e < M * N; e += 256) {
        const V v = red[(e / N) * NT + e % N];
        C[e] = V{v.x * scale, v.y * scale};
    }
}

// Sums of the k ranges' partial results, accumulated in FP64: the partials
// of a long product can be much larger than their sum (an amplitude is a sum
// of terms of both signs), so FP32 adds here would cost accuracy the k ranges
// kept.
template <typename T>
__global__ void reduce_partials(const typename C2<T>::type *__restrict__ part,
                                typename C2<T>::type *__restrict__ out,
                                int64_t len, int64_t S)
{
    using V = typename C2<T>::type;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        for (int64_t s = 0; s < S; ++s) {
            V v = part[s * len + i];
            re += v.x;
            im += v.y;
        }
        out[i] = V{(T)re, (T)im};
    }
}

// reduce_partials for few outputs over many partial sums (S >= 64): one warp
// per output, lane l adding partials l, l + 32, ... in order (FP64), then a
// fixed shuffle tree -- a fixed order, where one thread per output walked the
// S partials one dependent load at a time (93 us for 512 outputs of 456 k
// ranges).
template <typename T>
__global__ void reduce_partials_warp(const typename C2<T>::type *__restrict__ part,
                                     typename C2<T>::type *__restrict__ out, int64_t len,
                                     int64_t S)
{
    using V = typename C2<T>::type;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < len;
         i += warps) {
        double re = 0, im = 0;
#pragma unroll 4
        for (int64_t s = lane; s < S; s += 32) {
            const V v = part[s * len + i];
            re += v.x;
            im += v.y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if (lane == 0)
            out[i] = V{(T)re, (T)im};
    }
}

// Sums S partial results of `len` elements each into out (a fixed order).
template <typename T>
int ReducePartials(const typename C2<T>::type *part, typename C2<T>::type *out, int64_t len,
                   int64_t S, cudaStream_t stream)
{
    if (S >= 64 && len <= 65536) {
        reduce_partials_warp<T><<<GridFor((len * 32 + 255) / 256, 8), 256, 0, stream>>>(
            part, out, len, S);
        return CheckLaunch("reduce_partials_warp");
    }
    reduce_partials<T><<<GridFor((len + 255) / 256, 4), 256, 0, stream>>>(part, out, len, S);
    return CheckLaunch("reduce_partials");
}

template <typename T>
__global__ void fill_zero(typename C2<T>::type *out, int64_t len)
{
    using V = typename C2<T>::type;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = V{0, 0};
}

// Split-k factor of the matrix product when its tiles (times the batch) do
// not fill the GPU: up to two CTAs per SM, at least 256 k per split, and at
// most 32 MiB of partial sums (out_bytes: the bytes of C).
int64_t GemmSplits(int64_t ctas, int64_t batch, int64_t K, int64_t out_bytes)
{
    const int64_t target = (int64_t)SmCount() * 2;
    if (ctas >= target / 2 || K < 512)
        return 1;
    int64_t s = (target + ctas - 1) / ctas;
    s = min(s, K / 256);
    s = min(s, (int64_t)65535 / (batch > 0 ? batch : 1));
    s = min(s, (int64_t)(32ll << 20) / (out_bytes > 0 ? out_bytes : 1));
    return s < 2 ? 1 : s;
}

// The small-output kernel's tile (MT x NT; 0: the product is not one) and
// its k ranges: one wave of CTAs (the kernel's launch bounds guarantee three
// per SM for complex64, one for complex128; a second, partial wave cost a
// third of the time), at least 1024 k each, at most 32 MiB of partial sums.
inline void SmallTile(int64_t M, int64_t N, int64_t K, int &mt, int &nt)
{
    mt = nt = 0;
    if (K < 2048 || M < 2 || N < 2)
        return;
    if (M <= 16 && N <= 32) {
        mt = 16;
        nt = 32;
    } else if (M <= 32 && N <= 16) {
        mt = 32;
        nt = 16;
    }
}

int64_t SmallSplits(int64_t batch, int64_t K, int64_t out_bytes, size_t elem_bytes)
{
    int64_t s = (int64_t)SmCount() * (elem_bytes == 8 ? 3 : 1) / (batch > 0 ? batch : 1);
    s = min(s, K / 1024);
    s = min(s, (int64_t)(32ll << 20) / (out_bytes > 0 ? out_bytes : 1));
    return s < 2 ? 1 : s;
}

// Rows per thread of the SIMT product: the full 128 (complex64) / 64
// (complex128) row tiles, or 32-row tiles when M is at most 32 (skinny
// products would leave most of a full tile empty).
template <typename T> inline int GemmTM(int64_t M) { return M <= 32 ? 2 : GemmCfg<T>::TM; }

template <typename T> inline void GemmGrid(int64_t M, int64_t N, int64_t &tiles_n, int64_t &tiles_m)
{
    const int BM = GemmTM<T>(M) * kTY;
    constexpr int BN = kTN * kTX;
    tiles_n = (N + BN - 1) / BN;
    tiles_m = (M + BM - 1) / BM;
}

// Split-k factor for the vector kernels: enough CTAs to fill the GPU, with at
// least 1024 k per chunk.
int64_t SplitK(int64_t blocks_per_split, int64_t K)
{
    int64_t target = (int64_t)SmCount() * 4;
    int64_t s = blocks_per_split >= target ? 1 : target / blocks_per_split;
    int64_t max_s = (K + 1023) / 1024;
    if (s > max_s)
        s = max_s;
    return s < 1 ? 1 : s;
}

// Smallest power of two >= v, at most `cap`.
inline int Pow2AtLeast(int64_t v, int cap)
{
    int p = 1;
    while (p < v && p < cap)
        p <<= 1;
    return p;
}

// CTAs per batch element of the vector kernels, the rows (gemv_rows_kernel)
// or columns (gemv_cols_kernel) each CTA covers, and the vector length.
inline void VectorShape(int64_t m, int64_t n, int64_t &blocks, int &per_cta, int64_t &len)
{
    if (n == 1 && m > 1) {
        per_cta = Pow2AtLeast(m, 8);
        len = m;
    }
    else {
        per_cta = Pow2AtLeast(n, 256); // 1: the dot product
        len = n;
    }
    blocks = (len + per_cta - 1) / per_cta;
}

// Bytes of partial sums the split-k vector products of `batch` products use
// (0 for matrix products or when one split suffices).
template <typename T>
size_t VectorWorkspace(int64_t batch, int64_t m, int64_t n, int64_t k)
{
    using V = typename C2<T>::type;
    if (batch < 1)
        return 0;
    if (m > 1 && n > 1) {
        int mt, nt;
        SmallTile(m, n, k, mt, nt);
        if (mt) { // small output, long k: partial sums of its k ranges
            const int64_t S =
                SmallSplits(batch, k, batch * m * n * (int64_t)sizeof(V), sizeof(V));
            return S > 1 ? (size_t)(S * batch * m * n) * sizeof(V) : 0;
        }
        // Matrix products: partial sums of the k splits (GemmSplits).
        int64_t tn, tm;
        GemmGrid<T>(m, n, tn, tm);
        const int64_t S = GemmSplits(tn * tm * batch, batch, k, batch * m * n * (int64_t)sizeof(V));
        return S > 1 ? (size_t)(S * batch * m * n) * sizeof(V) : 0;
    }
    int64_t blocks, len;
    int per_cta;
    VectorShape(m, n, blocks, per_cta, len);
    const int64_t S = SplitK(blocks * batch, k);
    return S > 1 ? (size_t)(S * batch * len) * sizeof(V) : 0;
}

// GEMV (n == 1), GEMV^T (m == 1) and DOTU (both) of `batch` products, split
// over k into partial sums when the caller supplied room for them, reduced
// in a fixed order (deterministic).
template <typename T>
int MultiplyVectorT(const typename C2<T>::type *A, const typename C2<T>::type *B,
                    typename C2<T>::type *C, int64_t batch, int64_t sa, int64_t sb, int64_t M,
                    int64_t N, int64_t K, T scale, void *ws, size_t ws_bytes,
                    cudaStream_t stream)
{
    using V = typename C2<T>::type;
    JETGPU_REQUIRE(batch <= 65535, "batch too large for one launch");
    const size_t need = VectorWorkspace<T>(batch, M, N, K);
    const bool split = need > 0 && ws != nullptr && ws_bytes >= need;
    int64_t blocks, len;
    int per_cta;
    VectorShape(M, N, blocks, per_cta, len);
    const int64_t S = split ? SplitK(blocks * batch, K) : 1;
    const int64_t kchunk = (K + S - 1) / S;
    V *dst = S > 1 ? (V *)ws : C;
    const dim3 grid((unsigned)blocks, (unsigned)S, (unsigned)batch);
    if (N == 1 && M > 1)
        gemv_rows_kernel<T><<<grid, 256, 0, stream>>>(A, B, dst, M, K, kchunk, scale, sa, sb,
                                                      per_cta);
    else
        gemv_cols_kernel<T><<<grid, 256, 0, stream>>>(A, B, dst, N, K, kchunk, scale, sa, sb,
                                                      per_cta);
    int rc = CheckLaunch(N == 1 && M > 1 ? "gemv_rows_kernel" : "gemv_cols_kernel");
    if (rc || S == 1)
        return rc;
    return ReducePartials<T>(dst, C, batch * len, S, stream);
}

// Matrix product of `batch` pairs (strides sa, sb; 0 = shared), split over k
// into the workspace when the tiles alone would leave SMs idle and the caller
// supplied room for the partial sums (reduced in a fixed order).
template <typename T>
int GemmT(const typename C2<T>::type *A, const typename C2<T>::type *B, typename C2<T>::type *C,
          int64_t batch, int64_t sa, int64_t sb, int64_t M, int64_t N, int64_t K, T scale,
          void *ws, size_t ws_bytes, cudaStream_t stream)
{
    using V = typename C2<T>::type;
    const size_t need = VectorWorkspace<T>(batch, M, N, K);
    int mt, nt;
    SmallTile(M, N, K, mt, nt);
    if (mt) {
        JETGPU_REQUIRE(batch <= 65535, "batch too large for one launch");
        const int64_t S = (need > 0 && ws != nullptr && ws_bytes >= need)
                              ? SmallSplits(batch, K, batch * M * N * (int64_t)sizeof(V),
                                            sizeof(V))
                              : 1;
        const int64_t kchunk = (K + S - 1) / S;
        V *dst = S > 1 ? (V *)ws : C;
        const dim3 grid((unsigned)S, 1u, (unsigned)batch);
        if (mt == 16)
            gemm_small_kernel<T, 16, 32><<<grid, 256, 0, stream>>>(A, B, dst, M, N, K, scale, sa,
                                                                   sb, kchunk);
        else
            gemm_small_kernel<T, 32, 16><<<grid, 256, 0, stream>>>(A, B, dst, M, N, K, scale, sa,
                                                                   sb, kchunk);
        int rc = CheckLaunch("gemm_small_kernel");
        if (rc || S == 1)
            return rc;
        return ReducePartials<T>(dst, C, batch * M * N, S, stream);
    }
    int64_t tn, tm;
    GemmGrid<T>(M, N, tn, tm);
    const int64_t S =
        (need > 0 && ws != nullptr && ws_bytes >= need)
            ? GemmSplits(tn * tm * batch, batch, K, batch * M * N * (int64_t)sizeof(V))
            : 1;
    const int64_t kchunk = (K + S - 1) / S;
    JETGPU_REQUIRE(tn * tm <= 0x7fffffffLL && batch * S <= 65535,
                   "product too large for one launch");
    const dim3 grid((unsigned)(tn * tm), 1u, (unsigned)(batch * S));
    V *dst = S > 1 ? (V *)ws : C;
    if (GemmTM<T>(M) == 2)
        gemm_kernel<T, 2><<<grid, 256, 0, stream>>>(A, B, dst, M, N, K, scale, sa, sb, (int)S,
                                                    kchunk);
    else
        gemm_kernel<T, GemmCfg<T>::TM><<<grid, 256, 0, stream>>>(A, B, dst, M, N, K, scale, sa,
                                                                 sb, (int)S, kchunk);
    int rc = CheckLaunch("gemm_kernel");
    if (rc || S == 1)
        return rc;
    return ReducePartials<T>(dst, C, batch * M * N, S, stream);
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
    if (M > 1 && N > 1)
        return GemmT<T>(A, B, C, 1, 0, 0, M, N, K, scale, ws, ws_bytes, stream);
    return MultiplyVectorT<T>(A, B, C, 1, 0, 0, M, N, K, scale, ws, ws_bytes, stream);
}

template <typename T>
int MultiplyBatchedT(const void *Av, const void *Bv, void *Cv, int64_t batch, int64_t sa,
                     int64_t sb, int64_t M, int64_t N, int64_t K, int scale_exp, void *ws,
                     size_t ws_bytes, cudaStream_t stream)
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
    if (M > 1 && N > 1)
        return GemmT<T>(A, B, C, batch, sa, sb, M, N, K, scale, ws, ws_bytes, stream);
    return MultiplyVectorT<T>(A, B, C, batch, sa, sb, M, N, K, scale, ws, ws_bytes, stream);
}

} // namespace

int MultiplyPlainBatched(const void *A, const void *B, void *C, uint64_t batch, uint64_t sa,
                         uint64_t sb, uint64_t m, uint64_t n, uint64_t k, int dtype,
                         int scale_exp, void *workspace, size_t ws_bytes, cudaStream_t stream)
{
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    if (dtype == JETGPU_C128)
        return MultiplyBatchedT<double>(A, B, C, (int64_t)batch, (int64_t)sa, (int64_t)sb,
                                        (int64_t)m, (int64_t)n, (int64_t)k, scale_exp, workspace,
                                        ws_bytes, stream);
    return MultiplyBatchedT<float>(A, B, C, (int64_t)batch, (int64_t)sa, (int64_t)sb, (int64_t)m,
                                   (int64_t)n, (int64_t)k, scale_exp, workspace, ws_bytes,
                                   stream);
}

size_t MultiplyPlainWorkspace(uint64_t m, uint64_t n, uint64_t k, int dtype)
{
    return MultiplyPlainBatchedWorkspace(1, m, n, k, dtype);
}

size_t MultiplyPlainBatchedWorkspace(uint64_t batch, uint64_t m, uint64_t n, uint64_t k,
                                     int dtype)
{
    return dtype == JETGPU_C128 ? VectorWorkspace<double>(batch, m, n, k)
                                : VectorWorkspace<float>(batch, m, n, k);
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
