// Skinny contractions: one side of the product at most 16 wide and at most 64
// contracted values -- a gate, or any small tensor, applied to a large one.
// Most slice-dependent steps of the reference's paper-benchmark networks
// (examples/paper_benchmarks/data_files/m10.json, m12.json) have this shape:
// a 2^25-row tensor times a 4 x 4 or 8 x 8 gate.
//
// The reference contracts every pair the same way (Tensor.hpp:708-752,
// ContractTensors): transpose both operands into (free, contracted) order,
// then one BLAS call. For a skinny step the transpose moves the large tensor
// twice more than the product does, and a GEMM tile 64 columns wide computes
// up to 64 times the useful work. Here one kernel reads the large operand in
// its own layout -- a row's offset from its free axes, the contracted
// offsets from a table of k entries -- keeps the small operand in (c, j)
// order in shared memory, and writes C in the product's row-major layout. The
// large tensor is read once and C written once: HBM-bound at (k + s) elements
// per row.
//
// Arithmetic: per output, FP32 (FP64) FMAs over c in increasing order with
// the plain form's complex multiply-add (re: +a.re b.re, -a.im b.im; im:
// +a.re b.im, +a.im b.re), then the power-of-two scale -- the sequence
// gemm_kernel runs when k <= 64, so products with m, n > 1 round as the
// transposing path does.
#include "common.cuh"

#include <cstring>
#include <type_traits>
#include <vector>

namespace jetgpu {
namespace {

constexpr int kSkAxes = 12; // axes of one index after merging
constexpr int kSkMaxS = 16; // small operand's free extent
constexpr int kSkMaxK = 64; // contracted extent
constexpr int kSkThreads = 256;

// The axes of one index of an operand, innermost first: the index's digits
// in mixed radix dim[] give the element offset sum_i digit_i stride[i].
struct SkAxes {
    int n;
    uint64_t dim[kSkAxes];
    uint64_t stride[kSkAxes];
};

struct SkinnyParams {
    uint64_t rows; // extent of the large operand's free index
    int s, k;      // small operand's free extent, contracted extent
    int narrow;    // rows < 2^32: row digits by 32-bit multiply-shift
    int vec;       // complex64 rows of C stored 16 bytes at a time
    SkAxes row;    // large operand: free axes
    uint32_t row_magic[kSkAxes], row_shift[kSkAxes];
    SkAxes big_c, big_b;               // large operand: contracted, batch axes
    SkAxes small_c, small_f, small_b;  // small operand: contracted, free, batch
    uint64_t out_row, out_col, out_batch; // C's element strides
};

template <typename T> struct C2;
template <> struct C2<float> {
    using type = float2;
};
template <> struct C2<double> {
    using type = double2;
};

__device__ __forceinline__ uint64_t AxesOffset(const SkAxes &a, uint64_t idx)
{
    uint64_t off = 0;
#pragma unroll
    for (int i = 0; i < kSkAxes; ++i)
        if (i < a.n) {
            const uint64_t q = idx / a.dim[i];
            off += (idx - q * a.dim[i]) * a.stride[i];
            idx = q;
        }
    return off;
}

__device__ __forceinline__ uint64_t RowOffset(const SkinnyParams &p, uint64_t r)
{
    if (!p.narrow)
        return AxesOffset(p.row, r);
    uint32_t x = (uint32_t)r;
    uint64_t off = 0;
#pragma unroll
    for (int i = 0; i < kSkAxes; ++i)
        if (i < p.row.n) {
            const uint32_t q = DivMagic(x, p.row_magic[i], p.row_shift[i]);
            off += (uint64_t)(x - q * (uint32_t)p.row.dim[i]) * p.row.stride[i];
            x = q;
        }
    return off;
}

// acc += a b in the plain form's FMA order.
template <typename V> __device__ __forceinline__ void Mac(V &acc, const V &a, const V &b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// One CTA per (row range, batch item); each thread one row of the large
// operand at a time. S: the small extent rounded up to a power of two (table
// columns j >= s are zero and not stored). BigIsA: the large operand is A
// (C's rows), else B (C's columns); the operands keep their roles in Mac.
template <typename T, int S, bool BigIsA>
__global__ void __launch_bounds__(kSkThreads)
    skinny_kernel(const typename C2<T>::type *__restrict__ big,
                  const typename C2<T>::type *__restrict__ small,
                  typename C2<T>::type *__restrict__ C, const __grid_constant__ SkinnyParams p,
                  T scale)
{
    using V = typename C2<T>::type;
    __shared__ V tab[kSkMaxK][S];
    __shared__ uint64_t coff[kSkMaxK];
    const uint64_t b = blockIdx.y;
    big += AxesOffset(p.big_b, b);
    small += AxesOffset(p.small_b, b);
    C += b * p.out_batch;
    for (int e = threadIdx.x; e < p.k * S; e += blockDim.x) {
        const int c = e / S, j = e % S;
        tab[c][j] = j < p.s ? small[AxesOffset(p.small_c, c) + AxesOffset(p.small_f, j)]
                            : V{0, 0};
    }
    for (int c = threadIdx.x; c < p.k; c += blockDim.x)
        coff[c] = AxesOffset(p.big_c, c);
    __syncthreads();

    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < p.rows; r += step) {
        const V *x = big + RowOffset(p, r);
        V acc[S];
#pragma unroll
        for (int j = 0; j < S; ++j)
            acc[j] = V{0, 0};
        for (int c0 = 0; c0 < p.k; c0 += 8) {
            V v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                v[u] = c0 + u < p.k ? __ldg(x + coff[c0 + u]) : V{0, 0};
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (c0 + u >= p.k)
                    break;
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    if (BigIsA)
                        Mac(acc[j], v[u], tab[c0 + u][j]);
                    else
                        Mac(acc[j], tab[c0 + u][j], v[u]);
                }
            }
        }
        V *out = C + r * p.out_row;
        if constexpr (std::is_same<T, float>::value && BigIsA && S >= 2) {
            if (p.vec) {
                float4 *o4 = reinterpret_cast<float4 *>(out);
#pragma unroll
                for (int j = 0; j < S; j += 2)
                    o4[j / 2] = make_float4(acc[j].x * scale, acc[j].y * scale,
                                            acc[j + 1].x * scale, acc[j + 1].y * scale);
                continue;
            }
        }
#pragma unroll
        for (int j = 0; j < S; ++j)
            if (j < p.s)
                out[j * p.out_col] = V{acc[j].x * scale, acc[j].y * scale};
    }
}

struct Ax {
    uint64_t d, s; // dimension, element stride
};

// Packs axes given outermost first, dropping unit axes and merging neighbours
// that are contiguous (outer stride = inner stride x inner dim).
bool Pack(const std::vector<Ax> &outer_first, SkAxes &out)
{
    std::vector<Ax> m;
    for (const Ax &a : outer_first) {
        if (a.d == 1)
            continue;
        if (!m.empty() && m.back().s == a.s * a.d) {
            m.back().d *= a.d;
            m.back().s = a.s;
        } else {
            m.push_back(a);
        }
    }
    if ((int)m.size() > kSkAxes)
        return false;
    out.n = (int)m.size();
    for (int i = 0; i < out.n; ++i) {
        out.dim[i] = m[out.n - 1 - i].d;
        out.stride[i] = m[out.n - 1 - i].s;
    }
    return true;
}

// Appends the axes perm[j], perm[j + 1], ... whose dimensions multiply to
// `extent` (false if no run of them does).
bool Take(int rank, const uint64_t *shape, const int32_t *perm, const std::vector<uint64_t> &st,
          int &j, uint64_t extent, std::vector<Ax> &out)
{
    uint64_t p = 1;
    while (p < extent && j < rank) {
        out.push_back({shape[perm[j]], st[perm[j]]});
        p *= shape[perm[j]];
        ++j;
    }
    return p == extent;
}

struct OperandAxes {
    std::vector<Ax> batch, first, second;
};

// An operand's permutation as (batch axes) (first group) (second group) with
// the groups' extents e1, e2. mode 0: shared; 1: `batch` tensors back to
// back; 2: one tensor whose permutation leads with the batch axes.
bool SplitOperand(int rank, const uint64_t *shape, const int32_t *perm, int mode,
                  uint64_t batch, uint64_t e1, uint64_t e2, OperandAxes &o)
{
    std::vector<uint64_t> st(rank, 1);
    for (int i = rank - 2; i >= 0; --i)
        st[i] = st[i + 1] * shape[i + 1];
    const uint64_t size = rank ? st[0] * shape[0] : 1;
    int j = 0;
    if (mode == 2 && !Take(rank, shape, perm, st, j, batch, o.batch))
        return false;
    if (mode == 1)
        o.batch.push_back({batch, size});
    return Take(rank, shape, perm, st, j, e1, o.first) &&
           Take(rank, shape, perm, st, j, e2, o.second);
}

bool Plan(uint64_t batch, int a_rank, const uint64_t *a_shape, const int32_t *a_perm,
          int a_batched, int b_rank, const uint64_t *b_shape, const int32_t *b_perm,
          int b_batched, uint64_t m, uint64_t n, uint64_t k, SkinnyParams &p, bool &big_is_a)
{
    if (k == 0 || k > kSkMaxK || m == 0 || n == 0 || batch == 0 || batch > 65535)
        return false;
    big_is_a = m >= n;
    const uint64_t s = big_is_a ? n : m;
    if (s > kSkMaxS)
        return false;
    OperandAxes a, b;
    if (!SplitOperand(a_rank, a_shape, a_perm, batch > 1 ? a_batched : 0, batch, m, k, a) ||
        !SplitOperand(b_rank, b_shape, b_perm, batch > 1 ? b_batched : 0, batch, k, n, b))
        return false;
    std::memset(&p, 0, sizeof(p));
    p.rows = big_is_a ? m : n;
    p.s = (int)s;
    p.k = (int)k;
    const bool ok = big_is_a ? (Pack(a.first, p.row) && Pack(a.second, p.big_c) &&
                                Pack(a.batch, p.big_b) && Pack(b.first, p.small_c) &&
                                Pack(b.second, p.small_f) && Pack(b.batch, p.small_b))
                             : (Pack(b.second, p.row) && Pack(b.first, p.big_c) &&
                                Pack(b.batch, p.big_b) && Pack(a.second, p.small_c) &&
                                Pack(a.first, p.small_f) && Pack(a.batch, p.small_b));
    if (!ok)
        return false;
    p.narrow = p.rows < (1ull << 32) ? 1 : 0;
    if (p.narrow)
        for (int i = 0; i < p.row.n; ++i)
            Magic32(p.row.dim[i], p.row_magic[i], p.row_shift[i]);
    p.out_row = big_is_a ? n : 1;
    p.out_col = big_is_a ? 1 : n;
    p.out_batch = m * n;
    return true;
}

// CTAs of skinny_kernel<T, S, BigIsA> that fit on an SM at once (cached).
template <typename T, int S, bool BigIsA> int Resident()
{
    static int n = 0;
    if (n == 0) {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, skinny_kernel<T, S, BigIsA>,
                                                          kSkThreads, 0) != cudaSuccess ||
            v < 1)
            v = 1;
        n = v;
    }
    return n;
}

template <typename T, int S, bool BigIsA>
int LaunchS(const void *big, const void *small, void *C, SkinnyParams &p, uint64_t batch,
            T scale, cudaStream_t st)
{
    using V = typename C2<T>::type;
    auto kernel = skinny_kernel<T, S, BigIsA>;
    p.vec = (std::is_same<T, float>::value && BigIsA && S >= 2 && p.s == S &&
             (reinterpret_cast<uintptr_t>(C) & 15) == 0)
                ? 1
                : 0;
    const uint64_t slots = (uint64_t)Resident<T, S, BigIsA>() * SmCount();
    uint64_t gx = (p.rows + kSkThreads - 1) / kSkThreads;
    const uint64_t per_item = slots / batch > 0 ? slots / batch : 1;
    if (gx > per_item)
        gx = per_item;
    kernel<<<dim3((unsigned)gx, (unsigned)batch), kSkThreads, 0, st>>>(
        static_cast<const V *>(big), static_cast<const V *>(small), static_cast<V *>(C), p,
        scale);
    return CheckLaunch("skinny_kernel");
}

template <typename T, bool BigIsA>
int LaunchT(const void *big, const void *small, void *C, SkinnyParams &p, uint64_t batch,
            int scale_exp, cudaStream_t st)
{
    const T scale = (T)ldexp(1.0, scale_exp);
    if (p.s <= 1)
        return LaunchS<T, 1, BigIsA>(big, small, C, p, batch, scale, st);
    if (p.s <= 2)
        return LaunchS<T, 2, BigIsA>(big, small, C, p, batch, scale, st);
    if (p.s <= 4)
        return LaunchS<T, 4, BigIsA>(big, small, C, p, batch, scale, st);
    if (p.s <= 8)
        return LaunchS<T, 8, BigIsA>(big, small, C, p, batch, scale, st);
    return LaunchS<T, 16, BigIsA>(big, small, C, p, batch, scale, st);
}

} // namespace

bool SkinnyApplies(uint64_t batch, int a_rank, const uint64_t *a_shape, const int32_t *a_perm,
                   int a_batched, int b_rank, const uint64_t *b_shape, const int32_t *b_perm,
                   int b_batched, uint64_t m, uint64_t n, uint64_t k)
{
    SkinnyParams p;
    bool big_is_a;
    return Plan(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape, b_perm, b_batched,
                m, n, k, p, big_is_a);
}

int SkinnyContract(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                   const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                   const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                   uint64_t m, uint64_t n, uint64_t k, int dtype, int scale_exp,
                   cudaStream_t st)
{
    SkinnyParams p;
    bool big_is_a;
    if (!Plan(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape, b_perm, b_batched, m,
              n, k, p, big_is_a))
        return SetError(JETGPU_ERR_UNSUPPORTED, "skinny product planned for an unsupported shape");
    const void *big = big_is_a ? A : B;
    const void *small = big_is_a ? B : A;
    if (dtype == JETGPU_C128)
        return big_is_a ? LaunchT<double, true>(big, small, C, p, batch, scale_exp, st)
                        : LaunchT<double, false>(big, small, C, p, batch, scale_exp, st);
    return big_is_a ? LaunchT<float, true>(big, small, C, p, batch, scale_exp, st)
                    : LaunchT<float, false>(big, small, C, p, batch, scale_exp, st);
}

} // namespace jetgpu
