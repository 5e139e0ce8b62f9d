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
#include <utility>

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
    int vec;       // complex64 rows of C stored 16 bytes at a time (s = S even)
    uint32_t s_magic, s_shift; // division by s (DivMagic)
    SkAxes row;    // large operand: free axes
    uint32_t row_magic[kSkAxes], row_shift[kSkAxes];
    SkAxes big_b, small_b;                // batch axes of the two operands
    uint64_t out_row, out_col, out_batch; // C's element strides
    // Offsets tabulated on the host: the large operand's per contracted
    // index c, the small operand's per c and per free index j.
    uint64_t coff[kSkMaxK];
    uint32_t s_coff[kSkMaxK], s_foff[kSkMaxS];
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

// AxesOffset for an index below 2^32 (table entries, batch items): 32-bit
// digit arithmetic.
__device__ __forceinline__ uint64_t SmallOffset(const SkAxes &a, uint32_t idx)
{
    uint64_t off = 0;
#pragma unroll
    for (int i = 0; i < kSkAxes; ++i)
        if (i < a.n) {
            const uint32_t d = (uint32_t)a.dim[i];
            const uint32_t q = idx / d;
            off += (uint64_t)(idx - q * d) * a.stride[i];
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

// Rows of the large operand one thread carries at once (more loads in
// flight for narrow products; each table value read from shared memory
// serves R rows). FP64 products are FMA-bound on this GPU: fewer.
template <typename T, int S> struct SkRows {
    static constexpr int R = sizeof(T) == 8 ? (S <= 4 ? 2 : 1) : (S <= 4 ? 4 : 2);
    // CTAs per SM the register allocation must leave room for, for the
    // HBM-bound complex64 widths: four up to S = 4 (2-qubit gates on 2^27
    // elements 5.7 -> 6.1 TB/s), three for S = 8 (at four it spills and loses
    // 7 %; at two it lost 25 %).
    static constexpr int kMinBlocks =
        sizeof(T) != 4 ? 1 : S <= 4 ? 4 : S <= 8 ? 3 : 1;
};

// One CTA per (row range, batch item); each thread R rows of the large
// operand at a time, `step` apart, so that every row's loads and stores are
// coalesced across the warp. S: the small extent, or the next width the
// kernel is built for (table columns j >= s are zero and not stored).
// BigIsA: the large operand is A (C's rows), else B (C's columns); the
// operands keep their roles in Mac.
template <typename T, int S, bool BigIsA>
__global__ void __launch_bounds__(kSkThreads, SkRows<T, S>::kMinBlocks)
    skinny_kernel(const typename C2<T>::type *__restrict__ big,
                  const typename C2<T>::type *__restrict__ small,
                  typename C2<T>::type *__restrict__ C, const __grid_constant__ SkinnyParams p,
                  T scale)
{
    using V = typename C2<T>::type;
    constexpr int R = SkRows<T, S>::R;
    constexpr int KC = 8 / R; // contracted values loaded per row at once
    // Complex64 rows of 9 outputs (qutrit pairs) leave through shared memory:
    // each warp's 32 rows of C are one contiguous run, written 16 bytes a
    // lane, where direct 8-byte stores 72 bytes apart cost four times the
    // store requests (measured: 3,233 -> 3,870 GB/s on 3^17). For 3, 4 and 8
    // outputs the stage's registers and shared memory cost more occupancy
    // than it saves (measured slower). Row stride in the stage odd (in 8-byte
    // words): conflict-free writes.
    constexpr bool kStage = std::is_same<T, float>::value && BigIsA && S == 9;
    __shared__ __align__(16) V tab[kSkMaxK][S];
    __shared__ V stage[kStage ? kSkThreads / 32 : 1][kStage ? 32 * (S + 1) : 1];
    // Launched with programmatic stream serialisation (LaunchPdl): every
    // memory access follows this wait for the previous kernel of the stream,
    // and the next kernel may start launching once every CTA is past it.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t b = blockIdx.y;
    big += SmallOffset(p.big_b, b);
    small += SmallOffset(p.small_b, b);
    C += (uint64_t)b * p.out_batch;
    for (int e = threadIdx.x; e < p.k * S; e += blockDim.x) {
        const int c = e / S, j = e % S;
        tab[c][j] = j < p.s ? small[p.s_coff[c] + p.s_foff[j]] : V{0, 0};
    }
    __syncthreads();

    // The loop runs per warp (its first row wb), so that all 32 lanes stay in
    // it together for the staged stores; lanes past the end only skip work.
    const int lane = threadIdx.x & 31;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t wb = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x - lane); wb < p.rows;
         wb += step * R) {
        const uint64_t r0 = wb + lane;
        const V *x[R];
        bool ok[R];
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const uint64_t r = r0 + i * step;
            ok[i] = r < p.rows;
            x[i] = big + (ok[i] ? RowOffset(p, r) : 0);
        }
        V acc[R][S];
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < S; ++j)
                acc[i][j] = V{0, 0};
        for (int c0 = 0; c0 < p.k; c0 += KC) {
            V v[R][KC];
#pragma unroll
            for (int u = 0; u < KC; ++u) {
                const bool in = c0 + u < p.k;
                const uint64_t o = in ? p.coff[c0 + u] : 0;
#pragma unroll
                for (int i = 0; i < R; ++i)
                    v[i][u] = (in && ok[i]) ? __ldg(x[i] + o) : V{0, 0};
            }
#pragma unroll
            for (int u = 0; u < KC; ++u) {
                if (c0 + u >= p.k)
                    break;
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    const V t = tab[c0 + u][j];
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        if (BigIsA)
                            Mac(acc[i][j], v[i][u], t);
                        else
                            Mac(acc[i][j], t, v[i][u]);
                    }
                }
            }
        }
        if constexpr (kStage) {
            V *w = stage[threadIdx.x >> 5];
            const int ws = p.s | 1;
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const uint64_t rw = wb + i * step; // the warp's first row
                if (rw >= p.rows)
                    continue;
                const int nv = (int)min((uint64_t)32, p.rows - rw);
                __syncwarp();
#pragma unroll
                for (int j = 0; j < S; ++j)
                    if (j < p.s)
                        w[lane * ws + j] = V{acc[i][j].x * scale, acc[i][j].y * scale};
                __syncwarp();
                V *dst = C + rw * p.out_row;
                const uint32_t tot = (uint32_t)(nv * p.s);
                if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
                    for (uint32_t q = lane; q < tot / 2; q += 32) {
                        const uint32_t e = 2 * q;
                        const uint32_t r = DivMagic(e, p.s_magic, p.s_shift);
                        const uint32_t c = e - r * p.s;
                        const V lo = w[r * ws + c];
                        const V hi = c + 1 < (uint32_t)p.s ? w[r * ws + c + 1] : w[(r + 1) * ws];
                        reinterpret_cast<float4 *>(dst)[q] = make_float4(lo.x, lo.y, hi.x, hi.y);
                    }
                    if ((tot & 1) && lane == 0) {
                        const uint32_t r = DivMagic(tot - 1, p.s_magic, p.s_shift);
                        dst[tot - 1] = w[r * ws + (tot - 1 - r * p.s)];
                    }
                } else {
                    for (uint32_t e = lane; e < tot; e += 32) {
                        const uint32_t r = DivMagic(e, p.s_magic, p.s_shift);
                        dst[e] = w[r * ws + (e - r * p.s)];
                    }
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < R; ++i) {
                if (!ok[i])
                    continue;
                V *out = C + (r0 + i * step) * p.out_row;
                if constexpr (std::is_same<T, float>::value && BigIsA && S % 2 == 0) {
                    if (p.vec) {
                        float4 *o4 = reinterpret_cast<float4 *>(out);
#pragma unroll
                        for (int j = 0; j < S; j += 2)
                            o4[j / 2] =
                                make_float4(acc[i][j].x * scale, acc[i][j].y * scale,
                                            acc[i][j + 1].x * scale, acc[i][j + 1].y * scale);
                        continue;
                    }
                }
#pragma unroll
                for (int j = 0; j < S; ++j)
                    if (j < p.s)
                        out[j * p.out_col] = V{acc[i][j].x * scale, acc[i][j].y * scale};
            }
        }
    }
}

// Small outputs (rows x s at most kSkTiny, a step of a few gates): one
// thread per output element reads its row's k values and the small operand's
// k values straight from global memory, all loads issued before any
// arithmetic, no shared memory and no barrier: one memory round trip, where
// skinny_kernel's table and rows take two. Same FMA sequence.
constexpr int kSkTiny = 4096;

template <typename T, bool BigIsA>
__global__ void __launch_bounds__(kSkThreads)
    skinny_tiny_kernel(const typename C2<T>::type *__restrict__ big,
                       const typename C2<T>::type *__restrict__ small,
                       typename C2<T>::type *__restrict__ C,
                       const __grid_constant__ SkinnyParams p, T scale)
{
    using V = typename C2<T>::type;
    // Launched with programmatic stream serialisation: the launch may begin
    // while the previous kernel of the stream finishes; every memory access
    // here follows this wait for it (a no-op when launched plainly).
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // The next tiny step may start launching now (it waits for this one).
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t b = blockIdx.y;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (uint32_t)p.rows * (uint32_t)p.s)
        return;
    const uint32_t r = DivMagic(e, p.s_magic, p.s_shift);
    const uint32_t j = e - r * (uint32_t)p.s;
    const V *x = big + SmallOffset(p.big_b, b) + RowOffset(p, r);
    const V *y = small + SmallOffset(p.small_b, b) + p.s_foff[j];
    V acc{0, 0};
    for (int c0 = 0; c0 < p.k; c0 += 8) {
        V xv[8], yv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const bool in = c0 + u < p.k;
            xv[u] = in ? __ldg(x + p.coff[c0 + u]) : V{0, 0};
            yv[u] = in ? __ldg(y + p.s_coff[c0 + u]) : V{0, 0};
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (c0 + u >= p.k)
                break;
            if (BigIsA)
                Mac(acc, xv[u], yv[u]);
            else
                Mac(acc, yv[u], xv[u]);
        }
    }
    C[(uint64_t)b * p.out_batch + r * p.out_row + j * p.out_col] =
        V{acc.x * scale, acc.y * scale};
}

struct Ax {
    uint64_t d, s; // dimension, element stride
};

// Axes of one index group, outermost first (at most the 64 axes of a tensor;
// on the stack: planning runs several times per contraction).
struct AxList {
    int n = 0;
    Ax a[65];
    void push(Ax x) { a[n++] = x; }
};

// Packs axes given outermost first, dropping unit axes and merging neighbours
// that are contiguous (outer stride = inner stride x inner dim).
bool Pack(const AxList &outer_first, SkAxes &out)
{
    AxList m;
    for (int i = 0; i < outer_first.n; ++i) {
        const Ax &a = outer_first.a[i];
        if (a.d == 1)
            continue;
        if (m.n > 0 && m.a[m.n - 1].s == a.s * a.d) {
            m.a[m.n - 1].d *= a.d;
            m.a[m.n - 1].s = a.s;
        } else {
            m.push(a);
        }
    }
    if (m.n > kSkAxes)
        return false;
    out.n = m.n;
    for (int i = 0; i < out.n; ++i) {
        out.dim[i] = m.a[out.n - 1 - i].d;
        out.stride[i] = m.a[out.n - 1 - i].s;
    }
    return true;
}

// Appends the axes perm[j], perm[j + 1], ... whose dimensions multiply to
// `extent` (false if no run of them does).
bool Take(int rank, const uint64_t *shape, const int32_t *perm, const uint64_t *st, int &j,
          uint64_t extent, AxList &out)
{
    uint64_t p = 1;
    while (p < extent && j < rank) {
        out.push({shape[perm[j]], st[perm[j]]});
        p *= shape[perm[j]];
        ++j;
    }
    return p == extent;
}

struct OperandAxes {
    AxList batch, first, second;
};

// An operand's permutation as (batch axes) (first group) (second group) with
// the groups' extents e1, e2. mode 0: shared; 1: `batch` tensors back to
// back; 2: one tensor whose permutation leads with the batch axes.
bool SplitOperand(int rank, const uint64_t *shape, const int32_t *perm, int mode,
                  uint64_t batch, uint64_t e1, uint64_t e2, OperandAxes &o)
{
    if (rank < 0 || rank > 64)
        return false;
    uint64_t st[64];
    if (rank > 0)
        st[rank - 1] = 1;
    for (int i = rank - 2; i >= 0; --i)
        st[i] = st[i + 1] * shape[i + 1];
    const uint64_t size = rank ? st[0] * shape[0] : 1;
    int j = 0;
    if (mode == 2 && !Take(rank, shape, perm, st, j, batch, o.batch))
        return false;
    if (mode == 1)
        o.batch.push({batch, size});
    return Take(rank, shape, perm, st, j, e1, o.first) &&
           Take(rank, shape, perm, st, j, e2, o.second);
}

// The kernel parameters of a skinny contraction (false: not one). `tables`:
// also tabulate the offsets (needed for a launch, not to decide).
bool Plan(uint64_t batch, int a_rank, const uint64_t *a_shape, const int32_t *a_perm,
          int a_batched, int b_rank, const uint64_t *b_shape, const int32_t *b_perm,
          int b_batched, uint64_t m, uint64_t n, uint64_t k, SkinnyParams &p, bool &big_is_a,
          bool tables = true)
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
    const bool ok = big_is_a ? (Pack(a.first, p.row) && Pack(a.batch, p.big_b) &&
                                Pack(b.batch, p.small_b))
                             : (Pack(b.second, p.row) && Pack(b.batch, p.big_b) &&
                                Pack(a.batch, p.small_b));
    if (!ok)
        return false;
    // The contracted and small free offsets, digit by digit (innermost axis
    // fastest), k + k + s entries.
    auto tabulate = [](const AxList &axes, uint64_t count, auto *out) {
        for (uint64_t idx = 0; idx < count; ++idx) {
            uint64_t x = idx, off = 0;
            for (int i = axes.n - 1; i >= 0; --i) {
                off += (x % axes.a[i].d) * axes.a[i].s;
                x /= axes.a[i].d;
            }
            out[idx] = static_cast<std::remove_pointer_t<decltype(out)>>(off);
        }
    };
    const AxList &sc = big_is_a ? b.first : a.second;
    const AxList &sf = big_is_a ? b.second : a.first;
    uint64_t small_size = 1; // elements of one small operand
    for (int i = 0; i < sc.n; ++i)
        small_size += (sc.a[i].d - 1) * sc.a[i].s;
    for (int i = 0; i < sf.n; ++i)
        small_size += (sf.a[i].d - 1) * sf.a[i].s;
    if (small_size > 0xffffffffull)
        return false;
    if (!tables)
        return true;
    tabulate(big_is_a ? a.second : b.first, k, p.coff);
    tabulate(sc, k, p.s_coff);
    tabulate(sf, s, p.s_foff);
    p.narrow = p.rows < (1ull << 32) ? 1 : 0;
    if (p.narrow)
        for (int i = 0; i < p.row.n; ++i)
            Magic32(p.row.dim[i], p.row_magic[i], p.row_shift[i]);
    Magic32((uint64_t)p.s, p.s_magic, p.s_shift);
    p.out_row = big_is_a ? n : 1;
    p.out_col = big_is_a ? 1 : n;
    p.out_batch = m * n;
    return true;
}

// Launches `kernel` with programmatic stream serialisation: the launch may
// begin while the previous kernel of the stream finishes, which a chain of
// small steps is bound by (the kernels wait for it before touching memory).
template <typename... P, typename... A>
cudaError_t LaunchPdl(void (*kernel)(P...), dim3 grid, cudaStream_t st, A &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kSkThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
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
    p.vec = (std::is_same<T, float>::value && BigIsA && S % 2 == 0 && p.s == S &&
             (reinterpret_cast<uintptr_t>(C) & 15) == 0)
                ? 1
                : 0;
    const uint64_t slots = (uint64_t)Resident<T, S, BigIsA>() * SmCount();
    uint64_t gx = (p.rows + kSkThreads - 1) / kSkThreads;
    const uint64_t per_item = slots / batch > 0 ? slots / batch : 1;
    if (gx > per_item)
        gx = per_item;
    JETGPU_CUDA_TRY(LaunchPdl(kernel, dim3((unsigned)gx, (unsigned)batch), st,
                              static_cast<const V *>(big), static_cast<const V *>(small),
                              static_cast<V *>(C), p, scale));
    return CheckLaunch("skinny_kernel");
}

template <typename T, bool BigIsA>
int LaunchT(const void *big, const void *small, void *C, SkinnyParams &p, uint64_t batch,
            int scale_exp, cudaStream_t st)
{
    const T scale = (T)ldexp(1.0, scale_exp);
    if (p.rows * (uint64_t)p.s <= (uint64_t)kSkTiny) {
        using V = typename C2<T>::type;
        const unsigned gx = (unsigned)((p.rows * p.s + kSkThreads - 1) / kSkThreads);
        JETGPU_CUDA_TRY(LaunchPdl(skinny_tiny_kernel<T, BigIsA>, dim3(gx, (unsigned)batch), st,
                                  static_cast<const V *>(big), static_cast<const V *>(small),
                                  static_cast<V *>(C), p, scale));
        return CheckLaunch("skinny_tiny_kernel");
    }
    switch (p.s) {
    case 1:
        return LaunchS<T, 1, BigIsA>(big, small, C, p, batch, scale, st);
    case 2:
        return LaunchS<T, 2, BigIsA>(big, small, C, p, batch, scale, st);
    case 3:
        return LaunchS<T, 3, BigIsA>(big, small, C, p, batch, scale, st);
    case 4:
        return LaunchS<T, 4, BigIsA>(big, small, C, p, batch, scale, st);
    case 9:
        return LaunchS<T, 9, BigIsA>(big, small, C, p, batch, scale, st);
    default:
        break;
    }
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
                m, n, k, p, big_is_a, false);
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
