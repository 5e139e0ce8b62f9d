// Index permutation kernels (Tensor::Transpose / Permuter backends).
//
// Reference algorithm being replaced: QFlexPermuter (permute/QFlex.hpp) splits
// every power-of-2 dimension into binary sub-indices and runs up to three
// out-of-place passes over the whole tensor; DefaultPermuter
// (permute/Default.hpp) walks the old index with an odometer. Both produce
// out[new multi-index] = in[old multi-index].
//
// GB300 design:
//  * Power-of-2 tensors: the permutation is a permutation of the bits of the
//    linear index. One pass. Each CTA owns a tile of 2^u elements spanned by
//    the t lowest input bits, the t lowest output bits and further input bits
//    up to u; the remaining bits enumerate tiles. Loads read runs of 2^t
//    consecutive input elements (512 B per warp, 16-byte vectors), stores
//    write runs of 2^t consecutive output elements; the tile sits in shared
//    memory with an XOR swizzle. All bit-scatter arithmetic is folded into
//    small lookup tables built on the host and passed as __grid_constant__
//    kernel parameters (warp-uniform reads).
//  * Any other shape: a mixed-radix gather (one thread per output element,
//    coalesced stores).
//  * PermuteSplitTf32: the same two kernels with a store stage that writes the
//    tensor-core operand planes (TF32 hi/lo of re/im) directly.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace jetgpu {
namespace {

constexpr int kMaxRank = 64;
constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// Host-side simplification: drop unit axes, merge input axes that stay
// adjacent and in order in the output.
// ---------------------------------------------------------------------------
struct Simplified {
    std::vector<uint64_t> dims; // input dims (row-major)
    std::vector<int> perm;      // output axis j = input axis perm[j]
    uint64_t size = 1;
};

int Simplify(int rank, const uint64_t *shape, const int32_t *perm,
             Simplified &s)
{
    JETGPU_REQUIRE(rank >= 0 && rank <= kMaxRank, "rank out of range");
    std::vector<int> seen(rank, 0);
    for (int j = 0; j < rank; ++j) {
        JETGPU_REQUIRE(perm[j] >= 0 && perm[j] < rank && !seen[perm[j]],
                       "perm is not a permutation of 0..rank-1");
        seen[perm[j]] = 1;
    }
    s.size = 1;
    for (int i = 0; i < rank; ++i) {
        JETGPU_REQUIRE(shape[i] >= 1, "zero-sized dimension");
        s.size *= shape[i];
    }
    // Keep non-unit axes.
    std::vector<int> keep_id(rank, -1);
    std::vector<uint64_t> d;
    for (int i = 0; i < rank; ++i)
        if (shape[i] != 1) {
            keep_id[i] = (int)d.size();
            d.push_back(shape[i]);
        }
    std::vector<int> p;
    for (int j = 0; j < rank; ++j)
        if (keep_id[perm[j]] >= 0)
            p.push_back(keep_id[perm[j]]);
    // Merge runs: output-consecutive axes p[j], p[j+1] with p[j+1] == p[j]+1.
    std::vector<int> group_of(d.size(), -1);
    std::vector<std::vector<int>> groups; // in output order
    for (size_t j = 0; j < p.size(); ++j) {
        if (j > 0 && p[j] == p[j - 1] + 1)
            groups.back().push_back(p[j]);
        else
            groups.push_back({p[j]});
    }
    // Input order of groups = sort by first input axis.
    std::vector<int> order(groups.size());
    for (size_t g = 0; g < groups.size(); ++g)
        order[g] = (int)g;
    std::sort(order.begin(), order.end(),
              [&](int a, int b) { return groups[a][0] < groups[b][0]; });
    std::vector<int> in_pos(groups.size());
    s.dims.clear();
    for (size_t r = 0; r < order.size(); ++r) {
        in_pos[order[r]] = (int)r;
        uint64_t m = 1;
        for (int ax : groups[order[r]])
            m *= d[ax];
        s.dims.push_back(m);
    }
    s.perm.clear();
    for (size_t g = 0; g < groups.size(); ++g)
        s.perm.push_back(in_pos[g]);
    return JETGPU_OK;
}

// ---------------------------------------------------------------------------
// Mixed-radix gather kernel.
// ---------------------------------------------------------------------------
struct GatherParams {
    int rank;
    int narrow;                    // total < 2^32: the 32-bit index path
    uint64_t out_dims[kMaxRank];   // output dims, [rank-1] fastest
    uint64_t in_strides[kMaxRank]; // input element stride of output axis j
    uint64_t size;                 // elements per tensor
    uint64_t total;                // batch * size
    // Division by out_dims[j] (and by size) on the 32-bit path: multiply and
    // shift (Granlund-Montgomery invariant divisors); magic 0 means d = 1.
    uint32_t magic[kMaxRank], shift[kMaxRank];
    uint32_t size_magic, size_shift;
};

// Input offset of output element idx: the mixed-radix walk over the output
// dims, in 32-bit indices with multiply-shift division when the tensor has
// fewer than 2^32 elements, else in 64 bits.
__device__ __forceinline__ uint64_t GatherSrc(const GatherParams &p, uint64_t idx)
{
    if (p.narrow) {
        uint32_t o = (uint32_t)idx;
        const uint32_t b = DivMagic(o, p.size_magic, p.size_shift);
        o -= b * (uint32_t)p.size;
        uint32_t src = b * (uint32_t)p.size;
        for (int j = p.rank - 1; j >= 0; --j) {
            const uint32_t q = DivMagic(o, p.magic[j], p.shift[j]);
            src += (o - q * (uint32_t)p.out_dims[j]) * (uint32_t)p.in_strides[j];
            o = q;
        }
        return src;
    }
    const uint64_t b = idx / p.size;
    uint64_t o = idx - b * p.size;
    uint64_t src = b * p.size;
    for (int j = p.rank - 1; j >= 0; --j) {
        const uint64_t d = p.out_dims[j];
        const uint64_t q = o / d;
        src += (o - q * d) * p.in_strides[j];
        o = q;
    }
    return src;
}

template <typename E>
__global__ void __launch_bounds__(kThreads)
    gather_kernel(const __grid_constant__ GatherParams p,
                  const E *__restrict__ in, E *__restrict__ out)
{
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < p.total;
         idx += (uint64_t)gridDim.x * blockDim.x)
        out[idx] = in[GatherSrc(p, idx)];
}

// TF32 rounding to nearest (ties away from zero) by adding half a unit in the
// last TF32 place and truncating the 13 low mantissa bits.
__device__ __forceinline__ float RoundTf32(float x)
{
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) // inf / nan: keep
        return x;
    return __uint_as_float((u + 0x1000u) & 0xffffe000u);
}

// Two floats to packed BF16 words, round to nearest even (one hardware
// conversion): `lower` in bits 0-15, `upper` in bits 16-31.
__device__ __forceinline__ uint32_t PackBf16x2(float lower, float upper)
{
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(upper), "f"(lower));
    return r;
}

// BF16 hi/lo splits of two values x0, x1, packed as (x0 low half, x1 high
// half): hi = RN_bf16(x), lo = RN_bf16(x - hi); x - hi is exact in FP32.
__device__ __forceinline__ void SplitBf16x2(float x0, float x1, uint32_t &hi, uint32_t &lo)
{
    hi = PackBf16x2(x0, x1);
    lo = PackBf16x2(x0 - __uint_as_float(hi << 16), x1 - __uint_as_float(hi & 0xffff0000u));
}

// Two floats to packed FP16 words, round to nearest even, and back.
__device__ __forceinline__ uint32_t PackF16x2(float lower, float upper)
{
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(upper), "f"(lower));
    return r;
}

__device__ __forceinline__ void UnpackF16x2(uint32_t r, float &lower, float &upper)
{
    asm("{\n\t.reg .b16 l, h;\n\t"
        "mov.b32 {l, h}, %2;\n\t"
        "cvt.f32.f16 %0, l;\n\t"
        "cvt.f32.f16 %1, h;\n\t}"
        : "=f"(lower), "=f"(upper)
        : "r"(r));
}

// FP16 hi/lo splits of two (already scaled) values, packed like SplitBf16x2.
__device__ __forceinline__ void SplitF16x2(float x0, float x1, uint32_t &hi, uint32_t &lo)
{
    hi = PackF16x2(x0, x1);
    float h0, h1;
    UnpackF16x2(hi, h0, h1);
    lo = PackF16x2(x0 - h0, x1 - h1);
}

struct SplitOut {
    void *planes;          // 4 planes, or 6 with an extra pair (see `extra`)
    uint64_t plane_stride; // words between planes
    uint64_t cols;         // logical columns of the permuted view
    uint64_t pitch;        // words per row in a plane
    float scale;           // exact power of two
    int extra;             // planes 4, 5: kSplitNegIm -im_hi, -im_lo;
                           // kSplitSum hi, lo of re + im (the 3M product's sums)
    int bf16;              // 16-bit BF16 words instead of TF32-in-FP32 words
    int fp16;              // 16-bit FP16 words of the operand scaled by its FP16 scale
    const int *e_max_dev;  // FP16: the operand's max exponent (sets the scale)
    int cols_log2;         // log2(cols) when cols is a power of 2 (bit-permutation path)
};

__device__ __forceinline__ float SplitScale(const SplitOut &so)
{
    // With sum planes the FP16 scale is one power of two lower: the operand's
    // largest |re| or |im| lies in [2^13, 2^14), so |re + im| < 2^15 stays
    // below the FP16 maximum 65504.
    return so.fp16 ? Pow2f(Fp16ScaleExp(*so.e_max_dev) - (so.extra == kSplitSum ? 1 : 0))
                   : so.scale;
}

__device__ __forceinline__ void Split16x2(const SplitOut &so, float x0, float x1, uint32_t &hi,
                                          uint32_t &lo)
{
    if (so.fp16)
        SplitF16x2(x0, x1, hi, lo);
    else
        SplitBf16x2(x0, x1, hi, lo);
}

__device__ __forceinline__ void WriteSplit(const SplitOut &so, uint64_t o,
                                           float2 v)
{
    uint64_t row = o / so.cols;
    uint64_t col = o - row * so.cols;
    uint64_t off = row * so.pitch + col;
    const float sc = SplitScale(so);
    float re = v.x * sc, im = v.y * sc;
    if (so.bf16 || so.fp16) {
        uint16_t *pl = static_cast<uint16_t *>(so.planes);
        uint32_t h, l; // (re, im) packed
        Split16x2(so, re, im, h, l);
        pl[off] = (uint16_t)(h & 0xffffu);
        pl[off + so.plane_stride] = (uint16_t)(l & 0xffffu);
        pl[off + 2 * so.plane_stride] = (uint16_t)(h >> 16);
        pl[off + 3 * so.plane_stride] = (uint16_t)(l >> 16);
        if (so.extra == kSplitNegIm) { // -x: the sign bit of each piece flipped
            pl[off + 4 * so.plane_stride] = (uint16_t)((h >> 16) ^ 0x8000u);
            pl[off + 5 * so.plane_stride] = (uint16_t)((l >> 16) ^ 0x8000u);
        }
        if (so.extra == kSplitSum) {
            Split16x2(so, re + im, 0.f, h, l);
            pl[off + 4 * so.plane_stride] = (uint16_t)(h & 0xffffu);
            pl[off + 5 * so.plane_stride] = (uint16_t)(l & 0xffffu);
        }
        return;
    }
    float *planes = static_cast<float *>(so.planes);
    float rh = RoundTf32(re), ih = RoundTf32(im);
    float rl = RoundTf32(re - rh), il = RoundTf32(im - ih);
    planes[off] = rh;
    planes[off + so.plane_stride] = rl;
    planes[off + 2 * so.plane_stride] = ih;
    planes[off + 3 * so.plane_stride] = il;
    if (so.extra == kSplitNegIm) {
        planes[off + 4 * so.plane_stride] = -ih;
        planes[off + 5 * so.plane_stride] = -il;
    }
    else if (so.extra == kSplitSum) {
        const float sm = re + im, sh = RoundTf32(sm);
        planes[off + 4 * so.plane_stride] = sh;
        planes[off + 5 * so.plane_stride] = RoundTf32(sm - sh);
    }
}

__global__ void __launch_bounds__(kThreads)
    gather_split_kernel(const __grid_constant__ GatherParams p,
                        const float2 *__restrict__ in, SplitOut so)
{
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < p.total;
         idx += (uint64_t)gridDim.x * blockDim.x)
        WriteSplit(so, idx, in[GatherSrc(p, idx)]);
}

// ---------------------------------------------------------------------------
// Tiled permute for any dims (the non-power-of-2 path).
//
// A tile is every index combination of a set U of axes: the innermost input
// axes (I) until their extent reaches a threshold, joined with the input
// axes that become the innermost output axes (O), so T = prod_{a in U} dim(a)
// elements (at most kTileMax). The other axes (and the batch) enumerate the
// tiles. A CTA reads its tile in input order, where the I axes vary fastest
// (runs of at least the threshold's contiguous elements), places each element
// at its output-order position in shared memory, and writes the tile in
// output order, where the O axes vary fastest. in_off[e] / out_off[f] are the
// element offsets of tile element e (input order) / f (output order) from the
// tile's bases; pos[e] is e's output-order position. The gather kernel reads
// one scattered element per output element; this reads and writes runs.
// ---------------------------------------------------------------------------
constexpr int kTileMax = 1024;

struct TileParams {
    int nr;          // tile-enumerating axes (batch first)
    int T;           // elements per tile
    int G;           // tiles per pass of a CTA (G * T elements fill at most 32 KB)
    uint32_t t_magic, t_shift; // division by T (DivMagic)
    uint64_t tiles;
    uint64_t r_dims[kMaxRank + 1];
    uint64_t r_in[kMaxRank + 1];  // input element stride of each
    uint64_t r_out[kMaxRank + 1]; // output element stride of each
    uint32_t r_magic[kMaxRank + 1], r_shift[kMaxRank + 1]; // division by r_dims
    int narrow;                   // tiles < 2^32: 32-bit tile decode
    alignas(16) int32_t in_off[kTileMax];
    alignas(16) int32_t out_off[kTileMax];
    alignas(16) uint16_t pos[kTileMax];
};

// Below this many elements (per launch) the gather kernel runs: a small
// permute is bound by its launch, and the tile plan's 12 KB parameter block and
// host-side tables would only add to that.
constexpr uint64_t kTileMinElements = 1ull << 18;
constexpr int kTileGroupMax = kThreads; // tiles per pass (one base per thread)
constexpr int kTileSlotBytes = 32768;    // shared memory for one pass's elements

// Tile bases: tile t decoded over the enumerating axes (last fastest).
__device__ __forceinline__ void TileBases(const TileParams &p, uint64_t t, uint64_t &bi,
                                          uint64_t &bo)
{
    bi = 0;
    bo = 0;
    if (p.narrow) {
        uint32_t x = (uint32_t)t;
        for (int a = p.nr - 1; a >= 0; --a) {
            const uint32_t q = DivMagic(x, p.r_magic[a], p.r_shift[a]);
            const uint64_t c = x - q * (uint32_t)p.r_dims[a];
            bi += c * p.r_in[a];
            bo += c * p.r_out[a];
            x = q;
        }
        return;
    }
    for (int a = p.nr - 1; a >= 0; --a) {
        const uint64_t d = p.r_dims[a];
        const uint64_t q = t / d;
        const uint64_t c = t - q * d;
        bi += c * p.r_in[a];
        bo += c * p.r_out[a];
        t = q;
    }
}

template <typename E> struct TilePlainStore {
    E *out;
    __device__ __forceinline__ void operator()(uint64_t o, const E &v) const { out[o] = v; }
};

struct TileSplitStore {
    SplitOut so;
    __device__ __forceinline__ void operator()(uint64_t o, const uint2 &v) const
    {
        WriteSplit(so, o, make_float2(__uint_as_float(v.x), __uint_as_float(v.y)));
    }
};

// Asynchronous copy of one element from global to shared memory: a thread
// issues all its loads of a pass without holding them in registers.
template <typename E> __device__ __forceinline__ void CopyAsync(E *dst, const E *src)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(E) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

// Each pass moves G consecutive tiles (G * T elements, up to 32 KB) through
// shared memory: slot u holds element u mod T of the pass's tile u / T.
template <typename E, typename Store>
__global__ void __launch_bounds__(kThreads)
    tile_permute_kernel(const __grid_constant__ TileParams p, const E *__restrict__ in, Store store)
{
    __shared__ E tile[kTileSlotBytes / sizeof(E)];
    __shared__ uint64_t base_in[kTileGroupMax], base_out[kTileGroupMax];
    // The offset tables move to shared memory once, in 16-byte words: indexed
    // per thread, a kernel-parameter array serialises every warp's load, so
    // the tile loops read them from shared memory instead.
    __shared__ alignas(16) int32_t in_off[kTileMax];
    __shared__ alignas(16) int32_t out_off[kTileMax];
    __shared__ alignas(16) uint16_t pos[kTileMax];
    {
        const int n4 = (p.T + 3) / 4, n8 = (p.T + 7) / 8; // within the 1024-entry arrays
        const int4 *src_in = reinterpret_cast<const int4 *>(p.in_off);
        const int4 *src_out = reinterpret_cast<const int4 *>(p.out_off);
        const int4 *src_pos = reinterpret_cast<const int4 *>(p.pos);
        for (int i = threadIdx.x; i < n4; i += blockDim.x) {
            reinterpret_cast<int4 *>(in_off)[i] = src_in[i];
            reinterpret_cast<int4 *>(out_off)[i] = src_out[i];
        }
        for (int i = threadIdx.x; i < n8; i += blockDim.x)
            reinterpret_cast<int4 *>(pos)[i] = src_pos[i];
    }
    const uint64_t passes = (p.tiles + p.G - 1) / p.G;
    for (uint64_t ps = blockIdx.x; ps < passes; ps += gridDim.x) {
        const uint64_t t0 = ps * p.G;
        const int g = (int)min((uint64_t)p.G, p.tiles - t0);
        if ((int)threadIdx.x < g)
            TileBases(p, t0 + threadIdx.x, base_in[threadIdx.x], base_out[threadIdx.x]);
        __syncthreads();
        // Tiles of at least two thread sweeps go one tile at a time (no
        // division per element; measured 4-5 % faster on 3^16, 3^18, 5^11);
        // smaller tiles (81, 243 elements) share the sweeps across tiles.
        const bool per_tile = p.T >= 2 * kThreads;
        const int n = g * p.T;
        if (per_tile) {
            for (int j = 0; j < g; ++j) {
                const E *src = in + base_in[j];
                E *dst = tile + j * p.T;
                for (int e = threadIdx.x; e < p.T; e += blockDim.x)
                    CopyAsync(&dst[pos[e]], src + in_off[e]);
            }
        } else {
#pragma unroll 4
            for (int u = threadIdx.x; u < n; u += blockDim.x) {
                const int j = (int)DivMagic((uint32_t)u, p.t_magic, p.t_shift);
                const int e = u - j * p.T;
                CopyAsync(&tile[j * p.T + pos[e]], in + base_in[j] + (uint64_t)in_off[e]);
            }
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        __syncthreads();
        if (per_tile) {
            for (int j = 0; j < g; ++j) {
                const uint64_t bo = base_out[j];
                const E *src = tile + j * p.T;
                for (int f = threadIdx.x; f < p.T; f += blockDim.x)
                    store(bo + (uint64_t)out_off[f], src[f]);
            }
        } else {
#pragma unroll 4
            for (int u = threadIdx.x; u < n; u += blockDim.x) {
                const int j = (int)DivMagic((uint32_t)u, p.t_magic, p.t_shift);
                const int f = u - j * p.T;
                store(base_out[j] + (uint64_t)out_off[f], tile[u]);
            }
        }
        __syncthreads();
    }
}

// The tile plan of a simplified permutation (false: no tile of at most
// kTileMax elements, or offsets past 32 bits; the gather kernel then runs).
bool BuildTile(const Simplified &s, uint64_t batch, size_t elem_bytes, TileParams &p)
{
    const int r = (int)s.dims.size();
    if (r < 2)
        return false;
    std::vector<uint64_t> in_stride(r, 1);
    for (int i = r - 2; i >= 0; --i)
        in_stride[i] = in_stride[i + 1] * s.dims[i + 1];
    std::vector<uint64_t> out_stride(r); // output stride of input axis a
    {
        uint64_t st = 1;
        for (int j = r - 1; j >= 0; --j) {
            out_stride[s.perm[j]] = st;
            st *= s.dims[s.perm[j]];
        }
    }
    for (uint64_t thr : {32ull, 16ull, 8ull}) {
        std::vector<char> in_u(r, 0);
        uint64_t pi = 1;
        for (int a = r - 1; a >= 0 && pi < thr; --a) {
            in_u[a] = 1;
            pi *= s.dims[a];
        }
        uint64_t po = 1;
        for (int j = r - 1; j >= 0 && po < thr; --j) {
            in_u[s.perm[j]] = 1;
            po *= s.dims[s.perm[j]];
        }
        uint64_t T = 1;
        for (int a = 0; a < r; ++a)
            if (in_u[a])
                T *= s.dims[a];
        if (T > (uint64_t)kTileMax)
            continue;
        std::vector<int> u_in, u_out;
        for (int a = 0; a < r; ++a)
            if (in_u[a])
                u_in.push_back(a);
        for (int j = 0; j < r; ++j)
            if (in_u[s.perm[j]])
                u_out.push_back(s.perm[j]);
        std::vector<uint64_t> fstride(r, 0);
        {
            uint64_t st = 1;
            for (int i = (int)u_out.size() - 1; i >= 0; --i) {
                fstride[u_out[i]] = st;
                st *= s.dims[u_out[i]];
            }
        }
        std::memset(&p, 0, sizeof(p));
        p.T = (int)T;
        std::vector<uint64_t> c(r, 0);
        for (uint64_t e = 0; e < T; ++e) {
            uint64_t x = e, io = 0, oo = 0, f = 0;
            for (int i = (int)u_in.size() - 1; i >= 0; --i) {
                const int a = u_in[i];
                const uint64_t ca = x % s.dims[a];
                x /= s.dims[a];
                io += ca * in_stride[a];
                oo += ca * out_stride[a];
                f += ca * fstride[a];
            }
            if (io > 0x7fffffffull || oo > 0x7fffffffull)
                return false;
            p.in_off[e] = (int32_t)io;
            p.pos[e] = (uint16_t)f;
            p.out_off[f] = (int32_t)oo;
        }
        int nr = 0;
        if (batch > 1) {
            p.r_dims[nr] = batch;
            p.r_in[nr] = s.size;
            p.r_out[nr] = s.size;
            ++nr;
        }
        // Tiles are enumerated in output order (the axis with the smallest
        // output stride fastest): consecutive tiles then write neighbouring
        // output runs, which complete each other's partially written sectors
        // while they are still in L2. In input order the runs of a sector
        // were written far apart in time; measured on random permutations,
        // 3^18 complex64 went from 3.1 to 4.8 TB/s.
        std::vector<int> rest;
        for (int a = 0; a < r; ++a)
            if (!in_u[a])
                rest.push_back(a);
        std::stable_sort(rest.begin(), rest.end(),
                         [&](int x, int y) { return out_stride[x] > out_stride[y]; });
        for (int a : rest) {
            p.r_dims[nr] = s.dims[a];
            p.r_in[nr] = in_stride[a];
            p.r_out[nr] = out_stride[a];
            ++nr;
        }
        p.nr = nr;
        p.tiles = (s.size / T) * batch;
        p.narrow = p.tiles < (1ull << 32) ? 1 : 0;
        for (int a = 0; a < nr; ++a)
            Magic32(p.r_dims[a], p.r_magic[a], p.r_shift[a]);
        p.G = (int)std::min<uint64_t>(
            {(uint64_t)kTileSlotBytes / elem_bytes / T, (uint64_t)kTileGroupMax, p.tiles});
        Magic32(T, p.t_magic, p.t_shift);
        return true;
    }
    return false;
}

// The permutation with unit axes dropped and no axes merged. Merging shortens
// the rank, but a merged axis can be too long for a tile on both sides (e.g.
// 81 innermost in the input, 729 innermost in the output); the original axes
// then still give one. `perm` must already have passed Simplify's checks.
void Unmerged(int rank, const uint64_t *shape, const int32_t *perm, Simplified &u)
{
    std::vector<int> keep_id(rank, -1);
    u.dims.clear();
    u.perm.clear();
    u.size = 1;
    for (int i = 0; i < rank; ++i)
        if (shape[i] != 1) {
            keep_id[i] = (int)u.dims.size();
            u.dims.push_back(shape[i]);
            u.size *= shape[i];
        }
    for (int j = 0; j < rank; ++j)
        if (keep_id[perm[j]] >= 0)
            u.perm.push_back(keep_id[perm[j]]);
}

// A tile plan for the simplified permutation `s` of (rank, shape, perm):
// first on the merged axes, then on the original ones.
bool PlanTile(const Simplified &s, int rank, const uint64_t *shape, const int32_t *perm,
              uint64_t batch, size_t elem_bytes, TileParams &p)
{
    if (BuildTile(s, batch, elem_bytes, p))
        return true;
    Simplified u;
    Unmerged(rank, shape, perm, u);
    return u.dims.size() > s.dims.size() && BuildTile(u, batch, elem_bytes, p);
}

template <typename E, typename Store>
int LaunchTile(const TileParams &p, const void *in, Store store, cudaStream_t stream)
{
    const unsigned grid = GridFor((p.tiles + p.G - 1) / p.G, 4);
    tile_permute_kernel<E, Store><<<grid, kThreads, 0, stream>>>(p, (const E *)in, store);
    return CheckLaunch("tile_permute_kernel");
}

// Multiplier and shift for dividing 32-bit values by d (d = 1: magic 0):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, s = l - 1.
void BuildGather(const Simplified &s, uint64_t batch, GatherParams &p)
{
    int r = (int)s.dims.size();
    std::vector<uint64_t> in_stride(r, 1);
    for (int i = r - 2; i >= 0; --i)
        in_stride[i] = in_stride[i + 1] * s.dims[i + 1];
    std::memset(&p, 0, sizeof(p));
    p.rank = r;
    for (int j = 0; j < r; ++j) {
        p.out_dims[j] = s.dims[s.perm[j]];
        p.in_strides[j] = in_stride[s.perm[j]];
    }
    p.size = s.size;
    p.total = s.size * batch;
    p.narrow = p.total < (1ull << 32) ? 1 : 0;
    if (p.narrow) {
        for (int j = 0; j < r; ++j)
            Magic32(p.out_dims[j], p.magic[j], p.shift[j]);
        Magic32(p.size, p.size_magic, p.size_shift);
    }
}

// ---------------------------------------------------------------------------
// Bit-permutation tiled kernel (power-of-2 tensors).
// ---------------------------------------------------------------------------
constexpr int kTileTables = 3; // 3 x 8 outer bits

struct BitParams {
    int n;       // bits of the linear index
    int u;       // tile bits
    int t;       // run bits (t lowest input / output bits)
    int n_outer; // n - u
    uint64_t total_tiles;
    uint64_t in_hi[64];  // input offset of run h (h = L >> t)
    uint64_t out_hi[64]; // output offset of run h (h = M >> t)
    uint32_t l_lo[64];   // tile-local input index of M & (2^t - 1)
    uint32_t l_hi[64];   // tile-local input index of (M >> t) << t
    uint64_t tile_in[kTileTables][256];
    uint64_t tile_out[kTileTables][256];
};

__device__ __forceinline__ uint32_t Swz(uint32_t h, int log_ve)
{
    return ((h ^ (h >> 5)) & 31u) << log_ve;
}

__device__ __forceinline__ uint64_t TileBase(const uint64_t (*tbl)[256],
                                             uint64_t tt)
{
    return tbl[0][tt & 255] + tbl[1][(tt >> 8) & 255] +
           tbl[2][(tt >> 16) & 255];
}

// Store stage functor: plain element copy.
template <typename E> struct PlainStore {
    E *out;
    __device__ __forceinline__ void operator()(uint64_t off, const E *v,
                                               int ve) const
    {
        if (sizeof(E) == 8) {
            uint4 w;
            const uint2 *a = reinterpret_cast<const uint2 *>(v);
            w.x = a[0].x;
            w.y = a[0].y;
            w.z = a[1].x;
            w.w = a[1].y;
            *reinterpret_cast<uint4 *>(out + off) = w;
        }
        else {
            *reinterpret_cast<uint4 *>(out + off) =
                *reinterpret_cast<const uint4 *>(v);
        }
    }
};

// Store stage functor: hi/lo planes (complex64 only, 2 elements).
struct SplitStore {
    SplitOut so;
    __device__ __forceinline__ void operator()(uint64_t off, const uint2 *v,
                                               int) const
    {
        // off is even and cols >= 2 is a power of 2: both elements share a row
        // (shift and mask: a 64-bit division here made the kernel
        // instruction bound).
        uint64_t row = off >> so.cols_log2;
        uint64_t col = off & (so.cols - 1);
        uint64_t base = row * so.pitch + col;
        float2 a = make_float2(__uint_as_float(v[0].x), __uint_as_float(v[0].y));
        float2 b = make_float2(__uint_as_float(v[1].x), __uint_as_float(v[1].y));
        const float sc = SplitScale(so);
        float ar = a.x * sc, ai = a.y * sc;
        float br = b.x * sc, bi = b.y * sc;
        if (so.bf16 || so.fp16) {
            // Two 16-bit words per plane: one 4-byte store (base is even).
            uint16_t *pl = static_cast<uint16_t *>(so.planes);
            uint32_t rh, rl, ih, il; // (element a, element b) packed per plane
            Split16x2(so, ar, br, rh, rl);
            Split16x2(so, ai, bi, ih, il);
            *reinterpret_cast<uint32_t *>(pl + base) = rh;
            *reinterpret_cast<uint32_t *>(pl + base + so.plane_stride) = rl;
            *reinterpret_cast<uint32_t *>(pl + base + 2 * so.plane_stride) = ih;
            *reinterpret_cast<uint32_t *>(pl + base + 3 * so.plane_stride) = il;
            if (so.extra == kSplitNegIm) { // -x: the sign bit of each piece flipped
                *reinterpret_cast<uint32_t *>(pl + base + 4 * so.plane_stride) = ih ^ 0x80008000u;
                *reinterpret_cast<uint32_t *>(pl + base + 5 * so.plane_stride) = il ^ 0x80008000u;
            }
            if (so.extra == kSplitSum) {
                uint32_t sh, sl;
                Split16x2(so, ar + ai, br + bi, sh, sl);
                *reinterpret_cast<uint32_t *>(pl + base + 4 * so.plane_stride) = sh;
                *reinterpret_cast<uint32_t *>(pl + base + 5 * so.plane_stride) = sl;
            }
            return;
        }
        float *planes = static_cast<float *>(so.planes);
        float arh = RoundTf32(ar), aih = RoundTf32(ai);
        float brh = RoundTf32(br), bih = RoundTf32(bi);
        float2 rh = make_float2(arh, brh);
        float2 rl = make_float2(RoundTf32(ar - arh), RoundTf32(br - brh));
        float2 ih = make_float2(aih, bih);
        float2 il = make_float2(RoundTf32(ai - aih), RoundTf32(bi - bih));
        *reinterpret_cast<float2 *>(planes + base) = rh;
        *reinterpret_cast<float2 *>(planes + base + so.plane_stride) = rl;
        *reinterpret_cast<float2 *>(planes + base + 2 * so.plane_stride) = ih;
        *reinterpret_cast<float2 *>(planes + base + 3 * so.plane_stride) = il;
        if (so.extra == kSplitNegIm) {
            *reinterpret_cast<float2 *>(planes + base + 4 * so.plane_stride) =
                make_float2(-ih.x, -ih.y);
            *reinterpret_cast<float2 *>(planes + base + 5 * so.plane_stride) =
                make_float2(-il.x, -il.y);
        }
        else if (so.extra == kSplitSum) {
            const float sa = ar + ai, sb = br + bi;
            const float sah = RoundTf32(sa), sbh = RoundTf32(sb);
            *reinterpret_cast<float2 *>(planes + base + 4 * so.plane_stride) =
                make_float2(sah, sbh);
            *reinterpret_cast<float2 *>(planes + base + 5 * so.plane_stride) =
                make_float2(RoundTf32(sa - sah), RoundTf32(sb - sbh));
        }
    }
};

// E: element (uint2 = complex64, uint4 = complex128); LOG_VE: log2 of
// elements per 16-byte vector.
template <typename E, int LOG_VE, typename Store>
__global__ void __launch_bounds__(kThreads)
    bitperm_kernel(const __grid_constant__ BitParams p,
                   const E *__restrict__ in, Store store)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    E *tile = reinterpret_cast<E *>(smem_raw);
    constexpr int VE = 1 << LOG_VE;
    const int t = p.t;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int runs = 1 << (p.u - t);
    const uint64_t outer_mask = (1ull << p.n_outer) - 1;

    uint32_t llo[VE];
#pragma unroll
    for (int e = 0; e < VE; ++e)
        llo[e] = p.l_lo[lane * VE + e];

    for (uint64_t g = blockIdx.x; g < p.total_tiles; g += gridDim.x) {
        const uint64_t b = g >> p.n_outer;
        const uint64_t tt = g & outer_mask;
        const uint64_t in_base = (b << p.n) + TileBase(p.tile_in, tt);
        const uint64_t out_base = (b << p.n) + TileBase(p.tile_out, tt);

        // Load: run h covers tile-local input indices [h << t, (h+1) << t).
        for (int h = warp; h < runs; h += nwarps) {
            const uint64_t off = in_base + p.in_hi[h] + (uint64_t)(lane * VE);
            uint4 v = __ldg(reinterpret_cast<const uint4 *>(in + off));
            const uint32_t L = ((uint32_t)h << t) | (uint32_t)(lane * VE);
            const uint32_t phys = L ^ Swz((uint32_t)h, LOG_VE);
            *reinterpret_cast<uint4 *>(tile + phys) = v;
        }
        __syncthreads();
        // Store: run h covers tile-local output indices [h << t, (h+1) << t).
        for (int h = warp; h < runs; h += nwarps) {
            const uint32_t lhi = p.l_hi[h];
            E vals[VE];
#pragma unroll
            for (int e = 0; e < VE; ++e) {
                const uint32_t L = llo[e] | lhi;
                vals[e] = tile[L ^ Swz(L >> t, LOG_VE)];
            }
            store(out_base + p.out_hi[h] + (uint64_t)(lane * VE), vals, VE);
        }
        __syncthreads();
    }
}

// Builds the bit-permutation tables. Returns false when the tensor does not
// suit the tiled kernel (too small, or too many outer bits).
bool BuildBitParams(const Simplified &s, uint64_t batch, int log_ve,
                    BitParams &p)
{
    const int r = (int)s.dims.size();
    int n = 0;
    std::vector<int> logd(r);
    for (int i = 0; i < r; ++i) {
        if (!IsPow2(s.dims[i]))
            return false;
        logd[i] = Log2(s.dims[i]);
        n += logd[i];
    }
    const int t = 5 + log_ve;
    const int umax = log_ve == 1 ? 12 : 11; // 32 KB tile
    if (n < umax || n - umax > 8 * kTileTables)
        return false;
    // Input bit offsets of each input axis (axis r-1 is fastest).
    std::vector<int> in_off(r), out_off(r), out_axis_of_in(r);
    for (int i = r - 1, o = 0; i >= 0; --i) {
        in_off[i] = o;
        o += logd[i];
    }
    for (int j = 0; j < r; ++j)
        out_axis_of_in[s.perm[j]] = j;
    for (int j = r - 1, o = 0; j >= 0; --j) {
        out_off[j] = o;
        o += logd[s.perm[j]];
    }
    std::vector<int> dst(n), src(n);
    for (int i = 0; i < r; ++i)
        for (int q = 0; q < logd[i]; ++q) {
            int ib = in_off[i] + q;
            int ob = out_off[out_axis_of_in[i]] + q;
            dst[ib] = ob;
            src[ob] = ib;
        }
    // Tile bit set U (input positions).
    std::vector<char> inU(n, 0);
    int u = 0;
    for (int b = 0; b < t; ++b)
        if (!inU[b]) {
            inU[b] = 1;
            ++u;
        }
    for (int j = 0; j < t; ++j)
        if (!inU[src[j]]) {
            inU[src[j]] = 1;
            ++u;
        }
    for (int b = 0; b < n && u < umax; ++b)
        if (!inU[b]) {
            inU[b] = 1;
            ++u;
        }
    std::vector<int> Us, Vs;
    for (int b = 0; b < n; ++b)
        (inU[b] ? Us : Vs).push_back(b);
    // Output positions of U, sorted.
    std::vector<int> Os;
    for (int b : Us)
        Os.push_back(dst[b]);
    std::sort(Os.begin(), Os.end());
    std::vector<int> pos_in_Us(n, -1);
    for (size_t i = 0; i < Us.size(); ++i)
        pos_in_Us[Us[i]] = (int)i;

    std::memset(&p, 0, sizeof(p));
    p.n = n;
    p.u = u;
    p.t = t;
    p.n_outer = n - u;
    p.total_tiles = batch << (n - u);
    const int hb = u - t; // bits of a run index
    for (int h = 0; h < (1 << hb); ++h) {
        uint64_t vin = 0, vout = 0;
        uint32_t lh = 0;
        for (int j = 0; j < hb; ++j)
            if ((h >> j) & 1) {
                vin |= 1ull << Us[t + j];
                vout |= 1ull << Os[t + j];
                lh |= 1u << pos_in_Us[src[Os[t + j]]];
            }
        p.in_hi[h] = vin;
        p.out_hi[h] = vout;
        p.l_hi[h] = lh;
    }
    for (int m = 0; m < (1 << t); ++m) {
        uint32_t l = 0;
        for (int j = 0; j < t; ++j)
            if ((m >> j) & 1)
                l |= 1u << pos_in_Us[src[Os[j]]];
        p.l_lo[m] = l;
    }
    const int nv = (int)Vs.size();
    for (int k = 0; k < kTileTables; ++k)
        for (int v = 0; v < 256; ++v) {
            uint64_t ti = 0, to = 0;
            for (int j = 0; j < 8; ++j) {
                int bit = 8 * k + j;
                if (bit < nv && ((v >> j) & 1)) {
                    ti |= 1ull << Vs[bit];
                    to |= 1ull << dst[Vs[bit]];
                }
            }
            p.tile_in[k][v] = ti;
            p.tile_out[k][v] = to;
        }
    return true;
}

template <typename E, int LOG_VE, typename Store>
int LaunchBitperm(const BitParams &p, const void *in, Store store,
                  cudaStream_t stream)
{
    const size_t smem = (sizeof(E) << p.u);
    auto kern = bitperm_kernel<E, LOG_VE, Store>;
    static thread_local bool configured = false;
    if (!configured) {
        JETGPU_CUDA_TRY(cudaFuncSetAttribute(
            kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
        configured = true;
    }
    unsigned grid = GridFor(p.total_tiles, 6);
    kern<<<grid, kThreads, smem, stream>>>(p, reinterpret_cast<const E *>(in),
                                           store);
    return CheckLaunch("bitperm_kernel");
}

} // namespace

int PermuteImpl(const void *in, void *out, uint64_t batch, int rank,
                const uint64_t *shape, const int32_t *perm, int dtype,
                cudaStream_t stream)
{
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    Simplified s;
    int rc = Simplify(rank, shape, perm, s);
    if (rc)
        return rc;
    if (batch == 0 || s.size == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in != nullptr && out != nullptr, "null data pointer");
    const size_t eb = ElemBytes(dtype);
    bool identity = true;
    for (size_t j = 0; j < s.perm.size(); ++j)
        identity = identity && (s.perm[j] == (int)j);
    if (identity) {
        JETGPU_CUDA_TRY(cudaMemcpyAsync(out, in, s.size * batch * eb,
                                        cudaMemcpyDeviceToDevice, stream));
        return JETGPU_OK;
    }
    const bool aligned = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0);
    if (aligned) {
        static thread_local BitParams bp; // ~14 KB: keep off the stack
        if (dtype == JETGPU_C64 && BuildBitParams(s, batch, 1, bp))
            return LaunchBitperm<uint2, 1>(bp, in,
                                           PlainStore<uint2>{(uint2 *)out},
                                           stream);
        if (dtype == JETGPU_C128 && BuildBitParams(s, batch, 0, bp))
            return LaunchBitperm<uint4, 0>(bp, in,
                                           PlainStore<uint4>{(uint4 *)out},
                                           stream);
    }
    {
        static thread_local TileParams tp; // ~12 KB: keep off the stack
        if (s.size * batch >= kTileMinElements && (uintptr_t)in % eb == 0 &&
            PlanTile(s, rank, shape, perm, batch, eb, tp))
            return dtype == JETGPU_C64
                       ? LaunchTile<uint2>(tp, in, TilePlainStore<uint2>{(uint2 *)out}, stream)
                       : LaunchTile<uint4>(tp, in, TilePlainStore<uint4>{(uint4 *)out}, stream);
    }
    GatherParams gp;
    BuildGather(s, batch, gp);
    unsigned grid = GridFor((gp.total + kThreads - 1) / kThreads, 8);
    if (dtype == JETGPU_C64)
        gather_kernel<uint2><<<grid, kThreads, 0, stream>>>(
            gp, (const uint2 *)in, (uint2 *)out);
    else
        gather_kernel<uint4><<<grid, kThreads, 0, stream>>>(
            gp, (const uint4 *)in, (uint4 *)out);
    return CheckLaunch("gather_kernel");
}

int PermuteSplitTf32(const void *in, float *planes, int rank,
                     const uint64_t *shape, const int32_t *perm, uint64_t rows,
                     uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                     int scale_exp, cudaStream_t stream)
{
    return PermuteSplitTf32Batched(in, planes, 1, rank, shape, perm, rows, cols, pitch,
                                   plane_stride, scale_exp, stream);
}

int PermuteSplitTf32Batched(const void *in, float *planes, uint64_t batch, int rank,
                            const uint64_t *shape, const int32_t *perm, uint64_t rows,
                            uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                            int scale_exp, cudaStream_t stream, int neg_im)
{
    return PermuteSplitPlanes(in, planes, batch, rank, shape, perm, rows, cols, pitch,
                              plane_stride, scale_exp, SplitFormat::kTf32,
                              neg_im ? kSplitNegIm : kSplitNone, stream);
}

int PermuteSplitPlanes(const void *in, void *planes, uint64_t batch, int rank,
                       const uint64_t *shape, const int32_t *perm, uint64_t rows, uint64_t cols,
                       uint64_t pitch, uint64_t plane_stride, int scale_exp, SplitFormat fmt,
                       int extra, cudaStream_t stream, const int *e_max_dev)
{
    JETGPU_REQUIRE(extra == kSplitNone || extra == kSplitNegIm || extra == kSplitSum,
                   "unknown extra plane pair");
    JETGPU_REQUIRE(fmt != SplitFormat::kFp16 || e_max_dev != nullptr,
                   "FP16 planes need the operand's max exponent");
    Simplified s;
    int rc = Simplify(rank, shape, perm, s);
    if (rc)
        return rc;
    JETGPU_REQUIRE(rows * cols == s.size, "split view does not match size");
    JETGPU_REQUIRE(batch >= 1, "empty batch");
    // Tensor b occupies rows [b * rows, (b + 1) * rows): the batch folds into
    // the row index of the split view.
    rows *= batch;
    JETGPU_REQUIRE(scale_exp >= -126 && scale_exp <= 127, "scale out of range");
    SplitOut so;
    so.planes = planes;
    so.plane_stride = plane_stride;
    so.cols = cols;
    so.pitch = pitch;
    so.scale = ldexpf(1.0f, scale_exp);
    so.extra = extra;
    so.bf16 = fmt == SplitFormat::kBf16 ? 1 : 0;
    so.fp16 = fmt == SplitFormat::kFp16 ? 1 : 0;
    so.e_max_dev = e_max_dev;
    so.cols_log2 = IsPow2(cols) ? Log2(cols) : -1;
    const bool aligned = ((uintptr_t)in % 16 == 0) && ((uintptr_t)planes % 16 == 0) &&
                         (pitch % 2 == 0) && (plane_stride % 2 == 0);
    static thread_local BitParams bp;
    if (aligned && IsPow2(cols) && cols >= 2 && BuildBitParams(s, batch, 1, bp))
        return LaunchBitperm<uint2, 1>(bp, in, SplitStore{so}, stream);
    {
        static thread_local TileParams tp;
        if (s.size * batch >= kTileMinElements && (uintptr_t)in % 8 == 0 &&
            PlanTile(s, rank, shape, perm, batch, 8, tp))
            return LaunchTile<uint2>(tp, in, TileSplitStore{so}, stream);
    }
    GatherParams gp;
    BuildGather(s, batch, gp);
    unsigned grid = GridFor((gp.total + kThreads - 1) / kThreads, 8);
    gather_split_kernel<<<grid, kThreads, 0, stream>>>(gp, (const float2 *)in,
                                                       so);
    return CheckLaunch("gather_split_kernel");
}

} // namespace jetgpu

extern "C" {

int jetgpu_permute(const void *in, void *out, int rank, const uint64_t *shape,
                   const int32_t *perm, int dtype, void *stream)
{
    jetgpu::NvtxRange range("jetgpu_permute");
    jetgpu::ClearError();
    return jetgpu::PermuteImpl(in, out, 1, rank, shape, perm, dtype,
                               jetgpu::AsStream(stream));
}

int jetgpu_permute_batched(const void *in, void *out, uint64_t batch, int rank,
                           const uint64_t *shape, const int32_t *perm,
                           int dtype, void *stream)
{
    jetgpu::NvtxRange range("jetgpu_permute_batched");
    jetgpu::ClearError();
    return jetgpu::PermuteImpl(in, out, batch, rank, shape, perm, dtype,
                               jetgpu::AsStream(stream));
}

} // extern "C"
