// Tensor-core complex product in split precision (3xTF32 or 3xBF16), sm_103a.
//
// Replaces the cgemm of TensorHelpers::MultiplyTensorData
// (include/jet/TensorHelpers.hpp:47-61, 147-152) for large steps.
//
// Operands arrive as planar hi/lo splits written by PermuteSplitPlanes:
//   A: planes {Ar_hi, Ar_lo, Ai_hi, Ai_lo}, each M x K (K contiguous)
//   B: planes {Br_hi, Br_lo, Bi_hi, Bi_lo}, each N x K (K contiguous)
// and the complex product uses four real products ("4M"), each as three
// tensor-core products (hi*hi + hi*lo + lo*hi) accumulated in FP32 in TMEM:
//   Cr += Ar Br - Ai Bi,   Ci += Ar Bi + Ai Br.
// TF32 planes (FP32 words with 13 zero mantissa bits) leave a relative
// truncation of about 2^-22 per product; BF16 planes (16-bit words, twice the
// tensor rate and half the bytes) about 2^-17.
//
// One CTA computes a 128 x 128 complex tile. Warp 0 lane 0 feeds a 3-stage
// ring of shared-memory stages with TMA (8 boxes of 128 rows x 64 bytes,
// 64-byte swizzle); warp 1 lane 0 issues tcgen05.mma (M=128, N=128, 32 bytes
// of K per instruction: K=8 kind::tf32 or K=16 kind::f16) into one of two
// TMEM accumulator sets (Cr, Ci: 2 x 256 columns) and releases stages with
// tcgen05.commit; eight accumulator warps fold each finished K chunk into
// FP32 registers (see the kernel comment) and write C.
// The 3M ("Gauss") form uses three real products instead of four:
//   P1 = Ar Br,  P2 = Ai Bi,  P3 = (Ar + Ai)(Br + Bi),
//   Cr = P1 - P2,  Ci = P3 - P1 - P2,
// each again as hi*hi + hi*lo + lo*hi, on six planes per operand (the split
// also writes hi/lo of re + im). 9 tensor-core products per K step instead
// of 12; Ci's error grows with |P3| ~ 2|A||B| (see the kernel comment).
// Every mbarrier wait is bounded: on timeout the kernel records
// JETGPU_ERR_TIMEOUT in a device status word, skips the remaining work,
// frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include "common.cuh"

namespace jetgpu {

__device__ int g_tc_status = 0;

namespace {

constexpr int kBM = 128;
constexpr int kBN = 128;
constexpr int kTmemCols = 512;                // two (Cr, Ci) accumulator sets
constexpr int kAccWarps = 8;                  // accumulator warps
constexpr int kStoreBytes = 32 * 128;         // per accumulator warp: a 32 x 16 complex C block
constexpr int kThreads = 32 * (2 + kAccWarps); // + TMA and MMA warps
constexpr int kGroupM = 8;                    // default tile rows per group of the tile order
constexpr int kTileRing = 4;                  // tile indices in flight between the warp roles

// Every stage holds boxes of 128 rows x RowBytes (swizzled by RowBytes);
// every MMA consumes 32 bytes of K per row. Main-loop variants:
//  0 TF32 narrow: 64-byte rows (16 k), 3 stages of 4 A + 4 B plane boxes;
//                 12 MMAs of N = 128 per k step.
//  1 TF32 wide:   64-byte rows, 2 stages of 4 A boxes and two B triples
//                 [-Bi, Br, Bi] (hi, lo); 6 MMAs of N = 256 per k step:
//                 Ar [Br; Bi] -> [ArBr | ArBi] and Ai [-Bi; Br] ->
//                 [-AiBi | AiBr] land on (Cr | Ci) in one instruction each.
//  2 BF16 narrow: variant 0 on BF16 planes (kind::f16, 32 k per stage).
//  4 FP16 narrow: variant 2 on FP16 planes of power-of-two scaled operands.
//  3 BF16 deep:   32-byte rows (16 k, 32-byte swizzle), 6 stages of 32 KB:
//                 the same shared memory as variant 2 in twice as many,
//                 half-size stages.
// A chunk is the K extent accumulated in TMEM before the FP32 fold, in
// stages (a kernel argument; see the kernel comment).
//  8, 9 BF16 / FP16 wide: variant 1's N = 256 main loop on 16-bit planes
//                 (two stages of 4 A + 6 B boxes of 32 k; the B triples of
//                 variant 1 with the negated imaginary planes).
//  5, 6, 7 3M:    TF32 / BF16 / FP16 planes, 64-byte rows, 2 stages of six A
//                 plane boxes (re, im, re + im; hi, lo) and six B boxes;
//                 9 MMAs of N = 128 per k step, each product into its own
//                 TMEM slot (see the kernel comment).
template <int V> struct TcCfg;
// Operand formats: 0 TF32 (kind::tf32), 1 BF16, 2 FP16 (both kind::f16).
constexpr int kFmtTf32 = 0, kFmtBf16 = 1, kFmtFp16 = 2;
template <> struct TcCfg<0> {
    static constexpr bool Wide = false, ThreeM = false;
    static constexpr int Fmt = kFmtTf32, Stages = 3, Tiles = 8, RowBytes = 64;
};
template <> struct TcCfg<1> {
    static constexpr bool Wide = true, ThreeM = false;
    static constexpr int Fmt = kFmtTf32, Stages = 2, Tiles = 10, RowBytes = 64;
};
template <> struct TcCfg<2> {
    static constexpr bool Wide = false, ThreeM = false;
    static constexpr int Fmt = kFmtBf16, Stages = 3, Tiles = 8, RowBytes = 64;
};
template <> struct TcCfg<3> {
    static constexpr bool Wide = false, ThreeM = false;
    static constexpr int Fmt = kFmtBf16, Stages = 6, Tiles = 8, RowBytes = 32;
};
template <> struct TcCfg<4> {
    static constexpr bool Wide = false, ThreeM = false;
    static constexpr int Fmt = kFmtFp16, Stages = 3, Tiles = 8, RowBytes = 64;
};
template <> struct TcCfg<8> {
    static constexpr bool Wide = true, ThreeM = false;
    static constexpr int Fmt = kFmtBf16, Stages = 2, Tiles = 10, RowBytes = 64;
};
template <> struct TcCfg<9> {
    static constexpr bool Wide = true, ThreeM = false;
    static constexpr int Fmt = kFmtFp16, Stages = 2, Tiles = 10, RowBytes = 64;
};
template <> struct TcCfg<5> {
    static constexpr bool Wide = false, ThreeM = true;
    static constexpr int Fmt = kFmtTf32, Stages = 2, Tiles = 12, RowBytes = 64;
};
template <> struct TcCfg<6> {
    static constexpr bool Wide = false, ThreeM = true;
    static constexpr int Fmt = kFmtBf16, Stages = 2, Tiles = 12, RowBytes = 64;
};
template <> struct TcCfg<7> {
    static constexpr bool Wide = false, ThreeM = true;
    static constexpr int Fmt = kFmtFp16, Stages = 2, Tiles = 12, RowBytes = 64;
};
template <int V> constexpr int TileBytes() { return kBM * TcCfg<V>::RowBytes; }
template <int V> constexpr int ElemBytes() { return TcCfg<V>::Fmt == kFmtTf32 ? 4 : 2; }
template <int V> constexpr int BlockK() { return TcCfg<V>::RowBytes / ElemBytes<V>(); }
template <int V> constexpr int StageBytes() { return TcCfg<V>::Tiles * TileBytes<V>(); }

// Default K depth accumulated in TMEM per chunk. TF32: 16, one fold per
// stage. The tensor core's accumulation rounds magnitudes toward zero, so its
// error does not average out along a network: measured on a 53-qubit sliced
// circuit amplitude (AUTO form), depth 16 / 32 / 64 / 128 gave relative
// errors 7.0e-6 / 1.0e-5 / 1.2e-5 / 1.9e-5 against FP64, at 1.10 / 1.04 /
// 1.01 / 1.00 times the depth-128 product time. BF16: 128, since its split
// truncation (about 4.5e-6 per product) dominates any accumulation error.
// FP16: 32, one stage (the same number of accumulations per chunk as TF32 at
// 16: two MMA k steps).
constexpr int kDefaultChunkKTf32 = 16;
constexpr int kDefaultChunkKBf16 = 128;
constexpr int kDefaultChunkKFp16 = 32;
// K depth per TMEM chunk (jetgpu_set_tc_chunk_depth; 0 = default). Process-wide,
// read at every launch: atomic so a setter on one thread never tears a read.
std::atomic<int> g_tc_chunk_k{0};

inline int ChunkStages(int fmt, int stage_k)
{
    const int set = g_tc_chunk_k.load(std::memory_order_relaxed);
    int depth = set > 0 ? set
                        : fmt == kFmtBf16 ? kDefaultChunkKBf16
                                          : fmt == kFmtFp16 ? kDefaultChunkKFp16
                                                            : kDefaultChunkKTf32;
    int stages = depth / stage_k;
    return stages < 1 ? 1 : stages;
}
constexpr unsigned long long kWaitNs = 4000000000ull; // 4 s bound per wait

__device__ __forceinline__ uint32_t SmemAddr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t GlobalTimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void MbarInit(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void MbarArriveExpectTx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool MbarTryWait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}

// Bounded wait for the phase of parity `parity`: gives up after limit_ns of
// %globaltimer or max_iters polls, whichever comes first, records
// JETGPU_ERR_TIMEOUT in the device status word and returns false.
__device__ __forceinline__ bool MbarWaitFor(uint32_t bar, uint32_t parity,
                                            unsigned long long limit_ns, uint32_t max_iters)
{
    if (MbarTryWait(bar, parity))
        return true;
    const uint64_t t0 = GlobalTimer();
    for (uint32_t i = 1;; ++i) {
        if (MbarTryWait(bar, parity))
            return true;
        if (i >= max_iters || ((i & 255u) == 0 && GlobalTimer() - t0 > limit_ns)) {
            atomicExch(&g_tc_status, JETGPU_ERR_TIMEOUT);
            return false;
        }
    }
}

__device__ __forceinline__ bool MbarWait(uint32_t bar, uint32_t parity)
{
    return MbarWaitFor(bar, parity, kWaitNs, 0xffffffffu);
}

__device__ __forceinline__ void TmaLoad3d(uint32_t dst, const CUtensorMap *map,
                                          int c0, int c1, int c2, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::"
                 "complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2),
                 "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void TmaLoad4d(uint32_t dst, const CUtensorMap *map,
                                          int c0, int c1, int c2, int c3, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::"
                 "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
                 "r"(bar)
                 : "memory");
}

// Shared-memory matrix descriptor: K-major operand, rows of kRow bytes
// swizzled over kRow bytes (layout code 4 = 64-byte, 6 = 32-byte swizzle),
// 8-row groups 8 * kRow bytes apart.
template <int kRow> __device__ __forceinline__ uint64_t SmemDesc(uint32_t addr)
{
    static_assert(kRow == 64 || kRow == 32, "64- or 32-byte rows");
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);                 // start address
    d |= (uint64_t)1 << 16;                                  // leading byte offset (unused)
    d |= (uint64_t)((8 * kRow) >> 4) << 32;                  // stride byte offset
    d |= (uint64_t)1 << 46;                                  // descriptor version
    d |= (uint64_t)(kRow == 64 ? 4 : 6) << 61;               // swizzle mode
    return d;
}

// Instruction descriptor: D = F32, both operands K-major, M x N; operand
// format code 2 = TF32 (kind::tf32), 1 = BF16, 0 = FP16 (kind::f16). A and B
// share it.
__host__ __device__ constexpr uint32_t InstrDesc(int m, int n, bool neg_a, int fmt)
{
    const uint32_t code = fmt == kFmtTf32 ? 2u : fmt == kFmtBf16 ? 1u : 0u;
    return (1u << 4) | (code << 7) | (code << 10) | ((neg_a ? 1u : 0u) << 13) |
           ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

template <bool kHalf>
__device__ __forceinline__ void Mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                    uint32_t accumulate)
{
    if constexpr (kHalf)
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "setp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                         d_tmem),
                     "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                     : "memory");
    else
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "setp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                         d_tmem),
                     "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                     : "memory");
}

__device__ __forceinline__ void MmaCommit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     bar)
                 : "memory");
}

__device__ __forceinline__ void FenceBeforeSync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void FenceAfterSync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void TmemLoad16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
                   "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
                   "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i)
        v[i] = __uint_as_float(r[i]);
}

// (a0, a1) += (b0, b1) with one packed instruction; each lane is an IEEE
// round-to-nearest FP32 add, so the result equals two scalar adds.
__device__ __forceinline__ void AddF32x2(float &a0, float &a1, float b0, float b1)
{
    asm("{\n\t.reg .b64 pa, pb;\n\t"
        "mov.b64 pa, {%0, %1};\n\t"
        "mov.b64 pb, {%2, %3};\n\t"
        "add.rn.f32x2 pa, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pa;\n\t}"
        : "+f"(a0), "+f"(a1)
        : "f"(b0), "f"(b1));
}

__device__ __forceinline__ void TmemWaitLoad()
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Warp roles: warp 0 issues TMA loads, warp 1 allocates TMEM and issues the
// MMAs, warps 2..9 ("accumulator warps") drain finished K chunks from TMEM.
// Precision: the tensor core's FP32 accumulation in TMEM loses accuracy with
// every MMA it adds (measured: the output-relative error of a 3xTF32 product
// grows with the K depth accumulated in TMEM, 5e-7 at 16 and 1.9e-6 at 128,
// independent of cancellation), so the MMAs accumulate only `chunk_stages`
// stages into one of two TMEM accumulator sets; the accumulator warps add
// every finished chunk into FP32 registers (round-to-nearest) while the next
// chunk accumulates in the other set. Accumulator warp w (w = 2..9) owns TMEM lanes 32*(w%4)..+31
// (tile rows) and columns [64*h, 64*h + 64) of Cr and Ci, h = (w - 2) / 4.
// Register budget: the ten warps spread over the SM's four register-file
// partitions (16K registers each) three to a partition at most, so a thread
// gets at most 168 registers (a few bytes of the epilogue spill).
// 3M variants: three accumulators (P1, P2, P3) of 128 columns do not fit
// twice in the 512 TMEM columns, so the products rotate through four
// 128-column slots instead: product q = 3 g + p (stage g, product p) goes to
// slot q mod 4, and the MMA warp waits for that slot's previous product to be
// folded (two products' MMA time later) before reusing it. The chunk is one
// stage; the fold adds P1 to Cr and subtracts it from Ci, subtracts P2 from
// both and adds P3 to Ci. The error of Ci grows with |P3| ~ 2 |A| |B|, about
// twice the 4M form's; Cr's is the 4M form's.
template <int V>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_split_kernel(const __grid_constant__ CUtensorMap tmA,
                          const __grid_constant__ CUtensorMap tmB,
                          float2 *__restrict__ C, int M, int N, int ktiles, int batch,
                          float scale, int a_batched, int b_batched, int chunk_stages,
                          const int *__restrict__ scale_exps, int group_m,
                          unsigned int *__restrict__ tile_counter, int *__restrict__ out_emax)
{
    using Cfg = TcCfg<V>;
    constexpr bool kWide = Cfg::Wide;
    constexpr bool kThreeM = Cfg::ThreeM;
    constexpr int kAPlanes = kThreeM ? 6 : 4;
    constexpr int kFmt = Cfg::Fmt;
    constexpr bool kHalf = kFmt != kFmtTf32;
    constexpr int kBK = BlockK<V>();
    constexpr int kStages = Cfg::Stages;
    constexpr int kStageBytes = StageBytes<V>();
    constexpr int kTileBytes = TileBytes<V>();
    constexpr int kRowBytes = Cfg::RowBytes;
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kStages];
    __shared__ __align__(8) uint64_t empty_bar[kStages];
    __shared__ __align__(8) uint64_t acc_full[4];  // 4M: two sets; 3M: four slots
    __shared__ __align__(8) uint64_t acc_empty[4];
    __shared__ __align__(8) uint64_t tile_full[kTileRing];
    __shared__ __align__(8) uint64_t tile_empty[kTileRing];
    __shared__ int tile_ring[kTileRing];
    __shared__ uint32_t tmem_slot;

    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    // Persistent: the batch's tiles laid end to end are handed out in order,
    // by an atomic counter when the launch has one (tile_counter, zeroed
    // before the launch), else CTA c takes tiles c, c + G, c + 2G, ...
    // (G = gridDim.x). The producer warp draws each tile and passes its index
    // to the MMA and accumulator warps through a ring in shared memory
    // (tile_full / tile_empty); an index past the end stops them. Drawing
    // from a counter keeps the tiles in flight a compact window of the order
    // however the CTAs' speeds drift apart. Within one product the order is
    // grouped: consecutive tiles walk group_m tile rows down one tile column
    // before moving to the next column, so the tiles in flight at one time
    // cover a compact block of C (about 8 x 19 tiles on 152 SMs) and share
    // their A and B tiles through L2 instead of each tile row streaming all
    // of B from HBM. The stage ring and the two TMEM accumulator sets run on
    // across tiles, so one tile's epilogue overlaps the next tile's loads and
    // MMAs. Batch b of a batched operand is read through a 4-D map (k, row,
    // batch, plane), a shared one through a 3-D map (k, row, plane).
    const int n_tiles = (N + kBN - 1) / kBN;
    const int m_tiles = (M + kBM - 1) / kBM;
    const int tiles_per_product = m_tiles * n_tiles;
    const int span = group_m * n_tiles;
    const int total_tiles = tiles_per_product * batch;
    auto tile_at = [&](int t, int &bz, int &m0, int &n0) {
        bz = t / tiles_per_product;
        const int u = t - bz * tiles_per_product;
        const int group = u / span;
        const int first_m = group * group_m;
        const int gm = min(group_m, m_tiles - first_m);
        const int in_group = u - group * span;
        m0 = (first_m + in_group % gm) * kBM;
        n0 = (in_group / gm) * kBN;
    };
    const int nchunks = (ktiles + chunk_stages - 1) / chunk_stages;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            MbarInit(SmemAddr(&full_bar[s]), 1);
            MbarInit(SmemAddr(&empty_bar[s]), 1);
        }
        for (int b = 0; b < 4; ++b) {
            MbarInit(SmemAddr(&acc_full[b]), 1);
            MbarInit(SmemAddr(&acc_empty[b]), kAccWarps);
        }
        for (int r = 0; r < kTileRing; ++r) {
            MbarInit(SmemAddr(&tile_full[r]), 1);
            MbarInit(SmemAddr(&tile_empty[r]), 1 + kAccWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         SmemAddr(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    FenceBeforeSync();
    __syncthreads();
    FenceAfterSync();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // Tile scheduler and TMA producer.
            bool ok = true;
            for (int i = 0; ok; ++i) {
            const int r = i % kTileRing;
            if (!MbarWait(SmemAddr(&tile_empty[r]), ((uint32_t)(i / kTileRing) & 1u) ^ 1u))
                break;
            int t = tile_counter ? (int)atomicAdd(tile_counter, 1u)
                                 : (int)blockIdx.x + i * (int)gridDim.x;
            t = min(t, total_tiles);
            tile_ring[r] = t;
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                             SmemAddr(&tile_full[r]))
                         : "memory");
            if (t >= total_tiles)
                break;
            int bz, m0, n0;
            tile_at(t, bz, m0, n0);
            for (int kt = 0; kt < ktiles; ++kt) {
                const long long g = (long long)i * ktiles + kt; // stage-ring position
                const int s = (int)(g % kStages);
                const uint32_t phase = (uint32_t)(g / kStages) & 1u;
                if (!MbarWait(SmemAddr(&empty_bar[s]), phase ^ 1u)) {
                    ok = false;
                    break;
                }
                const uint32_t fb = SmemAddr(&full_bar[s]);
                MbarArriveExpectTx(fb, kStageBytes);
                const uint32_t base = SmemAddr(smem + s * kStageBytes);
                const int k0 = kt * kBK;
#pragma unroll
                for (int p = 0; p < kAPlanes; ++p) {
                    if (a_batched)
                        TmaLoad4d(base + p * kTileBytes, &tmA, k0, m0, bz, p, fb);
                    else
                        TmaLoad3d(base + p * kTileBytes, &tmA, k0, m0, p, fb);
                }
                // B tiles: narrow {Br_hi, Br_lo, Bi_hi, Bi_lo}; wide
                // {-Bi_hi, Br_hi, Bi_hi, -Bi_lo, Br_lo, Bi_lo} (plane numbers
                // 0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo, 4 -im_hi, 5 -im_lo);
                // 3M {Br_hi, Br_lo, Bi_hi, Bi_lo, Bs_hi, Bs_lo} (4, 5: re + im).
                constexpr int kBTiles = Cfg::Tiles - kAPlanes;
#pragma unroll
                for (int t = 0; t < kBTiles; ++t) {
                    const int plane = kWide ? (t == 0 ? 4 : t == 1 ? 0 : t == 2 ? 2
                                               : t == 3 ? 5 : t == 4 ? 1 : 3)
                                            : t;
                    if (b_batched)
                        TmaLoad4d(base + (kAPlanes + t) * kTileBytes, &tmB, k0, n0, bz, plane,
                                  fb);
                    else
                        TmaLoad3d(base + (kAPlanes + t) * kTileBytes, &tmB, k0, n0, plane, fb);
                }
            }
            }
        }
        __syncwarp();
    }
    else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer.
            constexpr uint32_t kIdesc = InstrDesc(kBM, kBN, false, kFmt);
            constexpr uint32_t kIdescNeg = InstrDesc(kBM, kBN, true, kFmt);
            bool ok = true;
            for (int i = 0; ok; ++i) {
            const int r = i % kTileRing;
            if (!MbarWait(SmemAddr(&tile_full[r]), (uint32_t)(i / kTileRing) & 1u))
                break;
            const int t = tile_ring[r];
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                             SmemAddr(&tile_empty[r]))
                         : "memory");
            if (t >= total_tiles)
                break;
            if constexpr (kThreeM) {
            for (int kt = 0; kt < ktiles && ok; ++kt) {
                const long long g = (long long)i * ktiles + kt;
                const int s = (int)(g % kStages);
                const uint32_t phase = (uint32_t)(g / kStages) & 1u;
                if (!MbarWait(SmemAddr(&full_bar[s]), phase)) {
                    ok = false;
                    break;
                }
                FenceAfterSync();
                const uint32_t base = SmemAddr(smem + s * kStageBytes);
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    // Product p of stage g into slot q mod 4, free once the
                    // product four back has been folded.
                    const long long q = 3 * g + p;
                    const int slot = (int)(q & 3);
                    if (!MbarWait(SmemAddr(&acc_empty[slot]), ((uint32_t)(q >> 2) & 1u) ^ 1u)) {
                        ok = false;
                        break;
                    }
                    FenceAfterSync();
                    const uint32_t d = tmem + slot * kBN;
#pragma unroll
                    for (int kk = 0; kk < kRowBytes / 32; ++kk) {
                        const uint32_t koff = kk * 32; // 32 bytes of K per MMA
                        // Planes 2p (hi), 2p + 1 (lo) of A (tiles 0..5) and B (6..11).
                        const uint64_t ah = SmemDesc<kRowBytes>(base + (2 * p) * kTileBytes + koff);
                        const uint64_t al =
                            SmemDesc<kRowBytes>(base + (2 * p + 1) * kTileBytes + koff);
                        const uint64_t bh =
                            SmemDesc<kRowBytes>(base + (6 + 2 * p) * kTileBytes + koff);
                        const uint64_t bl =
                            SmemDesc<kRowBytes>(base + (7 + 2 * p) * kTileBytes + koff);
                        Mma<kHalf>(d, ah, bh, kIdesc, kk == 0 ? 0u : 1u);
                        Mma<kHalf>(d, ah, bl, kIdesc, 1u);
                        Mma<kHalf>(d, al, bh, kIdesc, 1u);
                    }
                    MmaCommit(SmemAddr(&acc_full[slot]));
                }
                MmaCommit(SmemAddr(&empty_bar[s]));
            }
            }
            else
            for (int kt = 0; kt < ktiles && ok; ++kt) {
                const int chunk = kt / chunk_stages;
                // Accumulator set: chunks alternate across tiles too.
                const long long gc = (long long)i * nchunks + chunk;
                const int buf = (int)(gc & 1);
                const int in_chunk = kt - chunk * chunk_stages;
                const bool chunk_start = in_chunk == 0;
                const bool chunk_end = in_chunk == chunk_stages - 1 || kt == ktiles - 1;
                if (chunk_start &&
                    !MbarWait(SmemAddr(&acc_empty[buf]), ((uint32_t)(gc >> 1) & 1u) ^ 1u)) {
                    ok = false;
                    break;
                }
                const long long g = (long long)i * ktiles + kt;
                const int s = (int)(g % kStages);
                const uint32_t phase = (uint32_t)(g / kStages) & 1u;
                if (!MbarWait(SmemAddr(&full_bar[s]), phase)) {
                    ok = false;
                    break;
                }
                FenceAfterSync();
                const uint32_t d_re = tmem + buf * 2 * kBN;
                const uint32_t d_im = d_re + kBN;
                const uint32_t base = SmemAddr(smem + s * kStageBytes);
                if constexpr (kWide) {
                    constexpr uint32_t kIdescW = InstrDesc(kBM, 2 * kBN, false, kFmt);
#pragma unroll
                    for (int kk = 0; kk < kRowBytes / 32; ++kk) {
                        const uint32_t koff = kk * 32; // 32 bytes of K per MMA
                        const uint64_t arh = SmemDesc<kRowBytes>(base + 0 * kTileBytes + koff);
                        const uint64_t arl = SmemDesc<kRowBytes>(base + 1 * kTileBytes + koff);
                        const uint64_t aih = SmemDesc<kRowBytes>(base + 2 * kTileBytes + koff);
                        const uint64_t ail = SmemDesc<kRowBytes>(base + 3 * kTileBytes + koff);
                        // [-Bi; Br] starts at tile 4, [Br; Bi] at tile 5 (hi); 7, 8 (lo).
                        const uint64_t b_nr_hi = SmemDesc<kRowBytes>(base + 4 * kTileBytes + koff);
                        const uint64_t b_rc_hi = SmemDesc<kRowBytes>(base + 5 * kTileBytes + koff);
                        const uint64_t b_nr_lo = SmemDesc<kRowBytes>(base + 7 * kTileBytes + koff);
                        const uint64_t b_rc_lo = SmemDesc<kRowBytes>(base + 8 * kTileBytes + koff);
                        const uint32_t acc = (chunk_start && kk == 0) ? 0u : 1u;
                        // (Cr | Ci) += Ar [Br; Bi]
                        Mma<kHalf>(d_re, arh, b_rc_hi, kIdescW, acc);
                        Mma<kHalf>(d_re, arh, b_rc_lo, kIdescW, 1u);
                        Mma<kHalf>(d_re, arl, b_rc_hi, kIdescW, 1u);
                        // (Cr | Ci) += Ai [-Bi; Br]
                        Mma<kHalf>(d_re, aih, b_nr_hi, kIdescW, 1u);
                        Mma<kHalf>(d_re, aih, b_nr_lo, kIdescW, 1u);
                        Mma<kHalf>(d_re, ail, b_nr_hi, kIdescW, 1u);
                    }
                }
                else
#pragma unroll
                for (int kk = 0; kk < kRowBytes / 32; ++kk) {
                    const uint32_t koff = kk * 32; // 32 bytes of K per MMA
                    const uint64_t arh = SmemDesc<kRowBytes>(base + 0 * kTileBytes + koff);
                    const uint64_t arl = SmemDesc<kRowBytes>(base + 1 * kTileBytes + koff);
                    const uint64_t aih = SmemDesc<kRowBytes>(base + 2 * kTileBytes + koff);
                    const uint64_t ail = SmemDesc<kRowBytes>(base + 3 * kTileBytes + koff);
                    const uint64_t brh = SmemDesc<kRowBytes>(base + 4 * kTileBytes + koff);
                    const uint64_t brl = SmemDesc<kRowBytes>(base + 5 * kTileBytes + koff);
                    const uint64_t bih = SmemDesc<kRowBytes>(base + 6 * kTileBytes + koff);
                    const uint64_t bil = SmemDesc<kRowBytes>(base + 7 * kTileBytes + koff);
                    const uint32_t acc = (chunk_start && kk == 0) ? 0u : 1u;
                    // Cr += Ar Br
                    Mma<kHalf>(d_re, arh, brh, kIdesc, acc);
                    Mma<kHalf>(d_re, arh, brl, kIdesc, 1u);
                    Mma<kHalf>(d_re, arl, brh, kIdesc, 1u);
                    // Cr -= Ai Bi
                    Mma<kHalf>(d_re, aih, bih, kIdescNeg, 1u);
                    Mma<kHalf>(d_re, aih, bil, kIdescNeg, 1u);
                    Mma<kHalf>(d_re, ail, bih, kIdescNeg, 1u);
                    // Ci += Ar Bi
                    Mma<kHalf>(d_im, arh, bih, kIdesc, acc);
                    Mma<kHalf>(d_im, arh, bil, kIdesc, 1u);
                    Mma<kHalf>(d_im, arl, bih, kIdesc, 1u);
                    // Ci += Ai Br
                    Mma<kHalf>(d_im, aih, brh, kIdesc, 1u);
                    Mma<kHalf>(d_im, aih, brl, kIdesc, 1u);
                    Mma<kHalf>(d_im, ail, brh, kIdesc, 1u);
                }
                MmaCommit(SmemAddr(&empty_bar[s]));
                if (chunk_end)
                    MmaCommit(SmemAddr(&acc_full[buf]));
            }
            }
        }
        __syncwarp();
    }
    else {
        // Accumulator warps.
        const int quad = warp & 3;
        const int half = (warp - 2) >> 2;
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        // The FP16 form's operand scales, undone in the epilogue by two exact
        // multiplies (each factor inside the float range).
        float f1 = 1.f, f2 = 1.f;
        if (scale_exps != nullptr) {
            // 3M planes were scaled one power of two lower (sum headroom).
            const int e = -(Fp16ScaleExp(scale_exps[0]) + Fp16ScaleExp(scale_exps[1])) +
                          (kThreeM ? 2 : 0);
            f1 = Pow2f(e / 2);
            f2 = Pow2f(e - e / 2);
        }
        bool ok = true;
        for (int i = 0; ok; ++i) {
        const int r = i % kTileRing;
        ok = MbarWait(SmemAddr(&tile_full[r]), (uint32_t)(i / kTileRing) & 1u);
        __syncwarp();
        if (!ok)
            break;
        const int t = tile_ring[r];
        __syncwarp();
        if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                             SmemAddr(&tile_empty[r]))
                         : "memory");
        if (t >= total_tiles)
            break;
        int bz, m0, n0;
        tile_at(t, bz, m0, n0);
        float acc_re[64], acc_im[64];
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            acc_re[j] = 0.f;
            acc_im[j] = 0.f;
        }
        if constexpr (kThreeM) {
        for (int kt = 0; kt < ktiles && ok; ++kt) {
            const long long g = (long long)i * ktiles + kt;
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                const long long q = 3 * g + p;
                const int slot = (int)(q & 3);
                ok = MbarWait(SmemAddr(&acc_full[slot]), (uint32_t)(q >> 2) & 1u);
                __syncwarp();
                if (!ok)
                    break;
                FenceAfterSync();
                const uint32_t col0 = tmem + lane_base + slot * kBN + half * 64;
#pragma unroll
                for (int c = 0; c < 64; c += 32) {
                    float v0[16], v1[16];
                    TmemLoad16(col0 + c, v0);
                    TmemLoad16(col0 + c + 16, v1);
                    TmemWaitLoad();
#pragma unroll
                    for (int j = 0; j < 16; j += 2) {
                        // P1: Cr += P1, Ci -= P1; P2: Cr -= P2, Ci -= P2; P3: Ci += P3.
                        if (p != 2) {
                            const float sr = p == 0 ? 1.f : -1.f;
                            AddF32x2(acc_re[c + j], acc_re[c + j + 1], sr * v0[j], sr * v0[j + 1]);
                            AddF32x2(acc_re[c + 16 + j], acc_re[c + 17 + j], sr * v1[j],
                                     sr * v1[j + 1]);
                            AddF32x2(acc_im[c + j], acc_im[c + j + 1], -v0[j], -v0[j + 1]);
                            AddF32x2(acc_im[c + 16 + j], acc_im[c + 17 + j], -v1[j], -v1[j + 1]);
                        }
                        else {
                            AddF32x2(acc_im[c + j], acc_im[c + j + 1], v0[j], v0[j + 1]);
                            AddF32x2(acc_im[c + 16 + j], acc_im[c + 17 + j], v1[j], v1[j + 1]);
                        }
                    }
                }
                FenceBeforeSync();
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                     SmemAddr(&acc_empty[slot]))
                                 : "memory");
            }
        }
        }
        else
        for (int chunk = 0; chunk < nchunks; ++chunk) {
            const long long gc = (long long)i * nchunks + chunk;
            const int buf = (int)(gc & 1);
            ok = MbarWait(SmemAddr(&acc_full[buf]), (uint32_t)(gc >> 1) & 1u);
            __syncwarp();
            if (!ok)
                break;
            FenceAfterSync();
            const uint32_t col0 = tmem + lane_base + buf * 2 * kBN + half * 64;
#pragma unroll
            for (int c = 0; c < 64; c += 16) {
                float re[16], im[16];
                TmemLoad16(col0 + c, re);
                TmemLoad16(col0 + kBN + c, im);
                TmemWaitLoad();
#pragma unroll
                for (int j = 0; j < 16; j += 2) {
                    AddF32x2(acc_re[c + j], acc_re[c + j + 1], re[j], re[j + 1]);
                    AddF32x2(acc_im[c + j], acc_im[c + j + 1], im[j], im[j + 1]);
                }
            }
            FenceBeforeSync();
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                 SmemAddr(&acc_empty[buf]))
                             : "memory");
        }
        if (scale_exps != nullptr) {
#pragma unroll
            for (int j = 0; j < 64; ++j) {
                acc_re[j] = acc_re[j] * f1 * f2;
                acc_im[j] = acc_im[j] * f1 * f2;
            }
        }
        if (out_emax != nullptr && ok) {
            // Binary exponent of the largest |re| or |im| written (as the
            // max-exponent pass defines it); accumulators outside C hold 0.
            uint32_t best = 0;
#pragma unroll
            for (int j = 0; j < 64; ++j)
                best = max(best, max(__float_as_uint(acc_re[j] * scale) & 0x7fffffffu,
                                     __float_as_uint(acc_im[j] * scale) & 0x7fffffffu));
            const int biased = (int)(best >> 23);
            int ex = best == 0 ? kExpZero : (biased == 0 ? -127 : biased - 127);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, o));
            if (lane == 0)
                atomicMax(out_emax, ex);
        }
        const int row = m0 + quad * 32 + lane;
        const int cbase = n0 + half * 64;
        float2 *Cb = C + (size_t)bz * M * N;
        // Whole 32-row block with 16-byte aligned rows: stage each 32 x 16
        // complex block through shared memory (16-byte chunks XOR-swizzled by
        // row) so every warp store writes four full 128-byte row segments
        // instead of 32 scattered 16-byte pieces, one per row.
        const bool staged = ok && m0 + quad * 32 + 32 <= M && cbase + 64 <= N && (N & 1) == 0 &&
                            (reinterpret_cast<uintptr_t>(Cb) & 15) == 0;
        if (staged) {
            float4 *buf = reinterpret_cast<float4 *>(smem + kStages * kStageBytes +
                                                     (warp - 2) * kStoreBytes);
            const int sub = lane >> 3; // row within a group of 4 rows
            const int chunk = lane & 7;
            // Row m0 + quad * 32 + sub, columns cbase + 2 chunk, + 1; 4 rows
            // further down per step (2 N float4).
            float4 *gp = reinterpret_cast<float4 *>(Cb + (size_t)(m0 + quad * 32 + sub) * N +
                                                    cbase + 2 * chunk);
            const size_t step4 = (size_t)2 * N;
#pragma unroll
            for (int c0 = 0; c0 < 64; c0 += 16) {
#pragma unroll
                for (int p = 0; p < 8; ++p)
                    buf[lane * 8 + (p ^ (lane & 7))] =
                        make_float4(acc_re[c0 + 2 * p] * scale, acc_im[c0 + 2 * p] * scale,
                                    acc_re[c0 + 2 * p + 1] * scale, acc_im[c0 + 2 * p + 1] * scale);
                __syncwarp();
                float4 *g = gp + c0 / 2;
#pragma unroll 1
                for (int it = 0; it < 8; ++it) {
                    const int r = it * 4 + sub;
                    *g = buf[r * 8 + (chunk ^ (r & 7))];
                    g += step4;
                }
                __syncwarp();
            }
        }
        else if (ok && row < M) {
            // Edge blocks (rows past M, columns past N) and unaligned rows.
            float2 *dst = Cb + (size_t)row * N + cbase;
#pragma unroll
            for (int j = 0; j < 64; ++j)
                if (cbase + j < N)
                    dst[j] = make_float2(acc_re[j] * scale, acc_im[j] * scale);
        }
        }
    }
    FenceBeforeSync();
    __syncthreads();
    if (warp == 1) {
        FenceAfterSync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

// The failure path of the bounded waits, exercised without a fault: one
// thread waits on an mbarrier that nothing arrives on (phase 0 never
// completes), gives up after limit_ns (or 2^24 polls) and records the timeout.
__global__ void bounded_wait_probe_kernel(unsigned long long limit_ns)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        MbarInit(SmemAddr(&bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0)
        MbarWaitFor(SmemAddr(&bar), 0, limit_ns, 1u << 24);
    __syncthreads();
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

int GetEncoder()
{
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode)
        return SetError(JETGPU_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    return JETGPU_OK;
}

// 3-D map over planes: (k, row, plane), box (row_bytes of k) x 128 x 1,
// swizzled over row_bytes (64 or 32).
int EncodePlanes(CUtensorMap *map, const void *base, uint64_t rows, uint64_t k,
                 uint64_t kpitch, bool half, int planes, int row_bytes)
{
    const uint64_t eb = half ? 2 : 4;
    cuuint64_t dims[3] = {k, rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {kpitch * eb, rows * kpitch * eb};
    cuuint32_t box[3] = {(cuuint32_t)(row_bytes / eb), kBM, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = g_encode(map,
                          half ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                          3, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE,
                          row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return SetError(JETGPU_ERR_CUDA,
                        "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return JETGPU_OK;
}

// 4-D map over batched planes laid out [plane][batch][rows][kpitch]:
// (k, row, batch, plane), box (row_bytes of k) x 128 x 1 x 1.
int EncodePlanesBatched(CUtensorMap *map, const void *base, uint64_t rows, uint64_t k,
                        uint64_t kpitch, uint64_t batch, bool half, int planes, int row_bytes)
{
    const uint64_t eb = half ? 2 : 4;
    cuuint64_t dims[4] = {k, rows, batch, (cuuint64_t)planes};
    cuuint64_t strides[3] = {kpitch * eb, rows * kpitch * eb, batch * rows * kpitch * eb};
    cuuint32_t box[4] = {(cuuint32_t)(row_bytes / eb), kBM, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = g_encode(map,
                          half ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                          4, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE,
                          row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return SetError(JETGPU_ERR_CUDA,
                        "cuTensorMapEncodeTiled (4-D) failed: " + std::to_string((int)r));
    return JETGPU_OK;
}

// Persistent launch (one CTA per SM walking the tiles) or one CTA per tile
// (jetgpu_set_tc_persistent).
std::atomic<int> g_tc_persistent{1};

// A zeroed tile counter for a persistent launch whose caller gave no
// workspace word (the two-stage entry points): a slot of a per-device ring,
// reset by a memset enqueued before the launch (so a captured graph resets
// it on every replay). Consecutive launches take consecutive slots, so two
// launches share a slot only 4096 launches apart. nullptr (the static tile
// order) if the ring cannot be made. Contractions through jetgpu_contract*
// keep their counter in their own workspace instead.
unsigned int *TileCounter(cudaStream_t stream)
{
    constexpr uint32_t kSlots = 4096;
    static std::mutex mu;
    static unsigned int *slots[64] = {};
    static std::atomic<uint32_t> next[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (slots[dev] == nullptr) {
            // Allowed even while a stream of this thread is being captured.
            cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
            cudaThreadExchangeStreamCaptureMode(&mode);
            void *p = nullptr;
            const cudaError_t err = cudaMalloc(&p, kSlots * sizeof(unsigned int));
            cudaThreadExchangeStreamCaptureMode(&mode);
            if (err != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            slots[dev] = static_cast<unsigned int *>(p);
        }
    }
    unsigned int *c = slots[dev] + next[dev].fetch_add(1u, std::memory_order_relaxed) % kSlots;
    if (cudaMemsetAsync(c, 0, sizeof(unsigned int), stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return c;
}
// Tile rows per group of the tile order (jetgpu_set_tc_group_m).
std::atomic<int> g_tc_group_m{kGroupM};

template <int V>
int LaunchTc(const CUtensorMap &ta, const CUtensorMap &tb, void *C, uint64_t batch, uint64_t m,
             uint64_t n, uint64_t k, float out_scale, int a_batched, int b_batched,
             cudaStream_t stream, const int *e_max_dev = nullptr, int group_m = 0,
             int *out_emax = nullptr, unsigned int *tile_counter = nullptr)
{
    const size_t smem = (size_t)TcCfg<V>::Stages * StageBytes<V>() + kAccWarps * kStoreBytes + 1024;
    static thread_local int configured_dev = -1;
    int dev = 0;
    JETGPU_CUDA_TRY(cudaGetDevice(&dev));
    if (configured_dev != dev) {
        JETGPU_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_split_kernel<V>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem));
        configured_dev = dev;
    }
    // Persistent: one CTA per SM (at most one per 128 x 128 tile of C), each
    // walking the batch's tiles in the grouped order; otherwise one CTA per
    // tile.
    const uint64_t tiles = ((n + kBN - 1) / kBN) * ((m + kBM - 1) / kBM) * batch;
    JETGPU_REQUIRE(tiles <= 0x7fffffffull, "too many tiles");
    const bool persistent = g_tc_persistent.load(std::memory_order_relaxed) != 0;
    const unsigned grid =
        (unsigned)(persistent ? std::min<uint64_t>(tiles, (uint64_t)SmCount()) : tiles);
    unsigned int *counter = nullptr;
    if (persistent && grid < tiles) {
        if (tile_counter != nullptr) {
            JETGPU_CUDA_TRY(cudaMemsetAsync(tile_counter, 0, sizeof(unsigned int), stream));
            counter = tile_counter;
        }
        else {
            counter = TileCounter(stream);
        }
    }
    const int ktiles = (int)((k + BlockK<V>() - 1) / BlockK<V>());
    tc_gemm_split_kernel<V><<<grid, kThreads, smem, stream>>>(
        ta, tb, reinterpret_cast<float2 *>(C), (int)m, (int)n, ktiles, (int)batch, out_scale,
        a_batched, b_batched, ChunkStages(TcCfg<V>::Fmt, BlockK<V>()), e_max_dev,
        group_m > 0 ? group_m : g_tc_group_m.load(std::memory_order_relaxed), counter, out_emax);
    return CheckLaunch("tc_gemm_split_kernel");
}

// Main-loop variant (jetgpu_set_tc_variant): 0 default, 1 N = 256 (any
// format; six B planes), 2 BF16 with 32-byte rows and 6 stages.
std::atomic<int> g_tc_variant{0};

} // namespace

int GemmTf32x3Planar(const float *a_planes, const float *b_planes, void *C,
                     uint64_t m, uint64_t n, uint64_t k, uint64_t kpitch,
                     float out_scale, cudaStream_t stream)
{
    return GemmSplitPlanarBatched(a_planes, 0, b_planes, 0, C, 1, m, n, k, kpitch, out_scale,
                                  SplitFormat::kTf32, stream);
}

int GemmTf32x3PlanarBatched(const float *a_planes, int a_batched, const float *b_planes,
                            int b_batched, void *C, uint64_t batch, uint64_t m, uint64_t n,
                            uint64_t k, uint64_t kpitch, float out_scale, cudaStream_t stream)
{
    return GemmSplitPlanarBatched(a_planes, a_batched, b_planes, b_batched, C, batch, m, n, k,
                                  kpitch, out_scale, SplitFormat::kTf32, stream);
}

int GemmSplitPlanarBatched(const void *a_planes, int a_batched, const void *b_planes,
                           int b_batched, void *C, uint64_t batch, uint64_t m, uint64_t n,
                           uint64_t k, uint64_t kpitch, float out_scale, SplitFormat fmt,
                           cudaStream_t stream, int variant, const int *e_max_dev, int group_m,
                           int *out_emax, unsigned int *tile_counter, int algo)
{
    JETGPU_REQUIRE(algo == JETGPU_ALGO_4M || algo == JETGPU_ALGO_3M, "bad algorithm");
    const bool three_m = algo == JETGPU_ALGO_3M;
    JETGPU_REQUIRE(batch >= 1 && batch <= 65535, "batch out of range");
    if (batch == 1) {
        a_batched = 0;
        b_batched = 0;
    }
    const bool bf16 = fmt == SplitFormat::kBf16;
    const bool fp16 = fmt == SplitFormat::kFp16;
    const bool half = bf16 || fp16;
    JETGPU_REQUIRE(!fp16 || e_max_dev != nullptr, "FP16 planes need their max exponents");
    JETGPU_REQUIRE(m > 0 && n > 0 && k > 0, "empty product");
    JETGPU_REQUIRE(m < (1ull << 31) && n < (1ull << 31) && k < (1ull << 31),
                   "dimension too large");
    JETGPU_REQUIRE(kpitch >= k && kpitch % SplitPitchAlign(fmt) == 0, "bad k pitch");
    JETGPU_REQUIRE(((uintptr_t)a_planes % 16) == 0 && ((uintptr_t)b_planes % 16) == 0,
                   "planes must be 16-byte aligned");
    JETGPU_REQUIRE(((n + kBN - 1) / kBN) * ((m + kBM - 1) / kBM) <= 0x7fffffffull,
                   "grid too large");
    if (!TcAvailable())
        return SetError(JETGPU_ERR_UNSUPPORTED, "tensor-core path needs an sm_103 device");
    int rc = GetEncoder();
    if (rc)
        return rc;
    if (variant < 0)
        variant = TcVariant();
    const bool wide = variant == 1 && !three_m;
    const bool deep = bf16 && variant == 2 && !three_m;
    const int row_bytes = deep ? TcCfg<3>::RowBytes : TcCfg<0>::RowBytes;
    const int aplanes = three_m ? 6 : 4;
    CUtensorMap ta, tb;
    if ((rc = a_batched
                  ? EncodePlanesBatched(&ta, a_planes, m, k, kpitch, batch, half, aplanes,
                                        row_bytes)
                  : EncodePlanes(&ta, a_planes, m, k, kpitch, half, aplanes, row_bytes)))
        return rc;
    const int bplanes = (wide || three_m) ? 6 : 4;
    if ((rc = b_batched
                  ? EncodePlanesBatched(&tb, b_planes, n, k, kpitch, batch, half, bplanes, row_bytes)
                  : EncodePlanes(&tb, b_planes, n, k, kpitch, half, bplanes, row_bytes)))
        return rc;
    if (three_m) {
        if (fp16)
            return LaunchTc<7>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched,
                               stream, e_max_dev, group_m, out_emax, tile_counter);
        if (bf16)
            return LaunchTc<6>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched,
                               stream, nullptr, group_m, out_emax, tile_counter);
        return LaunchTc<5>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                           nullptr, group_m, out_emax, tile_counter);
    }
    if (wide && fp16)
        return LaunchTc<9>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                           e_max_dev, group_m, out_emax, tile_counter);
    if (wide && bf16)
        return LaunchTc<8>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                           nullptr, group_m, out_emax, tile_counter);
    if (fp16)
        return LaunchTc<4>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                           e_max_dev, group_m, out_emax, tile_counter);
    if (deep)
        return LaunchTc<3>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                           nullptr, group_m, out_emax, tile_counter);
    if (bf16)
        return LaunchTc<2>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                           nullptr, group_m, out_emax, tile_counter);
    return wide ? LaunchTc<1>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched, stream,
                              nullptr, group_m, out_emax, tile_counter)
                : LaunchTc<0>(ta, tb, C, batch, m, n, k, out_scale, a_batched, b_batched,
                              stream, nullptr, group_m, out_emax, tile_counter);
}

int TcVariant() { return g_tc_variant.load(std::memory_order_relaxed); }
bool TcWide() { return TcVariant() == 1; }

} // namespace jetgpu

extern "C" int jetgpu_tc_b_planes(void) { return jetgpu::TcWide() ? 6 : 4; }

extern "C" int jetgpu_set_tc_group_m(int group_m)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(group_m >= 1 && group_m <= 1024, "group_m must be in [1, 1024]");
    jetgpu::g_tc_group_m.store(group_m, std::memory_order_relaxed);
    return JETGPU_OK;
}

extern "C" int jetgpu_set_tc_persistent(int on)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(on == 0 || on == 1, "persistent must be 0 or 1");
    jetgpu::g_tc_persistent.store(on, std::memory_order_relaxed);
    return JETGPU_OK;
}

extern "C" int jetgpu_set_tc_variant(int variant)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(variant >= 0 && variant <= 2,
                   "variant must be 0 (default), 1 (N = 256) or 2 (BF16 6-stage)");
    jetgpu::g_tc_variant.store(variant, std::memory_order_relaxed);
    return JETGPU_OK;
}

extern "C" int jetgpu_set_tc_chunk_depth(int k_depth)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(k_depth >= 0 && k_depth <= 4096, "chunk depth out of range");
    jetgpu::g_tc_chunk_k.store(k_depth, std::memory_order_relaxed);
    return JETGPU_OK;
}

extern "C" int jetgpu_probe_bounded_wait(unsigned int limit_us, void *stream)
{
    jetgpu::ClearError();
    JETGPU_REQUIRE(limit_us >= 1 && limit_us <= 1000000, "limit must be 1 us .. 1 s");
    jetgpu::bounded_wait_probe_kernel<<<1, 32, 0, jetgpu::AsStream(stream)>>>(
        (unsigned long long)limit_us * 1000ull);
    return jetgpu::CheckLaunch("bounded_wait_probe_kernel");
}

extern "C" int jetgpu_take_device_status(int *status)
{
    jetgpu::ClearError();
    int v = 0;
    JETGPU_CUDA_TRY(cudaMemcpyFromSymbol(&v, jetgpu::g_tc_status, sizeof(int)));
    if (v != 0) {
        int zero = 0;
        JETGPU_CUDA_TRY(cudaMemcpyToSymbol(jetgpu::g_tc_status, &zero, sizeof(int)));
    }
    if (status)
        *status = v;
    return JETGPU_OK;
}
