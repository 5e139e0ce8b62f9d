// Shared helpers of the jetgpu C-ABI library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <string>

#include "../../include/jetgpu.h"

namespace jetgpu {

// Records `msg` as this thread's last error and returns `code`.
int SetError(int code, const std::string &msg);
// Clears this thread's last error.
void ClearError();

inline cudaStream_t AsStream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Checks the launch that was just enqueued.
int CheckLaunch(const char *what);

// An NVTX range for the scope (seen by nsys / ncu; no cost without a tool).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

#define JETGPU_CUDA_TRY(expr)                                                  \
    do {                                                                       \
        cudaError_t err__ = (expr);                                            \
        if (err__ != cudaSuccess)                                              \
            return ::jetgpu::SetError(JETGPU_ERR_CUDA,                         \
                                      std::string(#expr) + ": " +              \
                                          cudaGetErrorString(err__));          \
    } while (0)

#define JETGPU_REQUIRE(cond, msg)                                              \
    do {                                                                       \
        if (!(cond))                                                           \
            return ::jetgpu::SetError(JETGPU_ERR_INVALID, (msg));              \
    } while (0)

inline size_t ElemBytes(int dtype) { return dtype == JETGPU_C128 ? 16 : 8; }

inline bool IsPow2(uint64_t v) { return v && !(v & (v - 1)); }

inline int Log2(uint64_t v)
{
    int r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

// Number of SMs of the current device (cached per device).
int SmCount();

// Grid size for a persistent / grid-stride kernel: `per_sm` CTAs per SM,
// never more than `work_items`.
inline unsigned GridFor(uint64_t work_items, int per_sm)
{
    uint64_t g = (uint64_t)SmCount() * (uint64_t)per_sm;
    if (work_items < g)
        g = work_items;
    return (unsigned)(g ? g : 1);
}

// Division by an invariant d (Granlund-Montgomery, the round-up method):
// Magic32(d) gives (m, s) with n / d = (t + (n - t) / 2) >> s, t = hi32(n m),
// exact for every 32-bit n; m = 0 marks d = 1.
inline void Magic32(uint64_t d, uint32_t &m, uint32_t &sh)
{
    if (d <= 1) {
        m = 0;
        sh = 0;
        return;
    }
    int l = 0;
    while ((1ull << l) < d)
        ++l;
    m = (uint32_t)(((((1ull << l) - d) << 32) / d) + 1);
    sh = (uint32_t)(l - 1);
}

__device__ __forceinline__ uint32_t DivMagic(uint32_t n, uint32_t m, uint32_t s)
{
    if (m == 0)
        return n;
    const uint32_t t = __umulhi(n, m);
    return (t + ((n - t) >> 1)) >> s;
}

// Internal entry points shared between translation units.
int PermuteImpl(const void *in, void *out, uint64_t batch, int rank,
                const uint64_t *shape, const int32_t *perm, int dtype,
                cudaStream_t stream);

// Permutes a complex64 tensor and writes it as TF32 hi/lo planes for the
// tensor-core product: plane p (0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo) holds a
// rows x cols fp32 matrix with row pitch `pitch` floats, where the permuted
// tensor is viewed as rows x cols (row-major). Values are multiplied by
// 2^scale_exp first.
int PermuteSplitTf32(const void *in, float *planes, int rank,
                     const uint64_t *shape, const int32_t *perm, uint64_t rows,
                     uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                     int scale_exp, cudaStream_t stream);

// Permute + TF32 split of `batch` tensors stored back to back; tensor b lands
// in rows [b * rows, (b + 1) * rows) of every plane (plane_stride >= batch *
// rows * pitch).
// neg_im != 0 also writes planes 4, 5 = -im_hi, -im_lo (the B operand of the
// N = 256 tensor-core product).
int PermuteSplitTf32Batched(const void *in, float *planes, uint64_t batch, int rank,
                            const uint64_t *shape, const int32_t *perm, uint64_t rows,
                            uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                            int scale_exp, cudaStream_t stream, int neg_im = 0);

// Word format of the split planes: TF32 (FP32 words, 13 low mantissa bits
// zero), BF16 or FP16 (16-bit words). pitch and plane_stride count words; a
// row pitch must span a multiple of 16 bytes (SplitPitchAlign words).
enum class SplitFormat { kTf32 = 0, kBf16 = 1, kFp16 = 2 };
inline uint64_t SplitWordBytes(SplitFormat f) { return f == SplitFormat::kTf32 ? 4 : 2; }
inline uint64_t SplitPitchAlign(SplitFormat f) { return f == SplitFormat::kTf32 ? 4 : 8; }

// FP16 split: an operand whose largest magnitude has binary exponent e_max
// (jetgpu_max_exponent; -1000 when all zero) is multiplied by 2^s before the
// split, s = 14 - e_max clamped to [-120, 120], so its largest value lies in
// [2^14, 2^15) (below the FP16 maximum 65504, hi and lo normal down to
// 2^-15 of it). The product's epilogue multiplies by 2^-(s_A + s_B).
__host__ __device__ inline int Fp16ScaleExp(int e_max)
{
    const int s = 14 - e_max;
    return s < -120 ? -120 : (s > 120 ? 120 : s);
}

// 2^e as a float, e in [-126, 127] (exact).
__host__ __device__ inline float Pow2f(int e)
{
    union {
        uint32_t u;
        float f;
    } v;
    v.u = (uint32_t)(e + 127) << 23;
    return v.f;
}

// Extra plane pair (planes 4 and 5) of a split: none; -im_hi, -im_lo (the
// N = 256 main loop's B operand); hi, lo of re + im (the 3M product's sums).
constexpr int kSplitNone = 0, kSplitNegIm = 1, kSplitSum = 2;

// PermuteSplitTf32Batched for any word format.
// For FP16, `e_max_dev` points at the operand's max exponent on the device
// and sets the scale (Fp16ScaleExp, one less with kSplitSum so the sums stay
// in range); scale_exp is then ignored.
int PermuteSplitPlanes(const void *in, void *planes, uint64_t batch, int rank,
                       const uint64_t *shape, const int32_t *perm, uint64_t rows, uint64_t cols,
                       uint64_t pitch, uint64_t plane_stride, int scale_exp, SplitFormat fmt,
                       int extra, cudaStream_t stream, const int *e_max_dev = nullptr);

// Device max exponent of `size` complex elements into *e_dev (stream-ordered).
int MaxExponent(const void *x, uint64_t size, int dtype, int *e_dev, cudaStream_t stream);

// Max exponents of two operands into e[0], e[1] in one fill and one launch.
// hint0 / hint1 (device ints, may be null): an operand whose hint holds an
// exponent (>= kExpZero, recorded by the kernel that wrote the operand) is
// not read.
int MaxExponent2(const void *x0, uint64_t n0, const void *x1, uint64_t n1, int dtype, int *e,
                 cudaStream_t stream, int operands = 2, const int *hint0 = nullptr,
                 const int *hint1 = nullptr);

// Max exponent of an all-zero operand; smaller values (the 0x80 byte fill)
// mean "no exponent recorded".
constexpr int kExpZero = -1000;

// C[b] = A[b] B[b] for b < batch (strides sa, sb in elements; 0 = shared
// operand), C packed as batch x m x n. Vector-shaped products split over k
// into the workspace when it holds MultiplyPlainBatchedWorkspace bytes.
int MultiplyPlainBatched(const void *A, const void *B, void *C, uint64_t batch, uint64_t sa,
                         uint64_t sb, uint64_t m, uint64_t n, uint64_t k, int dtype,
                         int scale_exp, void *workspace, size_t ws_bytes, cudaStream_t stream);

size_t MultiplyPlainBatchedWorkspace(uint64_t batch, uint64_t m, uint64_t n, uint64_t k,
                                     int dtype);

// Batched TF32x3 product: operand planes laid out [plane][batch][rows][kpitch]
// when batched (a_batched / b_batched), [plane][rows][kpitch] when shared.
int GemmTf32x3PlanarBatched(const float *a_planes, int a_batched, const float *b_planes,
                            int b_batched, void *C, uint64_t batch, uint64_t m, uint64_t n,
                            uint64_t k, uint64_t kpitch, float out_scale, cudaStream_t stream);

// The batched split product for either word format (kpitch in words).
// `variant`: main-loop variant (jetgpu_set_tc_variant) read once by the
// caller, so the planes it wrote and the loop that reads them agree; -1 reads
// the current setting.
// For FP16, `e_max_dev` points at the two operands' max exponents (A, B) and
// the epilogue undoes their scales. `group_m`: tile rows per group of the
// tile order (0: the jetgpu_set_tc_group_m setting). `tile_counter`: device
// word of the caller's workspace for the persistent launch's tile counter
// (null: a slot of a library-wide ring). `algo`: JETGPU_ALGO_4M (four planes
// per operand) or JETGPU_ALGO_3M (six: the split's kSplitSum pair added; FP16
// planes scaled one power of two lower, which the epilogue undoes).
int GemmSplitPlanarBatched(const void *a_planes, int a_batched, const void *b_planes,
                           int b_batched, void *C, uint64_t batch, uint64_t m, uint64_t n,
                           uint64_t k, uint64_t kpitch, float out_scale, SplitFormat fmt,
                           cudaStream_t stream, int variant = -1,
                           const int *e_max_dev = nullptr, int group_m = 0,
                           int *out_emax = nullptr, unsigned int *tile_counter = nullptr,
                           int algo = JETGPU_ALGO_4M);

// Workspace bytes of a (batched) contraction in `precision` (JETGPU_PREC_TUNED:
// the largest of its candidates' and AUTO's).
size_t ContractWorkspace(uint64_t batch, int a_rank, const uint64_t *a_shape,
                         const int32_t *a_perm, int a_batched, int b_rank,
                         const uint64_t *b_shape, const int32_t *b_perm, int b_batched, uint64_t m,
                         uint64_t n, uint64_t k, int dtype, int precision,
                         int algo = JETGPU_ALGO_4M);

// Max-exponent hints of one contraction (device ints; each may be null):
// `a` / `b` hold the operands' exponents when the kernels that wrote them
// recorded them (values below kExpZero: not recorded), so the FP16 form need
// not scan them; `c` receives C's when the product runs on the tensor cores
// and is left unrecorded otherwise.
struct ExpHints {
    const int *a = nullptr;
    const int *b = nullptr;
    int *c = nullptr;
};

// A checked (batched) contraction in one form: precision FP32, TF32X3,
// BF16X3, FP16X3 or AUTO; `variant` the tensor-core main loop (-1: the
// jetgpu_set_tc_variant setting), `group_m` its tile order (0: the
// jetgpu_set_tc_group_m setting).
int ContractForm(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                 const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                 const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                 uint64_t m, uint64_t n, uint64_t k, int dtype, int precision, int variant,
                 int scale_a, int scale_b, void *workspace, cudaStream_t st, int group_m = 0,
                 const ExpHints *hints = nullptr, int algo = JETGPU_ALGO_4M);

// JETGPU_PREC_TUNED: the form the autotuner measured fastest for this
// contraction's key, timing the candidates on first use (autotune.cu).
int ContractTuned(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                  const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                  const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                  uint64_t m, uint64_t n, uint64_t k, int dtype, int scale_a, int scale_b,
                  void *workspace, cudaStream_t st, const ExpHints *hints = nullptr);

// Skinny contractions (skinny.cu): one side of the product at most 16 wide,
// k <= 64, read straight from the operands' layouts without transposes or
// workspace. SkinnyApplies: whether the kernel takes this contraction (its
// operands' axes fit its index tables); arguments as ContractForm's, after
// its batch normalisation (batch 1: both flags 0).
bool SkinnyApplies(uint64_t batch, int a_rank, const uint64_t *a_shape, const int32_t *a_perm,
                   int a_batched, int b_rank, const uint64_t *b_shape, const int32_t *b_perm,
                   int b_batched, uint64_t m, uint64_t n, uint64_t k);
int SkinnyContract(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                   const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                   const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                   uint64_t m, uint64_t n, uint64_t k, int dtype, int scale_exp,
                   cudaStream_t st);

int MultiplyPlain(const void *A, const void *B, void *C, uint64_t m,
                  uint64_t n, uint64_t k, int dtype, int scale_exp,
                  void *workspace, size_t ws_bytes, cudaStream_t stream);

size_t MultiplyPlainWorkspace(uint64_t m, uint64_t n, uint64_t k, int dtype);

// Tensor-core 3xTF32 complex product of planar operands (see gemm_tc.cu).
int GemmTf32x3Planar(const float *a_planes, const float *b_planes, void *C,
                     uint64_t m, uint64_t n, uint64_t k, uint64_t kpitch,
                     float out_scale, cudaStream_t stream);

bool TcAvailable();

// Main-loop shape of the tensor-core product: wide (N = 256 MMAs) needs six B
// planes (re hi/lo, im hi/lo, -im hi/lo), narrow four.
bool TcWide();
int TcVariant();

} // namespace jetgpu
