// Pairwise contraction orchestration (Tensor::ContractTensors, device side).
//
// Reference: include/jet/Tensor.hpp:708-752 transposes A to (left ++ common)
// and B to (common ++ right) with the Permuter backends, then calls
// TensorHelpers::MultiplyTensorData. The label algebra stays on the host;
// this file receives the two orderings as axis permutations.
//
// Plain form:  At = permute(A), Bt = permute(B) into the workspace (skipped
//              when already ordered), then the SIMT complex product.
// Split form: A is permuted straight into hi/lo planes (M x K; TF32 words for
//              TF32x3, BF16 words for BF16x3, FP16 words of the operand
//              scaled by a power of two for FP16x3), B into planes of its
//              (right ++ common) order (N x K, K-major), then the tcgen05
//              product writes C. FP16x3 first writes each operand's max
//              exponent into the workspace; the splits and the product's
//              epilogue read the scales from there (no host round trip).
#include <atomic>
#include <vector>

#include "common.cuh"

namespace jetgpu {
namespace {

constexpr size_t kAlign = 256;

inline size_t AlignUp(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Word format, row pitch and plane counts of the split form.
struct SplitLayout {
    SplitFormat fmt;
    int variant;      // main-loop variant, read once
    int algo;         // JETGPU_ALGO_4M or JETGPU_ALGO_3M
    uint64_t kp;      // row pitch in words
    uint64_t word;    // bytes per word
    int a_planes;     // 4, or 6 for 3M (re + im hi, lo)
    int b_planes;     // 4, or 6 for the N = 256 TF32 main loop and for 3M
    int group_m;      // tile order (0: the setting)
    size_t a_bytes(uint64_t rows) const { return AlignUp(a_planes * rows * kp * word); }
    size_t b_bytes(uint64_t rows) const { return AlignUp(b_planes * rows * kp * word); }
    // After the planes: the operands' max exponents (two ints, FP16) and the
    // product's tile counter (one unsigned int at byte 16).
    size_t exp_bytes() const { return kAlign; }
};

// The split form JETGPU_PREC_AUTO uses on tensor-core steps
// (jetgpu_set_auto_form). FP16x3 by default: TF32x3's precision at twice its
// rate (measured on sliced 49- and 53-qubit circuit amplitudes: 5.7e-6 and
// 7.4e-6 from FP64, against TF32x3's 6.7e-6 and 7.0e-6, at 1.55x and 1.74x
// the slices/s).
std::atomic<int> g_auto_form{JETGPU_PREC_FP16X3};

// AUTO gives FP16x3 steps of at least this many complex multiply-adds
// (m n k, summed over a batch); below it, where the operands' max-exponent
// pass costs more than the faster product saves, TF32x3 (same precision).
constexpr double kAutoFp16MinWork = 1073741824.0; // 2^30

SplitLayout LayoutFor(int precision, uint64_t k, double work, int variant = -1,
                      int group_m = 0, int algo = JETGPU_ALGO_4M)
{
    if (precision == JETGPU_PREC_AUTO) {
        precision = g_auto_form.load(std::memory_order_relaxed);
        if (precision == JETGPU_PREC_FP16X3 && work < kAutoFp16MinWork)
            precision = JETGPU_PREC_TF32X3;
    }
    SplitLayout l;
    l.fmt = precision == JETGPU_PREC_BF16X3   ? SplitFormat::kBf16
            : precision == JETGPU_PREC_FP16X3 ? SplitFormat::kFp16
                                              : SplitFormat::kTf32;
    const uint64_t al = SplitPitchAlign(l.fmt);
    l.kp = (k + al - 1) / al * al;
    l.word = SplitWordBytes(l.fmt);
    l.variant = variant >= 0 ? variant : TcVariant();
    l.algo = algo;
    l.a_planes = algo == JETGPU_ALGO_3M ? 6 : 4;
    l.b_planes = (algo == JETGPU_ALGO_3M || l.variant == 1) ? 6 : 4;
    l.group_m = group_m;
    return l;
}

// The main-loop setting for the 16-bit stage entry points, whose B operand
// has four planes: the N = 256 loop (variant 1) needs six, so it runs as 0.
int FourPlaneVariant()
{
    const int v = TcVariant();
    return v == 1 ? 0 : v;
}

bool IsIdentity(int rank, const int32_t *perm)
{
    for (int i = 0; i < rank; ++i)
        if (perm[i] != i)
            return false;
    return true;
}

// Number of leading axes of `perm` whose dimensions multiply to `lead`
// (-1 if no prefix does).
int SplitPoint(int rank, const uint64_t *shape, const int32_t *perm, uint64_t lead)
{
    uint64_t p = 1;
    if (lead == 1)
        return 0;
    for (int j = 0; j < rank; ++j) {
        p *= shape[perm[j]];
        if (p == lead)
            return j + 1;
        if (p > lead)
            return -1;
    }
    return -1;
}

bool UseTensorCores(uint64_t m, uint64_t n, uint64_t k, int dtype, int precision)
{
    if (dtype != JETGPU_C64 || precision == JETGPU_PREC_FP32)
        return false;
    if (m < 2 || n < 2)
        return false; // vector-shaped steps are bandwidth bound
    if (precision == JETGPU_PREC_AUTO && (m < 128 || n < 64 || k < 32))
        return false;
    return TcAvailable();
}

int Validate(int rank, const uint64_t *shape, const int32_t *perm, uint64_t lead,
             uint64_t tail, const char *which)
{
    JETGPU_REQUIRE(rank >= 0 && rank <= 64, std::string(which) + ": rank out of range");
    uint64_t size = 1;
    for (int i = 0; i < rank; ++i)
        size *= shape[i];
    JETGPU_REQUIRE(size == lead * tail, std::string(which) + ": size does not match the product dimensions");
    JETGPU_REQUIRE(SplitPoint(rank, shape, perm, lead) >= 0,
                   std::string(which) + ": permutation does not split into the product dimensions");
    return JETGPU_OK;
}

// The split form of one contraction or of a batch of them: operand planes
// (and, for FP16, the operands' max exponents) in `ws`, then the tcgen05
// product. ba / bb: tensors of A / B (batch or 1, shared operands are 1).
int SplitProduct(const SplitLayout &l, uint64_t batch, const void *A, int a_rank,
                 const uint64_t *a_shape, const int32_t *a_perm, uint64_t ba, int a_mode,
                 const void *B, int b_rank, const uint64_t *b_shape, const int32_t *b_perm,
                 uint64_t bb, int b_mode, void *C, uint64_t m, uint64_t n, uint64_t k, int dtype,
                 int scale_a, int scale_b, uint8_t *ws, cudaStream_t st, const ExpHints *hints)
{
    int rc;
    uint8_t *pa = ws;
    uint8_t *pb = ws + l.a_bytes(ba * m);
    uint8_t *tail = pb + AlignUp((size_t)l.b_planes * bb * n * l.kp * l.word);
    unsigned int *tile_counter = reinterpret_cast<unsigned int *>(tail + 16);
    int *e_dev = nullptr;
    float out_scale = 1.0f;
    if (l.fmt == SplitFormat::kFp16) {
        // Each operand's max exponent sets its FP16 scale; the user's exact
        // scales move to the epilogue.
        JETGPU_REQUIRE(scale_a + scale_b >= -126 && scale_a + scale_b <= 126,
                       "scale_a + scale_b out of range for FP16x3");
        e_dev = reinterpret_cast<int *>(tail);
        if ((rc = MaxExponent2(A, ba * m * k, B, bb * k * n, dtype, e_dev, st, 2,
                               hints ? hints->a : nullptr, hints ? hints->b : nullptr)))
            return rc;
        out_scale = Pow2f(scale_a + scale_b);
        scale_a = scale_b = 0;
    }
    // B is wanted as (right ++ common): rotate its (common ++ right) order,
    // behind its batch axes when they are part of its permutation (mode 2).
    const int nb = b_mode == 2 ? SplitPoint(b_rank, b_shape, b_perm, bb) : 0;
    const int nc = SplitPoint(b_rank, b_shape, b_perm, (b_mode == 2 ? bb : 1) * k);
    std::vector<int32_t> bt(b_perm, b_perm + b_rank);
    for (int j = nb; j < b_rank; ++j)
        bt[j] = b_perm[nb + (j - nb + nc - nb) % (b_rank - nb)];
    // Mode 1: `ba` tensors back to back; mode 2: one tensor whose leading
    // permuted axes are the batch, i.e. ba * m rows of one split.
    const bool three_m = l.algo == JETGPU_ALGO_3M;
    if ((rc = PermuteSplitPlanes(A, pa, a_mode == 1 ? ba : 1, a_rank, a_shape, a_perm,
                                 (a_mode == 2 ? ba : 1) * m, k, l.kp, ba * m * l.kp, scale_a,
                                 l.fmt, three_m ? kSplitSum : kSplitNone, st, e_dev)))
        return rc;
    const int b_extra = three_m ? kSplitSum : (l.b_planes == 6 ? kSplitNegIm : kSplitNone);
    if ((rc = PermuteSplitPlanes(B, pb, b_mode == 1 ? bb : 1, b_rank, b_shape, bt.data(),
                                 (b_mode == 2 ? bb : 1) * n, k, l.kp, bb * n * l.kp, scale_b,
                                 l.fmt, b_extra, st, e_dev ? e_dev + 1 : nullptr)))
        return rc;
    return GemmSplitPlanarBatched(pa, ba > 1, pb, bb > 1, C, batch, m, n, k, l.kp, out_scale,
                                  l.fmt, st, l.variant, e_dev, l.group_m,
                                  hints ? hints->c : nullptr, tile_counter, l.algo);
}

} // namespace
} // namespace jetgpu

using namespace jetgpu;

extern "C" {

int jetgpu_multiply(const void *A, const void *B, void *C, uint64_t m, uint64_t n,
                    uint64_t k, int dtype, void *stream)
{
    NvtxRange range("jetgpu_multiply");
    ClearError();
    return MultiplyPlain(A, B, C, m, n, k, dtype, 0, nullptr, 0, AsStream(stream));
}


int jetgpu_split_tf32(const void *in, int rank, const uint64_t *shape, const int32_t *perm,
                      uint64_t rows, uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                      int scale_exp, int n_planes, float *planes, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(n_planes == 4 || n_planes == 6, "n_planes must be 4 or 6");
    JETGPU_REQUIRE(pitch >= cols && pitch % 4 == 0, "pitch must be >= cols and a multiple of 4");
    JETGPU_REQUIRE(plane_stride >= rows * pitch, "plane stride too small");
    if (rows * cols == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in != nullptr && planes != nullptr, "null pointer");
    return PermuteSplitTf32Batched(in, planes, 1, rank, shape, perm, rows, cols, pitch,
                                   plane_stride, scale_exp, AsStream(stream),
                                   n_planes == 6 ? 1 : 0);
}

int jetgpu_gemm_tf32x3(const float *a_planes, const float *b_planes, void *C, uint64_t m,
                       uint64_t n, uint64_t k, uint64_t kpitch, float out_scale, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(C != nullptr && a_planes != nullptr && b_planes != nullptr, "null pointer");
    return GemmTf32x3Planar(a_planes, b_planes, C, m, n, k, kpitch, out_scale, AsStream(stream));
}

int jetgpu_split_bf16(const void *in, int rank, const uint64_t *shape, const int32_t *perm,
                      uint64_t rows, uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                      int scale_exp, uint16_t *planes, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(pitch >= cols && pitch % 8 == 0, "pitch must be >= cols and a multiple of 8");
    JETGPU_REQUIRE(plane_stride >= rows * pitch, "plane stride too small");
    if (rows * cols == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in != nullptr && planes != nullptr, "null pointer");
    return PermuteSplitPlanes(in, planes, 1, rank, shape, perm, rows, cols, pitch, plane_stride,
                              scale_exp, SplitFormat::kBf16, 0, AsStream(stream));
}

int jetgpu_set_auto_form(int precision)
{
    ClearError();
    JETGPU_REQUIRE(precision == JETGPU_PREC_TF32X3 || precision == JETGPU_PREC_BF16X3 ||
                       precision == JETGPU_PREC_FP16X3,
                   "the AUTO form must be TF32X3, BF16X3 or FP16X3");
    g_auto_form.store(precision, std::memory_order_relaxed);
    return JETGPU_OK;
}

int jetgpu_split_fp16(const void *in, int rank, const uint64_t *shape, const int32_t *perm,
                      uint64_t rows, uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                      const int *e_max_dev, uint16_t *planes, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(pitch >= cols && pitch % 8 == 0, "pitch must be >= cols and a multiple of 8");
    JETGPU_REQUIRE(plane_stride >= rows * pitch, "plane stride too small");
    JETGPU_REQUIRE(e_max_dev != nullptr, "null exponent pointer");
    if (rows * cols == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in != nullptr && planes != nullptr, "null pointer");
    return PermuteSplitPlanes(in, planes, 1, rank, shape, perm, rows, cols, pitch, plane_stride,
                              0, SplitFormat::kFp16, 0, AsStream(stream), e_max_dev);
}

int jetgpu_gemm_fp16x3(const uint16_t *a_planes, const uint16_t *b_planes, void *C, uint64_t m,
                       uint64_t n, uint64_t k, uint64_t kpitch, const int *e_max_dev,
                       float out_scale, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(C != nullptr && a_planes != nullptr && b_planes != nullptr &&
                       e_max_dev != nullptr,
                   "null pointer");
    return GemmSplitPlanarBatched(a_planes, 0, b_planes, 0, C, 1, m, n, k, kpitch, out_scale,
                                  SplitFormat::kFp16, AsStream(stream), FourPlaneVariant(),
                                  e_max_dev);
}

int jetgpu_split_planes(const void *in, int rank, const uint64_t *shape, const int32_t *perm,
                        uint64_t rows, uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                        int fmt, int extra, const int *e_max_dev, void *planes, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(fmt >= 0 && fmt <= 2, "fmt must be 0 (TF32), 1 (BF16) or 2 (FP16)");
    JETGPU_REQUIRE(extra == kSplitNone || extra == kSplitNegIm || extra == kSplitSum,
                   "extra must be 0, 1 or 2");
    const SplitFormat f = static_cast<SplitFormat>(fmt);
    JETGPU_REQUIRE(pitch >= cols && pitch % SplitPitchAlign(f) == 0,
                   "pitch must be >= cols and span a multiple of 16 bytes");
    JETGPU_REQUIRE(plane_stride >= rows * pitch, "plane stride too small");
    JETGPU_REQUIRE(f != SplitFormat::kFp16 || e_max_dev != nullptr, "null exponent pointer");
    if (rows * cols == 0)
        return JETGPU_OK;
    JETGPU_REQUIRE(in != nullptr && planes != nullptr, "null pointer");
    return PermuteSplitPlanes(in, planes, 1, rank, shape, perm, rows, cols, pitch, plane_stride,
                              0, f, extra, AsStream(stream), e_max_dev);
}

int jetgpu_gemm_split(const void *a_planes, const void *b_planes, void *C, uint64_t m,
                      uint64_t n, uint64_t k, uint64_t kpitch, int fmt, int algo, int variant,
                      const int *e_max_dev, float out_scale, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(fmt >= 0 && fmt <= 2, "fmt must be 0 (TF32), 1 (BF16) or 2 (FP16)");
    JETGPU_REQUIRE(variant == 0 || variant == 1, "variant must be 0 or 1");
    JETGPU_REQUIRE(C != nullptr && a_planes != nullptr && b_planes != nullptr, "null pointer");
    return GemmSplitPlanarBatched(a_planes, 0, b_planes, 0, C, 1, m, n, k, kpitch, out_scale,
                                  static_cast<SplitFormat>(fmt), AsStream(stream), variant,
                                  e_max_dev, 0, nullptr, nullptr, algo);
}

int jetgpu_gemm_bf16x3(const uint16_t *a_planes, const uint16_t *b_planes, void *C, uint64_t m,
                       uint64_t n, uint64_t k, uint64_t kpitch, float out_scale, void *stream)
{
    ClearError();
    JETGPU_REQUIRE(C != nullptr && a_planes != nullptr && b_planes != nullptr, "null pointer");
    return GemmSplitPlanarBatched(a_planes, 0, b_planes, 0, C, 1, m, n, k, kpitch, out_scale,
                                  SplitFormat::kBf16, AsStream(stream), FourPlaneVariant());
}

} // extern "C"

// ---------------------------------------------------------------------------
// Batched contraction (the slice batch of the sliced-network executor).
// ---------------------------------------------------------------------------
namespace jetgpu {
namespace {

struct BatchPlan {
    bool fold;     // A batched, B shared: the batch folds into M
    bool tc;       // tensor-core form
    uint64_t ba;   // tensors of A (batch or 1)
    uint64_t bb;   // tensors of B
};

BatchPlan PlanBatch(uint64_t batch, int a_batched, int b_batched, uint64_t m, uint64_t n,
                    uint64_t k, int dtype, int precision)
{
    BatchPlan p;
    p.fold = batch > 1 && a_batched && !b_batched;
    p.tc = UseTensorCores(p.fold ? batch * m : m, n, k, dtype, precision);
    p.ba = (batch > 1 && a_batched) ? batch : 1;
    p.bb = (batch > 1 && b_batched) ? batch : 1;
    return p;
}

void FoldShape(int rank, const uint64_t *shape, const int32_t *perm, uint64_t batch,
               std::vector<uint64_t> &s, std::vector<int32_t> &pm)
{
    s.assign(1, batch);
    s.insert(s.end(), shape, shape + rank);
    pm.assign(1, 0);
    for (int j = 0; j < rank; ++j)
        pm.push_back(perm[j] + 1);
}

// Workspace of one form (precision FP32, TF32X3, BF16X3, FP16X3 or AUTO).
size_t FormWorkspace(uint64_t batch, int a_rank, const uint64_t *a_shape, const int32_t *a_perm,
                     int a_batched, int b_rank, const uint64_t *b_shape, const int32_t *b_perm,
                     int b_batched, uint64_t m, uint64_t n, uint64_t k, int dtype, int precision,
                     int algo = JETGPU_ALGO_4M)
{
    if (batch <= 1 || (!a_batched && !b_batched)) {
        batch = 1;
        a_batched = b_batched = 0;
    }
    const BatchPlan p = PlanBatch(batch, a_batched, b_batched, m, n, k, dtype, precision);
    if (p.fold) {
        if (a_batched == 2) // the batch axes already lead A's permutation
            return FormWorkspace(1, a_rank, a_shape, a_perm, 0, b_rank, b_shape, b_perm, 0,
                                 batch * m, n, k, dtype, precision, algo);
        std::vector<uint64_t> s;
        std::vector<int32_t> pm;
        FoldShape(a_rank, a_shape, a_perm, batch, s, pm);
        return FormWorkspace(1, a_rank + 1, s.data(), pm.data(), 0, b_rank, b_shape, b_perm, 0,
                             batch * m, n, k, dtype, precision, algo);
    }
    if (p.tc) {
        // Sized for six B planes whatever the main-loop variant.
        const SplitLayout l = LayoutFor(precision, k, (double)batch * m * n * k, -1, 0, algo);
        return l.a_bytes(p.ba * m) + AlignUp(6 * p.bb * n * l.kp * l.word) + l.exp_bytes();
    }
    if (k > 0 && SkinnyApplies(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape,
                               b_perm, b_batched, m, n, k))
        return 0;
    const size_t eb = ElemBytes(dtype);
    size_t ws = 0;
    if (!IsIdentity(a_rank, a_perm))
        ws += AlignUp(p.ba * m * k * eb);
    if (!IsIdentity(b_rank, b_perm))
        ws += AlignUp(p.bb * k * n * eb);
    ws += AlignUp(batch == 1 ? MultiplyPlainWorkspace(m, n, k, dtype)
                             : MultiplyPlainBatchedWorkspace(batch, m, n, k, dtype));
    return ws;
}

} // namespace

size_t ContractWorkspace(uint64_t batch, int a_rank, const uint64_t *a_shape,
                         const int32_t *a_perm, int a_batched, int b_rank,
                         const uint64_t *b_shape, const int32_t *b_perm, int b_batched, uint64_t m,
                         uint64_t n, uint64_t k, int dtype, int precision, int algo)
{
    if (precision != JETGPU_PREC_TUNED)
        return FormWorkspace(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape, b_perm,
                             b_batched, m, n, k, dtype, precision, algo);
    // Any candidate of the tuner, and AUTO (untuned steps).
    size_t ws = 0;
    for (int prec : {JETGPU_PREC_FP32, JETGPU_PREC_AUTO, JETGPU_PREC_TF32X3, JETGPU_PREC_FP16X3}) {
        if (dtype != JETGPU_C64 && prec != JETGPU_PREC_FP32)
            continue;
        const size_t w = FormWorkspace(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape,
                                       b_perm, b_batched, m, n, k, dtype, prec);
        ws = w > ws ? w : ws;
    }
    return ws;
}

int ContractForm(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                 const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                 const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                 uint64_t m, uint64_t n, uint64_t k, int dtype, int precision, int variant,
                 int scale_a, int scale_b, void *workspace, cudaStream_t st, int group_m,
                 const ExpHints *hints, int algo)
{
    if (batch <= 1 || (!a_batched && !b_batched)) {
        batch = 1;
        a_batched = b_batched = 0;
    }
    const BatchPlan p = PlanBatch(batch, a_batched, b_batched, m, n, k, dtype, precision);
    if (p.fold) {
        if (a_batched == 2) // the batch axes already lead A's permutation
            return ContractForm(1, A, a_rank, a_shape, a_perm, 0, B, b_rank, b_shape, b_perm, 0,
                                C, batch * m, n, k, dtype, precision, variant, scale_a, scale_b,
                                workspace, st, group_m, hints, algo);
        std::vector<uint64_t> s;
        std::vector<int32_t> pm;
        FoldShape(a_rank, a_shape, a_perm, batch, s, pm);
        return ContractForm(1, A, a_rank + 1, s.data(), pm.data(), 0, B, b_rank, b_shape, b_perm,
                            0, C, batch * m, n, k, dtype, precision, variant, scale_a, scale_b,
                            workspace, st, group_m, hints, algo);
    }
    uint8_t *ws = static_cast<uint8_t *>(workspace);
    if (k > 0 && p.tc)
        return SplitProduct(LayoutFor(precision, k, (double)batch * m * n * k, variant, group_m,
                                      algo),
                            batch, A, a_rank, a_shape, a_perm, p.ba, p.ba > 1 ? a_batched : 0, B,
                            b_rank, b_shape, b_perm, p.bb, p.bb > 1 ? b_batched : 0, C, m, n, k,
                            dtype, scale_a, scale_b, ws, st, hints);
    if (k > 0 && SkinnyApplies(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape,
                               b_perm, b_batched, m, n, k))
        return SkinnyContract(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape,
                              b_perm, b_batched, C, m, n, k, dtype, scale_a + scale_b, st);
    int rc;
    const size_t eb = ElemBytes(dtype);
    const void *at = A;
    const void *btp = B;
    // Mode 2 operands are one tensor whose permutation leads with the batch.
    if (k > 0 && !IsIdentity(a_rank, a_perm)) {
        if ((rc = PermuteImpl(A, ws, a_batched == 2 ? 1 : p.ba, a_rank, a_shape, a_perm, dtype,
                              st)))
            return rc;
        at = ws;
        ws += AlignUp(p.ba * m * k * eb);
    }
    if (k > 0 && !IsIdentity(b_rank, b_perm)) {
        if ((rc = PermuteImpl(B, ws, b_batched == 2 ? 1 : p.bb, b_rank, b_shape, b_perm, dtype,
                              st)))
            return rc;
        btp = ws;
        ws += AlignUp(p.bb * k * n * eb);
    }
    if (batch == 1) {
        const size_t vec_ws = MultiplyPlainWorkspace(m, n, k, dtype);
        return MultiplyPlain(at, btp, C, m, n, k, dtype, scale_a + scale_b, ws, vec_ws, st);
    }
    const size_t vec_ws = MultiplyPlainBatchedWorkspace(batch, m, n, k, dtype);
    return MultiplyPlainBatched(at, btp, C, batch, p.ba > 1 ? m * k : 0, p.bb > 1 ? k * n : 0, m,
                                n, k, dtype, scale_a + scale_b, vec_ws ? ws : nullptr, vec_ws, st);
}

namespace {

// Argument checks shared by both entry points; JETGPU_OK when the product
// has work to do, a status otherwise (*empty set when m n = 0).
int CheckContract(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                  const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                  const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                  uint64_t m, uint64_t n, uint64_t k, int dtype, int precision, int algo,
                  void *workspace, size_t workspace_bytes, bool *empty)
{
    *empty = false;
    JETGPU_REQUIRE(dtype == JETGPU_C64 || dtype == JETGPU_C128, "bad dtype");
    JETGPU_REQUIRE(precision >= JETGPU_PREC_FP32 && precision <= JETGPU_PREC_TUNED,
                   "bad precision");
    JETGPU_REQUIRE(algo == JETGPU_ALGO_4M || algo == JETGPU_ALGO_3M, "bad algorithm");
    const bool split_form = precision == JETGPU_PREC_TF32X3 || precision == JETGPU_PREC_BF16X3 ||
                            precision == JETGPU_PREC_FP16X3;
    if (split_form && dtype != JETGPU_C64)
        return SetError(JETGPU_ERR_UNSUPPORTED, "split precision needs complex64 operands");
    if (algo == JETGPU_ALGO_3M && (!split_form || batch > 1))
        return SetError(JETGPU_ERR_UNSUPPORTED,
                        "the 3M product is available for single contractions in the TF32X3, "
                        "BF16X3 and FP16X3 forms");
    JETGPU_REQUIRE(a_batched >= 0 && a_batched <= 2 && b_batched >= 0 && b_batched <= 2,
                   "batched flags must be 0, 1 or 2");
    // Mode 2: the operand is one tensor whose permutation leads with axes of
    // total extent `batch` (the batch), then its (left ++ common) or
    // (common ++ right) axes.
    const uint64_t a_lead = (batch > 1 && a_batched == 2) ? batch : 1;
    const uint64_t b_lead = (batch > 1 && b_batched == 2) ? batch : 1;
    int rc = Validate(a_rank, a_shape, a_perm, a_lead * m, k, "A");
    if (rc)
        return rc;
    if ((rc = Validate(b_rank, b_shape, b_perm, b_lead * k, n, "B")))
        return rc;
    JETGPU_REQUIRE(SplitPoint(a_rank, a_shape, a_perm, a_lead) >= 0 &&
                       SplitPoint(b_rank, b_shape, b_perm, b_lead) >= 0,
                   "permutation does not lead with the batch axes");
    if (m * n == 0) {
        *empty = true;
        return JETGPU_OK;
    }
    JETGPU_REQUIRE(C != nullptr, "null output");
    JETGPU_REQUIRE(k == 0 || (A != nullptr && B != nullptr), "null operand");
    const size_t need = ContractWorkspace(batch, a_rank, a_shape, a_perm, a_batched, b_rank,
                                          b_shape, b_perm, b_batched, m, n, k, dtype, precision,
                                          algo);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return SetError(JETGPU_ERR_WORKSPACE,
                        "workspace too small: need " + std::to_string(need) + " bytes");
    return JETGPU_OK;
}

int Contract(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
             const int32_t *a_perm, int a_batched, const void *B, int b_rank,
             const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C, uint64_t m,
             uint64_t n, uint64_t k, int dtype, int precision, int algo, int scale_a, int scale_b,
             void *workspace, size_t workspace_bytes, cudaStream_t st,
             const ExpHints *hints = nullptr)
{
    bool empty = false;
    int rc = CheckContract(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape,
                           b_perm, b_batched, C, m, n, k, dtype, precision, algo, workspace,
                           workspace_bytes, &empty);
    if (rc)
        return rc;
    if (hints != nullptr && hints->c != nullptr) // unrecorded until a product records it
        JETGPU_CUDA_TRY(cudaMemsetAsync(hints->c, 0x80, sizeof(int), st));
    if (empty)
        return JETGPU_OK;
    if (precision == JETGPU_PREC_TUNED)
        return ContractTuned(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape,
                             b_perm, b_batched, C, m, n, k, dtype, scale_a, scale_b, workspace,
                             st, hints);
    return ContractForm(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape, b_perm,
                        b_batched, C, m, n, k, dtype, precision, -1, scale_a, scale_b, workspace,
                        st, 0, hints, algo);
}

} // namespace
} // namespace jetgpu

extern "C" {

size_t jetgpu_contract_workspace_size(int a_rank, const uint64_t *a_shape,
                                      const int32_t *a_perm, int b_rank,
                                      const uint64_t *b_shape, const int32_t *b_perm,
                                      uint64_t m, uint64_t n, uint64_t k, int dtype,
                                      int precision)
{
    return ContractWorkspace(1, a_rank, a_shape, a_perm, 0, b_rank, b_shape, b_perm, 0, m, n, k,
                             dtype, precision);
}

int jetgpu_contract(const void *A, int a_rank, const uint64_t *a_shape,
                    const int32_t *a_perm, const void *B, int b_rank,
                    const uint64_t *b_shape, const int32_t *b_perm, void *C,
                    uint64_t m, uint64_t n, uint64_t k, int dtype, int precision,
                    int algo, int scale_a, int scale_b, void *workspace,
                    size_t workspace_bytes, void *stream)
{
    NvtxRange range("jetgpu_contract");
    ClearError();
    return Contract(1, A, a_rank, a_shape, a_perm, 0, B, b_rank, b_shape, b_perm, 0, C, m, n, k,
                    dtype, precision, algo, scale_a, scale_b, workspace, workspace_bytes,
                    AsStream(stream));
}

size_t jetgpu_contract_workspace_size_algo(int a_rank, const uint64_t *a_shape,
                                           const int32_t *a_perm, int b_rank,
                                           const uint64_t *b_shape, const int32_t *b_perm,
                                           uint64_t m, uint64_t n, uint64_t k, int dtype,
                                           int precision, int algo)
{
    return ContractWorkspace(1, a_rank, a_shape, a_perm, 0, b_rank, b_shape, b_perm, 0, m, n, k,
                             dtype, precision, algo);
}

size_t jetgpu_contract_batched_workspace_size(uint64_t batch, int a_rank, const uint64_t *a_shape,
                                              const int32_t *a_perm, int a_batched, int b_rank,
                                              const uint64_t *b_shape, const int32_t *b_perm,
                                              int b_batched, uint64_t m, uint64_t n, uint64_t k,
                                              int dtype, int precision)
{
    return ContractWorkspace(batch, a_rank, a_shape, a_perm, a_batched, b_rank, b_shape, b_perm,
                             b_batched, m, n, k, dtype, precision);
}

int jetgpu_contract_batched(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                            const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                            const uint64_t *b_shape, const int32_t *b_perm, int b_batched,
                            void *C, uint64_t m, uint64_t n, uint64_t k, int dtype, int precision,
                            int algo, int scale_a, int scale_b, void *workspace,
                            size_t workspace_bytes, void *stream)
{
    NvtxRange range("jetgpu_contract_batched");
    ClearError();
    JETGPU_REQUIRE(batch >= 1, "batch must be at least 1");
    JETGPU_REQUIRE(batch == 1 || a_batched || b_batched,
                   "a batch needs at least one batched operand");
    return Contract(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape, b_perm,
                    b_batched, C, m, n, k, dtype, precision, algo, scale_a, scale_b, workspace,
                    workspace_bytes, AsStream(stream));
}

int jetgpu_contract_batched_hinted(uint64_t batch, const void *A, int a_rank,
                                   const uint64_t *a_shape, const int32_t *a_perm, int a_batched,
                                   const void *B, int b_rank, const uint64_t *b_shape,
                                   const int32_t *b_perm, int b_batched, void *C, uint64_t m,
                                   uint64_t n, uint64_t k, int dtype, int precision, int algo,
                                   const int *a_emax, const int *b_emax, int *c_emax,
                                   void *workspace, size_t workspace_bytes, void *stream)
{
    NvtxRange range("jetgpu_contract_batched_hinted");
    ClearError();
    JETGPU_REQUIRE(batch >= 1, "batch must be at least 1");
    JETGPU_REQUIRE(batch == 1 || a_batched || b_batched,
                   "a batch needs at least one batched operand");
    ExpHints hints;
    hints.a = a_emax;
    hints.b = b_emax;
    hints.c = c_emax;
    return Contract(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape, b_perm,
                    b_batched, C, m, n, k, dtype, precision, algo, 0, 0, workspace,
                    workspace_bytes, AsStream(stream), &hints);
}

} // extern "C"
