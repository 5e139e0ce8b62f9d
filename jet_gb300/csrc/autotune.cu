// Autotuner of the contraction form (JETGPU_PREC_TUNED).
//
// The reference contracts every path step with one BLAS call
// (TensorHelpers::MultiplyTensorData, TensorHelpers.hpp:128-168), so it has
// nothing to choose. Here a step can run as the plain FP32 product or as a
// tensor-core split product (TF32x3 with either main loop, FP16x3 in the
// grouped or the row-major tile order), all within the same error bound, and
// which is fastest depends on the step's shape, batch and operand
// permutations (the permute passes differ per form; the tile order decides
// how the operands are shared through L2 and where in memory the tiles in
// flight write).
//
// The first contraction with a given key -- device, batch, which operands are
// batched, m, n, k, dtype, and both operands' shapes and permutations -- runs
// every candidate once untimed (a first launch configures its kernels), then
// times it with CUDA events on the caller's stream, and keeps the fastest in
// a table; later contractions with that key run the kept form directly,
// including inside a stream capture. Candidates are tried fastest-expected
// first, and one whose untimed run already took more than twice the best
// time so far is not timed. Steps below a work threshold (m n k times the
// batch; jetgpu_set_autotune_min_work) and contractions met first during a
// capture take AUTO's fixed rule instead, without an entry.
#include <atomic>
#include <cfloat>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace jetgpu {
namespace {

constexpr int kCandidates = JETGPU_AUTOTUNE_CANDIDATES;
struct Candidate {
    int precision;
    int variant; // tensor-core main loop
    int group_m; // tile order: tile rows per group (0: the setting, 8 by default)
};
// Reporting order (jetgpu_autotune_entry's times).
constexpr Candidate kCandidate[kCandidates] = {{JETGPU_PREC_FP32, -1, 0},
                                               {JETGPU_PREC_TF32X3, 0, 0},
                                               {JETGPU_PREC_TF32X3, 1, 0},
                                               {JETGPU_PREC_FP16X3, 0, 0},
                                               {JETGPU_PREC_FP16X3, 0, 1},
                                               {JETGPU_PREC_FP16X3, 1, 0}};
// Trial order: fastest expected first, so the slow forms are cut short.
constexpr int kTrialOrder[kCandidates] = {3, 5, 4, 1, 2, 0};

struct Entry {
    uint64_t batch, m, n, k;
    int choice; // index into kCandidate
    float ms[kCandidates];
};

std::mutex g_mutex;
std::map<std::vector<int64_t>, size_t> g_index; // key -> position in g_entries
std::vector<Entry> g_entries;
std::atomic<uint64_t> g_min_work{1ull << 20};

std::vector<int64_t> Key(uint64_t batch, int a_rank, const uint64_t *a_shape,
                         const int32_t *a_perm, int a_batched, int b_rank,
                         const uint64_t *b_shape, const int32_t *b_perm, int b_batched,
                         uint64_t m, uint64_t n, uint64_t k, int dtype)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        dev = -1;
    std::vector<int64_t> key{dev,          (int64_t)batch, a_batched, b_batched, (int64_t)m,
                             (int64_t)n,   (int64_t)k,     dtype,     a_rank,    b_rank};
    for (int i = 0; i < a_rank; ++i) {
        key.push_back((int64_t)a_shape[i]);
        key.push_back(a_perm[i]);
    }
    for (int i = 0; i < b_rank; ++i) {
        key.push_back((int64_t)b_shape[i]);
        key.push_back(b_perm[i]);
    }
    return key;
}

bool Capturing(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError(); // not sticky; treat as capturing
        return true;
    }
    return cs != cudaStreamCaptureStatusNone;
}

// Elapsed ms between two events recorded on `st` around `reps` runs of `run`.
template <class F> int Time(F run, int reps, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1,
                           float *ms)
{
    JETGPU_CUDA_TRY(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) {
        const int rc = run();
        if (rc)
            return rc;
    }
    JETGPU_CUDA_TRY(cudaEventRecord(e1, st));
    JETGPU_CUDA_TRY(cudaEventSynchronize(e1));
    float t = 0;
    JETGPU_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / reps;
    return JETGPU_OK;
}

struct Events {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Events()
    {
        if (e0)
            cudaEventDestroy(e0);
        if (e1)
            cudaEventDestroy(e1);
    }
};

} // namespace

int ContractTuned(uint64_t batch, const void *A, int a_rank, const uint64_t *a_shape,
                  const int32_t *a_perm, int a_batched, const void *B, int b_rank,
                  const uint64_t *b_shape, const int32_t *b_perm, int b_batched, void *C,
                  uint64_t m, uint64_t n, uint64_t k, int dtype, int scale_a, int scale_b,
                  void *workspace, cudaStream_t st, const ExpHints *hints)
{
    if (batch <= 1 || (!a_batched && !b_batched)) {
        batch = 1;
        a_batched = b_batched = 0;
    }
    // Trials read the operand hints but record no exponent of C: only the
    // run whose result is kept does.
    ExpHints trial;
    if (hints != nullptr) {
        trial.a = hints->a;
        trial.b = hints->b;
    }
    auto run_with = [&](int precision, int variant, int group_m, const ExpHints *h) {
        return ContractForm(batch, A, a_rank, a_shape, a_perm, a_batched, B, b_rank, b_shape,
                            b_perm, b_batched, C, m, n, k, dtype, precision, variant, scale_a,
                            scale_b, workspace, st, group_m, h);
    };
    auto run = [&](int precision, int variant, int group_m = 0) {
        return run_with(precision, variant, group_m, hints);
    };
    if (dtype != JETGPU_C64)
        return run(JETGPU_PREC_FP32, -1);
    const uint64_t m_eff = (a_batched && !b_batched) ? batch * m : m;
    const double work = (double)batch * (double)m * (double)n * (double)k;
    if (k == 0 || m_eff < 2 || n < 2 || work < (double)g_min_work.load() || !TcAvailable())
        return run(JETGPU_PREC_AUTO, -1);

    const std::vector<int64_t> key = Key(batch, a_rank, a_shape, a_perm, a_batched, b_rank,
                                         b_shape, b_perm, b_batched, m, n, k, dtype);
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        const auto it = g_index.find(key);
        if (it != g_index.end()) {
            const Candidate c = kCandidate[g_entries[it->second].choice];
            return run(c.precision, c.variant, c.group_m);
        }
    }
    if (Capturing(st))
        return run(JETGPU_PREC_AUTO, -1);

    Events ev;
    JETGPU_CUDA_TRY(cudaEventCreate(&ev.e0));
    JETGPU_CUDA_TRY(cudaEventCreate(&ev.e1));
    Entry e{batch, m, n, k, -1, {}};
    for (int c = 0; c < kCandidates; ++c)
        e.ms[c] = -1.f;
    float best = FLT_MAX;
    int last = -1;
    for (int t = 0; t < kCandidates; ++t) {
        const int ci = kTrialOrder[t];
        const Candidate c = kCandidate[ci];
        auto once = [&] { return run_with(c.precision, c.variant, c.group_m, &trial); };
        float first = 0;
        int rc = Time(once, 1, st, ev.e0, ev.e1, &first);
        if (rc != JETGPU_OK) {
            // A form this contraction cannot take (e.g. an FP16 scale out of
            // range) is skipped; a CUDA error is the caller's.
            if (rc == JETGPU_ERR_CUDA)
                return rc;
            ClearError();
            continue;
        }
        last = ci;
        if (first > 2.0f * best)
            continue; // clearly slower even with its set-up cost removed
        float ms = 0;
        if ((rc = Time(once, first < 1.0f ? 4 : 1, st, ev.e0, ev.e1, &ms)))
            return rc;
        e.ms[ci] = ms;
        if (ms < best) {
            best = ms;
            e.choice = ci;
        }
    }
    if (e.choice < 0)
        return SetError(JETGPU_ERR_UNSUPPORTED, "no contraction form accepted these operands");
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (g_index.find(key) == g_index.end()) {
            g_index.emplace(key, g_entries.size());
            g_entries.push_back(e);
        }
    }
    ClearError();
    if (last == e.choice && (hints == nullptr || hints->c == nullptr))
        return JETGPU_OK; // C holds the chosen form's result
    const Candidate c = kCandidate[e.choice];
    return run(c.precision, c.variant, c.group_m);
}

} // namespace jetgpu

using namespace jetgpu;

extern "C" {

int jetgpu_set_autotune_min_work(uint64_t mnk)
{
    ClearError();
    g_min_work.store(mnk);
    return JETGPU_OK;
}

size_t jetgpu_autotune_count(void)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    return g_entries.size();
}

int jetgpu_autotune_entry(size_t index, uint64_t *batch_m_n_k, int *precision, int *variant,
                          int *group_m, float *times_ms)
{
    ClearError();
    std::lock_guard<std::mutex> lock(g_mutex);
    JETGPU_REQUIRE(index < g_entries.size(), "autotune entry index out of range");
    const Entry &e = g_entries[index];
    if (batch_m_n_k) {
        batch_m_n_k[0] = e.batch;
        batch_m_n_k[1] = e.m;
        batch_m_n_k[2] = e.n;
        batch_m_n_k[3] = e.k;
    }
    if (precision)
        *precision = kCandidate[e.choice].precision;
    if (variant)
        *variant = kCandidate[e.choice].variant < 0 ? 0 : kCandidate[e.choice].variant;
    if (group_m)
        *group_m = kCandidate[e.choice].group_m;
    if (times_ms)
        for (int i = 0; i < kCandidates; ++i)
            times_ms[i] = e.ms[i];
    return JETGPU_OK;
}

int jetgpu_autotune_clear(void)
{
    ClearError();
    std::lock_guard<std::mutex> lock(g_mutex);
    g_index.clear();
    g_entries.clear();
    return JETGPU_OK;
}

} // extern "C"
