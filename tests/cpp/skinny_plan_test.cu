// Host-side check of the skinny contraction's launch parameters
// (jet_gb300/csrc/skinny.cu): for random operand shapes (dims 1..4, ranks up
// to 15, gate-like small operands), random axis orders and all three batch
// modes of each operand, the offsets the kernels compute -- the row digits by
// 32-bit multiply-shift division over the merged free axes, the tabulated
// contracted and small-operand offsets, the batch offsets and C's strides --
// are replayed on the CPU and compared with the offsets of the permuted
// operands computed directly (row-major tensor, axis order
// (batch) (left ++ common) for A and (batch) (common ++ right) for B, the
// layout jetgpu_contract_batched defines). Every offset is also checked to
// lie inside its tensor. No GPU is used.
#include "../../jet_gb300/csrc/skinny.cu"

#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

using namespace jetgpu;

namespace {

#define FAIL(...)                                                                                  \
    do {                                                                                           \
        std::printf(__VA_ARGS__);                                                                  \
        return 1;                                                                                  \
    } while (0)

uint32_t Div(uint32_t n, uint32_t m, uint32_t s)
{
    if (m == 0)
        return n;
    const uint32_t t = (uint32_t)(((uint64_t)n * m) >> 32);
    return (t + ((n - t) >> 1)) >> s;
}

uint64_t Axes(const SkAxes &a, uint64_t idx)
{
    uint64_t off = 0;
    for (int i = 0; i < a.n; ++i) {
        off += (idx % a.dim[i]) * a.stride[i];
        idx /= a.dim[i];
    }
    return off;
}

// The kernels' row offset (RowOffset): 32-bit multiply-shift digits.
int Row(const SkinnyParams &p, uint64_t r, uint64_t &off)
{
    if (!p.narrow) {
        off = Axes(p.row, r);
        return 0;
    }
    uint32_t x = (uint32_t)r;
    off = 0;
    for (int i = 0; i < p.row.n; ++i) {
        const uint32_t q = Div(x, p.row_magic[i], p.row_shift[i]);
        if (q != x / (uint32_t)p.row.dim[i])
            FAIL("row digit division\n");
        off += (uint64_t)(x - q * (uint32_t)p.row.dim[i]) * p.row.stride[i];
        x = q;
    }
    return 0;
}

// Element offset of multi-index `idx` over axes `order` (outermost first) of
// a row-major tensor of `shape`; `flat` is the index in that order.
uint64_t Offset(const std::vector<uint64_t> &shape, const std::vector<int> &order, uint64_t flat)
{
    std::vector<uint64_t> st(shape.size(), 1);
    for (int i = (int)shape.size() - 2; i >= 0; --i)
        st[i] = st[i + 1] * shape[i + 1];
    uint64_t off = 0;
    for (int i = (int)order.size() - 1; i >= 0; --i) {
        off += (flat % shape[order[i]]) * st[order[i]];
        flat /= shape[order[i]];
    }
    return off;
}

struct Operand {
    std::vector<uint64_t> shape; // of the tensor as stored (mode 2: with its batch axes)
    std::vector<int32_t> perm;   // (batch) (first) (second)
    int nb = 0, n1 = 0;          // axes in the batch group, in the first group
    uint64_t size = 1;           // elements of one stored tensor
};

// A random operand: `batch_dims` (mode 2 only), first / second group dims.
Operand Make(std::mt19937 &rng, const std::vector<uint64_t> &bdims,
             const std::vector<uint64_t> &g1, const std::vector<uint64_t> &g2)
{
    Operand o;
    std::vector<uint64_t> dims(bdims);
    dims.insert(dims.end(), g1.begin(), g1.end());
    dims.insert(dims.end(), g2.begin(), g2.end());
    const int r = (int)dims.size();
    std::vector<int> pos(r);
    for (int i = 0; i < r; ++i)
        pos[i] = i;
    std::shuffle(pos.begin(), pos.end(), rng); // logical axis i is stored at pos[i]
    o.shape.assign(r, 1);
    for (int i = 0; i < r; ++i)
        o.shape[pos[i]] = dims[i];
    o.perm.assign(pos.begin(), pos.end());
    o.nb = (int)bdims.size();
    o.n1 = (int)g1.size();
    for (auto d : o.shape)
        o.size *= d;
    return o;
}

uint64_t Prod(const std::vector<uint64_t> &v)
{
    uint64_t p = 1;
    for (auto d : v)
        p *= d;
    return p;
}

std::vector<uint64_t> Dims(std::mt19937 &rng, int n, int lo, int hi)
{
    std::uniform_int_distribution<int> d(lo, hi);
    std::vector<uint64_t> v(n);
    for (auto &x : v)
        x = (uint64_t)d(rng);
    return v;
}

// Expected offset of element (b, x, y) of an operand whose groups are
// (first: x, second: y) in its permutation; mode 1 adds b * size.
uint64_t Expect(const Operand &o, int mode, uint64_t b, uint64_t x, uint64_t y,
                uint64_t e1, uint64_t e2)
{
    const std::vector<int> order(o.perm.begin(), o.perm.end());
    if (mode == 2) // the batch axes lead the permutation
        return Offset(o.shape, order, (b * e1 + x) * e2 + y);
    return (mode == 1 ? b * o.size : 0) + Offset(o.shape, order, x * e2 + y);
}

int Check(std::mt19937 &rng, int a_mode, int b_mode, bool big_a, int trial)
{
    const uint64_t batch = (a_mode || b_mode) ? (uint64_t)(2 + trial % 3) : 1;
    // Batch axes of a mode-2 operand: `batch` split into 1 or 2 axes.
    auto batch_axes = [&](int mode) {
        std::vector<uint64_t> v;
        if (mode != 2)
            return v;
        if (batch == 4 && trial % 2)
            v = {2, 2};
        else
            v = {batch};
        return v;
    };
    const int big_rank = 2 + (int)(rng() % 9), small_free = 1 + (int)(rng() % 2);
    const int common_rank = 1 + (int)(rng() % 3);
    auto bigfree = Dims(rng, big_rank, 1, 4);
    auto common = Dims(rng, common_rank, 1, 4);
    auto smallfree = Dims(rng, small_free, 1, 4);
    if (Prod(smallfree) > 16 || Prod(common) > 64)
        return 2; // not a skinny shape
    const auto &left = big_a ? bigfree : smallfree;
    const auto &right = big_a ? smallfree : bigfree;
    const uint64_t m = Prod(left), n = Prod(right), k = Prod(common);
    if (std::min(m, n) > 16 || (big_a ? m < n : n <= m) || batch * m * n * k > 1000000)
        return 2;
    Operand A = Make(rng, batch_axes(a_mode), left, common);
    Operand B = Make(rng, batch_axes(b_mode), common, right);
    SkinnyParams p;
    bool big_is_a = false;
    if (!Plan(batch, (int)A.shape.size(), A.shape.data(), A.perm.data(), a_mode,
              (int)B.shape.size(), B.shape.data(), B.perm.data(), b_mode, m, n, k, p, big_is_a))
        return 2; // more than the index tables hold: the transposing path runs
    if (big_is_a != big_a)
        FAIL("trial %d: large operand %d, expected %d\n", trial, big_is_a, big_a);
    const uint64_t a_total = A.size * (a_mode == 1 ? batch : 1);
    const uint64_t b_total = B.size * (b_mode == 1 ? batch : 1);
    for (uint64_t b = 0; b < batch; ++b)
        for (uint64_t r = 0; r < p.rows; ++r) {
            uint64_t roff;
            if (Row(p, r, roff))
                return 1;
            const uint64_t big_base = Axes(p.big_b, b) + roff;
            for (uint64_t c = 0; c < k; ++c)
                for (uint64_t j = 0; j < (uint64_t)p.s; ++j) {
                    const uint64_t got_big = big_base + p.coff[c];
                    const uint64_t got_small = Axes(p.small_b, b) + p.s_coff[c] + p.s_foff[j];
                    // (i, c) of A and (c, j) of B in the product's view.
                    const uint64_t i = big_a ? r : j, jj = big_a ? j : r;
                    const uint64_t want_a = Expect(A, a_mode, b, i, c, m, k);
                    const uint64_t want_b = Expect(B, b_mode, b, c, jj, k, n);
                    const uint64_t got_a = big_a ? got_big : got_small;
                    const uint64_t got_b = big_a ? got_small : got_big;
                    if (got_a != want_a || got_b != want_b)
                        FAIL("trial %d (modes %d %d, big %s): b %llu r %llu c %llu j %llu: A %llu/%llu B "
                             "%llu/%llu\n",
                             trial, a_mode, b_mode, big_a ? "A" : "B", (unsigned long long)b,
                             (unsigned long long)r, (unsigned long long)c,
                             (unsigned long long)j, (unsigned long long)got_a,
                             (unsigned long long)want_a, (unsigned long long)got_b,
                             (unsigned long long)want_b);
                    if (got_a >= a_total || got_b >= b_total)
                        FAIL("trial %d: offset outside its operand\n", trial);
                }
            // C: batch x m x n row-major.
            for (uint64_t j = 0; j < (uint64_t)p.s; ++j) {
                const uint64_t i = big_a ? r : j, jj = big_a ? j : r;
                const uint64_t got = b * p.out_batch + r * p.out_row + j * p.out_col;
                if (got != (b * m + i) * n + jj)
                    FAIL("trial %d: C offset\n", trial);
            }
        }
    return 0;
}

} // namespace

int main()
{
    std::mt19937 rng(20240601);
    int checked = 0;
    for (int trial = 0; trial < 1800; ++trial) {
        const int a_mode = trial % 3, b_mode = (trial / 3) % 3;
        const bool big_a = (trial / 9) % 2 == 0;
        const int rc = Check(rng, a_mode, b_mode, big_a, trial);
        if (rc == 1)
            return 1;
        checked += rc == 0;
    }
    if (checked < 300) {
        std::printf("only %d skinny plans checked\n", checked);
        return 1;
    }
    std::printf("ok %d plans\n", checked);
    return 0;
}
