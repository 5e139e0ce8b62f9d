// Host-side check of the tiled permute's plan (jet_gb300/csrc/permute.cu):
// the kernel's passes are replayed on the CPU over random shapes (dims 1..10,
// ranks 1..6, batches 1..3; then fixed qutrit-sized shapes up to 3^12 with
// batches of 2) and both element sizes, with input element i
// holding i, and the result compared with the plain row-major permutation
// (output axis j = input axis perm[j], the convention of the reference's
// Permuter, include/jet/permute/Permuter.hpp:36-80). The replay checks every
// shared-memory slot and global offset against its buffer, that no output is
// written twice, and that the 32-bit multiply-shift divisions the kernel uses
// equal plain division.
#include "../../jet_gb300/csrc/permute.cu"

#include <algorithm>
#include <cstdio>
#include <random>

using namespace jetgpu;

namespace {

uint32_t Div(uint32_t n, uint32_t m, uint32_t s)
{
    if (m == 0)
        return n;
    const uint32_t t = (uint32_t)(((uint64_t)n * m) >> 32);
    return (t + ((n - t) >> 1)) >> s;
}

#define FAIL(...)                                                                                  \
    do {                                                                                           \
        std::printf(__VA_ARGS__);                                                                  \
        return 1;                                                                                  \
    } while (0)

int Replay(const TileParams &tp, size_t eb, uint64_t total, std::vector<uint64_t> &got)
{
    const size_t slots = kTileSlotBytes / eb;
    if (tp.T < 1 || tp.T > kTileMax || tp.G < 1 || tp.G > kTileGroupMax ||
        (size_t)tp.G * tp.T > slots)
        FAIL("bad tile shape T=%d G=%d\n", tp.T, tp.G);
    if (!tp.narrow)
        FAIL("expected the 32-bit tile decode\n");
    std::vector<uint64_t> tile(slots), bin(tp.G), bout(tp.G);
    const uint64_t passes = (tp.tiles + tp.G - 1) / tp.G;
    for (uint64_t ps = 0; ps < passes; ++ps) {
        const uint64_t t0 = ps * tp.G;
        const int g = (int)std::min<uint64_t>(tp.G, tp.tiles - t0);
        for (int j = 0; j < g; ++j) {
            uint64_t bi = 0, bo = 0;
            uint32_t x = (uint32_t)(t0 + j);
            for (int a = tp.nr - 1; a >= 0; --a) {
                const uint32_t q = Div(x, tp.r_magic[a], tp.r_shift[a]);
                if (q != x / tp.r_dims[a])
                    FAIL("tile decode division\n");
                const uint64_t c = x - q * (uint32_t)tp.r_dims[a];
                bi += c * tp.r_in[a];
                bo += c * tp.r_out[a];
                x = q;
            }
            bin[j] = bi;
            bout[j] = bo;
        }
        const int n = g * tp.T;
        for (int u = 0; u < n; ++u) {
            const int j = (int)Div((uint32_t)u, tp.t_magic, tp.t_shift);
            if (j != u / tp.T)
                FAIL("slot division\n");
            const int e = u - j * tp.T;
            const uint64_t src = bin[j] + (uint64_t)tp.in_off[e];
            const size_t slot = (size_t)j * tp.T + tp.pos[e];
            if (src >= total || tp.pos[e] >= tp.T || slot >= slots)
                FAIL("read out of range\n");
            tile[slot] = src;
        }
        for (int u = 0; u < n; ++u) {
            const int j = (int)Div((uint32_t)u, tp.t_magic, tp.t_shift);
            const int f = u - j * tp.T;
            const uint64_t dst = bout[j] + (uint64_t)tp.out_off[f];
            if (dst >= total)
                FAIL("write out of range\n");
            if (got[dst] != ~0ull)
                FAIL("output %llu written twice\n", (unsigned long long)dst);
            got[dst] = tile[u];
        }
    }
    return 0;
}

} // namespace

// 1: planned and replayed equal to the plain permutation; 0: no plan; -1: failure.
int Check(const std::vector<uint64_t> &shape, const std::vector<int32_t> &perm, uint64_t batch,
          size_t eb)
{
    static TileParams tp;
    const int rank = (int)shape.size();
    uint64_t size = 1;
    for (uint64_t d : shape)
        size *= d;
    Simplified s;
    if (Simplify(rank, shape.data(), perm.data(), s)) {
        std::printf("simplify failed\n");
        return -1;
    }
    if (!PlanTile(s, rank, shape.data(), perm.data(), batch, eb, tp))
        return 0;
    std::vector<uint64_t> ref(size * batch), got(size * batch, ~0ull);
    std::vector<uint64_t> stride(rank, 1);
    for (int i = rank - 2; i >= 0; --i)
        stride[i] = stride[i + 1] * shape[i + 1];
    for (uint64_t b = 0; b < batch; ++b)
        for (uint64_t o = 0; o < size; ++o) {
            uint64_t x = o, src = 0;
            for (int j = rank - 1; j >= 0; --j) {
                src += (x % shape[perm[j]]) * stride[perm[j]];
                x /= shape[perm[j]];
            }
            ref[b * size + o] = b * size + src;
        }
    if (Replay(tp, eb, size * batch, got))
        return -1;
    if (got != ref) {
        std::printf("mismatch\n");
        return -1;
    }
    return 1;
}

int main()
{
    std::mt19937_64 rng(7);
    int planned = 0, cases = 0;
    for (int trial = 0; trial < 3000; ++trial) {
        const int rank = 1 + (int)(rng() % 6);
        std::vector<uint64_t> shape(rank);
        uint64_t size = 1;
        for (auto &d : shape) {
            d = 1 + rng() % 10;
            size *= d;
        }
        if (size > 200000)
            continue;
        std::vector<int32_t> perm(rank);
        for (int i = 0; i < rank; ++i)
            perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), rng);
        const uint64_t batch = 1 + rng() % 3;
        const size_t eb = (trial & 1) ? 8 : 16;
        ++cases;
        const int rc = Check(shape, perm, batch, eb);
        if (rc < 0)
            FAIL("  (trial %d)\n", trial);
        planned += rc;
    }
    if (planned < cases / 2)
        FAIL("only %d of %d cases planned\n", planned, cases);
    // Sizes the GPU runs take: qutrit and other uniform radices (729- and
    // 81-element tiles, several per pass), random permutations, both
    // element sizes, with and without a batch. Axes that stay adjacent and in
    // order are merged first; where the merged axes leave no tile of at most
    // 1024 elements, the original axes must give one for radices 3, 5 and 9.
    // Radix 6 may have none: two axes (36) are needed on each side to reach 8,
    // and 36 x 36 > 1024; mixed radices likewise (e.g. 7 x 4 against 4 x 11).
    struct Big {
        std::vector<uint64_t> shape;
        bool must_plan;
    };
    const std::vector<Big> big = {{std::vector<uint64_t>(12, 3), true},
                                  {std::vector<uint64_t>(6, 9), true},
                                  {std::vector<uint64_t>(8, 5), true},
                                  {std::vector<uint64_t>(7, 6), false},
                                  {{9, 5, 7, 3, 11, 4, 7}, false}};
    int big_cases = 0, big_planned = 0;
    for (const auto &b : big)
        for (int rep = 0; rep < 8; ++rep) {
            std::vector<int32_t> perm(b.shape.size());
            for (size_t i = 0; i < perm.size(); ++i)
                perm[i] = (int32_t)i;
            std::shuffle(perm.begin(), perm.end(), rng);
            const int rc = Check(b.shape, perm, 1 + (rep & 1), (rep & 2) ? 16 : 8);
            if (rc < 0 || (rc == 0 && b.must_plan))
                FAIL("large case %d of shape %zu axes: %s\n", rep, b.shape.size(),
                     rc < 0 ? "failed" : "no plan");
            ++big_cases;
            big_planned += rc;
        }
    // Blocks of axes that stay in order: merged, they are too long for a tile
    // on both sides, so the plan comes from the original axes (the cases of
    // the GPU test test_merged_axes_tiled_on_original_axes_vs_oracle).
    struct Fixed {
        std::vector<uint64_t> shape;
        std::vector<int32_t> perm;
        uint64_t batch;
        size_t eb;
    };
    const std::vector<Fixed> fixed = {
        {std::vector<uint64_t>(12, 3), {8, 9, 10, 11, 4, 5, 6, 7, 0, 1, 2, 3}, 1, 8},
        {std::vector<uint64_t>(12, 3), {8, 9, 10, 11, 4, 5, 6, 7, 0, 1, 2, 3}, 2, 16},
        {std::vector<uint64_t>(12, 3), {6, 7, 8, 9, 10, 11, 0, 1, 2, 3, 4, 5}, 1, 8},
        {std::vector<uint64_t>(6, 9), {3, 4, 5, 0, 1, 2}, 1, 8}};
    for (size_t c = 0; c < fixed.size(); ++c) {
        const Fixed &f = fixed[c];
        Simplified s;
        if (Simplify((int)f.shape.size(), f.shape.data(), f.perm.data(), s))
            FAIL("simplify failed\n");
        static TileParams merged;
        if (BuildTile(s, f.batch, f.eb, merged))
            FAIL("fixed case %zu: expected no tile on the merged axes\n", c);
        if (Check(f.shape, f.perm, f.batch, f.eb) != 1)
            FAIL("fixed case %zu: no plan or failed\n", c);
    }
    // A plan on the original axes of a rank-58 tensor with a batch of 2 (the
    // second try of PlanTile): the batch and every axis outside the tile
    // enumerate the tiles, and must fit the plan's kMaxRank + 1 entries. Too
    // large to replay; the plan's tiles must cover the tensor exactly.
    {
        std::vector<uint64_t> shape = {3, 3};
        shape.insert(shape.end(), 56, 2);
        const int rank = (int)shape.size();
        std::vector<int32_t> perm(rank);
        for (int i = 0; i < rank; ++i)
            perm[i] = i;
        std::reverse(perm.end() - 6, perm.end());
        Simplified u;
        Unmerged(rank, shape.data(), perm.data(), u);
        static TileParams tp;
        if ((int)u.dims.size() != rank || !BuildTile(u, 2, 8, tp))
            FAIL("rank-%d plan on the original axes: none\n", rank);
        if (tp.nr < 1 || tp.nr > kMaxRank + 1)
            FAIL("rank-%d plan: %d enumerating axes\n", rank, tp.nr);
        uint64_t covered = (uint64_t)tp.T;
        for (int a = 0; a < tp.nr; ++a)
            covered *= tp.r_dims[a];
        if (covered != (9ull << 56) * 2 || covered / tp.T != tp.tiles)
            FAIL("rank-%d plan covers %llu elements\n", rank, (unsigned long long)covered);
    }
    std::printf("ok %d of %d cases tiled, %d of %d large cases, %zu merged-axes cases\n", planned,
                cases, big_planned, big_cases, fixed.size());
    return 0;
}
