// Host-side check of Jet::Tensor's label -> dimension map, which is built
// from the labels and shape when first read: every state it can reach through
// construction, RenameIndex, SetShape, copies and moves must equal the map the
// reference's Tensor (include/jet/Tensor.hpp: InitIndicesAndShape,
// RenameIndex, SetShape) keeps eagerly -- restated below as `Model`, which
// applies each operation to its map at once. No GPU is used.
#include <complex>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include "Jet.hpp"

using namespace Jet;
using c64 = std::complex<float>;
using Map = std::unordered_map<std::string, size_t>;

static int failures = 0;
#define CHECK(...)                                                                     \
    do {                                                                               \
        if (!(__VA_ARGS__)) {                                                          \
            ++failures;                                                                \
            std::printf("FAILED line %d: %s\n", __LINE__, #__VA_ARGS__);              \
        }                                                                              \
    } while (0)

// The eager rules: the map is rebuilt (last label wins) on construction and
// copy; a rename moves the old label's dimension to the new label without
// overwriting an existing entry; SetShape leaves the map alone.
struct Model {
    std::vector<std::string> indices;
    std::vector<size_t> shape;
    Map map;
    Model(const std::vector<std::string> &i, const std::vector<size_t> &s) : indices(i), shape(s)
    {
        for (size_t q = 0; q < s.size(); ++q)
            map[i[q]] = s[q];
    }
    void Rename(size_t pos, const std::string &label)
    {
        const std::string old = indices[pos];
        const size_t dim = map[old];
        map.erase(old);
        indices[pos] = label;
        map.emplace(label, dim);
    }
    Model Copy() const { return Model(indices, shape); }
};

static bool Same(const Tensor<c64> &t, const Model &m)
{
    return t.GetIndices() == m.indices && t.GetShape() == m.shape &&
           t.GetIndexToDimension() == m.map;
}

int main()
{
    {
        Tensor<c64> t({"i", "j", "k"}, {1, 2, 3});
        CHECK(Same(t, Model({"i", "j", "k"}, {1, 2, 3})));
    }
    { // repeated label: the last dimension wins
        Tensor<c64> t({"a", "a"}, {2, 3});
        CHECK(Same(t, Model({"a", "a"}, {2, 3})));
    }
    { // rename before and after the map was first read
        Tensor<c64> t({"i", "j"}, {2, 3});
        Model m({"i", "j"}, {2, 3});
        t.RenameIndex(0, "x");
        m.Rename(0, "x");
        CHECK(Same(t, m));
        t.RenameIndex(1, "y");
        m.Rename(1, "y");
        CHECK(Same(t, m));
    }
    { // rename onto a label already present: its entry is kept
        Tensor<c64> t({"i", "j"}, {2, 3});
        Model m({"i", "j"}, {2, 3});
        t.RenameIndex(0, "j");
        m.Rename(0, "j");
        CHECK(Same(t, m));
        const Tensor<c64> c(t); // a copy rebuilds the map from labels and shape
        CHECK(Same(c, m.Copy()));
    }
    { // SetShape on a tensor whose map was never read keeps the old dimensions
        Tensor<c64> t({"i", "j"}, {2, 3});
        Model m({"i", "j"}, {2, 3});
        t.SetShape({5, 6});
        m.shape = {5, 6};
        CHECK(Same(t, m));
        Tensor<c64> c({"q"}, {7});
        c = t;
        CHECK(Same(c, m.Copy()));
    }
    { // moves carry the map over, read or not
        Tensor<c64> t({"i", "j"}, {2, 3});
        Model m({"i", "j"}, {2, 3});
        t.RenameIndex(1, "k");
        m.Rename(1, "k");
        Tensor<c64> u(std::move(t));
        CHECK(Same(u, m));
        Tensor<c64> v({"p", "q"}, {4, 4});
        v.SetShape({8, 8});
        Model mv({"p", "q"}, {4, 4});
        mv.shape = {8, 8};
        Tensor<c64> w({"z"}, {1});
        w = std::move(v);
        CHECK(Same(w, mv));
    }
    { // equality compares the maps too
        const std::vector<c64> data{{1, 2}, {3, 4}, {5, 6}, {7, 8}, {9, 1}, {2, 3}};
        Tensor<c64> a({"i", "j"}, {2, 3}, data), b({"i", "j"}, {2, 3}, data);
        CHECK(a == b);
        b.SetShape({2, 3});
        CHECK(a == b);
        Tensor<c64> c({"i", "j"}, {3, 2}, data);
        c.SetShape({2, 3}); // same labels and shape as a, map still {i: 3, j: 2}
        CHECK(c != a);
    }
    if (failures) {
        std::printf("%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("ok\n");
    return 0;
}
