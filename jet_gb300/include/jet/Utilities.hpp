// Label algebra and index helpers of the Jet API (reference:
// include/jet/Utilities.hpp). The set operations keep the order of their first
// argument; ContractTensors' output label order depends on exactly that.
#pragma once

#include <algorithm>
#include <cstddef>
#include <string>
#include <unordered_set>
#include <vector>

#include "Abort.hpp"

namespace Jet {
namespace Utilities {

constexpr inline bool is_pow_2(size_t v) { return v != 0 && (v & (v - 1)) == 0; }

constexpr inline size_t fast_log2(size_t v)
{
    size_t r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

// Labels a, b, ..., z, A, ..., Z, then a0, ..., Z0, a1, ... (Utilities.hpp:86-97).
inline std::string GenerateStringIndex(size_t id)
{
    static const char *letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ";
    const size_t n = 52;
    std::string s(1, letters[id % n]);
    if (id >= n)
        s += std::to_string(id / n - 1);
    return s;
}

template <class T> inline bool InVector(const T &e, const std::vector<T> &v)
{
    return std::find(v.begin(), v.end(), e) != v.end();
}

// Elements of v1 that are also in v2, in v1's order.
template <class T>
inline std::vector<T> VectorIntersection(const std::vector<T> &v1, const std::vector<T> &v2)
{
    std::unordered_set<T> s2(v2.begin(), v2.end());
    std::vector<T> out;
    for (const auto &x : v1)
        if (s2.count(x))
            out.push_back(x);
    return out;
}

// v1 followed by the elements of v2 missing from v1.
template <class T>
inline std::vector<T> VectorUnion(const std::vector<T> &v1, const std::vector<T> &v2)
{
    std::unordered_set<T> s1(v1.begin(), v1.end());
    std::vector<T> out = v1;
    for (const auto &x : v2)
        if (!s1.count(x))
            out.push_back(x);
    return out;
}

// Elements of v1 missing from v2, in v1's order.
template <class T>
inline std::vector<T> VectorSubtraction(const std::vector<T> &v1, const std::vector<T> &v2)
{
    std::unordered_set<T> s2(v2.begin(), v2.end());
    std::vector<T> out;
    for (const auto &x : v1)
        if (!s2.count(x))
            out.push_back(x);
    return out;
}

template <class T>
inline std::vector<T> VectorDisjunctiveUnion(const std::vector<T> &v1, const std::vector<T> &v2)
{
    return VectorSubtraction(VectorUnion(v1, v2), VectorIntersection(v1, v2));
}

template <class T>
inline std::vector<T> VectorConcatenation(const std::vector<T> &v1, const std::vector<T> &v2)
{
    std::vector<T> out = v1;
    out.insert(out.end(), v2.begin(), v2.end());
    return out;
}

inline std::string JoinStringVector(const std::vector<std::string> &v)
{
    std::string s;
    for (const auto &x : v)
        s += x;
    return s;
}

inline size_t ShapeToSize(const std::vector<size_t> &shape)
{
    size_t n = 1;
    for (size_t d : shape)
        n *= d;
    return n;
}

// Row-major multi-index of `index` (Utilities.hpp:463-475).
inline std::vector<size_t> UnravelIndex(unsigned long long index, const std::vector<size_t> &shape)
{
    JET_ABORT_IF(ShapeToSize(shape) <= index, "Linear index does not fit in the shape.");
    std::vector<size_t> out(shape.size());
    for (size_t i = shape.size(); i-- > 0;) {
        out[i] = index % shape[i];
        index /= shape[i];
    }
    return out;
}

inline unsigned long long RavelIndex(const std::vector<size_t> &index,
                                     const std::vector<size_t> &shape)
{
    JET_ABORT_IF_NOT(index.size() == shape.size(),
                     "Number of index and shape dimensions must match.");
    unsigned long long linear = 0, stride = 1;
    for (size_t i = shape.size(); i-- > 0;) {
        JET_ABORT_IF(index[i] >= shape[i], "Index does not fit in the shape.");
        linear += index[i] * stride;
        stride *= shape[i];
    }
    return linear;
}

} // namespace Utilities
} // namespace Jet
