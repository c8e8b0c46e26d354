// Host-side sort of 64-bit keys for the AMR table builders (the reflux grouping
// of a level pair sorts one key per coarse-fine face, about 1.6e5 of them on a
// 3-level jet hierarchy, at every regrid while the device waits).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

namespace ocfd {

// Ascending sort of `k`: least-significant-digit radix sort in 11-bit digits
// (2048 buckets: the counters and the scatter's open lines stay in the L1/L2
// caches) over the bits the keys use, one counting pass and one stable scatter
// per digit, so the result is the same sequence std::sort gives.
inline void radix_sort_u64(std::vector<uint64_t>& k) {
    const size_t n = k.size();
    if (n < 2) return;
    uint64_t used = 0;
    for (uint64_t v : k) used |= v;
    constexpr int DIGIT = 11;
    constexpr uint64_t MASK = (1u << DIGIT) - 1;
    int bits = 0;
    while (bits < 64 && (used >> bits) != 0) bits += DIGIT;
    std::vector<uint64_t> tmp(n);
    std::vector<size_t> start(size_t(1) << DIGIT);
    uint64_t* src = k.data();
    uint64_t* dst = tmp.data();
    for (int sh = 0; sh < bits; sh += DIGIT) {
        std::fill(start.begin(), start.end(), 0);
        for (size_t i = 0; i < n; ++i) ++start[(src[i] >> sh) & MASK];
        size_t s = 0;
        for (size_t& c : start) {
            const size_t m = c;
            c = s;
            s += m;
        }
        for (size_t i = 0; i < n; ++i) dst[start[(src[i] >> sh) & MASK]++] = src[i];
        std::swap(src, dst);
    }
    if (src != k.data()) std::memcpy(k.data(), src, n * sizeof(uint64_t));
}

}  // namespace ocfd
