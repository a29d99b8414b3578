// Stand-in for the absent `samplesortlib.hpp` that GPLUM's hard.h includes.
// TEST INFRASTRUCTURE ONLY.  The original is a parallel sample sort by key;
// here it is a stable sort by the same key, which fixes the order of members
// inside each cluster to ascending input order.  The device path uses the same
// member order, so cluster integrations are compared member for member.
#pragma once
#include <algorithm>

namespace SampleSortLib {
template <class T, class KeyFn>
void samplesort(T *a, long n, KeyFn key) {
    std::stable_sort(a, a + n, [&](const T &l, const T &r) {
        return key(const_cast<T &>(l)) < key(const_cast<T &>(r));
    });
}
}  // namespace SampleSortLib
