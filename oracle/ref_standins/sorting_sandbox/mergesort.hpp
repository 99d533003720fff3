// Stand-in for the un-vendored sorting_sandbox submodule's merge_sort,
// used by the reference's argsort (src/fri_utils.cpp:9,22-25). Test
// infrastructure only: it lets oracle/Makefile compile the reference's own
// sources into oracle/_ref/.
//
// The submodule (jamesETsmith/sorting_sandbox, commit not recorded in the
// reference checkout) is absent. Its published contract, as used at
// src/fri_utils.cpp:22, is "sort the vector in place with the comparator";
// the second argument names a parallelisation strategy. A stable sort is
// the only choice that makes the reference deterministic among equal
// magnitudes: equal |x| keep ascending flat-index order.
#pragma once
#include <algorithm>
#include <vector>

template <typename T, typename Cmp>
void merge_sort(std::vector<T>& v, const char* /*strategy*/, Cmp cmp) {
  std::stable_sort(v.begin(), v.end(), cmp);
}
