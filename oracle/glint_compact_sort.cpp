/*
 * glint_compact_sort.cpp -- the sorts of the reference's compaction done with
 * the C++ library's own std::sort, for the oracle's exact-tie mode.
 *
 * TEST INFRASTRUCTURE: linked into liboracle.so only.
 *
 * merge_dump (tools/compaction.cpp:729-1215) sorts with std::sort, whose
 * order of equivalent elements the C++ standard leaves unspecified; with
 * libstdc++ it is fixed by the comparison outcomes alone.  Calling the same
 * std::sort with the same comparators on the same sequences reproduces the
 * reference's order exactly, ties included (std::execution::par falls back
 * to std::sort without a TBB backend):
 *   compare_two_level (:139-155)  objects marked 2 first, by x middle
 *   compare_y         (:157-159)  each x part by y middle
 *   cmp_ki            (:92-97)    one object's keys by target, and the
 *                                 extra oversize list by (oid, target)
 */
#include <algorithm>
#include <cstdint>
#include <vector>

namespace {
struct Loc {
    double x, y;
    uint32_t oid;
};
} // namespace

extern "C" {

/* order[N]: object ids after std::sort of all N objects (in id order) by
 * compare_two_level, where last[oid] marks the objects not marked 2 */
void go_cmp_std_sort_objects(const uint8_t *last, const double *ax, const double *ay, uint32_t N, uint32_t *order) {
    std::vector<Loc> v(N);
    for (uint32_t o = 0; o < N; ++o) v[o] = Loc{ax[o], ay[o], o};
    std::sort(v.begin(), v.end(), [last](const Loc &a, const Loc &b) {
        const bool a_last = last[a.oid] != 0, b_last = last[b.oid] != 0;
        if (a_last != b_last) return b_last;
        if (!a_last) return a.x < b.x;
        return false;
    });
    for (uint32_t i = 0; i < N; ++i) order[i] = v[i].oid;
}

/* std::sort of order[lo, hi) by compare_y */
void go_cmp_std_sort_y(const double *ay, uint32_t *order, uint32_t lo, uint32_t hi) {
    std::vector<Loc> v;
    v.reserve(hi - lo);
    for (uint32_t i = lo; i < hi; ++i) v.push_back(Loc{0.0, ay[order[i]], order[i]});
    std::sort(v.begin(), v.end(), [](const Loc &a, const Loc &b) { return a.y < b.y; });
    for (uint32_t i = lo; i < hi; ++i) order[i] = v[i - lo].oid;
}

/* idx[n]: one object's keys (in source order) after std::sort by target */
void go_cmp_std_sort_targets(const uint32_t *target, uint64_t *idx, uint64_t n) {
    std::vector<std::pair<uint32_t, uint64_t>> v(n);
    for (uint64_t i = 0; i < n; ++i) v[i] = {target[i], idx[i]};
    std::sort(v.begin(), v.end(),
              [](const std::pair<uint32_t, uint64_t> &a, const std::pair<uint32_t, uint64_t> &b) {
                  return a.first < b.first;
              });
    for (uint64_t i = 0; i < n; ++i) idx[i] = v[i].second;
}

/* idx[n]: the extra oversize list (in source order) after std::sort by
 * (oid, target) */
void go_cmp_std_sort_pairs(const uint32_t *oid, const uint32_t *target, uint64_t *idx, uint64_t n) {
    struct P {
        uint32_t oid, target;
        uint64_t idx;
    };
    std::vector<P> v(n);
    for (uint64_t i = 0; i < n; ++i) v[i] = P{oid[i], target[i], idx[i]};
    std::sort(v.begin(), v.end(), [](const P &a, const P &b) {
        if (a.oid == b.oid) return a.target < b.target;
        return a.oid < b.oid;
    });
    for (uint64_t i = 0; i < n; ++i) idx[i] = v[i].idx;
}

} /* extern "C" */
