// Rectangle algebra of the residency runtime: which parts of an array hold
// defined values, and which of them are current on the host and on the device.
//
// A Box is a rank-r product of half-open index ranges [lo, hi) in physical
// zero-based coordinates. A Region is a list of pairwise disjoint boxes. The
// sets a runtime keeps per array stay within kRegionLimit boxes (the reference
// bounds its lists the same way, compiler/runtime/scoped_regions.hpp:13):
// results are computed as unbounded temporaries and the runtime reconciles an
// array to whole-array boxes when a result would not fit.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace f2c::rt {

constexpr int kMaxRank = 7;
constexpr size_t kRegionLimit = 128;

struct Box {
    int rank = 0;
    size_t lo[kMaxRank] = {};
    size_t hi[kMaxRank] = {};

    bool empty() const {
        for (int d = 0; d < rank; ++d)
            if (hi[d] <= lo[d]) return true;
        return rank == 0;
    }
    size_t volume() const {
        if (empty()) return 0;
        size_t v = 1;
        for (int d = 0; d < rank; ++d) v *= hi[d] - lo[d];
        return v;
    }
};

inline Box whole(int rank, const size_t *extents) {
    Box b;
    b.rank = rank;
    for (int d = 0; d < rank; ++d) {
        b.lo[d] = 0;
        b.hi[d] = extents[d];
    }
    return b;
}

inline Box intersect(const Box &a, const Box &b) {
    Box r;
    r.rank = a.rank;
    for (int d = 0; d < a.rank; ++d) {
        r.lo[d] = std::max(a.lo[d], b.lo[d]);
        r.hi[d] = std::min(a.hi[d], b.hi[d]);
    }
    return r;
}

inline bool overlaps(const Box &a, const Box &b) { return !intersect(a, b).empty(); }

inline bool contains(const Box &outer, const Box &inner) {
    if (inner.empty()) return true;
    for (int d = 0; d < outer.rank; ++d)
        if (inner.lo[d] < outer.lo[d] || inner.hi[d] > outer.hi[d]) return false;
    return true;
}

// a \ b as at most 2*rank disjoint boxes appended to out: peel slabs off `a`
// below and above `b` one dimension at a time.
inline void subtract(const Box &a, const Box &b, std::vector<Box> &out) {
    if (a.empty()) return;
    if (!overlaps(a, b)) {
        out.push_back(a);
        return;
    }
    Box rest = a;
    for (int d = 0; d < a.rank; ++d) {
        if (rest.lo[d] < b.lo[d]) {
            Box below = rest;
            below.hi[d] = b.lo[d];
            out.push_back(below);
            rest.lo[d] = b.lo[d];
        }
        if (rest.hi[d] > b.hi[d]) {
            Box above = rest;
            above.lo[d] = b.hi[d];
            out.push_back(above);
            rest.hi[d] = b.hi[d];
        }
    }
}

class Region {
public:
    std::vector<Box> boxes;

    bool empty() const { return boxes.empty(); }
    void clear() { boxes.clear(); }
    size_t volume() const {
        size_t v = 0;
        for (const auto &b : boxes) v += b.volume();
        return v;
    }

    bool fits() const { return boxes.size() <= kRegionLimit; }

    // Union with b.
    void add(const Box &b) {
        if (b.empty()) return;
        std::vector<Box> pieces{b}, next;
        for (const auto &e : boxes) {
            next.clear();
            for (const auto &p : pieces) subtract(p, e, next);
            pieces.swap(next);
            if (pieces.empty()) return;
        }
        boxes.insert(boxes.end(), pieces.begin(), pieces.end());
        merge();
    }
    void add(const Region &r) {
        for (const auto &b : r.boxes) add(b);
    }

    // Difference with b.
    void remove(const Box &b) {
        if (b.empty()) return;
        std::vector<Box> next;
        bool touched = false;
        for (const auto &e : boxes) {
            if (overlaps(e, b)) {
                touched = true;
                subtract(e, b, next);
            } else {
                next.push_back(e);
            }
        }
        if (!touched) return;
        boxes.swap(next);
        merge();
    }
    void remove(const Region &r) {
        for (const auto &b : r.boxes) remove(b);
    }

    // The parts of b inside this region.
    Region clip(const Box &b) const {
        Region r;
        for (const auto &e : boxes) {
            Box x = intersect(e, b);
            if (!x.empty()) r.boxes.push_back(x);
        }
        return r;
    }
    Region clip(const Region &other) const {
        Region r;
        for (const auto &o : other.boxes)
            for (const auto &e : boxes) {
                Box x = intersect(e, o);
                if (!x.empty()) r.boxes.push_back(x);
            }
        return r;
    }

    // The parts of b outside this region.
    Region missing(const Box &b) const {
        std::vector<Box> pieces{b}, next;
        if (b.empty()) return Region{};
        for (const auto &e : boxes) {
            next.clear();
            for (const auto &p : pieces) subtract(p, e, next);
            pieces.swap(next);
            if (pieces.empty()) break;
        }
        Region r;
        r.boxes = std::move(pieces);
        return r;
    }

    bool covers(const Box &b) const { return missing(b).empty(); }
    bool intersects(const Box &b) const {
        for (const auto &e : boxes)
            if (overlaps(e, b)) return true;
        return false;
    }

private:
    // Join neighbours that differ in one dimension only and touch there, so that
    // repeated updates of the same sections do not fragment the list.
    void merge() {
        bool changed = true;
        while (changed && boxes.size() > 1) {
            changed = false;
            for (size_t a = 0; a < boxes.size() && !changed; ++a)
                for (size_t b = a + 1; b < boxes.size() && !changed; ++b) {
                    const Box &x = boxes[a], &y = boxes[b];
                    int differ = -1, count = 0;
                    for (int d = 0; d < x.rank; ++d)
                        if (x.lo[d] != y.lo[d] || x.hi[d] != y.hi[d]) {
                            differ = d;
                            ++count;
                        }
                    if (count != 1) continue;
                    if (x.hi[differ] == y.lo[differ] || y.hi[differ] == x.lo[differ]) {
                        Box m = x;
                        m.lo[differ] = std::min(x.lo[differ], y.lo[differ]);
                        m.hi[differ] = std::max(x.hi[differ], y.hi[differ]);
                        boxes[a] = m;
                        boxes.erase(boxes.begin() + (long)b);
                        changed = true;
                    }
                }
        }
    }
};

} // namespace f2c::rt
