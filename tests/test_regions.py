"""The runtime's rectangle algebra (csrc/runtime/regions.hpp), cell by cell.

Behaviours restated from the reference's region tests
(compiler/tests/test_scoped_regions.py: touching faces merge, holes and
non-rectangular neighbours are kept exactly, differences keep interior holes,
a stencil's shifted footprints collapse to a few boxes, extreme endpoints need
no overflowing arithmetic, and the box limit is not extended). A C++ driver
builds each case with the header and checks every result against an explicit
set of cells; the Python side only compiles and runs it.
"""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
RUNTIME = ROOT / "fortran-to-cuda_gb300" / "csrc" / "runtime"

DRIVER = r"""
#include <cstdio>
#include <cstdint>
#include <set>
#include <vector>
#include "regions.hpp"
using namespace f2c::rt;
using Cell = std::vector<size_t>;

static Box box(std::vector<size_t> lo, std::vector<size_t> hi) {
    Box b;
    b.rank = (int)lo.size();
    for (int d = 0; d < b.rank; ++d) { b.lo[d] = lo[d]; b.hi[d] = hi[d]; }
    return b;
}
static void cells_of(const Box &b, std::set<Cell> &out) {
    if (b.empty()) return;
    Cell c(b.lo, b.lo + b.rank);
    while (true) {
        out.insert(c);
        int d = 0;
        while (d < b.rank && ++c[d] == b.hi[d]) { c[d] = b.lo[d]; ++d; }
        if (d == b.rank) return;
    }
}
static std::set<Cell> cells(const Region &r) {
    std::set<Cell> out;
    for (const Box &b : r.boxes) cells_of(b, out);
    return out;
}
static int failures = 0;
static void expect(bool ok, const char *what) {
    if (!ok) { std::printf("FAIL %s\n", what); ++failures; }
}
// exact cells, and the boxes disjoint (their volumes add up to the cell count)
static void exact(const Region &r, const std::set<Cell> &want, const char *what) {
    expect(cells(r) == want, what);
    expect(r.volume() == want.size(), what);
}

int main() {
    for (int axis = 0; axis < 3; ++axis) {  // touching faces merge on each axis
        std::vector<size_t> lo{1, 1, 1}, mid{4, 4, 4}, hi{4, 4, 4};
        mid[axis] = 2;
        hi[axis] = 5;
        std::vector<size_t> lo2 = lo;
        lo2[axis] = 2;
        Region r;
        r.add(box(lo, mid));
        r.add(box(lo2, hi));
        std::set<Cell> want;
        cells_of(box(lo, mid), want);
        cells_of(box(lo2, hi), want);
        exact(r, want, "touching faces: cells");
        expect(r.boxes.size() == 1, "touching faces: one box");
    }
    {  // non-rectangular neighbours keep their missing cells
        const Box cases[3][2] = {{box({0, 0}, {2, 2}), box({3, 0}, {5, 2})},
                                 {box({0, 0}, {2, 2}), box({2, 2}, {4, 4})},
                                 {box({0, 0}, {2, 2}), box({2, 0}, {4, 1})}};
        for (const auto &c : cases) {
            Region r;
            r.add(c[0]);
            r.add(c[1]);
            std::set<Cell> want;
            cells_of(c[0], want);
            cells_of(c[1], want);
            exact(r, want, "neighbours: cells");
            expect(r.boxes.size() == 2, "neighbours: two boxes");
        }
    }
    {  // an overlapping union keeps its holes
        Region r;
        r.add(box({0, 0}, {3, 2}));
        r.add(box({2, 1}, {4, 3}));
        std::set<Cell> want;
        cells_of(box({0, 0}, {3, 2}), want);
        cells_of(box({2, 1}, {4, 3}), want);
        exact(r, want, "overlap: cells");
        expect(!cells(r).count(Cell{3, 0}) && !cells(r).count(Cell{0, 2}), "overlap: holes");
    }
    {  // a difference keeps the interior hole, in at most four pieces
        Region r;
        r.add(box({0, 0}, {4, 4}));
        r.remove(box({1, 1}, {3, 3}));
        std::set<Cell> want, hole;
        cells_of(box({0, 0}, {4, 4}), want);
        cells_of(box({1, 1}, {3, 3}), hole);
        for (const Cell &c : hole) want.erase(c);
        exact(r, want, "difference: cells");
        expect(r.boxes.size() <= 4, "difference: at most four pieces");
        Region s;
        s.add(box({0, 0}, {2, 2}));
        s.add(box({2, 0}, {4, 2}));
        expect(s.boxes.size() == 1 && s.volume() == 8, "difference: touching pieces coalesce");
        Region t;  // removing what is not there changes nothing
        t.add(box({0, 0}, {4, 4}));
        t.remove(box({5, 5}, {6, 6}));
        expect(t.boxes.size() == 1 && t.volume() == 16, "difference: disjoint removal");
    }
    {  // a stencil's ten shifted footprints collapse to three boxes
        const long shifts[10][3] = {{0, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {-1, 1, 0}, {0, -1, 0},
                                    {-1, -1, 0}, {0, 0, 1}, {-1, 0, 1}, {0, 0, -1}, {-1, 0, -1}};
        const size_t shape[3] = {5, 4, 3};
        Region r;
        std::set<Cell> want;
        for (const auto &s : shifts) {
            std::vector<size_t> lo(3), hi(3);
            for (int d = 0; d < 3; ++d) {
                lo[d] = (size_t)(2 + s[d]);
                hi[d] = (size_t)(2 + s[d]) + shape[d];
            }
            r.add(box(lo, hi));
            cells_of(box(lo, hi), want);
        }
        exact(r, want, "stencil: cells");
        std::printf("stencil boxes %zu\n", r.boxes.size());
        expect(r.boxes.size() <= 3, "stencil: three boxes");
    }
    {  // adjacent boxes at the top of the index range merge without overflow
        const size_t top = SIZE_MAX;
        Region r;
        r.add(box({top - 4}, {top - 2}));
        r.add(box({top - 2}, {top}));
        expect(r.boxes.size() == 1 && r.boxes[0].lo[0] == top - 4 && r.boxes[0].hi[0] == top, "extremes: merged");
        expect(r.volume() == 4, "extremes: volume");
    }
    {  // the box limit: 129 disjoint boxes do not fit, 128 do
        Region r;
        for (size_t n = 0; n < 128; ++n) r.add(box({2 * n}, {2 * n + 1}));
        expect(r.fits(), "limit: 128 boxes fit");
        r.add(box({1000}, {1001}));
        expect(!r.fits(), "limit: 129 boxes do not");
        r.add(box({1001}, {1002}));  // touching: merges, the count stays
        expect(r.boxes.size() == 129, "limit: merge keeps the count");
    }
    {  // clip, missing and covers agree with the cells
        Region r;
        r.add(box({0, 0, 0}, {4, 4, 4}));
        r.remove(box({1, 1, 1}, {2, 2, 2}));
        const Box probe = box({0, 0, 0}, {3, 3, 3});
        const Region in = r.clip(probe), out = r.missing(probe);
        std::set<Cell> all, inside, hole;
        cells_of(probe, all);
        cells_of(box({1, 1, 1}, {2, 2, 2}), hole);
        for (const Cell &c : all)
            if (!hole.count(c)) inside.insert(c);
        exact(in, inside, "clip");
        exact(out, hole, "missing");
        expect(!r.covers(probe) && r.covers(box({2, 2, 2}, {4, 4, 4})), "covers");
    }
    std::printf(failures ? "failed %d\n" : "ok\n", failures);
    return failures ? 1 : 0;
}
"""


def test_rectangle_algebra():
    compiler = shutil.which("g++")
    if compiler is None:
        pytest.skip("no C++ compiler")
    import tempfile

    with tempfile.TemporaryDirectory() as tmp:
        source, exe = Path(tmp) / "regions.cpp", Path(tmp) / "regions"
        source.write_text(DRIVER)
        built = subprocess.run([compiler, "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{RUNTIME}", str(source), "-o",
                                str(exe)], capture_output=True, text=True)
        assert built.returncode == 0, built.stderr
        run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.rstrip().endswith("ok")
