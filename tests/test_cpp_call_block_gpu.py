"""A C++ caller drives a generated entry exactly as the spliced Fortran call block does.

No Fortran compiler exists on these machines, so the call block's sequence is
written in C++ against the installed headers (`include/scoped_runtime.h`,
`include/fort_shared_entries.h`) and linked against libf2c_gb300.so: the
residency domain opened as `begin_epoch` opens it (default budget, domain,
context in the domain, budget set), the arrays registered by address with
their extents and lower bounds, the entry called with the context, GPU mode,
the handles and the scalars by reference, then the observation and
unregistration of `end_epoch` and the closing of `close`. The output it writes
must equal the C oracle's bit for bit.
"""

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from compiler import emission, native
from compiler import workloads as wl
from oracle import api

pytestmark = pytest.mark.gpu

CALLER = r"""
#include <cstdio>
#include <cstdint>
#include <vector>
#include "scoped_runtime.h"
#include "fort_shared_entries.h"

static int require(int status, const char *what) {
    if (status != FORT_SCOPE_OK) std::fprintf(stderr, "%s: status %d: %s\n", what, status, fort_scope_error());
    return status;
}

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    const bool fast = argv[3][0] == 'f';
    int nx = NX, ny = NY, nz = NZ;
    const size_t ex = nx + 2, ey = ny + 2, ez = nz + 2, n = ex * ey * ez;
    std::vector<double> u(n), v(n), w(n), u2(n, 0.0);
    FILE *in = std::fopen(argv[1], "rb");
    if (!in || std::fread(u.data(), 8, n, in) != n || std::fread(v.data(), 8, n, in) != n ||
        std::fread(w.data(), 8, n, in) != n) return 3;
    std::fclose(in);
    double dx = 1.0 / nx, dy = 1.0 / ny, dz = 1.0 / nz;

    // begin_epoch: default budget, a domain, a context in it, the budget set
    size_t budget = 0;
    fort_scope_domain_t domain = 0;
    fort_scope_t context = 0;
    if (require(fort_scope_device_budget_default_v1(0, &budget), "budget") ||
        require(fort_scope_domain_create_v1(0, &domain), "domain") ||
        require(fort_scope_create_in_domain_v1(domain, &context), "context") ||
        require(fort_scope_set_device_budget(context, budget), "set budget")) return 4;
    // a build prepared with --fast-fp: the domain opens its context under the fast-fp contract
    if (fast && require(fort_scope_numerics_set_v1(context, FORT_SCOPE_NUMERICS_FAST), "numerics")) return 4;

    // bind_real64: register each array by the address of its first element, extents and lower bounds 1
    const size_t extents[3] = {ex, ey, ez};
    const int64_t lower[3] = {1, 1, 1};
    double *arrays[4] = {u2.data(), u.data(), v.data(), w.data()};
    const int initialized[4] = {0, 1, 1, 1};
    fort_buffer_t handles[4];
    for (int a = 0; a < 4; ++a) {
        fort_scope_layout layout{};
        layout.rank = 3;
        layout.type = FORT_SCOPE_REAL64;
        layout.element_bytes = 8;
        layout.host = arrays[a];
        layout.extents = extents;
        layout.lower_bounds = lower;
        layout.generation = 1;
        if (require(fort_scope_register(context, (uint64_t)(uintptr_t)arrays[a], 1, &layout, initialized[a],
                                        &handles[a]), "register")) return 5;
    }

    // bind_real32 and bind_integer32: a REAL32 and an INTEGER32 array kept by the same domain, taken to the
    // device and published back exactly
    std::vector<float> singles(n);
    std::vector<int32_t> integers(n);
    for (size_t i = 0; i < n; ++i) {
        singles[i] = 0.25f * (float)(i % 977) - 3.0f;
        integers[i] = (int32_t)(i * 2654435761u);
    }
    const std::vector<float> singles0 = singles;
    const std::vector<int32_t> integers0 = integers;
    void *narrow[2] = {singles.data(), integers.data()};
    const uint32_t narrow_type[2] = {FORT_SCOPE_REAL32, FORT_SCOPE_INTEGER32};
    fort_buffer_t narrow_handle[2];
    for (int a = 0; a < 2; ++a) {
        fort_scope_layout layout{};
        layout.rank = 3;
        layout.type = narrow_type[a];
        layout.element_bytes = 4;
        layout.host = narrow[a];
        layout.extents = extents;
        layout.lower_bounds = lower;
        layout.generation = 1;
        if (require(fort_scope_register(context, (uint64_t)(uintptr_t)narrow[a], 1, &layout, 1, &narrow_handle[a]),
                    "register 4-byte")) return 12;
        fort_scope_access rw{};
        rw.flags = FORT_SCOPE_READ_ALL | FORT_SCOPE_WRITE_ALL;
        void *device = nullptr;
        if (require(fort_scope_device_begin(context, narrow_handle[a], &rw, &device), "device begin") || !device ||
            require(fort_scope_device_end(context, narrow_handle[a]), "device end")) return 13;
        fort_scope_layout back{};
        if (require(fort_scope_layout_get(context, narrow_handle[a], &back), "layout") || back.type != narrow_type[a] ||
            back.element_bytes != 4) return 14;
    }
    // the host copies are stale now: scribble over them, the observation must bring the device's values back
    for (size_t i = 0; i < n; ++i) {
        singles[i] = -1.0f;
        integers[i] = -1;
    }
    if (require(fort_scope_observe_v1(context, narrow_handle, 2), "observe 4-byte")) return 15;
    for (size_t i = 0; i < n; ++i)
        if (singles[i] != singles0[i] || integers[i] != integers0[i]) return 16;

    // the call block: context, GPU mode, handles, scalars by reference
    for (int step = 0; step < 3; ++step) {
        const int status = ENTRY(context, FORT_SCOPE_GPU, handles[0], handles[1], handles[2], handles[3],
                                 &dx, &dy, &dz, &nx, &ny, &nz);
        if (status == FORT_SCOPE_DECLINED) return 6;   // the original statements would run: not expected here
        if (require(status, "entry")) return 7;
    }

    // end_epoch: observe and unregister; close
    if (require(fort_scope_observe_v1(context, handles, 4), "observe")) return 8;
    for (int a = 0; a < 4; ++a)
        if (require(fort_scope_unregister(context, handles[a]), "unregister")) return 9;
    for (int a = 0; a < 2; ++a)
        if (require(fort_scope_unregister(context, narrow_handle[a]), "unregister 4-byte")) return 9;
    if (require(fort_scope_close(context), "close") || require(fort_scope_domain_close_v1(domain), "domain close"))
        return 10;

    FILE *out = std::fopen(argv[2], "wb");
    if (!out || std::fwrite(u2.data(), 8, n, out) != n) return 11;
    std::fclose(out);
    return 0;
}
"""


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_cpp_caller_runs_the_cdu_entry_like_the_call_block(cuda, tmp_path, numerics):
    compiler = shutil.which("g++")
    if compiler is None:
        pytest.skip("no C++ compiler")
    nx, ny, nz = 40, 24, 18
    library = native.build()
    entry = emission.entry_for("momentumadvection::cdu").symbol
    source = tmp_path / "caller.cpp"
    source.write_text(CALLER)
    exe = tmp_path / "caller"
    cuda_lib = Path(native.nvcc()).resolve().parent.parent / "lib64"
    subprocess.run([compiler, "-O2", "-std=c++17", f"-DNX={nx}", f"-DNY={ny}", f"-DNZ={nz}", f"-DENTRY={entry}",
                    f"-I{native.INCLUDE}", str(source), "-o", str(exe), str(library),
                    f"-Wl,-rpath,{library.parent}", f"-Wl,-rpath-link,{cuda_lib}"], check=True, capture_output=True,
                   text=True)
    f = wl.reference_driver_fields(nx, ny, nz, seed=5)
    inputs = tmp_path / "in.bin"
    with open(inputs, "wb") as fh:
        for a in (f.U, f.V, f.W):
            fh.write(np.ascontiguousarray(a).tobytes())
    result = tmp_path / "out.bin"
    run = subprocess.run([str(exe), str(inputs), str(result), numerics], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    got = np.fromfile(result, dtype=np.float64).reshape(f.U.shape)
    geo = f.geometry
    want = api.momentum("cdu", np.zeros_like(f.U), f.U, f.V, f.W, geo.dx, geo.dy, geo.dz, 1)
    interior = (slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1))
    if numerics == "strict":
        assert np.array_equal(got[interior].view(np.int64), want[interior].view(np.int64))
    else:
        import tolerance

        tolerance.check(got[interior], want[interior], "U2")
