"""The CUDA kernels against golden vectors computed by executing the reference's own Fortran source."""

import ctypes as c
from pathlib import Path

import numpy as np
import pytest

from compiler import native

pytestmark = pytest.mark.gpu

FIXTURE = np.load(Path(__file__).with_name("golden") / "reference_kernels.npz")


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _case(n, torch):
    nx, ny, nz, g, dx, dy, dz, _ = FIXTURE[f"adv{n}_case"]
    nx, ny, nz, g = int(nx), int(ny), int(nz), int(g)
    grid = native.make_grid(nx, ny, nz, g, dx, dy, dz)
    dev = [torch.from_numpy(FIXTURE[f"adv{n}_{k}"].copy()).cuda() for k in "UVW"]
    inner = (slice(g, g + nz), slice(g, g + ny), slice(g, g + nx))
    return grid, dev, inner


@pytest.mark.parametrize("n", [0, 1, 2])
@pytest.mark.parametrize("variant", [native.FACES, native.DIRECT, native.FAST])
def test_fused_step_equals_the_reference(cuda, n, variant):
    from tolerance import check

    grid, dev, inner = _case(n, cuda)
    out = [cuda.full_like(t, float("nan")) for t in dev]
    native.advection(grid, *[t.data_ptr() for t in dev], *[t.data_ptr() for t in out], variant=variant)
    cuda.cuda.synchronize()
    for t, c_ in zip(out, "uvw"):
        got, want = t.cpu().numpy()[inner], FIXTURE[f"adv{n}_cd{c_}"]
        if variant == native.FAST:
            check(got, want, c_)
        else:
            assert np.array_equal(_bits(got), _bits(want)), c_


@pytest.mark.parametrize("n", [0, 1])
@pytest.mark.parametrize("variant", [native.FACES, native.FAST])
def test_kernels_reproduce_the_reference_test_programs(cuda, n, variant):
    """The values the reference's cdu_main.f90, cvd_main.f90 and cdw_main.f90 write, from the fused launch."""
    from tolerance import check

    nx, ny, nz = (int(v) for v in FIXTURE[f"main{n}_size"])
    grid = native.make_grid(nx, ny, nz, 1, 1.0 / nx, 1.0 / ny, 1.0 / nz)
    dev = [cuda.from_numpy(FIXTURE[f"main{n}_{k}"].copy()).cuda() for k in "UVW"]
    out = [cuda.full_like(t, float("nan")) for t in dev]
    native.advection(grid, *[t.data_ptr() for t in dev], *[t.data_ptr() for t in out], variant=variant)
    cuda.cuda.synchronize()
    inner = (slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1))
    for t, which in zip(out, ("cdu", "cdv", "cdw")):
        got, written = t.cpu().numpy()[inner].ravel(), FIXTURE[f"main{n}_{which}"]
        if variant == native.FAST:
            check(got, written, which)
        else:
            assert np.array_equal(_bits(got), _bits(written)), which


def test_procedure_launches_equal_the_reference(cuda):
    """Each procedure as one launch (the reference's structure) on case 0's inputs, bit for bit."""
    grid, d, inner = _case(0, cuda)
    u, v, w = (t.data_ptr() for t in d)
    ops = {"u": (native.CDU_DIV, native.CDU_ADV), "v": (native.CDV_DIV, native.CDV_ADV),
           "w": (native.CDW_DIV, native.CDW_ADV)}
    for comp, (div, adv) in ops.items():
        out = cuda.full_like(d[0], float("nan"))
        native.procedure(native.SET, grid, out.data_ptr(), value=0.0)
        native.procedure(div, grid, out.data_ptr(), u, v, w)
        cuda.cuda.synchronize()
        assert np.array_equal(_bits(out.cpu().numpy()[inner]), _bits(FIXTURE[f"proc_cd{comp}div"])), comp
        native.procedure(native.MULTIPLY, grid, out.data_ptr(), value=0.5)
        cuda.cuda.synchronize()
        assert np.array_equal(_bits(out.cpu().numpy()[inner]), _bits(FIXTURE[f"proc_cd{comp}half"])), comp
        native.procedure(native.SET, grid, out.data_ptr(), value=0.0)
        native.procedure(adv, grid, out.data_ptr(), u, v, w)
        cuda.cuda.synchronize()
        assert np.array_equal(_bits(out.cpu().numpy()[inner]), _bits(FIXTURE[f"proc_cd{comp}adv"])), comp


def test_stencils_equal_the_reference(cuda):
    lib = native.load()
    lib.f2c_diffusion7_v1.argtypes = [c.POINTER(native.Grid), c.c_void_p, c.c_void_p, c.c_double, c.c_double,
                                      c.c_void_p]
    lib.f2c_jacobi5_v1.argtypes = [c.c_void_p, c.c_void_p, c.c_int64, c.c_int64, c.c_int64, c.c_int64, c.c_void_p]
    nx, ny, nz, dx, dt, nu, _ = FIXTURE["diff_case"]
    a = cuda.from_numpy(FIXTURE["diff_a"].copy()).cuda()
    b = cuda.full_like(a, float("nan"))
    grid = native.make_grid(int(nx), int(ny), int(nz), 2, dx, dx, dx)
    native.check(lib.f2c_diffusion7_v1(c.byref(grid), a.data_ptr(), b.data_ptr(), dt, nu, None))
    u = cuda.from_numpy(FIXTURE["jac_u"].copy()).cuda()
    v = cuda.full_like(u, float("nan"))
    n = int(FIXTURE["jac_case"][0])
    native.check(lib.f2c_jacobi5_v1(u.data_ptr(), v.data_ptr(), n, n, 1, n + 2, None))
    cuda.cuda.synchronize()
    assert np.array_equal(_bits(b.cpu().numpy()[2:-2, 2:-2, 2:-2]), _bits(FIXTURE["diff_b"]))
    assert np.array_equal(_bits(v.cpu().numpy()[1:-1, 1:-1]), _bits(FIXTURE["jac_v"]))
