"""Generality stencils (diffusion 7-point, Jacobi 5-point, 2-D Yee) against the C oracle, bit for bit."""

import ctypes as c

import numpy as np
import pytest

from compiler import emission, native
from compiler.resident.domain import ResidentDomain
from compiler.runtime import abi
from oracle import api

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _lib():
    lib = native.load()
    lib.f2c_diffusion7_v1.argtypes = [c.POINTER(native.Grid), c.c_void_p, c.c_void_p, c.c_double, c.c_double,
                                      c.c_void_p]
    lib.f2c_jacobi5_v1.argtypes = [c.c_void_p, c.c_void_p, c.c_int64, c.c_int64, c.c_int64, c.c_int64, c.c_void_p]
    lib.f2c_yee2d_v1.argtypes = [c.c_void_p] * 3 + [c.c_int64] * 4 + [c.c_double, c.c_double, c.c_void_p]
    return lib


def _interior_random(shape, h, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(shape)
    inner = tuple(slice(h, s - h) for s in shape)
    a[inner] = rng.random(tuple(s - 2 * h for s in shape))
    return a


@pytest.mark.parametrize("dx", [1.0, 0.3])
def test_diffusion_steps(cuda, dx):
    lib = _lib()
    n, h, dt, nu, steps = (37, 20, 18), 1, 0.125, 1.0, 6
    shape = (n[2] + 2, n[1] + 2, n[0] + 2)
    a = _interior_random(shape, h, 1)
    d = [cuda.from_numpy(a).cuda(), cuda.zeros(shape, dtype=cuda.float64, device="cuda")]
    grid = native.make_grid(*n, h, dx, dx, dx)
    for s in range(steps):
        native.check(lib.f2c_diffusion7_v1(c.byref(grid), d[s % 2].data_ptr(), d[1 - s % 2].data_ptr(), dt, nu, None))
    cuda.cuda.synchronize()
    ref = [a.copy(), np.zeros(shape)]
    for s in range(steps):
        api.diffusion7(ref[1 - s % 2], ref[s % 2], dt, nu, dx, h)
    assert np.array_equal(_bits(d[steps % 2].cpu().numpy()), _bits(ref[steps % 2]))


def test_jacobi_sweeps(cuda):
    lib = _lib()
    nx, ny, h, sweeps = 70, 45, 1, 7
    shape = (ny + 2, nx + 2)
    u = _interior_random(shape, h, 2)
    d = [cuda.from_numpy(u).cuda(), cuda.zeros(shape, dtype=cuda.float64, device="cuda")]
    for s in range(sweeps):
        native.check(lib.f2c_jacobi5_v1(d[s % 2].data_ptr(), d[1 - s % 2].data_ptr(), nx, ny, h, nx + 2, None))
    cuda.cuda.synchronize()
    ref = [u.copy(), np.zeros(shape)]
    for s in range(sweeps):
        api.jacobi5(ref[1 - s % 2], ref[s % 2], h)
    assert np.array_equal(_bits(d[sweeps % 2].cpu().numpy()), _bits(ref[sweeps % 2]))


def test_yee_steps(cuda):
    lib = _lib()
    nx, ny, h, steps, ch, ce = 66, 39, 1, 5, 0.5, 0.7
    shape = (ny + 2, nx + 2)
    fields = [_interior_random(shape, h, s) for s in (3, 4, 5)]
    d = [cuda.from_numpy(f).cuda() for f in fields]
    for _ in range(steps):
        native.check(lib.f2c_yee2d_v1(*[t.data_ptr() for t in d], nx, ny, h, nx + 2, ch, ce, None))
    cuda.cuda.synchronize()
    ref = [f.copy() for f in fields]
    for _ in range(steps):
        api.yee2d(*ref, ch, ce, h)
    for got, want in zip(d, ref):
        assert np.array_equal(_bits(got.cpu().numpy()), _bits(want))


def test_stencil_entries_replay_as_graphs(cuda):
    lib = native.runtime()
    fns = emission.bind(lib)
    dom = ResidentDomain(lib)
    dom.begin_epoch()
    # diffusion through its entry, ping-pong
    n, h = (24, 16, 12), 1
    shape = (n[2] + 2, n[1] + 2, n[0] + 2)
    a = _interior_random(shape, h, 7)
    b = np.zeros(shape)
    ha, hb = dom.bind_real64(a), dom.bind_real64(b)
    for s in range(4):
        src, dst = (ha, hb) if s % 2 == 0 else (hb, ha)
        assert emission.call(fns, "stencil::diffuse7", dom.context, abi.GPU, [dst, src], [0.125, 1.0, 1.0],
                             [*n, h]) == abi.OK
    # Jacobi
    u = _interior_random((30, 40), 1, 8)
    v = np.zeros_like(u)
    hu, hv = dom.bind_real64(u), dom.bind_real64(v)
    for s in range(4):
        src, dst = (hu, hv) if s % 2 == 0 else (hv, hu)
        assert emission.call(fns, "stencil::jacobi5", dom.context, abi.GPU, [dst, src], [], [38, 28, 1]) == abi.OK
    # Yee
    ez, hx, hy = (_interior_random((26, 34), 1, s) for s in (9, 10, 11))
    hs = [dom.bind_real64(x) for x in (ez, hx, hy)]
    originals = [x.copy() for x in (ez, hx, hy)]
    for _ in range(3):
        assert emission.call(fns, "stencil::yee2d", dom.context, abi.GPU, hs, [0.5, 0.7], [32, 24, 1]) == abi.OK
    dom.end_epoch()
    dom.close()
    ra, rb = _interior_random(shape, h, 7), np.zeros(shape)
    for s in range(4):
        src, dst = (ra, rb) if s % 2 == 0 else (rb, ra)
        api.diffusion7(dst, src, 0.125, 1.0, 1.0, h)
    assert np.array_equal(_bits(a), _bits(ra))
    ru, rv = _interior_random((30, 40), 1, 8), np.zeros((30, 40))
    for s in range(4):
        src, dst = (ru, rv) if s % 2 == 0 else (rv, ru)
        api.jacobi5(dst, src, 1)
    assert np.array_equal(_bits(u), _bits(ru))
    for _ in range(3):
        api.yee2d(*originals, 0.5, 0.7, 1)
    for got, want in zip((ez, hx, hy), originals):
        assert np.array_equal(_bits(got), _bits(want))
