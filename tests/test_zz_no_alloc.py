"""The batched step that allocates nothing (f2c_batch_step_static_v1), through the C ABI.

A caller whose device memory is already fully taken by another allocator, or
that must not bring the device-wide synchronisation of freeing memory into its
time loop, cannot hand f2c_batch_step_v1 a freshly allocated workspace. For
such callers the library keeps the batch's scratch (work counter, instance
descriptors, tile queue) in a fixed device array of its own. These tests check
that its results equal the workspace-based step bit for bit on consecutive
calls (the array keeps the previous call's contents, so the second call shows
that everything that must start from zero is cleared), that it leaves the
device's free memory unchanged once the library is loaded, and that batches
beyond the stated limits are refused with a message naming the limit.
"""

import ctypes

import numpy as np
import pytest

from compiler import native
from compiler import workloads as wl

pytestmark = pytest.mark.gpu

SHAPES = [(64, 40, 20), (37, 19, 33), (96, 24, 12), (8, 9, 45)]


def _lib():
    lib = native.load()
    lib.f2c_batch_step_static_v1.argtypes = [ctypes.POINTER(native.Grid), ctypes.POINTER(native.Fields),
                                             ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_void_p]
    lib.f2c_batch_step_static_v1.restype = ctypes.c_int
    return lib


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _instances(torch):
    inst = []
    for n, (nx, ny, nz) in enumerate(SHAPES):
        geo = wl.Geometry(nx, ny, nz, halo=2)
        f = wl.advection_fields(geo, seed=300 + n, nscalar=1)
        ins = [torch.from_numpy(a).cuda() for a in f.arrays()]
        inst.append((geo, ins, native.make_grid(nx, ny, nz, 2, geo.dx, geo.dy, geo.dz)))
    return inst


def _fields(inst, outs):
    fields = []
    for (geo, ins, grid), out in zip(inst, outs):
        p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in out]
        fields.append(native.make_fields(*p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:]))
    return fields


def test_no_alloc_step_equals_workspace_step_on_consecutive_calls(cuda):
    lib = _lib()
    inst = _instances(cuda)
    kz = [8, 16, 12, 32]
    # the existing entry point, with a workspace the test allocates
    ref_out = [[cuda.full_like(t, float("nan")) for t in ins] for (_, ins, _) in inst]
    batch = native.Batch([g for (_, _, g) in inst], _fields(inst, ref_out), kz=kz)
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.step()
    cuda.cuda.synchronize()
    # the entry point that allocates nothing, called three times in a row
    out = [[cuda.full_like(t, float("nan")) for t in ins] for (_, ins, _) in inst]
    grids = (native.Grid * len(inst))(*[g for (_, _, g) in inst])
    fields = (native.Fields * len(inst))(*_fields(inst, out))
    depths = (ctypes.c_int32 * len(inst))(*kz)
    free_after_first = None
    for call in range(3):
        for group in out:
            for t in group:
                t.fill_(float("nan"))
        cuda.cuda.synchronize()
        status = lib.f2c_batch_step_static_v1(grids, fields, depths, len(inst), None)
        assert status == 0, lib.f2c_last_error().decode()
        cuda.cuda.synchronize()
        free_now = cuda.cuda.mem_get_info()[0]
        if call == 0:
            free_after_first = free_now
        else:
            assert free_now >= free_after_first  # nothing allocated by later calls
        for (geo, _, _), got, want in zip(inst, out, ref_out):
            for a, b in zip(got, want):
                assert np.array_equal(_bits(a.cpu().numpy()[geo.interior()]), _bits(b.cpu().numpy()[geo.interior()]))


def test_no_alloc_step_refuses_batches_beyond_its_limits(cuda):
    lib = _lib()
    geo, ins, grid = _instances(cuda)[0]
    p = [t.data_ptr() for t in ins]
    one = native.make_fields(*p[:3], *p[:3], scalars=[], scalar_out=[])
    many = 129
    grids = (native.Grid * many)(*[grid] * many)
    fields = (native.Fields * many)(*[one] * many)
    assert lib.f2c_batch_step_static_v1(grids, fields, None, many, None) == 1
    assert "F2C_BATCH_NO_ALLOC_MAX_INSTANCES" in lib.f2c_last_error().decode()
    big = native.make_grid(4096, 2048, 64, 2, 10.0, 10.0, 5.0)
    depth = (ctypes.c_int32 * 1)(1)
    assert lib.f2c_batch_step_static_v1(ctypes.byref(big), ctypes.byref(one), depth, 1, None) == 1
    assert "F2C_BATCH_NO_ALLOC_MAX_ITEMS" in lib.f2c_last_error().decode()
