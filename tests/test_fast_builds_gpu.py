"""The fast-fp tile's two builds give the same bits.

Single-instance launches with at least 8 CTAs per SM of work run the tile compiled for three CTAs per SM
(`advection_fast_kernel<NS, MASK, 8, 3>`, 72 registers); smaller launches and the batched persistent kernel run it
compiled for two (96 registers). Register allocation must not change a value: a 512 x 512 x 64 instance through
the single launch (three-CTA build) equals the same instance through a one-instance batch (two-CTA build), bit
for bit, in both output modes.
"""
import numpy as np
import pytest

from compiler import native
from compiler import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,dt", [(native.TENDENCY, 0.0), (native.ADVANCE, 0.1)])
def test_three_cta_build_equals_two_cta_build(cuda, mode, dt):
    torch = cuda
    geo = wl.Geometry(512, 512, 64, halo=2)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    tiles = (geo.nx // 32) * (geo.ny // 8)
    kz = min(32, max(2, -(-tiles * geo.nz // (4 * sms))))
    assert tiles * -(-geo.nz // kz) >= 8 * sms  # the single launch takes the three-CTA build
    ins = wl.advection_fields_device(geo, 11, 1, torch)
    single = [torch.full_like(t, float("nan")) for t in ins]
    batched = [torch.full_like(t, float("nan")) for t in ins]
    p = [t.data_ptr() for t in ins]
    q = [t.data_ptr() for t in single]
    r = [t.data_ptr() for t in batched]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
    native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=mode, dt=dt, variant=native.FAST)
    fields = native.make_fields(*p[:3], *r[:3], scalars=p[3:], scalar_out=r[3:], mode=mode, dt=dt)
    batch = native.Batch([grid], [fields])
    ws = torch.empty(batch.workspace_bytes(), dtype=torch.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.set_fast_fp(True)
    batch.step()
    torch.cuda.synchronize()
    inner = geo.interior()
    for a, b in zip(single, batched):
        x, y = a.cpu().numpy()[inner], b.cpu().numpy()[inner]
        assert not np.isnan(x).any()
        assert np.array_equal(x.view(np.int64), y.view(np.int64))
