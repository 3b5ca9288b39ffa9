"""Residency runtime ABI on the CPU test backend (no GPU).

Each scenario drives the fort_scope_* entry points through ctypes. Scenarios
marked ``both`` run against this repository's runtime and, where the reference
checkout is present on this machine, against the reference's own runtime built
with its CPU test switch (oracle/build_ref.py): both must return the same
statuses, host values and transfer counts. The behaviours restated here are
those the reference's runtime tests exercise (compiler/tests/test_scoped_runtime.py,
test_scoped_domains.py, test_scoped_graph_replay.py, test_scoped_graph_queue.py,
test_scoped_host_completion.py, test_scoped_access_batch.py, test_scoped_scratch.py,
test_scoped_direct_transport.py, test_scoped_residency.py), each citing the scenario it follows. Scenarios
that need the reference's CPU build to leave device kernels unrun are not
restated: this runtime's CPU backend runs test kernels as host functions.
"""

import ctypes as c
import json
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from compiler import native
from compiler.runtime import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ours():
    return abi.bind(c.CDLL(str(native.build_cpu_runtime())))


def _reference():
    from oracle import build_ref

    path = build_ref.build_if_available()
    if path is None:
        pytest.skip("reference runtime not buildable here")
    return abi.bind(c.CDLL(str(path)))


@pytest.fixture(scope="module")
def ours():
    return _ours()


@pytest.fixture(scope="module", params=["gb300", "reference"])
def both(request):
    return _ours() if request.param == "gb300" else _reference()


def _array(values):
    a = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
    return a, a.ctypes.data


def _dev(pointer, count):
    return np.ctypeslib.as_array(c.cast(pointer, c.POINTER(c.c_double)), shape=(count,))


def _device_begin(scope, handle, access):
    out = c.c_void_p()
    status = scope.lib.fort_scope_device_begin(scope.handle, handle, c.byref(access), c.byref(out))
    return status, out.value


# ------------------------------------------------------------------------------- both runtimes


def test_read_mirror_and_duplicate_registration(both):
    scope = abi.Scope(both)
    host, address = _array(range(8))
    status, h = scope.register(address, [8], lower=[-2])
    assert status == abi.OK
    status, again = scope.register(address, [8], lower=[-2])
    assert (status, again) == (abi.OK, h)
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[:] += 10
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == [i + 10.0 for i in range(8)]
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    status, dev = _device_begin(scope, again, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and _dev(dev, 8)[7] == 17.0
    assert both.fort_scope_device_end(scope.handle, again) == abi.OK
    stats = scope.stats()
    assert (stats.uploads, stats.downloads, stats.allocations) == (1, 1, 1)
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_wait(scope.handle) == abi.STALE


def test_device_interior_and_host_faces_both_survive(both):
    """The device writes the interior of a 4x4x4 array, the host its opposite x faces; both persist."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(64.0))
    status, h = scope.register(address, [4, 4, 4])
    assert status == abi.OK
    interior = ((1, 1, 1), (3, 3, 3))
    acc = abi.access(read=[interior], write=[interior], overwrite=[interior])
    status, dev = _device_begin(scope, h, acc)
    assert status == abi.OK
    d = _dev(dev, 64).reshape(4, 4, 4)  # [k][j][i]
    d[1:3, 1:3, 1:3] = -1.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    faces = [((0, 0, 0), (1, 4, 4)), ((3, 0, 0), (4, 4, 4))]
    acc = abi.access(write=faces, overwrite=faces)
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(acc)) == abi.OK
    view = host.reshape(4, 4, 4)
    view[:, :, 0] = 100.0
    view[:, :, 3] = 200.0
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    arr = (abi.U64 * 1)(h)
    assert both.fort_scope_observe_v1(scope.handle, arr, 1) == abi.OK
    expect = np.arange(64.0).reshape(4, 4, 4)
    expect[1:3, 1:3, 1:3] = -1.0
    expect[:, :, 0] = 100.0
    expect[:, :, 3] = 200.0
    assert np.array_equal(view, expect)
    # and the device copy agrees where the device is current
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    assert np.array_equal(_dev(dev, 64).reshape(4, 4, 4), expect)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_undefined_reads_are_rejected(both):
    scope = abi.Scope(both)
    host, address = _array(np.zeros(6))
    status, h = scope.register(address, [6], initialized=False)
    assert status == abi.OK
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.UNINITIALIZED
    # an overwrite defines the values; then they can be read
    status, dev = _device_begin(scope, h, abi.access(write=[((0,), (6,))], overwrite=[((0,), (6,))]))
    assert status == abi.OK
    _dev(dev, 6)[:] = 4.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [4.0] * 6


def test_partial_initialization(both):
    scope = abi.Scope(both)
    host, address = _array(np.arange(10.0))
    status, h = scope.register(address, [10], defined=[((2,), (8,))])
    assert status == abi.OK
    status, _ = _device_begin(scope, h, abi.access(read=[((1,), (5,))]))
    assert status == abi.UNINITIALIZED
    status, dev = _device_begin(scope, h, abi.access(read=[((2,), (8,))], write=[((2,), (8,))]))
    assert status == abi.OK
    _dev(dev, 10)[2:8] *= 2
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [0, 1, 4, 6, 8, 10, 12, 14, 8, 9]


def test_forget_definition_keeps_values_but_forbids_reads(both):
    scope = abi.Scope(both)
    host, address = _array(np.ones(4))
    status, h = scope.register(address, [4])
    assert status == abi.OK
    assert both.fort_scope_forget_definition(scope.handle, h) == abi.OK
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [1.0] * 4


def test_prepared_access_rules(both):
    scope = abi.Scope(both)
    _, address = _array(np.ones(4))
    _, h = scope.register(address, [4])
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    # a second access on a prepared array, and definition changes under it, are refused
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status != abi.OK
    assert both.fort_scope_forget_definition(scope.handle, h) != abi.OK
    assert both.fort_scope_cancel_access(scope.handle, h) == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) != abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_alias_and_layout_errors(both):
    scope = abi.Scope(both)
    host, address = _array(np.zeros(16))
    status, h = scope.register(address, [16])
    assert status == abi.OK
    # overlapping host storage under another identity
    status, _ = scope.register(address + 8 * 4, [4], identity=address + 32)
    assert status == abi.ALIAS
    # the layout comes back as registered
    layout = abi.Layout()
    assert both.fort_scope_layout_get(scope.handle, h, c.byref(layout)) == abi.OK
    assert (layout.rank, layout.type, layout.element_bytes, layout.extents[0]) == (1, abi.REAL64, 8, 16)
    assert both.fort_scope_unregister(scope.handle, h) == abi.OK
    assert both.fort_scope_layout_get(scope.handle, h, c.byref(layout)) == abi.STALE
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_unregister_publishes_device_values(both):
    scope = abi.Scope(both)
    host, address = _array(np.zeros(5))
    _, h = scope.register(address, [5])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 5)[:] = 3.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert host.tolist() == [0.0] * 5
    assert both.fort_scope_unregister(scope.handle, h) == abi.OK
    assert host.tolist() == [3.0] * 5
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_observation_publishes_each_array_once_in_one_wait(both):
    """Observing three arrays whose middle a device task defined: one wait, one download each, and the
    undefined ends stay undefined on the host (reference: test_scoped_graph_replay.py:83-104)."""
    scope = abi.Scope(both)
    middle = [((2,), (6,))]
    arrays = []
    for n in range(1, 4):
        host, address = _array(np.arange(8, dtype=np.float64))
        status, h = scope.register(address, [8], identity=n, initialized=False)
        assert status == abi.OK
        status, dev = _device_begin(scope, h, abi.access(write=middle, overwrite=middle))
        assert status == abi.OK
        _dev(dev, 8)[2:6] = [100.0 * n + i for i in range(2, 6)]
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
        arrays.append((host, h))
    before = scope.stats()
    assert both.fort_scope_observe_v1(scope.handle, (abi.U64 * 3)(*[h for _, h in arrays]), 3) == abi.OK
    after = scope.stats()
    assert (after.waits, after.downloads) == (before.waits + 1, before.downloads + 3)
    for n, (host, h) in enumerate(arrays, 1):
        assert host.tolist() == [0, 1, *[100.0 * n + i for i in range(2, 6)], 6, 7]
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == \
            abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_an_invalid_observation_publishes_nothing(both):
    """A batch naming an unknown handle, or one handle twice, is refused before any array is published
    (reference: test_scoped_graph_replay.py:108-123)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[0] = 1000.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    before = bytes(scope.stats())
    for other, status in ((2**63, abi.STALE), (h, abi.ALIAS)):
        assert both.fort_scope_observe_v1(scope.handle, (abi.U64 * 2)(h, other), 2) == status
        assert bytes(scope.stats()) == before and host[0] == 0.0
    assert both.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(h), 1) == abi.OK
    assert host[0] == 1000.0
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_discard_and_retire_publish_no_dead_values(both):
    """Discard drops the device's values without a transfer (the host may not read them any more); retire
    frees the storage without publishing and the handle goes stale (reference:
    test_scoped_graph_replay.py:127-150)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[0] = 1000.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    before = scope.stats()
    assert both.fort_scope_discard_v1(scope.handle, h) == abi.OK
    after = scope.stats()
    assert (after.downloads, after.waits) == (before.downloads, before.waits)
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[:] = 2000.0 + np.arange(8)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert scope.stats().allocations == 1                    # the discarded storage was reused
    assert both.fort_scope_retire_v1(scope.handle, h) == abi.OK
    final = scope.stats()
    assert (final.downloads, final.allocated_bytes) == (0, 0)
    assert host.tolist() == list(range(8))
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.STALE
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_retire_and_discard_refuse_an_open_access(both):
    """Neither drops an array a device access still holds; an empty observation waits for nothing, a retirement
    for the array's work (reference: test_scoped_graph_replay.py:154-168)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    assert both.fort_scope_discard_v1(scope.handle, h) == abi.STATE
    assert both.fort_scope_retire_v1(scope.handle, h) == abi.STATE
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    waits = scope.stats().waits
    assert both.fort_scope_observe_v1(scope.handle, None, 0) == abi.OK
    assert scope.stats().waits == waits
    assert both.fort_scope_retire_v1(scope.handle, h) == abi.OK
    assert scope.stats().waits == waits + 1
    assert both.fort_scope_close(scope.handle) == abi.OK


def _domain(lib, device=0):
    handle = abi.U64()
    assert lib.fort_scope_domain_create_v1(device, c.byref(handle)) == abi.OK
    return handle.value


def test_domain_ordinal_is_metadata_and_stale_after_close(both):
    """The device ordinal of a domain is a query that allocates nothing; after close the handle is stale
    (reference: test_scoped_domains.py:188-195)."""
    domain = _domain(both, 3)
    ordinal = c.c_int(-1)
    assert both.fort_scope_domain_device_get_v1(domain, c.byref(ordinal)) == abi.OK and ordinal.value == 3
    stats = abi.Stats()
    assert both.fort_scope_domain_stats_get_v1(domain, c.byref(stats)) == abi.OK
    assert bytes(stats) == bytes(abi.Stats())
    assert both.fort_scope_domain_close_v1(domain) == abi.OK
    assert both.fort_scope_domain_device_get_v1(domain, c.byref(ordinal)) == abi.STALE


def test_retired_storage_never_lends_its_handle_or_definition(both):
    """After retirement a new registration of the same host array gets a new handle, the old one is stale, and a
    later context of the same domain finds the new storage (with its definition) and refuses an older allocation
    generation (reference: test_scoped_domains.py:198-219)."""
    domain = _domain(both)
    host, address = _array([1.0, 2.0, 3.0, 4.0])
    scope = abi.Scope(both, domain=domain)
    status, old = scope.register(address, [4])
    assert status == abi.OK
    assert both.fort_scope_retire_v1(scope.handle, old) == abi.OK
    status, new = scope.register(address, [4], generation=2, initialized=False)
    assert status == abi.OK and new != old
    out = c.c_void_p()
    read = abi.access(flags=abi.READ_ALL)
    assert both.fort_scope_device_begin(scope.handle, old, c.byref(read), c.byref(out)) == abi.STALE
    assert both.fort_scope_device_begin(scope.handle, new, c.byref(read), c.byref(out)) == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK
    again = abi.Scope(both, domain=domain)
    assert again.register(address, [4], generation=1)[0] == abi.STALE
    status, same = again.register(address, [4], generation=2, initialized=True)
    assert status == abi.OK and same == new
    assert both.fort_scope_device_begin(again.handle, same, c.byref(read), c.byref(out)) == abi.UNINITIALIZED
    assert both.fort_scope_close(again.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK


def test_contexts_never_adopt_foreign_handles(both):
    """The same host array registered in another domain, or in a private context, gets its own handle, and
    neither context accepts the other's (reference: test_scoped_domains.py:297-316)."""
    first, second = _domain(both), _domain(both)
    owner, foreign, private = abi.Scope(both, domain=first), abi.Scope(both, domain=second), abi.Scope(both)
    host, address = _array([7.0, 9.0])
    status, owned = owner.register(address, [2])
    assert status == abi.OK
    read = abi.access(flags=abi.READ_ALL)
    for scope in (foreign, private):
        status, handle = scope.register(address, [2])
        assert status == abi.OK and handle != owned
        assert both.fort_scope_host_begin(scope.handle, owned, c.byref(read)) == abi.STALE
        assert both.fort_scope_host_begin(owner.handle, handle, c.byref(read)) == abi.STALE
    for scope in (owner, foreign, private):
        assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(first) == abi.OK and both.fort_scope_domain_close_v1(second) == abi.OK


def _completion(scope):
    out = abi.CompletionStats()
    assert scope.lib.fort_scope_completion_stats_get_v1(scope.handle, c.byref(out)) == abi.OK
    assert out.version == 1
    return out


def test_host_access_to_an_untouched_array_waits_for_nothing(both):
    """Device work on one array does not make host work on another wait (reference:
    test_scoped_host_completion.py:40-54)."""
    scope = abi.Scope(both)
    _, a = _array(np.arange(8, dtype=np.float64))
    host, b = _array(np.arange(8, dtype=np.float64))
    _, on_device = scope.register(a, [8], identity=1)
    _, on_host = scope.register(b, [8], identity=2)
    status, dev = _device_begin(scope, on_device, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[0] = 100.0
    assert both.fort_scope_device_end(scope.handle, on_device) == abi.OK
    waits = scope.stats().waits
    assert both.fort_scope_host_begin(scope.handle, on_host, c.byref(abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))) \
        == abi.OK
    host[0] = 999.0
    assert both.fort_scope_host_end(scope.handle, on_host) == abi.OK
    assert scope.stats().waits == waits
    assert _completion(scope).independent_host_tasks == 1
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_an_upload_in_flight_fences_only_overlapping_host_writes(both):
    """While an upload reads part of the host copy, host reads and writes elsewhere go ahead; a write over it
    waits on its event. A cancelled write leaves the device copy valid (reference:
    test_scoped_host_completion.py:57-85)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8], identity=1)
    middle = [((2,), (6,))]
    status, _ = _device_begin(scope, h, abi.access(read=middle))
    assert status == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    waits = scope.stats().waits
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == list(range(8))
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    first = [((0,), (2,))]
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(write=first, overwrite=first))) == abi.OK
    host[0], host[1] = -1.0, -2.0
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert scope.stats().waits == waits
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(write=middle, overwrite=middle))) == abi.OK
    assert scope.stats().waits == waits + 1
    assert both.fort_scope_cancel_access(scope.handle, h) == abi.OK
    uploads = scope.stats().uploads
    status, dev = _device_begin(scope, h, abi.access(read=middle))
    assert status == abi.OK and _dev(dev, 8)[2:6].tolist() == [2.0, 3.0, 4.0, 5.0]
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert scope.stats().uploads == uploads
    assert _completion(scope).event_waits == 1
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_one_upload_batch_shares_one_event(both):
    """A device access over five arrays records one event for its uploads, and a host write over all five waits
    on it once (reference: test_scoped_host_completion.py:88-104)."""
    scope = abi.Scope(both)
    handles, keep = [], []
    for n in range(1, 6):
        host, address = _array(np.arange(8, dtype=np.float64))
        keep.append(host)
        handles.append(scope.register(address, [8], identity=n)[1])
    reads = [abi.access(flags=abi.READ_ALL) for _ in handles]
    bindings = (abi.Binding * 5)(*[abi.Binding(h, r) for h, r in zip(handles, reads)])
    pointers = (c.c_void_p * 5)()
    assert both.fort_scope_access_begin_v1(scope.handle, bindings, 5, 1, pointers) == abi.OK
    for h in handles:
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert _completion(scope).event_records == 1
    writes = [abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL) for _ in handles]
    bindings = (abi.Binding * 5)(*[abi.Binding(h, w) for h, w in zip(handles, writes)])
    waits = scope.stats().waits
    assert both.fort_scope_access_begin_v1(scope.handle, bindings, 5, 0, None) == abi.OK
    assert scope.stats().waits == waits + 1 and _completion(scope).event_waits == 1
    for h in handles:
        assert both.fort_scope_cancel_access(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_host_only_work_records_no_events(both):
    """Host accesses with no device work behind them need no event and no wait (reference:
    test_scoped_host_completion.py:107-118)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8], identity=1)
    for _ in range(5):
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))) \
            == abi.OK
        host[0] += 1.0
        assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    done = _completion(scope)
    assert (done.event_records, done.created_events, done.event_waits, done.stream_waits) == (0, 0, 0, 0)
    assert done.independent_host_tasks == 5
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_detached_context_leaves_values_to_the_domain(both):
    """Closing a context of a domain publishes nothing; the next context finds the same storage, downloads only
    what the host reads and re-uploads nothing; closing the domain publishes (reference:
    test_scoped_domains.py:130-163)."""
    domain = _domain(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    first = abi.Scope(both, domain=domain)
    _, h = first.register(address, [8], lower=[-2])
    interior = [((1,), (7,))]
    status, dev = _device_begin(first, h, abi.access(read=interior, write=interior))
    assert status == abi.OK
    _dev(dev, 8)[1:7] += 100.0
    assert both.fort_scope_device_end(first.handle, h) == abi.OK
    assert both.fort_scope_close(first.handle) == abi.OK
    assert host.tolist() == list(range(8))                       # not published at detach
    stats = abi.Stats()
    assert both.fort_scope_domain_stats_get_v1(domain, c.byref(stats)) == abi.OK and stats.download_bytes == 0
    second = abi.Scope(both, domain=domain)
    status, same = second.register(address, [8], lower=[-2], initialized=False)
    assert status == abi.OK and same == h
    assert both.fort_scope_host_begin(second.handle, same, c.byref(abi.access(read=[((3,), (4,))]))) == abi.OK
    assert (host[3], host[2]) == (103.0, 2.0)                    # only the element read came home
    assert both.fort_scope_host_end(second.handle, same) == abi.OK
    status, dev = _device_begin(second, same, abi.access(read=interior))
    assert status == abi.OK and _dev(dev, 8)[1:7].tolist() == [100.0 + i for i in range(1, 7)]
    assert both.fort_scope_device_end(second.handle, same) == abi.OK
    after = second.stats()
    assert (after.upload_bytes, after.download_bytes) == (48, 8)
    assert both.fort_scope_close(second.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK
    assert host.tolist() == [0.0, *[100.0 + i for i in range(1, 7)], 7.0]
    assert both.fort_scope_wait(first.handle) == abi.STALE
    assert both.fort_scope_create_in_domain_v1(domain, c.byref(abi.U64())) == abi.STALE


def test_one_context_at_a_time_and_no_detach_under_an_access(both):
    """A domain lends itself to one context at a time and cannot close while lent; a context cannot close while
    an access is prepared; a private context has no domain to report (reference: test_scoped_domains.py:166-185)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    assert both.fort_scope_create_in_domain_v1(domain, c.byref(abi.U64())) == abi.STATE
    assert both.fort_scope_domain_close_v1(domain) == abi.STATE
    found = abi.U64()
    assert both.fort_scope_domain_get_v1(scope.handle, c.byref(found)) == abi.OK and found.value == domain
    host, address = _array([1.0, 2.0])
    _, h = scope.register(address, [2])
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.STATE
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK
    private = abi.Scope(both)
    assert both.fort_scope_domain_get_v1(private.handle, c.byref(found)) == abi.OK and found.value == 0
    assert both.fort_scope_close(private.handle) == abi.OK


def test_stencil_sections_move_exactly_their_cells(both):
    """An array defined only on a stencil's ten shifted footprints (negative lower bounds) moves exactly those
    cells, coalesced into three transfers each way; a read of the whole array is refused as uninitialized and moves
    nothing (reference: test_scoped_runtime.py:228-261)."""
    scope = abi.Scope(both)
    shape, interior = (8, 7, 6), (5, 4, 3)
    host, address = _array(np.arange(8 * 7 * 6, dtype=np.float64))
    shifts = [(0, 0, 0), (-1, 0, 0), (0, 1, 0), (-1, 1, 0), (0, -1, 0), (-1, -1, 0), (0, 0, 1), (-1, 0, 1),
              (0, 0, -1), (-1, 0, -1)]
    boxes = [(tuple(1 + d for d in s), tuple(n + 1 + d for n, d in zip(interior, s))) for s in shifts]
    cells = {i + 8 * (j + 7 * k) for lo, hi in boxes for k in range(lo[2], hi[2]) for j in range(lo[1], hi[1])
             for i in range(lo[0], hi[0])}
    status, h = scope.register(address, list(shape), lower=[-2, -5, -9], defined=boxes)
    assert status == abi.OK
    status, dev = _device_begin(scope, h, abi.access(read=boxes, write=boxes))
    assert status == abi.OK
    stats = scope.stats()
    assert (stats.uploads, stats.upload_bytes) == (3, 8 * len(cells))
    view = _dev(dev, 8 * 7 * 6)
    assert all(view[o] == o for o in cells)
    for o in cells:
        view[o] += 1000.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    before = bytes(scope.stats())
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    assert bytes(scope.stats()) == before
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(read=boxes))) == abi.OK
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    stats = scope.stats()
    assert (stats.downloads, stats.download_bytes) == (3, 8 * len(cells))
    assert all(host[o] == o + 1000.0 for o in cells)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_partial_device_write_keeps_the_host_values_around_it(both):
    """A device write that need not cover its section first brings the section's host values along, so cells it
    skips keep them; an uninitialized array cannot be read, and a complete overwrite uploads nothing (reference:
    test_scoped_runtime.py:264-291)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, dev = _device_begin(scope, h, abi.access(write=[((2,), (6,))]))
    assert status == abi.OK
    _dev(dev, 8)[2], _dev(dev, 8)[4] = 102.0, 104.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(read=[((1,), (7,))]))) == abi.OK
    assert host.tolist() == [0, 1, 102, 3, 104, 5, 6, 7]
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    stats = scope.stats()
    assert stats.upload_bytes == stats.download_bytes == 32
    assert both.fort_scope_close(scope.handle) == abi.OK
    scope = abi.Scope(both)
    out, address = _array(np.zeros(8))
    _, h = scope.register(address, [8], initialized=False)
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.UNINITIALIZED
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[:] = 2.0 * np.arange(8)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert scope.stats().upload_bytes == 0
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert out.tolist() == [2.0 * i for i in range(8)]


def test_registration_aliases_generations_sizes_and_empty_arrays(both):
    """Another identity over the same host storage is an alias; the same identity with another allocation
    generation is stale until it is unregistered; an array whose size overflows is an argument error; an empty
    array registers without storage and allocates nothing (reference: test_scoped_runtime.py:322-342)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    status, first = scope.register(address, [8])
    assert status == abi.OK
    assert scope.register(address, [8], identity=2)[0] == abi.ALIAS
    assert scope.register(address, [8], generation=2)[0] == abi.STALE
    assert both.fort_scope_unregister(scope.handle, first) == abi.OK
    status, second = scope.register(address, [8], generation=2)
    assert status == abi.OK and second != first
    assert both.fort_scope_host_begin(scope.handle, first, c.byref(abi.access(flags=abi.READ_ALL))) == abi.STALE
    huge = (1 << (8 * c.sizeof(abi.SIZE))) - 1
    assert scope.register(address, [huge], identity=3)[0] == abi.ARGUMENT
    status, empty = scope.register(None, [huge, 0], identity=3)
    assert status == abi.OK
    status, dev = _device_begin(scope, empty, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and not dev
    assert both.fort_scope_device_end(scope.handle, empty) == abi.OK
    assert scope.stats().allocations == 0
    assert both.fort_scope_close(scope.handle) == abi.OK


def _inject(monkeypatch, what):
    """Turn on a host-side failure in both runtimes (each reads its own switch)."""
    monkeypatch.setenv(f"F2C_TEST_FAIL_{what}", "1")
    monkeypatch.setenv(f"FORT_SCOPE_TEST_FAIL_{what}", "1")


def test_definitions_past_the_section_limit_are_refused_before_the_access(both):
    """A host write that would need a 129th defined section is refused at preparation, with nothing committed and
    no access left open (reference: test_scoped_runtime.py:345-360)."""
    scope = abi.Scope(both)
    limit = 128
    host, address = _array(np.zeros(2 * limit + 16))
    _, h = scope.register(address, [2 * limit + 16], initialized=False)
    for i in range(limit):
        box = [((2 * i,), (2 * i + 1,))]
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(write=box, overwrite=box))) == abi.OK
        host[2 * i] = i + 10.0
        assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    box = [((2 * limit,), (2 * limit + 1,))]
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(write=box, overwrite=box))) == \
        abi.BOUNDARY
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert [host[2 * i] for i in range(limit)] == [i + 10.0 for i in range(limit)]


def test_an_allocation_failure_keeps_earlier_work_and_the_context(both, monkeypatch):
    """A device access that cannot allocate fails with RESOURCE before any change; earlier results stay
    reachable and the host can carry on where the device could not (reference: test_scoped_runtime.py:363-386)."""
    scope = abi.Scope(both)
    host, a = _array(np.arange(8, dtype=np.float64))
    other, b = _array(np.zeros(8))
    _, h = scope.register(a, [8])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[:] += 10.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    _, unused = scope.register(b, [8], identity=2, initialized=False)
    _inject(monkeypatch, "ALLOC")
    status, _ = _device_begin(scope, unused, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.RESOURCE
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == [i + 10.0 for i in range(8)]
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, unused,
                                      c.byref(abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))) == abi.OK
    other[:] = host * 2
    assert both.fort_scope_host_end(scope.handle, unused) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert other.tolist() == [2 * (i + 10.0) for i in range(8)]


def test_a_failed_completion_poisons_the_context(both, monkeypatch):
    """When waiting for device work fails, the context refuses everything after (no replay) until it is
    abandoned (reference: test_scoped_runtime.py:389-403)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[0] = 100.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    _inject(monkeypatch, "WAIT")
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.EXECUTION
    assert both.fort_scope_close(scope.handle) == abi.EXECUTION
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert both.fort_scope_wait(scope.handle) == abi.STALE


def test_contexts_on_several_threads_stay_independent(both):
    """Twelve contexts on four threads, each doubling its own array on the device (reference:
    test_scoped_runtime.py:406-425)."""
    from concurrent.futures import ThreadPoolExecutor

    def run(seed):
        scope = abi.Scope(both)
        host, address = _array(seed + np.arange(32, dtype=np.float64))
        _, h = scope.register(address, [32])
        status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
        assert status == abi.OK
        _dev(dev, 32)[:] *= 2.0
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
        assert both.fort_scope_close(scope.handle) == abi.OK
        return host.tolist()

    with ThreadPoolExecutor(max_workers=4) as pool:
        results = list(pool.map(run, range(12)))
    assert results == [[2.0 * (seed + i) for i in range(32)] for seed in range(12)]


def test_undefined_halos_are_never_moved_or_read(both):
    """An array defined only in its middle uploads only the middle; a read of its undefined halo is refused, even
    after a re-registration that claims the array initialized (reference: test_scoped_runtime.py:486-506)."""
    scope = abi.Scope(both)
    host, address = _array(101.0 + np.arange(8))
    middle = [((2,), (6,))]
    status, h = scope.register(address, [8], defined=middle, lower=[-2])
    assert status == abi.OK
    status, dev = _device_begin(scope, h, abi.access(read=middle, write=middle))
    assert status == abi.OK
    _dev(dev, 8)[2:6] += 10.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert scope.stats().upload_bytes == 32
    halo = abi.access(read=[((0,), (1,))])
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(halo)) == abi.UNINITIALIZED
    status, again = scope.register(address, [8], lower=[-2], initialized=True)
    assert status == abi.OK and again == h
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(halo)) == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [101, 102, 113, 114, 115, 116, 107, 108]


def test_forgetting_a_definition_keeps_the_values_already_written(both):
    """forget_definition makes reads illegal without moving anything, but what the device already wrote still
    reaches the host at close, and the allocation is reused (reference: test_scoped_runtime.py:509-530)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[:] = 1000.0 + np.arange(8)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_forget_definition(scope.handle, h) == abi.OK
    assert scope.stats().downloads == 0
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    middle = [((2,), (6,))]
    status, dev = _device_begin(scope, h, abi.access(write=middle, overwrite=middle))
    assert status == abi.OK
    _dev(dev, 8)[2:6] = 2000.0 + np.arange(2, 6)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert scope.stats().allocations == 1
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [1000, 1001, 2002, 2003, 2004, 2005, 1006, 1007]


def test_forgetting_a_definition_cannot_lose_executed_device_writes(both):
    """After forget_definition a read is refused, nothing moves and nothing waits, yet closing publishes the
    device's writes exactly (reference: test_scoped_runtime.py:533-557)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    written = [((1,), (7,))]
    status, dev = _device_begin(scope, h, abi.access(write=written, overwrite=written))
    assert status == abi.OK
    _dev(dev, 8)[1:7] = 3000.0 + np.arange(1, 7)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    before = scope.stats()
    assert both.fort_scope_forget_definition(scope.handle, h) == abi.OK
    after = scope.stats()
    assert (after.download_bytes, after.waits) == (before.download_bytes, before.waits)
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(read=[((3,), (4,))]))) == \
        abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [0, 3001, 3002, 3003, 3004, 3005, 3006, 7]


@pytest.mark.parametrize("source", ["host", "device"])
def test_reconciling_fragmented_reads_keeps_the_current_copy(both, source):
    """129 single-cell reads fragment the current sections past the limit; the reconciliation brings the other copy
    up to date once, so a later whole-array access moves nothing more (reference: test_scoped_runtime.py:563-601)."""
    scope = abi.Scope(both)
    size = 2 * 128 + 16
    host, address = _array(np.arange(size, dtype=np.float64))
    _, h = scope.register(address, [size])
    if source == "device":
        status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
        assert status == abi.OK
        _dev(dev, size)[:] = np.arange(size) + 100.0
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    else:
        status, _ = _device_begin(scope, h, abi.access())  # storage without values
        assert status == abi.OK
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    for i in range(128 + 1):
        cell = abi.access(read=[((2 * i,), (2 * i + 1,))])
        if source == "device":
            assert both.fort_scope_host_begin(scope.handle, h, c.byref(cell)) == abi.OK
            assert host[2 * i] == 2 * i + 100.0
            assert both.fort_scope_host_end(scope.handle, h) == abi.OK
        else:
            status, dev = _device_begin(scope, h, cell)
            assert status == abi.OK and _dev(dev, size)[2 * i] == 2 * i
            assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert scope.stats().reconciliations
    before = scope.stats()
    if source == "device":
        status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
        assert status == abi.OK and _dev(dev, size).tolist() == [i + 100.0 for i in range(size)]
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
        assert scope.stats().upload_bytes == before.upload_bytes
    else:
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
        assert both.fort_scope_host_end(scope.handle, h) == abi.OK
        assert scope.stats().download_bytes == before.download_bytes
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_wait(scope.handle) == abi.STALE


def test_definitions_cannot_change_under_a_prepared_access(both):
    """(reference: test_scoped_runtime.py:604-613)"""
    scope = abi.Scope(both)
    _, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))) == \
        abi.OK
    assert both.fort_scope_forget_definition(scope.handle, h) == abi.STATE
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_initialized_sections_are_checked_before_registration(both):
    """A section outside the array is refused; an empty list registers an array with nothing defined (reference:
    test_scoped_runtime.py:616-625)."""
    scope = abi.Scope(both)
    _, address = _array(np.arange(8, dtype=np.float64))
    assert scope.register(address, [8], defined=[((0,), (9,))])[0] == abi.ARGUMENT
    status, h = scope.register(address, [8], defined=[])
    assert status == abi.OK
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_declared_budget_evicts_and_the_host_carries_on(both):
    """Under a budget of one array the second array's device access evicts the first, publishing its device values;
    the budget cannot be declared again; the host finishes the work (reference: test_scoped_runtime.py:628-653)."""
    scope = abi.Scope(both)
    host, a = _array(np.arange(8, dtype=np.float64))
    other, b = _array(np.zeros(8))
    _, first = scope.register(a, [8])
    _, second = scope.register(b, [8], identity=2, initialized=False)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    status, dev = _device_begin(scope, first, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[:] += 100.0
    assert both.fort_scope_device_end(scope.handle, first) == abi.OK
    assert both.fort_scope_set_device_budget(scope.handle, 128) == abi.STATE
    status, _ = _device_begin(scope, second, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    stats = scope.stats()
    assert stats.allocated_bytes == stats.peak_device_bytes == 64
    assert host.tolist() == [i + 100.0 for i in range(8)]
    assert both.fort_scope_cancel_access(scope.handle, second) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, first, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert both.fort_scope_host_end(scope.handle, first) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, second,
                                      c.byref(abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))) == abi.OK
    other[:] = host * 2
    assert both.fort_scope_host_end(scope.handle, second) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert other.tolist() == [2 * (i + 100.0) for i in range(8)]


def test_a_zero_budget_allocates_nothing(both):
    """A device access that cannot fit a zero budget is refused before the device is brought up (reference:
    test_scoped_runtime.py:659-668)."""
    scope = abi.Scope(both)
    _, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    assert both.fort_scope_set_device_budget(scope.handle, 0) == abi.OK
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.RESOURCE and scope.stats().allocations == 0
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_workspace_leases_share_the_budget_and_outlive_the_context(both):
    """A provider's workspace lease counts against the domain's budget exactly, can shrink to make room, survives
    the context, holds the domain open, and belongs to its domain alone (reference:
    test_scoped_domains.py:222-245)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    assert both.fort_scope_set_device_budget(scope.handle, 96) == abi.OK
    lease = abi.U64()
    assert both.fort_scope_domain_workspace_reserve_v1(domain, 64, c.byref(lease)) == abi.OK
    _, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.RESOURCE and scope.stats().allocations == 0
    assert both.fort_scope_domain_workspace_resize_v1(domain, lease.value, 32) == abi.OK
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_domain_workspace_resize_v1(domain, lease.value, 33) == abi.RESOURCE
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.STATE
    other = _domain(both)
    assert both.fort_scope_domain_workspace_release_v1(other, lease.value) == abi.STALE
    assert both.fort_scope_domain_close_v1(other) == abi.OK
    assert both.fort_scope_domain_workspace_release_v1(domain, lease.value) == abi.OK
    assert both.fort_scope_domain_workspace_release_v1(domain, lease.value) == abi.STALE
    assert both.fort_scope_domain_close_v1(domain) == abi.OK


def test_after_a_storage_cut_identities_bind_to_their_new_arrays(both):
    """Closing a domain publishes and cuts storage; a new domain binds each identity to whatever array it now
    names, at a new generation, with fresh handles; an identity cannot be moved to other storage or back to an old
    generation while registered (reference: test_scoped_domains.py:248-296)."""
    left, la = _array([1.0, 2.0])
    right, ra = _array([3.0, 4.0])
    first = _domain(both)
    before = abi.Scope(both, domain=first)
    old = []
    for identity, address, increment in ((1, la, 10.0), (2, ra, 20.0)):
        _, h = before.register(address, [2], identity=identity)
        old.append(h)
        status, dev = _device_begin(before, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
        assert status == abi.OK
        _dev(dev, 2)[:] += increment
        assert both.fort_scope_device_end(before.handle, h) == abi.OK
    assert both.fort_scope_close(before.handle) == abi.OK
    assert (left.tolist(), right.tolist()) == ([1.0, 2.0], [3.0, 4.0])
    assert both.fort_scope_domain_close_v1(first) == abi.OK
    assert (left.tolist(), right.tolist()) == ([11.0, 12.0], [23.0, 24.0])
    second = _domain(both)
    after = abi.Scope(both, domain=second)
    current = []
    for identity, address, expected in ((1, ra, [23.0, 24.0]), (2, la, [11.0, 12.0])):
        status, h = after.register(address, [2], identity=identity, generation=2)
        assert status == abi.OK
        current.append(h)
        status, dev = _device_begin(after, h, abi.access(flags=abi.READ_ALL))
        assert status == abi.OK and _dev(dev, 2).tolist() == expected
        assert both.fort_scope_device_end(after.handle, h) == abi.OK
    for h in old:
        assert _device_begin(after, h, abi.access(flags=abi.READ_ALL))[0] == abi.STALE
    assert not set(old) & set(current)
    assert after.register(la, [2], identity=1, generation=2)[0] == abi.ARGUMENT   # other storage
    assert after.register(ra, [2], identity=1, generation=1)[0] == abi.STALE      # an older generation
    assert both.fort_scope_close(after.handle) == abi.OK
    again = abi.Scope(both, domain=second)
    for identity, address, h in ((1, ra, current[0]), (2, la, current[1])):
        status, same = again.register(address, [2], identity=identity, generation=2, initialized=False)
        assert status == abi.OK and same == h
    assert both.fort_scope_host_begin(after.handle, current[0], c.byref(abi.access(flags=abi.READ_ALL))) == abi.STALE
    assert both.fort_scope_close(again.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(second) == abi.OK


def _descriptor(address, shape, generation, lower, keep):
    extents = (abi.SIZE * len(shape))(*shape)
    bounds = (c.c_int64 * len(shape))(*lower)
    keep += [extents, bounds]
    return abi.Layout(len(shape), abi.REAL64, 8, address, extents, bounds, generation)


def _swap(lib, scope, first, second, after_first, after_second):
    now_first, now_second = abi.U64(111), abi.U64(222)
    status = lib.fort_scope_identity_swap_v1(scope.handle, first, second, c.byref(after_first), c.byref(after_second),
                                             c.byref(now_first), c.byref(now_second))
    return status, now_first.value, now_second.value


def test_an_exchange_renames_storage_without_moving_it(both):
    """After the host swapped two arrays' descriptors, the exchange tells each identity which storage it now names:
    no copy, allocation, wait or replay; each name finds its dirty device values, generation and layout; the
    domain publishes them to the right arrays (reference: test_scoped_domains.py:319-371)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    a, pa = _array([1.0, 2.0, 3.0, 4.0])
    b, pb = _array([11.0, 12.0, 13.0, 14.0, 15.0, 16.0])
    handles = []
    for identity, address, shape, lower, generation, n in ((1, pa, [2, 2], [-2, 3], 11, 4), (2, pb, [3, 2], [-7, 9], 27, 6)):
        status, h = scope.register(address, shape, identity=identity, lower=lower, generation=generation)
        assert status == abi.OK
        handles.append(h)
        status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
        assert status == abi.OK
        _dev(dev, n)[:] += 100.0 * identity
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    again = abi.Scope(both, domain=domain)
    before = bytes(again.stats())
    keep = []
    status, now_a, now_b = _swap(both, again, handles[0], handles[1], _descriptor(pb, [3, 2], 27, [-7, 9], keep),
                                 _descriptor(pa, [2, 2], 11, [-2, 3], keep))
    assert status == abi.OK and (now_a, now_b) == (handles[1], handles[0])
    assert bytes(again.stats()) == before
    for identity, address, shape, lower, generation, expected_handle, expected in (
            (1, pb, [3, 2], [-7, 9], 27, now_a, [211.0 + i for i in range(6)]),
            (2, pa, [2, 2], [-2, 3], 11, now_b, [101.0 + i for i in range(4)])):
        status, h = again.register(address, shape, identity=identity, lower=lower, generation=generation)
        assert status == abi.OK and h == expected_handle
        layout = abi.Layout()
        assert both.fort_scope_layout_get(again.handle, h, c.byref(layout)) == abi.OK
        assert layout.generation == generation
        status, dev = _device_begin(again, h, abi.access(flags=abi.READ_ALL))
        assert status == abi.OK and _dev(dev, len(expected)).tolist() == expected
        assert both.fort_scope_device_end(again.handle, h) == abi.OK
    assert (again.stats().upload_bytes, again.stats().download_bytes) == (80, 0)
    assert both.fort_scope_close(again.handle) == abi.OK
    assert (a.tolist(), b.tolist()) == ([1.0, 2.0, 3.0, 4.0], [11.0 + i for i in range(6)])
    assert both.fort_scope_domain_close_v1(domain) == abi.OK
    assert (a.tolist(), b.tolist()) == ([101.0 + i for i in range(4)], [211.0 + i for i in range(6)])


def test_an_exchange_never_defines_from_the_new_name(both):
    """A name that moves to undefined storage stays undefined even when re-registered as initialized (reference:
    test_scoped_domains.py:374-394)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    a, pa = _array([-9.0, -8.0])
    b, pb = _array([3.0, 5.0])
    _, old_a = scope.register(pa, [2], initialized=False, generation=2, lower=[0])
    _, old_b = scope.register(pb, [2], identity=2, generation=7, lower=[0])
    keep = []
    status, new_a, new_b = _swap(both, scope, old_a, old_b, _descriptor(pb, [2], 7, [0], keep), _descriptor(pa, [2], 2, [0], keep))
    assert status == abi.OK
    assert scope.register(pa, [2], identity=2, generation=2, initialized=True, lower=[0])[1] == new_b
    assert _device_begin(scope, new_b, abi.access(flags=abi.READ_ALL))[0] == abi.UNINITIALIZED
    status, dev = _device_begin(scope, new_a, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and _dev(dev, 2).tolist() == [3.0, 5.0]
    assert both.fort_scope_device_end(scope.handle, new_a) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK
    assert a.tolist() == [-9.0, -8.0]


@pytest.mark.parametrize("invalid", ["host", "generation", "extent", "lower", "same_handle", "prepared"])
def test_an_inconsistent_exchange_is_fatal(both, invalid):
    """The exchange reports a mutation that already happened, so an inconsistent report cannot be refused and
    retried: it poisons context and domain without publishing (reference: test_scoped_domains.py:397-430)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    a, pa = _array([1.0, 2.0])
    b, pb = _array([3.0, 4.0])
    _, old_a = scope.register(pa, [2], generation=2, lower=[0])
    _, old_b = scope.register(pb, [2], identity=2, generation=7, lower=[0])
    status, dev = _device_begin(scope, old_a, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 2)[0] = 1000.0
    assert both.fort_scope_device_end(scope.handle, old_a) == abi.OK
    keep = []
    after_a, after_b = _descriptor(pb, [2], 7, [0], keep), _descriptor(pa, [2], 2, [0], keep)
    if invalid == "host":
        after_a.host = pa
    elif invalid == "generation":
        after_a.generation = 2
    elif invalid == "extent":
        after_a = _descriptor(pb, [1], 7, [0], keep)
    elif invalid == "lower":
        after_a = _descriptor(pb, [2], 7, [-1], keep)
    elif invalid == "same_handle":
        old_b = old_a
    elif invalid == "prepared":
        assert _device_begin(scope, old_b, abi.access(flags=abi.READ_ALL))[0] == abi.OK
    status, now_a, now_b = _swap(both, scope, old_a, old_b, after_a, after_b)
    assert status == abi.EXECUTION and (now_a, now_b) == (111, 222)
    assert both.fort_scope_wait(scope.handle) == abi.EXECUTION
    assert both.fort_scope_close(scope.handle) == abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert both.fort_scope_domain_abandon_v1(domain) == abi.OK
    assert (a.tolist(), b.tolist()) == ([1.0, 2.0], [3.0, 4.0])


@pytest.mark.parametrize("invalid", ["key", "version", "reserved", "function", "grid", "block", "arguments"])
def test_invalid_kernel_groups_fail_before_any_launch(both, invalid):
    """A zero group key, an unknown record version, a nonzero reserved field, no function, an empty launch
    dimension or arguments without storage are refused, with nothing built or launched (reference:
    test_scoped_graph_replay.py:64-79)."""
    scope = abi.Scope(both)
    kernel = abi.Kernel(1, 0, 1, (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0, None, 0)
    key = 0 if invalid == "key" else 1
    if invalid == "version":
        kernel.version = 0
    elif invalid == "reserved":
        kernel.reserved = 1
    elif invalid == "function":
        kernel.function = None
    elif invalid in ("grid", "block"):
        getattr(kernel, invalid)[0] = 0
    elif invalid == "arguments":
        kernel.argument_count = 1
    assert both.fort_scope_graph_submit_v1(scope.handle, key, c.byref(kernel), 1) == abi.ARGUMENT
    graphs = abi.GraphStats()
    assert both.fort_scope_graph_stats_get_v1(scope.handle, c.byref(graphs)) == abi.OK
    assert graphs.creations == scope.stats().launches == 0
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_reservation_changes_only_storage_and_a_bad_group_commits_nothing(both):
    """Reserving twice allocates once and moves nothing; a group whose second task names a stale array is refused
    as a whole, so the first task defines nothing (reference: test_scoped_graph_replay.py:197-218)."""
    scope = abi.Scope(both)
    _, address = _array(np.zeros(8))
    _, h = scope.register(address, [8], initialized=False)
    first, second = c.c_void_p(), c.c_void_p()
    assert both.fort_scope_device_reserve_v1(scope.handle, h, c.byref(first)) == abi.OK
    assert both.fort_scope_device_reserve_v1(scope.handle, h, c.byref(second)) == abi.OK
    assert first.value == second.value
    stats = scope.stats()
    assert (stats.allocations, stats.uploads, stats.downloads) == (1, 0, 0)
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    produce = abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL)
    stale = abi.access(flags=abi.READ_ALL)
    kernel = abi.Kernel(1, 0, 1, (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0, None, 0)
    one, two = (abi.Binding * 1)(abi.Binding(h, produce)), (abi.Binding * 1)(abi.Binding(2**63, stale))
    tasks = (abi.Task * 2)(abi.Task(kernel, one, 1), abi.Task(kernel, two, 1))
    before = bytes(scope.stats())
    assert both.fort_scope_graph_execute_v1(scope.handle, 9, tasks, 2) == abi.STALE
    assert bytes(scope.stats()) == before
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK


def _batch(lib, scope, items, *, device=False, outputs=None):
    bindings = (abi.Binding * max(1, len(items)))(*[abi.Binding(h, acc) for h, acc in items])
    return lib.fort_scope_access_begin_v1(scope.handle, bindings if items else None, len(items), int(device),
                                          outputs)


def _counted(scope, identity, *, initialized=True, count=8):
    host, address = _array(identity * 10.0 + np.arange(count))
    status, h = scope.register(address, [count], identity=identity, initialized=initialized)
    assert status == abi.OK
    return host, h


@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("failure", ["stale", "effects", "undefined", "duplicate"])
def test_a_bad_late_binding_changes_nothing(both, device, failure):
    """A batch whose last binding is stale, out of bounds, reads undefined values or repeats an array is refused
    before anything is published, prepared or written out (reference: test_scoped_access_batch.py:130-166)."""
    scope = abi.Scope(both)
    values, first = _counted(scope, 1)
    _, second = _counted(scope, 2, initialized=False)
    status, dev = _device_begin(scope, first, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[0] = 987.0
    assert both.fort_scope_device_end(scope.handle, first) == abi.OK
    read = abi.access(flags=abi.READ_ALL)
    final, expected = {"stale": ((2**63, abi.access(flags=abi.READ_ALL)), abi.STALE),
                       "effects": ((second, abi.access(write=[((0,), (9,))])), abi.ARGUMENT),
                       "undefined": ((second, abi.access(flags=abi.READ_ALL)), abi.UNINITIALIZED),
                       "duplicate": ((first, abi.access(flags=abi.READ_ALL)), abi.ALIAS)}[failure]
    outputs = (c.c_void_p * 2)(123, 456)
    before = bytes(scope.stats())
    assert _batch(both, scope, [(first, read), final], device=device, outputs=outputs) == expected
    assert bytes(scope.stats()) == before and list(outputs) == [123, 456]
    assert values[0] == 10.0
    assert both.fort_scope_host_begin(scope.handle, first, c.byref(read)) == abi.OK
    assert values[0] == 987.0
    assert both.fort_scope_host_end(scope.handle, first) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, second, c.byref(read)) == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_failed_allocation_leaves_the_batch_unprepared(both, monkeypatch):
    """When the second allocation of a device batch fails, nothing is prepared, uploaded or defined; the first
    storage stays allocated (reference: test_scoped_access_batch.py:169-184)."""
    scope = abi.Scope(both)
    _, first = _counted(scope, 1, initialized=False)
    _, second = _counted(scope, 2, initialized=False)
    write = abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL)
    outputs = (c.c_void_p * 2)(123, 456)
    monkeypatch.setenv("F2C_TEST_FAIL_ALLOC_AFTER", "1")
    monkeypatch.setenv("FORT_SCOPE_TEST_FAIL_ALLOC_AFTER", "1")
    assert _batch(both, scope, [(first, write), (second, write)], device=True, outputs=outputs) == abi.RESOURCE
    monkeypatch.delenv("F2C_TEST_FAIL_ALLOC_AFTER")
    monkeypatch.delenv("FORT_SCOPE_TEST_FAIL_ALLOC_AFTER")
    assert list(outputs) == [123, 456]
    assert (scope.stats().uploads, scope.stats().allocations) == (0, 1)
    for h in (first, second):
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == \
            abi.UNINITIALIZED
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(write)) == abi.OK
        assert both.fort_scope_cancel_access(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_batch_over_the_budget_allocates_nothing(both):
    """(reference: test_scoped_access_batch.py:187-197)"""
    scope = abi.Scope(both)
    _, first = _counted(scope, 1)
    _, second = _counted(scope, 2)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    outputs = (c.c_void_p * 2)(123, 456)
    read = abi.access(flags=abi.READ_ALL)
    assert _batch(both, scope, [(first, read), (second, read)], device=True, outputs=outputs) == abi.RESOURCE
    assert list(outputs) == [123, 456]
    assert (scope.stats().allocations, scope.stats().upload_bytes) == (0, 0)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_cancelled_batch_keeps_definitions_and_device_values(both):
    """A host batch that may write part of an array brings that part home first; cancelling it defines nothing
    new and leaves the device's latest values valid (reference: test_scoped_access_batch.py:200-225)."""
    scope = abi.Scope(both)
    values, first = _counted(scope, 1, initialized=False)
    _, second = _counted(scope, 2, initialized=False)
    middle = [((2,), (6,))]
    status, dev = _device_begin(scope, first, abi.access(write=middle, overwrite=middle))
    assert status == abi.OK
    _dev(dev, 8)[2:6] = 1000.0 + np.arange(2, 6)
    assert both.fort_scope_device_end(scope.handle, first) == abi.OK
    assert _batch(both, scope, [(first, abi.access(write=middle)),
                                (second, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))]) == abi.OK
    assert values.tolist()[2:6] == [1002.0, 1003.0, 1004.0, 1005.0]
    for h in (first, second):
        assert both.fort_scope_cancel_access(scope.handle, h) == abi.OK
    for h in (first, second):
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == \
            abi.UNINITIALIZED
    status, dev = _device_begin(scope, first, abi.access(read=middle))
    assert status == abi.OK and _dev(dev, 8)[2:6].tolist() == [1002.0, 1003.0, 1004.0, 1005.0]
    assert both.fort_scope_device_end(scope.handle, first) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_an_empty_batch_waits_for_nothing_and_an_overwrite_fences_an_upload(both, monkeypatch):
    """An empty batch neither waits nor fails; a host overwrite of an array whose upload may still be reading it
    waits once, and the device then sees the new value (reference: test_scoped_access_batch.py:228-245)."""
    scope = abi.Scope(both)
    values, h = _counted(scope, 1)
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    waits = scope.stats().waits
    _inject(monkeypatch, "WAIT")
    assert _batch(both, scope, []) == abi.OK and scope.stats().waits == waits
    monkeypatch.delenv("F2C_TEST_FAIL_WAIT")
    monkeypatch.delenv("FORT_SCOPE_TEST_FAIL_WAIT")
    assert _batch(both, scope, [(h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))]) == abi.OK
    assert scope.stats().waits == waits + 1
    values[0] = 555.0
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and _dev(dev, 8)[0] == 555.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_failed_wait_in_a_batch_poisons_without_replay(both, monkeypatch):
    """(reference: test_scoped_access_batch.py:248-261)"""
    scope = abi.Scope(both)
    handles = [_counted(scope, identity)[1] for identity in (1, 2)]
    for h in handles:
        status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
        assert status == abi.OK
        _dev(dev, 8)[0] += 100.0
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    _inject(monkeypatch, "WAIT")
    items = [(h, abi.access(flags=abi.READ_ALL)) for h in handles]
    assert _batch(both, scope, items) == abi.EXECUTION
    assert _batch(both, scope, items) == abi.EXECUTION
    assert both.fort_scope_close(scope.handle) == abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK


def test_a_refused_batch_leaves_an_existing_access_alone(both):
    """A batch naming an array another access already holds is refused; that access stays valid and the batch's
    other array was never prepared (reference: test_scoped_access_batch.py:275-287)."""
    scope = abi.Scope(both)
    _, first = _counted(scope, 1)
    _, second = _counted(scope, 2)
    read = abi.access(flags=abi.READ_ALL)
    assert both.fort_scope_host_begin(scope.handle, first, c.byref(read)) == abi.OK
    assert _batch(both, scope, [(second, read), (first, read)]) == abi.STATE
    assert both.fort_scope_host_end(scope.handle, first) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, second, c.byref(read)) == abi.OK
    assert both.fort_scope_host_end(scope.handle, second) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_retired_generation_is_refused_before_any_transfer(both):
    """(reference: test_scoped_access_batch.py:290-307)"""
    scope = abi.Scope(both)
    _, first = _counted(scope, 1)
    old_values, old = _counted(scope, 2)
    assert both.fort_scope_unregister(scope.handle, old) == abi.OK
    status, current = scope.register(old_values.ctypes.data, [8], identity=2, generation=2)
    assert status == abi.OK
    read = abi.access(flags=abi.READ_ALL)
    outputs = (c.c_void_p * 2)()
    before = bytes(scope.stats())
    assert _batch(both, scope, [(first, read), (old, read)], device=True, outputs=outputs) == abi.STALE
    assert bytes(scope.stats()) == before
    assert _batch(both, scope, [(first, read), (current, read)], device=True, outputs=outputs) == abi.OK
    for h in (first, current):
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_empty_arrays_and_empty_batches_allocate_and_wait_for_nothing(both, monkeypatch):
    """(reference: test_scoped_access_batch.py:310-324)"""
    scope = abi.Scope(both)
    status, h = scope.register(None, [0], identity=5, initialized=False)
    assert status == abi.OK
    _inject(monkeypatch, "ALLOC")
    assert both.fort_scope_access_begin_v1(scope.handle, None, 0, 1, None) == abi.OK
    outputs = (c.c_void_p * 1)(123)
    assert _batch(both, scope, [(h, abi.access(flags=7))], device=True, outputs=outputs) == abi.OK
    assert outputs[0] is None
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert _batch(both, scope, [(h, abi.access(flags=abi.READ_ALL))]) == abi.OK
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert bytes(scope.stats()) == bytes(abi.Stats())
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_budget_eviction_publishes_dirty_values(both):
    scope = abi.Scope(both)
    a, pa = _array(np.zeros(128))
    b, pb = _array(np.zeros(128))
    assert both.fort_scope_set_device_budget(scope.handle, 128 * 8 + 512) == abi.OK
    _, ha = scope.register(pa, [128])
    _, hb = scope.register(pb, [128])
    status, dev = _device_begin(scope, ha, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 128)[:] = 7.0
    assert both.fort_scope_device_end(scope.handle, ha) == abi.OK
    status, dev = _device_begin(scope, hb, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 128)[:] += 1.0
    assert both.fort_scope_device_end(scope.handle, hb) == abi.OK
    assert a.tolist() == [7.0] * 128  # published when it was evicted
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert b.tolist() == [1.0] * 128


def test_oversized_footprint_fails_before_any_change(both):
    scope = abi.Scope(both)
    a, pa = _array(np.zeros(64))
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    _, ha = scope.register(pa, [64])
    status, _ = _device_begin(scope, ha, abi.access(flags=abi.READ_ALL))
    assert status == abi.RESOURCE
    assert scope.stats().allocations == 0
    assert both.fort_scope_close(scope.handle) == abi.OK


def _resident(scope, identity, *, initialized=True, defined=None):
    """Eight values identity*100 + i, kept alive with the scope."""
    host, address = _array(identity * 100.0 + np.arange(8))
    scope.keep.append(host)
    status, h = scope.register(address, [8], identity=identity, initialized=initialized, defined=defined)
    assert status == abi.OK
    return host, h


def _reserve_many(lib, scope, *handles, outputs=None):
    outputs = outputs if outputs is not None else (c.c_void_p * len(handles))()
    return lib.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * len(handles))(*handles), len(handles),
                                                 outputs), outputs


def _residency(lib, scope):
    out = abi.ResidencyStats()
    assert lib.fort_scope_residency_stats_get_v1(scope.handle, c.byref(out)) == abi.OK
    assert out.version == 1
    return out


def _on_device(lib, scope, h, acc, change=None):
    status, dev = _device_begin(scope, h, acc)
    assert status == abi.OK
    if change is not None:
        change(_dev(dev, 8))
    assert lib.fort_scope_device_end(scope.handle, h) == abi.OK


def _shift(amount):
    def change(d):
        d[:] += amount
    return change


def test_lru_dirty_eviction_publishes_once_and_reloads_exactly(both):
    """Two mirrors fill a 128-byte budget; reserving a third next to the clean one evicts the dirty one, which is
    published first and reloads exactly (reference: test_scoped_residency.py:49-72)."""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 128) == abi.OK
    host_a, a = _resident(scope, 1)
    _, b = _resident(scope, 2)
    _, other = _resident(scope, 3)
    _on_device(both, scope, a, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL), _shift(1000.0))
    _on_device(both, scope, b, abi.access(flags=abi.READ_ALL))
    before = scope.stats()
    assert _reserve_many(both, scope, other, b)[0] == abi.OK   # b pinned: only the dirty a can go
    assert host_a.tolist() == [1100.0 + i for i in range(8)]
    assert scope.stats().download_bytes - before.download_bytes == 64
    r = _residency(both, scope)
    assert (r.evictions, r.evicted_bytes, r.dirty_evictions, r.dirty_download_bytes) == (1, 64, 1, 64)
    status, dev = _device_begin(scope, a, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and _dev(dev, 8).tolist() == host_a.tolist()
    assert both.fort_scope_device_end(scope.handle, a) == abi.OK
    assert scope.stats().allocated_bytes == scope.stats().peak_device_bytes == 128
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_clean_replica_goes_before_older_dirty_storage(both):
    """Eviction takes the clean mirror before the older dirty one; when every alternative is pinned the dirty one
    is published exactly once (reference: test_scoped_residency.py:75-104)."""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 128) == abi.OK
    host_a, a = _resident(scope, 1)
    _, b = _resident(scope, 2)
    _, other = _resident(scope, 3)
    _on_device(both, scope, a, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL), _shift(1000.0))
    _on_device(both, scope, b, abi.access(flags=abi.READ_ALL))
    assert _reserve_many(both, scope, other)[0] == abi.OK
    assert host_a.tolist() == [100.0 + i for i in range(8)]    # a stayed on the device, unpublished
    assert scope.stats().download_bytes == 0
    r = _residency(both, scope)
    assert (r.evictions, r.dirty_evictions) == (1, 0)
    allocations, uploads = scope.stats().allocations, scope.stats().upload_bytes
    status, dev = _device_begin(scope, a, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and _dev(dev, 8).tolist() == [1100.0 + i for i in range(8)]
    assert both.fort_scope_device_end(scope.handle, a) == abi.OK
    assert (scope.stats().allocations, scope.stats().upload_bytes) == (allocations, uploads)
    assert _reserve_many(both, scope, b, other)[0] == abi.OK
    assert host_a.tolist() == [1100.0 + i for i in range(8)]
    assert scope.stats().download_bytes == 64
    r = _residency(both, scope)
    assert (r.evictions, r.dirty_evictions) == (2, 1)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_evicting_a_read_mirror_downloads_nothing(both):
    """(reference: test_scoped_residency.py:107-122)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    host, a = _resident(scope, 1)
    _, b = _resident(scope, 2)
    _on_device(both, scope, a, abi.access(flags=abi.READ_ALL))
    assert _reserve_many(both, scope, b)[0] == abi.OK
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == [100.0 + i for i in range(8)]
    assert both.fort_scope_host_end(scope.handle, a) == abi.OK
    assert scope.stats().download_bytes == 0
    r = _residency(both, scope)
    assert (r.evictions, r.dirty_evictions) == (1, 0)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_an_impossible_reservation_changes_nothing(both):
    """Two 64-byte arrays cannot both be reserved in 64 bytes: RESOURCE before the dirty one is published, the
    output slots untouched, every counter unchanged (reference: test_scoped_residency.py:125-146)."""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    host, a = _resident(scope, 1)
    _, b = _resident(scope, 2)

    def fill(d):
        d[:] = 999.0 + np.arange(8)
    _on_device(both, scope, a, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL), fill)
    before, metrics = bytes(scope.stats()), bytes(_residency(both, scope))
    outputs = (c.c_void_p * 2)(0x1234, 0x5678)
    assert _reserve_many(both, scope, a, b, outputs=outputs)[0] == abi.RESOURCE
    assert list(outputs) == [0x1234, 0x5678]
    assert bytes(scope.stats()) == before and bytes(_residency(both, scope)) == metrics
    assert host[0] == 100.0
    status, dev = _device_begin(scope, a, abi.access(flags=abi.READ_ALL))
    assert status == abi.OK and _dev(dev, 8)[0] == 999.0
    assert both.fort_scope_device_end(scope.handle, a) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host[0] == 999.0


def test_a_reservation_pins_duplicates_and_reuse_refreshes_the_lru(both):
    """(reference: test_scoped_residency.py:149-165)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 128) == abi.OK
    a, b, other = (_resident(scope, n)[1] for n in (1, 2, 3))
    assert _reserve_many(both, scope, a, b)[0] == abi.OK
    status, duplicate = _reserve_many(both, scope, a, a)
    assert status == abi.OK and duplicate[0] == duplicate[1]
    assert _reserve_many(both, scope, a, other)[0] == abi.OK
    allocations = scope.stats().allocations
    assert _reserve_many(both, scope, a)[0] == abi.OK
    assert scope.stats().allocations == allocations          # the recently used a survived
    assert _reserve_many(both, scope, b)[0] == abi.OK
    assert scope.stats().allocations == allocations + 1      # the cold b was evicted
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_eviction_publishes_exactly_the_defined_part_and_keeps_holes(both):
    """(reference: test_scoped_residency.py:168-185)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    host, a = _resident(scope, 1, defined=[((2,), (6,))])
    _, b = _resident(scope, 2)
    span = [((2,), (6,))]

    def fill(d):
        d[2:6] = 1000.0 + np.arange(2, 6)
    _on_device(both, scope, a, abi.access(read=span, write=span, overwrite=[((3,), (4,))]), fill)
    assert _reserve_many(both, scope, b)[0] == abi.OK
    assert host.tolist() == [100, 101, 1002, 1003, 1004, 1005, 106, 107]
    assert scope.stats().upload_bytes == scope.stats().download_bytes == 32
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(abi.access(flags=abi.READ_ALL))) \
        == abi.UNINITIALIZED
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(abi.access(read=span))) == abi.OK
    assert both.fort_scope_host_end(scope.handle, a) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_prepared_array_is_neither_evicted_nor_reserved(both):
    """(reference: test_scoped_residency.py:188-204)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    host, a = _resident(scope, 1)
    _, b = _resident(scope, 2)
    status, dev = _device_begin(scope, a, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    assert _reserve_many(both, scope, a)[0] == abi.STATE
    assert _reserve_many(both, scope, b)[0] == abi.RESOURCE
    assert _residency(both, scope).evictions == 0
    _dev(dev, 8)[0] = 987.0
    assert both.fort_scope_device_end(scope.handle, a) == abi.OK
    assert _reserve_many(both, scope, b)[0] == abi.OK
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host[0] == 987.0
    assert both.fort_scope_host_end(scope.handle, a) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_buffer_membership_is_per_context(both):
    """A handle belongs to the context that registered it, even for the same identity in another context; a closed
    context answers STALE (reference: test_scoped_residency.py:207-224)."""
    first, second = abi.Scope(both), abi.Scope(both)
    _, old = _resident(first, 1)
    _, current = _resident(second, 1)
    present = c.c_int(-1)
    assert both.fort_scope_buffer_valid_v1(first.handle, old, c.byref(present)) == abi.OK and present.value == 1
    assert both.fort_scope_buffer_valid_v1(second.handle, old, c.byref(present)) == abi.OK and present.value == 0
    assert both.fort_scope_close(first.handle) == abi.OK
    assert both.fort_scope_buffer_valid_v1(second.handle, old, c.byref(present)) == abi.OK and present.value == 0
    assert both.fort_scope_buffer_valid_v1(second.handle, current, c.byref(present)) == abi.OK
    assert present.value == 1
    assert second.stats().allocations == 0
    assert both.fort_scope_buffer_valid_v1(first.handle, old, c.byref(present)) == abi.STALE
    assert both.fort_scope_close(second.handle) == abi.OK


def test_eviction_keeps_device_values_whose_definition_was_forgotten(both):
    """Forgetting the definition of device-written values does not lose them: eviction still publishes them, and
    reads admitted afterwards see them without another download (reference: test_scoped_residency.py:227-249)."""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    host, a = _resident(scope, 1)
    _, b = _resident(scope, 2)

    def fill(d):
        d[:] = 5000.0 + np.arange(8)
    _on_device(both, scope, a, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL), fill)
    assert both.fort_scope_forget_definition(scope.handle, a) == abi.OK
    assert scope.stats().download_bytes == 0
    assert _reserve_many(both, scope, b)[0] == abi.OK
    assert host.tolist() == [5000.0 + i for i in range(8)]
    assert scope.stats().download_bytes == 64
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(abi.access(flags=abi.READ_ALL))) \
        == abi.UNINITIALIZED
    reads = abi.access(read=[((0,), (8,))])
    assert both.fort_scope_admit_source_reads_v1(scope.handle, a, reads.reads, reads.read_count) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == [5000.0 + i for i in range(8)]
    assert both.fort_scope_host_end(scope.handle, a) == abi.OK
    assert scope.stats().download_bytes == 64
    assert both.fort_scope_close(scope.handle) == abi.OK


HOST_ONLY = r"""
import ctypes as c, sys
import numpy as np
sys.path[:0] = sys.argv[3:]
from compiler.runtime import abi
lib = abi.bind(c.CDLL(sys.argv[1]))
scope = abi.Scope(lib)
arrays = [np.arange(1 << 18, dtype=np.float64) for _ in range(2)]     # 2 MiB each
handles = [scope.register(a.ctypes.data, [a.size], identity=n + 1)[1] for n, a in enumerate(arrays)]
assert all(handles)
acc = abi.access(flags=abi.READ_ALL | abi.WRITE_ALL)
assert lib.fort_scope_host_begin(scope.handle, handles[0], c.byref(acc)) == abi.OK
arrays[0][:] += 1.0
assert lib.fort_scope_host_end(scope.handle, handles[0]) == abi.OK
assert lib.fort_scope_observe_v1(scope.handle, (abi.U64 * 2)(*handles), 2) == abi.OK
assert lib.fort_scope_unregister(scope.handle, handles[1]) == abi.OK
if sys.argv[2] == "zero":  # a device access that cannot fit a zero budget is refused first
    assert lib.fort_scope_set_device_budget(scope.handle, 0) == abi.OK
    out = c.c_void_p()
    assert lib.fort_scope_device_begin(scope.handle, handles[0], c.byref(abi.access(flags=abi.READ_ALL)),
                                       c.byref(out)) == abi.RESOURCE
if sys.argv[2] == "device":
    out = c.c_void_p()
    assert lib.fort_scope_device_begin(scope.handle, handles[0], c.byref(abi.access(flags=abi.READ_ALL)),
                                       c.byref(out)) == abi.OK
    assert lib.fort_scope_device_end(scope.handle, handles[0]) == abi.OK
assert lib.fort_scope_close(scope.handle) == abi.OK
assert arrays[0][5] == 6.0
"""


@pytest.mark.parametrize("use", ["host", "zero", "device"])
def test_host_only_use_never_initializes_the_device(both, use, tmp_path):
    """Registration, host access, observation of host-current arrays, unregistration and close bring no device
    up, nor does a device access refused by a zero budget; the first device access does, once (reference:
    test_scoped_host_completion_cuda.py:205-210, test_scoped_runtime_cuda.py:404-410,
    test_scoped_runtime.py:659-668, traced as ``FORT_SCOPED initialize``)."""
    script = tmp_path / "host_only.py"
    script.write_text(HOST_ONLY)
    package = os.path.join(ROOT, "fortran-to-cuda_gb300")
    run = subprocess.run([sys.executable, str(script), both._name, use, package], capture_output=True, text=True,
                         timeout=120, env={**os.environ, "FORT_RUNTIME_TRACE": "1"})
    assert run.returncode == 0, run.stdout + run.stderr
    initialized = [line for line in run.stderr.splitlines() if line.startswith("FORT_SCOPED initialize")]
    assert len(initialized) == (use == "device")


@pytest.mark.parametrize("shared", [False, True])
def test_the_budget_warning_is_said_once_per_shared_domain(both, shared, capfd):
    """An eviction in a context of a shared domain (the resident application's) says once what exceeding the
    budget costs, in the reference's words; a private context says nothing (reference:
    compiler/runtime/scoped_runtime.cu:535-543, test_resident_application_cuda.py:118-135)."""
    domain = _domain(both) if shared else None
    scope = abi.Scope(both, domain=domain)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    handles = [_resident(scope, n)[1] for n in (1, 2, 3)]
    for h in handles * 2:
        assert _reserve_many(both, scope, h)[0] == abi.OK
    assert _residency(both, scope).evictions == 5
    assert both.fort_scope_close(scope.handle) == abi.OK
    if shared:
        assert both.fort_scope_domain_close_v1(domain) == abi.OK
    said = capfd.readouterr().err.count("Resident domain: the arrays in use exceed the device budget of 64 bytes; "
                                        "the least recently used ones now move back to the host.")
    assert said == (1 if shared else 0)


def test_scratch_leases(both):
    scope = abi.Scope(both)
    lease = abi.ScratchLease()
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 0, c.byref(lease)) == abi.OK
    assert lease.device is None and lease.token
    other = abi.ScratchLease()
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 16, c.byref(other)) == abi.STATE
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token + 1) != abi.OK
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 4096, c.byref(lease)) == abi.OK
    first = lease.device
    assert first and lease.capacity >= 4096
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 1024, c.byref(lease)) == abi.OK
    assert lease.device == first  # reused, not regrown
    assert both.fort_scope_close(scope.handle) == abi.STATE  # an active lease blocks close
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    stats = abi.ScratchStats()
    assert both.fort_scope_scratch_stats_get_v1(scope.handle, c.byref(stats)) == abi.OK
    assert (stats.acquisitions, stats.releases, stats.active) == (3, 3, 0)
    assert both.fort_scope_close(scope.handle) == abi.OK


def _lease(lib, scope, size):
    lease = abi.ScratchLease()
    assert lib.fort_scope_scratch_acquire_v1(scope.handle, size, c.byref(lease)) == abi.OK
    assert (lease.version, lease.reserved, lease.bytes) == (1, 0, size) and lease.token and lease.capacity >= size
    return lease


def _scratch(lib, scope):
    out = abi.ScratchStats()
    assert lib.fort_scope_scratch_stats_get_v1(scope.handle, c.byref(out)) == abi.OK and out.version == 1
    return out


def test_an_empty_lease_allocates_nothing(both, monkeypatch):
    """A zero-byte lease has no storage, allocates nothing and leaves the budget open to change (reference:
    test_scoped_scratch.py:89-105)."""
    scope = abi.Scope(both)
    _inject(monkeypatch, "ALLOC")
    lease = _lease(both, scope, 0)
    assert lease.device is None and lease.capacity == 0
    assert both.fort_scope_set_device_budget(scope.handle, 0) == abi.OK
    stats = _scratch(both, scope)
    assert (stats.active, stats.acquisitions, stats.allocations, stats.capacity_bytes) == (1, 1, 0, 0)
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


@pytest.mark.parametrize("budget, size", [(0, 1), (64, (1 << (8 * c.sizeof(abi.SIZE))) - 1)])
def test_an_impossible_lease_fails_before_the_device_is_used(both, budget, size):
    """(reference: test_scoped_scratch.py:108-121)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, budget) == abi.OK
    out = abi.ScratchLease()
    assert both.fort_scope_scratch_acquire_v1(scope.handle, size, c.byref(out)) == abi.RESOURCE
    assert bytes(out) == bytes(abi.ScratchLease())
    assert both.fort_scope_set_device_budget(scope.handle, 0) == abi.OK     # still before any device use
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_one_lease_at_a_time_and_tokens_never_return(both):
    """One active lease per context; a second acquisition is refused and its output cleared; tokens are the
    context's own and never reused; a closed context's tokens are stale (reference: test_scoped_scratch.py:124-146)."""
    first, second = abi.Scope(both), abi.Scope(both)
    assert both.fort_scope_scratch_acquire_v1(first.handle, 0, None) == abi.ARGUMENT
    assert both.fort_scope_scratch_stats_get_v1(first.handle, None) == abi.ARGUMENT
    lease, other = _lease(both, first, 0), _lease(both, second, 0)
    rejected = abi.ScratchLease(9, 9, 99, 17, 23, 23)
    assert both.fort_scope_scratch_acquire_v1(first.handle, 0, c.byref(rejected)) == abi.STATE
    assert bytes(rejected) == bytes(abi.ScratchLease())
    assert both.fort_scope_scratch_release_v1(second.handle, lease.token) == abi.STALE
    assert both.fort_scope_scratch_release_v1(first.handle, 0) == abi.STALE
    assert both.fort_scope_scratch_release_v1(first.handle, lease.token) == abi.OK
    assert both.fort_scope_scratch_release_v1(first.handle, lease.token) == abi.STALE
    renewed = _lease(both, first, 0)
    assert len({lease.token, other.token, renewed.token}) == 3
    assert both.fort_scope_scratch_release_v1(first.handle, lease.token) == abi.STALE
    assert both.fort_scope_scratch_release_v1(first.handle, renewed.token) == abi.OK
    assert both.fort_scope_scratch_release_v1(second.handle, other.token) == abi.OK
    assert both.fort_scope_close(first.handle) == abi.OK and both.fort_scope_close(second.handle) == abi.OK
    assert both.fort_scope_scratch_release_v1(first.handle, renewed.token) == abi.STALE
    assert both.fort_scope_scratch_stats_get_v1(first.handle, c.byref(abi.ScratchStats())) == abi.STALE


def test_a_reused_arena_keeps_its_capacity_without_waiting(both):
    """A smaller lease reuses the arena and its contents; nothing waits, publishes or counts as a mirror
    (reference: test_scoped_scratch.py:149-176)."""
    scope = abi.Scope(both)
    lease = _lease(both, scope, 64)
    (c.c_uint64 * 8).from_address(lease.device)[:] = list(range(8))
    assert both.fort_scope_note_launch(scope.handle) == abi.OK
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    waits = scope.stats().waits
    smaller = _lease(both, scope, 24)
    assert (smaller.device, smaller.capacity) == (lease.device, 64)
    assert list((c.c_uint64 * 8).from_address(smaller.device)) == list(range(8))
    assert both.fort_scope_scratch_release_v1(scope.handle, smaller.token) == abi.OK
    empty = _lease(both, scope, 0)
    assert empty.device is None and empty.capacity == 64
    assert both.fort_scope_scratch_release_v1(scope.handle, empty.token) == abi.OK
    assert scope.stats().waits == waits == 0
    stats = _scratch(both, scope)
    assert (stats.acquisitions, stats.allocations, stats.reuses, stats.releases, stats.grows) == (3, 1, 1, 3, 0)
    assert stats.capacity_bytes == stats.peak_scratch_bytes == stats.peak_total_device_bytes == 64
    assert not stats.active and stats.active_bytes == 0
    mirrors = scope.stats()
    assert (mirrors.allocations, mirrors.allocated_bytes, mirrors.peak_device_bytes) == (0, 0, 0)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_growing_arena_waits_for_its_old_work(both):
    """(reference: test_scoped_scratch.py:179-192)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 96) == abi.OK
    initial = _lease(both, scope, 64)
    assert both.fort_scope_note_launch(scope.handle) == abi.OK
    assert both.fort_scope_scratch_release_v1(scope.handle, initial.token) == abi.OK
    grown = _lease(both, scope, 96)
    assert grown.capacity == 96
    stats = _scratch(both, scope)
    assert (stats.allocations, stats.grows, stats.capacity_bytes, stats.peak_total_device_bytes) == (2, 1, 96, 96)
    assert scope.stats().waits == 1
    assert both.fort_scope_scratch_release_v1(scope.handle, grown.token) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


@pytest.mark.parametrize("scratch_first", [False, True])
def test_scratch_and_mirrors_share_the_budget_without_evicting_each_other(both, scratch_first):
    """(reference: test_scoped_scratch.py:195-223)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 160) == abi.OK
    values, address = _array(np.arange(16, dtype=np.float64))
    _, h = scope.register(address, [16])
    if scratch_first:
        lease = _lease(both, scope, 64)
        assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
        assert _device_begin(scope, h, abi.access(flags=abi.READ_ALL))[0] == abi.RESOURCE
        assert scope.stats().allocations == 0 and _scratch(both, scope).capacity_bytes == 64
    else:
        assert _device_begin(scope, h, abi.access(flags=abi.READ_ALL))[0] == abi.OK
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
        rejected = abi.ScratchLease()
        assert both.fort_scope_scratch_acquire_v1(scope.handle, 64, c.byref(rejected)) == abi.RESOURCE
        assert bytes(rejected) == bytes(abi.ScratchLease()) and _scratch(both, scope).capacity_bytes == 0
        lease = _lease(both, scope, 32)
        assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
        assert _scratch(both, scope).peak_total_device_bytes == 160
        assert scope.stats().peak_device_bytes == 128
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert values.tolist() == list(range(16))


def test_releasing_a_mirror_makes_room_for_scratch(both):
    """(reference: test_scoped_scratch.py:226-242)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 160) == abi.OK
    _, address = _array(np.arange(16, dtype=np.float64))
    _, h = scope.register(address, [16])
    assert _device_begin(scope, h, abi.access(flags=abi.READ_ALL))[0] == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    first = _lease(both, scope, 32)
    assert both.fort_scope_scratch_release_v1(scope.handle, first.token) == abi.OK
    assert both.fort_scope_unregister(scope.handle, h) == abi.OK
    grown = _lease(both, scope, 160)
    assert both.fort_scope_scratch_release_v1(scope.handle, grown.token) == abi.OK
    assert scope.stats().allocated_bytes == 0 and _scratch(both, scope).peak_total_device_bytes == 160
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_an_active_lease_blocks_close_before_publication(both):
    """(reference: test_scoped_scratch.py:245-261)"""
    scope = abi.Scope(both)
    values, address = _array(np.arange(4, dtype=np.float64))
    _, h = scope.register(address, [4])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 4)[:] = 10.0 + np.arange(4)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    lease = _lease(both, scope, 32)
    assert both.fort_scope_close(scope.handle) == abi.STATE
    assert values.tolist() == list(range(4)) and scope.stats().downloads == 0
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert values.tolist() == [10.0, 11.0, 12.0, 13.0]


@pytest.mark.parametrize("growing", [False, True])
def test_a_failed_scratch_allocation_grants_nothing(both, monkeypatch, growing):
    """(reference: test_scoped_scratch.py:264-280)"""
    scope = abi.Scope(both)
    if growing:
        lease = _lease(both, scope, 32)
        assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    _inject(monkeypatch, "SCRATCH_ALLOC")
    failed = abi.ScratchLease(1, 0, 9, 1, 64, 64)
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 64, c.byref(failed)) == abi.RESOURCE
    assert bytes(failed) == bytes(abi.ScratchLease())
    stats = _scratch(both, scope)
    assert stats.active == stats.capacity_bytes == 0
    monkeypatch.delenv("F2C_TEST_FAIL_SCRATCH_ALLOC")
    monkeypatch.delenv("FORT_SCOPE_TEST_FAIL_SCRATCH_ALLOC")
    recovered = _lease(both, scope, 64)
    assert both.fort_scope_scratch_release_v1(scope.handle, recovered.token) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_refused_growth_keeps_the_idle_arena(both):
    """(reference: test_scoped_scratch.py:283-295)"""
    scope = abi.Scope(both)
    assert both.fort_scope_set_device_budget(scope.handle, 64) == abi.OK
    initial = _lease(both, scope, 64)
    assert both.fort_scope_scratch_release_v1(scope.handle, initial.token) == abi.OK
    out = abi.ScratchLease()
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 65, c.byref(out)) == abi.RESOURCE
    assert bytes(out) == bytes(abi.ScratchLease())
    renewed = _lease(both, scope, 64)
    assert renewed.device == initial.device
    assert both.fort_scope_scratch_release_v1(scope.handle, renewed.token) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_failed_wait_while_growing_poisons(both, monkeypatch):
    """(reference: test_scoped_scratch.py:298-311)"""
    scope = abi.Scope(both)
    lease = _lease(both, scope, 32)
    assert both.fort_scope_note_launch(scope.handle) == abi.OK
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    _inject(monkeypatch, "WAIT")
    out = abi.ScratchLease()
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 64, c.byref(out)) == abi.EXECUTION
    assert bytes(out) == bytes(abi.ScratchLease())
    assert both.fort_scope_close(scope.handle) == abi.EXECUTION
    assert both.fort_scope_scratch_acquire_v1(scope.handle, 0, c.byref(out)) == abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.STALE


def test_close_publishes_fields_and_retires_the_idle_arena(both):
    """(reference: test_scoped_scratch.py:314-329)"""
    scope = abi.Scope(both)
    fields = []
    for identity in (1, 2):
        host, address = _array(np.arange(8, dtype=np.float64))
        fields.append(host)
        _, h = scope.register(address, [8], identity=identity, lower=[-identity])
        status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
        assert status == abi.OK
        _dev(dev, 8)[:] = 100.0 * identity + np.arange(8)
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    lease = _lease(both, scope, 256)
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert [f.tolist() for f in fields] == [[100.0 * n + i for i in range(8)] for n in (1, 2)]
    assert both.fort_scope_wait(scope.handle) == abi.STALE


def test_a_failed_wait_at_close_poisons(both, monkeypatch):
    """(reference: test_scoped_scratch.py:332-347)"""
    scope = abi.Scope(both)
    _, address = _array(np.arange(8, dtype=np.float64))
    _, h = scope.register(address, [8])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))
    assert status == abi.OK
    _dev(dev, 8)[0] = 100.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    lease = _lease(both, scope, 256)
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    _inject(monkeypatch, "WAIT")
    assert both.fort_scope_close(scope.handle) == abi.EXECUTION
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert both.fort_scope_wait(scope.handle) == abi.STALE


@pytest.mark.parametrize("active", [False, True])
def test_abandonment_is_for_failed_contexts_and_publishes_nothing(both, active):
    """A healthy context cannot be abandoned; after an execution error it can, its scratch is retired and nothing
    is published (reference: test_scoped_scratch.py:350-368)."""
    scope = abi.Scope(both)
    values, address = _array(np.arange(4, dtype=np.float64))
    _, h = scope.register(address, [4])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 4)[:] = 10.0 + np.arange(4)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    lease = _lease(both, scope, 32)
    if not active:
        assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.OK
    assert both.fort_scope_abandon(scope.handle) == abi.STATE
    assert both.fort_scope_execution_error(scope.handle, b"injected numerical failure") == abi.EXECUTION
    assert both.fort_scope_scratch_release_v1(scope.handle, lease.token) == abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert values.tolist() == list(range(4))


def _members(lib, scope, key, *members):
    """Enqueue one launch of independent members (each a list of (handle, access)); never submitted here."""
    value = c.c_int(7)
    arguments = (c.c_void_p * 1)(c.addressof(value))
    kernel = abi.Kernel(1, 0, 1, (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0, arguments, 1)
    packs = [(abi.Binding * len(m))(*[abi.Binding(h, acc) for h, acc in m]) for m in members]
    packed = (abi.Member * max(1, len(members)))(*[abi.Member(p, len(m)) for p, m in zip(packs, members)])
    return lib.fort_scope_graph_enqueue_members_v1(scope.handle, key, c.byref(kernel), (abi.SIZE * 1)(4),
                                                    packed if members else None, len(members))


def _reserved(lib, scope, identity, *, initialized=False):
    host, address = _array(np.arange(8, dtype=np.float64))
    scope.keep.append(host)                                   # the array outlives the registration
    status, h = scope.register(address, [8], identity=identity, initialized=initialized)
    assert status == abi.OK
    assert lib.fort_scope_device_reserve_v1(scope.handle, h, c.byref(c.c_void_p())) == abi.OK
    return h


def _queue(lib, scope):
    out = abi.QueueStats()
    assert lib.fort_scope_graph_queue_stats_get_v1(scope.handle, c.byref(out)) == abi.OK
    return out


def test_members_of_one_array_are_judged_on_their_sections(both):
    """Members may write disjoint halves of one array; overlapping writes, or a read of what another member
    writes, refuse the whole launch and leave no trace (reference: test_scoped_graph_queue.py:93-110)."""
    scope = abi.Scope(both)
    a = _reserved(both, scope, 1, initialized=True)
    halves = [abi.access(write=[((0,), (4,))], overwrite=[((0,), (4,))]),
              abi.access(write=[((4,), (8,))], overwrite=[((4,), (8,))])]
    assert _members(both, scope, 21, [(a, halves[0])], [(a, halves[1])]) == abi.OK
    assert _queue(both, scope).pending_tasks == 1
    before = bytes(_queue(both, scope))
    overlap = abi.access(write=[((3,), (5,))], overwrite=[((3,), (5,))])
    assert _members(both, scope, 22, [(a, halves[0])], [(a, overlap)]) == abi.BOUNDARY
    assert _members(both, scope, 23, [(a, halves[0])], [(a, abi.access(read=[((2,), (3,))]))]) == abi.BOUNDARY
    assert bytes(_queue(both, scope)) == before
    assert _members(both, scope, 24, [(a, abi.access(read=[((0,), (8,))]))]) == abi.OK
    assert _queue(both, scope).pending_tasks == 2
    assert both.fort_scope_graph_queue_cancel_v1(scope.handle) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_member_launch_validates_like_a_single_task(both):
    """No members, an array repeated within a member, or a read of undefined values: refused, nothing queued
    (reference: test_scoped_graph_queue.py:113-123)."""
    scope = abi.Scope(both)
    a = _reserved(both, scope, 1)
    b = _reserved(both, scope, 2)
    write = abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL)
    read = abi.access(flags=abi.READ_ALL)
    assert _members(both, scope, 31) == abi.ARGUMENT
    assert _members(both, scope, 32, [(a, write), (a, read)]) == abi.ALIAS
    assert _members(both, scope, 33, [(a, write)], [(b, read)]) == abi.UNINITIALIZED
    queued = _queue(both, scope)
    assert queued.pending_tasks == queued.accepted_tasks == 0
    assert both.fort_scope_close(scope.handle) == abi.OK


def _queued_task(lib, scope, key, items, *, scalar=7):
    """Queue one task (never submitted here) over (handle, access) items."""
    value = c.c_int(scalar)
    arguments = (c.c_void_p * 1)(c.addressof(value))
    kernel = abi.Kernel(1, 0, 1, (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0, arguments, 1)
    bindings = (abi.Binding * len(items))(*[abi.Binding(h, acc) for h, acc in items])
    task = abi.Task(kernel, bindings, len(items))
    return lib.fort_scope_graph_enqueue_v1(scope.handle, key, c.byref(task), (abi.SIZE * 1)(c.sizeof(value)))


def test_a_refused_enqueue_keeps_the_queue_it_found(both):
    """Refused enqueues change nothing queued; a later task may read what an earlier queued task defines; a
    cancelled queue leaves those definitions undone (reference: test_scoped_graph_queue.py:158-174)."""
    scope = abi.Scope(both)
    a = _reserved(both, scope, 1)
    b = _reserved(both, scope, 2)
    write = abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL)
    read = abi.access(flags=abi.READ_ALL)
    assert _queued_task(both, scope, 1, [(a, write)]) == abi.OK
    before = bytes(_queue(both, scope))
    assert _queued_task(both, scope, 2, [(b, read)]) == abi.UNINITIALIZED
    assert bytes(_queue(both, scope)) == before
    assert _queued_task(both, scope, 3, [(2**63, read)]) == abi.STALE
    assert bytes(_queue(both, scope)) == before
    assert _queued_task(both, scope, 4, [(a, read), (b, write)]) == abi.OK
    assert _queue(both, scope).pending_tasks == 2
    assert both.fort_scope_graph_queue_cancel_v1(scope.handle) == abi.OK
    assert both.fort_scope_host_begin(scope.handle, a, c.byref(read)) == abi.UNINITIALIZED
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_a_long_queued_chain_runs_nothing_until_submitted(both):
    """A hundred dependent tasks queue without launching, their arguments copied; cancelled, they leave the
    array untouched (reference: test_scoped_graph_queue.py:177-189)."""
    scope = abi.Scope(both)
    host, address = _array(np.arange(8, dtype=np.float64))
    scope.keep.append(host)
    _, h = scope.register(address, [8], identity=1, initialized=False)
    assert both.fort_scope_device_reserve_v1(scope.handle, h, c.byref(c.c_void_p())) == abi.OK
    for index in range(100):
        flags = abi.WRITE_ALL | abi.OVERWRITE_ALL if index == 0 else abi.READ_ALL | abi.WRITE_ALL
        assert _queued_task(both, scope, index + 1, [(h, abi.access(flags=flags))], scalar=index) == abi.OK
    queued = _queue(both, scope)
    assert queued.accepted_tasks == queued.pending_tasks == queued.peak_pending_tasks == 100
    assert queued.copied_argument_bytes == 100 * c.sizeof(c.c_int)
    assert scope.stats().launches == 0
    assert both.fort_scope_graph_queue_cancel_v1(scope.handle) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == list(range(8))


@pytest.mark.parametrize("exact_budget", [False, True])
def test_faces_move_exactly_and_round_trips_move_nothing(both, exact_budget):
    """The device wrote everything and the host then overwrote the interior: a host read moves just the six
    halo faces home, a device read moves just the interior back as one copy, and further read-only round trips
    move nothing (reference: test_scoped_direct_transport.py:13-58)."""
    x, y, z = 134, 70, 70
    count = x * y * z
    scope = abi.Scope(both)
    if exact_budget:
        assert both.fort_scope_set_device_budget(scope.handle, count * 8) == abi.OK
    host, address = _array(np.full(count, -7.0))
    _, h = scope.register(address, [x, y, z], lower=[-10, 2, -100])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, count)[:] = 1000000.0 + np.arange(count)
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    interior = [((3, 3, 2), (131, 67, 68))]
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(write=interior, overwrite=interior))) == \
        abi.OK
    view = host.reshape(z, y, x)
    view[2:68, 3:67, 3:131] = -42.0
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    read = abi.access(flags=abi.READ_ALL)
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(read)) == abi.OK
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    inner = 128 * 64 * 66
    stats = scope.stats()
    assert (stats.downloads, stats.download_bytes) == (6, (count - inner) * 8)
    expected = 1000000.0 + np.arange(count).reshape(z, y, x)
    expected[2:68, 3:67, 3:131] = -42.0
    assert np.array_equal(view, expected)
    assert _device_begin(scope, h, read)[0] == abi.OK
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    mirrored = scope.stats()
    assert (mirrored.uploads, mirrored.upload_bytes) == (1, inner * 8)
    for _ in range(20):
        assert both.fort_scope_host_begin(scope.handle, h, c.byref(read)) == abi.OK
        assert both.fort_scope_host_end(scope.handle, h) == abi.OK
        assert _device_begin(scope, h, read)[0] == abi.OK
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    final = scope.stats()
    assert (final.uploads, final.downloads, final.allocations) == (mirrored.uploads, mirrored.downloads, 1)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_domain_outlives_borrowing_context(both):
    domain = abi.U64()
    assert both.fort_scope_domain_create_v1(0, c.byref(domain)) == abi.OK
    scope = abi.Scope(both, domain=domain.value)
    host, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    status, dev = _device_begin(scope, h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))
    assert status == abi.OK
    _dev(dev, 4)[:] = 9.0
    assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    got = abi.U64()
    assert both.fort_scope_domain_get_v1(scope.handle, c.byref(got)) == abi.OK and got.value == domain.value
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [0.0] * 4  # a borrowed context does not publish
    second = abi.Scope(both, domain=domain.value)
    assert both.fort_scope_close(second.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain.value) == abi.OK
    assert host.tolist() == [9.0] * 4  # domain close is the publication frontier


def test_budget_default_from_environment(both, monkeypatch):
    """FORT_RESIDENT_DEVICE_BUDGET replaces the derived budget: a positive count of bytes with an optional K, M or
    G; anything else is refused with the reference's message (reference: test_resident_default_budget_cuda.py:91-99)."""
    out = c.c_size_t()
    for value, expected in (("3M", 3 << 20), ("3145728", 3145728), ("64K", 65536), ("5m", 5 << 20), ("1G", 1 << 30)):
        monkeypatch.setenv("FORT_RESIDENT_DEVICE_BUDGET", value)
        assert both.fort_scope_device_budget_default_v1(0, c.byref(out)) == abi.OK
        assert out.value == expected
    for value in ("12x", "lots", "-5", "0", "12Q", "1.5G", "+5", " 5", "99999999999999999999G"):
        monkeypatch.setenv("FORT_RESIDENT_DEVICE_BUDGET", value)
        assert both.fort_scope_device_budget_default_v1(0, c.byref(out)) == abi.ARGUMENT, value
        assert b"FORT_RESIDENT_DEVICE_BUDGET must be a positive count of bytes" in both.fort_scope_error()
    # an empty value reads as unset: the budget is derived (the reference's `stated && stated[0]`)
    monkeypatch.setenv("FORT_RESIDENT_DEVICE_BUDGET", "")
    assert both.fort_scope_device_budget_default_v1(0, c.byref(out)) == abi.OK
    assert out.value > 0


def test_budget_default_needs_free_memory_beyond_the_reserve(ours, monkeypatch):
    """The derived budget is the free memory less a sixteenth of the device (at least 512 MiB); a device with no
    more free than that is refused in the reference's words (scoped_runtime.cu:1766-1769), not given a zero
    budget. The CPU backend's device has 16 GiB; its free bytes come from F2C_TEST_FREE_BYTES."""
    monkeypatch.delenv("FORT_RESIDENT_DEVICE_BUDGET", raising=False)
    out = c.c_size_t()
    assert ours.fort_scope_device_budget_default_v1(0, c.byref(out)) == abi.OK
    assert out.value == (12 << 30) - (1 << 30)
    monkeypatch.setenv("F2C_TEST_FREE_BYTES", str((1 << 30) + 4096))
    assert ours.fort_scope_device_budget_default_v1(0, c.byref(out)) == abi.OK and out.value == 4096
    for free in (1 << 30, 100 << 20, 0):
        monkeypatch.setenv("F2C_TEST_FREE_BYTES", str(free))
        assert ours.fort_scope_device_budget_default_v1(0, c.byref(out)) == abi.RESOURCE
        assert b"the device has no free memory for a residency domain" in ours.fort_scope_error()


def test_execution_error_poisons(both):
    scope = abi.Scope(both)
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    assert both.fort_scope_execution_error(scope.handle, b"kernel failed") == abi.EXECUTION
    assert both.fort_scope_wait(scope.handle) == abi.EXECUTION
    status, _ = _device_begin(scope, h, abi.access(flags=abi.READ_ALL))
    assert status == abi.EXECUTION
    assert both.fort_scope_close(scope.handle) != abi.OK
    assert both.fort_scope_abandon(scope.handle) == abi.OK


# ------------------------------------------------------------------------------- this runtime

KERNEL = c.CFUNCTYPE(None, c.POINTER(c.c_void_p))


def _axpy_kernel(log):
    """A host 'kernel' for the CPU backend: x[i] = x[i] * a + b for i < n; arguments (double*, int, double, double)."""

    def run(args):
        pointer = c.cast(args[0], c.POINTER(c.c_void_p))[0]
        n = c.cast(args[1], c.POINTER(c.c_int))[0]
        a = c.cast(args[2], c.POINTER(c.c_double))[0]
        b = c.cast(args[3], c.POINTER(c.c_double))[0]
        x = _dev(pointer, n)
        x[:] = x * a + b
        log.append((n, a, b))

    return KERNEL(run)


def _enqueue(scope, fn, handle, n, a, b, key=7, grid=1, block=32):
    dev = (c.c_void_p * 1)()
    harr = (abi.U64 * 1)(handle)
    assert scope.lib.fort_scope_device_reserve_many_v1(scope.handle, harr, 1, dev) == abi.OK
    values = [c.c_void_p(dev[0]), c.c_int(n), c.c_double(a), c.c_double(b)]
    argv = (c.c_void_p * 4)(*[c.cast(c.pointer(v), c.c_void_p) for v in values])
    sizes = (c.c_size_t * 4)(8, 4, 8, 8)
    kernel = abi.Kernel(1, 0, c.cast(fn, c.c_void_p), (c.c_uint32 * 3)(grid, 1, 1), (c.c_uint32 * 3)(block, 1, 1),
                        0, argv, 4)
    acc = abi.access(flags=abi.READ_ALL | abi.WRITE_ALL)
    binding = (abi.Binding * 1)(abi.Binding(handle, acc))
    task = abi.Task(kernel, binding, 1)
    return scope.lib.fort_scope_graph_enqueue_v1(scope.handle, key, c.byref(task), sizes)


def test_queue_replays_as_graph_with_parameter_updates(ours):
    scope = abi.Scope(ours)
    host, address = _array(np.ones(8))
    _, h = scope.register(address, [8])
    log = []
    fn = _axpy_kernel(log)
    for step in range(4):
        assert _enqueue(scope, fn, h, 8, 2.0, float(step)) == abi.OK
        assert ours.fort_scope_graph_flush_v1(scope.handle) == abi.OK
    assert ours.fort_scope_wait(scope.handle) == abi.OK
    g = abi.GraphStats()
    assert ours.fort_scope_graph_stats_get_v1(scope.handle, c.byref(g)) == abi.OK
    # first reach direct, second instantiates, the rest replay; b changes every step
    assert (g.creations, g.instantiations, g.replays, g.parameter_updates) == (1, 1, 2, 2)
    q = abi.QueueStats()
    assert ours.fort_scope_graph_queue_stats_get_v1(scope.handle, c.byref(q)) == abi.OK
    assert (q.accepted_tasks, q.direct_submissions, q.explicit_flushes) == (4, 1, 4)
    assert [entry[2] for entry in log] == [0.0, 1.0, 2.0, 3.0]
    assert ours.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(h), 1) == abi.OK
    expect = 1.0
    for step in range(4):
        expect = expect * 2.0 + step
    assert host.tolist() == [expect] * 8
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_queue_flushes_itself_at_the_work_threshold(monkeypatch):
    monkeypatch.setenv("FORT_SCOPE_GRAPH_QUEUE_WORK", "64")
    lib = _ours()
    scope = abi.Scope(lib)
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    log = []
    fn = _axpy_kernel(log)
    assert _enqueue(scope, fn, h, 4, 1.0, 1.0, block=32) == abi.OK
    assert log == []  # 32 threads: still queued
    assert _enqueue(scope, fn, h, 4, 1.0, 1.0, block=32) == abi.OK
    assert len(log) == 2  # 64 threads: submitted
    assert lib.fort_scope_close(scope.handle) == abi.OK


def test_host_access_drains_queued_writers(ours):
    scope = abi.Scope(ours)
    host, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    log = []
    fn = _axpy_kernel(log)
    assert _enqueue(scope, fn, h, 4, 1.0, 5.0) == abi.OK
    assert log == []
    assert ours.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert len(log) == 1 and host.tolist() == [5.0] * 4
    assert ours.fort_scope_host_end(scope.handle, h) == abi.OK
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_queue_policies_are_captured_at_create(monkeypatch):
    monkeypatch.setenv("FORT_SCOPE_GRAPH_QUEUE", "0")
    monkeypatch.setenv("FORT_SCOPE_CUDA_GRAPHS", "0")
    lib = _ours()
    scope = abi.Scope(lib)
    monkeypatch.delenv("FORT_SCOPE_GRAPH_QUEUE")
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    log = []
    fn = _axpy_kernel(log)
    for _ in range(3):
        assert _enqueue(scope, fn, h, 4, 1.0, 1.0) == abi.OK
        assert len(log) >= 1  # submitted at once
    q = abi.QueueStats()
    assert lib.fort_scope_graph_queue_stats_get_v1(scope.handle, c.byref(q)) == abi.OK
    assert (q.queue_enabled, q.graphs_enabled, q.direct_kernels) == (0, 0, 3)
    assert lib.fort_scope_close(scope.handle) == abi.OK


def test_enqueue_requires_reserved_storage_and_valid_arguments(ours):
    scope = abi.Scope(ours)
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    fn = _axpy_kernel([])
    acc = abi.access(flags=abi.READ_ALL)
    binding = (abi.Binding * 1)(abi.Binding(h, acc))
    value = c.c_int(1)
    argv = (c.c_void_p * 1)(c.cast(c.pointer(value), c.c_void_p))
    kernel = abi.Kernel(1, 0, c.cast(fn, c.c_void_p), (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(1, 1, 1), 0, argv, 1)
    task = abi.Task(kernel, binding, 1)
    assert ours.fort_scope_graph_enqueue_v1(scope.handle, 1, c.byref(task), (c.c_size_t * 1)(4)) == abi.STATE
    assert ours.fort_scope_graph_enqueue_v1(scope.handle, 1, c.byref(task), None) == abi.ARGUMENT
    kernel.block[0] = 2048
    task = abi.Task(kernel, binding, 1)
    assert ours.fort_scope_graph_enqueue_v1(scope.handle, 1, c.byref(task), (c.c_size_t * 1)(4)) == abi.ARGUMENT
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_merged_members_must_be_independent(ours):
    scope = abi.Scope(ours)
    _, address = _array(np.zeros(10))
    _, h = scope.register(address, [10])
    dev = (c.c_void_p * 1)()
    assert ours.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(h), 1, dev) == abi.OK
    log = []
    fn = _axpy_kernel(log)
    values = [c.c_void_p(dev[0]), c.c_int(10), c.c_double(1.0), c.c_double(0.0)]
    argv = (c.c_void_p * 4)(*[c.cast(c.pointer(v), c.c_void_p) for v in values])
    sizes = (c.c_size_t * 4)(8, 4, 8, 8)
    kernel = abi.Kernel(1, 0, c.cast(fn, c.c_void_p), (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(1, 1, 1), 0, argv, 4)
    low = abi.access(read=[((0,), (1,))], write=[((0,), (1,))], overwrite=[((0,), (1,))])
    high = abi.access(read=[((9,), (10,))], write=[((9,), (10,))], overwrite=[((9,), (10,))])
    m1 = (abi.Binding * 1)(abi.Binding(h, low))
    m2 = (abi.Binding * 1)(abi.Binding(h, high))
    members = (abi.Member * 2)(abi.Member(m1, 1), abi.Member(m2, 1))
    assert ours.fort_scope_graph_enqueue_members_v1(scope.handle, 3, c.byref(kernel), sizes, members, 2) == abi.OK
    clash = abi.access(read=[((0,), (2,))])
    m2 = (abi.Binding * 1)(abi.Binding(h, clash))
    members = (abi.Member * 2)(abi.Member(m1, 1), abi.Member(m2, 1))
    assert ours.fort_scope_graph_enqueue_members_v1(scope.handle, 3, c.byref(kernel), sizes, members, 2) == abi.BOUNDARY
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_failed_launch_poisons_without_replay(monkeypatch):
    lib = _ours()
    scope = abi.Scope(lib)
    host, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    log = []
    fn = _axpy_kernel(log)
    assert _enqueue(scope, fn, h, 4, 1.0, 1.0) == abi.OK
    monkeypatch.setenv("F2C_TEST_FAIL_LAUNCH", "1")
    assert lib.fort_scope_graph_flush_v1(scope.handle) == abi.EXECUTION
    monkeypatch.delenv("F2C_TEST_FAIL_LAUNCH")
    assert "unsafe replay prohibited" in lib.fort_scope_error().decode()
    dev = (c.c_void_p * 1)()
    assert lib.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(h), 1, dev) == abi.EXECUTION
    assert lib.fort_scope_close(scope.handle) == abi.EXECUTION
    assert lib.fort_scope_abandon(scope.handle) == abi.OK
    assert log == [] and host.tolist() == [0.0] * 4


def test_graph_build_failure_falls_back_to_direct_launches(monkeypatch):
    lib = _ours()
    scope = abi.Scope(lib)
    host, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    log = []
    fn = _axpy_kernel(log)
    monkeypatch.setenv("F2C_TEST_FAIL_GRAPH_CREATE", "1")
    for _ in range(3):
        assert _enqueue(scope, fn, h, 4, 1.0, 1.0) == abi.OK
        assert lib.fort_scope_graph_flush_v1(scope.handle) == abi.OK
    q = abi.QueueStats()
    assert lib.fort_scope_graph_queue_stats_get_v1(scope.handle, c.byref(q)) == abi.OK
    assert q.graph_resource_fallbacks >= 1 and len(log) == 3
    assert lib.fort_scope_close(scope.handle) == abi.OK
    assert host.tolist() == [3.0] * 4


def test_fragmented_sections_reconcile(ours):
    scope = abi.Scope(ours)
    host, address = _array(np.zeros(600))
    _, h = scope.register(address, [600])
    for i in range(0, 600, 4):
        box = ((i,), (i + 1,))
        status, dev = _device_begin(scope, h, abi.access(write=[box], overwrite=[box]))
        assert status == abi.OK
        _dev(dev, 600)[i] = float(i)
        assert ours.fort_scope_device_end(scope.handle, h) == abi.OK
    assert ours.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(h), 1) == abi.OK
    expect = np.zeros(600)
    expect[::4] = np.arange(0, 600, 4)
    assert np.array_equal(host, expect)
    assert scope.stats().reconciliations >= 1
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_trace_lines(tmp_path):
    script = tmp_path / "trace.py"
    script.write_text(
        "import sys, ctypes as c, numpy as np\n"
        f"sys.path[:0] = [{os.path.join(ROOT, 'fortran-to-cuda_gb300')!r}]\n"
        "from compiler import native\n"
        "from compiler.runtime import abi\n"
        "lib = abi.bind(c.CDLL(str(native.build_cpu_runtime())))\n"
        "s = abi.Scope(lib)\n"
        "a = np.zeros(4)\n"
        "st, h = s.register(a.ctypes.data, [4])\n"
        "d = c.c_void_p()\n"
        "assert lib.fort_scope_device_begin(s.handle, h, c.byref(abi.access(flags=3)), c.byref(d)) == 0\n"
        "assert lib.fort_scope_device_end(s.handle, h) == 0\n"
        "assert lib.fort_scope_close(s.handle) == 0\n")
    env = dict(os.environ, FORT_RUNTIME_TRACE="1")
    out = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0, out.stderr
    events = [line.split()[1] for line in out.stderr.splitlines() if line.startswith("FORT_SCOPED ")]
    assert events.count("upload") == 1 and events.count("download") == 1 and "register" in events


PROVENANCE = r"""
import ctypes as c, sys
import numpy as np
sys.path[:0] = sys.argv[1:2]
from compiler import native
from compiler.runtime import abi
lib = abi.bind(c.CDLL(str(native.build_cpu_runtime())))
KERNEL = c.CFUNCTYPE(None, c.POINTER(c.c_void_p))


@KERNEL
def axpy(args):
    x = np.ctypeslib.as_array(c.cast(c.cast(args[0], c.POINTER(c.c_void_p))[0], c.POINTER(c.c_double)), shape=(8,))
    x[:] = x * c.cast(args[2], c.POINTER(c.c_double))[0] + c.cast(args[3], c.POINTER(c.c_double))[0]


scope = abi.Scope(lib)
a = np.ones(8)
_, h = scope.register(a.ctypes.data, [8])
dev = (c.c_void_p * 1)()
assert lib.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(h), 1, dev) == 0
lib.fort_scope_trace_set_v1(scope.handle, 0b1011, b"a" * 64, b"b" * 64, None, b"d" * 64, None, None, None)
values = [c.c_void_p(dev[0]), c.c_int(8), c.c_double(1.0), c.c_double(1.0)]
argv = (c.c_void_p * 4)(*[c.cast(c.pointer(v), c.c_void_p) for v in values])
sizes = (c.c_size_t * 4)(8, 4, 8, 8)
task = abi.Task(abi.Kernel(1, 0, c.cast(axpy, c.c_void_p), (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0,
                           argv, 4), (abi.Binding * 1)(abi.Binding(h, abi.access(flags=3))), 1)
for round_ in range(3):
    for label in (b"1", b"2", b"3"):
        lib.fort_scope_trace_set_v1(scope.handle, 1 << 4, None, None, None, None, label * 64, None, None)
        assert lib.fort_scope_graph_enqueue_v1(scope.handle, 7, c.byref(task), sizes) == 0
    lib.fort_scope_trace_set_v1(scope.handle, 1 << 4, None, None, None, None, b"9" * 64, None, None)
    assert lib.fort_scope_graph_flush_v1(scope.handle) == 0
assert lib.fort_scope_close(scope.handle) == 0
assert a.tolist() == [10.0] * 8
"""


def test_queued_launches_report_the_provenance_they_were_accepted_under(tmp_path):
    """A queued task's launch, direct or as a graph node, carries the trace state of its acceptance, not the one
    current at the flush; every line carries the reference's keys (reference:
    test_scoped_graph_queue_cuda.py:343-372)."""
    import re

    script = tmp_path / "provenance.py"
    script.write_text(PROVENANCE)
    run = subprocess.run([sys.executable, str(script), os.path.join(ROOT, "fortran-to-cuda_gb300")],
                         capture_output=True, text=True, timeout=120, env={**os.environ, "FORT_RUNTIME_TRACE": "1"})
    assert run.returncode == 0, run.stdout + run.stderr
    rows = [(m[1], dict(re.findall(r"(\w+)=([^\s]+)", m[2]))) for line in run.stderr.splitlines()
            if (m := re.match(r"FORT_SCOPED (launch|graph_kernel|graph_submit|register) (.*)", line))]
    assert [row["bytes"] for event, row in rows if event == "graph_submit"] == ["3", "3"]
    rows = [(event, row) for event, row in rows if event != "graph_submit"]
    launched = [row for event, row in rows if event in ("launch", "graph_kernel")]
    assert [row["implementation"] for row in launched] == [d * 64 for d in "123123123"]
    assert [event for event, _ in rows if event != "register"] == ["launch"] * 3 + ["graph_kernel"] * 6
    assert all(row["owner"] == "a" * 64 and row["procedure"] == "b" * 64 and row["operation"] == "d" * 64
               and row["segment"] == "unknown" and row["bytes"] == "0" and row["provenance_version"] == "1"
               for row in launched)
    (register,) = [row for event, row in rows if event == "register"]
    assert register["bytes"] == "64" and "buffer" in register and register["generation"] == "1"
    assert register["domain_role"] == "storage"
    # closing reports the context's statistics as evidence records, with the reference's keys
    records = {r["event"]: r for r in (json.loads(line.removeprefix("FORT_SCOPED evidence "))
                                       for line in run.stderr.splitlines() if line.startswith("FORT_SCOPED evidence "))}
    graphs, queue = records["graph_statistics"], records["command_queue_statistics"]
    assert graphs["complete"] and graphs["live_graphs"] == 0 and graphs["creations"] == graphs["destructions"] == 1
    assert (graphs["replays"], graphs["submissions"], graphs["schema_version"]) == (1, 3, 1)
    assert (queue["accepted_tasks"], queue["direct_submissions"], queue["direct_kernels"]) == (9, 1, 3)


# ------------------------------------------------------------------------------- slab pipelines

NX_S, NY_S, NZ_S = 4, 3, 10  # extents; planes 1..8 are the interior along the last dimension


def _plane_sum_kernel(log):
    """Host 'kernel': y[k] = x[k-1] + x[k] + x[k+1] on whole planes k0..k1-1; arguments (double*, double*, int, int)."""

    def run(args):
        x = _dev(c.cast(args[0], c.POINTER(c.c_void_p))[0], NX_S * NY_S * NZ_S).reshape(NZ_S, NY_S * NX_S)
        y = _dev(c.cast(args[1], c.POINTER(c.c_void_p))[0], NX_S * NY_S * NZ_S).reshape(NZ_S, NY_S * NX_S)
        k0 = c.cast(args[2], c.POINTER(c.c_int))[0]
        k1 = c.cast(args[3], c.POINTER(c.c_int))[0]
        y[k0:k1] = x[k0 - 1:k1 - 1] + x[k0:k1] + x[k0 + 1:k1 + 1]
        log.append((k0, k1))

    return KERNEL(run)


def _slab_tasks(fn, devices, hx, hy, bounds, nx=NX_S, ny=NY_S, reads=None):
    keep, tasks, sizes = [], [], []
    for k0, k1 in bounds:
        values = [c.c_void_p(devices[0]), c.c_void_p(devices[1]), c.c_int(k0), c.c_int(k1)]
        argv = (c.c_void_p * 4)(*[c.cast(c.pointer(v), c.c_void_p) for v in values])
        kernel = abi.Kernel(1, 0, c.cast(fn, c.c_void_p), (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0,
                            argv, 4)
        read = abi.access(read=reads(k0, k1) if reads else [((0, 0, k0 - 1), (nx, ny, k1 + 1))])
        write = abi.access(write=[((0, 0, k0), (nx, ny, k1))], overwrite=[((0, 0, k0), (nx, ny, k1))])
        binding = (abi.Binding * 2)(abi.Binding(hx, read), abi.Binding(hy, write))
        keep += [values, argv, read, write, binding]
        tasks.append(abi.Task(kernel, binding, 2))
        sizes += [8, 8, 4, 4]
    return (abi.Task * len(tasks))(*tasks), (c.c_size_t * len(sizes))(*sizes), keep


def _reserve_slabs(lib, scope, handles):
    devices = (c.c_void_p * len(handles))()
    pipelined = c.c_int(-1)
    status = lib.fort_scope_device_reserve_slabs_v1(scope.handle, (abi.U64 * len(handles))(*handles), len(handles),
                                                    devices, c.byref(pipelined))
    return status, list(devices), pipelined.value


def test_slab_pipeline_publishes_host_round_writes(monkeypatch):
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    lib = _ours()
    scope = abi.Scope(lib)
    x, xa = _array(np.arange(NX_S * NY_S * NZ_S, dtype=np.float64))
    y, ya = _array(np.full(NX_S * NY_S * NZ_S, -1.0))
    _, hx = scope.register(xa, [NX_S, NY_S, NZ_S])
    _, hy = scope.register(ya, [NX_S, NY_S, NZ_S])
    log = []
    fn = _plane_sum_kernel(log)
    bounds = [(1, 4), (4, 7), (7, 9)]

    def expected():
        p = x.reshape(NZ_S, -1)
        out = np.full_like(p, -1.0)
        out[1:9] = p[0:8] + p[1:9] + p[2:10]
        return out.ravel()

    for round_ in range(3):
        status, devices, pipelined = _reserve_slabs(lib, scope, [hx, hy])
        assert status == abi.OK
        # the first use has no history; later rounds are host-round for both arrays
        assert pipelined == (0 if round_ == 0 else 1)
        assert devices[0] != xa and devices[1] != ya  # never handed out in place
        tasks, sizes, keep = _slab_tasks(fn, devices, hx, hy, bounds)
        before = scope.stats()
        assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, len(bounds), sizes) == abi.OK
        after = scope.stats()
        assert log[-3:] == bounds
        if pipelined:
            # published slab by slab, before any host access asks for it
            assert after.downloads - before.downloads == len(bounds)
            assert np.array_equal(y, expected())
        assert lib.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(hy), 1) == abi.OK
        assert scope.stats().downloads == after.downloads + (0 if pipelined else 1)
        assert np.array_equal(y, expected())
        # the host rewrites the input: the next round uploads it slab by slab, whole planes each
        assert lib.fort_scope_host_begin(scope.handle, hx, c.byref(abi.access(flags=abi.WRITE_ALL))) == abi.OK
        x[:] = x * 0.5 + round_
        assert lib.fort_scope_host_end(scope.handle, hx) == abi.OK
        if round_ == 1:
            assert after.uploads - before.uploads == len(bounds)
    assert lib.fort_scope_close(scope.handle) == abi.OK


def test_slab_uploads_end_on_host_boundaries(monkeypatch):
    """A slab upload of 8 MiB or more runs on to the next 2 MiB boundary of the host array (where the host is
    current), so the next slab's upload starts on one; results and the total moved are unchanged."""
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    nx, ny, nz = 256, 256, 82                       # planes of 512 KiB, slabs of 20 planes
    plane, n = nx * ny, nx * ny * nz
    lib = _ours()
    scope = abi.Scope(lib)
    x, xa = _array(np.arange(n, dtype=np.float64))
    y, ya = _array(np.zeros(n))
    _, hx = scope.register(xa, [nx, ny, nz])
    _, hy = scope.register(ya, [nx, ny, nz])
    log = []

    def run(args):
        xd = _dev(c.cast(args[0], c.POINTER(c.c_void_p))[0], n)
        yd = _dev(c.cast(args[1], c.POINTER(c.c_void_p))[0], n)
        k0 = c.cast(args[2], c.POINTER(c.c_int))[0]
        k1 = c.cast(args[3], c.POINTER(c.c_int))[0]
        unfilled = np.isnan(xd)
        log.append((k0, k1, int(unfilled.argmax()) if unfilled.any() else n))
        xp, yp = xd.reshape(nz, plane), yd.reshape(nz, plane)
        yp[k0:k1] = xp[k0 - 1:k1 - 1] + xp[k0:k1] + xp[k0 + 1:k1 + 1]

    fn = KERNEL(run)
    bounds = [(1, 21), (21, 41), (41, 61), (61, 81)]

    def reads(k0, k1):
        # overlapping boxes whose union is the planes read, as the entries' cross-shaped stencils give
        return [((0, 0, k0 - 1), (nx - 1, ny, k1 + 1)), ((1, 0, k0 - 1), (nx, ny, k1 + 1)),
                ((0, 1, k0), (nx, ny - 1, k1))]

    for round_ in range(3):
        status, devices, pipelined = _reserve_slabs(lib, scope, [hx, hy])
        assert status == abi.OK and pipelined == (0 if round_ == 0 else 1)
        if pipelined:
            _dev(devices[0], n)[:] = np.nan                        # nothing of x on the device yet
        tasks, sizes, keep = _slab_tasks(fn, devices, hx, hy, bounds, nx, ny, reads)
        before = scope.stats()
        assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, len(bounds), sizes) == abi.OK
        after = scope.stats()
        if pipelined:
            filled = [f for _, _, f in log[-len(bounds):]]
            for (k0, k1), f in zip(bounds[:-1], filled[:-1]):
                assert f >= (k1 + 1) * plane                       # what the slab reads is there
                assert (xa + 8 * f) % (2 << 20) == 0               # and the upload ended on a host boundary
            assert filled[-1] == n
            assert after.uploads - before.uploads == len(bounds)   # one copy a slab
            assert after.upload_bytes - before.upload_bytes == x.nbytes
            assert after.reconciliations == before.reconciliations  # the valid sections stay a few boxes
        assert lib.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(hy), 1) == abi.OK
        p = x.reshape(nz, plane)
        assert np.array_equal(y.reshape(nz, plane)[1:81], p[0:80] + p[1:81] + p[2:82])
        assert lib.fort_scope_host_begin(scope.handle, hx, c.byref(abi.access(flags=abi.WRITE_ALL))) == abi.OK
        x[:] = x * 0.5 + round_
        assert lib.fort_scope_host_end(scope.handle, hx) == abi.OK
    assert lib.fort_scope_close(scope.handle) == abi.OK


def test_slab_uploads_of_the_advection_step_stay_few(monkeypatch):
    """The 512 x 512 x 128 step (halo 2) in its 14 slabs, with the read sections the advection entries declare
    for U (interior plus one cell, cross-shaped): one upload a slab and no reconciliation. Marking the upload's
    cross-shaped pieces valid before the whole run splintered the valid sections past their limit at slab 11,
    and the runtime then reconciled synchronously."""
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    n_in, nz, h = 512, 128, 2
    ex, ez = n_in + 2 * h, nz + 2 * h
    lib = _ours()
    scope = abi.Scope(lib)
    _, xa = _array(np.zeros(ex * ex * ez))
    _, ya = _array(np.zeros(ex * ex * ez))
    _, hx = scope.register(xa, [ex, ex, ez])
    _, hy = scope.register(ya, [ex, ex, ez])
    fn = KERNEL(lambda args: None)
    edges = [0, 5, 14, 24, 34, 44, 54, 64, 73, 83, 93, 103, 113, 123, 128]
    i0, i1 = h, h + n_in

    def reads(k0, k1):
        z0, z1 = k0 + h, k1 + h
        return [((i0 - 1, i0, z0), (i1 + 1, i1, z1)), ((i0, i0 - 1, z0), (i1, i1 + 1, z1)),
                ((i0, i0, z0 - 1), (i1, i1, z1 + 1)), ((i0 - 1, i0, z0), (i1, i1 + 1, z1)),
                ((i0 - 1, i0, z0), (i1, i1, z1 + 1))]

    keep = []
    for round_ in range(3):
        status, devices, pipelined = _reserve_slabs(lib, scope, [hx, hy])
        assert status == abi.OK and pipelined == (0 if round_ == 0 else 1)
        tasks, sizes = [], []
        for k0, k1 in zip(edges, edges[1:]):
            values = [c.c_void_p(devices[0]), c.c_void_p(devices[1])]
            argv = (c.c_void_p * 2)(*[c.cast(c.pointer(v), c.c_void_p) for v in values])
            kernel = abi.Kernel(1, 0, c.cast(fn, c.c_void_p), (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1),
                                0, argv, 2)
            read = abi.access(read=reads(k0, k1))
            box = [((i0, i0, k0 + h), (i1, i1, k1 + h))]
            write = abi.access(write=box, overwrite=box)
            binding = (abi.Binding * 2)(abi.Binding(hx, read), abi.Binding(hy, write))
            keep += [values, argv, read, write, binding]
            tasks.append(abi.Task(kernel, binding, 2))
            sizes += [8, 8]
        before = scope.stats()
        assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, (abi.Task * len(tasks))(*tasks), len(tasks),
                                              (c.c_size_t * len(sizes))(*sizes)) == abi.OK
        after = scope.stats()
        if pipelined:
            assert after.uploads - before.uploads == len(tasks)
            assert after.reconciliations == before.reconciliations
        assert lib.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(hy), 1) == abi.OK
        assert lib.fort_scope_host_begin(scope.handle, hx, c.byref(abi.access(flags=abi.WRITE_ALL))) == abi.OK
        assert lib.fort_scope_host_end(scope.handle, hx) == abi.OK
    assert lib.fort_scope_close(scope.handle) == abi.OK


def test_slab_enqueue_validates_before_work(monkeypatch):
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    lib = _ours()
    scope = abi.Scope(lib)
    _, xa = _array(np.zeros(NX_S * NY_S * NZ_S))
    _, ya = _array(np.zeros(NX_S * NY_S * NZ_S))
    _, hx = scope.register(xa, [NX_S, NY_S, NZ_S])
    _, hy = scope.register(ya, [NX_S, NY_S, NZ_S], initialized=False)
    log = []
    fn = _plane_sum_kernel(log)
    tasks, sizes, keep = _slab_tasks(fn, [xa, ya], hx, hy, [(1, 9)])
    # no device storage reserved yet
    assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, 1, sizes) == abi.STATE
    assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, 0, sizes) == abi.ARGUMENT
    assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, 65, sizes) == abi.ARGUMENT
    status, devices, pipelined = _reserve_slabs(lib, scope, [hx, hy])
    assert (status, pipelined) == (abi.OK, 0)
    # a task that reads undefined values is refused and nothing runs
    tasks, sizes, keep = _slab_tasks(fn, devices, hy, hx, [(1, 9)])
    assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, 1, sizes) == abi.UNINITIALIZED
    assert log == []
    assert lib.fort_scope_close(scope.handle) == abi.OK


def test_reserve_many_hands_host_round_arrays_out_in_place(monkeypatch):
    """The single-task path still maps host-round arrays in place; the slab reservation never does."""
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    lib = _ours()
    scope = abi.Scope(lib)
    _, xa = _array(np.ones(8))
    _, hx = scope.register(xa, [8])
    log = []
    fn = _axpy_kernel(log)
    for round_ in range(2):
        devices = (c.c_void_p * 1)()
        assert lib.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(hx), 1, devices) == abi.OK
        assert (devices[0] == xa) == (round_ == 1)
        assert _enqueue(scope, fn, hx, 8, 1.0, 1.0) == abi.OK
        assert lib.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(hx), 1) == abi.OK
    assert lib.fort_scope_close(scope.handle) == abi.OK


# ------------------------------------------------------------------------------- external providers


def _external(lib, scope, handle, worker, *, type_=abi.REAL64, rank=1, flags=abi.READ_ALL | abi.WRITE_ALL):
    acc = abi.access(flags=flags)
    binding = (abi.ExternalBinding * 1)(abi.ExternalBinding(handle, type_, rank, 8, acc))
    call = abi.ExternalCall(1, 0, binding, 1, 0, 0)
    report = abi.ExternalReport()
    status = lib.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report))
    return status, report


def _worker(log, *, started, result, scale=2.0):
    def run(user, views, count, stream, flag):
        v = views[0]
        log.append((count, v.rank, v.extents[0], v.strides[0], v.element_bytes))
        flag[0] = started
        if started == 1 and result == abi.OK:
            _dev(v.device, v.extents[0])[:] *= scale
        return result

    return abi.EXTERNAL_WORKER(run)


def test_external_transaction_commits_its_effects(both):
    scope = abi.Scope(both)
    host, address = _array(np.arange(6.0))
    _, h = scope.register(address, [6])
    log = []
    status, report = _external(both, scope, h, _worker(log, started=1, result=abi.OK))
    assert status == abi.OK
    assert (report.status, report.started, report.committed) == (abi.OK, 1, 1)
    assert log == [(1, 1, 6, 8, 8)]  # one view: rank 1, extent 6, byte stride 8
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == [2.0 * i for i in range(6)]
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_external_rejection_before_start_changes_nothing(both):
    scope = abi.Scope(both)
    host, address = _array(np.arange(4.0))
    _, h = scope.register(address, [4])
    status, report = _external(both, scope, h, _worker([], started=0, result=abi.RESOURCE))
    assert status == abi.RESOURCE
    assert (report.started, report.committed) == (0, 0)
    # the context stays usable and the values are those of the host
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert host.tolist() == [0.0, 1.0, 2.0, 3.0]
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK


@pytest.mark.parametrize("started, result", [(1, abi.ARGUMENT), (-1, abi.OK), (0, abi.OK), (0, abi.EXECUTION)])
def test_external_failure_after_start_or_without_a_report_poisons(both, started, result):
    scope = abi.Scope(both)
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    status, report = _external(both, scope, h, _worker([], started=started, result=result))
    assert status == abi.EXECUTION
    # nothing is replayed: the context refuses further work
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.EXECUTION
    both.fort_scope_abandon(scope.handle)


def test_an_empty_external_request_touches_nothing(both):
    """No bindings: the worker is not called, nothing is reported as started or committed, no statistic moves
    (reference: test_scoped_domains.py:607-623)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    calls = []

    def run(user, views, count, stream, flag):
        calls.append(count)
        return abi.OK

    worker = abi.EXTERNAL_WORKER(run)
    call = abi.ExternalCall(1, 0, None, 0, 0, 0)
    report = abi.ExternalReport()
    assert both.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report)) == abi.OK
    assert (report.status, report.started, report.committed) == (abi.OK, 0, 0) and calls == []
    assert bytes(scope.stats()) == bytes(abi.Stats())
    assert both.fort_scope_close(scope.handle) == abi.OK
    stats = abi.Stats()
    assert both.fort_scope_domain_stats_get_v1(domain, c.byref(stats)) == abi.OK
    assert bytes(stats) == bytes(abi.Stats())
    assert both.fort_scope_domain_close_v1(domain) == abi.OK


def test_a_failed_domain_is_abandoned_only_after_its_provider_workspace(both):
    """After a provider failed mid-transaction the context is abandoned; the domain refuses abandonment while the
    provider's workspace lease is held, and accepts it once the lease is released; nothing is published
    (reference: test_scoped_domains.py:582-604)."""
    domain = _domain(both)
    lease = abi.U64()
    assert both.fort_scope_domain_workspace_reserve_v1(domain, 16, c.byref(lease)) == abi.OK
    scope = abi.Scope(both, domain=domain)
    host, address = _array([1.0, 2.0])
    _, h = scope.register(address, [2])
    binding = (abi.ExternalBinding * 1)(abi.ExternalBinding(h, abi.REAL64, 1, 8,
                                                            abi.access(flags=abi.READ_ALL | abi.WRITE_ALL)))
    call = abi.ExternalCall(1, 0, binding, 1, lease.value, 16)
    report = abi.ExternalReport()
    worker = _worker([], started=1, result=abi.EXECUTION)
    assert both.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report)) == \
        abi.EXECUTION
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert both.fort_scope_domain_abandon_v1(domain) == abi.STATE
    assert both.fort_scope_domain_workspace_release_v1(domain, lease.value) == abi.OK
    assert both.fort_scope_domain_abandon_v1(domain) == abi.OK
    assert host.tolist() == [1.0, 2.0]


CALLBACK_THROWS = r"""
#include <cassert>
#include <stdexcept>
#include "scoped_runtime.h"
static int worker(void *, const fort_scope_external_view_v1 *, size_t, void *, int *) {
    throw std::runtime_error("provider exception");
}
int main() {
    fort_scope_domain_t domain = 0;
    fort_scope_t context = 0;
    fort_buffer_t buffer = 0;
    if (fort_scope_domain_create_v1(0, &domain) || fort_scope_create_in_domain_v1(domain, &context)) return 2;
    double host[2] = {3, 5};
    size_t extents[1] = {2};
    int64_t lower[1] = {-1};
    fort_scope_layout layout{1, FORT_SCOPE_REAL64, 8, host, extents, lower, 1};
    if (fort_scope_register(context, 1, 1, &layout, 1, &buffer)) return 3;
    fort_scope_access access{};
    access.flags = FORT_SCOPE_READ_ALL | FORT_SCOPE_WRITE_ALL;
    fort_scope_external_binding_v1 binding{buffer, FORT_SCOPE_REAL64, 1, 8, access};
    fort_scope_external_call_v1 call{1, 0, &binding, 1, 0, 0};
    fort_scope_external_report_v1 report{};
    if (fort_scope_external_execute_v1(context, &call, worker, nullptr, &report) != FORT_SCOPE_EXECUTION) return 4;
    if (report.started != 1 || report.committed) return 5;
    if (fort_scope_close(context) != FORT_SCOPE_EXECUTION) return 6;   // poisoned: no publication, no replay
    if (fort_scope_abandon(context) || fort_scope_domain_abandon_v1(domain)) return 7;
    return host[0] == 3 && host[1] == 5 ? 0 : 8;
}
"""


def test_a_throwing_provider_is_contained(both, tmp_path):
    """A provider callback that throws a C++ exception is caught at the C boundary: the call fails as an execution
    error, the context is poisoned, nothing is published (reference: test_scoped_domains.py:671-706)."""
    compiler = shutil.which("g++")
    if compiler is None:
        pytest.skip("no C++ compiler")
    source, exe = tmp_path / "throws.cpp", tmp_path / "throws"
    source.write_text(CALLBACK_THROWS)
    built = subprocess.run([compiler, "-std=c++17", f"-I{os.path.join(ROOT, 'include')}", str(source), both._name,
                            "-o", str(exe)], capture_output=True, text=True, timeout=120)
    assert built.returncode == 0, built.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stderr)


def _execute(lib, scope, bindings, worker, *, lease=0, workspace=0):
    """bindings: (handle, access, type, rank) tuples."""
    items = (abi.ExternalBinding * max(1, len(bindings)))(
        *[abi.ExternalBinding(h, t, r, 8, acc) for h, acc, t, r in bindings])
    call = abi.ExternalCall(1, 0, items if bindings else None, len(bindings), lease, workspace)
    report = abi.ExternalReport()
    status = lib.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report))
    return status, report


def test_external_views_partial_effects_and_workspace(both):
    """The provider sees each array's generation, extents, byte strides and lower bounds; a workspace beyond its
    lease is refused before the call; a partial overwrite defines exactly its section, which the host gets when it
    reads it; the provider's kernels are not counted as launches (reference: test_scoped_domains.py:433-470)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    source, sa = _array(np.arange(6, dtype=np.float64))
    output, oa = _array(np.full(6, -99.0))
    _, a = scope.register(sa, [6], lower=[-3], generation=11)
    _, b = scope.register(oa, [6], identity=2, initialized=False)
    box = [((1,), (5,))]
    bindings = [(a, abi.access(read=box), abi.REAL64, 1), (b, abi.access(write=box, overwrite=box), abi.REAL64, 1)]
    seen = []

    def run(user, views, count, stream, started):
        v = views
        seen.append((count, stream, v[0].generation, v[0].extents[0], v[0].strides[0], v[0].lower_bounds[0],
                     v[1].bytes))
        started[0] = 1
        av, bv = _dev(v[0].device, 6), _dev(v[1].device, 6)
        bv[1:5] = 3 * av[1:5]
        return abi.OK

    worker = abi.EXTERNAL_WORKER(run)
    lease = abi.U64()
    assert both.fort_scope_domain_workspace_reserve_v1(domain, 24, c.byref(lease)) == abi.OK
    status, _ = _execute(both, scope, bindings, worker, lease=lease.value, workspace=25)
    assert status == abi.RESOURCE and seen == []
    status, report = _execute(both, scope, bindings, worker, lease=lease.value, workspace=24)
    assert status == abi.OK
    assert (report.version, report.status, report.started, report.committed) == (1, abi.OK, 1, 1)
    assert seen == [(2, None, 11, 6, 8, -3, 48)]
    assert output.tolist() == [-99.0] * 6
    assert both.fort_scope_host_begin(scope.handle, b, c.byref(abi.access(read=box))) == abi.OK
    assert both.fort_scope_host_end(scope.handle, b) == abi.OK
    assert output.tolist() == [-99.0, 3.0, 6.0, 9.0, 12.0, -99.0]
    stats = scope.stats()
    assert (stats.upload_bytes, stats.download_bytes, stats.launches) == (32, 32, 0)
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_workspace_release_v1(domain, lease.value) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK


@pytest.mark.parametrize("invalid", ["type", "rank", "duplicate", "undefined"])
def test_external_preflight_refuses_before_the_provider(both, invalid):
    """A wrong type or rank, an array bound twice, or a read of undefined values is refused before the provider
    runs and before storage is allocated; a call under a prepared access is refused, and so is closing the context
    (reference: test_scoped_domains.py:473-511)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    _, address = _array([1.0, 2.0, 3.0, 4.0])
    _, h = scope.register(address, [4], initialized=invalid != "undefined")
    read = abi.access(flags=abi.READ_ALL)
    item = (h, read, abi.REAL32 if invalid == "type" else abi.REAL64, 2 if invalid == "rank" else 1)
    bindings = [item, item] if invalid == "duplicate" else [item]
    expected = {"type": abi.ARGUMENT, "rank": abi.ARGUMENT, "duplicate": abi.ALIAS, "undefined": abi.UNINITIALIZED}
    calls = []

    def run(user, views, count, stream, started):
        calls.append(count)
        started[0] = 1
        return abi.OK

    worker = abi.EXTERNAL_WORKER(run)
    status, report = _execute(both, scope, bindings, worker)
    assert status == expected[invalid]
    assert (report.started, report.committed) == (0, 0) and calls == []
    assert scope.stats().allocations == 0
    if invalid != "undefined":
        status, _ = _device_begin(scope, h, read)
        assert status == abi.OK
        status, _ = _execute(both, scope, [(h, read, abi.REAL64, 1)], worker)
        assert status == abi.STATE
        assert both.fort_scope_close(scope.handle) == abi.STATE
        assert both.fort_scope_device_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK


def test_a_rejecting_provider_defines_nothing_and_the_host_recovers(both):
    """A provider that rejects before starting grants no definitions; the host then writes the values itself
    (reference: test_scoped_domains.py:514-536)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    host, address = _array(np.full(4, -8.0))
    _, h = scope.register(address, [4], initialized=False)

    def reject(user, views, count, stream, started):
        started[0] = 0
        return abi.RESOURCE

    worker = abi.EXTERNAL_WORKER(reject)
    status, report = _execute(both, scope, [(h, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL), abi.REAL64, 1)],
                              worker)
    assert status == report.status == abi.RESOURCE and (report.started, report.committed) == (0, 0)
    assert both.fort_scope_host_begin(scope.handle, h, c.byref(abi.access(flags=abi.READ_ALL))) == abi.UNINITIALIZED
    assert both.fort_scope_host_begin(scope.handle, h,
                                      c.byref(abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))) == abi.OK
    host[:] = 2.0 * np.arange(4)
    assert both.fort_scope_host_end(scope.handle, h) == abi.OK
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(domain) == abi.OK
    assert host.tolist() == [0.0, 2.0, 4.0, 6.0]


@pytest.mark.parametrize("mode", ["submitted_failure", "missing_marker", "success_without_submission",
                                  "execution_failure", "commit_failure"])
def test_an_uncertain_provider_outcome_poisons_the_domain(both, monkeypatch, mode):
    """A failure after submission, a missing submission marker, success without submission, an execution failure
    or a failed commit poison context and domain: nothing is published or replayed, and only abandonment ends them
    (reference: test_scoped_domains.py:539-579)."""
    domain = _domain(both)
    scope = abi.Scope(both, domain=domain)
    host, address = _array([1.0, 2.0, 3.0, 4.0])
    _, h = scope.register(address, [4])
    calls = []

    def run(user, views, count, stream, started):
        calls.append(count)
        if mode in ("submitted_failure", "commit_failure"):
            started[0] = 1
            _dev(views[0].device, 4)[0] = 1000.0
            return abi.RESOURCE if mode == "submitted_failure" else abi.OK
        if mode == "missing_marker":
            return abi.OK
        started[0] = 0
        return abi.OK if mode == "success_without_submission" else abi.EXECUTION

    if mode == "commit_failure":
        _inject(monkeypatch, "EXTERNAL_COMMIT")
    worker = abi.EXTERNAL_WORKER(run)
    binding = [(h, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL), abi.REAL64, 1)]
    status, report = _execute(both, scope, binding, worker)
    assert status == report.status == abi.EXECUTION and report.committed == 0 and len(calls) == 1
    assert both.fort_scope_wait(scope.handle) == abi.EXECUTION
    assert both.fort_scope_domain_close_v1(domain) == abi.EXECUTION
    assert both.fort_scope_create_in_domain_v1(domain, c.byref(abi.U64())) == abi.EXECUTION
    status, _ = _execute(both, scope, binding, worker)
    assert status == abi.EXECUTION and len(calls) == 1
    found = abi.U64()
    assert both.fort_scope_domain_get_v1(scope.handle, c.byref(found)) == abi.OK and found.value == domain
    assert both.fort_scope_domain_abandon_v1(domain) == abi.STATE
    assert both.fort_scope_abandon(scope.handle) == abi.OK
    assert both.fort_scope_domain_abandon_v1(domain) == abi.OK
    assert host.tolist() == [1.0, 2.0, 3.0, 4.0]


def test_external_bindings_are_checked_before_the_worker_runs(both):
    scope = abi.Scope(both)
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    log = []
    status, _ = _external(both, scope, h, _worker(log, started=1, result=abi.OK), type_=abi.REAL32)
    assert status == abi.ARGUMENT
    status, _ = _external(both, scope, h, _worker(log, started=1, result=abi.OK), rank=2)
    assert status == abi.ARGUMENT
    assert log == []
    # no bindings: nothing is called
    call = abi.ExternalCall(1, 0, None, 0, 0, 0)
    report = abi.ExternalReport()
    assert both.fort_scope_external_execute_v1(scope.handle, c.byref(call), _worker(log, started=1, result=abi.OK),
                                               None, c.byref(report)) == abi.OK
    assert log == []
    assert both.fort_scope_close(scope.handle) == abi.OK


# ------------------------------------------------------------------------------- identity exchange


def _layout(address, shape, generation=1, lower=None):
    extents = (abi.SIZE * len(shape))(*shape)
    bounds = (c.c_int64 * len(shape))(*(lower or [1] * len(shape)))
    layout = abi.Layout(len(shape), abi.REAL64, 8, address, extents, bounds, generation)
    layout.keep = (extents, bounds)
    return layout


def test_identity_swap_exchanges_names_not_storage(both):
    scope = abi.Scope(both)
    x, xa = _array(np.arange(4.0))
    y, ya = _array(np.arange(4.0) + 10)
    _, hx = scope.register(xa, [4], identity=1001)
    _, hy = scope.register(ya, [4], identity=1002)
    now_x, now_y = abi.U64(), abi.U64()
    status = both.fort_scope_identity_swap_v1(scope.handle, hx, hy, c.byref(_layout(ya, [4])), c.byref(_layout(xa, [4])),
                                              c.byref(now_x), c.byref(now_y))
    assert status == abi.OK
    assert (now_x.value, now_y.value) == (hy, hx)
    # each identity now names the other array: registering it again finds that array's handle
    status, again = scope.register(ya, [4], identity=1001)
    assert (status, again) == (abi.OK, hy)
    assert both.fort_scope_close(scope.handle) == abi.OK


def test_identity_swap_with_a_wrong_layout_poisons(both):
    scope = abi.Scope(both)
    _, xa = _array(np.zeros(4))
    _, ya = _array(np.zeros(4))
    _, hx = scope.register(xa, [4], identity=2001)
    _, hy = scope.register(ya, [4], identity=2002)
    now_x, now_y = abi.U64(), abi.U64()
    # the first layout describes its own array instead of the other one
    status = both.fort_scope_identity_swap_v1(scope.handle, hx, hy, c.byref(_layout(xa, [4])), c.byref(_layout(xa, [4])),
                                              c.byref(now_x), c.byref(now_y))
    assert status == abi.EXECUTION
    assert both.fort_scope_host_begin(scope.handle, hx, c.byref(abi.access(flags=abi.READ_ALL))) == abi.EXECUTION
    both.fort_scope_abandon(scope.handle)


# ------------------------------------------------------------------------------- workspace claims


def test_workspace_claims_count_against_the_budget(both):
    dom = abi.U64()
    assert both.fort_scope_domain_create_v1(0, c.byref(dom)) == abi.OK
    scope = abi.Scope(both, domain=dom.value)
    assert both.fort_scope_set_device_budget(scope.handle, 1 << 20) == abi.OK
    budget, free = abi.SIZE(), abi.SIZE()
    lease = abi.U64()
    assert both.fort_scope_domain_workspace_reserve_v1(dom.value, 4096, c.byref(lease)) == abi.OK
    assert both.fort_scope_domain_budget_get_v1(dom.value, c.byref(budget), c.byref(free)) == abi.OK
    assert (budget.value, free.value) == (1 << 20, (1 << 20) - 4096)
    assert both.fort_scope_domain_workspace_resize_v1(dom.value, lease.value, 1024) == abi.OK
    assert both.fort_scope_domain_budget_get_v1(dom.value, c.byref(budget), c.byref(free)) == abi.OK
    assert free.value == (1 << 20) - 1024
    # a claim beyond the budget fails and changes nothing
    assert both.fort_scope_domain_workspace_resize_v1(dom.value, lease.value, 2 << 20) == abi.RESOURCE
    assert both.fort_scope_domain_budget_get_v1(dom.value, c.byref(budget), c.byref(free)) == abi.OK
    assert free.value == (1 << 20) - 1024
    # an external call may use the lease up to its size
    _, address = _array(np.zeros(4))
    _, h = scope.register(address, [4])
    binding = (abi.ExternalBinding * 1)(abi.ExternalBinding(h, abi.REAL64, 1, 8,
                                                           abi.access(flags=abi.READ_ALL | abi.WRITE_ALL)))
    worker = _worker([], started=1, result=abi.OK)
    report = abi.ExternalReport()
    call = abi.ExternalCall(1, 0, binding, 1, lease.value, 2048)
    assert both.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report)) == \
        abi.RESOURCE
    call = abi.ExternalCall(1, 0, binding, 1, lease.value, 1024)
    assert both.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report)) == abi.OK
    assert both.fort_scope_domain_workspace_release_v1(dom.value, lease.value) == abi.OK
    assert both.fort_scope_domain_workspace_release_v1(dom.value, lease.value) == abi.STALE
    call = abi.ExternalCall(1, 0, binding, 1, lease.value, 0)
    assert both.fort_scope_external_execute_v1(scope.handle, c.byref(call), worker, None, c.byref(report)) == \
        abi.STALE
    assert both.fort_scope_close(scope.handle) == abi.OK
    assert both.fort_scope_domain_close_v1(dom.value) == abi.OK


# ------------------------------------------------------------------------------- checked graph execution


def _scale_kernel(log):
    """dst[i] = 2 * src[i] for i < n; arguments (double *src, double *dst, int n)."""

    def run(args):
        src = _dev(c.cast(args[0], c.POINTER(c.c_void_p))[0], 8)
        dst = _dev(c.cast(args[1], c.POINTER(c.c_void_p))[0], 8)
        n = c.cast(args[2], c.POINTER(c.c_int))[0]
        dst[:n] = 2.0 * src[:n]
        log.append("scale")

    return KERNEL(run)


def _task(fn, values, bindings):
    argv = (c.c_void_p * len(values))(*[c.cast(c.pointer(v), c.c_void_p) for v in values])
    kernel = abi.Kernel(1, 0, c.cast(fn, c.c_void_p), (c.c_uint32 * 3)(1, 1, 1), (c.c_uint32 * 3)(32, 1, 1), 0,
                        argv, len(values))
    packed = (abi.Binding * len(bindings))(*[abi.Binding(h, acc) for h, acc in bindings])
    task = abi.Task(kernel, packed, len(bindings))
    task.keep = (values, argv, bindings, packed)
    return task


def test_graph_group_may_read_what_an_earlier_task_defines(ours):
    scope = abi.Scope(ours)
    x, xa = _array(np.arange(8.0))
    y, ya = _array(np.full(8, -1.0))
    _, hx = scope.register(xa, [8])
    _, hy = scope.register(ya, [8], initialized=False)
    devices = (c.c_void_p * 2)()
    assert ours.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 2)(hx, hy), 2, devices) == abi.OK
    log = []
    scale, axpy = _scale_kernel(log), _axpy_kernel(log)
    produce = _task(scale, [c.c_void_p(devices[0]), c.c_void_p(devices[1]), c.c_int(8)],
                    [(hx, abi.access(flags=abi.READ_ALL)), (hy, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))])
    consume = _task(axpy, [c.c_void_p(devices[1]), c.c_int(8), c.c_double(1.0), c.c_double(1.0)],
                    [(hy, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))])
    group = (abi.Task * 2)(produce, consume)
    before = scope.stats()
    assert ours.fort_scope_graph_execute_v1(scope.handle, 77, group, 2) == abi.OK
    assert log == ["scale", (8, 1.0, 1.0)]
    assert scope.stats().uploads - before.uploads == 1  # x only: y is defined inside the group
    assert ours.fort_scope_host_begin(scope.handle, hy, c.byref(abi.access(flags=abi.READ_ALL))) == abi.OK
    assert y.tolist() == [2.0 * i + 1.0 for i in range(8)]
    assert ours.fort_scope_host_end(scope.handle, hy) == abi.OK
    # in the other order the first task reads y before anything defines it: refused, nothing runs
    log.clear()
    assert ours.fort_scope_forget_definition(scope.handle, hy) == abi.OK
    group = (abi.Task * 2)(consume, produce)
    assert ours.fort_scope_graph_execute_v1(scope.handle, 78, group, 2) == abi.UNINITIALIZED
    assert ours.fort_scope_graph_execute_v1(scope.handle, 0, group, 2) == abi.ARGUMENT
    assert log == []
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_a_checked_group_warms_up_then_replays_its_graph(ours):
    """Under one key the first execution runs the kernels directly, the second instantiates the group's graph,
    later ones copy every node's arguments in again and replay it; another sequence of functions under the key
    replaces the graph (the reference's submit_graph policy, compiler/runtime/scoped_runtime.cu:1046-1078)."""
    scope = abi.Scope(ours)
    x, xa = _array(np.ones(8))
    _, hx = scope.register(xa, [8])
    devices = (c.c_void_p * 1)()
    assert ours.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(hx), 1, devices) == abi.OK
    log = []
    axpy, scale = _axpy_kernel(log), _scale_kernel(log)
    for step in range(4):
        task = _task(axpy, [c.c_void_p(devices[0]), c.c_int(8), c.c_double(2.0), c.c_double(float(step))],
                     [(hx, abi.access(flags=abi.READ_ALL | abi.WRITE_ALL))])
        assert ours.fort_scope_graph_execute_v1(scope.handle, 31, (abi.Task * 1)(task), 1) == abi.OK
    g, q = abi.GraphStats(), abi.QueueStats()
    assert ours.fort_scope_graph_stats_get_v1(scope.handle, c.byref(g)) == abi.OK
    assert ours.fort_scope_graph_queue_stats_get_v1(scope.handle, c.byref(q)) == abi.OK
    assert (g.creations, g.instantiations, g.replays, g.parameter_updates, g.live_graphs) == (1, 1, 2, 2, 1)
    assert q.direct_submissions == 1
    assert [entry[2] for entry in log] == [0.0, 1.0, 2.0, 3.0]      # each replay saw its own arguments
    y, ya = _array(np.zeros(8))
    _, hy = scope.register(ya, [8], initialized=False)
    assert ours.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(hy), 1, devices) == abi.OK
    dy = devices[0]
    assert ours.fort_scope_device_reserve_many_v1(scope.handle, (abi.U64 * 1)(hx), 1, devices) == abi.OK
    other = _task(scale, [c.c_void_p(devices[0]), c.c_void_p(dy), c.c_int(8)],
                  [(hx, abi.access(flags=abi.READ_ALL)), (hy, abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL))])
    for _ in range(2):
        assert ours.fort_scope_graph_execute_v1(scope.handle, 31, (abi.Task * 1)(other), 1) == abi.OK
    assert ours.fort_scope_graph_stats_get_v1(scope.handle, c.byref(g)) == abi.OK
    assert (g.rebuilds, g.creations, g.live_graphs) == (1, 2, 1)
    assert ours.fort_scope_observe_v1(scope.handle, (abi.U64 * 2)(hx, hy), 2) == abi.OK
    want = 1.0
    for step in range(4):
        want = want * 2.0 + step
    assert x.tolist() == [want] * 8 and y.tolist() == [2.0 * want] * 8
    assert ours.fort_scope_close(scope.handle) == abi.OK


def test_slab_pipeline_keeps_coherence_compact(monkeypatch):
    """Ten slabs publish ten interior boxes that merge back into one: no reconciliation is ever needed."""
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    lib = _ours()
    scope = abi.Scope(lib)
    x, xa = _array(np.arange(NX_S * NY_S * NZ_S, dtype=np.float64))
    y, ya = _array(np.zeros(NX_S * NY_S * NZ_S))
    _, hx = scope.register(xa, [NX_S, NY_S, NZ_S])
    _, hy = scope.register(ya, [NX_S, NY_S, NZ_S])
    log = []
    fn = _plane_sum_kernel(log)
    bounds = [(k, k + 1) for k in range(1, 9)]  # one level per slab: eight slabs
    for round_ in range(4):
        status, devices, pipelined = _reserve_slabs(lib, scope, [hx, hy])
        assert status == abi.OK
        tasks, sizes, keep = _slab_tasks(fn, devices, hx, hy, bounds)
        assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, len(bounds), sizes) == abi.OK
        assert lib.fort_scope_observe_v1(scope.handle, (abi.U64 * 1)(hy), 1) == abi.OK
        assert lib.fort_scope_host_begin(scope.handle, hx, c.byref(abi.access(flags=abi.WRITE_ALL))) == abi.OK
        assert lib.fort_scope_host_end(scope.handle, hx) == abi.OK
    p = x.reshape(NZ_S, -1)
    want = np.zeros_like(p)
    want[1:9] = p[0:8] + p[1:9] + p[2:10]
    assert np.array_equal(y, want.ravel())
    assert scope.stats().reconciliations == 0
    assert lib.fort_scope_close(scope.handle) == abi.OK


# ------------------------------------------------------------------------------- numerical contract


def test_numerics_contract_per_context(ours):
    """The strict contract is every context's default; a context can switch to fast-fp and back, unknown
    contracts and null outputs are argument errors, and a closed context is stale (extension: the reference
    fixes the contract when its entries are compiled, compiler/resident/build.py:22,66-67)."""
    a, b = abi.Scope(ours), abi.Scope(ours)
    got = c.c_int(-1)
    assert ours.fort_scope_numerics_get_v1(a.handle, c.byref(got)) == abi.OK
    assert got.value == abi.NUMERICS_STRICT
    assert ours.fort_scope_numerics_set_v1(a.handle, abi.NUMERICS_FAST) == abi.OK
    assert ours.fort_scope_numerics_get_v1(a.handle, c.byref(got)) == abi.OK and got.value == abi.NUMERICS_FAST
    # the other context keeps its own contract
    assert ours.fort_scope_numerics_get_v1(b.handle, c.byref(got)) == abi.OK and got.value == abi.NUMERICS_STRICT
    assert ours.fort_scope_numerics_set_v1(a.handle, 2) == abi.ARGUMENT
    assert ours.fort_scope_numerics_set_v1(a.handle, -1) == abi.ARGUMENT
    assert ours.fort_scope_numerics_get_v1(a.handle, None) == abi.ARGUMENT
    assert ours.fort_scope_numerics_get_v1(a.handle, c.byref(got)) == abi.OK and got.value == abi.NUMERICS_FAST
    assert ours.fort_scope_numerics_set_v1(a.handle, abi.NUMERICS_STRICT) == abi.OK
    assert ours.fort_scope_close(b.handle) == abi.OK
    assert ours.fort_scope_numerics_set_v1(b.handle, abi.NUMERICS_FAST) == abi.STALE
    assert ours.fort_scope_numerics_get_v1(12345, c.byref(got)) == abi.ARGUMENT


def test_slab_timing_reports_the_last_sequence(monkeypatch):
    """Timing of slab sequences is off by default (nothing to report: FORT_SCOPE_STATE); once enabled, the last
    sequence's slab count is reported with its intervals (zero on the synchronous CPU backend); disabling drops it."""
    monkeypatch.setenv("F2C_TEST_MAPPED", "1")
    lib = _ours()
    scope = abi.Scope(lib)
    x, xa = _array(np.arange(NX_S * NY_S * NZ_S, dtype=np.float64))
    y, ya = _array(np.zeros(NX_S * NY_S * NZ_S))
    _, hx = scope.register(xa, [NX_S, NY_S, NZ_S])
    _, hy = scope.register(ya, [NX_S, NY_S, NZ_S])
    fn = _plane_sum_kernel([])
    timing = abi.SlabTiming()
    assert lib.fort_scope_slab_timing_get_v1(scope.handle, c.byref(timing)) == abi.STATE
    assert lib.fort_scope_slab_timing_get_v1(scope.handle, None) == abi.ARGUMENT
    assert lib.fort_scope_slab_timing_set_v1(scope.handle, 1) == abi.OK
    for bounds in ([(1, 4), (4, 7), (7, 9)], [(1, 5), (5, 9)]):
        status, devices, _ = _reserve_slabs(lib, scope, [hx, hy])
        assert status == abi.OK
        tasks, sizes, keep = _slab_tasks(fn, devices, hx, hy, bounds)
        assert lib.fort_scope_slab_enqueue_v1(scope.handle, 11, tasks, len(bounds), sizes) == abi.OK
        assert lib.fort_scope_slab_timing_get_v1(scope.handle, c.byref(timing)) == abi.OK
        assert (timing.version, timing.slabs) == (1, len(bounds))
        assert timing.span_ms >= 0.0 and timing.kernel_ms >= 0.0
    assert lib.fort_scope_slab_timing_set_v1(scope.handle, 0) == abi.OK
    assert lib.fort_scope_slab_timing_get_v1(scope.handle, c.byref(timing)) == abi.STATE
    assert lib.fort_scope_close(scope.handle) == abi.OK
    assert lib.fort_scope_slab_timing_set_v1(scope.handle, 1) == abi.STALE
