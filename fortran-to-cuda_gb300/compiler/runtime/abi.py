"""ctypes mirrors of the fort_scope_* records and entry points (include/scoped_runtime.h)."""

from __future__ import annotations

import ctypes as c

SIZE = c.c_size_t
U64 = c.c_uint64

OK, ARGUMENT, STALE, ALIAS, RESOURCE, BOUNDARY, EXECUTION, UNINITIALIZED, STATE, DECLINED = range(10)
BYTES, REAL32, REAL64, INTEGER32, LOGICAL = range(5)
READ_ALL, WRITE_ALL, OVERWRITE_ALL = 1, 2, 4
NATIVE, GPU = 0, 1
NUMERICS_STRICT, NUMERICS_FAST = 0, 1


class SlabTiming(c.Structure):
    _fields_ = [("version", c.c_uint32), ("slabs", c.c_uint32), ("span_ms", c.c_double), ("upload_ms", c.c_double),
                ("kernel_ms", c.c_double), ("publish_ms", c.c_double), ("longest_upload_ms", c.c_double),
                ("longest_kernel_ms", c.c_double), ("longest_publish_ms", c.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "version"}


class Section(c.Structure):
    _fields_ = [("lower", c.POINTER(SIZE)), ("upper", c.POINTER(SIZE))]


class Access(c.Structure):
    _fields_ = [("flags", c.c_uint32), ("read_count", SIZE), ("reads", c.POINTER(Section)),
                ("write_count", SIZE), ("writes", c.POINTER(Section)),
                ("overwrite_count", SIZE), ("overwrites", c.POINTER(Section))]


class Layout(c.Structure):
    _fields_ = [("rank", c.c_uint32), ("type", c.c_uint32), ("element_bytes", SIZE), ("host", c.c_void_p),
                ("extents", c.POINTER(SIZE)), ("lower_bounds", c.POINTER(c.c_int64)), ("generation", U64)]


class Stats(c.Structure):
    _fields_ = [(n, U64) for n in ("uploads", "downloads", "upload_bytes", "download_bytes", "allocations",
                                   "allocated_bytes", "peak_device_bytes", "launches", "waits", "reconciliations")]


class Binding(c.Structure):
    _fields_ = [("buffer", U64), ("access", Access)]


class Kernel(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32), ("function", c.c_void_p),
                ("grid", c.c_uint32 * 3), ("block", c.c_uint32 * 3), ("shared_bytes", SIZE),
                ("arguments", c.POINTER(c.c_void_p)), ("argument_count", SIZE)]


class Task(c.Structure):
    _fields_ = [("kernel", Kernel), ("bindings", c.POINTER(Binding)), ("binding_count", SIZE)]


class Member(c.Structure):
    _fields_ = [("bindings", c.POINTER(Binding)), ("binding_count", SIZE)]


class GraphStats(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32)] + [
        (n, U64) for n in ("creations", "instantiations", "rebuilds", "submissions", "replays", "parameter_updates",
                           "logical_kernels", "live_graphs", "destructions")]


class CompletionStats(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32)] + [
        (n, U64) for n in ("event_records", "event_queries", "event_waits", "stream_waits", "created_events",
                           "reused_events", "independent_host_tasks")]


class QueueStats(c.Structure):
    _fields_ = [("version", c.c_uint32), ("queue_enabled", c.c_uint32), ("graphs_enabled", c.c_uint32),
                ("reserved", c.c_uint32)] + [
        (n, U64) for n in ("accepted_tasks", "submissions", "conflict_flushes", "explicit_flushes", "pending_tasks",
                           "peak_pending_tasks", "copied_argument_bytes", "direct_submissions", "direct_kernels",
                           "graph_resource_fallbacks")]


class ResidencyStats(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32)] + [
        (n, U64) for n in ("reserve_batches", "requested_resources", "reuse_hits", "evictions", "evicted_bytes",
                           "dirty_evictions", "dirty_download_bytes", "pressure_flushes")]


class ScratchLease(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32), ("token", U64), ("device", c.c_void_p),
                ("bytes", SIZE), ("capacity", SIZE)]


class ScratchStats(c.Structure):
    _fields_ = [("version", c.c_uint32), ("active", c.c_uint32)] + [
        (n, U64) for n in ("acquisitions", "allocations", "reuses", "releases", "grows", "capacity_bytes",
                           "active_bytes", "peak_scratch_bytes", "peak_total_device_bytes")]


class TraceState(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32)] + [
        (n, c.c_char * 65) for n in ("owner", "procedure", "segment", "operation", "implementation", "boundary")]


class ExternalBinding(c.Structure):
    _fields_ = [("buffer", U64), ("type", c.c_uint32), ("rank", c.c_uint32), ("element_bytes", SIZE),
                ("access", Access)]


class ExternalView(c.Structure):
    _fields_ = [("buffer", U64), ("generation", U64), ("type", c.c_uint32), ("rank", c.c_uint32),
                ("element_bytes", SIZE), ("bytes", SIZE), ("extents", c.POINTER(SIZE)), ("strides", c.POINTER(SIZE)),
                ("lower_bounds", c.POINTER(c.c_int64)), ("device", c.c_void_p)]


class ExternalCall(c.Structure):
    _fields_ = [("version", c.c_uint32), ("reserved", c.c_uint32), ("bindings", c.POINTER(ExternalBinding)),
                ("binding_count", SIZE), ("workspace_lease", U64), ("workspace_bytes", SIZE)]


class ExternalReport(c.Structure):
    _fields_ = [("version", c.c_uint32), ("status", c.c_int32), ("started", c.c_uint32), ("committed", c.c_uint32)]


# int worker(void *user, const fort_scope_external_view_v1 *views, size_t count, void *stream, int *started)
EXTERNAL_WORKER = c.CFUNCTYPE(c.c_int, c.c_void_p, c.POINTER(ExternalView), SIZE, c.c_void_p, c.POINTER(c.c_int))

P = c.POINTER
SIGNATURES = {
    "abi_version": ([], c.c_uint32),
    "error": ([], c.c_char_p),
    "report_error": ([c.c_int, c.c_char_p], c.c_int),
    "execution_error": ([U64, c.c_char_p], c.c_int),
    "trace_set_v1": ([U64, c.c_uint32] + [c.c_char_p] * 6 + [P(TraceState)], None),
    "trace_restore_v1": ([U64, P(TraceState)], None),
    "create": ([c.c_int, P(U64)], c.c_int),
    "domain_create_v1": ([c.c_int, P(U64)], c.c_int),
    "create_in_domain_v1": ([U64, P(U64)], c.c_int),
    "domain_get_v1": ([U64, P(U64)], c.c_int),
    "domain_device_get_v1": ([U64, P(c.c_int)], c.c_int),
    "domain_stats_get_v1": ([U64, P(Stats)], c.c_int),
    "domain_close_v1": ([U64], c.c_int),
    "domain_abandon_v1": ([U64], c.c_int),
    "set_device_budget": ([U64, SIZE], c.c_int),
    "device_budget_default_v1": ([c.c_int, P(SIZE)], c.c_int),
    "domain_budget_get_v1": ([U64, P(SIZE), P(SIZE)], c.c_int),
    "close": ([U64], c.c_int),
    "abandon": ([U64], c.c_int),
    "wait": ([U64], c.c_int),
    "register": ([U64, U64, U64, P(Layout), c.c_int, P(U64)], c.c_int),
    "register_sections": ([U64, U64, U64, P(Layout), P(Section), SIZE, P(U64)], c.c_int),
    "admit_source_reads_v1": ([U64, U64, P(Section), SIZE], c.c_int),
    "forget_definition": ([U64, U64], c.c_int),
    "layout_get": ([U64, U64, P(Layout)], c.c_int),
    "buffer_valid_v1": ([U64, U64, P(c.c_int)], c.c_int),
    "access_begin_v1": ([U64, P(Binding), SIZE, c.c_int, P(c.c_void_p)], c.c_int),
    "host_begin": ([U64, U64, P(Access)], c.c_int),
    "host_end": ([U64, U64], c.c_int),
    "device_begin": ([U64, U64, P(Access), P(c.c_void_p)], c.c_int),
    "device_end": ([U64, U64], c.c_int),
    "cancel_access": ([U64, U64], c.c_int),
    "device_reserve_v1": ([U64, U64, P(c.c_void_p)], c.c_int),
    "device_reserve_many_v1": ([U64, P(U64), SIZE, P(c.c_void_p)], c.c_int),
    "observe_v1": ([U64, P(U64), SIZE], c.c_int),
    "observe_all_v1": ([U64], c.c_int),
    "discard_v1": ([U64, U64], c.c_int),
    "recycle_v1": ([U64, U64], c.c_int),
    "retire_v1": ([U64, U64], c.c_int),
    "unregister": ([U64, U64], c.c_int),
    "stats_get": ([U64, P(Stats)], c.c_int),
    "residency_stats_get_v1": ([U64, P(ResidencyStats)], c.c_int),
    "scratch_acquire_v1": ([U64, SIZE, P(ScratchLease)], c.c_int),
    "scratch_release_v1": ([U64, U64], c.c_int),
    "scratch_stats_get_v1": ([U64, P(ScratchStats)], c.c_int),
    "gpu_enter": ([U64, P(c.c_int), P(c.c_void_p)], c.c_int),
    "gpu_leave": ([U64, c.c_int], c.c_int),
    "note_launch": ([U64], c.c_int),
    "graph_enqueue_v1": ([U64, U64, P(Task), P(SIZE)], c.c_int),
    "graph_enqueue_members_v1": ([U64, U64, P(Kernel), P(SIZE), P(Member), SIZE], c.c_int),
    "graph_flush_v1": ([U64], c.c_int),
    "graph_queue_cancel_v1": ([U64], c.c_int),
    "graph_queue_stats_get_v1": ([U64, P(QueueStats)], c.c_int),
    "graph_stats_get_v1": ([U64, P(GraphStats)], c.c_int),
    "completion_stats_get_v1": ([U64, P(CompletionStats)], c.c_int),
    "graph_execute_v1": ([U64, U64, P(Task), SIZE], c.c_int),
    "graph_submit_v1": ([U64, U64, P(Kernel), SIZE], c.c_int),
    "device_reserve_slabs_v1": ([U64, P(U64), SIZE, P(c.c_void_p), P(c.c_int)], c.c_int),
    "slab_enqueue_v1": ([U64, U64, P(Task), SIZE, P(SIZE)], c.c_int),
    "numerics_set_v1": ([U64, c.c_int], c.c_int),
    "host_pinning_set_v1": ([U64, c.c_int], c.c_int),
    "slab_timing_set_v1": ([U64, c.c_int], c.c_int),
    "slab_timing_get_v1": ([U64, P(SlabTiming)], c.c_int),
    "numerics_get_v1": ([U64, P(c.c_int)], c.c_int),
    "domain_workspace_reserve_v1": ([U64, SIZE, P(U64)], c.c_int),
    "domain_workspace_resize_v1": ([U64, U64, SIZE], c.c_int),
    "domain_workspace_release_v1": ([U64, U64], c.c_int),
    "identity_swap_v1": ([U64, U64, U64, P(Layout), P(Layout), P(U64), P(U64)], c.c_int),
    "external_execute_v1": ([U64, P(ExternalCall), EXTERNAL_WORKER, c.c_void_p, P(ExternalReport)], c.c_int),
}


def bind(lib):
    """Declare argument and result types of every fort_scope_* entry point the library exports."""
    for name, (args, result) in SIGNATURES.items():
        fn = getattr(lib, "fort_scope_" + name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = result
    return lib


def access(*, read=(), write=(), overwrite=(), flags=0) -> Access:
    """An access record; boxes are (lower, upper) coordinate tuples. Keeps its storage alive."""
    result = Access(flags=flags)
    result.keep = []
    for label, boxes in (("read", read), ("write", write), ("overwrite", overwrite)):
        sections = []
        for lo, hi in boxes:
            lower, upper = (SIZE * len(lo))(*lo), (SIZE * len(hi))(*hi)
            result.keep.extend([lower, upper])
            sections.append(Section(lower, upper))
        packed = (Section * max(1, len(sections)))(*sections)
        result.keep.append(packed)
        setattr(result, label + "s", packed if sections else None)
        setattr(result, label + "_count", len(sections))
    return result


class RuntimeError_(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"fort_scope status {status}: {message}")
        self.status = status


class Scope:
    """A context over one library (private domain unless ``domain`` is given)."""

    def __init__(self, lib, device=0, domain=None):
        self.lib = lib
        self.handle = U64()
        self.keep = []
        if domain is None:
            self.check(lib.fort_scope_create(device, c.byref(self.handle)))
        else:
            self.check(lib.fort_scope_create_in_domain_v1(domain, c.byref(self.handle)))

    def check(self, status):
        if status != OK:
            raise RuntimeError_(status, self.lib.fort_scope_error().decode(errors="replace"))
        return status

    def register(self, address, shape, *, identity=None, generation=1, initialized=True, lower=None,
                 type_=REAL64, element_bytes=8, defined=None):
        extents = (SIZE * len(shape))(*shape)
        bounds = (c.c_int64 * len(shape))(*(lower or [1] * len(shape)))
        layout = Layout(len(shape), type_, element_bytes, address, extents, bounds, generation)
        self.keep.extend([extents, bounds, layout])
        out = U64()
        if defined is None:
            status = self.lib.fort_scope_register(self.handle, identity or address, generation, c.byref(layout),
                                                  1 if initialized else 0, c.byref(out))
        else:
            eff = access(read=defined)
            self.keep.append(eff)
            status = self.lib.fort_scope_register_sections(self.handle, identity or address, generation,
                                                           c.byref(layout), eff.reads, eff.read_count, c.byref(out))
        return status, out.value

    def stats(self) -> Stats:
        s = Stats()
        self.check(self.lib.fort_scope_stats_get(self.handle, c.byref(s)))
        return s
