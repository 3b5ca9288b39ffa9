"""A residency domain driven from Python, with the semantics of the Fortran ``resident_domain``.

Follows compiler/runtime/resident_domain.f90 of the reference:
``begin_epoch`` (:162-187) creates the domain and its context on first use with
the default budget (``fort_scope_device_budget_default_v1``) and advances the
generation; ``bind_real64`` (:429-457, ``register_storage`` :265-363)
registers an array by the address of its first element, its extents and lower
bounds, returning the handle already held for that address inside the epoch;
``observe`` (:525) publishes; ``publish`` (:898-926) observes every handle and
unregisters it; ``end_epoch`` (:928-940) publishes and ends the epoch;
``close`` (:942-976) closes the context and the domain. A nonzero status
raises, as ``resident_require`` error-stops (:108-137).
"""

from __future__ import annotations

import ctypes as c

import numpy as np

from ..runtime import abi


class ResidentError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"Resident runtime failed: status {status}: {message}; source work will not be replayed")
        self.status = status


class ResidentDomain:
    def __init__(self, lib, fast_fp: bool = False):
        self.lib = lib
        self.fast_fp = fast_fp  # the context runs the fast-fp kernels (a resident build prepared with --fast-fp)
        self.domain = 0
        self.context = 0
        self.generation = 0
        self.active = False
        self._storage = {}  # address -> (handle, extents, persistent)
        self._keep = []

    def require(self, status: int) -> None:
        if status != abi.OK:
            raise ResidentError(status, self.lib.fort_scope_error().decode(errors="replace"))

    def begin_epoch(self, device: int = 0, budget: int | None = None) -> None:
        if self.active:
            raise ResidentError(abi.STATE, "nested storage epoch")
        if not self.domain:
            if budget is None:
                out = c.c_size_t()
                self.require(self.lib.fort_scope_device_budget_default_v1(device, c.byref(out)))
                budget = out.value
            dom, ctx = abi.U64(), abi.U64()
            self.require(self.lib.fort_scope_domain_create_v1(device, c.byref(dom)))
            self.require(self.lib.fort_scope_create_in_domain_v1(dom.value, c.byref(ctx)))
            self.require(self.lib.fort_scope_set_device_budget(ctx.value, budget))
            if self.fast_fp:
                self.require(self.lib.fort_scope_numerics_set_v1(ctx.value, abi.NUMERICS_FAST))
            self.domain, self.context = dom.value, ctx.value
        self.generation += 1
        self.active = True

    def bind_real64(self, array: np.ndarray, initialized: bool = True, persistent: bool = False,
                    lower=None) -> int:
        """Register a float64 array given as numpy (C order == Fortran column-major of the reversed shape)."""
        if not self.active:
            raise ResidentError(abi.STATE, "registration outside a storage epoch")
        if array.dtype != np.float64 or not array.flags.c_contiguous or array.size == 0:
            raise ResidentError(abi.ARGUMENT, "a kept array must be a non-empty contiguous float64 array")
        address = array.ctypes.data
        extents = tuple(reversed(array.shape))
        held = self._storage.get(address)
        if held is not None:
            if held[1] != extents:
                raise ResidentError(abi.ALIAS, "storage shape changed inside an epoch")
            return held[0]
        ext = (abi.SIZE * len(extents))(*extents)
        low = (c.c_int64 * len(extents))(*(lower or [1] * len(extents)))
        layout = abi.Layout(len(extents), abi.REAL64, 8, address, ext, low, 1 if persistent else self.generation)
        out = abi.U64()
        self.require(self.lib.fort_scope_register(self.context, address, layout.generation, c.byref(layout),
                                                  1 if initialized else 0, c.byref(out)))
        self._storage[address] = (out.value, extents, persistent)
        self._keep.append(array)
        return out.value

    def held(self, array: np.ndarray) -> int:
        entry = self._storage.get(array.ctypes.data)
        return entry[0] if entry else 0

    def observe(self, handles) -> None:
        handles = [h for h in dict.fromkeys(handles) if h]
        if not handles:
            return
        arr = (abi.U64 * len(handles))(*handles)
        self.require(self.lib.fort_scope_observe_v1(self.context, arr, len(handles)))

    def host_modify(self, handles) -> None:
        """Declare that host code rewrites these arrays entirely (their device copies become stale)."""
        for h in handles:
            acc = abi.access(flags=abi.WRITE_ALL | abi.OVERWRITE_ALL)
            self.require(self.lib.fort_scope_host_begin(self.context, h, c.byref(acc)))
            self.require(self.lib.fort_scope_host_end(self.context, h))

    def publish(self) -> None:
        handles = [h for (h, _, persistent) in self._storage.values() if not persistent]
        self.observe(handles)
        for address, (h, _, persistent) in list(self._storage.items()):
            if persistent:
                continue
            self.require(self.lib.fort_scope_unregister(self.context, h))
            del self._storage[address]
        self._keep = [a for a in self._keep if a.ctypes.data in self._storage]

    def end_epoch(self) -> None:
        if not self.active:
            raise ResidentError(abi.STATE, "no storage epoch to end")
        self.publish()
        self.active = False

    def close(self) -> None:
        if self.active:
            self.end_epoch()
        if self.context:
            self.require(self.lib.fort_scope_close(self.context))
            self.require(self.lib.fort_scope_domain_close_v1(self.domain))
        self.context = self.domain = 0
        self._storage.clear()
        self._keep.clear()

    def stats(self) -> abi.Stats:
        s = abi.Stats()
        self.require(self.lib.fort_scope_stats_get(self.context, c.byref(s)))
        return s

    def graph_stats(self) -> abi.GraphStats:
        s = abi.GraphStats()
        self.require(self.lib.fort_scope_graph_stats_get_v1(self.context, c.byref(s)))
        return s
