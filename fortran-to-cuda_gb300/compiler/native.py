"""Build and load the native library ``libf2c_gb300.so`` (sm_103a kernels + residency runtime).

The library is compiled in-tree with nvcc for ``sm_103a`` only, under the
reference's strict numerical contract (``--fmad=false --ftz=false
--prec-div=true --prec-sqrt=true`` and ``-ffp-contract=off`` for host code,
compiler/emission/numerical_contract.py:13-15), so the kernels round exactly
like the Fortran control. There is no CPU fallback: loading fails loudly when
the library cannot be built or found.
"""

from __future__ import annotations

import ctypes
import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from functools import lru_cache
from pathlib import Path

PACKAGE_ROOT = Path(__file__).resolve().parent.parent
CSRC = PACKAGE_ROOT / "csrc"
REPO_ROOT = PACKAGE_ROOT.parent
INCLUDE = REPO_ROOT / "include"
BUILD_DIR = PACKAGE_ROOT / "_build"
LIBRARY = BUILD_DIR / "libf2c_gb300.so"

ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")
STRICT_CUDA = ("--fmad=false", "--ftz=false", "--prec-div=true", "--prec-sqrt=true")
HOST_OPTIONS = ("-fPIC", "-ffp-contract=off", "-fopenmp")
NVCC_FLAGS = ("-O3", "-std=c++17", "-lineinfo", *ARCH, *STRICT_CUDA, "-Xcompiler", ",".join(HOST_OPTIONS),
              f"-I{INCLUDE}", f"-I{CSRC}")


def nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(found).exists():
        raise RuntimeError("nvcc not found: the GB300 library cannot be built")
    return found


PROBE_DIR = CSRC / "probes"
PROBE_LIBRARY = BUILD_DIR / "libf2c_probe.so"


def sources() -> list[Path]:
    """Every translation unit of the library (kernels, runtime, generated entries); measurement probes apart."""
    found = sorted(CSRC.rglob("*.cu")) + sorted(CSRC.rglob("*.cpp"))
    return [p for p in found if "_build" not in p.parts and PROBE_DIR not in p.parents]


def _headers() -> list[Path]:
    return sorted(CSRC.rglob("*.cuh")) + sorted(CSRC.rglob("*.hpp")) + sorted(CSRC.rglob("*.h")) + \
        sorted(INCLUDE.glob("*.h"))


LINK_TAG = "link:-Bsymbolic"


def _fingerprint(files) -> str:
    digest = hashlib.sha256(LINK_TAG.encode())
    for flag in NVCC_FLAGS:
        digest.update(flag.encode())
    for path in files:
        digest.update(str(path.relative_to(REPO_ROOT)).encode())
        digest.update(path.read_bytes())
    return digest.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every source in parallel and link ``libf2c_gb300.so``; skip when up to date."""
    from . import emission  # the generated entries are part of the library

    emission.write_entries()
    srcs = sources()
    stamp = BUILD_DIR / "fingerprint"
    fingerprint = _fingerprint([*srcs, *_headers()])
    if not force and LIBRARY.exists() and stamp.exists() and stamp.read_text() == fingerprint:
        return LIBRARY
    BUILD_DIR.mkdir(exist_ok=True)
    compiler = nvcc()

    def compile_one(src: Path) -> Path:
        rel = src.relative_to(CSRC)
        obj = BUILD_DIR / (str(rel).replace(os.sep, "__") + ".o")
        cmd = [compiler, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd[1:1] = ["-x", "cu"]
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"nvcc failed on {rel}:\n{result.stdout}\n{result.stderr}")
        if verbose and result.stderr:
            print(result.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as pool:
        objects = list(pool.map(compile_one, srcs))
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    link = [compiler, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-Xlinker", "-Bsymbolic", *map(str, objects),
            "-o", str(tmp), "-lcudart"]
    result = subprocess.run(link, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stdout}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    stamp.write_text(fingerprint)
    return LIBRARY


def build_probe(force: bool = False) -> Path:
    """The benchmark's measurement probes (the live FP64 rate), a library of their own beside the product."""
    srcs = sorted(PROBE_DIR.glob("*.cu"))
    stamp = BUILD_DIR / "probe.fingerprint"
    fingerprint = _fingerprint(srcs)
    if not force and PROBE_LIBRARY.exists() and stamp.exists() and stamp.read_text() == fingerprint:
        return PROBE_LIBRARY
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = PROBE_LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    cmd = [nvcc(), *NVCC_FLAGS, "-shared", "-Xcompiler", "-fPIC", *map(str, srcs), "-o", str(tmp), "-lcudart"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"probe build failed:\n{result.stdout}\n{result.stderr}")
    os.replace(tmp, PROBE_LIBRARY)
    stamp.write_text(fingerprint)
    return PROBE_LIBRARY


@lru_cache(maxsize=1)
def probe() -> ctypes.CDLL:
    """The measurement probe library (not part of the product path)."""
    lib = ctypes.CDLL(str(PROBE_LIBRARY if PROBE_LIBRARY.exists() else build_probe()))
    lib.f2c_fp64_rate_v1.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double)]
    lib.f2c_fp64_rate_v1.restype = ctypes.c_int
    return lib


def runtime() -> ctypes.CDLL:
    """The product library with the fort_scope_* signatures declared."""
    from .runtime import abi

    return abi.bind(load())


CPU_RUNTIME = BUILD_DIR / "libf2c_runtime_cpu.so"
RUNTIME_SOURCE = CSRC / "runtime" / "scoped_runtime.cpp"


def build_cpu_runtime(force: bool = False) -> Path:
    """The residency runtime built with its CPU test backend (g++, no CUDA): for ABI tests without a GPU."""
    deps = [RUNTIME_SOURCE, *sorted((CSRC / "runtime").glob("*.hpp")), INCLUDE / "scoped_runtime.h"]
    if not force and CPU_RUNTIME.exists() and all(CPU_RUNTIME.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return CPU_RUNTIME
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = CPU_RUNTIME.with_suffix(f".{os.getpid()}.tmp")
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-fPIC", "-shared", "-pthread",
           "-Wl,-Bsymbolic", "-DF2C_RUNTIME_CPU_BACKEND", "-x", "c++", str(RUNTIME_SOURCE), "-o", str(tmp)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"CPU runtime build failed:\n{result.stderr}")
    os.replace(tmp, CPU_RUNTIME)
    return CPU_RUNTIME


# --- ctypes mirrors of include/f2c_advection.h -------------------------------------------------

MAX_SCALARS = 4


class Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int64), ("ny", ctypes.c_int64), ("nz", ctypes.c_int64),
                ("halo", ctypes.c_int64), ("sx", ctypes.c_int64), ("sy", ctypes.c_int64),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double)]


class Fields(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("w", ctypes.c_void_p),
                ("ut", ctypes.c_void_p), ("vt", ctypes.c_void_p), ("wt", ctypes.c_void_p),
                ("nscalar", ctypes.c_int32), ("mode", ctypes.c_int32), ("dt", ctypes.c_double),
                ("s", ctypes.c_void_p * MAX_SCALARS), ("st", ctypes.c_void_p * MAX_SCALARS)]


TENDENCY, ADVANCE, ADVANCE_FILLED = 0, 1, 2


BATCH_HALO_OK, BATCH_FAST_FP = 1, 2  # f2c_batch_plan_v1.reserved flags


class BatchPlan(ctypes.Structure):
    _fields_ = [("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t), ("count", ctypes.c_int32),
                ("nscalar", ctypes.c_int32), ("mask", ctypes.c_int32), ("items", ctypes.c_int32),
                ("ctas", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class ServeOptions(ctypes.Structure):
    _fields_ = [("version", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("max_active", ctypes.c_uint32),
                ("depth", ctypes.c_uint32), ("budget_bytes", ctypes.c_uint64), ("reserve_bytes", ctypes.c_uint64),
                ("tick_points", ctypes.c_uint64), ("burst_points", ctypes.c_uint64), ("starve_s", ctypes.c_double)]


class ServeJob(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int64), ("ny", ctypes.c_int64), ("nz", ctypes.c_int64), ("halo", ctypes.c_int64),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
                ("nscalar", ctypes.c_int32), ("steps", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("arrival", ctypes.c_double), ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class ServeDone(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("arrival", ctypes.c_double), ("admitted", ctypes.c_double),
                ("finished", ctypes.c_double), ("status", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class ServeStats(ctypes.Structure):
    _fields_ = [("version", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                *[(n, ctypes.c_uint64) for n in ("admitted", "finished", "ticks", "bursts", "graph_builds",
                                                  "graph_replays", "direct_launches", "plan_builds",
                                                  "refused_admissions", "peak_active", "peak_job_bytes")],
                ("idle_s", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name not in ("version", "reserved")}


SERVE_ABI_VERSION = 1
SERVE_DIRECT = 1        # f2c_serve_options_v1.flags
SERVE_KEEP_RESULT = 1   # f2c_serve_job_v1.flags


@lru_cache(maxsize=1)
def load() -> ctypes.CDLL:
    """Load the native library (building it first if needed). Raises if it cannot be had."""
    path = LIBRARY if LIBRARY.exists() else build()
    lib = ctypes.CDLL(str(path))
    lib.f2c_advection_abi_version.restype = ctypes.c_uint32
    lib.f2c_last_error.restype = ctypes.c_char_p
    lib.f2c_advection_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(Fields), ctypes.c_void_p]
    lib.f2c_advection_v1.restype = ctypes.c_int
    lib.f2c_advection_variant_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(Fields), ctypes.c_int,
                                             ctypes.c_void_p]
    lib.f2c_advection_variant_v1.restype = ctypes.c_int
    lib.f2c_halo_fill_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_void_p]
    lib.f2c_halo_fill_v1.restype = ctypes.c_int
    lib.f2c_batch_workspace_bytes_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]
    lib.f2c_batch_workspace_bytes_v1.restype = ctypes.c_size_t
    lib.f2c_batch_prepare_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(Fields), ctypes.POINTER(ctypes.c_int32),
                                         ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                         ctypes.POINTER(BatchPlan)]
    lib.f2c_batch_prepare_v1.restype = ctypes.c_int
    lib.f2c_batch_step_v1.argtypes = [ctypes.POINTER(BatchPlan), ctypes.c_void_p]
    lib.f2c_batch_step_v1.restype = ctypes.c_int
    lib.f2c_batch_prepare_async_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(Fields),
                                               ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_void_p,
                                               ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(BatchPlan)]
    lib.f2c_batch_prepare_async_v1.restype = ctypes.c_int
    lib.f2c_batch_workspace_bytes_rows_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(ctypes.c_int32),
                                                      ctypes.c_int32, ctypes.c_int32]
    lib.f2c_batch_workspace_bytes_rows_v1.restype = ctypes.c_size_t
    lib.f2c_batch_prepare_rows_v1.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(Fields),
                                              ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_int32,
                                              ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.POINTER(BatchPlan)]
    lib.f2c_batch_prepare_rows_v1.restype = ctypes.c_int
    lib.f2c_batch_graph_create_v1.argtypes = [ctypes.POINTER(BatchPlan), ctypes.POINTER(ctypes.c_void_p)]
    lib.f2c_batch_graph_create_v1.restype = ctypes.c_int
    lib.f2c_batch_graph_launch_v1.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.f2c_batch_graph_launch_v1.restype = ctypes.c_int
    lib.f2c_batch_graph_destroy_v1.argtypes = [ctypes.c_void_p]
    lib.f2c_batch_graph_destroy_v1.restype = ctypes.c_int
    lib.f2c_batch_halo_v1.argtypes = [ctypes.POINTER(BatchPlan), ctypes.c_void_p]
    lib.f2c_batch_halo_v1.restype = ctypes.c_int
    lib.f2c_procedure_v1.argtypes = [ctypes.c_int, ctypes.POINTER(Grid), ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
    lib.f2c_procedure_v1.restype = ctypes.c_int
    lib.f2c_seed_fields_v1.argtypes = [ctypes.POINTER(Grid), ctypes.c_uint64, ctypes.c_int32,
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
    lib.f2c_seed_fields_v1.restype = ctypes.c_int
    u64 = ctypes.c_uint64
    for name, args in (("create", [u64, ctypes.POINTER(ServeOptions), ctypes.POINTER(u64)]),
                       ("submit", [u64, ctypes.POINTER(ServeJob), ctypes.POINTER(u64)]),
                       ("poll", [u64, ctypes.POINTER(ServeDone), ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
                       ("drain", [u64, ctypes.c_double]),
                       ("result", [u64, u64, ctypes.c_int32, ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]),
                       ("release", [u64, u64]),
                       ("stats_get", [u64, ctypes.POINTER(ServeStats)]),
                       ("destroy", [u64])):
        fn = getattr(lib, f"f2c_serve_{name}_v1")
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.f2c_serve_clock_v1.argtypes = [u64]
    lib.f2c_serve_clock_v1.restype = ctypes.c_double
    lib.f2c_serve_error_v1.argtypes = [u64]
    lib.f2c_serve_error_v1.restype = ctypes.c_char_p
    return lib


class NativeError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"status {status}: {message}")
        self.status = status


def check(status: int) -> None:
    if status != 0:
        raise NativeError(status, load().f2c_last_error().decode(errors="replace"))


def make_grid(nx, ny, nz, halo, dx, dy, dz, sx=None, sy=None) -> Grid:
    return Grid(nx, ny, nz, halo, sx or nx + 2 * halo, sy or ny + 2 * halo, dx, dy, dz)


FACES, DIRECT, FAST = 0, 1, 2  # enum f2c_kernel_variant


def advection(grid: Grid, u, v, w, ut=None, vt=None, wt=None, scalars=(), scalar_out=(), mode=TENDENCY,
              dt=0.0, stream=0, variant=FACES) -> None:
    """Enqueue the fused advection launch on device pointers (ints).

    ``variant`` FACES is the face-sharing kernel (the strict, bit-exact product
    path); DIRECT is the straightforward per-point kernel kept as a cross-check;
    FAST is the fast-fp kernel (FMA-contracted, factored; within 1e-12 of each
    field's maximum).
    """
    fields = Fields()
    fields.u, fields.v, fields.w = u, v, w
    fields.ut, fields.vt, fields.wt = ut, vt, wt
    fields.nscalar = len(scalars)
    fields.mode = mode
    fields.dt = dt
    for n, (s, st) in enumerate(zip(scalars, scalar_out, strict=True)):
        fields.s[n] = s
        fields.st[n] = st
    check(load().f2c_advection_variant_v1(ctypes.byref(grid), ctypes.byref(fields), variant,
                                          ctypes.c_void_p(stream)))


def halo_fill(grid: Grid, pointers, kinds, stream=0) -> None:
    n = len(pointers)
    ptrs = (ctypes.c_void_p * n)(*pointers)
    ks = (ctypes.c_int32 * n)(*kinds)
    check(load().f2c_halo_fill_v1(ctypes.byref(grid), ptrs, ks, n, ctypes.c_void_p(stream)))


def fp64_rate(op: int, scratch_ptr: int, scratch_elems: int) -> float:
    """FP64 instructions/s of the current GPU: op 0 = add.rn.f64, op 1 = fma.rn.f64 (synchronous)."""
    out = ctypes.c_double(0.0)
    status = probe().f2c_fp64_rate_v1(op, ctypes.c_void_p(scratch_ptr), scratch_elems, ctypes.byref(out))
    if status != 0:
        raise NativeError(status, "FP64 rate probe failed")
    return out.value


def make_fields(u, v, w, ut=None, vt=None, wt=None, scalars=(), scalar_out=(), mode=TENDENCY, dt=0.0) -> Fields:
    fields = Fields()
    fields.u, fields.v, fields.w = u, v, w
    fields.ut, fields.vt, fields.wt = ut, vt, wt
    fields.nscalar = len(scalars)
    fields.mode = mode
    fields.dt = dt
    for n, (s, st) in enumerate(zip(scalars, scalar_out, strict=True)):
        fields.s[n] = s
        fields.st[n] = st
    return fields


class Batch:
    """A prepared batch: instances' grids and fields, a device workspace (caller-owned pointer) and the plan.

    ``tile_rows`` is the tile height (4, 8 or 16; 4 and 16 run the fast-fp kernel only). ``graph_step`` replays
    the step as a CUDA graph the batch captures on its first call and keeps until it is re-prepared or freed.
    """

    def __init__(self, grids, fields, kz=None, tile_rows: int = 8):
        self.count = len(grids)
        self.grids = (Grid * self.count)(*grids)
        self.fields = (Fields * self.count)(*fields)
        self.kz = (ctypes.c_int32 * self.count)(*kz) if kz else None
        self.tile_rows = tile_rows
        self.plan = BatchPlan()
        self._graph = None

    def workspace_bytes(self) -> int:
        return load().f2c_batch_workspace_bytes_rows_v1(self.grids, self.kz, self.count, self.tile_rows)

    def prepare(self, workspace: int, nbytes: int, stream: int = 0) -> None:
        self._drop_graph()
        check(load().f2c_batch_prepare_rows_v1(self.grids, self.fields, self.kz, self.count, self.tile_rows,
                                               ctypes.c_void_p(workspace), nbytes, None, ctypes.c_void_p(stream),
                                               ctypes.byref(self.plan)))

    def prepare_async(self, workspace: int, nbytes: int, staging: int, stream: int = 0) -> None:
        """Plan through host ``staging`` memory without waiting (see f2c_batch_prepare_async_v1)."""
        self._drop_graph()
        check(load().f2c_batch_prepare_rows_v1(self.grids, self.fields, self.kz, self.count, self.tile_rows,
                                               ctypes.c_void_p(workspace), nbytes, ctypes.c_void_p(staging),
                                               ctypes.c_void_p(stream), ctypes.byref(self.plan)))

    def set_fast_fp(self, fast: bool = True) -> None:
        """Step with the fast-fp kernel (F2C_BATCH_FAST_FP); preparation clears the choice for 8-row tiles."""
        self._drop_graph()
        if fast:
            self.plan.reserved |= BATCH_FAST_FP
        else:
            self.plan.reserved &= ~BATCH_FAST_FP

    def step(self, stream: int = 0) -> None:
        check(load().f2c_batch_step_v1(ctypes.byref(self.plan), ctypes.c_void_p(stream)))

    def graph_step(self, stream: int = 0) -> None:
        """The step as a replay of the batch's own CUDA graph (captured on the first call)."""
        if self._graph is None:
            out = ctypes.c_void_p()
            check(load().f2c_batch_graph_create_v1(ctypes.byref(self.plan), ctypes.byref(out)))
            self._graph = out.value
        check(load().f2c_batch_graph_launch_v1(ctypes.c_void_p(self._graph), ctypes.c_void_p(stream)))

    def halo(self, stream: int = 0) -> None:
        """Boundary fill of every instance's outputs, one launch."""
        check(load().f2c_batch_halo_v1(ctypes.byref(self.plan), ctypes.c_void_p(stream)))

    def _drop_graph(self) -> None:
        if self._graph is not None:
            load().f2c_batch_graph_destroy_v1(ctypes.c_void_p(self._graph))
            self._graph = None

    def __del__(self):
        try:
            self._drop_graph()
        except Exception:
            pass


def seed_fields(grid: Grid, seed: int, pointers, stream=0) -> None:
    """Seeded sine-mode fields (U, V, W, then scalars) written on the device, ghosts filled (f2c_seed_fields_v1)."""
    n = len(pointers)
    ptrs = (ctypes.c_void_p * n)(*pointers)
    check(load().f2c_seed_fields_v1(ctypes.byref(grid), seed, n - 3, ptrs, ctypes.c_void_p(stream)))


SET, MULTIPLY, CDU_DIV, CDU_ADV, CDV_DIV, CDV_ADV, CDW_DIV, CDW_ADV = range(8)


def procedure(op: int, grid: Grid, out, u=None, v=None, w=None, value=0.0, stream=0) -> None:
    """One reference procedure as one launch (device pointers)."""
    check(load().f2c_procedure_v1(op, ctypes.byref(grid), out, u, v, w, value, ctypes.c_void_p(stream)))
