"""Thin emitter of C-ABI numerical entries into the hand-written sm_103a templates.

The reference compiler lowers each selected procedure's loop nests through its
IR and emits a generic grid-stride kernel per nest plus an ``extern "C"``
entry (compiler/emission/cuda/scoped.py:69-553). Here the numerical work of
the advection procedures is hand-written once (csrc/kernels); emission only
maps a selected procedure to its template and writes

* ``csrc/entries/shared_entries.cu``: one ``extern "C" int
  cpp_fort_shared_<digest>(fort_scope_t, int mode, fort_buffer_t ..., const
  double *..., const int *...)`` per entry, packing its arguments for the
  template runner (the reference's entry signature, scoped.py:96-102,237,533);
* ``include/fort_shared_entries.h``: their declarations;
* ``fortran/fort_shared_entries.f90``: ``module fort_shared_<digest>`` with
  ``function run(...) bind(C, name='cpp_fort_shared_<digest>')`` per entry
  (the reference's interface module shape, scoped.py:514-523);
* ``compiler/emission/entries.json``: the entry report (argument order,
  modes, the written arrays, the template).

The digest is the first 12 hex digits of the SHA-256 of the entry identity,
as the reference names its entries (scoped.py:74-80); the identity here names
the template instead of a lowered plan, so the symbols are this build's own.
Output is deterministic: regenerating yields identical bytes.
"""

from __future__ import annotations

import json
from dataclasses import dataclass
from functools import lru_cache
from hashlib import sha256
from pathlib import Path

PACKAGE_ROOT = Path(__file__).resolve().parent.parent.parent
REPO_ROOT = PACKAGE_ROOT.parent
ENTRY_SOURCE = PACKAGE_ROOT / "csrc" / "entries" / "shared_entries.cu"
ENTRY_HEADER = REPO_ROOT / "include" / "fort_shared_entries.h"
FORTRAN_INTERFACES = PACKAGE_ROOT / "fortran" / "fort_shared_entries.f90"
REPORT = Path(__file__).resolve().parent / "entries.json"

ENTRY_ABI = "gb300-entry-abi:1"


@dataclass(frozen=True)
class Param:
    name: str
    kind: str  # "array", "real" or "int"
    intent: str = "in"


@dataclass(frozen=True)
class Entry:
    procedure: str      # module::procedure, lower case
    template: str       # f2c::entries::Template enumerator
    params: tuple
    nscalar: int = 0
    source: str = ""    # the reference procedure it replaces (file:line), or a description
    notes: str = ""

    @property
    def identity(self) -> str:
        signature = ",".join(f"{p.kind}:{p.intent}:{p.name.lower()}" for p in self.params)
        return f"{ENTRY_ABI}:{self.procedure}:template={self.template}:scalars={self.nscalar}:({signature})"

    @property
    def digest(self) -> str:
        return sha256(self.identity.encode()).hexdigest()[:12]

    @property
    def fortran_module(self) -> str:
        return "fort_shared_" + self.digest

    @property
    def symbol(self) -> str:
        return "cpp_fort_shared_" + self.digest

    @property
    def code_key(self) -> int:
        return int(sha256((self.identity + ":graph").encode()).hexdigest()[:16], 16)

    def arrays(self):
        return [p for p in self.params if p.kind == "array"]

    def reals(self):
        return [p for p in self.params if p.kind == "real"]

    def ints(self):
        return [p for p in self.params if p.kind == "int"]


def _a(name, intent="in"):
    return Param(name, "array", intent)


def _r(name):
    return Param(name, "real")


def _i(name):
    return Param(name, "int")


def _momentum(letter: str, which: str, source_file: str, lines: dict):
    """set / div / adv / whole procedure entries of one momentum component (U, V or W)."""
    out = f"{letter}2"
    n = [f"{letter}nx", f"{letter}ny", f"{letter}nz"]
    velocity = [_a("U"), _a("V"), _a("W")]
    spacing = [_r("dxmin"), _r("dymin"), _r("dzmin")]
    cap = which.capitalize()
    return [
        Entry(f"momentumadvection::{which}div", f"{cap}Div", (_a(out, "out"), *velocity, *spacing, *map(_i, n)),
              source=f"{source_file}:{lines['div']}"),
        Entry(f"momentumadvection::{which}adv", f"{cap}Adv", (_a(out, "inout"), *velocity, *spacing, *map(_i, n)),
              source=f"{source_file}:{lines['adv']}"),
        Entry(f"momentumadvection::{which}", cap, (_a(out, "out"), *velocity, *spacing, *map(_i, n)),
              source=f"{source_file}:{lines['whole']}",
              notes="set, div, adv and multiply by one half fused into one face-sharing launch"),
    ]


def _step_entries():
    entries = []
    for ns in range(5):
        scal = [_a(f"S{n + 1}") for n in range(ns)]
        tend = [_a(f"S{n + 1}t", "out") for n in range(ns)]
        newer = [_a(f"S{n + 1}n", "out") for n in range(ns)]
        grid = [_i("nx"), _i("ny"), _i("nz"), _i("halo")]
        entries.append(Entry(f"advection::step{ns}", "Step",
                             (_a("U2", "out"), _a("V2", "out"), _a("W2", "out"), _a("U"), _a("V"), _a("W"),
                              *scal, *tend, _r("dx"), _r("dy"), _r("dz"), *grid), nscalar=ns,
                             source="benchmarks/cdu/src/cdu.f90:113-133 with cvd.f90/cdw.f90:105-125 and "
                                    f"{ns} passive scalars",
                             notes="U, V, W tendencies (CDU, CDV, CDW) and scalar tendencies in one launch"))
        entries.append(Entry(f"advection::advance{ns}", "StepAdvance",
                             (_a("Un", "out"), _a("Vn", "out"), _a("Wn", "out"), _a("U"), _a("V"), _a("W"),
                              *scal, *newer, _r("dx"), _r("dy"), _r("dz"), _r("dt"), *grid), nscalar=ns,
                             source="forward-Euler update of the tendencies of advection::step",
                             notes="out = in + dt * tendency, double-buffered"))
        entries.append(Entry(f"advection::halo{ns}", "Halo",
                             (_a("U", "inout"), _a("V", "inout"), _a("W", "inout"),
                              *[_a(f"S{n + 1}", "inout") for n in range(ns)], *grid), nscalar=ns,
                             source="periodic x/y boundary fill in the order of compiler/tests/apps/box/"
                                    "boundaries.f90:6-41; walls in z (W zero, mirrored)"))
    return entries


def registry() -> list[Entry]:
    """Every entry this build emits, in a fixed order."""
    return list(_registry())


@lru_cache(maxsize=1)
def _registry() -> tuple:
    cdu = "benchmarks/cdu/src/cdu.f90"
    stencils = "compiler/tests/fixtures/stencils"
    entries = [
        Entry("momentumadvection::set", "Set", (_a("arr", "out"), _r("val"), _i("Unx"), _i("Uny"), _i("Unz")),
              source=f"{cdu}:12-27"),
        Entry("momentumadvection::multiply", "Multiply",
              (_a("arr", "inout"), _r("val"), _i("Unx"), _i("Uny"), _i("Unz")), source=f"{cdu}:30-45"),
    ]
    entries += _momentum("U", "cdu", cdu, {"div": "48-76", "adv": "79-106", "whole": "113-133"})
    entries += _momentum("V", "cdv", f"{stencils}/cvd.f90", {"div": "44-70", "adv": "73-98", "whole": "105-125"})
    entries += _momentum("W", "cdw", f"{stencils}/cdw.f90", {"div": "44-70", "adv": "73-98", "whole": "105-125"})
    entries += _step_entries()
    entries += [
        Entry("stencil::diffuse7", "Diffusion",
              (_a("b", "inout"), _a("a"), _r("dt"), _r("nu"), _r("dx"), _i("nx"), _i("ny"), _i("nz"), _i("halo")),
              source="compiler/tests/apps/box/stepper.f90:8-30 (diffuse with laplacian)"),
        Entry("stencil::jacobi5", "Jacobi", (_a("v", "inout"), _a("u"), _i("nx"), _i("ny"), _i("halo")),
              source="compiler/tests/apps/relax/relax.f90:28-33 (one Jacobi sweep)"),
        Entry("stencil::yee2d", "Yee",
              (_a("ez", "inout"), _a("hx", "inout"), _a("hy", "inout"), _r("ch"), _r("ce"), _i("nx"), _i("ny"),
               _i("halo")),
              source="2-D TM Yee leapfrog (no reference source in the mount)", notes="H task then E task"),
    ]
    return tuple(entries)


@lru_cache(maxsize=None)
def entry_for(procedure: str) -> Entry:
    for entry in _registry():
        if entry.procedure == procedure.lower():
            return entry
    raise KeyError(procedure)


def _c_param(p: Param) -> str:
    if p.kind == "array":
        return f"fort_buffer_t {p.name.lower()}_handle"
    if p.kind == "real":
        return f"const double *{p.name.lower()}"
    return f"const int *{p.name.lower()}"


def _signature(entry: Entry) -> str:
    params = ["fort_scope_t fort_context", "int fort_mode", *[_c_param(p) for p in entry.params]]
    return f"int {entry.symbol}({', '.join(params)})"


def render_source(entries) -> str:
    lines = ["// Generated by compiler/emission from the template registry; regenerate, do not edit.",
             "// Each entry packs its arguments for the hand-written template runner (entry_runner.cu).",
             '#include "entry_runner.hpp"', "",
             "using f2c::entries::EntryCall;", "using f2c::entries::Template;", "using f2c::entries::run_entry;", ""]
    for e in entries:
        lines.append(f"// {e.procedure}: {e.source}")
        lines.append(f'extern "C" {_signature(e)} {{')
        lines.append("    EntryCall call{};")
        lines.append("    call.context = fort_context;")
        lines.append("    call.mode = fort_mode;")
        lines.append(f"    call.kind = Template::{e.template};")
        lines.append(f"    call.code_key = 0x{e.code_key:016x}ULL;")
        lines.append(f"    call.nscalar = {e.nscalar};")
        arrays, reals, ints = e.arrays(), e.reals(), e.ints()
        lines.append(f"    call.narrays = {len(arrays)};")
        for n, p in enumerate(arrays):
            lines.append(f"    call.arrays[{n}] = {p.name.lower()}_handle;")
        lines.append(f"    call.nreals = {len(reals)};")
        for n, p in enumerate(reals):
            lines.append(f"    call.reals[{n}] = {p.name.lower()};")
        lines.append(f"    call.nints = {len(ints)};")
        for n, p in enumerate(ints):
            lines.append(f"    call.ints[{n}] = {p.name.lower()};")
        lines.append("    return run_entry(call);")
        lines.append("}")
        lines.append("")
    return "\n".join(lines)


def render_header(entries) -> str:
    lines = ["/* Numerical entries of the GB300 resident advection build (generated by compiler/emission).",
             " *",
             " * Each replaces the entry the reference compiler generates for the named",
             " * procedure (compiler/emission/cuda/scoped.py:237-553): same argument order",
             " * (context, mode, array handles in declaration order, scalars by reference),",
             " * same statuses (scoped_runtime.h). FORT_SCOPE_NATIVE mode, device resources",
             " * unavailable before any work, or arrays of differing shapes return",
             " * FORT_SCOPE_DECLINED with nothing done: the caller runs its original statements.",
             " */",
             "#ifndef FORT_SHARED_ENTRIES_H", "#define FORT_SHARED_ENTRIES_H",
             '#include "scoped_runtime.h"', "#ifdef __cplusplus", 'extern "C" {', "#endif", ""]
    for e in entries:
        lines.append(f"/* {e.procedure} -- replaces {e.source}" + (f"; {e.notes}" if e.notes else "") + " */")
        lines.append(_signature(e) + ";")
    lines += ["", "#ifdef __cplusplus", "}", "#endif", "#endif", ""]
    return "\n".join(lines)


def _fortran_args(names, width=100):
    out, line = [], "      "
    for n, name in enumerate(names):
        piece = name + (", " if n + 1 < len(names) else "")
        if len(line) + len(piece) > width:
            out.append(line.rstrip() + " &")
            line = "      "
        line += piece
    out.append(line)
    return out


def render_fortran(entries) -> str:
    lines = ["! Fortran interfaces of the GB300 numerical entries (generated by compiler/emission).",
             "! One module per entry, the shape of the reference's shared_interface.f90", ""]
    for e in entries:
        names = ["fort_context", "fort_mode", *[
            (p.name.lower() + "_handle") if p.kind == "array" else p.name.lower() for p in e.params]]
        lines += [f"module {e.fortran_module}", "  use iso_c_binding", "  implicit none", "  private",
                  "  public :: run", "  interface", "    function run( &"]
        lines += _fortran_args(names)
        lines[-1] += f") bind(C, name='{e.symbol}') result(fort_status)"
        lines += ["      import :: c_int, c_int64_t, c_double", "      integer(c_int) :: fort_status",
                  "      integer(c_int64_t), value :: fort_context", "      integer(c_int), value :: fort_mode"]
        for p in e.params:
            if p.kind == "array":
                lines.append(f"      integer(c_int64_t), value :: {p.name.lower()}_handle")
            elif p.kind == "real":
                lines.append(f"      real(c_double), intent(in) :: {p.name.lower()}")
            else:
                lines.append(f"      integer(c_int), intent(in) :: {p.name.lower()}")
        lines += ["    end function", "  end interface", f"end module {e.fortran_module}", ""]
    return "\n".join(lines)


def render_report(entries) -> str:
    report = []
    for e in entries:
        report.append({
            "procedure": e.procedure, "entry": e.symbol, "fortran_module": e.fortran_module,
            "fortran_procedure": "run", "template": e.template, "scalars": e.nscalar, "source": e.source,
            "argument_order": ["context", "mode", *[p.name for p in e.params]],
            "array_parameters": [{"name": p.name, "rank": 2 if e.template in ("Jacobi", "Yee") else 3,
                                  "dtype": "real64", "written": p.intent != "in"} for p in e.arrays()],
            "scalar_parameters": [{"name": p.name, "dtype": "real64" if p.kind == "real" else "integer32",
                                   "passing": "reference"} for p in e.params if p.kind != "array"],
            "definition_changes": [p.name for p in e.arrays() if p.intent == "out"],
            "modes": {"native": 0, "gpu": 1}, "native_mode": "declined",
            "graph_execution": {"runtime_api": "fort_scope_graph_enqueue_v1", "code_key": f"0x{e.code_key:016x}"},
            "numerical_contract": {"cuda": ["--fmad=false", "--ftz=false", "--prec-div=true", "--prec-sqrt=true"],
                                   "host": ["-ffp-contract=off"]},
        })
    return json.dumps({"schema_version": 1, "abi": ENTRY_ABI, "entries": report}, indent=1, sort_keys=True) + "\n"


def outputs() -> dict:
    entries = registry()
    return {ENTRY_SOURCE: render_source(entries), ENTRY_HEADER: render_header(entries),
            FORTRAN_INTERFACES: render_fortran(entries), REPORT: render_report(entries)}


def write_entries() -> None:
    """Write the generated files, touching only those whose contents changed."""
    for path, text in outputs().items():
        path.parent.mkdir(parents=True, exist_ok=True)
        if not path.exists() or path.read_text() != text:
            path.write_text(text)


def bind(lib) -> dict:
    """ctypes functions of every generated entry in ``lib``, keyed by procedure name.

    Arguments are (context, mode, array handles..., scalars by reference...) as
    the spliced Fortran call block passes them; reals are ``ctypes.c_double``
    and integers ``ctypes.c_int`` passed with ``ctypes.byref``.
    """
    import ctypes

    functions = {}
    for e in registry():
        fn = getattr(lib, e.symbol)
        args = [ctypes.c_uint64, ctypes.c_int]
        for p in e.params:
            if p.kind == "array":
                args.append(ctypes.c_uint64)
            elif p.kind == "real":
                args.append(ctypes.POINTER(ctypes.c_double))
            else:
                args.append(ctypes.POINTER(ctypes.c_int))
        fn.argtypes = args
        fn.restype = ctypes.c_int
        functions[e.procedure] = fn
    return functions


def call(functions: dict, procedure: str, context: int, mode: int, arrays, reals=(), ints=()) -> int:
    """Call one entry with plain Python values (arrays are handles)."""
    import ctypes

    entry = entry_for(procedure)
    if len(arrays) != len(entry.arrays()) or len(reals) != len(entry.reals()) or len(ints) != len(entry.ints()):
        raise ValueError(f"{procedure}: wrong argument counts")
    real_values = [ctypes.c_double(v) for v in reals]
    int_values = [ctypes.c_int(v) for v in ints]
    return functions[entry.procedure](context, mode, *arrays, *[ctypes.byref(v) for v in real_values],
                                      *[ctypes.byref(v) for v in int_values])
