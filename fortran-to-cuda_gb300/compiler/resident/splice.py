"""The call block that replaces a selected procedure's statements, and the splice that puts it in place.

Shape of the block (the reference's ``entry_call_block``,
compiler/scopes/resident_splice.py:72-203, in its conditional form): while the
residency domain is active, bind every array argument (by address and
extents, tolerant: an empty or strided array gets no handle), call the entry
with ``FORT_SCOPE_GPU``, the handles and the scalars; a nonzero status stops
the program through ``resident_require``, except ``FORT_SCOPE_DECLINED``, and
a declined call, an unbound array or an inactive domain publishes the domain
and runs the original statements.
"""

from __future__ import annotations

from dataclasses import dataclass

from .. import emission
from . import fortran
from .directives import Domain


@dataclass
class Spliced:
    procedure: str
    entry: str
    module: str
    nests: int


def call_block(entry: emission.Entry, original: str, domain: Domain = Domain(), indent: str = "    ") -> str:
    r = domain.object
    arrays = entry.arrays()
    handles = [f"{domain.prefix}_handle_{p.name.lower()}" for p in arrays]
    run = f"{domain.prefix}_device_run"
    on = f"{domain.prefix}_resident"
    status = f"{domain.prefix}_status"
    proc = entry.procedure
    lines = ["block",
             "  use, intrinsic :: iso_c_binding",
             "  use fort_scoped_memory, only: FORT_SCOPE_GPU, FORT_SCOPE_DECLINED",
             f"  use {domain.module}, only: {r}, {domain.check}",
             f"  use {entry.fortran_module}, only: {run} => run",
             f"  integer(c_int64_t) :: {', '.join(handles)}",
             f"  integer(c_int) :: {status}",
             f"  logical :: {on}",
             f"  {on} = {r}%active",
             f"  if ({on}) then"]
    for p, h in zip(arrays, handles):
        lines.append(f"    {h} = {r}%bind_real64({p.name}, lbound({p.name}), .true., &")
        lines.append(f"      origin='{proc}::{p.name.lower()}', tolerant=.true.)")
    lines.append(f"    {on} = all([" + ", ".join(handles) + "] /= 0_c_int64_t)")
    lines.append("  endif")
    by_name = dict(zip((p.name for p in arrays), handles))
    args = [f"{r}%context", "FORT_SCOPE_GPU", *[by_name.get(p.name, p.name) for p in entry.params]]
    lines.append(f"  if ({on}) then")
    lines.append(f"    {status} = {run}( &")
    lines.append("      " + ", &\n      ".join(args) + ")")
    lines.append(f"    {on} = {status} /= FORT_SCOPE_DECLINED")
    lines.append(f"    if ({on}) call {domain.check}({status})")
    lines.append("  endif")
    lines.append(f"  if (.not. {on}) then")
    lines.append(f"    if ({r}%active) call {r}%publish()")
    body = [indent + ln for ln in ("\n".join(lines)).split("\n")]
    text = "\n".join(body) + "\n" + original
    if not original.endswith("\n"):
        text += "\n"
    text += indent + "  endif\n" + indent + "end block\n"
    return text


def _nests(statements: str) -> int:
    """Outermost DO loops among the statements (each is one loop nest)."""
    depth, nests = 0, 0
    for line in statements.splitlines():
        code = line.split("!", 1)[0].strip().lower()
        if code.startswith("do ") or code == "do":
            if depth == 0:
                nests += 1
            depth += 1
        elif code.startswith("end do") or code.startswith("enddo"):
            depth = max(0, depth - 1)
    return nests


def matches(pattern: str, qualified: str) -> bool:
    module, _, name = pattern.lower().partition("::")
    pm, _, pn = qualified.partition("::")
    return module == pm and (name == "*" or name == pn)


def splice(text: str, patterns, domain: Domain = Domain()):
    """Replace the executable part of every selected procedure that has a template. Returns (text, [Spliced])."""
    lines = text.splitlines(keepends=True)
    found = fortran.procedures(text)
    registry = {e.procedure: e for e in emission.registry()}
    edits, done = [], []
    for proc in found:
        if not any(matches(p, proc.qualified) for p in patterns):
            continue
        entry = registry.get(proc.qualified)
        if entry is None or proc.body >= proc.end:
            continue
        original = "".join(lines[proc.body:proc.end])
        edits.append((proc.body, proc.end, call_block(entry, original, domain)))
        done.append(Spliced(proc.qualified, entry.symbol, entry.fortran_module, _nests(original)))
    for start, end, block in sorted(edits, reverse=True):
        lines[start:end] = [block]
    return "".join(lines), done
