"""The ``!$fort`` residency directives and the Fortran they expand to.

Grammar (the reference's surface, compiler/resident/directives.py:8-35):

    !$fort enter [budget(<bytes>)] [if(<condition>)] [device(<ordinal>)]
    !$fort leave
    !$fort close
    !$fort publish [if(<condition>)]
    !$fort observe(<array>[, <array>...]) [if(<condition>)]
    !$fort release(<array>[, <array>...])
    !$fort active(<logical variable>)
    !$fort host
    !$fort reduction(<operator>: <scalar>[, ...]) [private(...)]

Each directive becomes a ``block`` calling the application's residency object
``resident`` (module ``fort_resident_application``): ``enter`` starts an
epoch unless one is active (``begin_epoch``), ``leave`` ends it
(``end_epoch``, which publishes), ``close`` releases the device state,
``publish`` brings every value home, ``observe`` brings named arrays home and
keeps their device copies, ``release`` retires arrays without publication (before they are deallocated),
``active`` stores whether an epoch is active. ``host`` and ``reduction``
annotate loop nests for the compiler and generate no code here. A directive is
a comment, so the native build ignores it.
"""

from __future__ import annotations

import re
from dataclasses import dataclass

_LINE = re.compile(r"^(?P<indent>\s*)!\$fort\s+(?P<body>.*?)\s*$", re.I)
_WORD = re.compile(r"\s*([A-Za-z_]\w*)\s*")
_NAME = re.compile(r"[A-Za-z]\w*(?:%[A-Za-z]\w*)*$")
CLAUSES = {"enter": {"budget", "if", "device"}, "leave": set(), "close": set(), "publish": {"if"},
           "observe": {"if"}, "release": set(), "active": set(), "host": set(), "reduction": {"private"}}
TAKES_LIST = {"observe", "release", "active", "reduction"}


@dataclass(frozen=True)
class Domain:
    module: str = "fort_resident_application"
    object: str = "resident"
    check: str = "resident_require"
    prefix: str = "fort"


class DirectiveError(ValueError):
    pass


def parse(body: str, line: int):
    """``name(args) clause(value) ...`` -> (name, [args], {clause: value})."""
    words, pos = [], 0
    while pos < len(body):
        m = _WORD.match(body, pos)
        if not m:
            raise DirectiveError(f"line {line}: malformed residency directive {body!r}")
        word, pos, value = m.group(1).lower(), m.end(), None
        if pos < len(body) and body[pos] == "(":
            depth, start = 0, pos
            while pos < len(body):
                depth += (body[pos] == "(") - (body[pos] == ")")
                pos += 1
                if depth == 0:
                    break
            if depth:
                raise DirectiveError(f"line {line}: unbalanced parentheses in {body!r}")
            value = body[start + 1:pos - 1].strip()
        words.append((word, value))
    if not words:
        raise DirectiveError(f"line {line}: empty residency directive")
    (name, args), rest = words[0], words[1:]
    if name not in CLAUSES:
        raise DirectiveError(f"line {line}: unknown residency directive {name!r}")
    clauses = dict(rest)
    if len(clauses) != len(rest) or set(clauses) - CLAUSES[name] or any(v is None for v in clauses.values()):
        raise DirectiveError(f"line {line}: unsupported clause in {body!r}")
    if (args is not None) != (name in TAKES_LIST):
        raise DirectiveError(f"line {line}: {name} " + ("needs a list" if name in TAKES_LIST else "takes no list"))
    items = []
    if args is not None and name != "reduction":
        items = [a.strip() for a in re.split(r",(?![^()]*\))", args)]
        if not all(_NAME.match(a) for a in items):
            raise DirectiveError(f"line {line}: {name} takes array names, not expressions")
        if name == "active" and len(items) != 1:
            raise DirectiveError(f"line {line}: active takes one logical variable")
    return name, items, clauses


def _block(indent: str, domain: Domain, body: list[str], binding: bool = False) -> str:
    out = ["block"]
    if binding:
        out.append("  use, intrinsic :: iso_c_binding")
    out.append(f"  use {domain.module}, only: {domain.object}")
    out += ["  " + b for b in body]
    out.append("end block")
    return "".join(indent + line + "\n" for line in out)


def generate(name: str, items: list, clauses: dict, indent: str, domain: Domain, origin: str) -> str:
    r = domain.object
    cond = clauses.get("if")
    active = f"{r}%active" + (f" .and. ({cond})" if cond else "")
    if name == "enter":
        budget = f", int({clauses['budget']}, c_size_t)" if "budget" in clauses else ""
        call = f"call {r}%begin_epoch(int({clauses.get('device', '0')}, c_int){budget})"
        inner = [f"if ({cond}) {call}"] if cond else [call]
        return _block(indent, domain, [f"if (.not. {r}%active) then", *("  " + x for x in inner), "endif"], True)
    if name == "leave":
        return _block(indent, domain, [f"if ({r}%active) call {r}%end_epoch()"])
    if name == "close":
        return _block(indent, domain, [f"call {r}%close()"])
    if name == "publish":
        return _block(indent, domain, [f"if ({active}) call {r}%publish()"])
    if name == "active":
        return _block(indent, domain, [f"{items[0]} = {r}%active"])
    if name == "release":
        return _block(indent, domain, [f"if ({r}%active) then", *(f"  call {r}%release({a})" for a in items),
                                       "endif"])
    if name == "observe":
        handles = f"{domain.prefix}_observed"
        body = [f"integer(c_int64_t) :: {handles}({len(items)})", f"if ({active}) then"]
        body += [f"  {handles}({n}) = {r}%bind_real64({a}, lbound({a}), .true., origin='{origin}::{a.lower()}')"
                 for n, a in enumerate(items, 1)]
        body += [f"  call {r}%observe({handles})", "endif"]
        return _block(indent, domain, body, True)
    return ""  # host, reduction: annotations only


def expand(text: str, domain: Domain = Domain(), origin: str = "source"):
    """Replace each directive line by its code. Returns (new text, records)."""
    out, records = [], []
    for number, line in enumerate(text.splitlines(keepends=True), 1):
        m = _LINE.match(line.rstrip("\r\n"))
        if not m:
            out.append(line)
            continue
        name, items, clauses = parse(m.group("body"), number)
        out.append(generate(name, items, clauses, m.group("indent"), domain, origin))
        records.append({"line": number, "directive": name, "arrays": items, "clauses": clauses})
    return "".join(out), records
