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
epoch unless one is active (``begin_epoch``; without ``budget`` the domain
takes what the device has free), ``leave`` ends it (``end_epoch``, which
publishes), ``close`` releases the device state and is unconditional,
``publish`` brings every value home, ``observe`` brings named arrays home and
keeps their device copies (one field of an array of derived type is named
``objects(:)%field`` and goes through ``observe_field``), ``release`` retires
arrays without publication (before they are deallocated), ``active`` stores
whether an epoch is active. ``host`` and ``reduction`` annotate loop nests for
the compiler: their lines are removed and generate no code. A directive is a
comment, so the native build ignores it.

The generated text and the error messages follow the reference's expander
(directives.py:44-153, tests/test_resident_directives.py): every malformed
line is refused with its line number.
"""

from __future__ import annotations

import re
from dataclasses import dataclass

# ``!$fort`` at the start of a line (case-insensitive, whole word); the rest is the body
_LINE = re.compile(r"^(?P<indent>[ \t]*)!\$fort\b[ \t]*(?P<body>.*?)[ \t]*$", re.I)
_IDENT = re.compile(r"[ \t]*([A-Za-z_]\w*)[ \t]*")
_NAME = re.compile(r"[A-Za-z]\w*(?:%[A-Za-z]\w*)*\Z")
_FIELD = re.compile(r"([A-Za-z]\w*)\s*\(\s*:\s*\)\s*%\s*([A-Za-z]\w*)\Z")
CLAUSES = {"enter": {"budget", "if", "device"}, "leave": set(), "close": set(), "publish": {"if"},
           "observe": {"if"}, "release": set(), "active": set()}
TAKES_LIST = {"observe", "release", "active"}
ANNOTATIONS = {"host", "reduction"}


@dataclass(frozen=True)
class Domain:
    module: str = "fort_resident_application"
    object: str = "resident"
    check: str = "resident_require"
    prefix: str = "fort"


class DirectiveError(ValueError):
    pass


def _closing(text: str, start: int) -> int:
    """Index just past the parenthesis that closes the one at ``start``; -1 when it never closes."""
    depth = 0
    for index in range(start, len(text)):
        depth += {"(": 1, ")": -1}.get(text[index], 0)
        if depth == 0:
            return index + 1
    return -1


def _words(body: str, line: int) -> list:
    """``word[(argument)] word[(argument)] ...`` -> [(lower-case word, argument or None)]."""
    words, at = [], 0
    while at < len(body):
        m = _IDENT.match(body, at)
        if m is None:
            raise DirectiveError(f"Malformed residency directive on line {line}: {body!r}")
        at, argument = m.end(), None
        if body.startswith("(", at):
            end = _closing(body, at)
            if end < 0:
                raise DirectiveError(f"Unbalanced parentheses in the residency directive on line {line}")
            argument, at = body[at + 1:end - 1].strip(), end
        words.append((m.group(1).lower(), argument))
    return words


def _items(argument: str) -> list:
    """Split a list at the commas outside parentheses."""
    return [item.strip() for item in re.split(r",(?![^()]*\))", argument)]


def _check_annotation(name: str, words: list, body: str, line: int) -> None:
    """``host`` stands alone; ``reduction`` names at least one ``operator: scalars`` list."""
    if name == "host":
        ok = len(words) == 1 and words[0][1] is None
    else:
        reductions = [arg for word, arg in words if word == "reduction"]
        ok = bool(reductions) and all(word in ("reduction", "private") and arg is not None for word, arg in words)
        for arg in reductions if ok else []:
            operator, colon, names = arg.partition(":")
            ok = ok and bool(colon) and bool(operator.strip()) and any(n.strip() for n in names.split(","))
    if not ok:
        raise DirectiveError(f"Malformed residency directive on line {line}: {body!r}")


def parse(body: str, line: int):
    """A directive body -> (name, [array names], {clause: value}); annotations give no arrays or clauses."""
    words = _words(body, line)
    if not words:
        raise DirectiveError(f"Empty residency directive on line {line}")
    name, argument = words[0]
    if name in ANNOTATIONS:
        _check_annotation(name, words, body, line)
        return name, [], {}
    if name not in CLAUSES:
        raise DirectiveError(f"Unknown residency directive on line {line}: {name}")
    clauses = dict(words[1:])
    if len(clauses) != len(words) - 1 or not set(clauses) <= CLAUSES[name] or None in clauses.values():
        raise DirectiveError(f"Unsupported clause in the residency directive on line {line}: {body!r}")
    if name not in TAKES_LIST:
        if argument is not None:
            raise DirectiveError(f"The {name} directive on line {line} takes no arguments")
        return name, [], clauses
    if argument is None:
        raise DirectiveError(f"The {name} directive on line {line} needs a list of arrays")
    items = _items(argument)
    if not all(_NAME.match(i) or (name == "observe" and _FIELD.match(i)) for i in items):
        raise DirectiveError(f"The {name} directive on line {line} takes array names, not expressions")
    if name == "active" and len(items) != 1:
        raise DirectiveError(f"The active directive on line {line} takes one logical variable")
    return name, items, clauses


def _block(indent: str, domain: Domain, body: list[str], binding: bool = False) -> str:
    out = ["block"]
    if binding:
        out.append("  use, intrinsic :: iso_c_binding")
    out.append(f"  use {domain.module}, only: {domain.object}")
    out += ["  " + b for b in body]
    out.append("end block")
    return "".join(indent + line + "\n" for line in out)


def _observe(items: list, active: str, indent: str, domain: Domain, origin: str) -> str:
    r, handles = domain.object, f"{domain.prefix}_observed"
    arrays = [a for a in items if not _FIELD.match(a)]
    fields = [_FIELD.match(a).groups() for a in items if _FIELD.match(a)]
    body = [f"integer(c_int64_t) :: {handles}({len(arrays)})"] if arrays else []
    body.append(f"if ({active}) then")
    body += [f"  {handles}({n}) = {r}%bind({a}, lbound({a}), .true., origin='{origin}::{a.lower()}')"
             for n, a in enumerate(arrays, 1)]
    if arrays:
        body.append(f"  call {r}%observe({handles})")
    body += [f"  if (size({objects}) > 0) call {r}%observe_field(c_loc({objects}(lbound({objects},1))%{member}))"
             for objects, member in fields]
    body.append("endif")
    return _block(indent, domain, body, True)


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
        return _block(indent, domain, [f"if ({r}%active) then", *(f"  call {r}%release_real({a})" for a in items),
                                       "endif"])
    if name == "observe":
        return _observe(items, active, indent, domain, origin)
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
