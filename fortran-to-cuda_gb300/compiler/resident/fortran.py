"""Just enough of free-form Fortran to find procedures and their executable parts.

The reference locates procedures with fparser (compiler/frontend). The resident
build here only needs, for each program unit, where its executable statements
start and end, so this module scans the text: ``module`` blocks, ``program``,
``subroutine`` and ``function`` headers (with prefixes, continuation lines and
matching ``end``), the specification part (declarations, ``use``,
``implicit``), and ``contains`` sections, whose internal procedures are
reported as procedures of their own.
"""

from __future__ import annotations

import re
from dataclasses import dataclass

_MODULE = re.compile(r"^\s*module\s+(?!procedure\b)([A-Za-z]\w*)\s*(?:!.*)?$", re.I)
_END_MODULE = re.compile(r"^\s*end\s*module\b", re.I)
_HEADER = re.compile(
    r"^\s*(?:(?:pure|elemental|impure|recursive|module|non_recursive)\s+)*"
    r"(?:(?:integer|real|logical|complex|character|double\s+precision|type\s*\([^)]*\))(?:\s*\([^)]*\))?\s+)?"
    r"(subroutine|function)\s+([A-Za-z]\w*)", re.I)
_PROGRAM = re.compile(r"^\s*program\s+([A-Za-z]\w*)", re.I)
_END_PROC = re.compile(r"^\s*end\s*(subroutine|function|program)?\s*([A-Za-z]\w*)?\s*(?:!.*)?$", re.I)
_END_GENERIC = re.compile(r"^\s*end\s*(?:!.*)?$", re.I)
_CONTAINS = re.compile(r"^\s*contains\s*(?:!.*)?$", re.I)
_DECLARATION = re.compile(
    r"^\s*(implicit\b|use\b|integer\b|real\b|logical\b|complex\b|character\b|double\s+precision\b|"
    r"type\s*\(|class\s*\(|dimension\b|parameter\b|external\b|intrinsic\b|save\b|data\b|procedure\b|"
    r"import\b|include\b|common\b|equivalence\b|namelist\b|interface\b)", re.I)


@dataclass
class Procedure:
    module: str            # lower case, "" outside a module
    name: str              # as written
    kind: str              # "subroutine", "function" or "program"
    header: int            # line index of the header
    body: int              # first line index of the executable part
    end: int               # line index of the END statement (exclusive end of the executable part)

    @property
    def qualified(self) -> str:
        return f"{self.module}::{self.name.lower()}" if self.module else self.name.lower()


def _continued(line: str) -> bool:
    code = line.split("!", 1)[0].rstrip()
    return code.endswith("&")


def _blank_or_comment(line: str) -> bool:
    stripped = line.strip()
    return not stripped or (stripped.startswith("!") and not stripped.lower().startswith("!$"))


def procedures(text: str) -> list[Procedure]:
    lines = text.splitlines()
    out: list[Procedure] = []
    module = ""
    i = 0
    while i < len(lines):
        line = lines[i]
        if _blank_or_comment(line):
            i += 1
            continue
        m = _MODULE.match(line)
        if m:
            module = m.group(1).lower()
            i += 1
            continue
        if _END_MODULE.match(line):
            module = ""
            i += 1
            continue
        h = _HEADER.match(line)
        p = _PROGRAM.match(line)
        if (h or p) and not line.strip().lower().startswith("end"):
            kind, name = ("program", p.group(1)) if p else (h.group(1).lower(), h.group(2))
            header = i
            while _continued(lines[i]):
                i += 1
            i += 1
            # specification part
            while i < len(lines) and (_blank_or_comment(lines[i]) or _DECLARATION.match(lines[i])):
                while _continued(lines[i]):
                    i += 1
                i += 1
            body = i
            depth = 0
            end = None
            while i < len(lines):
                cur = lines[i]
                if _blank_or_comment(cur):
                    i += 1
                    continue
                inner = _HEADER.match(cur)
                if inner and not cur.strip().lower().startswith("end"):
                    depth += 1
                elif (_END_PROC.match(cur) and (_END_PROC.match(cur).group(1) or _END_GENERIC.match(cur))):
                    if depth == 0:
                        end = i
                        break
                    depth -= 1
                elif _CONTAINS.match(cur) and depth == 0 and end is None:
                    # internal procedures follow: the executable part ends here, and the scan goes on
                    # into them (the unit's own END is passed over like any other line)
                    out.append(Procedure(module, name, kind, header, body, i))
                    end = -1
                    break
                i += 1
            if end is None:
                raise ValueError(f"no END for {kind} {name}")
            if end >= 0:
                out.append(Procedure(module, name, kind, header, body, end))
            i += 1
            continue
        i += 1
    return out


def find(text: str, module: str, name: str) -> Procedure | None:
    for p in procedures(text):
        if p.module == module.lower() and p.name.lower() == name.lower():
            return p
    return None
