"""The Fortran modules against the reference's, declaration by declaration (CPU only).

No Fortran compiler exists on these machines, so the modules are checked by
reading them: every interface of the reference's fort_scoped_memory
(compiler/runtime/scoped_memory.f90) must be declared here with the same dummy
arguments in the same order, each with the same type, kind and attributes
(VALUE, INTENT, ...); every public method and generic of the reference's
resident_domain type (compiler/runtime/resident_domain.f90:72-106) must be
bound here, its procedure taking the same dummy arguments with the same types,
kinds and attributes. Code that compiles against the reference's modules then
compiles against these. Without the reference checkout only the parser and
this repository's own modules are exercised.
"""

import re
from pathlib import Path

import pytest

from compiler import native
from oracle.build_ref import REFERENCE

OURS = native.PACKAGE_ROOT / "fortran"
THEIRS = REFERENCE / "compiler" / "runtime"

TYPE_SPEC = re.compile(r"^(type\s*\([^)]*\)|class\s*\([^)]*\)|integer(\s*\([^)]*\))?|real(\s*\([^)]*\))?|"
                       r"logical(\s*\([^)]*\))?|character(\s*\([^)]*\))?)\s*(,.*?)?::(.*)$", re.I)
HEAD = re.compile(r"^(?:[a-z]+\s+)*?(function|subroutine)\s+(\w+)\s*\(([^)]*)\)", re.I)


def _lines(path: Path):
    """Statements of a free-form source: comments (and OpenMP sentinels) dropped, continuations joined."""
    out, pending = [], ""
    for raw in path.read_text().splitlines():
        line = raw
        quote = None
        for n, ch in enumerate(line):  # cut a comment outside quotes
            if quote:
                if ch == quote:
                    quote = None
            elif ch in "'\"":
                quote = ch
            elif ch == "!":
                line = line[:n]
                break
        line = line.strip()
        if pending:
            line = pending + " " + line.lstrip("&").strip()
            pending = ""
        if line.endswith("&"):
            pending = line[:-1].rstrip()
            continue
        if line and not line.startswith("#"):
            out.append(line)
    return out


def _split_entities(text: str):
    """Names of an entity list with their array specs: 'a(:), b, c(3)' -> [('a', '(:)'), ('b', ''), ...]."""
    items, depth, cur = [], 0, ""
    for ch in text:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            items.append(cur)
            cur = ""
        else:
            cur += ch
    items.append(cur)
    result = []
    for item in items:
        item = item.split("=")[0].strip()
        m = re.match(r"(\w+)\s*(\(.*\))?", item)
        if m:
            result.append((m.group(1).lower(), re.sub(r"\s+", "", (m.group(2) or "")).lower()))
    return result


def _norm(text: str) -> str:
    return re.sub(r"\s+", "", text or "").lower()


def procedures(path: Path):
    """{name: [(dummy, type, attributes, array spec), ...]} of every function and subroutine in a module."""
    found, current, args, decls = {}, None, [], {}
    for line in _lines(path):
        low = line.lower()
        if current is None:
            m = HEAD.match(line)
            if m and not low.startswith("end"):
                current, args, decls = m.group(2).lower(), [a.strip().lower() for a in m.group(3).split(",") if
                                                              a.strip()], {}
            continue
        if re.match(r"^end\s*(function|subroutine)\b", low):
            found[current] = [(a, *decls.get(a, ("?", (), ""))) for a in args]
            current = None
            continue
        m = TYPE_SPEC.match(line)
        if m:
            base = _norm(m.group(1))
            attrs = tuple(sorted(_norm(a) for a in _split_top(m.group(6) or "") if a.strip()))
            for name, spec in _split_entities(m.group(7)):
                if name in args:
                    decls[name] = (base, attrs, spec)
    return found


def _split_top(attrs: str):
    out, depth, cur = [], 0, ""
    for ch in attrs.lstrip(","):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return out


def type_bindings(path: Path, type_name: str):
    """Type-bound procedure and generic names of a derived type: {binding: tuple of specifics}."""
    bindings, inside, contains = {}, False, False
    for line in _lines(path):
        low = line.lower()
        if re.match(rf"^type\s*(,[^:]*)?::\s*{type_name}\b", low):
            inside = True
            continue
        if inside and re.match(r"^end\s*type", low):
            break
        if inside and low == "contains":
            contains = True
            continue
        if inside and contains:
            m = re.match(r"^(procedure|generic)\s*(,[^:]*)?::\s*(\w+)\s*(=>\s*(.*))?$", low)
            if m:
                specifics = tuple(s.strip() for s in (m.group(5) or m.group(3)).split(","))
                bindings[m.group(3)] = specifics
    return bindings


def interfaces(path: Path):
    """Interfaces declared inside INTERFACE blocks only (bind(C) declarations)."""
    text_lines = _lines(path)
    keep, inside = [], False
    for line in text_lines:
        low = line.lower()
        if low == "interface":
            inside = True
            continue
        if low.startswith("end interface"):
            inside = False
            continue
        if inside:
            keep.append(line)
    tmp = "\n".join(keep)
    fake = Path(path.parent / "__interfaces__")
    found = {}
    current, args, decls = None, [], {}
    for line in tmp.splitlines():
        low = line.lower()
        if current is None:
            m = HEAD.match(line)
            if m:
                current, args, decls = m.group(2).lower(), [a.strip().lower() for a in m.group(3).split(",") if
                                                              a.strip()], {}
            continue
        if re.match(r"^end\s*(function|subroutine)\b", low):
            found[current] = [(a, *decls.get(a, ("?", (), ""))) for a in args]
            current = None
            continue
        m = TYPE_SPEC.match(line)
        if m:
            base = _norm(m.group(1))
            attrs = tuple(sorted(_norm(a) for a in _split_top(m.group(6) or "") if a.strip()))
            for name, spec in _split_entities(m.group(7)):
                if name in args:
                    decls[name] = (base, attrs, spec)
    del fake
    return found


def test_own_modules_parse_and_every_dummy_is_declared():
    ours = interfaces(OURS / "fort_scoped_memory.f90")
    assert len(ours) >= 50
    for name, dummies in ours.items():
        for dummy in dummies:
            assert dummy[1] != "?", f"{name}: dummy {dummy[0]} is not declared"
    methods = type_bindings(OURS / "fort_resident_domain.f90", "resident_domain")
    procs = procedures(OURS / "fort_resident_domain.f90")
    for binding, specifics in methods.items():
        for specific in specifics:
            assert specific in procs, f"{binding} => {specific} has no procedure"
            for dummy in procs[specific]:
                assert dummy[1] != "?", f"{specific}: dummy {dummy[0]} is not declared"


needs_reference = pytest.mark.skipif(not (THEIRS / "scoped_memory.f90").exists(),
                                     reason="the reference's runtime modules are not on this machine")


@needs_reference
def test_every_reference_interface_is_declared_alike():
    theirs = interfaces(THEIRS / "scoped_memory.f90")
    ours = interfaces(OURS / "fort_scoped_memory.f90")
    assert len(theirs) > 40
    for name, dummies in theirs.items():
        assert name in ours, f"{name} is not declared"
        assert ours[name] == dummies, f"{name}: {ours[name]} != {dummies}"


@needs_reference
def test_every_reference_method_is_bound_with_the_same_dummies():
    theirs_bindings = type_bindings(THEIRS / "resident_domain.f90", "resident_domain")
    ours_bindings = type_bindings(OURS / "fort_resident_domain.f90", "resident_domain")
    assert len(theirs_bindings) > 30
    theirs_procs = procedures(THEIRS / "resident_domain.f90")
    ours_procs = procedures(OURS / "fort_resident_domain.f90")
    for binding, specifics in theirs_bindings.items():
        assert binding in ours_bindings, f"method {binding} is missing"
        assert set(specifics) <= set(ours_bindings[binding]), f"{binding}: {ours_bindings[binding]} != {specifics}"
        for specific in specifics:
            assert ours_procs[specific] == theirs_procs[specific], \
                f"{specific}:\n ours   {ours_procs[specific]}\n theirs {theirs_procs[specific]}"
