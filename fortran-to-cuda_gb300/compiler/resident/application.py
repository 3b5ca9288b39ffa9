"""The TOML application description and the preparation of a resident build.

The description format is the reference's (compiler/resident/application.py:1-86);
this module reads the part of it that describes a single-source-tree
application such as ``benchmarks/cdu/cdu.toml``:

    name = "CDU"                                  # the CMake project
    sources = ["src/cdu.f90", "src/main.f90"]     # paths relative to the description
    program = "src/main.f90"                      # the main program among them
    [variants.default] defines = [...]            # the first variant is the default
    [[selection]] label, procedures = ["module::*" | "module::name"], minimum_nests
    [[edit]] file, at, action = before|after|replace, text
    [build] fortran_options, link, resident_link, libraries, include
    [[executable]] name, library = resident|native

Preparation copies the sources, splices a call block into every selected
procedure that has a template (compiler.emission), applies the edits (which
may add residency directives), wraps the host statements that touch arrays the
entries keep on the device (compiler.resident.host_access), expands the
directives, and writes the build.
Keys of the full format that describe multi-tree applications (``inputs``,
``patch``, ``rewrite``, ``held``, ``domain``, ``rewrites``) are refused with a
clear message: the procedures they serve are outside the advection path.
"""

from __future__ import annotations

import re
import tomllib
from dataclasses import dataclass, field
from pathlib import Path

from .. import emission
from . import directives, fortran, host_access, splice

SUPPORTED = {"name", "sources", "program", "variants", "selection", "edit", "build", "executable", "addressable"}
UNSUPPORTED = {"inputs", "patch", "rewrite", "held", "domain", "rewrites", "program_edit"}


class DescriptionError(ValueError):
    pass


@dataclass
class Selection:
    label: str
    procedures: list
    minimum_nests: int = 0


@dataclass
class Edit:
    """One edit of a source (the reference's format, compiler/resident/application.py:49-57): a place found by
    ``at`` (text found once, tolerant of layout), ``between`` (from the start of the first text to the end of the
    second), ``call`` (the CALL statement of that subroutine, from the start of its line) or ``module_end`` (before
    END MODULE of that module), or with none of them the whole ``procedure``; ``procedure`` also confines the
    others to that procedure."""
    file: str
    action: str
    text: str
    at: str | None = None
    procedure: str | None = None
    between: list | None = None
    call: str | None = None
    module_end: str | None = None


@dataclass
class Executable:
    name: str
    library: str


@dataclass
class Application:
    path: Path
    name: str
    sources: list
    program: Path
    defines: list
    selections: list
    edits: list
    build: dict
    executables: list
    variant: str = "default"
    report: dict = field(default_factory=dict)


def load(path, variant: str | None = None) -> Application:
    path = Path(path).resolve()
    data = tomllib.loads(path.read_text())
    bad = set(data) & UNSUPPORTED
    if bad:
        raise DescriptionError(f"{path.name}: {sorted(bad)} describe applications outside the advection path")
    unknown = set(data) - SUPPORTED - UNSUPPORTED
    if unknown:
        raise DescriptionError(f"{path.name}: unknown keys {sorted(unknown)}")
    for key in ("name", "sources", "program"):
        if key not in data:
            raise DescriptionError(f"{path.name}: missing {key!r}")
    base = path.parent
    sources = [(base / s).resolve() for s in data["sources"]]
    program = (base / data["program"]).resolve()
    if program not in sources:
        raise DescriptionError(f"{path.name}: the program must be one of the sources")
    for s in sources:
        if not s.exists():
            raise DescriptionError(f"{path.name}: source {s} does not exist")
    variants = data.get("variants", {"default": {}})
    chosen = variant or next(iter(variants))
    if chosen not in variants:
        raise DescriptionError(f"{path.name}: no variant {chosen!r}")
    selections = [Selection(s["label"], list(s["procedures"]), int(s.get("minimum_nests", 0)))
                  for s in data.get("selection", [])]
    edits = []
    edit_keys = {"file", "action", "text", "template", "at", "procedure", "function", "between", "call", "module_end"}
    for e in data.get("edit", []):
        unknown_keys = set(e) - edit_keys
        if unknown_keys:
            raise DescriptionError(f"{path.name}: unknown keys in edit: {sorted(unknown_keys)}")
        if e.get("action") not in {"before", "after", "replace"}:
            raise DescriptionError(f"{path.name}: edit action must be before, after or replace")
        if ("text" in e) == ("template" in e):
            raise DescriptionError(f"{path.name}: an edit needs text or a template, not both")
        text = e["text"] if "text" in e else (path.parent / e["template"]).read_text()
        if not any(k in e for k in ("at", "between", "call", "module_end", "procedure")):
            raise DescriptionError(f"{path.name}: an edit of {e.get('file')!r} locates no place")
        between = e.get("between")
        if between is not None and (not isinstance(between, list) or len(between) != 2):
            raise DescriptionError(f"{path.name}: between takes two pieces of text")
        edits.append(Edit(e["file"], e["action"], text, e.get("at"), e.get("procedure"), between, e.get("call"),
                          e.get("module_end")))
    executables = [Executable(x["name"], x.get("library", "resident")) for x in data.get("executable", [])]
    return Application(path, data["name"], sources, program, list(variants[chosen].get("defines", [])),
                       selections, edits, dict(data.get("build", {})), executables, chosen)


def _locate(text: str, at: str) -> tuple[int, int]:
    """Find ``at`` once in ``text``: exactly, or with any run of blanks matching any other."""
    count = text.count(at)
    if count == 1:
        start = text.index(at)
        return start, start + len(at)
    if count > 1:
        raise DescriptionError(f"edit anchor found {count} times, expected one: {at!r}")
    pattern = re.compile(r"\s+".join(re.escape(w) for w in at.split()) + (r"\s*\n" if at.endswith("\n") else ""))
    found = list(pattern.finditer(text))
    if len(found) != 1:
        raise DescriptionError(f"edit anchor found {len(found)} times, expected one: {at!r}")
    return found[0].start(), found[0].end()


def _procedure_span(text: str, name: str) -> tuple[int, int]:
    """Offsets of a procedure (``name`` or ``module::name``) from its header line to the end of its END line."""
    module, _, proc = name.lower().rpartition("::")
    lines = text.splitlines(keepends=True)
    found = [p for p in fortran.procedures(text) if p.name.lower() == proc and (not module or p.module == module)]
    if len(found) != 1:
        raise DescriptionError(f"edit: procedure {name!r} found {len(found)} times, expected one")
    p = found[0]
    last = p.end
    if re.match(r"\s*contains\b", lines[last], re.I):  # internal procedures follow: find the unit's own END
        pattern = re.compile(rf"\s*end\s*(subroutine|function|program)?\s*{re.escape(p.name)}?\s*(!.*)?$", re.I)
        last = next(i for i in range(last + 1, len(lines))
                    if pattern.match(lines[i].rstrip("\n")) and re.match(r"\s*end\s*(subroutine|function|program)\b",
                                                                         lines[i], re.I))
    start = sum(len(x) for x in lines[:p.header])
    return start, sum(len(x) for x in lines[:last + 1])


def _line_bounds(text: str, at: int) -> tuple[int, int]:
    """Start of the line holding offset ``at`` and the end of its statement (continuations), before the newline."""
    start = text.rfind("\n", 0, at) + 1
    end = text.find("\n", at)
    end = len(text) if end < 0 else end
    while text[start:end].split("!", 1)[0].rstrip().endswith("&"):
        nxt = text.find("\n", end + 1)
        end = len(text) if nxt < 0 else nxt
    return start, end


def _place(text: str, edit: Edit) -> tuple[int, int]:
    """The span an edit acts on, as offsets into ``text``."""
    lo, hi = (0, len(text)) if not edit.procedure else _procedure_span(text, edit.procedure)
    region = text[lo:hi]
    if edit.at is not None:
        start, end = _locate(region, edit.at)
    elif edit.between is not None:
        first, _ = _locate(region, edit.between[0])
        tail_start, end = _locate(region[first:], edit.between[1])
        end += first
        start = first
    elif edit.call is not None:
        calls = [m for m in re.finditer(rf"(?im)^[ \t]*call[ \t]+{re.escape(edit.call)}\b", region)]
        if len(calls) != 1:
            raise DescriptionError(f"edit: CALL {edit.call} found {len(calls)} times, expected one")
        start, end = _line_bounds(region, calls[0].start())
    elif edit.module_end is not None:
        ends = [m for m in re.finditer(rf"(?im)^[ \t]*end[ \t]*module[ \t]+{re.escape(edit.module_end)}\b", region)]
        if len(ends) != 1:
            raise DescriptionError(f"edit: END MODULE {edit.module_end} found {len(ends)} times, expected one")
        start = end = ends[0].start()
    elif edit.procedure is not None:
        return lo, hi
    else:
        raise DescriptionError("edit: locates no place")
    return lo + start, lo + end


def apply_edit(text: str, edit: Edit) -> str:
    start, end = _place(text, edit)
    if edit.action == "before":
        return text[:start] + edit.text + text[start:]
    if edit.action == "after":
        return text[:end] + edit.text + text[end:]
    return text[:start] + edit.text.replace("{original}", text[start:end]) + text[end:]


def prepare(app: Application, output, fast_fp: bool = False) -> Application:
    """Write the resident sources, the native copies and the build into ``output``.

    ``fast_fp`` is the reference's --fast-fp (compiler/resident/build.py:22,66-67): both builds drop the strict
    host option, and the resident one opens its contexts under the fast-fp numerical contract."""
    output = Path(output)
    resident_dir = output / "resident"
    native_dir = output / "native"
    resident_dir.mkdir(parents=True, exist_ok=True)
    native_dir.mkdir(parents=True, exist_ok=True)
    patterns = [p for s in app.selections for p in s.procedures]
    report = {"application": app.name, "variant": app.variant, "entries": [], "directives": [],
              "numerics": "fast" if fast_fp else "strict"}
    nests = {s.label: 0 for s in app.selections}
    texts, spliced_units, entry_arrays = {}, set(), {}
    for src in app.sources:
        text = src.read_text()
        (native_dir / src.name).write_text(text)
        spliced, done = splice.splice(text, patterns)
        for d in done:
            report["entries"].append({"procedure": d.procedure, "entry": d.entry, "module": d.module,
                                      "nests": d.nests, "file": src.name})
            spliced_units.add(d.procedure)
            entry = emission.entry_for(d.procedure)
            entry_arrays[d.procedure.split("::")[-1]] = [(n, p.name.lower()) for n, p in enumerate(entry.params)
                                                         if p.kind == "array"]
            for s in app.selections:
                if any(splice.matches(p, d.procedure) for p in s.procedures):
                    nests[s.label] += d.nests
        for edit in app.edits:
            if edit.file == src.name:
                spliced = apply_edit(spliced, edit)
        texts[src.name] = spliced
    # host statements that touch arrays the entries keep on the device
    try:
        texts, report["host_blocks"] = host_access.wrap(texts, entry_arrays, spliced_units)
    except host_access.HostAccessError as error:
        raise DescriptionError(str(error)) from None
    for src in app.sources:
        expanded, records = directives.expand(texts[src.name], origin=src.stem)
        report["directives"] += [{"file": src.name, **r} for r in records]
        (resident_dir / src.name).write_text(expanded)
    for s in app.selections:
        if nests[s.label] < s.minimum_nests:
            raise DescriptionError(f"selection {s.label!r}: {nests[s.label]} loop nests compiled, "
                                   f"fewer than minimum_nests = {s.minimum_nests}")
    report["nests"] = nests
    app.report = report
    from . import build

    build.write_cmake(app, output, fast_fp=fast_fp)
    return app
