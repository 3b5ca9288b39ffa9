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
from . import directives, host_access, splice

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
    file: str
    action: str
    text: str
    at: str | None = None
    procedure: str | None = None


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
    for e in data.get("edit", []):
        if e.get("action") not in {"before", "after", "replace"}:
            raise DescriptionError(f"{path.name}: edit action must be before, after or replace")
        if "text" not in e:
            raise DescriptionError(f"{path.name}: an edit needs text")
        edits.append(Edit(e["file"], e["action"], e["text"], e.get("at"), e.get("procedure")))
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
        raise DescriptionError(f"edit anchor found {count} times: {at!r}")
    pattern = re.compile(r"\s+".join(re.escape(w) for w in at.split()) + (r"\s*\n" if at.endswith("\n") else ""))
    found = list(pattern.finditer(text))
    if len(found) != 1:
        raise DescriptionError(f"edit anchor found {len(found)} times: {at!r}")
    return found[0].start(), found[0].end()


def apply_edit(text: str, edit: Edit) -> str:
    if edit.at is None:
        raise DescriptionError("edits need an `at` anchor here")
    start, end = _locate(text, edit.at)
    if edit.action == "before":
        return text[:start] + edit.text + text[start:]
    if edit.action == "after":
        return text[:end] + edit.text + text[end:]
    return text[:start] + edit.text.replace("{original}", text[start:end]) + text[end:]


def prepare(app: Application, output) -> Application:
    """Write the resident sources, the native copies and the build into ``output``."""
    output = Path(output)
    resident_dir = output / "resident"
    native_dir = output / "native"
    resident_dir.mkdir(parents=True, exist_ok=True)
    native_dir.mkdir(parents=True, exist_ok=True)
    patterns = [p for s in app.selections for p in s.procedures]
    report = {"application": app.name, "variant": app.variant, "entries": [], "directives": []}
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

    build.write_cmake(app, output)
    return app
