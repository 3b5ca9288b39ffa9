"""Host statements that touch arrays the entries keep on the device, and the blocks around them.

While an epoch is active the arrays that entries bind live on the device, and
host code that names them must see, and leave behind, current values. The
reference wraps every such host statement as it splices
(compiler/scopes/resident_splice.py:209-300, ``host_access_block``): arrays the
statements only read are brought up to date and keep their device copies
(``observe``); arrays they may change are handed to the host for the
statements and handed back after them (``host_modify`` / ``host_done``); an
array they deallocate is released first; where control can leave before the
hand-back, or an array is both used and deallocated, everything is published
instead; statements inside which entries run beside host uses of the same
arrays end the epoch. Each block asks the domain at run time which arrays it
holds (``held``), so outside an epoch a block costs one test of
``resident%active``.

The reference learns which statements touch which arrays from its compiler's
export. Here they are found in the free-form source text:

* the executable part of every program unit is split into statements (joined
  continuation lines; comments and string contents dropped) and constructs;
* an array is *bound* in a unit when the unit passes it to an entry (a call of
  a spliced procedure, at one of its array arguments) or to a procedure that
  passes the matching dummy on, transitively; a bound name the unit does not
  declare is a module variable, bound wherever it is named undeclared, and an
  internal procedure sees the bound names of its host;
* a statement writes an array it assigns to, reads into, passes to
  ``random_number`` or to a procedure whose dummy is not ``intent(in)``;
  ``deallocate`` releases it; any other mention reads it;
* a span is a run of consecutive statements (or whole constructs) that name
  bound arrays and call no entry; a construct that calls an entry is entered,
  and the conditions it evaluates once are read before it, while a
  ``do while`` condition that names a bound array ends the epoch (it is
  evaluated between entry calls).

A span is wrapped in a ``block``; a branch from outside into a wrapped span
would be illegal Fortran, so a span starting at a label that a ``go to``
names is refused with an error that says where.
"""

from __future__ import annotations

import re
from dataclasses import dataclass, field

from . import fortran
from .directives import Domain


class HostAccessError(ValueError):
    pass


_IDENT = re.compile(r"(?<![\w%])[a-z_]\w*")
_TYPE = re.compile(r"(?:integer|real|logical|complex|character|double\s*precision|double\s*complex|"
                   r"type\s*\([^)]*\)|class\s*\([^)]*\))(?:\s*\*\s*\d+)?(?:\s*\((?:[^()]|\([^()]*\))*\))?")
_ATTRIBUTE_STMT = re.compile(r"(allocatable|pointer|optional|target|dimension|contiguous|intent\s*\([^)]*\))\s+(.*)")
_CLOSE = re.compile(r"end\s*(do|if|select|where|forall|associate|block|critical)\b")
_MIDDLE = re.compile(r"(else\s*if\b|elsewhere\b|else\b|case\b|type\s+is\b|class\s+is\b|class\s+default\b|"
                     r"rank\s*\(|rank\s+default\b)")
_CONSTRUCT_NAME = re.compile(r"([a-z]\w*)\s*:\s*(?=(do|if|select|where|forall|associate|block|critical)\b)")
_GOTO = re.compile(r"go\s*to\s*\(?([\d,\s]+)\)?")


@dataclass
class Statement:
    first: int           # first line index
    last: int            # last line index (inclusive)
    code: str            # lower case; comments, string contents, label and construct name removed
    label: str = ""
    name: str = ""       # construct name
    role: str = "simple"  # simple, open, middle, close or directive (a residency directive line)
    construct: str = ""  # do, while, if, select, where, forall, associate, block or critical
    target: str = ""     # terminal label of a labelled DO


@dataclass
class Unit:
    proc: fortran.Procedure
    file: str
    lines: list
    dummies: list
    attrs: dict          # declared name -> set of attributes
    stmts: list
    host: "Unit | None" = None
    terminals: set = field(default_factory=set)   # statements that end labelled DO loops
    calls: list = field(default_factory=list)   # (callee, [actual argument code])

    @property
    def name(self) -> str:
        return self.proc.name.lower()

    def declares(self, name: str) -> bool:
        return name in self.attrs or name in self.dummies


@dataclass
class Block:
    """One edit: lines ``before`` ahead of statements first..last and ``after`` behind them (or the
    statements replaced by ``replace``)."""
    file: str
    first: int
    last: int
    kind: str            # observe, hand-over, release, publish or leave
    arrays: list
    before: str
    after: str = ""
    replace: str | None = None


# ---- text ------------------------------------------------------------------------------------

def _code(line: str, keep_strings: bool = False) -> str:
    """The line without its comment, every string literal emptied (or kept)."""
    out, quote = [], None
    for ch in line:
        if quote:
            if ch == quote:
                quote = None
                out.append(ch)
            elif keep_strings:
                out.append(ch)
            continue
        if ch in "'\"":
            quote = ch
            out.append(ch)
            continue
        if ch == "!":
            break
        out.append(ch)
    return "".join(out)


def _paren_end(s: str, i: int) -> int:
    """Index just past the parenthesis that closes the one at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j + 1
    return len(s)


def _split_top(s: str, sep: str = ",") -> list:
    parts, depth, start = [], 0, 0
    for j, ch in enumerate(s):
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == sep and depth == 0:
            parts.append(s[start:j])
            start = j + 1
    parts.append(s[start:])
    return [p.strip() for p in parts if p.strip()]


def _names(code: str) -> set:
    """Identifiers a statement mentions (not components, not keyword-argument names)."""
    code = re.sub(r"\s*%\s*", "%", code)
    out = set()
    for m in _IDENT.finditer(code):
        rest = code[m.end():].lstrip()
        if rest.startswith("=") and not rest.startswith("==") and not rest.startswith("=>"):
            continue  # a keyword argument, or an assignment target (classified on its own)
        out.add(m.group(0))
    return out


def _base(actual: str) -> str:
    """The array an actual argument or assignment target names: ``u`` for ``u`` or ``u(1:n, :, k)``."""
    m = re.fullmatch(r"([a-z_]\w*)\s*(\(.*\))?", actual.strip())
    return m.group(1) if m else ""


def _classify(st: Statement) -> None:
    code = st.code
    m = re.match(r"(\d+)\s+(.*)", code)
    if m:
        st.label, code = m.group(1), m.group(2)
    m = _CONSTRUCT_NAME.match(code)
    if m:
        st.name, code = m.group(1), code[m.end():]
    st.code = code
    if _CLOSE.match(code):
        st.role, st.construct = "close", _CLOSE.match(code).group(1)
    elif _MIDDLE.match(code):
        st.role = "middle"
    elif re.match(r"do\b", code):
        st.role, st.construct = "open", "do"
        lab = re.match(r"do\s+(\d+)\b", code)
        if lab:
            st.target = lab.group(1)
        if re.match(r"do\s*(\d+\s*,?\s*)?while\b", code):
            st.construct = "while"
    elif re.match(r"if\s*\(", code):
        if code[_paren_end(code, code.index("(")):].strip() == "then":
            st.role, st.construct = "open", "if"
    elif re.match(r"select\s*(case|type|rank)\b", code):
        st.role, st.construct = "open", "select"
    elif re.match(r"(where|forall)\s*\(", code):
        if not code[_paren_end(code, code.index("(")):].strip():
            st.role, st.construct = "open", "where" if code.startswith("where") else "forall"
    elif re.match(r"associate\s*\(", code):
        st.role, st.construct = "open", "associate"
    elif code == "block":
        st.role, st.construct = "open", "block"
    elif re.match(r"critical\b", code):
        st.role, st.construct = "open", "critical"


def statements(lines: list, start: int, end: int) -> list:
    """The statements of lines[start:end] (directives, comments and preprocessor lines skipped)."""
    out = []
    i = start
    while i < end:
        raw = lines[i]
        if re.match(r"\s*!\$fort\b", raw, re.I):
            out.append(Statement(i, i, raw.strip().lower(), role="directive"))
            i += 1
            continue
        code = "" if raw.lstrip().startswith("#") else _code(raw).strip()
        if not code:
            i += 1
            continue
        first = i
        while code.endswith("&") and i + 1 < end:
            i += 1
            nxt = _code(lines[i]).strip()
            code = code[:-1].rstrip() + " " + (nxt[1:] if nxt.startswith("&") else nxt).strip()
        code = code.rstrip("&").strip().lower()
        for part in _split_top(code, ";"):
            st = Statement(first, i, part)
            _classify(st)
            out.append(st)
        i += 1
    return out


def _terminals(stmts: list) -> set:
    """Indices of the statements that end labelled DO loops (an END DO there closes no other construct)."""
    return {_close_of(stmts, j, set()) for j, s in enumerate(stmts) if s.role == "open" and s.target}


def _close_of(stmts: list, k: int, terminals: set) -> int:
    """Index of the statement that closes the construct opened at k."""
    if stmts[k].target:
        for j in range(k + 1, len(stmts)):
            if stmts[j].label == stmts[k].target:
                return j
        raise HostAccessError(f"line {stmts[k].first + 1}: no statement labelled {stmts[k].target}")
    depth = 0
    for j in range(k, len(stmts)):
        s = stmts[j]
        if s.role == "open" and not s.target:
            depth += 1
        elif s.role == "close" and j not in terminals:
            depth -= 1
            if depth == 0:
                return j
    raise HostAccessError(f"line {stmts[k].first + 1}: construct is not closed")


# ---- units -----------------------------------------------------------------------------------

def _declare(code: str, attrs: dict) -> None:
    if "::" in code:
        left, right = code.split("::", 1)
        words = _split_top(left)
        kind = {"type"} if words and _TYPE.fullmatch(words[0]) else set()
        given = {re.sub(r"\s+", "", w) for w in (words[1:] if kind else words)} | kind
        for item in _split_top(right):
            m = re.match(r"[a-z_]\w*", item)
            if m:
                attrs.setdefault(m.group(0), set()).update(given)
        return
    m = _TYPE.match(code)
    if m and m.end() < len(code):
        for item in _split_top(code[m.end():]):
            n = re.match(r"[a-z_]\w*", item)
            if n:
                attrs.setdefault(n.group(0), set()).add("type")
        return
    m = _ATTRIBUTE_STMT.fullmatch(code)
    if m:
        for item in _split_top(m.group(2)):
            n = re.match(r"[a-z_]\w*", item)
            if n:
                attrs.setdefault(n.group(0), set()).add(re.sub(r"\s+", "", m.group(1)))


def _dummies(lines: list, proc: fortran.Procedure) -> list:
    header = " ".join(_code(lines[i]).strip().rstrip("&") for i in range(proc.header, proc.body)
                      if i == proc.header or _code(lines[i - 1]).rstrip().endswith("&")).lower()
    m = re.search(rf"\b{re.escape(proc.name.lower())}\s*\(", header)
    if proc.kind == "program" or not m:
        return []
    start = m.end() - 1
    return [a for a in (x.strip() for x in header[start + 1:_paren_end(header, start) - 1].split(",")) if a]


def _module_variables(lines: list) -> dict:
    """Names declared in the specification parts of the modules of a file."""
    attrs, inside = {}, False
    spec = []
    for n, raw in enumerate(lines):
        code = _code(raw).strip().lower()
        if re.match(r"module\s+(?!procedure\b)[a-z]\w*\s*$", code):
            inside = True
            continue
        if inside and (code == "contains" or re.match(r"end\s*module\b", code)):
            inside = False
        if inside and code:
            spec.append(n)
    for st in statements(lines, 0, len(lines)):
        if st.first in spec:
            _declare(st.code, attrs)
    return attrs


def _units(files: dict) -> list:
    units = []
    for name, text in files.items():
        lines = text.splitlines()
        for proc in fortran.procedures(text):
            attrs = {}
            for st in statements(lines, proc.header + 1, proc.body):
                _declare(st.code, attrs)
            stmts = statements(lines, proc.body, proc.end)
            units.append(Unit(proc, name, lines, _dummies(lines, proc), attrs, stmts, terminals=_terminals(stmts)))
    # an internal procedure's host: the innermost unit whose CONTAINS section holds its header
    for u in units:
        hosts = [h for h in units if h is not u and h.file == u.file and h.proc.end < u.proc.header
                 and _code(h.lines[h.proc.end]).strip().lower() == "contains" and _inside(h, u)]
        u.host = max(hosts, key=lambda h: h.proc.end, default=None)
    return units


def _inside(host: Unit, unit: Unit) -> bool:
    """Whether ``unit`` is one of ``host``'s internal procedures (before the host's own END)."""
    depth = 0
    for i in range(host.proc.end + 1, len(host.lines)):
        code = _code(host.lines[i]).strip().lower()
        if i == unit.proc.header:
            return depth == 0
        if re.match(r"((pure|elemental|impure|recursive|module|non_recursive)\s+)*"
                    r"(\w+(\([^)]*\))?\s+)?(subroutine|function)\s+\w+", code) and not code.startswith("end"):
            depth += 1
        elif re.match(r"end\s*(subroutine|function|program)\b", code) or code == "end":
            if depth == 0:
                return False
            depth -= 1
    return False


def _call(code: str):
    """(callee, [actual arguments]) of a CALL statement, or None."""
    m = re.match(r"call\s+([a-z_]\w*)\s*", code)
    if not m:
        return None
    rest = code[m.end():]
    args = _split_top(rest[1:_paren_end(rest, 0) - 1]) if rest.startswith("(") else []
    return m.group(1), args


def _action(code: str) -> str:
    """The action of a one-line IF (or the statement itself)."""
    if re.match(r"if\s*\(", code):
        end = _paren_end(code, code.index("("))
        rest = code[end:].strip()
        if rest and rest != "then":
            return rest
    return code


# ---- analysis --------------------------------------------------------------------------------

class Analysis:
    def __init__(self, files: dict, entries: dict, skip: set):
        """``files``: name -> text; ``entries``: bare procedure name -> array dummy names in declaration order
        (as [(position, name)]); ``skip``: qualified names of the spliced units."""
        self.units = [u for u in _units(files) if u.proc.qualified not in skip]
        self.entries = entries
        self.module_vars = {}
        for text in files.values():
            for k, v in _module_variables(text.splitlines()).items():
                self.module_vars.setdefault(k, set()).update(v)
        self.by_name = {}
        for u in self.units:
            self.by_name.setdefault(u.name, []).append(u)
            for st in u.stmts:
                c = _call(_action(st.code))
                if c:
                    u.calls.append(c)
        self.reach = set(entries)
        self.bound = {id(u): set() for u in self.units}
        self.shared = set()   # bound names no unit that binds them declares: module variables
        self._propagate()

    def _binding_dummies(self, callee: str) -> list:
        """(position, dummy) pairs through which a call of ``callee`` hands arrays to entries."""
        if callee in self.entries:
            return list(self.entries[callee])
        out = []
        for u in self.by_name.get(callee, []):
            out += [(n, d) for n, d in enumerate(u.dummies) if d in self.bound[id(u)]]
        return out

    def _propagate(self) -> None:
        changed = True
        while changed:
            changed = False
            for u in self.units:
                for callee, args in u.calls:
                    if callee in self.reach and u.name not in self.reach:
                        self.reach.add(u.name)
                        changed = True
                    targets = self._binding_dummies(callee)
                    if not targets:
                        continue
                    by_pos = {n for n, _ in targets}
                    by_key = {d for _, d in targets}
                    for n, a in enumerate(args):
                        key = re.match(r"([a-z_]\w*)\s*=(?!=)(.*)", a)
                        if key and key.group(1) in by_key:
                            name = _base(key.group(2))
                        elif not key and n in by_pos:
                            name = _base(a)
                        else:
                            continue
                        if not name:
                            continue
                        owner = self._owner(u, name)
                        if owner is None:
                            if name not in self.shared:
                                self.shared.add(name)
                                changed = True
                        elif name not in self.bound[id(owner)]:
                            self.bound[id(owner)].add(name)
                            changed = True

    def _owner(self, u: Unit, name: str):
        """The unit that declares ``name`` as seen from ``u`` (itself or a host), or None for a module variable."""
        while u is not None:
            if u.declares(name):
                return u
            u = u.host
        return None

    def bound_in(self, u: Unit) -> set:
        names = set(self.bound[id(u)])
        h = u.host
        while h is not None:
            names |= {n for n in self.bound[id(h)] if not u.declares(n)}
            h = h.host
        names |= {n for n in self.shared if self._owner(u, n) is None}
        return names

    def attrs_of(self, u: Unit, name: str) -> set:
        owner = self._owner(u, name)
        return owner.attrs.get(name, set()) if owner else self.module_vars.get(name, set())

    def calls_entry(self, st: Statement) -> bool:
        """Whether device work or a change of epoch happens at the statement (an entry path or a directive)."""
        if st.role == "directive":
            return True
        c = _call(_action(st.code))
        return bool(c) and c[0] in self.reach

    # -- what one statement does to the bound arrays --

    def access(self, u: Unit, code: str, bound: set, out: dict, flags: set, released: set) -> None:
        """Add {name: read|write} for the bound names ``code`` mentions, and the names it deallocates to
        ``released``; flags: leaves, moves."""
        def read(text):
            for n in _names(text) & bound:
                out.setdefault(n, "read")

        def write(n):
            if n in bound:
                out[n] = "write"

        if re.match(r"if\s*\(", code) and not code.endswith("then"):
            end = _paren_end(code, code.index("("))
            read(code[:end])
            action = code[end:].strip()
            if action:
                self.access(u, action, bound, out, flags, released)
            return
        if re.match(r"(return|stop|error\s*stop|go\s*to|exit|cycle)\b", code):
            flags.add("leaves")
        c = _call(code)
        if c:
            callee, args = c
            if callee in self.reach:
                targets = self._binding_dummies(callee)
                bypos, bykey = {n for n, _ in targets}, {d for _, d in targets}
                for n, a in enumerate(args):
                    key = re.match(r"([a-z_]\w*)\s*=(?!=)(.*)", a)
                    if (key and key.group(1) in bykey) or (not key and n in bypos):
                        continue
                    read(key.group(2) if key else a)
                return
            if callee == "move_alloc" and (_names(code) & bound):
                flags.add("moves")
            if any(a.startswith("*") for a in args):
                flags.add("leaves")
            dummies = self.by_name.get(callee, [])
            for n, a in enumerate(args):
                key = re.match(r"([a-z_]\w*)\s*=(?!=)(.*)", a)
                actual = key.group(2) if key else a
                name = _base(actual)
                if name in bound:
                    dummy = key.group(1) if key else None
                    intents = set()
                    for d in dummies:
                        nm = dummy or (d.dummies[n] if n < len(d.dummies) else None)
                        intents |= {x for x in d.attrs.get(nm, set()) if x.startswith("intent")}
                    if intents == {"intent(in)"}:
                        read(actual)
                    else:
                        write(name)
                        read(actual[len(name):])
                else:
                    read(actual)
            return
        m = re.match(r"(read)\s*(\(.*)?", code)
        if m and m.group(2) is not None:
            end = _paren_end(code, code.index("("))
            read(code[:end])
            for item in _split_top(code[end:]):
                write(_base(item)) if _base(item) in bound else read(item)
            return
        if re.match(r"read\s+[^=(]", code):
            items = _split_top(code[4:])
            for item in items[1:]:
                write(_base(item)) if _base(item) in bound else read(item)
            return
        m = re.match(r"deallocate\s*\(", code)
        if m:
            for item in _split_top(code[m.end():_paren_end(code, m.end() - 1) - 1]):
                name = _base(item)
                if name in bound:
                    released.add(name)
            return
        m = re.match(r"allocate\s*\(", code)
        if m:
            for item in _split_top(code[m.end():_paren_end(code, m.end() - 1) - 1]):
                key = re.match(r"(source|mold)\s*=(.*)", item)
                if key:
                    read(key.group(2))
            return
        if re.match(r"(where|forall)\s*\(", code):
            end = _paren_end(code, code.index("("))
            read(code[:end])
            code = code[end:].strip()
        m = re.match(r"([a-z_]\w*)\s*(\((?:[^()]|\((?:[^()]|\([^()]*\))*\))*\))?\s*=(?![=>])(.*)", code)
        if m:
            if m.group(1) in bound:
                write(m.group(1))
            read(m.group(2) or "")
            read(m.group(3))
            return
        read(code)


# ---- blocks ----------------------------------------------------------------------------------

def _guard(attrs: set, name: str, statement: str, margin: str) -> list:
    tests = [f"{t}({name})" for t, a in (("present", "optional"), ("allocated", "allocatable"),
                                         ("associated", "pointer")) if a in attrs]
    if not tests:
        return [f"{margin}{statement}"]
    if len(tests) == 1:
        return [f"{margin}if ({tests[0]}) {statement}"]
    lines = [f"{margin}if ({tests[0]}) then", *_guard(attrs - {"optional"}, name, statement, margin + "  "),
             f"{margin}endif"]
    return lines


def _handles(an: Analysis, u: Unit, var: str, names: list, margin: str, r: str) -> list:
    lines = [f"{margin}{var} = 0_c_int64_t"]
    for n, name in enumerate(names, 1):
        lines += _guard(an.attrs_of(u, name), name, f"{var}({n}) = {r}%held({name})", margin)
    return lines


def _precise(an: Analysis, u: Unit, ind: str, modes: dict, dom: Domain, released=()) -> tuple:
    """Observe what is read, then release what is deallocated, then hand over what is written."""
    r, p = dom.object, dom.prefix
    reads = sorted(n for n, m in modes.items() if m == "read")
    writes = sorted(n for n, m in modes.items() if m == "write")
    releases = sorted(released)
    head = [f"{ind}block", f"{ind}  use, intrinsic :: iso_c_binding, only: c_int64_t",
            f"{ind}  use {dom.module}, only: {r}", f"{ind}  logical :: {p}_host"]
    if reads:
        head.append(f"{ind}  integer(c_int64_t) :: {p}_seen({len(reads)})")
    if writes:
        head.append(f"{ind}  integer(c_int64_t) :: {p}_held({len(writes)})")
    head += [f"{ind}  {p}_host = {r}%active", f"{ind}  if ({p}_host) then"]
    if reads:
        head += _handles(an, u, f"{p}_seen", reads, ind + "    ", r) + [f"{ind}    call {r}%observe({p}_seen)"]
    for name in releases:
        head += _guard(an.attrs_of(u, name), name, f"call {r}%release_real({name})", ind + "    ")
    if writes:
        head += _handles(an, u, f"{p}_held", writes, ind + "    ", r) + [f"{ind}    call {r}%host_modify({p}_held)"]
    head.append(f"{ind}  endif")
    tail = ([f"{ind}  if ({p}_host) call {r}%host_done({p}_held)"] if writes else []) + [f"{ind}end block"]
    kind = "hand-over" if writes else "observe" if reads else "release"
    return kind, "\n".join(head) + "\n", "\n".join(tail) + "\n"


def _simple(ind: str, call: str, dom: Domain) -> str:
    return (f"{ind}block\n{ind}  use {dom.module}, only: {dom.object}\n"
            f"{ind}  if ({dom.object}%active) call {dom.object}%{call}()\n{ind}end block\n")


def _indent(line: str) -> str:
    return line[:len(line) - len(line.lstrip())]


def _referenced_labels(u: Unit) -> set:
    labels = set()
    for st in u.stmts:
        for m in _GOTO.finditer(st.code):
            labels |= {x.strip() for x in m.group(1).split(",") if x.strip()}
        if re.match(r"if\s*\(", st.code):
            rest = st.code[_paren_end(st.code, st.code.index("(")):]
            if re.fullmatch(r"\s*\d+\s*,\s*\d+\s*,\s*\d+\s*", rest):      # arithmetic IF
                labels |= {x.strip() for x in rest.split(",")}
        labels |= set(re.findall(r"[(,]\s*\*\s*(\d+)", st.code))           # alternate returns
        labels |= set(re.findall(r"\b(?:err|end|eor)\s*=\s*(\d+)", st.code))
    return labels


def blocks(an: Analysis, dom: Domain = Domain()) -> list:
    """Every block the units need, as edits of their files."""
    out = []
    for u in an.units:
        bound = an.bound_in(u)
        if not bound:
            continue
        labels = _referenced_labels(u)
        _walk(an, u, bound, labels, 0, len(u.stmts), out, dom)
    return out


def _touches(an, u, stmts, bound):
    """({name: read|write}, names deallocated, flags) over the statements."""
    modes, flags, released = {}, set(), set()
    for st in stmts:
        if st.role in ("close", "directive"):
            continue
        code = st.code
        if st.role == "middle":
            code = re.sub(r"^(else\s*if|case|type\s+is|class\s+is|rank)\s*", "", code)
        an.access(u, code, bound, modes, flags, released)
    if any(modes.get(n) == "write" for n in released):
        flags.add("moves")      # written and deallocated: nothing precise can hand it back
    return modes, released, flags


def _leaves(stmts: list) -> bool:
    """Whether control can leave the statements other than at their end."""
    names, depth = set(), 0
    for st in stmts:
        if st.role == "open" and st.construct in ("do", "while"):
            depth += 1
            if st.name:
                names.add(st.name)
        elif st.role == "close" and st.construct == "do":
            depth -= 1
        action = _action(st.code)
        m = re.match(r"(exit|cycle)\b\s*([a-z]\w*)?", action)
        if m:
            if (m.group(2) and m.group(2) not in names) or (not m.group(2) and depth <= 0):
                return True
        elif re.match(r"(return|stop|error\s*stop|go\s*to)\b", action) or \
                re.search(r"[(,]\s*\*\s*\d+", action):
            return True
    return False


def _wrap(an, u, bound, labels, stmts, out, dom):
    modes, released, flags = _touches(an, u, stmts, bound)
    if not modes and not released:
        return
    first, last = stmts[0], stmts[-1]
    if first.label and first.label in labels:
        raise HostAccessError(f"{u.file}:{first.first + 1}: statement {first.label} is a branch target and "
                              f"touches arrays kept on the device; move the label to a CONTINUE before it")
    lines = u.lines
    ind = _indent(lines[first.first])
    arrays = sorted(set(modes) | released)
    writes = any(m == "write" for m in modes.values())
    if "moves" in flags or (writes and _leaves(stmts)):
        out.append(Block(u.file, first.first, last.last, "publish", arrays, _simple(ind, "publish", dom)
                         .replace(f"{ind}end block\n", ""), f"{ind}end block\n"))
        return
    # a one-line IF whose condition names none of the arrays: the access belongs to the action
    if len(stmts) == 1 and first.first == last.last and first.role == "simple" and not first.label \
            and re.match(r"if\s*\(", first.code) and not (_names(first.code[:_paren_end(first.code, first.code.index(
                "("))]) & set(arrays)):
        raw = _code(lines[first.first], keep_strings=True).rstrip()
        start = raw.lower().index("if")
        end = _raw_paren_end(raw, raw.index("(", start))
        kind, before, after = _precise(an, u, ind + "  ", modes, dom, released)
        text = f"{raw[:end]} then\n{before}{ind}  {raw[end:].strip()}\n{after}{ind}endif\n"
        out.append(Block(u.file, first.first, last.last, kind, arrays, "", replace=text))
        return
    kind, before, after = _precise(an, u, ind, modes, dom, released)
    out.append(Block(u.file, first.first, last.last, kind, arrays, before, after))


def _raw_paren_end(raw: str, i: int) -> int:
    depth, quote = 0, None
    for j in range(i, len(raw)):
        ch = raw[j]
        if quote:
            quote = None if ch == quote else quote
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return j + 1
    return len(raw)


def _walk(an, u, bound, labels, lo, hi, out, dom):
    stmts = u.stmts
    run = []

    def flush():
        if run:
            _wrap(an, u, bound, labels, [x for k in run for x in k], out, dom)
            run.clear()

    k = lo
    while k < hi:
        st = stmts[k]
        if st.role == "open":
            e = _close_of(stmts, k, u.terminals)
            span = stmts[k:e + 1]
            if any(an.calls_entry(x) for x in span):
                flush()
                _enter(an, u, bound, labels, k, e, out, dom)
            else:
                if st.label and st.label in labels:
                    flush()
                run.append(span)
                if _leaves(span):
                    flush()
            k = e + 1
            continue
        if st.role in ("middle", "close"):
            k += 1
            continue
        if an.calls_entry(st):
            flush()
            modes, _, _ = _touches(an, u, [st], bound)
            reads = {n: m for n, m in modes.items() if m == "read"}
            if reads:
                ind = _indent(u.lines[st.first])
                kind, before, _ = _precise(an, u, ind, reads, dom)
                out.append(Block(u.file, st.first, st.first, kind, sorted(reads), before + f"{ind}end block\n"))
            k += 1
            continue
        modes, released, _ = _touches(an, u, [st], bound)
        touched = bool(modes or released)
        # a one-line IF whose condition names none of the arrays stands alone: its access goes inside it
        alone = touched and re.match(r"if\s*\(", st.code) is not None and not (
            _names(st.code[:_paren_end(st.code, st.code.index("("))]) & bound)
        if not touched or alone or (st.label and st.label in labels) or _leaves_any([st]):
            flush()
        if touched:
            run.append([st])
            if alone or _leaves_any([st]):
                flush()
        k += 1
    flush()


def _leaves_any(stmts):
    return any(re.match(r"(return|stop|error\s*stop|go\s*to|exit|cycle)\b", _action(s.code)) for s in stmts)


def _enter(an, u, bound, labels, k, e, out, dom):
    """A construct inside which entries run: its own conditions first, then its bodies."""
    stmts = u.stmts
    opener = stmts[k]
    heads = [opener] + [stmts[j] for j in _middles(stmts, k, e, u.terminals)]
    modes, _, _ = _touches(an, u, heads, bound)
    ind = _indent(u.lines[opener.first])
    if modes:
        if opener.label and opener.label in labels:
            raise HostAccessError(f"{u.file}:{opener.first + 1}: statement {opener.label} is a branch target and "
                                  f"touches arrays kept on the device; move the label to a CONTINUE before it")
        if opener.construct in ("while", "associate") or any(m != "read" for m in modes.values()):
            out.append(Block(u.file, opener.first, opener.first, "leave", sorted(modes),
                             _simple(ind, "end_epoch", dom)))
        else:
            kind, before, _ = _precise(an, u, ind, modes, dom)
            out.append(Block(u.file, opener.first, opener.first, kind, sorted(modes), before + f"{ind}end block\n"))
    cut = [k] + _middles(stmts, k, e, u.terminals) + [e]
    for a, b in zip(cut, cut[1:]):
        _walk(an, u, bound, labels, a + 1, b, out, dom)


def _middles(stmts, k, e, terminals):
    out, depth = [], 0
    for j in range(k, e + 1):
        s = stmts[j]
        if s.role == "open" and not s.target:
            depth += 1
        elif s.role == "close" and j not in terminals:
            depth -= 1
        elif s.role == "middle" and depth == 1:
            out.append(j)
    return out


def apply(text: str, edits: list) -> str:
    """The text with the blocks of one file put in place."""
    lines = text.splitlines(keepends=True)
    for b in sorted(edits, key=lambda b: (b.first, b.last), reverse=True):
        if b.replace is not None:
            lines[b.first:b.last + 1] = [b.replace]
        else:
            lines[b.first:b.last + 1] = [b.before, *lines[b.first:b.last + 1], b.after]
    return "".join(lines)


def wrap(files: dict, entries: dict, spliced: set, dom: Domain = Domain()) -> tuple:
    """Put host-access blocks into ``files`` (name -> text). Returns (new files, report records)."""
    an = Analysis(files, entries, spliced)
    found = blocks(an, dom)
    edits = {}
    for b in found:
        edits.setdefault(b.file, []).append(b)
    new = {name: apply(text, edits.get(name, [])) for name, text in files.items()}
    records = [{"file": b.file, "line": b.first + 1, "block": b.kind, "arrays": b.arrays}
               for b in sorted(found, key=lambda b: (b.file, b.first))]
    return new, records
