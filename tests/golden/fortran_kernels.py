"""Run the reference's Fortran loop kernels on numpy arrays (test infrastructure: golden-vector generator).

No Fortran compiler exists on the machines this project runs on, so the golden
vectors of the advection procedures are produced by executing the reference's
own source text with this interpreter of the free-form Fortran subset those
kernels and their test programs are written in: modules, programs, subroutines
and functions, type declarations with intent, parameter, allocatable and
explicit or assumed lower bounds, ALLOCATE and DEALLOCATE, DO loops, CALL,
scalar, element, section and whole-array assignment, WRITE of values (kept, not
formatted), the intrinsics sin, cos, exp, log, sqrt, abs, real, dble, min and
max, and expressions of numeric literals (kind suffixes and d exponents),
names, array elements, unary and binary + - * / ** and parentheses. The C
preprocessor's #define, #ifdef, #ifndef, #else and #endif are applied first,
with the caller's definitions. OpenMP directives are comments.

Arithmetic is IEEE binary64 with round-to-nearest, evaluated in the order the
Fortran expression tree gives (left to right within one precedence level,
parentheses kept, unary minus below * and /, no contraction): the semantics of
the reference's strict native build (-ffp-contract=off, no value-changing
reassociation). A perfect DO nest whose body only assigns scalars and array
elements, and reads every array it writes at exactly the written element, is
evaluated for all iterations at once with numpy (elementwise, so each element
sees the same operations in the same order); any other loop runs iteration by
iteration.

Arrays are numpy arrays in C order with the Fortran index order reversed
(element (i, j, k) of a Fortran array is ``a[k - l3, j - l2, i - l1]``).
"""

from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

# ---- lexing -----------------------------------------------------------------------------------------

_TOKEN = re.compile(r"""
    (?P<str>'[^']*'|"[^"]*")
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?(_[a-z_]\w*)?)
  | (?P<name>[a-z_]\w*)
  | (?P<op>\*\*|::|[-+*/(),=:%])
  | (?P<space>\s+)
""", re.X | re.I)


def _tokens(text: str) -> list[str]:
    out, pos = [], 0
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise SyntaxError(f"cannot read Fortran text at: {text[pos:pos + 30]!r}")
        pos = m.end()
        if m.lastgroup == "str":
            out.append(m.group(0))
        elif m.lastgroup != "space":
            out.append(m.group(0).lower())
    return out


def _preprocess(source: str, defines: dict) -> str:
    """#define / #ifdef / #ifndef / #else / #endif, then the macros substituted as whole words."""
    macros = {k.lower(): str(v) for k, v in defines.items()}
    out, active = [], [True]
    for raw in source.splitlines():
        text = raw.strip()
        if text.startswith("#"):
            words = text[1:].split()
            if not words:
                continue
            word = words[0]
            if word in ("ifdef", "ifndef"):
                present = words[1].lower() in macros
                active.append(active[-1] and (present if word == "ifdef" else not present))
            elif word == "else":
                active[-1] = active[-2] and not active[-1]
            elif word == "endif":
                active.pop()
            elif word == "define" and active[-1]:
                macros[words[1].lower()] = " ".join(words[2:])
            continue
        if not active[-1]:
            continue
        for name, value in macros.items():
            raw = re.sub(rf"\b{re.escape(name)}\b", value, raw, flags=re.I)
        out.append(raw)
    return "\n".join(out)


def _strip_comment(line: str) -> str:
    quote = None
    for n, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "!":
            return line[:n]
    return line


def _statements(source: str) -> list[str]:
    """Free-form lines joined across '&' continuations, comments (and OpenMP sentinels) removed."""
    lines, pending = [], ""
    for raw in source.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip() or line.lstrip().startswith("#"):  # blank, comment or preprocessor line
            continue
        text = line.strip()
        if pending:
            text = text[1:].lstrip() if text.startswith("&") else text
        if text.endswith("&"):
            pending += text[:-1] + " "
            continue
        lines.append(pending + text)
        pending = ""
    return lines


# ---- syntax tree ------------------------------------------------------------------------------------

@dataclass
class Num:
    value: float | int


@dataclass
class Name:
    name: str


@dataclass
class Ref:
    name: str
    args: list


@dataclass
class Section:
    lower: object  # None: the array's lower bound
    upper: object  # None: its upper bound


@dataclass
class Unary:
    op: str
    operand: object


@dataclass
class Bin:
    op: str
    left: object
    right: object


@dataclass
class Assign:
    target: object
    value: object


@dataclass
class Do:
    var: str
    lower: object
    upper: object
    body: list


@dataclass
class Call:
    name: str
    args: list


@dataclass
class Allocate:
    items: list  # (name, [subscripts]) pairs


@dataclass
class Write:
    values: list


@dataclass
class Decl:
    intent: str | None = None
    array: bool = False
    lower: tuple = ()
    parameter: object = None


@dataclass
class Subroutine:
    name: str
    args: list
    decls: dict = field(default_factory=dict)
    body: list = field(default_factory=list)
    result: str | None = None  # a function's result variable


class _Expr:
    def __init__(self, toks: list[str]):
        self.t, self.i = toks, 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else None

    def take(self, want=None):
        tok = self.peek()
        if want is not None and tok != want:
            raise SyntaxError(f"expected {want!r}, found {tok!r} in {' '.join(self.t)}")
        self.i += 1
        return tok

    def expr(self):
        # level-2 expression: [sign] term { (+|-) term }; a leading sign applies to the first term
        sign = self.take() if self.peek() in ("+", "-") else None
        node = self.term()
        if sign == "-":
            node = Unary("-", node)
        while self.peek() in ("+", "-"):
            op = self.take()
            node = Bin(op, node, self.term())
        return node

    def term(self):
        node = self.power()
        while self.peek() in ("*", "/"):
            op = self.take()
            node = Bin(op, node, self.power())
        return node

    def power(self):
        base = self.primary()
        if self.peek() == "**":
            self.take()
            return Bin("**", base, self.power())
        return base

    def primary(self):
        tok = self.take()
        if tok == "(":
            node = self.expr()
            self.take(")")
            return node
        if tok in ("+", "-"):  # a signed operand after * or / (accepted as gfortran does)
            return Unary(tok, self.power())
        if re.match(r"^(\d|\.\d)", tok):
            text = tok.split("_", 1)[0].replace("d", "e")
            return Num(float(text) if re.search(r"[.e]", text) else int(text))
        if self.peek() == "(":
            self.take("(")
            args = []
            if self.peek() != ")":
                args.append(self.subscript())
                while self.peek() == ",":
                    self.take(",")
                    args.append(self.subscript())
            self.take(")")
            return Ref(tok, args)
        return Name(tok)

    def subscript(self):
        lower = None if self.peek() == ":" else self.expr()
        if self.peek() != ":":
            return lower
        self.take(":")
        upper = None if self.peek() in (",", ")") else self.expr()
        return Section(lower, upper)


def _parse_expr(toks):
    p = _Expr(toks)
    node = p.expr()
    if p.peek() is not None:
        raise SyntaxError(f"unexpected {p.peek()!r} in {' '.join(toks)}")
    return node


def _split_top(toks, sep=","):
    parts, depth, cur = [], 0, []
    for tok in toks:
        if tok == "(":
            depth += 1
        elif tok == ")":
            depth -= 1
        if tok == sep and depth == 0:
            parts.append(cur)
            cur = []
        else:
            cur.append(tok)
    parts.append(cur)
    return parts


class Source:
    """The subroutines of one or more Fortran source files."""

    def __init__(self, *texts: str, defines: dict | None = None):
        self.subroutines: dict[str, Subroutine] = {}
        self.programs: dict[str, Subroutine] = {}
        self.parameters: dict[str, object] = {}
        self.globals: dict[str, object] = {}  # module variables (the caller sets them before a call)
        self.output: list = []                # the values WRITE statements produced, in order
        self.program_arrays: dict = {}        # the arrays of the last program run (DEALLOCATE keeps them here)
        for text in texts:
            self._read(_statements(_preprocess(text, defines or {})))

    def _read(self, lines):
        stack: list[list] = []
        current: Subroutine | None = None
        for line in lines:
            toks = _tokens(line)
            head = toks[0]
            if head == "module" and len(toks) == 2:
                continue
            if head in ("contains", "implicit", "private", "public", "use"):
                continue
            if head == "end":
                what = toks[1] if len(toks) > 1 else ""
                if what in ("do",):
                    loop = stack.pop()
                    continue
                if what in ("subroutine", "function"):
                    self.subroutines[current.name] = current
                    current = None
                elif what == "program":
                    self.programs[current.name] = current
                    current = None
                continue
            if head == "enddo":
                stack.pop()
                continue
            if head == "program":
                current = Subroutine(toks[1], [])
                stack = [current.body]
                continue
            if head == "allocate":
                items = []
                for item in _split_top(toks[2:-1]):
                    ref = _parse_expr(item)
                    items.append((ref.name, ref.args))
                stack[-1].append(Allocate(items))
                continue
            if head == "deallocate":
                continue
            if head == "write":
                close = next(n for n in range(1, len(toks)) if toks[n] == ")" and
                             toks[:n + 1].count("(") == toks[:n + 1].count(")"))
                stack[-1].append(Write([_parse_expr(a) for a in _split_top(toks[close + 1:]) if a]))
                continue
            if head == "subroutine":
                name = toks[1]
                args = [a[0] for a in _split_top(toks[3:-1]) if a] if len(toks) > 3 else []
                current = Subroutine(name, args)
                stack = [current.body]
                continue
            if "function" in toks and current is None and "::" not in toks:
                f = toks.index("function")
                name = toks[f + 1]
                close = toks.index(")", f)
                args = [a[0] for a in _split_top(toks[f + 3:close]) if a]
                result = toks[toks.index("result") + 2] if "result" in toks[close:] else name
                current = Subroutine(name, args, result=result)
                stack = [current.body]
                continue
            if "::" in toks:
                self._declare(current, toks)
                continue
            if head == "do" and len(toks) > 2 and toks[2] == "=":
                bounds = _split_top(toks[3:])
                loop = Do(toks[1], _parse_expr(bounds[0]), _parse_expr(bounds[1]), [])
                stack[-1].append(loop)
                stack.append(loop.body)
                continue
            if head == "call":
                args = [_parse_expr(a) for a in _split_top(toks[3:-1]) if a] if len(toks) > 3 else []
                stack[-1].append(Call(toks[1], args))
                continue
            eq = _split_top(toks, "=")
            if len(eq) == 2 and current is not None:
                stack[-1].append(Assign(_parse_expr(eq[0]), _parse_expr(eq[1])))
                continue
            raise SyntaxError(f"statement outside the supported subset: {line}")

    def _declare(self, sub, toks):
        cut = toks.index("::")
        spec = _split_top(toks[:cut])
        attrs = [a for a in spec[1:]]
        decl = Decl()
        for a in attrs:
            if a and a[0] == "intent":
                decl.intent = a[2]
            if a and a[0] == "parameter":
                decl.parameter = True
            if a and a[0] == "allocatable":
                decl.array = True
        for entity in _split_top(toks[cut + 1:]):
            name = entity[0]
            d = Decl(decl.intent, decl.array, (), None)
            if len(entity) > 1 and entity[1] == "(":
                dims = _split_top(entity[2:entity.index(")") if ")" in entity else len(entity)])
                d.array = True
                lows = []
                for dim in dims:
                    colon = dim.index(":") if ":" in dim else None
                    lows.append(_parse_expr(dim[:colon]) if colon else Num(1))
                d.lower = tuple(lows)
            if decl.parameter and "=" in entity:
                d.parameter = _parse_expr(entity[entity.index("=") + 1:])
                if sub is None:
                    self.parameters[name] = d.parameter
            elif sub is None:  # a module variable, with its initial value if it has one
                self.globals[name] = self._eval(_parse_expr(entity[entity.index("=") + 1:]), {}) \
                    if "=" in entity else None
            if sub is not None:
                sub.decls[name] = d

    # ---- execution ----------------------------------------------------------------------------

    def call(self, name: str, *args):
        """Run subroutine `name`; arrays (numpy, C order, Fortran indices reversed) are updated in place.
        A function's result is returned."""
        sub = self.subroutines[name.lower()]
        if len(args) != len(sub.args):
            raise TypeError(f"{name} takes {len(sub.args)} arguments")
        env = {}
        for name, d in sub.decls.items():  # the unit's own named constants
            if d.parameter is not None and d.parameter is not True and name not in sub.args:
                env[name] = self._eval(d.parameter, env)
        for formal, actual in zip(sub.args, args):
            d = sub.decls.get(formal, Decl())
            if d.array:
                lows = tuple(int(self._eval(lo, env)) for lo in d.lower)
                env[formal] = ("array", actual, lows)
            else:
                env[formal] = actual
        self._run(sub.body, env)
        return env.get(sub.result) if sub.result else None

    def run_program(self, name: str) -> list:
        """Run a main program; returns (and keeps in ``output``) the values its WRITE statements produced."""
        self.output = []
        prog = self.programs[name.lower()]
        env = {}
        for nm, d in prog.decls.items():
            if d.parameter is not None and d.parameter is not True:
                env[nm] = self._eval(d.parameter, env)
        self._run(prog.body, env)
        self.program_arrays = {k: v[1] for k, v in env.items() if isinstance(v, tuple)}
        return self.output

    def _run(self, body, env):
        for st in body:
            if isinstance(st, Assign):
                self._assign(st.target, self._eval(st.value, env), env)
            elif isinstance(st, Do):
                if not self._vectorised(st, env):
                    lo, hi = int(self._eval(st.lower, env)), int(self._eval(st.upper, env))
                    for v in range(lo, hi + 1):
                        env[st.var] = v
                        self._run(st.body, env)
            elif isinstance(st, Allocate):
                for name, dims in st.items:
                    lows, extents = [], []
                    for d in dims:
                        if isinstance(d, Section):
                            lo, hi = int(self._eval(d.lower, env)), int(self._eval(d.upper, env))
                        else:
                            lo, hi = 1, int(self._eval(d, env))
                        lows.append(lo)
                        extents.append(hi - lo + 1)
                    env[name] = ("array", np.full(tuple(reversed(extents)), np.nan), tuple(lows))
            elif isinstance(st, Write):
                for v in st.values:
                    self.output.append(float(self._eval(v, env)))
            elif isinstance(st, Call):
                actual = []
                for a in st.args:
                    if isinstance(a, Name) and isinstance(env.get(a.name), tuple):
                        actual.append(env[a.name][1])
                    else:
                        actual.append(self._eval(a, env))
                self.call(st.name, *actual)

    def _index(self, args, lows, env):
        idx = []
        for a, lo in zip(reversed(args), reversed(lows)):
            if isinstance(a, Section):
                first = 0 if a.lower is None else self._eval(a.lower, env) - lo
                last = None if a.upper is None else self._eval(a.upper, env) - lo + 1
                idx.append(slice(first, last))
            else:
                idx.append(self._eval(a, env) - lo)
        return tuple(idx)

    def _assign(self, target, value, env):
        if isinstance(target, Name):
            entry = env.get(target.name)
            if isinstance(entry, tuple):  # the whole array
                entry[1][...] = value
            else:
                env[target.name] = value
            return
        kind, arr, lows = env[target.name]
        arr[self._index(target.args, lows, env)] = value

    def _eval(self, node, env):
        if isinstance(node, Num):
            return node.value
        if isinstance(node, Name):
            if node.name in env:
                return env[node.name]
            if self.globals.get(node.name) is not None:
                return self.globals[node.name]
            if node.name in self.parameters:
                return self._eval(self.parameters[node.name], env)
            raise NameError(node.name)
        if isinstance(node, Ref):
            entry = env.get(node.name)
            if not isinstance(entry, tuple) and node.name in self.subroutines:
                actual = [env[a.name][1] if isinstance(a, Name) and isinstance(env.get(a.name), tuple)
                          else self._eval(a, env) for a in node.args]
                return self.call(node.name, *actual)
            if not isinstance(entry, tuple) and node.name in _INTRINSICS:
                return _INTRINSICS[node.name](self, node.args, env)
            if not isinstance(entry, tuple):
                raise NameError(f"{node.name} is not an array here")
            _, arr, lows = entry
            return arr[self._index(node.args, lows, env)]
        if isinstance(node, Unary):
            v = self._eval(node.operand, env)
            return -v if node.op == "-" else v
        a, b = self._eval(node.left, env), self._eval(node.right, env)
        if node.op in ("*", "/", "+", "-") and _mixed(a, b):
            a, b = _real(a), _real(b)
        if node.op == "+":
            return a + b
        if node.op == "-":
            return a - b
        if node.op == "*":
            return a * b
        if node.op == "/":
            if _is_int(a) and _is_int(b):
                return int(a / b) if not isinstance(a, np.ndarray) else np.trunc(a / b).astype(np.int64)
            return a / b
        return a ** b

    # ---- a perfect nest evaluated for every iteration at once ----------------------------------

    def _vectorised(self, loop: Do, env) -> bool:
        nest, body = [loop], loop.body
        while len(body) == 1 and isinstance(body[0], Do):
            nest.append(body[0])
            body = body[0].body
        if not body or not all(isinstance(st, Assign) for st in body):
            return False
        loop_vars = [d.var for d in nest]
        written = {st.target.name for st in body if isinstance(st.target, Ref)}
        exact = [Name(v) for v in reversed(loop_vars)]  # element (i, j, k) for a k-j-i nest

        def refs(node, out):
            if isinstance(node, Ref):
                out.append(node)
                for a in node.args:
                    refs(a, out)
            elif isinstance(node, Unary):
                refs(node.operand, out)
            elif isinstance(node, Bin):
                refs(node.left, out)
                refs(node.right, out)
            return out

        for st in body:
            for r in refs(st.value, []) + ([st.target] if isinstance(st.target, Ref) else []):
                if r.name in written and r.args != exact:
                    return False  # an array read or written at another element than the one written
                if r.name in self.subroutines and any(isinstance(a, Name) and a.name in written for a in r.args):
                    return False  # a function given an array the nest writes
        ranges = []
        for n, d in enumerate(nest):
            lo, hi = int(self._eval(d.lower, env)), int(self._eval(d.upper, env))
            shape = [1] * len(nest)
            shape[n] = max(0, hi - lo + 1)
            ranges.append(np.arange(lo, hi + 1, dtype=np.int64).reshape(shape))
        if any(r.size == 0 for r in ranges):
            return True
        saved = {v: env.get(v) for v in loop_vars}
        for v, r in zip(loop_vars, ranges):
            env[v] = r
        full = tuple(int(r.size) for r in ranges)
        for st in body:
            value = self._eval(st.value, env)
            if isinstance(st.target, Ref):
                self._assign(st.target, np.broadcast_to(value, full), env)
            else:
                env[st.target.name] = np.broadcast_to(value, full)
        for v in loop_vars:
            if saved[v] is None:
                env.pop(v, None)
            else:
                env[v] = saved[v]
        return True


def _is_int(v) -> bool:
    return isinstance(v, int) or (isinstance(v, np.ndarray) and v.dtype.kind in "iu")


def _mixed(a, b) -> bool:
    return _is_int(a) != _is_int(b)


def _real(v):
    if isinstance(v, int):
        return float(v)
    if isinstance(v, np.ndarray) and v.dtype.kind in "iu":
        return v.astype(np.float64)
    return v


def _elementwise(fn):
    """A libm function applied value by value (the C library's results, as a compiled Fortran program gets)."""
    def apply(v):
        if isinstance(v, np.ndarray):
            return np.vectorize(fn, otypes=[np.float64])(v.astype(np.float64))
        return fn(float(v))
    return apply


def _intrinsic(fn):
    return lambda src, args, env: fn(src._eval(args[0], env))


def _real_intrinsic(src, args, env):  # real(x [, kind]) / dble(x): the kind is double precision here
    v = src._eval(args[0], env)
    return v.astype(np.float64) if isinstance(v, np.ndarray) else float(v)


def _fold(op):
    def apply(src, args, env):
        vals = [src._eval(a, env) for a in args]
        out = vals[0]
        for v in vals[1:]:
            out = op(out, v)
        return out
    return apply


_INTRINSICS = {
    "sin": _intrinsic(_elementwise(math.sin)), "cos": _intrinsic(_elementwise(math.cos)),
    "exp": _intrinsic(_elementwise(math.exp)), "log": _intrinsic(_elementwise(math.log)),
    "sqrt": _intrinsic(_elementwise(math.sqrt)), "abs": _intrinsic(np.abs),
    "real": _real_intrinsic, "dble": _real_intrinsic,
    "max": _fold(np.maximum), "min": _fold(np.minimum),
    "kind": lambda src, args, env: 8,  # kinds only name the precision; every real here is binary64
}
