"""Run a subset of fixed-form Fortran 77/90 on numpy by translating it to Python.

This is test infrastructure for generating golden vectors: it executes the
reference's own Fortran sources (no Fortran compiler exists in the
development image) so that the CPU oracle and the GPU kernels can be checked
against what the reference code itself computes.  The translated code is kept
in memory only.

Supported: fixed-form source with ``include``, implicit typing, ``integer`` /
``real*8`` / ``logical`` / ``character`` / ``dimension`` / ``parameter`` /
``common`` declarations (common and module variables live in one global
namespace), automatic and allocatable arrays, F90 array syntax and sections,
vector subscripts, ``do``/``enddo`` and labelled ``do``/``continue`` loops,
block and logical ``if``, ``cycle``/``exit``/``return``, ``call`` with
by-reference scalars (copy-in/copy-out) and by-reference arrays (numpy views,
with sequence association by Fortran-order reshape), derived-type
components ``a(i)%p`` of module arrays, and the intrinsics the solver uses.
Single-precision literals (``0.1`` without a ``d`` exponent) and ``real()``/
``float()`` conversions are rounded to float32 as a Fortran compiler does.
Anything else raises ``FortranUnsupported`` when it is executed.
"""
from __future__ import annotations

import functools
import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


class FortranUnsupported(RuntimeError):
    pass


class FortranStop(RuntimeError):
    pass


# --------------------------------------------------------------------------- source reading

def _strip_comment(s: str) -> str:
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def _lower(s: str) -> str:
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


def read_fixed(path: Path, search: list[Path], skip_includes=("mpif.h", "auxmpi.h")) -> list[tuple[int | None, str, str]]:
    """Logical statements (label, text, where) of a fixed-form file, includes expanded."""
    stmts: list[list] = []
    raw = path.read_text(errors="replace").splitlines()
    for ln, line in enumerate(raw, 1):
        where = f"{path.name}:{ln}"
        if not line.strip():
            continue
        if line[0] in "cC*!#":
            continue
        lead = len(line.expandtabs(8)) - len(line.expandtabs(8).lstrip())
        if line.lstrip().startswith("!") and lead != 5:
            continue  # '!' outside column 6 as the first character: a comment line
        if line.startswith("\t"):
            # tab format: a digit right after the tab marks a continuation
            body = line[1:]
            if body[:1].isdigit() and body[:1] != "0" and stmts:
                stmts[-1][1] += " " + _strip_comment(body[1:])
                continue
            label, cont, text = "", " ", body
        else:
            line = line.expandtabs(8)
            label, cont, text = line[:5], line[5:6], line[6:]
        text = _strip_comment(text).rstrip()
        text = re.sub(r"\.\s*(eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\s*\.", r".\1.", text,
                      flags=re.I)
        if cont not in (" ", "0", "") and stmts:
            stmts[-1][1] += " " + text
            continue
        if not text.strip() and not label.strip():
            continue
        lab = int(label) if label.strip().isdigit() else None
        stmts.append([lab, text, where])
    out = []
    for lab, text, where in stmts:
        t = _lower(text).strip()
        m = re.match(r"include\s*['\"]([^'\"]+)['\"]", t)
        if m:
            name = m.group(1)
            if name in skip_includes:
                continue
            for d in [path.parent] + search:
                if (d / name).exists():
                    out.extend(read_fixed(d / name, search, skip_includes))
                    break
            else:
                raise FileNotFoundError(f"{where}: include {name}")
            continue
        # split on ';' outside strings
        parts, cur, q = [], [], None
        for ch in t:
            if q:
                cur.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                cur.append(ch)
            elif ch == ";":
                parts.append("".join(cur))
                cur = []
            else:
                cur.append(ch)
        parts.append("".join(cur))
        for i, p in enumerate(parts):
            if p.strip():
                out.append((lab if i == 0 else None, p.strip(), where))
    return out


# --------------------------------------------------------------------------- expressions

_DOTOPS = ("eq", "ne", "lt", "le", "gt", "ge", "and", "or", "not", "eqv", "neqv", "true", "false")
_TOK = re.compile(r"""
    (?P<ws>\s+)
  | (?P<dot>\.(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
  | (?P<num>(?:\d+\.(?!(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv)\.)\d*|\.\d+|\d+)(?:[ed][+-]?\d+)?(?:_\w+)?)
  | (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
  | (?P<id>[a-z_][a-z0-9_$]*)
  | (?P<op>\*\*|//|==|/=|<=|>=|\(/|/\)|[-+*/()<>=,:%])
""", re.X)


def tokenize(s: str) -> list[tuple[str, str]]:
    toks, i = [], 0
    while i < len(s):
        m = _TOK.match(s, i)
        if not m:
            raise FortranUnsupported(f"cannot tokenize {s[i:]!r} in {s!r}")
        i = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        toks.append((k, m.group()))
    return toks


@dataclass
class Num:
    text: str


@dataclass
class Str:
    text: str


@dataclass
class Name:
    name: str


@dataclass
class Ref:  # name(args) -- array element/section or function call
    name: str
    args: list


@dataclass
class Comp:  # base % field
    base: object
    field: str


@dataclass
class Slice:
    lo: object
    hi: object
    step: object = None


@dataclass
class Un:
    op: str
    e: object


@dataclass
class Bin:
    op: str
    a: object
    b: object


@dataclass
class ArrCons:
    items: list


@dataclass
class Logic:
    value: bool


class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise FortranUnsupported(f"expected {val!r}, got {tok[1]!r} in {self.t}")
        self.i += 1
        return tok

    def done(self):
        return self.i >= len(self.t)

    # precedence climbing, lowest first
    def expr(self):
        return self.eqv()

    def eqv(self):
        a = self.lor()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.take()[1]
            a = Bin(op, a, self.lor())
        return a

    def lor(self):
        a = self.land()
        while self.peek()[1] == ".or.":
            self.take()
            a = Bin(".or.", a, self.land())
        return a

    def land(self):
        a = self.lnot()
        while self.peek()[1] == ".and.":
            self.take()
            a = Bin(".and.", a, self.lnot())
        return a

    def lnot(self):
        if self.peek()[1] == ".not.":
            self.take()
            return Un(".not.", self.lnot())
        return self.rel()

    _REL = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
            "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}

    def rel(self):
        a = self.concat()
        if self.peek()[1] in self._REL:
            op = self._REL[self.take()[1]]
            a = Bin(op, a, self.concat())
        return a

    def concat(self):
        a = self.add()
        while self.peek()[1] == "//":
            self.take()
            a = Bin("//", a, self.add())
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.mul()
            a = Un(op, a)
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = Bin(op, a, self.mul())
        return a

    def mul(self):
        a = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = Bin(op, a, self.power())
        return a

    def power(self):
        a = self.postfix()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):
                op = self.take()[1]
                return Bin("**", a, Un(op, self.power()))
            return Bin("**", a, self.power())  # right associative
        return a

    def postfix(self):
        a = self.primary()
        while self.peek()[1] == "%":
            self.take()
            f = self.take()[1]
            if self.peek()[1] == "(":
                raise FortranUnsupported("indexed component")
            a = Comp(a, f)
        return a

    def primary(self):
        k, v = self.peek()
        if k == "num":
            self.take()
            return Num(v)
        if k == "str":
            self.take()
            return Str(v)
        if k == "dot" and v in (".true.", ".false."):
            self.take()
            return Logic(v == ".true.")
        if v == "(/":
            self.take()
            items = [self.expr()]
            while self.peek()[1] == ",":
                self.take()
                items.append(self.expr())
            self.take("/)")
            return ArrCons(items)
        if v == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return e
        if k == "id":
            self.take()
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    args.append(self.arg())
                    while self.peek()[1] == ",":
                        self.take()
                        args.append(self.arg())
                self.take(")")
                return Ref(v, args)
            return Name(v)
        raise FortranUnsupported(f"unexpected token {v!r} in {self.t}")

    def arg(self):
        # section a:b[:s], keyword arg name=value (kept as a tuple)
        if self.peek()[0] == "id" and self.peek(1)[1] == "=" :
            name = self.take()[1]
            self.take("=")
            return ("kw", name, self.expr())
        lo = None
        if self.peek()[1] != ":":
            lo = self.expr()
            if self.peek()[1] != ":":
                return lo
        self.take(":")
        hi = None
        if self.peek()[1] not in (",", ")", ":"):
            hi = self.expr()
        st = None
        if self.peek()[1] == ":":
            self.take()
            st = self.expr()
        return Slice(lo, hi, st)


def parse_expr(s: str):
    p = Parser(tokenize(s))
    e = p.expr()
    if not p.done():
        raise FortranUnsupported(f"trailing tokens in {s!r}")
    return e


# --------------------------------------------------------------------------- symbols

@dataclass
class Var:
    name: str
    type: str = ""           # 'i' 'r' 'l' 'c' ('' = implicit, resolved later)
    dims: list | None = None  # list of (lo, hi) AST (hi None = '*', lo None and hi None = ':')
    scope: str = "local"     # local | dummy | global | param
    alloc: bool = False
    value: object = None     # parameter value (python number)
    obj: bool = False        # derived-type array (module pointer arrays)


@dataclass
class Unit:
    kind: str
    name: str
    args: list
    body: list                 # (label, text, where) of executable statements
    decls: list                # (text, where)
    rtype: str = ""
    syms: dict = field(default_factory=dict)
    implicit: dict = field(default_factory=dict)
    uses: list = field(default_factory=list)
    src: str = ""


_TYPE_RE = re.compile(r"^(integer|real|double\s*precision|logical|character|complex)\s*(\*\s*\(?\s*[\d*]+\s*\)?|\(\s*(?:kind|len)?\s*=?\s*[\w*]+\s*\))?\s*")


def _split_top(s: str, sep=",") -> list[str]:
    out, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            out.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        out.append("".join(cur).strip())
    return out


def _tchar(tname: str) -> str:
    tname = tname.replace(" ", "")
    return {"integer": "i", "real": "r", "doubleprecision": "r", "logical": "l", "character": "c",
            "complex": "z"}[tname]


class Program:
    """A set of Fortran units, translated lazily into Python functions sharing one global namespace."""

    def __init__(self, search: list[Path]):
        self.search = [Path(p) for p in search]
        self.units: dict[str, Unit] = {}
        self.G = _Globals()
        self.F = _Funcs(self)
        self.stubs: dict[str, object] = {}
        self.global_syms: dict[str, Var] = {}
        self.params: dict[str, object] = {}
        self.modules: dict[str, dict[str, Var]] = {}
        self._compiled: dict[str, object] = {}

    # ---- loading
    def load(self, path):
        path = Path(path)
        stmts = read_fixed(path, self.search)
        cur = None
        for lab, text, where in stmts:
            m = re.match(r"^(?:(?:recursive\s+)?(?:(integer|real\*8|real|double\s*precision|logical)\s+)?"
                         r"(subroutine|function))\s+(\w+)\s*(?:\((.*)\))?\s*$", text)
            if cur is None:
                if m:
                    args = [a.strip() for a in (m.group(4) or "").split(",") if a.strip()]
                    cur = Unit(m.group(2), m.group(3), args, [], [], rtype=m.group(1) or "", src=where)
                    continue
                if re.match(r"^(module|program|block\s*data)\b", text):
                    cur = Unit("skip", text, [], [], [], src=where)
                    continue
                raise FortranUnsupported(f"{where}: statement outside a unit: {text}")
            if re.match(r"^end\s*(subroutine|function|module|program)?\b(\s+\w+)?\s*$", text) and not \
                    re.match(r"^end\s*(if|do|where|select|type|interface)", text):
                if cur.kind != "skip":
                    self.units[cur.name] = cur
                cur = None
                continue
            if cur.kind == "skip":
                continue
            if self._is_decl(text):
                cur.decls.append((text, where))
            else:
                cur.body.append((lab, text, where))
        if cur is not None and cur.kind != "skip":
            raise FortranUnsupported(f"{path}: unterminated unit {cur.name}")

    @staticmethod
    def _is_decl(t: str) -> bool:
        if re.match(r"^(implicit|dimension|parameter|common|save|external|intrinsic|data|use|equivalence)\b", t):
            return not re.match(r"^(dimension|common|parameter)\s*=", t)
        if _TYPE_RE.match(t) and not re.match(r"^(integer|real|logical|character)\w*\s*=", t):
            # a type statement, not an assignment to a variable named like a type
            return not re.match(r"^(real|integer|logical)\s*\(", t) or "::" in t or re.match(
                r"^(real|integer)\s*\(\s*(kind\s*=\s*)?\d+\s*\)\s*[a-z]", t) is not None
        return False

    # ---- declarations
    def _declare(self, u: Unit):
        implicit = {c: ("i" if "i" <= c <= "n" else "r") for c in "abcdefghijklmnopqrstuvwxyz"}
        syms: dict[str, Var] = {}
        for a in u.args:
            syms[a] = Var(a, scope="dummy")
        if u.kind == "function":
            syms[u.name] = Var(u.name, type=_tchar(u.rtype.split("*")[0]) if u.rtype else "", scope="result")
        in_common = set()

        def get(name):
            if name not in syms:
                syms[name] = Var(name)
            return syms[name]

        def dims_of(s):
            out = []
            for d in _split_top(s):
                if d == ":":
                    out.append((None, None))
                elif d == "*":
                    out.append((Num("1"), None))
                elif ":" in d and _split_top(d, ":") and len(_split_top(d, ":")) == 2:
                    lo, hi = _split_top(d, ":")
                    out.append((parse_expr(lo), None if hi == "*" else parse_expr(hi)))
                else:
                    out.append((Num("1"), parse_expr(d)))
            return out

        def entities(s):
            for ent in _split_top(s):
                ent = ent.strip()
                init = None
                if "=" in ent and "(" not in ent.split("=")[0]:
                    ent, init = [x.strip() for x in ent.split("=", 1)]
                m = re.match(r"^(\w+)\s*(\*\s*\d+)?\s*(?:\((.*)\))?\s*(\*\s*\d+)?$", ent)
                if not m:
                    raise FortranUnsupported(f"entity {ent!r}")
                yield m.group(1), (dims_of(m.group(3)) if m.group(3) else None), init

        for text, where in u.decls:
            t = text
            try:
                if t.startswith("implicit"):
                    if re.match(r"implicit\s+none", t):
                        continue
                    m = re.match(r"implicit\s+(\w+(?:\s*\*\s*\d+)?(?:\s+precision)?)\s*\((.*)\)", t)
                    tc = _tchar(re.sub(r"\*.*", "", m.group(1)).strip())
                    for rng in m.group(2).split(","):
                        rng = rng.strip()
                        if "-" in rng:
                            a, b = [x.strip() for x in rng.split("-")]
                            for c in range(ord(a), ord(b) + 1):
                                implicit[chr(c)] = tc
                        else:
                            implicit[rng] = tc
                    continue
                if t.startswith("use"):
                    u.uses.append(re.match(r"use\s+(\w+)", t).group(1))
                    continue
                if t.startswith(("save", "external", "intrinsic", "equivalence", "data")):
                    if t.startswith("equivalence") or t.startswith("data"):
                        raise FortranUnsupported(f"{where}: {t}")
                    continue
                if t.startswith("parameter"):
                    inner = t[t.index("(") + 1: t.rindex(")")]
                    for asg in _split_top(inner):
                        n, e = [x.strip() for x in asg.split("=", 1)]
                        v = get(n)
                        v.scope = "param"
                        v.value = self._const(parse_expr(e), syms, implicit)
                        if not v.type:
                            v.type = "i" if isinstance(v.value, (int, np.integer)) else implicit[n[0]]
                    continue
                if t.startswith("dimension"):
                    for n, d, _ in entities(t[len("dimension"):]):
                        get(n).dims = d
                    continue
                if t.startswith("common"):
                    rest = t[len("common"):].strip()
                    if rest.startswith("/"):
                        j = rest.index("/", 1)
                        rest = rest[j + 1:]
                    for n, d, _ in entities(rest):
                        v = get(n)
                        v.scope = "global"
                        if d is not None:
                            v.dims = d
                        in_common.add(n)
                    continue
                m = _TYPE_RE.match(t)
                if m:
                    tc = _tchar(m.group(1))
                    rest = t[m.end():]
                    attrs = []
                    if "::" in rest:
                        a, rest = rest.split("::", 1)
                        attrs = [x.strip() for x in _split_top(a.strip().lstrip(","))]
                    else:
                        rest = rest.lstrip(",")
                    for n, d, init in entities(rest):
                        v = get(n)
                        v.type = tc
                        if d is not None:
                            v.dims = d
                        for at in attrs:
                            if at.startswith("dimension"):
                                v.dims = dims_of(at[at.index("(") + 1: at.rindex(")")])
                            if at == "allocatable" or at == "pointer":
                                v.alloc = True
                            if at == "parameter":
                                v.scope = "param"
                                v.value = self._const(parse_expr(init), syms, implicit)
                    continue
                raise FortranUnsupported(f"{where}: declaration {t}")
            except FortranUnsupported:
                raise
            except Exception as exc:  # pragma: no cover - diagnostic
                raise FortranUnsupported(f"{where}: {t}: {exc}") from exc
        for n, v in syms.items():
            if not v.type:
                v.type = implicit[n[0]] if n[0] in implicit else "r"
        # module variables
        for mod in u.uses:
            for n, v in self.modules.get(mod, {}).items():
                if n not in syms:
                    syms[n] = v
        u.syms, u.implicit = syms, implicit
        # register globals (common) once with their shape
        for n in in_common:
            v = syms[n]
            if n not in self.global_syms:
                self.global_syms[n] = v
                self.G._define(n, v, self._shape_now(v, syms))

    def _const(self, e, syms, implicit):
        """Evaluate a constant expression (parameters)."""
        code, _ = _Gen(self, None, syms, implicit, const=True).expr(e)
        return eval(code, {"np": np, **_HELPERS})

    def _shape_now(self, v: Var, syms):
        if v.dims is None:
            return None
        shp = []
        for lo, hi in v.dims:
            lo_v = self._const(lo, syms, {}) if lo is not None else 1
            hi_v = self._const(hi, syms, {})
            shp.append((int(lo_v), int(hi_v)))
        return shp

    def module(self, name: str, variables: dict[str, object]):
        """Declare a module: variables = {name: value}; values live in the globals.

        A list value is an array of derived-type objects (``a(i)%p`` reads ``a[i-1].p``)."""
        self.modules[name] = {}
        for n, val in variables.items():
            t = "i" if isinstance(val, (int, np.integer)) or (isinstance(val, np.ndarray) and val.dtype.kind == "i") \
                else "r"
            v = Var(n, type=t, scope="global", obj=isinstance(val, list))
            if isinstance(val, np.ndarray):
                v.dims = [(Num("1"), Num(str(s))) for s in val.shape]
            self.modules[name][n] = v
            setattr(self.G, n, val)
            self.global_syms.setdefault(n, v)

    # ---- translation
    def function(self, name: str):
        name = name.lower()
        if name in self._compiled:
            return self._compiled[name]
        if name not in self.units:
            if name in self.stubs:
                return self.stubs[name]
            raise FortranUnsupported(f"no unit or stub named {name}")
        u = self.units[name]
        if not u.syms:
            self._declare(u)
        src = _Gen(self, u, u.syms, u.implicit).unit()
        env = {"np": np, "G": self.G, "F": self.F, **_HELPERS}
        try:
            code = compile(src, f"<fortran {u.name} {u.src}>", "exec")
        except SyntaxError as exc:
            lines = src.splitlines()
            ctx = "\n".join(lines[max(0, exc.lineno - 5): exc.lineno + 2])
            raise FortranUnsupported(f"generated Python for {u.name} does not compile: {exc}\n{ctx}") from exc
        exec(code, env)
        fn = env["f_" + u.name]
        fn._src = src
        self._compiled[name] = fn
        return fn

    def signature(self, name: str):
        """(list of dummy names, set of array dummies) of a unit, or None for stubs."""
        u = self.units.get(name)
        if u is None:
            return None
        if not u.syms:
            self._declare(u)
        arrays = {a for a in u.args if u.syms[a].dims is not None}
        return u.args, arrays, u.kind

    def call(self, name, *args):
        return self.function(name)(*args)


class _Globals:
    def _define(self, name, v: Var, shape):
        if hasattr(self, name):
            return
        if shape is None:
            val = {"i": 0, "r": 0.0, "l": False, "c": ""}.get(v.type, 0.0)
        else:
            dt = {"i": np.int64, "r": np.float64, "l": np.bool_}.get(v.type, np.float64)
            val = np.zeros([hi - lo + 1 for lo, hi in shape], dtype=dt, order="F")
        setattr(self, name, val)


class _Funcs:
    def __init__(self, prog):
        self._p = prog

    def __getattr__(self, name):
        return self._p.function(name)


# --------------------------------------------------------------------------- runtime helpers

class _Poison:
    """Stands in for an array actual that cannot be associated (e.g. a scalar dummy of no use)."""

    def __init__(self, what):
        self.what = what

    def __getitem__(self, k):
        raise FortranUnsupported(f"access to an unassociated array argument ({self.what})")

    def __setitem__(self, k, v):
        raise FortranUnsupported(f"store to an unassociated array argument ({self.what})")


def _view(x, shape, wb, dtype):
    if isinstance(x, _Poison):
        return x
    if x is None:
        return _Poison(f"missing actual for an array dummy {shape}")
    if not isinstance(x, np.ndarray):
        return _Poison(f"scalar {x!r} passed as array {shape}")
    if any(s is None for s in shape):  # assumed shape
        return x
    shape = [int(s) for s in shape]
    if -1 in shape:
        known = int(np.prod([s for s in shape if s != -1])) or 1
        shape[shape.index(-1)] = x.size // known
    need = int(np.prod(shape)) if shape else 1
    if tuple(x.shape) == tuple(shape):
        return x
    if x.size < need:
        return _Poison(f"actual of size {x.size} for dummy {shape}")
    if x.flags.f_contiguous or x.ndim <= 1 and (x.strides[0] == x.itemsize if x.ndim else True):
        flat = x.reshape(-1, order="F")
        y = flat[:need].reshape(shape, order="F")
        if np.shares_memory(y, x):
            return y
    flat = x.reshape(-1, order="F").copy()
    y = flat[:need].reshape(shape, order="F").copy(order="F")

    def back(x=x, y=y, need=need):
        f = x.reshape(-1, order="F").copy()
        f[:need] = y.reshape(-1, order="F")
        x[...] = f.reshape(x.shape, order="F")
    wb.append(back)
    return y


def _flush(wb):
    for f in wb:
        f()


def _seq(a, idx):
    """Sequence association: the storage of a from element idx (0-based tuple) on, as a 1-D view."""
    if not isinstance(a, np.ndarray):
        raise FortranUnsupported("sequence association on a non-array")
    if not a.flags.f_contiguous:
        raise FortranUnsupported("sequence association on a non-contiguous array")
    off = int(np.ravel_multi_index(tuple(int(i) for i in idx), a.shape, order="F"))
    return a.reshape(-1, order="F")[off:]


def _alloc(shape, dt):
    dtype = {"i": np.int64, "r": np.float64, "l": np.bool_, "c": object}[dt]
    return np.zeros([max(int(s), 0) for s in shape], dtype=dtype, order="F")


def _idiv(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        q = np.trunc(np.asarray(a) / np.asarray(b))
        return q.astype(np.int64)
    q = abs(int(a)) // abs(int(b))
    return q if (a >= 0) == (b >= 0) else -q


def _toint(x):
    if isinstance(x, np.ndarray):
        return np.trunc(x).astype(np.int64)
    return int(x)


def _tofloat(x):
    if isinstance(x, np.ndarray):
        return x.astype(np.float64)
    return float(x)


def _r4(x):
    if isinstance(x, np.ndarray):
        return x.astype(np.float32).astype(np.float64)
    return float(np.float32(x))


def _nint(x):
    if isinstance(x, np.ndarray):
        return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)
    return int(np.sign(x) * np.floor(abs(x) + 0.5))


def _mod(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return np.fmod(a, b)
    if isinstance(a, int) and isinstance(b, int):
        r = abs(a) % abs(b)
        return r if a >= 0 else -r
    return float(np.fmod(a, b))


def _sign(a, b):
    return np.where(np.asarray(b) >= 0, np.abs(a), -np.abs(a)) if isinstance(a, np.ndarray) or isinstance(
        b, np.ndarray) else (abs(a) if b >= 0 else -abs(a))


def _max(*a):
    r = functools.reduce(np.maximum, a)
    return r.item() if isinstance(r, np.generic) else r


def _min(*a):
    r = functools.reduce(np.minimum, a)
    return r.item() if isinstance(r, np.generic) else r


def _sum(a, dim=None):
    """SUM as a compiled loop does it: sequential accumulation in array-element order."""
    a = np.asarray(a)
    if dim is None:
        if a.size == 0:
            return 0.0
        return np.cumsum(a.reshape(-1, order="F"))[-1].item()
    return np.take(np.cumsum(a, axis=int(dim) - 1), -1, axis=int(dim) - 1)


def _streq(a, b):
    return str(a).rstrip() == str(b).rstrip()


def _cond(x):
    if isinstance(x, np.ndarray):
        if x.size != 1:
            raise FortranUnsupported("array-valued condition")
        return bool(x.reshape(-1)[0])
    return bool(x)


def _land(a, b):
    return np.logical_and(a, b)


def _lor(a, b):
    return np.logical_or(a, b)


def _lnot(a):
    return np.logical_not(a)


def _frange(a, b, s=1):
    a, b, s = int(a), int(b), int(s)
    return range(a, b + 1, s) if s > 0 else range(a, b - 1, s)


def _pow(a, b):
    if isinstance(b, (int, np.integer)) and not isinstance(a, np.ndarray):
        if isinstance(a, (int, np.integer)):
            return int(a) ** int(b) if b >= 0 else _idiv(1, int(a) ** (-int(b)))
        return float(a) ** int(b)
    return np.power(a, b)


def _minloc(a):
    a = np.asarray(a)
    if a.ndim != 1:
        raise FortranUnsupported("minloc of a multi-dimensional array")
    return np.array([int(np.argmin(a)) + 1])


def _maxloc(a):
    a = np.asarray(a)
    if a.ndim != 1:
        raise FortranUnsupported("maxloc of a multi-dimensional array")
    return np.array([int(np.argmax(a)) + 1])


def _btest(i, pos):
    r = (np.right_shift(np.asarray(i, dtype=np.int64), int(pos)) & 1) != 0
    return bool(r) if r.ndim == 0 else r


def _ibits(i, pos, n):
    return np.bitwise_and(np.right_shift(i, int(pos)), (1 << int(n)) - 1)


def _ibset(i, pos):
    return np.bitwise_or(i, 1 << int(pos))


def _ibclr(i, pos):
    return np.bitwise_and(i, ~(1 << int(pos)))


def _unsupported(msg):
    raise FortranUnsupported(msg)


def _stop(msg=""):
    raise FortranStop(msg)


_HELPERS = {k: v for k, v in globals().items() if k.startswith("_") and callable(v) and not k.startswith("__")}
_HELPERS.update(_Poison=_Poison, FortranUnsupported=FortranUnsupported)

_INTRINSIC = {
    "sqrt": ("np.sqrt", "r"), "dsqrt": ("np.sqrt", "r"), "exp": ("np.exp", "r"), "dexp": ("np.exp", "r"),
    "log": ("np.log", "r"), "dlog": ("np.log", "r"), "log10": ("np.log10", "r"), "sin": ("np.sin", "r"),
    "cos": ("np.cos", "r"), "tan": ("np.tan", "r"), "asin": ("np.arcsin", "r"), "acos": ("np.arccos", "r"),
    "atan": ("np.arctan", "r"), "atan2": ("np.arctan2", "r"), "sinh": ("np.sinh", "r"),
    "cosh": ("np.cosh", "r"), "tanh": ("np.tanh", "r"), "dble": ("_tofloat", "r"),
    "real": ("_r4", "r"), "float": ("_r4", "r"), "sngl": ("_r4", "r"),
    "int": ("_toint", "i"), "ifix": ("_toint", "i"), "idint": ("_toint", "i"), "nint": ("_nint", "i"),
    "abs": ("np.abs", "="), "dabs": ("np.abs", "r"), "iabs": ("np.abs", "i"),
    "max": ("_max", "="), "min": ("_min", "="), "dmax1": ("_max", "r"), "dmin1": ("_min", "r"),
    "amax1": ("_max", "r"), "amin1": ("_min", "r"), "max0": ("_max", "i"), "min0": ("_min", "i"),
    "mod": ("_mod", "="), "sign": ("_sign", "="), "dsign": ("_sign", "r"), "isign": ("_sign", "i"),
    "sum": ("_sum", "="), "maxval": ("np.max", "="), "minval": ("np.min", "="), "size": ("np.size", "i"),
    "any": ("np.any", "l"), "all": ("np.all", "l"), "count": ("np.count_nonzero", "i"),
    "dot_product": ("np.dot", "="), "transpose": ("np.transpose", "="),
    "epsilon": ("(lambda x: float(np.finfo(np.float64).eps))", "r"),
    "huge": ("(lambda x: float(np.finfo(np.float64).max))", "r"),
    "tiny": ("(lambda x: float(np.finfo(np.float64).tiny))", "r"),
    "floor": ("(lambda x: np.floor(x).astype(np.int64) if isinstance(x, np.ndarray) else int(np.floor(x)))", "i"),
    "trim": ("(lambda s: str(s).rstrip())", "c"), "len": ("len", "i"),
    "btest": ("_btest", "l"), "ibits": ("_ibits", "i"), "minloc": ("_minloc", "i"), "maxloc": ("_maxloc", "i"), "ibset": ("_ibset", "i"), "ibclr": ("_ibclr", "i"),
    "iand": ("np.bitwise_and", "i"), "ior": ("np.bitwise_or", "i"), "ieor": ("np.bitwise_xor", "i"),
}


# --------------------------------------------------------------------------- code generation

class _Gen:
    def __init__(self, prog: Program, unit: Unit | None, syms: dict, implicit: dict, const=False):
        self.p = prog
        self.u = unit
        self.syms = syms
        self.implicit = implicit
        self.const = const
        self.lines: list[str] = []
        self.ind = 1
        self.tmp = 0
        self.cycle_labels, self.while_heads, self.while_gotos = set(), set(), set()

    # ---- names
    def var(self, name) -> Var:
        if name in self.syms:
            return self.syms[name]
        if name in self.p.global_syms:
            return self.p.global_syms[name]
        v = Var(name, type=self.implicit.get(name[0], "r"))
        self.syms[name] = v
        return v

    def pyname(self, v: Var) -> str:
        if v.scope == "global" or (v.name not in self.syms and v.name in self.p.global_syms):
            return f"G.{v.name}"
        if v.scope == "param":
            return repr(v.value)
        return f"v_{v.name}"

    def is_array(self, name) -> bool:
        v = self.syms.get(name) or self.p.global_syms.get(name)
        return v is not None and (v.dims is not None or v.obj or v.alloc)

    # ---- expressions: return (code, type)
    def expr(self, e):
        if isinstance(e, Num):
            t = e.text.split("_")[0]
            if re.fullmatch(r"\d+", t):
                return t, "i"
            if "d" in t:
                return repr(float(t.replace("d", "e"))), "r"
            return repr(float(np.float32(float(t)))), "r"
        if isinstance(e, Str):
            q = e.text[0]
            return repr(e.text[1:-1].replace(q + q, q)), "c"
        if isinstance(e, Logic):
            return ("True" if e.value else "False"), "l"
        if isinstance(e, Name):
            if self.const:
                v = self.syms.get(e.name) or self.p.global_syms.get(e.name)
                if v is None or v.scope != "param":
                    raise FortranUnsupported(f"non-constant {e.name} in a constant expression")
                return repr(v.value), v.type
            v = self.var(e.name)
            return self.pyname(v), v.type
        if isinstance(e, Un):
            c, t = self.expr(e.e)
            if e.op == ".not.":
                return f"_lnot({c})", "l"
            return f"({e.op}{c})", t
        if isinstance(e, Bin):
            a, ta = self.expr(e.a)
            b, tb = self.expr(e.b)
            if e.op == ".and.":
                return f"_land({a}, {b})", "l"
            if e.op == ".or.":
                return f"_lor({a}, {b})", "l"
            if e.op in (".eqv.",):
                return f"({a} == {b})", "l"
            if e.op in (".neqv.",):
                return f"({a} != {b})", "l"
            if e.op in ("==", "!=", "<", "<=", ">", ">="):
                if ta == "c" or tb == "c":
                    r = f"_streq({a}, {b})"
                    return (r if e.op == "==" else f"(not {r})"), "l"
                return f"({a} {e.op} {b})", "l"
            if e.op == "//":
                return f"(str({a}) + str({b}))", "c"
            t = "i" if ta == "i" and tb == "i" else "r"
            if e.op == "/" and t == "i":
                return f"_idiv({a}, {b})", "i"
            if e.op == "**":
                return f"_pow({a}, {b})", ("i" if ta == "i" and tb == "i" else "r")
            return f"({a} {e.op} {b})", t
        if isinstance(e, ArrCons):
            items = [self.expr(x) for x in e.items]
            t = "r" if any(tt == "r" for _, tt in items) else items[0][1]
            return f"np.array([{', '.join(c for c, _ in items)}])", t
        if isinstance(e, Comp):
            b, _ = self.expr(e.base)
            return f"{b}.{e.field}", "r"
        if isinstance(e, Ref):
            return self.ref(e)
        raise FortranUnsupported(f"expression {e}")

    def index(self, v: Var, args) -> str:
        if v.dims is None:
            # deferred-shape/allocatable or object array: 1-based
            dims = [(Num("1"), None)] * len(args)
        else:
            dims = v.dims
        if len(args) != len(dims):
            raise FortranUnsupported(f"{v.name}: {len(args)} subscripts for rank {len(dims)}")
        parts = []
        for a, (lo, _hi) in zip(args, dims):
            lo_c = "1" if lo is None else self.expr(lo)[0]
            if isinstance(a, Slice):
                s_lo = "" if a.lo is None else f"({self.expr(a.lo)[0]}) - ({lo_c})"
                s_hi = "" if a.hi is None else f"({self.expr(a.hi)[0]}) - ({lo_c}) + 1"
                if a.step is not None:
                    st = self.expr(a.step)[0]
                    parts.append(f"_slice({s_lo or 'None'}, {s_hi or 'None'}, {st})")
                else:
                    parts.append(f"{s_lo}:{s_hi}")
            else:
                c, _ = self.expr(a)
                parts.append(f"({c}) - ({lo_c})" if lo_c != "1" else self._minus1(c))
        return ", ".join(parts)

    @staticmethod
    def _minus1(c):
        if re.fullmatch(r"\d+", c):
            return str(int(c) - 1)
        return f"({c}) - 1"

    def ref(self, e: Ref):
        name = e.name
        if self.const:
            if name in _INTRINSIC:
                fn, rt = _INTRINSIC[name]
                args = [self.expr(a) for a in e.args]
                return f"{fn}({', '.join(c for c, _ in args)})", (args[0][1] if rt == "=" else rt)
            raise FortranUnsupported(f"{name}() in a constant expression")
        v = self.syms.get(name) or self.p.global_syms.get(name)
        if v is not None and (v.dims is not None or v.alloc or v.obj):
            if v.type == "c" and v.dims is None:
                raise FortranUnsupported("substring")
            return f"{self.pyname(v)}[{self.index(v, e.args)}]", v.type
        if v is not None and v.type == "c" and len(e.args) == 1 and isinstance(e.args[0], Slice):
            a = e.args[0]
            lo = "0" if a.lo is None else f"({self.expr(a.lo)[0]})-1"
            hi = "" if a.hi is None else self.expr(a.hi)[0]
            return f"{self.pyname(v)}[{lo}:{hi}]", "c"
        if name in _INTRINSIC and (v is None or v.scope not in ("dummy",)):
            fn, rt = _INTRINSIC[name]
            args = []
            for a in e.args:
                if isinstance(a, tuple):
                    args.append((self.expr(a[2])[0], "i"))
                else:
                    args.append(self.expr(a))
            t = rt
            if rt == "=":
                t = "r" if any(tt == "r" for _, tt in args) else args[0][1]
            return f"{fn}({', '.join(c for c, _ in args)})", t
        # user function
        sig = self.p.signature(name)
        if sig is None and name not in self.p.stubs:
            return f"_unsupported({('function ' + name)!r})", "r"
        code, _ = self.call_code(name, e.args, as_function=True)
        u = self.p.units.get(name)
        rt = "r"
        if u is not None:
            rt = _tchar(u.rtype.split("*")[0]) if u.rtype else (u.implicit or {}).get(name[0], "r") if u.implicit \
                else ("i" if "i" <= name[0] <= "n" else "r")
        return code, rt

    # ---- calls
    def call_code(self, name, args, as_function=False):
        sig = self.p.signature(name)
        if sig is None:
            # stub: plain values
            vals = [self.actual_value(a) for a in args]
            return f"F.{name}({', '.join(vals)})", []
        dummies, arrays, kind = sig
        args = list(args)[:len(dummies)]  # surplus actuals (no interface) are not associated
        vals, back = [], []
        scal_pos = [d for d in dummies if d not in arrays]
        for d, a in zip(dummies, args):
            if d in arrays:
                vals.append(self.actual_array(a))
            else:
                vals.append(self.actual_value(a))
                tgt = self.assignable(a)
                if tgt is not None:
                    back.append((scal_pos.index(d), tgt))
        return f"F.{name}({', '.join(vals)})", back

    def actual_array(self, a) -> str:
        if isinstance(a, Name):
            if self.is_array(a.name):
                return self.pyname(self.var(a.name))
            return self.expr(a)[0]
        if isinstance(a, Comp):
            return self.expr(a)[0]
        if isinstance(a, Ref) and self.is_array(a.name):
            v = self.var(a.name)
            if all(not isinstance(x, Slice) for x in a.args):
                # element actual for an array dummy: sequence association
                idx = self.index(v, a.args)
                return f"_seq({self.pyname(v)}, ({idx},))"
            return self.expr(a)[0]
        return f"np.asarray({self.expr(a)[0]})"

    def actual_value(self, a) -> str:
        if isinstance(a, Name) and self.is_array(a.name):
            return self.pyname(self.var(a.name))
        if isinstance(a, tuple):
            return self.expr(a[2])[0]
        c, _ = self.expr(a)
        return c

    def assignable(self, a):
        if isinstance(a, Name):
            v = self.var(a.name)
            if v.scope == "param" or self.is_array(a.name):
                return None
            return self.pyname(v)
        if isinstance(a, Ref) and self.is_array(a.name) and all(not isinstance(x, Slice) for x in a.args):
            v = self.var(a.name)
            return f"{self.pyname(v)}[{self.index(v, a.args)}]"
        return None

    # ---- statements
    def emit(self, s):
        self.lines.append("    " * self.ind + s)

    def unit(self) -> str:
        u = self.u
        hdr = f"def f_{u.name}({', '.join('v_' + a + '=None' for a in u.args)}):"
        self.lines.append(hdr)
        self.emit("_wb = []")
        # scalar dummies first (array bounds may use them), then arrays
        for a in u.args:
            v = u.syms[a]
            if v.dims is not None:
                continue
        for a in u.args:
            v = u.syms[a]
            if v.dims is not None:
                shape = []
                for lo, hi in v.dims:
                    if lo is None and hi is None:
                        shape.append("None")
                    elif hi is None:
                        shape.append("-1")
                    else:
                        lo_c = self.expr(lo)[0]
                        hi_c = self.expr(hi)[0]
                        shape.append(f"({hi_c}) - ({lo_c}) + 1")
                self.emit(f"v_{a} = _view(v_{a}, [{', '.join(shape)}], _wb, {v.type!r})")
        for n, v in u.syms.items():
            if v.scope in ("local",) and n not in self.p.global_syms:
                if v.dims is not None and not v.alloc:
                    shape = [f"({self.expr(hi)[0]}) - ({self.expr(lo)[0]}) + 1" for lo, hi in v.dims]
                    self.emit(f"v_{n} = _alloc([{', '.join(shape)}], {v.type!r})")
                elif v.alloc:
                    self.emit(f"v_{n} = None")
                else:
                    self.emit(f"v_{n} = {dict(i='0', r='0.0', l='False', c=chr(39) * 2).get(v.type, '0.0')}")
            if v.scope == "result":
                self.emit(f"v_{n} = {dict(i='0', r='0.0', l='False').get(v.type, '0.0')}")
        self.ret = self._ret_code()
        known = set(u.syms)
        init_at = len(self.lines)
        # labels of a loop's last statement ("L continue" right before the loop's end):
        # a forward goto there is a cycle of that loop
        self.cycle_labels = set()
        body = u.body
        for i, (lab, text, _w) in enumerate(body):
            if lab is None or text != "continue":
                continue
            nxt = body[i + 1][1] if i + 1 < len(body) else ""
            if re.match(r"^end\s*do$", nxt) or any(re.match(rf"^do\s+{lab}\b", t) for _l, t, _x in body[:i]):
                self.cycle_labels.add(lab)
        # "L if (c) then ... goto L endif" is a while loop
        self.while_heads, self.while_gotos = set(), set()
        for i, (lab, text, _w) in enumerate(body):
            if lab is None or not re.match(r"^if\s*\(.*\)\s*then$", text):
                continue
            depth, j = 0, i
            for j in range(i, len(body)):
                t = body[j][1]
                if re.match(r"^if\s*\(.*\)\s*then$", t) and self._balanced_if(t):
                    depth += 1
                elif re.match(r"^end\s*if$", t):
                    depth -= 1
                    if depth == 0:
                        break
            prev = body[j - 1][1] if j - 1 > i else ""
            if re.match(rf"^go\s*to\s+{lab}$", prev):
                self.while_heads.add(i)
                self.while_gotos.add(j - 1)
        stack = []  # ('if'|'do'|'dolab', label)
        for idx, (lab, text, where) in enumerate(u.body):
            self.cur = idx
            try:
                self.stmt(text, stack, where)
            except FortranUnsupported as exc:
                self.emit(f"_unsupported({(where + ': ' + str(exc))!r})")
            while lab is not None and stack and stack[-1][0] == "dolab" and stack[-1][1] == lab:
                stack.pop()
                self.ind -= 1
        if stack:
            raise FortranUnsupported(f"{u.name}: unclosed blocks {stack}")
        self.emit(self.ret)
        # variables first seen in executable statements (implicitly typed locals)
        extra = []
        for n, v in u.syms.items():
            if n not in known and v.scope == "local" and n not in self.p.global_syms and v.dims is None:
                extra.append("    " + f"v_{n} = {dict(i='0', r='0.0', l='False', c=chr(39) * 2).get(v.type, '0.0')}")
        self.lines[init_at:init_at] = extra
        return "\n".join(self.lines) + "\n"

    def _ret_code(self):
        u = self.u
        if u.kind == "function":
            return f"_flush(_wb); return v_{u.name}"
        scal = [a for a in u.args if u.syms[a].dims is None]
        return f"_flush(_wb); return ({''.join('v_' + a + ', ' for a in scal)})"

    def assign(self, lhs_s, rhs_s):
        lhs = parse_expr(lhs_s)
        rhs_c, rt = self.expr(parse_expr(rhs_s))
        if isinstance(lhs, Name):
            v = self.var(lhs.name)
            if self.is_array(lhs.name) and not (v.alloc and v.dims is None and False):
                self.emit(f"{self.pyname(v)}[...] = {rhs_c}")
                return
            if v.type == "i" and rt != "i":
                rhs_c = f"_toint({rhs_c})"
            elif v.type == "r" and rt == "i":
                rhs_c = f"_tofloat({rhs_c})"
            self.emit(f"{self.pyname(v)} = {rhs_c}")
            return
        if isinstance(lhs, Ref):
            v = self.var(lhs.name)
            if not self.is_array(lhs.name):
                raise FortranUnsupported(f"statement function or unknown array {lhs.name}")
            self.emit(f"{self.pyname(v)}[{self.index(v, lhs.args)}] = {rhs_c}")
            return
        if isinstance(lhs, Comp):
            b, _ = self.expr(lhs.base)
            self.emit(f"{b}.{lhs.field} = {rhs_c}")
            return
        raise FortranUnsupported(f"assignment to {lhs_s}")

    def stmt(self, t: str, stack, where):
        # block constructs
        m = re.match(r"^(?:(\w+)\s*:\s*)?do\s+(\d+)?\s*,?\s*(\w+)\s*=\s*(.*)$", t)
        if m and not re.match(r"^do\s*\w*\s*=\s*.*\.", t[:0]):
            bounds = _split_top(m.group(4))
            cs = [self.expr(parse_expr(b))[0] for b in bounds]
            var = self.pyname(self.var(m.group(3)))
            self.emit(f"for {var} in _frange({', '.join(cs)}):")
            self.ind += 1
            if m.group(2):
                stack.append(("dolab", int(m.group(2))))
            else:
                stack.append(("do", None))
            return
        if re.match(r"^do\s+while\b", t):
            raise FortranUnsupported("do while")
        if re.match(r"^end\s*do$", t):
            if not stack or stack[-1][0] != "do":
                raise FortranUnsupported(f"enddo without do at {where}")
            stack.pop()
            self.ind -= 1
            return
        m = re.match(r"^if\s*\((.*)\)\s*then$", t)
        if m and self._balanced_if(t):
            c = self.cond_code(m.group(1), where)
            self.emit(f"{'while' if getattr(self, 'cur', -1) in self.while_heads else 'if'} _cond({c}):")
            self.ind += 1
            self.emit("pass")
            stack.append(("if", None))
            return
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", t)
        if m:
            c = self.cond_code(m.group(1), where)
            self.ind -= 1
            self.emit(f"elif _cond({c}):")
            self.ind += 1
            self.emit("pass")
            return
        if re.match(r"^else$", t):
            self.ind -= 1
            self.emit("else:")
            self.ind += 1
            self.emit("pass")
            return
        if re.match(r"^end\s*if$", t):
            if not stack or stack[-1][0] != "if":
                raise FortranUnsupported(f"endif without if at {where}")
            stack.pop()
            self.ind -= 1
            return
        if re.match(r"^where\s*\(", t):
            inner, rest = self._paren_split(t[5:].strip())
            mc = self.expr(parse_expr(inner))[0]
            if rest:
                self.where_assign(mc, rest)
                return
            self.tmp += 1
            w = f"_w{self.tmp}"
            self.emit(f"{w}_all = np.asarray({mc}).copy(); {w} = {w}_all")
            stack.append(("where", w))
            return
        m = re.match(r"^else\s*where\s*(\(.*\))?$", t)
        if m:
            if not stack or stack[-1][0] != "where":
                raise FortranUnsupported("elsewhere outside where")
            w = stack[-1][1]
            if m.group(1):
                mc = self.expr(parse_expr(m.group(1)))[0]
                self.emit(f"{w} = _land(_lnot({w}_all), {mc}); {w}_all = _lor({w}_all, {w})")
            else:
                self.emit(f"{w} = _lnot({w}_all)")
            return
        if re.match(r"^end\s*where$", t):
            if not stack or stack[-1][0] != "where":
                raise FortranUnsupported("endwhere outside where")
            stack.pop()
            return
        if stack and stack[-1][0] == "where":
            self.where_assign(stack[-1][1], t)
            return
        # logical if
        if re.match(r"^if\s*\(", t):
            cond, rest = self._paren_split(t[2:].strip())
            c = self.cond_code(cond, where)
            self.emit(f"if _cond({c}):")
            self.ind += 1
            try:
                self.stmt(rest, stack, where)
            except FortranUnsupported as exc:
                self.emit(f"_unsupported({(where + ': ' + str(exc))!r})")
            finally:
                self.ind -= 1
            return
        if t == "continue":
            self.emit("pass")
            return
        if t == "cycle":
            self.emit("continue")
            return
        if t == "exit":
            self.emit("break")
            return
        if t == "return":
            self.emit(self.ret)
            return
        if re.match(r"^stop\b", t):
            self.emit(f"_stop({t!r})")
            return
        if re.match(r"^(write|print|format|flush|open|close|read)\b", t):
            self.emit("pass")
            return
        m = re.match(r"^go\s*to\s+(\d+)$", t)
        if m and getattr(self, "cur", -1) in self.while_gotos:
            self.emit("continue")
            return
        if m and int(m.group(1)) in self.cycle_labels and any(k in ("do", "dolab") for k, _ in stack):
            self.emit("continue")
            return
        if re.match(r"^(go\s*to)\b", t):
            raise FortranUnsupported("goto")
        if re.match(r"^deallocate\s*\(", t) or re.match(r"^nullify\s*\(", t):
            self.emit("pass")
            return
        m = re.match(r"^allocate\s*\((.*)\)$", t)
        if m:
            for ent in _split_top(m.group(1)):
                if ent.startswith("stat"):
                    continue
                mm = re.match(r"^(\w+)\s*\((.*)\)$", ent)
                v = self.var(mm.group(1))
                dims = []
                shape = []
                for d in _split_top(mm.group(2)):
                    if ":" in d:
                        lo, hi = _split_top(d, ":")
                        dims.append((parse_expr(lo), parse_expr(hi)))
                        shape.append(f"({self.expr(parse_expr(hi))[0]}) - ({self.expr(parse_expr(lo))[0]}) + 1")
                    else:
                        dims.append((Num("1"), parse_expr(d)))
                        shape.append(self.expr(parse_expr(d))[0])
                v.dims = dims
                self.emit(f"{self.pyname(v)} = _alloc([{', '.join(shape)}], {v.type!r})")
            return
        m = re.match(r"^call\s+(\w+)\s*(?:\((.*)\))?\s*$", t)
        if m:
            name = m.group(1)
            args = []
            if m.group(2) and m.group(2).strip():
                p = Parser(tokenize(m.group(2)))
                args.append(p.arg())
                while p.peek()[1] == ",":
                    p.take()
                    args.append(p.arg())
                if not p.done():
                    raise FortranUnsupported(f"call args {m.group(2)}")
            if self.p.signature(name) is None and name not in self.p.stubs:
                self.emit(f"_unsupported({('call ' + name + ' (no unit)')!r})")
                return
            code, back = self.call_code(name, args)
            if back:
                self.emit(f"_r = {code}")
                for k, tgt in back:
                    self.emit(f"{tgt} = _r[{k}]")
            else:
                self.emit(code)
            return
        parts = self._assign_split(t)
        if parts:
            self.assign(*parts)
            return
        raise FortranUnsupported(f"statement {t!r}")

    def where_assign(self, mask_code, t):
        parts = self._assign_split(t)
        if not parts:
            raise FortranUnsupported(f"statement {t!r} in a where block")
        lhs = parse_expr(parts[0])
        if isinstance(lhs, Name):
            lhs_c = self.pyname(self.var(lhs.name))
        else:
            lhs_c = self.expr(lhs)[0]
        rhs_c = self.expr(parse_expr(parts[1]))[0]
        self.emit(f"_m = np.asarray({mask_code}); _l = {lhs_c}")
        self.emit("with np.errstate(all='ignore'):")
        self.emit(f"    _r = np.broadcast_to({rhs_c}, _l.shape)")
        self.emit("_l[_m] = _r[_m]")

    def cond_code(self, s, where):
        try:
            return self.expr(parse_expr(s))[0]
        except FortranUnsupported as exc:
            return f"_unsupported({(where + ': ' + str(exc))!r})"

    @staticmethod
    def _balanced_if(t):
        inner, rest = _Gen._paren_split(t[2:].strip())
        return rest.strip() == "then"

    @staticmethod
    def _paren_split(s):
        """'(a) rest' -> ('a', 'rest')"""
        if not s.startswith("("):
            raise FortranUnsupported(f"expected ( in {s!r}")
        depth, q = 0, None
        for i, ch in enumerate(s):
            if q:
                if ch == q:
                    q = None
                continue
            if ch in "'\"":
                q = ch
            elif ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    return s[1:i], s[i + 1:].strip()
        raise FortranUnsupported(f"unbalanced parentheses in {s!r}")

    @staticmethod
    def _assign_split(t):
        depth, q = 0, None
        for i, ch in enumerate(t):
            if q:
                if ch == q:
                    q = None
                continue
            if ch in "'\"":
                q = ch
            elif ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            elif ch == "=" and depth == 0:
                nxt = t[i + 1: i + 2]
                prv = t[i - 1: i] if i else ""
                if nxt == "=" or prv in "<>/=":
                    continue
                return t[:i].strip(), t[i + 1:].strip()
        return None


def _slice(lo, hi, st):
    return slice(lo, hi, st)


_HELPERS["_slice"] = _slice
