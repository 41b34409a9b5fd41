"""TEST INFRASTRUCTURE ONLY: a translator for the Fortran 2008 subset the
reference is written in, to C++17, so that the reference's own source can be
compiled and run in an image that has no Fortran compiler.

The reference (Sinchanrc/Beach-Slope) is plain free-form Fortran: modules
with derived types (allocatable and pointer components, default
initialisation), allocatable arrays with explicit lower bounds, pointer
association, `associate`, array sections in assignments and reductions,
OpenMP directives (dropped: the translation runs serially, which is what the
orphaned `!$omp do` loops compute when one thread executes them).  This
module parses that subset and emits C++ that keeps Fortran's semantics where
they decide the numbers:

* kinds: `real(dp)` is double, default `real` and unsuffixed real literals
  (`1e-5`, `28.0*3.14`) are single precision, so expressions mix float and
  double exactly as gfortran's default REAL(4) does;
* integer division truncates, `**` with an integer exponent multiplies;
* DO loops fix their trip count on entry (the reference shrinks particle
  counts inside loops over them);
* arrays are column-major with per-dimension lower bounds; assignment of
  derived types copies their allocatable components (deep copy); pointer
  components alias.

Reading the reference's files is done only by oracle/ref_build.py, in the
build container; the generated C++ goes to oracle/_ref/ (never committed).
"""
import re

# ----------------------------------------------------------------- source

_STR = re.compile(r"('([^']|'')*'|\"([^\"]|\"\")*\")")


def _strip_comment(line):
    """Remove a trailing ! comment (not inside a string)."""
    out, q = [], None
    for ch in line:
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


def _lower_outside_strings(s):
    parts, last = [], 0
    for m in _STR.finditer(s):
        parts.append(s[last:m.start()].lower())
        parts.append(m.group(0))
        last = m.end()
    parts.append(s[last:].lower())
    return "".join(parts)


def logical_lines(text):
    """Free-form source -> list of (line number, statement text): comments
    and OpenMP directives removed, continuations joined, lower case outside
    strings, ';' separated statements split."""
    out = []
    buf, start = "", None
    for no, raw in enumerate(text.splitlines(), 1):
        s = raw.rstrip()
        if re.match(r"^\s*!\$", s):       # OpenMP / conditional compilation
            continue
        s = _strip_comment(s).rstrip()
        if not s.strip():
            continue
        t = s.strip()
        if buf and t.startswith("&"):
            t = t[1:]
        cont = t.endswith("&")
        if cont:
            t = t[:-1]
        if not buf:
            start = no
        buf += " " + t
        if not cont:
            st = _lower_outside_strings(buf.strip())
            for piece in _split_semicolons(st):
                if piece.strip():
                    out.append((start, piece.strip()))
            buf = ""
    return out


def _split_semicolons(s):
    parts, cur, q, depth = [], [], None, 0
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
        if ch == ";" and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


# ----------------------------------------------------------------- tokens

_TOK = re.compile(r"""
    (?P<ws>\s+)
  | (?P<real>(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?(_[a-z_][a-z0-9_]*)?(?![a-z_]))
  | (?P<dotop>\.(and|or|not|eqv|neqv|eq|ne|lt|le|gt|ge|true|false)\.(_[a-z_]\w*)?)
  | (?P<str>'([^']|'')*'|"([^"]|"")*")
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\(/|/\)|\*\*|//|==|/=|<=|>=|=>|::|[-+*/()<>=,%:])
""", re.X)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize at {s[pos:pos + 20]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        v = m.group(0)
        if kind == "real":
            body = v.split("_")[0]
            kind = "real" if re.search(r"[.ed]", body) else "int"
        toks.append((kind, v))
    return toks


# ----------------------------------------------------------------- expressions

class E:
    """Expression node: op in {num, log, str, name, ref, comp, bin, un, range, paren}."""
    __slots__ = ("op", "a", "b", "c", "t")

    def __init__(self, op, a=None, b=None, c=None):
        self.op, self.a, self.b, self.c = op, a, b, c
        self.t = None

    def __repr__(self):
        return f"E({self.op},{self.a!r},{self.b!r},{self.c!r})"


_BIN_PREC = [
    ({".eqv.", ".neqv."}, 1),
    ({".or."}, 2),
    ({".and."}, 3),
    ({"==", "/=", "<", "<=", ">", ">=", ".eq.", ".ne.", ".lt.", ".le.", ".gt.", ".ge."}, 5),
    ({"//"}, 6),
    ({"+", "-"}, 7),
    ({"*", "/"}, 8),
]
_PREC = {op: p for ops, p in _BIN_PREC for op in ops}
_NORM = {".eq.": "==", ".ne.": "/=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}


class ExprParser:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise SyntaxError(f"expected {val!r}, got {tok!r}")
        self.i += 1
        return tok

    def at(self, val):
        return self.peek()[1] == val

    def parse(self, min_prec=0):
        left = self.unary()
        while True:
            kind, v = self.peek()
            if kind is None:
                return left
            op = _NORM.get(v, v)
            p = _PREC.get(v)
            if p is None or p < min_prec:
                return left
            self.take()
            right = self.parse(p + 1)
            left = E("bin", op, left, right)

    def unary(self):
        kind, v = self.peek()
        if v == ".not.":
            self.take()
            return E("un", ".not.", self.parse(4))
        if v in ("-", "+"):
            self.take()
            # unary minus binds looser than * and / and **: -a*b = -(a*b)
            return E("un", v, self.parse(8))
        return self.power()

    def power(self):
        base = self.postfix()
        if self.at("**"):
            self.take()
            exp = self.unary_pow()
            return E("bin", "**", base, exp)
        return base

    def unary_pow(self):
        kind, v = self.peek()
        if v in ("-", "+"):
            self.take()
            return E("un", v, self.power())
        return self.power()

    def postfix(self):
        node = self.primary()
        while True:
            if self.at("(") and node.op in ("name", "ref", "comp"):
                self.take("(")
                args = self.arglist()
                self.take(")")
                node = E("ref", node, args)
            elif self.at("%"):
                self.take("%")
                _, nm = self.take()
                node = E("comp", node, nm)
            else:
                return node

    def arglist(self):
        args = []
        if self.at(")"):
            return args
        while True:
            args.append(self.arg())
            if self.at(","):
                self.take(",")
                continue
            return args

    def arg(self):
        # keyword argument, section (lo:hi), or expression
        kind, v = self.peek()
        if kind == "name" and self.peek(1)[1] == "=" and self.peek(2)[1] != "=":
            self.take()
            self.take("=")
            return E("kw", v, self.arg())
        lo = None
        if not self.at(":"):
            lo = self.parse()
        if self.at(":"):
            self.take(":")
            hi = None
            if not (self.at(",") or self.at(")") or self.at(":")):
                hi = self.parse()
            return E("range", lo, hi)
        return lo

    def primary(self):
        kind, v = self.take()
        if kind == "int":
            return E("num", v, "int")
        if kind == "real":
            return E("num", v, "real")
        if kind == "dotop":
            if v.startswith(".true."):
                return E("log", True)
            if v.startswith(".false."):
                return E("log", False)
            raise SyntaxError(f"unexpected {v}")
        if kind == "str":
            return E("str", v)
        if kind == "name":
            return E("name", v)
        if v == "(":
            e = self.parse()
            self.take(")")
            return E("paren", e)
        if v == "(/":
            items = [self.parse()]
            while self.at(","):
                self.take(",")
                items.append(self.parse())
            self.take("/)")
            return E("ctor", items)
        raise SyntaxError(f"unexpected token {v!r}")


def parse_expr(s):
    toks = tokenize(s) if isinstance(s, str) else s
    p = ExprParser(toks)
    e = p.parse()
    if p.i != len(p.t):
        raise SyntaxError(f"trailing tokens in {s!r}: {p.t[p.i:]}")
    return e


def split_top(s, sep=","):
    """Split on top-level separators (outside parentheses and strings)."""
    parts, cur, depth, q = [], [], 0, None
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
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


def match_paren(s, i):
    """Index of the ')' matching the '(' at s[i]."""
    depth, q = 0, None
    for j in range(i, len(s)):
        ch = s[j]
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
                return j
    raise SyntaxError(f"unbalanced parentheses in {s!r}")


# ----------------------------------------------------------------- declarations

class Var:
    """A declared entity: base type ('real', kind), ('int',), ('log',),
    ('char',), ('type', name); dims: list of (lo, hi) expression pairs
    (None for deferred ':'); attrs: set of attribute words."""

    def __init__(self, name, base, dims=None, attrs=None, init=None):
        self.name, self.base = name, base
        self.dims = dims or []
        self.attrs = set(attrs or ())
        self.init = init
        self.module = None      # owning module for module variables

    @property
    def rank(self):
        return len(self.dims)

    def is_alloc(self):
        return "allocatable" in self.attrs

    def is_ptr(self):
        return "pointer" in self.attrs

    def __repr__(self):
        return f"Var({self.name},{self.base},{self.rank},{sorted(self.attrs)})"


_TYPESPEC = re.compile(r"^(real|integer|logical|character|double\s+precision|type|class)\b")


def parse_typespec(s):
    """Leading type spec of a declaration -> (base, rest of the string)."""
    m = _TYPESPEC.match(s)
    if not m:
        return None, s
    kw = m.group(1)
    rest = s[m.end():].lstrip()
    sel = None
    if rest.startswith("("):
        j = match_paren(rest, 0)
        sel = rest[1:j].strip()
        rest = rest[j + 1:].lstrip()
    elif rest.startswith("*"):          # real*8
        m2 = re.match(r"\*\s*(\d+)", rest)
        sel = m2.group(1)
        rest = rest[m2.end():].lstrip()
    if kw == "real":
        k = (sel or "").replace("kind=", "").strip()
        base = ("real", "dp" if k in ("dp", "8", "real64") else ("sp" if not k or k in ("4", "real32", "sp") else k))
    elif kw.startswith("double"):
        base = ("real", "dp")
    elif kw == "integer":
        base = ("int",)
    elif kw == "logical":
        base = ("log",)
    elif kw == "character":
        base = ("char",)
    else:
        base = ("type", sel.strip())
    return base, rest


def parse_dims(s):
    out = []
    for d in split_top(s):
        if d == ":":
            out.append((None, None))
        elif ":" in d and not d.startswith("'"):
            lo, hi = d.split(":", 1)
            out.append((parse_expr(lo) if lo.strip() else None, parse_expr(hi) if hi.strip() else None))
        elif d == "*":
            out.append((None, None))
        else:
            out.append((E("num", "1", "int"), parse_expr(d)))
    return out


def parse_decl(s):
    """A type declaration statement -> list of Var (None if not one)."""
    base, rest = parse_typespec(s)
    if base is None:
        return None
    attrs, dims_attr = set(), None
    if "::" in rest:
        head, ents = rest.split("::", 1)
        for a in split_top(head.lstrip(",")):
            a = a.strip()
            if not a:
                continue
            if a.startswith("dimension"):
                j = a.index("(")
                dims_attr = parse_dims(a[j + 1:match_paren(a, j)])
            elif a.startswith("intent"):
                attrs.add("intent_" + re.sub(r"[()\s]", "", a[6:]))
            else:
                attrs.add(a.split("(")[0].strip())
    else:
        ents = rest
    out = []
    for ent in split_top(ents):
        ent = ent.strip()
        init = None
        m = re.match(r"^([a-z_]\w*)\s*(\((.*)\))?\s*(=>?\s*(.*))?$", ent)
        if not m:
            raise SyntaxError(f"bad entity {ent!r}")
        name = m.group(1)
        dims = dims_attr
        if m.group(2):
            k = ent.index("(")
            dims = parse_dims(ent[k + 1:match_paren(ent, k)])
            tail = ent[match_paren(ent, k) + 1:].strip()
            if tail.startswith("=>"):
                init = ("=>", parse_expr(tail[2:]))
            elif tail.startswith("="):
                init = ("=", parse_expr(tail[1:]))
        elif m.group(4):
            v = m.group(4)
            init = ("=>", parse_expr(v[2:])) if v.startswith("=>") else ("=", parse_expr(v[1:]))
        out.append(Var(name, base, list(dims) if dims else [], attrs, init))
    return out


# ----------------------------------------------------------------- statements

class S:
    """Statement: kind plus fields in a dict."""

    def __init__(self, kind, line, **kw):
        self.kind, self.line = kind, line
        self.__dict__.update(kw)

    def __repr__(self):
        return f"S({self.kind}@{self.line})"


class Proc:
    def __init__(self, kind, name, args, result=None, module=None):
        self.kind, self.name, self.args = kind, name, args
        self.result = result
        self.module = module
        self.vars = {}          # locals and dummies
        self.body = []
        self.rtype = None       # function result base from the prefix
        self.uses = []


class Module:
    def __init__(self, name):
        self.name = name
        self.uses = []          # (module, only-list or None)
        self.vars = {}
        self.types = {}         # name -> dict of Var components (ordered)
        self.procs = {}
        self.order = []         # variable declaration order


_END = re.compile(r"^end\s*(do|if|select|associate|subroutine|function|module|program|type|interface)?\b")


class Parser:
    def __init__(self, lines, fname):
        self.L, self.i, self.fname = lines, 0, fname

    def peek(self):
        return self.L[self.i] if self.i < len(self.L) else (None, None)

    def next(self):
        x = self.L[self.i]
        self.i += 1
        return x

    def units(self):
        mods = []
        while self.i < len(self.L):
            no, s = self.next()
            m = re.match(r"^module\s+(\w+)$", s)
            if m:
                mods.append(self.module(m.group(1)))
                continue
            m = re.match(r"^program\s+(\w+)$", s)
            if m:
                mods.append(self.program(m.group(1)))
                continue
            if s.startswith("include"):
                continue
            raise SyntaxError(f"{self.fname}:{no}: unexpected {s!r}")
        return mods

    def spec_part(self, owner, is_module):
        """use / implicit / declarations / type definitions, up to the first
        executable statement or 'contains'."""
        while self.i < len(self.L):
            no, s = self.peek()
            if s == "contains" or _END.match(s):
                return
            if s.startswith("use ") or s.startswith("use,"):
                self.next()
                s2 = re.sub(r"^use\s*(,\s*intrinsic\s*::)?\s*", "", s)
                m = re.match(r"^(\w+)\s*(,\s*(.*))?$", s2)
                owner.uses.append((m.group(1), m.group(3)))
                continue
            if s.startswith("implicit") or s in ("public", "private", "save") or s.startswith("include"):
                self.next()
                continue
            if re.match(r"^(public|private)\s*(::)?\s*\w", s):
                self.next()
                continue
            if re.match(r"^type\s*(,[^:]*)?(::)?\s*\w+\s*$", s) and not s.startswith("type("):
                self.next()
                name = re.sub(r"^type\s*(,[^:]*)?(::)?\s*", "", s).strip()
                comps = {}
                while True:
                    no2, s2 = self.next()
                    if re.match(r"^end\s*type", s2):
                        break
                    if s2 in ("private", "public", "sequence"):
                        continue
                    for v in parse_decl(s2):
                        comps[v.name] = v
                owner.types[name] = comps
                continue
            vs = parse_decl(s) if _TYPESPEC.match(s) and not re.match(r"^\w+\s*(\(.*\))?\s*=", s) else None
            if vs is not None and not re.match(r"^(real|integer|logical)\s*(\(.*\))?\s*function\b", s):
                self.next()
                for v in vs:
                    if is_module:
                        v.module = owner.name
                        owner.order.append(v.name)
                    owner.vars[v.name] = v
                continue
            return

    def module(self, name):
        mod = Module(name)
        self.spec_part(mod, True)
        no, s = self.peek()
        if s == "contains":
            self.next()
            while True:
                no, s = self.peek()
                if _END.match(s) and "module" in s:
                    self.next()
                    break
                p = self.procedure(mod)
                mod.procs[p.name] = p
        else:
            self.next()   # end module
        return mod

    def program(self, name):
        mod = Module("__program_" + name)
        p = Proc("subroutine", "main_program", [], module=mod.name)
        self.spec_part(p, False)
        p.body = self.block(("end",))
        self.next()
        mod.procs["main_program"] = p
        return mod

    def procedure(self, mod):
        no, s = self.next()
        m = re.match(r"^((?:recursive|pure|elemental|impure|\s)*)(real\s*(\([^)]*\))?|integer|logical)?\s*"
                     r"(subroutine|function)\s+(\w+)\s*(\(([^)]*)\))?\s*(result\s*\((\w+)\))?$", s)
        if not m:
            raise SyntaxError(f"{self.fname}:{no}: expected a procedure, got {s!r}")
        kind, name = m.group(4), m.group(5)
        args = [a.strip() for a in (m.group(7) or "").split(",") if a.strip()]
        p = Proc(kind, name, args, result=m.group(9) or (name if kind == "function" else None), module=mod.name)
        if m.group(2):
            p.rtype = parse_typespec(m.group(2))[0]
        self.spec_part(p, False)
        p.body = self.block(("end",))
        self.next()   # end subroutine/function
        return p

    def block(self, enders):
        """Statements until one that starts with an ender word (not consumed)."""
        out = []
        while True:
            no, s = self.peek()
            if s is None:
                raise SyntaxError(f"{self.fname}: unexpected end of file")
            if (_END.match(s) or re.match(r"^else(\s*if\s*\(|\s|$)", s) or re.match(r"^case\s*(\(|default)", s)
                    or s == "contains"):
                return out
            out.append(self.statement())

    def statement(self):
        no, s = self.next()
        # labelled statement (continue targets)
        m = re.match(r"^(\d+)\s+(.*)$", s)
        if m:
            s = m.group(2)
            if s == "continue":
                return S("noop", no)
        if s in ("continue",):
            return S("noop", no)
        m = re.match(r"^(\w+)\s*:\s*(do\b.*)$", s)      # named construct
        if m:
            s = m.group(2)
        if re.match(r"^if\s*\(", s):
            j = match_paren(s, s.index("("))
            cond = parse_expr(s[s.index("(") + 1:j])
            rest = s[j + 1:].strip()
            if rest == "then":
                branches = [(cond, self.block(()))]
                els = None
                while True:
                    no2, s2 = self.next()
                    if re.match(r"^else\s*if\s*\(", s2):
                        k = s2.index("(")
                        j2 = match_paren(s2, k)
                        c2 = parse_expr(s2[k + 1:j2])
                        branches.append((c2, self.block(())))
                    elif s2 == "else":
                        els = self.block(())
                    elif re.match(r"^end\s*if", s2):
                        break
                    else:
                        raise SyntaxError(f"{self.fname}:{no2}: in if: {s2!r}")
                return S("if", no, branches=branches, els=els)
            inner = self.L[self.i - 1]
            self.L.insert(self.i, (no, rest))
            st = self.statement()
            return S("if", no, branches=[(cond, [st])], els=None)
        m = re.match(r"^do\s+while\s*\((.*)\)$", s)
        if m:
            body = self.block(())
            self.next()
            return S("dowhile", no, cond=parse_expr(m.group(1)), body=body)
        m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s)
        if m:
            parts = split_top(m.group(2))
            body = self.block(())
            self.next()
            return S("do", no, var=m.group(1), lo=parse_expr(parts[0]), hi=parse_expr(parts[1]),
                     step=parse_expr(parts[2]) if len(parts) > 2 else None, body=body)
        if s == "do":
            body = self.block(())
            self.next()
            return S("doforever", no, body=body)
        m = re.match(r"^select\s+case\s*\((.*)\)$", s)
        if m:
            sel = parse_expr(m.group(1))
            cases = []
            while True:
                no2, s2 = self.next()
                if re.match(r"^end\s*select", s2):
                    break
                if s2 == "case default":
                    cases.append((None, self.block(())))
                    continue
                m2 = re.match(r"^case\s*\((.*)\)$", s2)
                if not m2:
                    raise SyntaxError(f"{self.fname}:{no2}: in select: {s2!r}")
                cases.append(([parse_expr(v) for v in split_top(m2.group(1))], self.block(())))
            return S("select", no, sel=sel, cases=cases)
        m = re.match(r"^associate\s*\((.*)\)$", s)
        if m:
            pairs = []
            for a in split_top(m.group(1)):
                nm, ex = a.split("=>", 1)
                pairs.append((nm.strip(), parse_expr(ex)))
            body = self.block(())
            self.next()
            return S("associate", no, pairs=pairs, body=body)
        m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", s)
        if m:
            args = [parse_expr(a) if not re.match(r"^\w+\s*=[^=]", a) else
                    E("kw", a.split("=", 1)[0].strip(), parse_expr(a.split("=", 1)[1]))
                    for a in split_top(m.group(3) or "")]
            return S("call", no, name=m.group(1), args=args)
        m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", s)
        if m:
            items = [parse_expr(a) for a in split_top(m.group(2)) if not re.match(r"^(stat|errmsg|source)\s*=", a)]
            return S(m.group(1), no, items=items)
        if s in ("exit", "cycle", "return", "stop") or s.startswith("stop ") or re.match(r"^(exit|cycle)\s+\w+$", s):
            return S(s.split()[0], no)
        if re.match(r"^(write|print|open|close|read|flush)\b", s):
            return S("noop", no)
        if re.match(r"^go\s*to\s+\d+$", s):
            return S("goto", no)
        # assignment / pointer assignment
        k = _assign_split(s)
        if k is not None:
            lhs, op, rhs = k
            return S("ptr" if op == "=>" else "assign", no, lhs=parse_expr(lhs), rhs=parse_expr(rhs))
        raise SyntaxError(f"{self.fname}:{no}: cannot parse {s!r}")


def _assign_split(s):
    """'lhs = rhs' or 'lhs => rhs' at top level -> (lhs, op, rhs)."""
    depth, q = 0, None
    for j, ch in enumerate(s):
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
        elif depth == 0 and ch == "=":
            nxt = s[j + 1] if j + 1 < len(s) else ""
            prv = s[j - 1] if j > 0 else ""
            if nxt == "=" or prv in "=/<>":
                continue
            if nxt == ">":
                return s[:j].strip(), "=>", s[j + 2:].strip()
            return s[:j].strip(), "=", s[j + 1:].strip()
    return None


def parse_source(text, fname):
    return Parser(logical_lines(text), fname).units()


# ----------------------------------------------------------------- C++ emitter

class Ty:
    """Type of an expression: base tuple, rank, and whether the C++ code is a
    pointer that value contexts must dereference."""

    def __init__(self, base, rank=0, ptr=False):
        self.base, self.rank, self.ptr = base, rank, ptr

    def num(self):
        return self.base[0] in ("int", "real")


def ctype(base):
    k = base[0]
    if k == "real":
        return "double" if base[1] == "dp" else "float"
    if k == "int":
        return "int"
    if k == "log":
        return "bool"
    if k == "char":
        return "std::string"
    return "T_" + base[1]


def promote(a, b):
    """Numeric type of a binary operation on two scalar bases."""
    rank = {"int": 0, "sp": 1, "dp": 2}

    def r(x):
        return rank["int"] if x[0] == "int" else rank[x[1] if x[1] in ("sp", "dp") else "sp"]
    ra, rb = r(a), r(b)
    m = max(ra, rb)
    return ("int",) if m == 0 else (("real", "sp") if m == 1 else ("real", "dp"))


def arr_type(v):
    return f"Arr<{ctype(v.base)},{v.rank}>"


INTRINSICS = {"sqrt", "abs", "min", "max", "exp", "log", "cos", "sin", "tan", "tanh", "atan", "acos", "asin",
              "real", "dble", "int", "nint", "floor", "ceiling", "mod", "sign", "size", "allocated", "associated",
              "maxval", "minval", "sum", "merge", "ieee_is_nan", "ieee_is_finite", "huge", "epsilon", "null",
              "trim", "present", "dot_product", "isnan", "log10"}
ELEMENTAL = {"sqrt", "abs", "exp", "log", "cos", "sin", "tan", "tanh", "atan", "acos", "asin", "real", "dble",
             "int", "nint", "floor", "ceiling", "mod", "sign", "min", "max", "merge", "ieee_is_nan",
             "ieee_is_finite", "log10"}


class Translator:
    def __init__(self, modules):
        self.mods = {m.name: m for m in modules}
        self.types = {}
        for m in modules:
            for tn, comps in m.types.items():
                self.types[tn] = comps
        self.out = []
        self.tmp = 0

    # ---------------------------------------------------------- naming
    def gname(self, mod, name):
        return f"{mod}__{name}"

    # ---------------------------------------------------------- scopes
    def visible_modules(self, mod_name, extra_uses=()):
        """Modules whose public entities are visible from module mod_name
        (itself first, then use-association, transitively)."""
        seen, order = set(), []

        def visit(name):
            if name in seen or name not in self.mods:
                return
            seen.add(name)
            order.append(name)
            for u, _ in self.mods[name].uses:
                visit(u)
        for u, _ in extra_uses:
            visit(u)
        visit(mod_name)
        # the module itself takes precedence over what it uses
        if mod_name in order:
            order.remove(mod_name)
            order.insert(0, mod_name)
        return order

    def lookup(self, name):
        """(kind, object, C++ name) for a name in the current scope."""
        if name in self.scope:
            v = self.scope[name]
            return ("var", v, self.local_name(name))
        for mn in self.vis:
            m = self.mods[mn]
            if name in m.vars:
                return ("var", m.vars[name], self.gname(mn, name))
            if name in m.procs:
                return ("proc", m.procs[name], self.gname(mn, name))
        return (None, None, None)

    def local_name(self, name):
        return self.alias.get(name, name + "_")

    # ---------------------------------------------------------- expressions
    def expr(self, e):
        """Scalar expression -> (C++ code, Ty).  Pointer-valued designators are
        dereferenced."""
        code, t = self.designator_or_value(e)
        if t.ptr and t.rank == 0:
            return f"(*{code})", Ty(t.base, 0, False)
        return code, t

    def designator_or_value(self, e):
        op = e.op
        if op == "num":
            v, kind = e.a, e.b
            if kind == "int":
                return v.split("_")[0], Ty(("int",))
            body = v.split("_")[0]
            suffix = v.split("_")[1] if "_" in v else None
            dbl = suffix in ("dp", "8", "real64") or "d" in body
            body = body.replace("d", "e")
            if "." not in body and "e" not in body:
                body += ".0"
            if body.startswith("."):
                body = "0" + body
            if body.endswith("."):
                body += "0"
            if ".e" in body:
                body = body.replace(".e", ".0e")
            return (body if dbl else body + "f"), Ty(("real", "dp" if dbl else "sp"))
        if op == "log":
            return ("true" if e.a else "false"), Ty(("log",))
        if op == "str":
            return "std::string(" + '"' + e.a[1:-1].replace('"', '\\"') + '"' + ")", Ty(("char",))
        if op == "paren":
            c, t = self.expr(e.a)
            return f"({c})", t
        if op == "un":
            c, t = self.expr(e.b)
            if e.a == ".not.":
                return f"(!{c})", Ty(("log",))
            return f"({e.a}{c})", t
        if op == "bin":
            return self.binop(e)
        if op in ("name", "ref", "comp"):
            return self.designator(e)
        if op == "ctor":
            items = [self.expr(x) for x in e.a]
            t = items[0][1]
            return ("std::vector<" + ctype(t.base) + ">{" + ", ".join(c for c, _ in items) + "}"), Ty(t.base, 1)
        raise NotImplementedError(f"expression {e!r}")

    def binop(self, e):
        o = e.a
        lc, lt = self.expr(e.b)
        rc, rt_ = self.expr(e.c)
        if o == "**":
            if rt_.base[0] == "int":
                return f"ipow({lc}, {rc})", lt
            t = promote(lt.base, rt_.base)
            return f"std::pow(({ctype(t)})({lc}), ({ctype(t)})({rc}))", Ty(t)
        if o in ("+", "-", "*", "/"):
            t = promote(lt.base, rt_.base)
            return f"({lc} {o} {rc})", Ty(t)
        if o in ("==", "/=", "<", "<=", ">", ">="):
            co = "!=" if o == "/=" else o
            return f"({lc} {co} {rc})", Ty(("log",))
        if o in (".and.", ".or."):
            return f"({lc} {'&&' if o == '.and.' else '||'} {rc})", Ty(("log",))
        if o == ".eqv.":
            return f"({lc} == {rc})", Ty(("log",))
        if o == ".neqv.":
            return f"({lc} != {rc})", Ty(("log",))
        if o == "//":
            return f"({lc} + {rc})", Ty(("char",))
        raise NotImplementedError(o)

    # ---------------------------------------------------------- designators
    def comp_var(self, base_t, cname):
        if base_t.base[0] != "type":
            raise TypeError(f"component {cname} of non-derived type {base_t.base}")
        comps = self.types[base_t.base[1]]
        if cname not in comps:
            raise KeyError(f"type {base_t.base[1]} has no component {cname}")
        return comps[cname]

    def is_section(self, args):
        return any(a is not None and a.op == "range" for a in args)

    def designator(self, e):
        """Designator or function call -> (code, Ty).  Whole arrays give
        rank > 0; sections raise (they are scalarised by the caller)."""
        if e.op == "name":
            kind, obj, cn = self.lookup(e.a)
            if kind == "var":
                return cn, Ty(obj.base, obj.rank, obj.is_ptr())
            if e.a in ("dp",):
                return "8", Ty(("int",))
            raise NameError(f"unknown name {e.a!r} in {self.where}")
        if e.op == "comp":
            bc, bt = self.designator(e.a)
            if bt.rank > 0:
                raise SectionError(e)
            cv = self.comp_var(bt, e.b)
            acc = "->" if bt.ptr else "."
            return f"{bc}{acc}{e.b}_", Ty(cv.base, cv.rank, cv.is_ptr())
        if e.op == "ref":
            base, args = e.a, e.b
            if base.op == "name":
                kind, obj, cn = self.lookup(base.a)
                if kind == "proc":
                    return self.call_expr(obj, cn, args)
                if kind is None:
                    return self.intrinsic(base.a, args)
            bc, bt = self.designator(base)
            if bt.rank == 0:
                raise TypeError(f"subscript on scalar {bc} in {self.where}")
            if self.is_section(args):
                raise SectionError(e)
            idx = [self.expr(a)[0] for a in args]
            if bt.ptr:
                bc = f"(*{bc})"
            return f"{bc}({', '.join(idx)})", Ty(bt.base, 0, False)
        return self.designator_or_value(e)

    # ---------------------------------------------------------- array elements
    def shape(self, e):
        """Extent code per dimension of an array-valued expression."""
        if e.op in ("paren",):
            return self.shape(e.a)
        if e.op == "un":
            return self.shape(e.b)
        if e.op == "bin":
            for x in (e.b, e.c):
                if self.rank_of(x) > 0:
                    return self.shape(x)
        if e.op == "ref" and e.a.op == "name" and self.lookup(e.a.a)[0] is None:
            for x in e.b:
                if x is not None and x.op != "kw" and self.rank_of(x) > 0:
                    return self.shape(x)
        if e.op == "comp":
            try:
                bc, bt = self.designator(e.a)
                if bt.rank == 0:
                    c, t = self.designator(e)
                    return [f"{c}.ex[{d}]" for d in range(t.rank)]
            except SectionError:
                pass
            return self.shape(e.a)
        if e.op == "name":
            c, t = self.designator(e)
            return [f"{c}.ex[{d}]" for d in range(t.rank)]
        if e.op == "ref":
            bc, bt = self.designator(e.a)
            out = []
            for d, a in enumerate(e.b):
                if a.op == "range":
                    lo = self.expr(a.a)[0] if a.a is not None else f"{bc}.lb[{d}]"
                    hi = self.expr(a.b)[0] if a.b is not None else f"({bc}.lb[{d}] + {bc}.ex[{d}] - 1)"
                    out.append(f"(({hi}) - ({lo}) + 1)")
            return out
        raise NotImplementedError(f"shape of {e!r}")

    def rank_of(self, e):
        if e is None:
            return 0
        if e.op in ("num", "log", "str"):
            return 0
        if e.op == "paren":
            return self.rank_of(e.a)
        if e.op == "un":
            return self.rank_of(e.b)
        if e.op == "bin":
            return max(self.rank_of(e.b), self.rank_of(e.c))
        if e.op == "range":
            return 1
        if e.op == "ctor":
            return 1
        if e.op == "name":
            k, obj, _ = self.lookup(e.a)
            return obj.rank if k == "var" else 0
        if e.op == "comp":
            r = self.rank_of(e.a)
            if r:
                return r
            try:
                return self.designator(e)[1].rank
            except SectionError:
                return 1
        if e.op == "ref":
            if e.a.op == "name":
                k, obj, _ = self.lookup(e.a.a)
                if k == "proc":
                    return 0
                if k is None:
                    nm = e.a.a
                    if nm in ELEMENTAL:
                        return max([self.rank_of(x) for x in e.b if x is not None and x.op != "kw"] + [0])
                    return 0
            sec = sum(1 for a in e.b if a is not None and a.op == "range")
            if sec:
                return sec
            base_rank = self.rank_of(e.a) if e.a.op == "comp" else 0
            return 0 if not base_rank else 0
        return 0

    def elem(self, e, kv):
        """Element (at normalised indices kv, one per array dimension of e) of
        an array-valued expression, as scalar C++ code -> (code, Ty)."""
        r = self.rank_of(e)
        if r == 0:
            return self.expr(e)
        if e.op == "paren":
            c, t = self.elem(e.a, kv)
            return f"({c})", t
        if e.op == "un":
            c, t = self.elem(e.b, kv)
            if e.a == ".not.":
                return f"(!{c})", Ty(("log",))
            return f"({e.a}{c})", t
        if e.op == "bin":
            save = (e.b, e.c)
            lc, lt = self.elem(e.b, kv)
            rc, rt_ = self.elem(e.c, kv)
            fake = E("bin", e.a, E("__code", lc, lt), E("__code", rc, rt_))
            return self.binop_codes(e.a, lc, lt, rc, rt_)
        if e.op == "name":
            c, t = self.designator(e)
            idx = ", ".join(f"{c}.lb[{d}] + {kv[d]}" for d in range(t.rank))
            return f"{c}({idx})", Ty(t.base)
        if e.op == "comp":
            try:
                bc, bt = self.designator(e.a)
                if bt.rank == 0:   # scalar base, array component
                    c, t = self.designator(e)
                    idx = ", ".join(f"{c}.lb[{d}] + {kv[d]}" for d in range(t.rank))
                    return f"{c}({idx})", Ty(t.base)
            except SectionError:
                pass
            bc, bt = self.elem(e.a, kv)
            cv = self.comp_var(bt, e.b)
            return f"{bc}.{e.b}_", Ty(cv.base, 0, cv.is_ptr())
        if e.op == "ref":
            if e.a.op == "name" and self.lookup(e.a.a)[0] is None:
                args = [self.elem(x, kv) if x is not None and x.op != "kw" else (None, None) for x in e.b]
                return self.intrinsic_codes(e.a.a, args)
            bc, bt = self.designator(e.a)
            idx, k = [], 0
            for d, a in enumerate(e.b):
                if a.op == "range":
                    lo = self.expr(a.a)[0] if a.a is not None else f"{bc}.lb[{d}]"
                    idx.append(f"({lo}) + {kv[k]}")
                    k += 1
                else:
                    idx.append(self.expr(a)[0])
            return f"{bc}({', '.join(idx)})", Ty(bt.base)
        raise NotImplementedError(f"element of {e!r}")

    def binop_codes(self, o, lc, lt, rc, rt_):
        class _C:
            pass
        if o == "**":
            if rt_.base[0] == "int":
                return f"ipow({lc}, {rc})", lt
            t = promote(lt.base, rt_.base)
            return f"std::pow(({ctype(t)})({lc}), ({ctype(t)})({rc}))", Ty(t)
        if o in ("+", "-", "*", "/"):
            return f"({lc} {o} {rc})", Ty(promote(lt.base, rt_.base))
        if o in ("==", "/=", "<", "<=", ">", ">="):
            return f"({lc} {'!=' if o == '/=' else o} {rc})", Ty(("log",))
        if o in (".and.", ".or."):
            return f"({lc} {'&&' if o == '.and.' else '||'} {rc})", Ty(("log",))
        raise NotImplementedError(o)

    # ---------------------------------------------------------- intrinsics
    def intrinsic(self, name, args):
        if name in ("maxval", "minval", "sum"):
            return self.reduction(name, args[0])
        if name == "size":
            c, t = self.designator(args[0])
            if len(args) > 1:
                return f"{c}.size({self.expr(args[1])[0]})", Ty(("int",))
            return f"{c}.size()", Ty(("int",))
        if name == "allocated":
            c, t = self.designator(args[0])
            return f"{c}.allocated()", Ty(("log",))
        if name == "associated":
            c, t = self.designator(args[0])
            return f"({c} != nullptr)", Ty(("log",))
        if name == "null":
            return "nullptr", Ty(("null",))
        if name == "huge":
            c, t = self.expr(args[0])
            return f"std::numeric_limits<{ctype(t.base)}>::max()", t
        if name == "epsilon":
            c, t = self.expr(args[0])
            return f"std::numeric_limits<{ctype(t.base)}>::epsilon()", t
        vals = [self.expr(a) if a.op != "kw" else (a, None) for a in args]
        return self.intrinsic_codes(name, vals, raw=args)

    def intrinsic_codes(self, name, vals, raw=None):
        def kindarg():
            for v in vals[1:]:
                if v[1] is None:   # keyword
                    return v[0].b
            if len(vals) > 1 and raw is not None:
                return raw[1]
            return None
        c = [v[0] for v in vals]
        t = [v[1] for v in vals]
        if name in ("sqrt", "exp", "log", "cos", "sin", "tan", "tanh", "atan", "acos", "asin", "log10"):
            return f"std::{name}({c[0]})", t[0]
        if name == "abs":
            return f"std::abs({c[0]})", t[0]
        if name in ("min", "max"):
            tt = t[0].base
            for x in t[1:]:
                tt = promote(tt, x.base)
            ct = ctype(tt)
            return f"f{name}<{ct}>({', '.join(f'({ct})({x})' for x in c)})", Ty(tt)
        if name in ("real", "dble"):
            k = kindarg()
            dbl = name == "dble" or (k is not None and (getattr(k, "op", None) == "name" and k.a == "dp"
                                                        or getattr(k, "op", None) == "num" and k.a == "8"))
            return f"(({'double' if dbl else 'float'})({c[0]}))", Ty(("real", "dp" if dbl else "sp"))
        if name == "int":
            return f"((int)({c[0]}))", Ty(("int",))
        if name == "nint":
            return f"((int)std::lround({c[0]}))", Ty(("int",))
        if name == "floor":
            return f"((int)std::floor({c[0]}))", Ty(("int",))
        if name == "ceiling":
            return f"((int)std::ceil({c[0]}))", Ty(("int",))
        if name == "mod":
            if t[0].base[0] == "int":
                return f"(({c[0]}) % ({c[1]}))", t[0]
            return f"std::fmod({c[0]}, {c[1]})", t[0]
        if name == "sign":
            return f"fsign({c[0]}, {c[1]})", t[0]
        if name == "merge":
            tt = promote(t[0].base, t[1].base) if t[0].num() else t[0].base
            return f"(({c[2]}) ? ({ctype(tt)})({c[0]}) : ({ctype(tt)})({c[1]}))", Ty(tt)
        if name in ("ieee_is_nan", "isnan"):
            return f"std::isnan({c[0]})", Ty(("log",))
        if name == "ieee_is_finite":
            return f"std::isfinite({c[0]})", Ty(("log",))
        if name == "trim":
            return c[0], t[0]
        raise NotImplementedError(f"intrinsic {name} in {self.where}")

    def reduction(self, name, arg):
        r = self.rank_of(arg)
        shp = self.shape(arg)
        kv = [self.fresh("k") for _ in range(r)]
        ec, et = self.elem(arg, kv)
        ct = ctype(et.base)
        init = {"maxval": f"-std::numeric_limits<{ct}>::max()", "minval": f"std::numeric_limits<{ct}>::max()",
                "sum": f"({ct})0"}[name]
        upd = {"maxval": f"if ({ec} > acc) acc = {ec};", "minval": f"if ({ec} < acc) acc = {ec};",
               "sum": f"acc += {ec};"}[name]
        loops = "".join(f"for (int {kv[d]} = 0; {kv[d]} < {shp[d]}; ++{kv[d]}) " for d in reversed(range(r)))
        return f"([&]() {{ {ct} acc = {init}; {loops}{{ {upd} }} return acc; }}())", Ty(et.base)

    def fresh(self, p="t"):
        self.tmp += 1
        return f"{p}{self.tmp}"

    # ---------------------------------------------------------- calls
    def actual(self, dummy, a):
        """C++ code of one actual argument for dummy Var `dummy`."""
        if dummy.rank > 0:
            r = self.rank_of(a)
            if a.op == "ref" and self.is_section(a.b):
                return self.section_view(a)
            if a.op == "comp" and r > 0:
                try:
                    c, t = self.designator(a)
                    return c if (dummy.is_alloc() or dummy.is_ptr()) else f"view1({c})"
                except SectionError:
                    raise NotImplementedError(f"array-of-component actual {a!r}")
            c, t = self.designator(a)
            if t.rank == 0:   # an element passed to an array dummy (sequence association)
                raise NotImplementedError(f"element actual for array dummy in {self.where}")
            return c if (dummy.is_alloc() or dummy.is_ptr()) else f"view1({c})"
        if dummy.is_ptr():
            c, t = self.designator(a)
            return c
        if a.op in ("name", "comp") or (a.op == "ref" and not (a.a.op == "name" and self.lookup(a.a.a)[0] != "var")):
            try:
                c, t = self.expr(a)
                want = ctype(dummy.base)
                if dummy.base[0] == "type" or want == ctype(t.base):
                    return c
                return f"lval(({want})({c}))"
            except SectionError:
                pass
        c, t = self.expr(a)
        return f"lval(({ctype(dummy.base)})({c}))"

    def section_view(self, a):
        bc, bt = self.designator(a.a)
        rngs = [(d, x) for d, x in enumerate(a.b) if x.op == "range"]
        if bt.rank == 1:
            x = a.b[0]
            lo = self.expr(x.a)[0] if x.a is not None else f"{bc}.lb[0]"
            hi = self.expr(x.b)[0] if x.b is not None else f"({bc}.lb[0] + {bc}.ex[0] - 1)"
            return f"section1({bc}, {lo}, {hi})"
        if bt.rank == 2 and len(rngs) == 1 and rngs[0][0] == 0 and a.b[0].a is None and a.b[0].b is None:
            return f"column({bc}, {self.expr(a.b[1])[0]})"
        raise NotImplementedError(f"section {a!r} in {self.where}")

    def call_args(self, proc, args):
        dummies = [proc.vars[n] for n in proc.args]
        out = [None] * len(dummies)
        pos = 0
        for a in args:
            if a.op == "kw":
                k = proc.args.index(a.a)
                out[k] = self.actual(dummies[k], a.b)
            else:
                out[pos] = self.actual(dummies[pos], a)
                pos += 1
        return ", ".join(x for x in out if x is not None)

    def call_expr(self, proc, cname, args):
        rv = proc.vars.get(proc.result)
        base = rv.base if rv is not None else proc.rtype
        return f"{cname}({self.call_args(proc, args)})", Ty(base)


class SectionError(Exception):
    pass


# ----------------------------------------------------------------- statements and units

class Emitter(Translator):
    def line(self, s):
        self.out.append("    " * self.ind + s)

    def stmts(self, body):
        for st in body:
            self.stmt(st)

    def stmt(self, st):
        self.where = f"{self.proc.module}.{self.proc.name}:{st.line}"
        k = st.kind
        if k == "noop":
            return
        if k == "assign":
            return self.assign(st.lhs, st.rhs)
        if k == "ptr":
            lc, lt = self.designator(st.lhs)
            if st.rhs.op == "ref" and st.rhs.a.op == "name" and st.rhs.a.a == "null":
                self.line(f"{lc} = nullptr;")
                return
            if lt.rank > 0:
                if st.rhs.op == "ref" and self.is_section(st.rhs.b):
                    self.line(f"{lc} = {self.section_view(st.rhs)};")
                else:
                    rc, rt_ = self.designator(st.rhs)
                    self.line(f"{lc} = view_of({rc});")
                return
            rc, rt_ = self.designator(st.rhs)
            self.line(f"{lc} = {rc};" if rt_.ptr else f"{lc} = &({rc});")
            return
        if k == "if":
            for n, (cond, body) in enumerate(st.branches):
                c, _ = self.expr(cond)
                self.line(("if" if n == 0 else "} else if") + f" ({c}) {{")
                self.ind += 1
                self.stmts(body)
                self.ind -= 1
            if st.els:
                self.line("} else {")
                self.ind += 1
                self.stmts(st.els)
                self.ind -= 1
            self.line("}")
            return
        if k == "do":
            v = self.local_name(st.var) if st.var in self.scope else self.lookup(st.var)[2]
            lo, _ = self.expr(st.lo)
            hi, _ = self.expr(st.hi)
            step = self.expr(st.step)[0] if st.step is not None else "1"
            tr, sp = self.fresh("trip"), self.fresh("st")
            # Fortran: the trip count is fixed when the loop starts
            self.line(f"{{ const int {sp} = {step}; {v} = {lo}; "
                      f"long {tr} = std::max(0L, ((long)({hi}) - (long){v} + {sp}) / {sp});")
            self.line(f"for (; {tr} > 0; --{tr}, {v} += {sp}) {{")
            self.ind += 1
            self.stmts(st.body)
            self.ind -= 1
            self.line("} }")
            return
        if k == "dowhile":
            c, _ = self.expr(st.cond)
            self.line(f"while ({c}) {{")
            self.ind += 1
            self.stmts(st.body)
            self.ind -= 1
            self.line("}")
            return
        if k == "doforever":
            self.line("for (;;) {")
            self.ind += 1
            self.stmts(st.body)
            self.ind -= 1
            self.line("}")
            return
        if k == "exit":
            self.line("break;")
            return
        if k == "cycle":
            self.line("continue;")
            return
        if k == "return":
            if self.proc.kind == "function":
                self.line(f"return {self.local_name(self.proc.result)};")
            else:
                self.line("return;")
            return
        if k == "stop":
            self.line("std::exit(0);")
            return
        if k == "goto":
            raise NotImplementedError(f"goto at {self.where}")
        if k == "call":
            kind, obj, cn = self.lookup(st.name)
            if kind is None and st.name == "random_number":
                # qsort.f90's random pivot: any sequence sorts the same (the
                # keys of a row are distinct column indices)
                c, t = self.designator(st.args[0])
                self.line(f"{c} = ({ctype(t.base)})frand01();")
                return
            if kind != "proc":
                raise NameError(f"call of unknown {st.name} at {self.where}")
            self.line(f"{cn}({self.call_args(obj, st.args)});")
            return
        if k == "allocate":
            for it in st.items:
                bc, bt = self.designator(it.a)
                bounds = []
                for a in it.b:
                    if a.op == "range":
                        bounds += [self.expr(a.a)[0], self.expr(a.b)[0]]
                    else:
                        bounds += ["1", self.expr(a)[0]]
                self.line(f"{bc}.alloc({', '.join(bounds)});")
            return
        if k == "deallocate":
            for it in st.items:
                bc, bt = self.designator(it)
                self.line(f"{bc}.dealloc();")
            return
        if k == "associate":
            self.line("{")
            self.ind += 1
            saved = dict(self.scope), dict(self.alias)
            for nm, ex in st.pairs:
                cname = self.fresh("as_" + nm)
                if ex.op == "ref" and self.is_section(ex.b):
                    code = self.section_view(ex)
                    _, bt = self.designator(ex.a)
                    self.line(f"auto {cname} = {code};")
                    var = Var(nm, bt.base, [(None, None)], set())
                else:
                    try:
                        c, t = self.designator(ex)
                        designator = ex.op in ("name", "comp", "ref") and not (
                            ex.op == "ref" and ex.a.op == "name" and self.lookup(ex.a.a)[0] != "var")
                    except SectionError:
                        raise
                    if designator:
                        if t.ptr and t.rank == 0:
                            self.line(f"auto& {cname} = *({c});")
                        else:
                            self.line(f"auto& {cname} = {c};")
                    else:
                        c, t = self.expr(ex)
                        self.line(f"auto {cname} = {c};")
                    var = Var(nm, t.base, [(None, None)] * t.rank, set())
                self.scope[nm] = var
                self.alias[nm] = cname
            self.stmts(st.body)
            self.scope, self.alias = saved
            self.ind -= 1
            self.line("}")
            return
        if k == "select":
            c, _ = self.expr(st.sel)
            sv = self.fresh("sel")
            self.line(f"{{ const auto {sv} = {c};")
            first = True
            for vals, body in st.cases:
                if vals is None:
                    self.line("} else {" if not first else "{")
                else:
                    conds = []
                    for v in vals:
                        if v.op == "range":
                            lo = self.expr(v.a)[0] if v.a is not None else None
                            hi = self.expr(v.b)[0] if v.b is not None else None
                            parts = ([f"{sv} >= {lo}"] if lo else []) + ([f"{sv} <= {hi}"] if hi else [])
                            conds.append("(" + " && ".join(parts) + ")")
                        else:
                            conds.append(f"{sv} == {self.expr(v)[0]}")
                    self.line(("if" if first else "} else if") + f" ({' || '.join(conds)}) {{")
                first = False
                self.ind += 1
                self.stmts(body)
                self.ind -= 1
            if not first:
                self.line("}")
            self.line("}")
            return
        raise NotImplementedError(f"statement {k} at {self.where}")

    def assign(self, lhs, rhs):
        lr = self.rank_of(lhs)
        if lr == 0:
            lc, lt = self.designator(lhs)
            if lt.ptr:
                lc = f"(*{lc})"
            rr = self.rank_of(rhs)
            if rr > 0:
                raise NotImplementedError(f"array to scalar at {self.where}")
            rc, rt_ = self.expr(rhs)
            if lt.base[0] in ("int", "real", "log") and ctype(lt.base) != ctype(rt_.base):
                rc = f"({ctype(lt.base)})({rc})"
            self.line(f"{lc} = {rc};")
            return
        # array assignment: loops over the left side's shape
        if rhs.op == "ctor":
            lc, lt = self.designator(lhs)
            for n, it in enumerate(rhs.a):
                c, _ = self.expr(it)
                self.line(f"{lc}({lc}.lb[0] + {n}) = {c};")
            return
        shp = self.shape(lhs)
        kv = [self.fresh("k") for _ in range(lr)]
        ec, et = self.elem(lhs, kv)
        rc, rt_ = self.elem(rhs, kv)
        if et.base[0] in ("int", "real", "log") and ctype(et.base) != ctype(rt_.base):
            rc = f"({ctype(et.base)})({rc})"
        loops = "".join(f"for (int {kv[d]} = 0; {kv[d]} < {shp[d]}; ++{kv[d]}) " for d in reversed(range(lr)))
        self.line(f"{loops}{{ {ec} = {rc}; }}")

    # ---------------------------------------------------------- declarations
    def decl_type(self, v, dummy=False):
        if v.rank > 0:
            t = arr_type(v)
            if dummy:
                return (t + "&") if (v.is_alloc() or v.is_ptr()) else f"const {t}&"
            return t
        t = ctype(v.base)
        if v.is_ptr():
            return t + "*"
        return t + "&" if dummy else t

    def proc_sig(self, p, cname):
        params = []
        for a in p.args:
            v = p.vars[a]
            params.append(f"{self.decl_type(v, True)} {a}_")
        if p.kind == "function":
            rv = p.vars.get(p.result)
            rt_ = ctype(rv.base if rv is not None else p.rtype)
        else:
            rt_ = "void"
        return f"{rt_} {cname}({', '.join(params)})"

    def proc_def(self, p, mod):
        self.proc = p
        self.scope = dict(p.vars)
        self.alias = {}
        if p.kind == "function" and p.result not in self.scope:
            self.scope[p.result] = Var(p.result, p.rtype)
        self.vis = self.visible_modules(mod.name, p.uses)
        cname = self.gname(mod.name, p.name)
        self.where = f"{mod.name}.{p.name}"
        self.line(self.proc_sig(p, cname) + " {")
        self.ind += 1
        for n, v in p.vars.items():
            if n in p.args:
                continue
            self.local_decl(v)
        if p.kind == "function" and p.result not in p.vars:
            self.line(f"{ctype(p.rtype)} {p.result}_{{}};")
        self.stmts(p.body)
        if p.kind == "function":
            self.line(f"return {self.local_name(p.result)};")
        self.ind -= 1
        self.line("}")
        self.line("")

    def local_decl(self, v):
        nm = v.name + "_"
        if v.rank > 0:
            self.line(f"{arr_type(v)} {nm};")
            if not v.is_alloc() and not v.is_ptr() and all(d[1] is not None for d in v.dims):
                b = []
                for lo, hi in v.dims:
                    b += [self.expr(lo)[0] if lo is not None else "1", self.expr(hi)[0]]
                self.line(f"{nm}.alloc({', '.join(b)});")
            return
        if v.is_ptr():
            self.line(f"{ctype(v.base)}* {nm} = nullptr;")
            return
        if "parameter" in v.attrs:
            c, _ = self.expr(v.init[1])
            self.line(f"const {ctype(v.base)} {nm} = {c};")
            return
        if v.init is not None and v.init[0] == "=":
            c, t = self.expr(v.init[1])
            # Fortran: an initialised local is implicitly SAVE'd
            self.line(f"static {ctype(v.base)} {nm} = {c};")
            return
        self.line(f"{ctype(v.base)} {nm}{{}};")

    # ---------------------------------------------------------- units
    def type_order(self):
        """Derived types in an order where every by-value component's type
        comes first."""
        done, order = set(), []

        def visit(tn, stack=()):
            if tn in done:
                return
            for v in self.types[tn].values():
                if v.base[0] == "type" and not v.is_ptr() and v.base[1] != tn and v.base[1] not in stack:
                    visit(v.base[1], stack + (tn,))
            done.add(tn)
            order.append(tn)
        for tn in self.types:
            visit(tn)
        return order

    def emit_types(self):
        for tn in self.types:
            self.line(f"struct T_{tn};")
        self.line("")
        self.proc = Proc("subroutine", "<types>", [])
        self.proc.module = "<types>"
        self.scope, self.alias, self.vis = {}, {}, list(self.mods)
        for tn in self.type_order():
            self.line(f"struct T_{tn} {{")
            self.ind += 1
            for v in self.types[tn].values():
                nm = v.name + "_"
                if v.rank > 0:
                    self.line(f"{arr_type(v)} {nm};")
                elif v.is_ptr():
                    self.line(f"{ctype(v.base)}* {nm} = nullptr;")
                elif v.init is not None and v.init[0] == "=":
                    c, _ = self.expr(v.init[1])
                    self.line(f"{ctype(v.base)} {nm} = {c};")
                else:
                    self.line(f"{ctype(v.base)} {nm}{{}};")
            self.ind -= 1
            self.line("};")
        self.line("")

    def module_order(self):
        done, order = set(), []

        def visit(mn):
            if mn in done or mn not in self.mods:
                return
            done.add(mn)
            for u, _ in self.mods[mn].uses:
                visit(u)
            for p in self.mods[mn].procs.values():
                for u, _ in p.uses:
                    visit(u)
            order.append(mn)
        for mn in self.mods:
            visit(mn)
        return order

    def emit_globals(self, mod):
        self.proc = Proc("subroutine", "<globals>", [])
        self.proc.module = mod.name
        self.scope, self.alias = {}, {}
        self.vis = self.visible_modules(mod.name)
        for n in mod.order:
            v = mod.vars[n]
            gn = self.gname(mod.name, n)
            self.where = gn
            if v.rank > 0:
                self.line(f"{arr_type(v)} {gn};")
                if not v.is_alloc() and not v.is_ptr() and all(d[1] is not None for d in v.dims):
                    b = []
                    for lo, hi in v.dims:
                        b += [self.expr(lo)[0] if lo is not None else "1", self.expr(hi)[0]]
                    self.line(f"static const bool {gn}_init = ({gn}.alloc({', '.join(b)}), true);")
            elif v.is_ptr():
                self.line(f"{ctype(v.base)}* {gn} = nullptr;")
            elif v.init is not None and v.init[0] == "=":
                c, _ = self.expr(v.init[1])
                q = "const " if "parameter" in v.attrs else ""
                self.line(f"{q}{ctype(v.base)} {gn} = {c};")
            else:
                self.line(f"{ctype(v.base)} {gn}{{}};")

    def translate(self):
        self.ind = 0
        self.out = [RUNTIME]
        self.emit_types()
        order = self.module_order()
        for mn in order:
            self.emit_globals(self.mods[mn])
        self.line("")
        for mn in order:
            m = self.mods[mn]
            for p in m.procs.values():
                self.proc = p
                self.line(self.proc_sig(p, self.gname(mn, p.name)) + ";")
        self.line("")
        for mn in order:
            m = self.mods[mn]
            for p in m.procs.values():
                self.proc_def(p, m)
        return "\n".join(self.out) + "\n"


RUNTIME = r"""// generated from Fortran source by oracle/ref_translate.py -- do not edit
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

// Fortran array: column-major, per-dimension lower bounds; owning (allocatable)
// or a view of another array's storage (sections, dummy arguments).
template <class T, int R>
struct Arr {
    T* p = nullptr;
    int lb[R] = {};
    int ex[R] = {};
    bool own = false;
    Arr() {}
    Arr(const Arr& o) { copy_from(o); }
    Arr& operator=(const Arr& o) {
        if (this == &o) return *this;
        if (own || !p) {   // allocatable: reallocate to the right side's shape
            if (!o.p) { dealloc(); return *this; }
            bool same = p != nullptr;
            for (int d = 0; d < R; ++d) same = same && ex[d] == o.ex[d];
            if (!same) { dealloc(); p = new T[o.count()](); own = true; }
            for (int d = 0; d < R; ++d) { lb[d] = o.lb[d]; ex[d] = o.ex[d]; }
        }
        const long n = count();
        for (long i = 0; i < n; ++i) p[i] = o.p[i];
        return *this;
    }
    ~Arr() { if (own) delete[] p; }
    void copy_from(const Arr& o) {
        if (!o.p) return;
        for (int d = 0; d < R; ++d) { lb[d] = o.lb[d]; ex[d] = o.ex[d]; }
        const long n = o.count();
        p = new T[n]();
        own = true;
        for (long i = 0; i < n; ++i) p[i] = o.p[i];
    }
    long count() const { long n = 1; for (int d = 0; d < R; ++d) n *= ex[d]; return p ? n : 0; }
    void alloc(int l0, int u0) {
        static_assert(R == 1, "rank");
        dealloc(); lb[0] = l0; ex[0] = std::max(0, u0 - l0 + 1);
        p = new T[std::max(1, ex[0])](); own = true;
    }
    void alloc(int l0, int u0, int l1, int u1) {
        static_assert(R == 2, "rank");
        dealloc(); lb[0] = l0; ex[0] = std::max(0, u0 - l0 + 1); lb[1] = l1; ex[1] = std::max(0, u1 - l1 + 1);
        p = new T[std::max(1L, (long)ex[0] * ex[1])](); own = true;
    }
    void dealloc() { if (own) delete[] p; p = nullptr; own = false; for (int d = 0; d < R; ++d) ex[d] = 0; }
    bool allocated() const { return p != nullptr; }
    int size() const { return (int)count(); }
    int size(int d) const { return ex[d - 1]; }
    T& operator()(int i) const { return p[i - lb[0]]; }
    T& operator()(int i, int j) const { return p[(long)(i - lb[0]) + (long)ex[0] * (j - lb[1])]; }
};

// a view with lower bounds 1 (assumed-shape and explicit-shape dummies)
template <class T, int R>
Arr<T, R> view1(const Arr<T, R>& a) {
    Arr<T, R> v;
    v.p = a.p;
    for (int d = 0; d < R; ++d) { v.lb[d] = 1; v.ex[d] = a.ex[d]; }
    return v;
}
template <class T, int R>
Arr<T, R> view_of(const Arr<T, R>& a) {
    Arr<T, R> v;
    v.p = a.p;
    for (int d = 0; d < R; ++d) { v.lb[d] = a.lb[d]; v.ex[d] = a.ex[d]; }
    return v;
}
// a(lo:hi) of a rank-1 array, lower bound 1
template <class T>
Arr<T, 1> section1(const Arr<T, 1>& a, int lo, int hi) {
    Arr<T, 1> v;
    v.p = a.p + (lo - a.lb[0]);
    v.lb[0] = 1;
    v.ex[0] = std::max(0, hi - lo + 1);
    return v;
}
// a(:, j) of a rank-2 array (contiguous), lower bound 1
template <class T>
Arr<T, 1> column(const Arr<T, 2>& a, int j) {
    Arr<T, 1> v;
    v.p = a.p + (long)a.ex[0] * (j - a.lb[1]);
    v.lb[0] = 1;
    v.ex[0] = a.ex[0];
    return v;
}

inline double frand01() {   // deterministic uniform [0, 1) (64-bit LCG)
    static unsigned long long s = 0x2545F4914F6CDD1DULL;
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
}
template <class T> T& lval(T&& x) { return x; }
template <class T> T& lval(T& x) { return x; }

template <class T> T fmin(T a) { return a; }
template <class T, class... R> T fmin(T a, T b, R... r) { return fmin<T>(b < a ? b : a, r...); }
template <class T> T fmax(T a) { return a; }
template <class T, class... R> T fmax(T a, T b, R... r) { return fmax<T>(b > a ? b : a, r...); }
template <class T, class U> T fsign(T a, U b) { return b >= 0 ? std::abs(a) : -std::abs(a); }

// x**n, n integer: repeated squaring (x**2 = x*x, x**3 = x*x*x)
template <class T>
T ipow(T x, int n) {
    if (n < 0) return T(1) / ipow(x, -n);
    if (n == 0) return T(1);
    if (n == 1) return x;
    if (n == 2) return x * x;
    if (n == 3) return x * x * x;
    T r = T(1), b = x;
    while (n) { if (n & 1) r *= b; b *= b; n >>= 1; }
    return r;
}
"""


def translate_files(named_sources):
    """[(file name, text)] -> C++ source of all their modules."""
    mods = []
    for fname, text in named_sources:
        mods += parse_source(text, fname)
    return Emitter(mods).translate()
