"""Execute routines of the reference's Fortran 90 source in Python, for test
vectors only (TEST INFRASTRUCTURE: no compiler for the reference exists in
this image, so its routines are translated statement by statement into
Python and run on numpy arrays, with Fortran's semantics kept where they
matter: 1-based, column-major arrays and inclusive array sections, sequential
sums, double precision throughout as the reference's -fdefault-real-8 build
has it; the routines translated here divide only reals, so '/' is Python's).

The subset is what the step path's leaf routines use: declarations (`real`,
`real*8`, `integer`, with `dimension(...)` or per-entity shapes), `do` loops,
block and one-line `if`, `select case`, one-line `where`, assignments to
scalars, elements, sections and whole arrays, `call`, and the intrinsics
sqrt, abs, min, max, sum, minval, maxval, exp, log, sin, cos, mod, real,
dble, int.  Anything else raises, so a routine outside the subset is refused
rather than mistranslated.

    ns = namespace(module_values)              # params and module arrays
    f = translate(source_text, "flux_hllc", ns) # a Python function
    f(Qlr, flr, fhllc, 1)                      # FArray arguments, in place
"""
from __future__ import annotations

import math
import re

import numpy as np


# ---- runtime --------------------------------------------------------------
class Section:
    """An inclusive Fortran section lo:hi (None: the bound of the dimension)."""
    __slots__ = ("lo", "hi")

    def __init__(self, lo, hi):
        self.lo, self.hi = lo, hi


class FArray:
    """A Fortran array: column-major storage, 1-based indices, inclusive
    sections; element reads give numpy float64 scalars."""
    __array_priority__ = 100

    def __init__(self, shape_or_data, dtype=np.float64):
        if isinstance(shape_or_data, np.ndarray):
            self.a = shape_or_data
        else:
            shape = tuple(int(s) for s in (shape_or_data if isinstance(shape_or_data, tuple) else (shape_or_data,)))
            self.a = np.zeros(shape, dtype=dtype, order="F")

    def _index(self, key):
        if key is Ellipsis:
            return Ellipsis
        if not isinstance(key, tuple):
            key = (key,)
        if len(key) != self.a.ndim:
            raise IndexError(f"rank {self.a.ndim} array indexed with {len(key)} subscripts")
        out = []
        for k in key:
            if isinstance(k, Section):
                out.append(slice(None if k.lo is None else int(k.lo) - 1, None if k.hi is None else int(k.hi)))
            else:
                if int(k) != k:
                    raise IndexError(f"non-integer subscript {k}")
                if int(k) < 1:
                    raise IndexError(f"subscript {k} below 1")
                out.append(int(k) - 1)
        return tuple(out)

    def __getitem__(self, key):
        return self.a[self._index(key)]

    def __setitem__(self, key, value):
        self.a[self._index(key)] = np.asarray(value) if isinstance(value, FArray) else value

    def __array__(self, dtype=None, copy=None):
        return self.a if dtype is None else self.a.astype(dtype)

    def _bin(op):
        def f(self, other):
            return op(self.a, other.a if isinstance(other, FArray) else other)
        return f

    def _rbin(op):
        def f(self, other):
            return op(other, self.a)
        return f

    import operator as _op
    __add__, __sub__, __mul__, __truediv__, __pow__ = (_bin(_op.add), _bin(_op.sub), _bin(_op.mul),
                                                       _bin(_op.truediv), _bin(_op.pow))
    __radd__, __rsub__, __rmul__, __rtruediv__, __rpow__ = (_rbin(_op.add), _rbin(_op.sub), _rbin(_op.mul),
                                                            _rbin(_op.truediv), _rbin(_op.pow))
    __eq__, __ne__, __lt__, __le__, __gt__, __ge__ = (_bin(_op.eq), _bin(_op.ne), _bin(_op.lt), _bin(_op.le),
                                                      _bin(_op.gt), _bin(_op.ge))
    __neg__ = lambda self: -self.a
    __hash__ = None


def _arr(x):
    return x.a if isinstance(x, FArray) else x


def _sum(x):
    """Fortran's sum of an array expression, left to right."""
    s = 0.0
    for v in np.ravel(np.asarray(_arr(x)), order="F"):
        s = s + v
    return s


def _min(*a):
    if any(isinstance(_arr(x), np.ndarray) and np.ndim(_arr(x)) for x in a):
        r = _arr(a[0])
        for x in a[1:]:
            r = np.minimum(r, _arr(x))
        return r
    r = a[0]
    for x in a[1:]:
        if x < r:
            r = x
    return r


def _max(*a):
    if any(isinstance(_arr(x), np.ndarray) and np.ndim(_arr(x)) for x in a):
        r = _arr(a[0])
        for x in a[1:]:
            r = np.maximum(r, _arr(x))
        return r
    r = a[0]
    for x in a[1:]:
        if x > r:
            r = x
    return r


def _mod(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        return int(math.fmod(a, b))
    return math.fmod(a, b)


def _idiv(a, b):
    """Fortran '/': truncating for two integers."""
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b >= 0) else -q
    return a / b


def _where(mask, target, value):
    t = target.a
    t[...] = np.where(np.asarray(mask), np.asarray(_arr(value)), t)


INTRINSICS = {
    "sqrt": "np.sqrt", "abs": "np.abs", "min": "_min", "max": "_max", "sum": "_sum",
    "minval": "np.min", "maxval": "np.max", "exp": "np.exp", "log": "np.log", "sin": "np.sin",
    "cos": "np.cos", "mod": "_mod", "real": "float", "dble": "float", "int": "int",
}


def namespace(values: dict) -> dict:
    ns = {"np": np, "math": math, "Section": Section, "FArray": FArray, "_sum": _sum, "_min": _min,
          "_max": _max, "_mod": _mod, "_idiv": _idiv, "_where": _where}
    ns.update({k.lower(): v for k, v in values.items()})
    return ns


# ---- translation ------------------------------------------------------------
_NUM = re.compile(r"(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?")
_TOK = re.compile(r"\s*('[^']*'|\*\*|==|/=|<=|>=|<|>|\.and\.|\.or\.|\.not\.|\.eq\.|\.ne\.|\.lt\.|\.le\.|\.gt\.|\.ge\."
                  r"|\.true\.|\.false\.|[A-Za-z_]\w*|\d+\.\d*(?:[ed][+-]?\d+)?|\.\d+(?:[ed][+-]?\d+)?"
                  r"|\d+(?:[ed][+-]?\d+)?|[-+*/(),:=])")
_LOGIC = {".and.": " and ", ".or.": " or ", ".not.": " not ", ".eq.": "==", ".ne.": "!=", ".lt.": "<",
          ".le.": "<=", ".gt.": ">", ".ge.": ">=", "/=": "!=", ".true.": "True", ".false.": "False"}
_PYKW = {"in", "is", "not", "and", "or", "if", "else", "for", "while", "def", "class", "return", "lambda",
         "pass", "del", "from", "import", "as", "with", "global", "yield", "try", "except", "raise", "break",
         "continue", "none", "true", "false"}


def _name(n):
    return n + "_" if n in _PYKW else n


def _tokens(s):
    out, pos = [], 0
    s = s.rstrip()
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m or m.end() == pos:
            raise SyntaxError(f"cannot tokenise {s[pos:]!r} in {s!r}")
        out.append(m.group(1))
        pos = m.end()
    return out


class _Expr:
    def __init__(self, arrays, ints):
        self.arrays, self.ints = arrays, ints

    def tr(self, s):
        toks = _tokens(s)
        py, _ = self._seq(toks, 0, stop=())
        return py

    def _seq(self, t, i, stop):
        out = []
        while i < len(t) and t[i] not in stop:
            tok = t[i]
            low = tok.lower()
            if low in _LOGIC:
                out.append(_LOGIC[low])
                i += 1
            elif re.match(r"[A-Za-z_]", tok):
                name = low
                if i + 1 < len(t) and t[i + 1] == "(":
                    args, i = self._args(t, i + 2)
                    if name in self.arrays:
                        out.append(_name(name) + "[" + ", ".join(args) + "]")
                    elif name in INTRINSICS:
                        out.append(INTRINSICS[name] + "(" + ", ".join(args) + ")")
                    else:
                        out.append(_name(name) + "(" + ", ".join(args) + ")")
                else:
                    out.append(_name(name))
                    i += 1
            elif tok.startswith("'"):
                out.append(repr(tok[1:-1]))
                i += 1
            elif _NUM.fullmatch(low):
                out.append(low.replace("d", "e"))
                i += 1
            elif tok == "(":
                inner, i = self._seq(t, i + 1, stop=(")",))
                out.append("(" + inner + ")")
                i += 1
            elif tok == "/":
                out.append(" / ")
                i += 1
            else:
                out.append(tok)
                i += 1
        return "".join(out), i

    def _args(self, t, i):
        """Arguments up to the matching ')'; sections a:b become Section(a, b)."""
        args, cur, depth = [], [], 0
        while True:
            tok = t[i]
            if tok == "(":
                depth += 1
            elif tok == ")":
                if depth == 0:
                    break
                depth -= 1
            if tok == "," and depth == 0:
                args.append(cur)
                cur = []
            else:
                cur.append(tok)
            i += 1
        args.append(cur)
        out = []
        for a in args:
            depth, split = 0, None
            for k, tok in enumerate(a):
                depth += tok == "("
                depth -= tok == ")"
                if tok == ":" and depth == 0:
                    split = k
            if split is None:
                out.append(self._seq(a, 0, ())[0] if a else "")
            else:
                lo = self._seq(a[:split], 0, ())[0] if split else "None"
                hi = self._seq(a[split + 1:], 0, ())[0] if split + 1 < len(a) else "None"
                out.append(f"Section({lo}, {hi})")
        return out, i + 1


def _logical_lines(text):
    lines, buf = [], ""
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip() if "!" in raw else raw.rstrip()
        s = line.strip()
        if buf and s.startswith("&"):
            s = s[1:].strip()
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        s = buf + s
        buf = ""
        if s:
            lines.append(s)
    return lines


def _decl_entities_raw(rest):
    """'a(n,m), b=1, c(k)' -> ['a(n,m)', 'b=1', 'c(k)']"""
    out, depth, cur = [], 0, ""
    for ch in rest:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _decl_entities(rest):
    """'a(n,m), b, c(k)' -> [(name, dims or None)]"""
    out, depth, cur = [], 0, ""
    for ch in rest:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    ents = []
    for e in out:
        m = re.match(r"(\w+)\s*(?:\((.*)\))?$", e)
        ents.append((m.group(1).lower(), m.group(2)))
    return ents


def translate(source: str, routine: str, ns: dict):
    """The Python function of subroutine or function `routine` of `source`."""
    low = source.lower()
    m = re.search(r"^\s*(?:real\s+)?(subroutine|function)\s+" + routine.lower() + r"\b\s*(?:\(([^)]*)\))?", low,
                  flags=re.M)
    if not m:
        raise KeyError(routine)
    kind = m.group(1)
    params = [p.strip() for p in (m.group(2) or "").split(",") if p.strip()]
    end = re.search(r"^\s*end\s+" + kind + r"(\s+" + routine.lower() + r")?\s*$", low[m.end():], flags=re.M)
    body = low[m.end():m.end() + end.start()]
    body = body.split("\n", 1)[1] if "\n" in body else ""
    lines = _logical_lines(body)

    arrays = {k for k, v in ns.items() if isinstance(v, FArray)}
    ints, local_arrays, code = set(), [], []
    stmts, inits = [], []
    for s in lines:
        d = re.match(r"(real\*8|real|integer|logical)\b\s*(,[^:]*)?(::)?\s*(.*)$", s)
        if d and (d.group(3) or ("=" not in s and not re.match(r"(real|integer|logical)\s*\(", s))):
            attrs = d.group(2) or ""
            dim = re.search(r"dimension\s*\(([^)]*)\)", attrs)
            ents = []
            for e in _decl_entities_raw(d.group(4)):
                if "=" in e and "(" not in e.split("=")[0]:
                    nm, val = e.split("=", 1)
                    inits.append((nm.strip().lower(), val.strip()))
                    e = nm
                ents.append(e)
            for name, dims in _decl_entities(", ".join(ents)):
                dims = dims or (dim.group(1) if dim else None)
                if d.group(1) == "integer" and not dims:
                    ints.add(name)
                if dims:
                    arrays.add(name)
                    if name not in params:
                        local_arrays.append((name, dims))
            continue
        if s in ("implicit none",) or s.startswith(("use ", "print", "write", "save")):
            continue
        stmts.append(s)

    ex = _Expr(arrays, ints)
    indent = 1
    sel = []
    # module scalars the routine assigns (kx ... set by the basis flags, c2d3cv by the point flux):
    # module variables, so 'global' in Python
    declared = {n for n, _ in local_arrays} | set(params)
    for s in lines:
        d = re.match(r"(real\*8|real|integer|logical)\b\s*(,[^:]*)?(::)?\s*(.*)$", s)
        if d and (d.group(3) or ("=" not in s and not re.match(r"(real|integer|logical)\s*\(", s))):
            declared |= {e.split("=")[0].strip().split("(")[0].strip().lower() for e in _decl_entities_raw(d.group(4))}
    assigned = set()
    for s in stmts:
        m = re.match(r"(?:if\s*\(.*\)\s*)?(\w+)\s*=(?!=)", s)
        if m:
            assigned.add(m.group(1))
    glob = sorted(n for n in assigned if n not in declared and n in ns and not isinstance(ns[n], FArray))
    if glob:
        code.append("    global " + ", ".join(_name(n) for n in glob))

    def emit(line):
        code.append("    " * indent + line)

    for name, dims in local_arrays:
        shape = ", ".join(ex.tr(x) for x in dims.split(","))
        emit(f"{_name(name)} = FArray(({shape},))")
    for name, val in inits:
        emit(f"{_name(name)} = {ex.tr(val)}")
    for s in stmts:
        if re.match(r"do\s+\w+\s*=", s):
            m = re.match(r"do\s+(\w+)\s*=\s*(.*)$", s)
            parts = ex._args(_tokens(m.group(2)) + [")"], 0)[0]
            step = f", {parts[2]}" if len(parts) > 2 else ""
            stop = f"({parts[1]}) + 1" if not step else f"({parts[1]}) + ({parts[2]} > 0) - ({parts[2]} < 0)"
            emit(f"for {_name(m.group(1))} in range({parts[0]}, {stop}{step}):")
            indent += 1
        elif re.match(r"end\s*do$", s):
            indent -= 1
        elif re.match(r"(else\s*if)\s*\(", s):
            cond = s[s.index("(") + 1:s.rindex(")")]
            indent -= 1
            emit(f"elif {ex.tr(cond)}:")
            indent += 1
        elif s == "else":
            indent -= 1
            emit("else:")
            indent += 1
        elif re.match(r"end\s*if$", s):
            indent -= 1
        elif re.match(r"if\s*\(", s):
            depth, k = 0, s.index("(")
            for k in range(s.index("("), len(s)):
                depth += s[k] == "("
                depth -= s[k] == ")"
                if depth == 0:
                    break
            cond, tail = s[s.index("(") + 1:k], s[k + 1:].strip()
            if tail == "then":
                emit(f"if {ex.tr(cond)}:")
                indent += 1
            else:
                emit(f"if {ex.tr(cond)}:")
                indent += 1
                emit(_stmt(tail, ex, arrays))
                indent -= 1
        elif re.match(r"select\s+case\s*\(", s):
            sel.append([f"_sel{len(sel)}", False])
            emit(f"{sel[-1][0]} = {ex.tr(s[s.index('(') + 1:s.rindex(')')])}")
        elif re.match(r"case\s+default$", s):
            if sel[-1][1]:
                indent -= 1
                emit("else:")
            else:
                emit("if True:")
            sel[-1][1] = True
            indent += 1
        elif re.match(r"case\s*\(", s):
            vals = ex._args(_tokens(s[s.index("(") + 1:]), 0)[0]
            if sel[-1][1]:
                indent -= 1
                emit(f"elif {sel[-1][0]} in ({', '.join(vals)},):")
            else:
                emit(f"if {sel[-1][0]} in ({', '.join(vals)},):")
            sel[-1][1] = True
            indent += 1
        elif re.match(r"end\s*select$", s):
            if sel.pop()[1]:
                indent -= 1
        elif re.match(r"where\s*\(", s):
            depth = 0
            for k in range(s.index("("), len(s)):
                depth += s[k] == "("
                depth -= s[k] == ")"
                if depth == 0:
                    break
            mask, tail = s[s.index("(") + 1:k], s[k + 1:].strip()
            lhs, rhs = tail.split("=", 1)
            emit(f"_where({ex.tr(mask)}, {_name(lhs.strip())}, {ex.tr(rhs)})")
        else:
            emit(_stmt(s, ex, arrays))
    if indent != 1 or sel:
        raise SyntaxError(f"{routine}: unbalanced blocks")
    ret = f"    return {_name(routine.lower())}" if kind == "function" else "    return None"
    src = f"def {_name(routine.lower())}({', '.join(_name(p) for p in params)}):\n" + "\n".join(code) + "\n" + ret + "\n"
    exec(compile(src, f"<{routine}>", "exec"), ns)
    fn = ns[_name(routine.lower())]
    fn.python_source = src
    return fn


def _stmt(s, ex, arrays):
    if s.startswith("call "):
        c = s[5:].strip()
        return ex.tr(c) if "(" in c else _name(c) + "()"
    if s in ("return",):
        return "pass"
    if s == "cycle":
        return "continue"
    if s == "exit":
        return "break"
    m = re.match(r"(\w+)\s*(\(.*\))?\s*=(?!=)\s*(.*)$", s)
    if not m:
        raise SyntaxError(f"statement outside the subset: {s!r}")
    name, sub, rhs = m.group(1), m.group(2), m.group(3)
    if sub:
        return f"{ex.tr(name + sub)} = {ex.tr(rhs)}"
    if name in arrays:
        return f"{_name(name)}[...] = {ex.tr(rhs)}"
    return f"{_name(name)} = {ex.tr(rhs)}"
