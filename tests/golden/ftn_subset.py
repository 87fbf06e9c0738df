"""Executes a subset of Fortran 90 -- the subset the OllinAxis-BiB evolution
path is written in -- by translating each program unit to Python/numpy.

This is golden-vector machinery, not part of the product and not part of the
oracle: it lets ``make_golden.py`` run the reference's *own* Fortran sources
(which cannot be compiled here: the image has no Fortran compiler) on small
grids and record the results as fixtures.  It only runs where the reference
sources exist; the committed fixtures are what travel.

Semantics that matter for floating-point agreement:
  * real literals without a ``d`` exponent are single precision
    (``np.float32``), exactly like default-kind reals in Fortran, so
    ``acos(-1.0)`` is the single-precision pi and ``3.0/4.0`` is computed in
    single precision; ``real(8)`` scalars are ``np.float64``;
  * integer powers ``x**n`` use square-and-multiply from the most significant
    bit (``ipow``), the same chain the C++ oracle uses;
  * integer ``/`` truncates toward zero, ``nint`` rounds half away from zero;
  * whole-array expressions are evaluated completely before assignment and
    assignments to existing arrays are in place, so pointer aliasing
    (``diffvar => alpha``) behaves as in Fortran.
"""
import math
import re

import numpy as np

F32 = np.float32
F64 = np.float64


# ----------------------------------------------------------------------------
# runtime helpers used by the generated code
# ----------------------------------------------------------------------------

import keyword as _keyword


def pyname(name):
    """Fortran names that are Python keywords (``lambda``) get a trailing '_'."""
    return name + "_" if _keyword.iskeyword(name) else name


class FArray(np.ndarray):
    """ndarray with Fortran lower bounds (attribute ``lb``)."""

    def __array_finalize__(self, obj):
        self.lb = getattr(obj, "lb", None)


def falloc(lbs, ubs, fill=0.0):
    shape = tuple(u - l + 1 for l, u in zip(lbs, ubs))
    a = np.full(shape, fill, dtype=np.float64, order="F").view(FArray)
    a.lb = tuple(lbs)
    return a


def _conv(arr, idx):
    out = []
    for k, ix in enumerate(idx):
        lb = arr.lb[k]
        if isinstance(ix, slice):
            start = 0 if ix.start is None else ix.start - lb
            stop = arr.shape[k] if ix.stop is None else ix.stop - lb + 1
            out.append(slice(start, stop))
        else:
            out.append(int(ix) - lb)
    return tuple(out)


# reads past the end of an allocation (see fget)
OOB_BEYOND = [0]


def fget(arr, idx):
    if isinstance(arr, str):
        # character substring s(a:b), 1-based and inclusive, blank padded
        sl = idx[0]
        lo = 1 if sl.start is None else int(sl.start)
        hi = len(arr) if sl.stop is None else int(sl.stop)
        return arr.ljust(hi)[lo - 1:hi]
    cidx = _conv(arr, idx)
    if all(isinstance(c, int) for c in cidx) and \
            any(c < 0 or c >= n for c, n in zip(cidx, arr.shape)):
        # an element outside the declared bounds: Fortran reads whatever
        # lies at that column-major offset of the same allocation
        off, stride = 0, 1
        for c, n in zip(cidx, arr.shape):
            off += c * stride
            stride *= n
        if not arr.flags.f_contiguous:
            raise IndexError("out-of-bounds read of a non-contiguous array")
        if not 0 <= off < arr.size:
            # past the allocation itself Fortran reads whatever memory
            # follows.  On the evolution path the only such reads are the
            # finebound history terms of strips deeper than the stored
            # history (m or n > ghost-1, which needs tp == tl): their time
            # weights (tl - tp)(...) are exactly zero, so any finite value
            # gives the reference's result.  0.0 stands in; the reads are
            # counted so that a fixture records them.
            OOB_BEYOND[0] += 1
            return 0.0
        return np.ndarray.ravel(arr, order="F")[off]
    v = np.ndarray.__getitem__(arr, cidx)
    if isinstance(v, np.ndarray):
        return v.view(np.ndarray)
    return v


def fset(arr, idx, val):
    np.ndarray.__setitem__(arr, _conv(arr, idx), val)


def ipow(x, n):
    if isinstance(x, (int, np.integer)) and not isinstance(x, bool):
        return int(x) ** n
    if n == 0:
        return x * 0 + 1
    if n < 0:
        return 1.0 / ipow(x, -n)
    bits = bin(n)[3:]
    r = x
    for b in bits:
        r = r * r
        if b == "1":
            r = r * x
    return r


def fpow(a, b):
    if isinstance(b, (int, np.integer)) and not isinstance(b, bool):
        return ipow(a, int(b))
    if isinstance(b, np.ndarray):
        return np.power(a, b)
    bb = F64(b) if not isinstance(b, np.float32) else b
    if isinstance(a, np.ndarray):
        return np.power(a, bb)
    return F64(math.pow(float(a), float(bb))) if not isinstance(a, np.float32) else np.power(a, bb)


def fdiv(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)) \
            and not isinstance(a, bool) and not isinstance(b, bool):
        q = abs(int(a)) // abs(int(b))
        return q if (a >= 0) == (b >= 0) else -q
    return a / b


def fmod(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        return int(a) - fdiv(int(a), int(b)) * int(b)
    return math.fmod(a, b)


def fnint(x):
    x = float(x)
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def fint(x):
    return int(float(x))


def fsign(a, b):
    if isinstance(a, (int, np.integer)):
        return abs(int(a)) if b >= 0 else -abs(int(a))
    return abs(a) if b >= 0 else -abs(a)


def fstreq(a, b):
    return str(a).rstrip() == str(b).rstrip()


def fcontains(string, pattern):
    items = [s for s in re.split(r"[,\s]+", str(string).strip()) if s]
    return str(pattern).strip() in items


def fmerge(a, b, m):
    if isinstance(m, np.ndarray):
        return np.where(m, a, b)
    return a if m else b


def fsqrt(x):
    if isinstance(x, np.ndarray):
        return np.sqrt(x)
    return np.sqrt(x)


INTRINSICS = {
    "exp": "np.exp", "dexp": "np.exp", "log": "np.log", "dlog": "np.log",
    "sqrt": "_h.fsqrt", "dsqrt": "_h.fsqrt", "abs": "np.abs", "dabs": "np.abs",
    "sin": "np.sin", "cos": "np.cos", "tan": "np.tan", "atan": "np.arctan",
    "acos": "np.arccos", "asin": "np.arcsin", "tanh": "np.tanh",
    "dble": "_h.F64", "real": "_h.F64", "float": "_h.F64",
    "nint": "_h.fnint", "int": "_h.fint", "mod": "_h.fmod", "sign": "_h.fsign",
    "min": "_h.fmin", "max": "_h.fmax", "merge": "_h.fmerge",
    "trim": "_h.ftrim", "index": "_h.findex", "len": "len",
    "maxval": "np.max", "minval": "np.min", "associated": "_h.fassociated",
}


def fassociated(x):
    return x is not None


def fmin(*a):
    if any(isinstance(x, np.ndarray) for x in a):
        r = a[0]
        for x in a[1:]:
            r = np.minimum(r, x)
        return r
    return min(a)


def fmax(*a):
    if any(isinstance(x, np.ndarray) for x in a):
        r = a[0]
        for x in a[1:]:
            r = np.maximum(r, x)
        return r
    return max(a)


def ftrim(s):
    return str(s).rstrip()


def findex(s, p):
    return str(s).find(str(p)) + 1


class FortranStop(RuntimeError):
    pass


# ----------------------------------------------------------------------------
# source preprocessing
# ----------------------------------------------------------------------------

def _strip_comment(line):
    out = []
    q = None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        else:
            if ch == "!":
                break
            if ch in "'\"":
                q = ch
            out.append(ch)
    return "".join(out)


def _lower_outside_strings(line):
    out = []
    q = None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        else:
            if ch in "'\"":
                q = ch
                out.append(ch)
            else:
                out.append(ch.lower())
    return "".join(out)


def logical_lines(text, include_dir=None):
    """Comment-free, continuation-joined, lower-cased statements."""
    raw = text.split("\n")
    stmts = []
    cur = ""
    for line in raw:
        s = _strip_comment(line).rstrip()
        if not s.strip():
            if cur:
                continue
            continue
        t = s.strip()
        if cur:
            if t.startswith("&"):
                t = t[1:]
            cur += t
        else:
            cur = t
        if cur.endswith("&"):
            cur = cur[:-1]
            continue
        stmt = _lower_outside_strings(cur.strip())
        cur = ""
        m = re.match(r"include\s+'([^']+)'", stmt)
        if m and include_dir is not None:
            import os
            path = os.path.join(include_dir, os.path.basename(m.group(1)))
            with open(path) as f:
                stmts.extend(logical_lines(f.read(), include_dir))
            continue
        # split on ';' outside strings
        parts, q, buf = [], None, ""
        for ch in stmt:
            if q:
                buf += ch
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                buf += ch
            elif ch == ";":
                parts.append(buf)
                buf = ""
            else:
                buf += ch
        parts.append(buf)
        stmts.extend(p.strip() for p in parts if p.strip())
    return stmts


# ----------------------------------------------------------------------------
# expression lexer / parser -> python source
# ----------------------------------------------------------------------------

_TOK = re.compile(r"""
  (?P<ws>\s+)
 |(?P<str>'[^']*'|"[^"]*")
 |(?P<dotop>\.(?:and|or|not|eqv|neqv|true|false|eq|ne|lt|le|gt|ge)\.)
 |(?P<real>(?:\d+\.(?!(?:and|or|not|eq|ne|lt|le|gt|ge|eqv|neqv)\.)\d*|\.\d+)(?:[ed][+-]?\d+)?|\d+[ed][+-]?\d+)
 |(?P<int>\d+)
 |(?P<name>[a-z_][a-z0-9_]*)
 |(?P<op>\*\*|==|/=|<=|>=|=>|//|[-+*/(),:%<>=])
""", re.X)


def lex(s):
    toks = []
    pos = 0
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise SyntaxError("cannot lex %r at %d" % (s, pos))
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        toks.append((kind, m.group(kind)))
    toks.append(("eof", None))
    return toks


class ExprParser:
    def __init__(self, unit, toks):
        self.u = unit
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise SyntaxError("expected %r got %r" % (val, tok))
        self.i += 1
        return tok

    def at(self, val):
        return self.t[self.i][1] == val

    # grammar -------------------------------------------------------------
    def expr(self):
        return self.or_()

    def or_(self):
        a = self.and_()
        while self.at(".or."):
            self.take()
            b = self.and_()
            a = "(%s or %s)" % (a, b)
        return a

    def and_(self):
        a = self.not_()
        while self.at(".and."):
            self.take()
            b = self.not_()
            a = "(%s and %s)" % (a, b)
        return a

    def not_(self):
        if self.at(".not."):
            self.take()
            return "(not %s)" % self.not_()
        return self.cmp()

    _CMP = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=",
            ".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def cmp(self):
        a = self.concat()
        tok = self.peek()[1]
        if tok in self._CMP:
            self.take()
            b = self.concat()
            op = self._CMP[tok]
            if op in ("==", "!="):
                return "(%s_h.fstreq(%s, %s))" % ("" if op == "==" else "not ", a, b) \
                    if ("'" in a or '"' in a or "'" in b or '"' in b) else "(%s %s %s)" % (a, op, b)
            return "(%s %s %s)" % (a, op, b)
        return a

    def concat(self):
        a = self.add()
        while self.at("//"):
            self.take()
            b = self.add()
            a = "(str(%s).rstrip() + str(%s))" % (a, b)
        return a

    def add(self):
        sign = None
        if self.at("-") or self.at("+"):
            sign = self.take()[1]
        a = self.mul()
        if sign == "-":
            a = "(-%s)" % a
        while self.at("+") or self.at("-"):
            op = self.take()[1]
            b = self.mul()
            a = "(%s %s %s)" % (a, op, b)
        return a

    def mul(self):
        a = self.power()
        while self.at("*") or self.at("/"):
            op = self.take()[1]
            b = self.power()
            if op == "*":
                a = "(%s * %s)" % (a, b)
            else:
                a = "_h.fdiv(%s, %s)" % (a, b)
        return a

    def power(self):
        a = self.unary_primary()
        if self.at("**"):
            self.take()
            b = self.power_rhs()
            return "_h.fpow(%s, %s)" % (a, b)
        return a

    def power_rhs(self):
        # exponent may carry a sign: x**(-2) is written with parens in practice
        if self.at("-") or self.at("+"):
            s = self.take()[1]
            b = self.power()
            return "(%s%s)" % (s, b)
        return self.power()

    def unary_primary(self):
        # gfortran extension: a * -b
        if self.at("-") or self.at("+"):
            s = self.take()[1]
            p = self.power()
            return "(%s%s)" % (s, p)
        return self.primary()

    def primary(self):
        kind, val = self.peek()
        if kind == "real":
            self.take()
            v = val
            if "d" in v:
                return "_h.F64(%r)" % float(v.replace("d", "e"))
            return "_h.F32(%r)" % float(v)
        if kind == "int":
            self.take()
            return val
        if kind == "str":
            self.take()
            return repr(val[1:-1])
        if kind == "dotop":
            self.take()
            if val == ".true.":
                return "True"
            if val == ".false.":
                return "False"
            raise SyntaxError(val)
        if val == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return "(%s)" % e
        if kind == "name":
            return self.designator()
        raise SyntaxError("unexpected %r" % (self.peek(),))

    def arglist(self):
        args = []
        self.take("(")
        if self.at(")"):
            self.take()
            return args
        while True:
            args.append(self.section())
            if self.at(","):
                self.take()
                continue
            self.take(")")
            return args

    def section(self):
        # a, a:b, :, a:, :b  (keyword args not used)
        if self.at(":"):
            self.take()
            if self.at(",") or self.at(")"):
                return ("slice", None, None)
            hi = self.expr()
            return ("slice", None, hi)
        lo = self.expr()
        if self.at(":"):
            self.take()
            if self.at(",") or self.at(")"):
                return ("slice", lo, None)
            hi = self.expr()
            return ("slice", lo, hi)
        return ("ix", lo)

    def designator(self):
        name = self.take()[1]
        base = self.u.ref(name)
        if self.at("(") :
            args = self.arglist()
            if self.u.is_callable(name):
                return self.u.call_expr(name, args)
            base = "_h.fget(%s, %s)" % (base, self.idx(args))
        while self.at("%"):
            self.take()
            comp = pyname(self.take()[1])
            base = "%s.%s" % (base, comp)
            if self.at("("):
                args = self.arglist()
                base = "_h.fget(%s, %s)" % (base, self.idx(args))
        return base

    @staticmethod
    def idx(args):
        parts = []
        for a in args:
            if a[0] == "ix":
                parts.append(a[1])
            else:
                parts.append("slice(%s, %s)" % (a[1] if a[1] is not None else "None",
                                                 a[2] if a[2] is not None else "None"))
        return "(" + ", ".join(parts) + ",)"


# ----------------------------------------------------------------------------
# program units
# ----------------------------------------------------------------------------

class Unit:
    """One subroutine or function, translated to a Python function."""

    def __init__(self, kind, name, args, stmts, functions, rettype=None):
        self.kind = kind
        self.name = name
        self.args = args
        self.stmts = stmts
        self.functions = functions
        self.locals = {}      # name -> (type, dims or None)
        self.rettype = rettype
        self.save_vars = set()
        self.data_init = {}

    # name handling --------------------------------------------------------
    def ref(self, name):
        if name in self.locals or name in self.args or (self.kind == "function" and name == self.name):
            return "L_" + name
        return "M." + pyname(name)

    def is_callable(self, name):
        if name in self.locals and self.locals[name][1] is not None:
            return False
        if self.kind == "function" and name == self.name:
            return False
        if name in self.locals and self.locals[name][0] == "logical" and name == "contains":
            return True
        if name in INTRINSICS or name in self.functions or name == "contains":
            if name in self.locals and self.locals[name][1] is not None:
                return False
            return True
        return False

    def call_expr(self, name, args):
        vals = []
        for a in args:
            if a[0] != "ix":
                raise SyntaxError("section passed to function %s" % name)
            vals.append(a[1])
        if name == "contains":
            return "_h.fcontains(%s)" % ", ".join(vals)
        if name in self.functions:
            return "F.%s(%s)" % (name, ", ".join(vals))
        return "%s(%s)" % (INTRINSICS[name], ", ".join(vals))

    def parse_expr(self, s):
        p = ExprParser(self, lex(s))
        e = p.expr()
        if p.peek()[0] != "eof":
            raise SyntaxError("trailing tokens in %r" % s)
        return e

    # declarations ---------------------------------------------------------
    _DECL = re.compile(r"^(integer|real\s*\(\s*8\s*\)|real|logical|character\s*(?:\(\s*(?:len\s*=\s*)?[^)]*\))?|double\s+precision)(?=[\s,(:])\s*(.*)$")

    def try_decl(self, st):
        m = self._DECL.match(st)
        if not m:
            return False
        # exclude assignment statements that start with a type-like name
        rest = m.group(2)
        if st.startswith("real") and re.match(r"^real\s*\(\s*8\s*\)\s*function", st):
            return False
        if re.match(r"^(integer|real|logical)\s*=", st):
            return False
        typ = m.group(1).replace(" ", "")
        typ = "real8" if typ.startswith("real(8)") or typ.startswith("doubleprecision") else \
            ("real4" if typ.startswith("real") else ("char" if typ.startswith("character") else typ))
        dims = None
        if rest.startswith(","):
            mm = re.match(r"^,\s*dimension\s*(\(.*?\))\s*::\s*(.*)$", rest)
            if mm:
                dims = mm.group(1)
                rest = mm.group(2)
            else:
                rest = rest.split("::", 1)[1]
        elif "::" in rest:
            rest = rest.split("::", 1)[1]
        for item in _split_top(rest):
            item = item.strip()
            mm = re.match(r"^([a-z_][a-z0-9_]*)\s*(\(.*\))?\s*(?:=\s*(.*))?$", item)
            if not mm:
                raise SyntaxError("bad declaration %r" % st)
            nm = mm.group(1)
            d = mm.group(2) or dims
            self.locals[nm] = (typ, d)
            if mm.group(3):
                self.data_init[nm] = mm.group(3)
        return True

    # translation ----------------------------------------------------------
    def translate(self):
        body = []
        ind = ["    "]
        stack = []

        def emit(line):
            body.append(ind[0] + line)

        # declarations first
        exec_stmts = []
        for st in self.stmts:
            if st.startswith("use ") or st == "implicit none" or st.startswith("save") \
                    or st.startswith("external"):
                if st.startswith("save"):
                    self.save_vars |= {v.strip() for v in st[4:].split(",") if v.strip()}
                continue
            if st.startswith("data "):
                mm = re.match(r"data\s+(\w+)\s*/\s*(.*?)\s*/", st)
                self.data_init[mm.group(1)] = mm.group(2)
                self.save_vars.add(mm.group(1))
                continue
            if self.try_decl(st):
                continue
            exec_stmts.append(st)
        # allocate local arrays / init
        for nm, (typ, d) in self.locals.items():
            if nm in self.args:
                continue
            if nm in self.save_vars:
                continue
            if d is not None:
                lbs, ubs = _dims(self, d)
                emit("L_%s = _h.falloc((%s,), (%s,))" % (nm, ", ".join(lbs), ", ".join(ubs)))
            else:
                init = {"real8": "_h.F64(0.0)", "real4": "_h.F32(0.0)", "integer": "0",
                        "logical": "False", "char": "''"}.get(typ, "None")
                emit("L_%s = %s" % (nm, init))
        for nm in sorted(self.save_vars):
            init = self.data_init.get(nm)
            val = self.parse_expr(init) if init else "None"
            emit("L_%s = _S.setdefault(%r, %s)" % (nm, nm, val))
        # cast real(8) scalar arguments
        for a in self.args:
            if a in self.locals and self.locals[a][0] == "real8" and self.locals[a][1] is None:
                emit("L_%s = _h.F64(L_%s) if not isinstance(L_%s, _h.np.ndarray) else L_%s" % (a, a, a, a))
        label_stack = []
        for st in exec_stmts:
            self._stmt(st, emit, ind, stack)
        while stack and isinstance(stack[-1], tuple) and stack[-1][0] == "label":
            emit("break")
            ind[0] = ind[0][:-4]
            stack.pop()
        if self.kind == "function":
            for nm in sorted(self.save_vars):
                emit("_S[%r] = L_%s" % (nm, nm))
            emit("return L_%s" % self.name)
        else:
            for nm in sorted(self.save_vars):
                emit("_S[%r] = L_%s" % (nm, nm))
        params = ", ".join("L_" + a for a in self.args)
        src = "def %s(%s):\n    _S = _SAVE.setdefault(%r, {})\n" % (self.name, params, self.name)
        if self.kind == "function" and self.name not in self.locals:
            src += "    L_%s = None\n" % self.name
        src += "\n".join(body) + "\n    pass\n"
        return src

    def _assign_code(self, lhs, rhs):
        """lhs: designator text; rhs: python expression."""
        m = re.match(r"^([a-z_][a-z0-9_]*)\s*(.*)$", lhs)
        name, rest = m.group(1), m.group(2).strip()
        base = self.ref(name)
        if rest == "":
            if base.startswith("L_"):
                typ = self.locals.get(name, (None, None))
                if typ[1] is not None or (self.kind == "function" and name == self.name and
                                          self.locals.get(name, (None, None))[1] is not None):
                    return "%s[...] = %s" % (base, rhs)
                if typ[0] == "real8":
                    return "%s = _h.F64(%s)" % (base, rhs)
                if typ[0] == "integer":
                    return "%s = int(%s)" % (base, rhs)
                return "%s = %s" % (base, rhs)
            return "_assign(M, %r, %s)" % (pyname(name), rhs)
        # indexed / component assignment
        p = ExprParser(self, lex(rest))
        chain = base
        pieces = []
        while p.peek()[0] != "eof":
            if p.at("("):
                args = p.arglist()
                pieces.append(("idx", ExprParser.idx(args)))
            elif p.at("%"):
                p.take()
                pieces.append(("comp", pyname(p.take()[1])))
            else:
                raise SyntaxError("bad lhs %r" % lhs)
        for kind, v in pieces[:-1]:
            chain = "_h.fget(%s, %s)" % (chain, v) if kind == "idx" else "%s.%s" % (chain, v)
        kind, v = pieces[-1]
        if kind == "idx":
            return "_h.fset(%s, %s, %s)" % (chain, v, rhs)
        return "_assign(%s, %r, %s)" % (chain, v, rhs)

    def _stmt(self, st, emit, ind, stack):
        def push():
            ind[0] += "    "
            emit("pass")

        def pop():
            ind[0] = ind[0][:-4]

        if st.startswith("if") and re.match(r"^if\s*\(", st):
            cond, rest = _paren_split(st[2:].strip())
            c = self.parse_expr(cond)
            rest = rest.strip()
            if rest == "then":
                emit("if %s:" % c)
                push()
                stack.append("if")
                return
            emit("if %s:" % c)
            push()
            self._stmt(rest, emit, ind, stack)
            pop()
            return
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", st)
        if m:
            cond, _ = _paren_split(st[st.index("("):])
            pop()
            emit("elif %s:" % self.parse_expr(cond))
            push()
            return
        if st == "else":
            pop()
            emit("else:")
            push()
            return
        if re.match(r"^end\s*if$", st):
            pop()
            stack.pop()
            return
        m = re.match(r"^do\s+while\s*(\(.*\))$", st)
        if m:
            cond, _ = _paren_split(m.group(1))
            emit("while %s:" % self.parse_expr(cond))
            push()
            stack.append("while")
            return
        # "NNN continue" that a later "goto NNN" jumps back to: the rest of
        # the routine becomes the body of a loop that the goto restarts
        m = re.match(r"^(\d+)\s+continue$", st)
        if m:
            emit("while True:")
            push()
            stack.append(("label", m.group(1)))
            return
        m = re.match(r"^go\s*to\s+(\d+)$", st)
        if m:
            open_loops = [e for e in stack if e == "while" or (isinstance(e, tuple) and e[0] in ("do", "label"))]
            if not open_loops or open_loops[-1] != ("label", m.group(1)):
                raise SyntaxError("only a backward goto to an enclosing 'NNN continue' is supported")
            emit("continue")
            return
        m = re.match(r"^do\s+([a-z_]\w*)\s*=\s*(.*)$", st)
        if m:
            var = m.group(1)
            parts = _split_top(m.group(2))
            lo, hi = self.parse_expr(parts[0]), self.parse_expr(parts[1])
            step = self.parse_expr(parts[2]) if len(parts) > 2 else "1"
            v = self.ref(var)
            emit("for %s in _h_range(%s, %s, %s):" % (v, lo, hi, step))
            push()
            stack.append(("do", v, hi, step, lo))
            return
        if re.match(r"^end\s*do$", st):
            pop()
            top = stack.pop()
            if isinstance(top, tuple) and top[0] == "do":
                # a loop that ends normally leaves its variable one step past
                # the last iteration (the first value for an empty loop), as
                # Fortran does; an ``exit`` keeps the current value
                _, v, hi, step, lo = top
                emit("else:")
                push()
                emit("%s = _h_last(%s, %s, %s)" % (v, lo, hi, step))
                pop()
            return
        m = re.match(r"^select\s+case\s*\((.*)\)$", st)
        if m:
            emit("_sel = %s" % self.parse_expr(m.group(1)))
            emit("if False:")
            push()
            emit("pass")
            pop()
            stack.append("select")
            return
        m = re.match(r"^case\s*\((.*)\)$", st)
        if m:
            if stack[-1] == "select_in":
                pop()
            vals = [self.parse_expr(x) for x in _split_top(m.group(1))]
            emit("elif _sel in (%s,):" % ", ".join(vals))
            push()
            stack[-1] = "select_in"
            return
        if st == "case default":
            if stack[-1] == "select_in":
                pop()
            emit("else:")
            push()
            stack[-1] = "select_in"
            return
        if re.match(r"^end\s*select$", st):
            if stack[-1] == "select_in":
                pop()
            stack.pop()
            return
        if st == "cycle":
            emit("continue")
            return
        if st == "exit":
            emit("break")
            return
        if st == "return":
            if self.kind == "function":
                for nm in sorted(self.save_vars):
                    emit("_S[%r] = L_%s" % (nm, nm))
                emit("return L_%s" % self.name)
            else:
                for nm in sorted(self.save_vars):
                    emit("_S[%r] = L_%s" % (nm, nm))
                emit("return")
            return
        if st.startswith("print") or st.startswith("write") or st.startswith("open") \
                or st.startswith("close") or st.startswith("flush"):
            return
        if st.startswith("stop"):
            emit("raise _h.FortranStop(%r)" % st)
            return
        m = re.match(r"^call\s+([a-z_]\w*)\s*(\(.*\))?$", st)
        if m:
            nm = m.group(1)
            args = []
            if m.group(2):
                inner, _ = _paren_split(m.group(2))
                args = [self.parse_expr(a) for a in _split_top(inner)] if inner.strip() else []
            if nm == "die":
                emit("raise _h.FortranStop('die')")
                return
            if nm == "mpi_allreduce":
                # serial run: the reduction of one rank's value is that value
                raw = _split_top(_paren_split(m.group(2))[0])
                emit(self._assign_code(raw[1].strip(), args[0]))
                return
            emit("F.%s(%s)" % (nm, ", ".join(args)))
            return
        # pointer assignment
        m = re.match(r"^(.*?)\s*=>\s*(.*)$", st)
        if m and "==" not in st:
            lhs, rhs = m.group(1), m.group(2)
            rhs_e = self.parse_expr(rhs)
            mm = re.match(r"^([a-z_]\w*)$", lhs.strip())
            if mm:
                emit("_ptr(M, %r, %s)" % (pyname(mm.group(1)), rhs_e))
            else:
                emit(self._assign_code(lhs.strip(), rhs_e))
            return
        # assignment: find top-level '='
        k = _find_assign(st)
        if k is not None:
            lhs = st[:k].strip()
            rhs = st[k + 1:].strip()
            emit(self._assign_code(lhs, self.parse_expr(rhs)))
            return
        raise SyntaxError("unhandled statement in %s: %r" % (self.name, st))


def _paren_split(s):
    """'(a(b)c) rest' -> ('a(b)c', ' rest')"""
    assert s[0] == "("
    depth = 0
    q = None
    for k, ch in enumerate(s):
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
                return s[1:k], s[k + 1:]
    raise SyntaxError("unbalanced %r" % s)


def _split_top(s):
    out, depth, q, buf = [], 0, None, ""
    for ch in s:
        if q:
            buf += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "," and depth == 0:
            out.append(buf)
            buf = ""
            continue
        buf += ch
    if buf.strip():
        out.append(buf)
    return out


def _find_assign(st):
    depth, q = 0, None
    for k, ch in enumerate(st):
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
            prev = st[k - 1] if k else ""
            nxt = st[k + 1] if k + 1 < len(st) else ""
            if nxt in "=>" or prev in "=/<>":
                continue
            return k
    return None


def _dims(unit, d):
    inner, _ = _paren_split(d)
    lbs, ubs = [], []
    for part in _split_top(inner):
        if ":" in part:
            lo, hi = part.split(":", 1)
        else:
            lo, hi = "1", part
        lbs.append("int(%s)" % unit.parse_expr(lo))
        ubs.append("int(%s)" % unit.parse_expr(hi))
    return lbs, ubs


_HEAD = re.compile(r"^(?:recursive\s+)?(?:(?:real\s*\(\s*8\s*\)|logical|integer)\s+)?(subroutine|function)\s+([a-z_]\w*)\s*(?:\((.*)\))?\s*$")


def parse_units(stmts, functions):
    units = []
    cur = None
    for st in stmts:
        if cur is None:
            if st.startswith("module ") or st == "contains" or re.match(r"^end\s*module", st):
                continue
            m = _HEAD.match(st)
            if m:
                args = [a.strip() for a in (m.group(3) or "").split(",") if a.strip()]
                cur = (m.group(1), m.group(2), args, [])
                continue
            continue
        if re.match(r"^end\s*(subroutine|function)\b", st) or st == "end":
            kind, name, args, body = cur
            units.append(Unit(kind, name, args, body, functions))
            cur = None
            continue
        cur[3].append(st)
    return units


def _h_range(lo, hi, step):
    return range(int(lo), int(hi) + (1 if step > 0 else -1), int(step))


def _h_last(lo, hi, step):
    lo, hi, step = int(lo), int(hi), int(step)
    return lo + max(0, (hi - lo + step) // step) * step


def _assign(obj, name, val):
    cur = getattr(obj, name, None)
    if isinstance(cur, np.ndarray):
        cur[...] = val
    else:
        tp = getattr(obj, "_types", {}).get(name) if hasattr(obj, "_types") else None
        if tp == "real8":
            val = F64(val)
        elif tp == "integer":
            val = int(val)
        setattr(obj, name, val)


def _ptr(obj, name, target):
    setattr(obj, name, target)


class Program:
    """A set of translated units sharing one module namespace ``M``."""

    def __init__(self, module_ns, include_dir=None):
        self.M = module_ns
        self.include_dir = include_dir
        self.sources = {}
        self.F = type("F", (), {})()
        self.save = {}

    def load(self, texts, names_filter=None, extra_functions=()):
        stmts_all = []
        for t in texts:
            stmts_all.append(logical_lines(t, self.include_dir))
        funcs = set(extra_functions)
        for stmts in stmts_all:
            for st in stmts:
                m = _HEAD.match(st)
                if m and m.group(1) == "function":
                    funcs.add(m.group(2))
        for stmts in stmts_all:
            for u in parse_units(stmts, funcs):
                if names_filter and u.name not in names_filter:
                    continue
                src = u.translate()
                self.sources[u.name] = src
                g = {"_h": _helpers, "np": np, "M": self.M, "F": self.F, "_SAVE": self.save,
                     "_assign": _assign, "_ptr": _ptr, "_h_range": _h_range, "_h_last": _h_last}
                try:
                    exec(compile(src, "<ftn:%s>" % u.name, "exec"), g)
                except SyntaxError:
                    print(src)
                    raise
                setattr(self.F, u.name, g[u.name])

    def define(self, name, fn):
        setattr(self.F, name, fn)


import sys as _sys  # noqa: E402
_helpers = _sys.modules[__name__]
