"""Execute the reference's Fortran source (a small language subset) in Python.

Test infrastructure for the golden fixtures: there is no Fortran compiler in
this image, so this module transpiles the statements ``3D/QMS_3D.f90`` uses
(declarations, allocate, do / if / cycle / stop, list-directed and stream
reads, unformatted sequential writes, scalar and array-section assignments,
the intrinsics mod/max/int/maxval/minval/real/trim) into a Python function and
runs it.  The external ``pardiso`` call is routed to a hook supplied by the
caller (a direct solver), which also lets the caller capture every CSR matrix
and right-hand side the program hands to the solver.

Floating-point semantics follow the Fortran source: real literals without a
kind suffix are default (single precision) reals, ``_dp`` literals are double,
integer/integer division truncates, mixed operands promote to the wider kind,
and expressions are evaluated in source order with Fortran operator
precedence (unary minus binds looser than * and /).  ``x**2`` is evaluated as
``x*x``.  Uninitialised variables start at zero, like the static storage of a
main program.
"""
from __future__ import annotations

import math
import re

import numpy as np

F32 = np.float32
F64 = np.float64


class FortranStop(Exception):
    pass


# --------------------------------------------------------------------------
# source normalisation
# --------------------------------------------------------------------------
def _strip_comment(line: str) -> str:
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
    return "".join(out).rstrip()


def _lower_outside_strings(s: str) -> str:
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


def logical_lines(src: str):
    lines, buf = [], ""
    for raw in src.splitlines():
        s = _strip_comment(raw).strip()
        if not s:
            continue
        if s.startswith("&"):
            s = s[1:].strip()
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        buf += s
        for part in _split_top(_lower_outside_strings(buf.strip()), ";"):
            if part:
                lines.append(part)
        buf = ""
    return lines


# --------------------------------------------------------------------------
# expressions
# --------------------------------------------------------------------------
_TOK = re.compile(r"""
    (?P<str>'[^']*'|"[^"]*")
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?(_dp|_8)?)
  | (?P<dotop>\.(or|and|not|eq|ne|lt|le|gt|ge)\.)
  | (?P<id>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|==|/=|<=|>=|[-+*/()<>,:])
  | (?P<ws>\s+)
""", re.X)


def tokenize(s):
    pos, out = 0, []
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[pos:pos + 20]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        out.append((kind, m.group(kind)))
    return out


INTRINSICS = {"mod", "max", "min", "int", "maxval", "minval", "real", "trim", "abs", "sqrt",
              "selected_real_kind"}


class ExprCompiler:
    """Recursive-descent translation of one Fortran expression to Python source."""

    def __init__(self, arrays, lbounds, funcs):
        self.arrays = arrays      # name -> rank
        self.lbounds = lbounds    # name -> tuple of lower bounds (static)
        self.funcs = funcs        # user functions

    def compile(self, s):
        self.toks = tokenize(s)
        self.i = 0
        r = self.level_or()
        if self.i != len(self.toks):
            raise SyntaxError(f"trailing tokens in {s!r}: {self.toks[self.i:]}")
        return r

    def peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else (None, None)

    def take(self, val=None):
        t = self.toks[self.i]
        if val is not None and t[1] != val:
            raise SyntaxError(f"expected {val}, got {t}")
        self.i += 1
        return t

    def level_or(self):
        left = self.level_and()
        while self.peek()[1] == ".or.":
            self.take()
            left = f"({left} or {self.level_and()})"
        return left

    def level_and(self):
        left = self.level_not()
        while self.peek()[1] == ".and.":
            self.take()
            left = f"({left} and {self.level_not()})"
        return left

    def level_not(self):
        if self.peek()[1] == ".not.":
            self.take()
            return f"(not {self.level_not()})"
        return self.level_rel()

    def level_rel(self):
        left = self.level_add()
        ops = {"==": "==", "/=": "!=", "<": "<", ">": ">", "<=": "<=", ">=": ">=",
               ".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}
        t = self.peek()[1]
        if t in ops:
            self.take()
            right = self.level_add()
            return f"({left} {ops[t]} {right})"
        return left

    def level_add(self):
        t = self.peek()[1]
        if t in ("+", "-"):
            self.take()
            term = self.level_mul()
            left = f"(-{term})" if t == "-" else term
        else:
            left = self.level_mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            right = self.level_mul()
            left = f"({left} {op} {right})"
        return left

    def level_mul(self):
        left = self.level_pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            right = self.level_pow()
            left = f"({left} * {right})" if op == "*" else f"_div({left}, {right})"
        return left

    def level_pow(self):
        base = self.primary()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):
                raise SyntaxError("signed exponent")
            exp = self.level_pow()
            if exp == "2":
                return f"_sq({base})"
            return f"_pow({base}, {exp})"
        return base

    def primary(self):
        kind, val = self.take()
        if kind == "num":
            return self.number(val)
        if kind == "str":
            return repr(val[1:-1])
        if val == "(":
            e = self.level_or()
            self.take(")")
            return f"({e})"
        if kind == "id":
            if self.peek()[1] == "(":
                self.take("(")
                args = self.arglist()
                self.take(")")
                return self.call_or_index(val, args)
            return val
        raise SyntaxError(f"unexpected token {val!r}")

    @staticmethod
    def number(val):
        if "_dp" in val or "_8" in val:
            v = val.replace("_dp", "").replace("_8", "").replace("d", "e")
            return f"F64({float(v)!r})"
        if any(c in val for c in ".e"):
            return f"F32({val!r})"
        if "d" in val:
            return f"F64({float(val.replace('d', 'e'))!r})"
        return str(int(val))

    def arglist(self):
        """Arguments, each either an expression or a section lo:hi / : ."""
        args = []
        if self.peek()[1] == ")":
            return args
        while True:
            if self.peek()[1] == ":":
                self.take()
                hi = None if self.peek()[1] in (",", ")") else self.level_or()
                args.append(("sec", None, hi))
            else:
                e = self.level_or()
                if self.peek()[1] == ":":
                    self.take()
                    hi = None if self.peek()[1] in (",", ")") else self.level_or()
                    args.append(("sec", e, hi))
                else:
                    args.append(("expr", e))
            if self.peek()[1] == ",":
                self.take()
                continue
            return args

    def call_or_index(self, name, args):
        if name in self.arrays:
            lbs = self.lbounds.get(name, (1,) * len(args))
            idx = []
            for d, a in enumerate(args):
                lb = lbs[d]
                if a[0] == "expr":
                    idx.append(f"({a[1]})-{lb}")
                else:
                    lo = "" if a[1] is None else f"({a[1]})-{lb}"
                    hi = "" if a[2] is None else f"({a[2]})-{lb}+1"
                    idx.append(f"{lo}:{hi}")
            return f"{name}[{', '.join(idx)}]"
        if name in INTRINSICS:
            return f"_{name}({', '.join(a[1] for a in args)})"
        if name in self.funcs:
            return f"{name}({', '.join(a[1] for a in args)})"
        raise NameError(f"unknown function or array {name!r}")


# --------------------------------------------------------------------------
# runtime helpers
# --------------------------------------------------------------------------
def _is_int(x):
    return isinstance(x, (int, np.integer)) and not isinstance(x, bool)


def _div(a, b):
    if _is_int(a) and _is_int(b):
        q = abs(int(a)) // abs(int(b))
        return q if (a >= 0) == (b >= 0) else -q
    return a / b


def _sq(x):
    return x * x


def _pow(a, b):
    return a ** b


def _mod(a, b):
    if _is_int(a) and _is_int(b):
        return int(math.fmod(int(a), int(b)))
    return np.fmod(a, b)


def _promote(*xs):
    if all(_is_int(x) for x in xs):
        return [int(x) for x in xs]
    if any(isinstance(x, (float, F64)) for x in xs):
        return [F64(x) for x in xs]
    return [F32(x) for x in xs]


def _max(*xs):
    ys = _promote(*xs)
    r = ys[0]
    for y in ys[1:]:
        if y > r:
            r = y
    return r


def _min(*xs):
    ys = _promote(*xs)
    r = ys[0]
    for y in ys[1:]:
        if y < r:
            r = y
    return r


def _int(x):
    if isinstance(x, np.ndarray):
        return np.trunc(x).astype(np.int64)
    return int(x)


def _maxval(a):
    return a.max()


def _minval(a):
    return a.min()


def _real(x):
    return F32(x)


def _trim(s):
    return s.rstrip()


def _abs(x):
    return abs(x)


def _sqrt(x):
    return np.sqrt(x)


def _selected_real_kind(*a):
    return 8


# --------------------------------------------------------------------------
# I/O layer
# --------------------------------------------------------------------------
class FortranIO:
    """Units, list-directed reads, stream reads, unformatted sequential writes."""

    def __init__(self, cwd, argv, pardiso_hook, echo=False):
        import os
        self.os = os
        self.cwd = cwd
        self.argv = argv
        self.units = {}
        self.pardiso_hook = pardiso_hook
        self.echo = echo
        self.stdout = []

    def path(self, name):
        return self.os.path.join(self.cwd, name.strip())

    def open(self, unit, file, form="formatted", access="sequential", status="unknown", action=None):
        if form == "unformatted" and access != "stream":
            self.units[unit] = {"kind": "seqw", "f": open(self.path(file), "wb")}
        elif access == "stream":
            self.units[unit] = {"kind": "stream", "f": open(self.path(file), "rb")}
        else:
            with open(self.path(file)) as fh:
                self.units[unit] = {"kind": "text", "lines": fh.read().splitlines(), "pos": 0}

    def close(self, unit):
        u = self.units.pop(unit)
        if "f" in u:
            u["f"].close()

    def read_list(self, unit, count):
        """List-directed read of `count` values starting at the next record."""
        u = self.units[unit]
        vals = []
        while len(vals) < count:
            if u["pos"] >= len(u["lines"]):
                raise EOFError("end of file in list-directed read")
            line = u["lines"][u["pos"]]
            u["pos"] += 1
            for tok in re.split(r"[,\s]+", line.strip()):
                if tok == "":
                    continue
                if tok.startswith("/"):
                    return vals + [None] * (count - len(vals))
                vals.append(tok.strip("'\""))
                if len(vals) == count:
                    break
        return vals

    def read_stream(self, unit, n):
        u = self.units[unit]
        data = u["f"].read(8 * n)
        if len(data) < 8 * n:
            raise EOFError("short stream read")
        return np.frombuffer(data, dtype="<f8").copy()

    def write_record(self, unit, arr):
        u = self.units[unit]
        data = np.asarray(arr, dtype="<f8").tobytes(order="F")
        m = np.array([len(data)], dtype="<i4").tobytes()
        u["f"].write(m + data + m)

    def say(self, *args):
        self.stdout.append(" ".join(str(a) for a in args))
        if self.echo:
            print(*args)


def _conv(kind, v):
    if v is None:
        return None
    if kind == "int":
        return int(v)
    if kind == "real":
        return F64(float(v.replace("d", "e").replace("D", "e")))
    return v


# --------------------------------------------------------------------------
# statement transpiler
# --------------------------------------------------------------------------
_DECL = re.compile(r"^(real|integer|character|logical)\b(\([^)]*\))?\s*(,\s*[a-z]+\s*)*::\s*(.*)$")


def _split_top(s, sep=","):
    """Split on `sep` outside parentheses and quotes."""
    out, depth, q, cur = [], 0, None, ""
    for ch in s:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == sep and depth == 0:
            out.append(cur)
            cur = ""
            continue
        cur += ch
    out.append(cur)
    return [x.strip() for x in out]


def _paren_span(s, start):
    depth = 0
    for k in range(start, len(s)):
        if s[k] == "(":
            depth += 1
        elif s[k] == ")":
            depth -= 1
            if depth == 0:
                return k
    raise SyntaxError(s)


class Transpiler:
    def __init__(self, src):
        self.lines = logical_lines(src)
        self.types = {}        # name -> 'int' | 'real' | 'char'
        self.arrays = {}       # name -> rank
        self.lbounds = {}
        self.params = {}
        self.funcs = set()
        self.dtypes = {}

    def scan(self):
        in_func = False
        for ln in self.lines:
            m = re.match(r"^function\s+([a-z_0-9]+)", ln)
            if m:
                self.funcs.add(m.group(1))
                in_func = True
            if ln.startswith("end function"):
                in_func = False
            if in_func:
                continue
            m = _DECL.match(ln)
            if not m:
                mm = re.match(r"^allocate\((.*)\)$", ln)
                if mm:
                    for item in _split_top(mm.group(1)):
                        nm = item[:item.index("(")].strip()
                        dims = _split_top(item[item.index("(") + 1:-1])
                        self.lbounds[nm] = tuple(int(d.split(":")[0]) if ":" in d and d.split(":")[0].strip().isdigit()
                                                 else 1 for d in dims)
                continue
            base, kind = m.group(1), m.group(2) or ""
            t = {"real": "real", "integer": "int", "character": "char", "logical": "int"}[base]
            for item in _split_top(m.group(4)):
                nm = re.match(r"[a-z_][a-z0-9_]*", item).group(0)
                self.types[nm] = t
                rest = item[len(nm):].strip()
                if rest.startswith("("):
                    end = _paren_span(rest, 0)
                    self.arrays[nm] = len(_split_top(rest[1:end]))
                    self.dtypes[nm] = np.float64 if t == "real" else np.int64
                    rest = rest[end + 1:].strip()
                if rest.startswith("="):
                    self.params[nm] = rest[1:].strip()

    def expr(self, s):
        return ExprCompiler(self.arrays, self.lbounds, self.funcs).compile(s)

    def target(self, s):
        return self.expr(s)

    def assign(self, lhs, rhs_code):
        nm = re.match(r"[a-z_][a-z0-9_]*", lhs).group(0)
        tcode = self.target(lhs)
        if nm in self.arrays:
            if lhs.strip() == nm:
                return f"{nm}[...] = {rhs_code}"
            return f"{tcode} = {rhs_code}"
        t = self.types.get(nm, "real")
        if t == "int":
            return f"{tcode} = _int({rhs_code})"
        if t == "real":
            return f"{tcode} = F64({rhs_code})"
        return f"{tcode} = {rhs_code}"

    def transpile(self):
        self.scan()
        out = ["def _main(_io):"]
        ind = 1
        P = lambda s: out.append("    " * ind + s)
        # zero-initialised scalars and parameters
        for nm, t in self.types.items():
            if nm in self.arrays:
                continue
            if nm in self.params:
                continue
            P(f"{nm} = " + ({"int": "0", "real": "F64(0.0)", "char": "''"}[t]))
        for nm, t in self.types.items():
            if nm in self.arrays and nm not in self.lbounds:
                pass
        # parameters in declaration order
        for nm, e in self.params.items():
            P(self.assign(nm, self.expr(e)))
        # fixed-size arrays (pt(64), iparm(64))
        for ln in self.lines:
            m = _DECL.match(ln)
            if not m or "allocatable" in ln:
                continue
            for item in _split_top(m.group(4)):
                nm = re.match(r"[a-z_][a-z0-9_]*", item).group(0)
                if nm in self.arrays:
                    dims = item[item.index("(") + 1:item.rindex(")")]
                    P(f"{nm} = np.zeros(({dims},), dtype=np.{np.dtype(self.dtypes[nm]).name}, order='F')")
        in_func = None
        func_lines = []
        for ln in self.lines:
            if ln.startswith("program ") or ln == "implicit none" or ln.startswith("end program") \
                    or ln == "contains" or _DECL.match(ln):
                continue
            m = re.match(r"^function\s+([a-z_0-9]+)\((.*)\)$", ln)
            if m:
                in_func = (m.group(1), [a.strip() for a in m.group(2).split(",")])
                func_lines = []
                continue
            if in_func:
                if ln.startswith("end function"):
                    self.emit_function(in_func, func_lines, out)
                    in_func = None
                else:
                    func_lines.append(ln)
                continue
            ind = self.statement(ln, P, ind, out)
        return "\n".join(out)

    def emit_function(self, sig, body, out):
        name, args = sig
        # the function is defined at module level before _main; hoist it
        code = [f"def {name}({', '.join(args)}):", f"    {name} = F64(0.0)"]
        ind = 0
        fn_out = []
        P = lambda s: fn_out.append("    " * ind + s)
        saved = dict(self.types)
        for a in args:
            self.types.setdefault(a, "real")
        for ln in body:
            if re.match(r"^(real|integer)(\([^)]*\))?\s+[a-z_][a-z0-9_]*$", ln):
                continue
            if _DECL.match(ln) or ln == "implicit none":
                m = _DECL.match(ln)
                if m:
                    base = m.group(1)
                    for item in _split_top(m.group(4)):
                        nm = re.match(r"[a-z_][a-z0-9_]*", item).group(0)
                        self.types[nm] = "int" if base == "integer" else "real"
                continue
            ind = self.statement(ln, P, ind, fn_out)
        self.types = saved
        code += ["    " + x for x in fn_out]
        code.append(f"    return {name}")
        out[0:0] = code

    def statement(self, ln, P, ind, out):
        if ln.startswith("do ") and "=" in ln:
            m = re.match(r"^do\s+([a-z_0-9]+)\s*=\s*(.*)$", ln)
            var = m.group(1)
            parts = _split_top(m.group(2))
            lo, hi = self.expr(parts[0]), self.expr(parts[1])
            P(f"for {var} in range(int({lo}), int({hi}) + 1):")
            return ind + 1
        if ln in ("end do", "enddo"):
            return ind - 1
        if ln.startswith("if") and ln.endswith("then") and ln[2:].lstrip().startswith("("):
            s = ln.index("(")
            e = _paren_span(ln, s)
            P(f"if {self.expr(ln[s:e + 1])}:")
            return ind + 1
        if ln.startswith("else if") or ln.startswith("elseif"):
            s = ln.index("(")
            e = _paren_span(ln, s)
            out.append("    " * (ind - 1) + f"elif {self.expr(ln[s:e + 1])}:")
            return ind
        if ln == "else":
            out.append("    " * (ind - 1) + "else:")
            return ind
        if ln in ("end if", "endif"):
            return ind - 1
        if ln == "cycle":
            P("continue")
            return ind
        if ln.startswith("stop"):
            msg = ln[4:].strip() or "''"
            P(f"raise FortranStop({msg})")
            return ind
        if ln.startswith("call "):
            self.call(ln[5:], P)
            return ind
        if ln.startswith("allocate("):
            for item in _split_top(ln[9:-1]):
                nm = item[:item.index("(")].strip()
                dims = _split_top(item[item.index("(") + 1:-1])
                shape = []
                for d in dims:
                    if ":" in d:
                        lo, hi = d.split(":", 1)
                        shape.append(f"({self.expr(hi)})-({self.expr(lo)})+1")
                    else:
                        shape.append(self.expr(d))
                dt = np.dtype(self.dtypes[nm]).name
                P(f"{nm} = np.zeros(({', '.join(shape)},), dtype=np.{dt}, order='F')")
            return ind
        if ln.startswith("deallocate("):
            return ind
        if ln.startswith("open("):
            args = _split_top(ln[5:-1])
            unit, kw = None, {}
            for a in args:
                if self._assign_split(a) is None:
                    unit = self.expr(a)
                    continue
                k, v = a.split("=", 1)
                if k.strip() == "unit":
                    unit = self.expr(v.strip())
                else:
                    kw[k.strip()] = self.expr(v.strip())
            kws = ", ".join(f"{k}={v}" for k, v in kw.items())
            P(f"_io.open({unit}, {kws})")
            return ind
        if ln.startswith("close("):
            P(f"_io.close({self.expr(ln[6:-1])})")
            return ind
        if ln.startswith("read("):
            e = _paren_span(ln, 4)
            ctl = _split_top(ln[5:e])
            targets = _split_top(ln[e + 1:].strip())
            unit = self.expr(ctl[0])
            if len(ctl) > 1 and ctl[1] == "*":
                P(f"_v = _io.read_list({unit}, {len(targets)})")
                for q, t in enumerate(targets):
                    nm = re.match(r"[a-z_][a-z0-9_]*", t).group(0)
                    P(f"{self.target(t)} = _conv({self.types.get(nm, 'real')!r}, _v[{q}])")
            else:
                (t,) = targets
                P(f"{t}[...] = _io.read_stream({unit}, {t}.size).reshape({t}.shape, order='F')")
            return ind
        if ln.startswith("write("):
            e = _paren_span(ln, 5)
            ctl = _split_top(ln[6:e])
            items = _split_top(ln[e + 1:].strip()) if ln[e + 1:].strip() else []
            if ctl[0] == "*":
                P(f"_io.say({', '.join(self.expr(x) for x in items)})")
            else:
                (item,) = items
                P(f"_io.write_record({self.expr(ctl[0])}, {self.expr(item)})")
            return ind
        # assignment
        eq = self._assign_split(ln)
        if eq is None:
            raise SyntaxError(f"unsupported statement: {ln}")
        lhs, rhs = ln[:eq].strip(), ln[eq + 1:].strip()
        P(self.assign(lhs, self.expr(rhs)))
        return ind

    @staticmethod
    def _assign_split(ln):
        depth, q = 0, None
        for k, ch in enumerate(ln):
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
            elif ch == "=" and depth == 0 and ln[k + 1:k + 2] != "=" and ln[k - 1:k] not in "<>/=":
                return k
        return None

    def call(self, s, P):
        name = s[:s.index("(")].strip() if "(" in s else s.strip()
        args = _split_top(s[s.index("(") + 1:s.rindex(")")]) if "(" in s else []
        if name == "system_clock":
            for a in args:
                P(f"{a} = 0")
        elif name == "get_command_argument":
            P(f"{args[1]} = _io.argv[{self.expr(args[0])}]")
        elif name == "pardiso":
            # pardiso(pt, maxfct, mnum, mtype, phase, n, a, ia, ja, perm, nrhs, iparm, msglvl, b, x, error)
            P(f"_io.pardiso_hook({args[4]}, {args[5]}, {args[6]}, {args[7]}, {args[8]}, {args[13]}, {args[14]})")
        else:
            raise SyntaxError(f"unsupported call {name}")


def run_program(src_path, cwd, argv, pardiso_hook, echo=False):
    src = open(src_path).read()
    tr = Transpiler(src)
    code = tr.transpile()
    ns = {"np": np, "F32": F32, "F64": F64, "FortranStop": FortranStop, "_conv": _conv}
    for k, v in list(globals().items()):
        if k.startswith("_") and callable(v) and k not in ("_conv",):
            ns[k] = v
    exec(compile(code, "<QMS_3D.f90>", "exec"), ns)
    io = FortranIO(cwd, argv, pardiso_hook, echo=echo)
    ns["_main"](io)
    return io
