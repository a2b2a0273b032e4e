"""Runs the reference's own Fortran subroutines here, through a translator for
the subset of free-form Fortran 90 its particle-side sources use.

TEST INFRASTRUCTURE ONLY.  It reads the reference's .F90 files at run time
(nothing of them is stored in this repository), translates every subroutine to
a Python function over one MPI rank's module state and runs it.  Fixtures made
this way pin the C restatement in oracle/ to the reference's statements instead
of to a second reading of them.

Semantics, as gfortran -O3 gives them on x86-64 without -march (no FMA, no
reassociation):
  * real*8 arithmetic is IEEE double, one rounding per operation, evaluated in
    the source's parse order (Python floats and numpy float64 element-wise
    operations do exactly this);
  * default-real literals (1.5, 2.08e-4) are single precision, rounded from the
    decimal; an operation between two default-real operands rounds to single,
    a mixed one promotes to double;
  * integer division truncates toward zero; mod takes the dividend's sign;
    assignment of a real to an integer truncates;
  * x**2 is x*x and x**3 is (x*x)*x (gfortran's expansion of small constant
    integer powers, each product rounded to the operand's precision); a real
    power calls pow();
  * a single-precision sqrt or exp is the double result rounded once to
    single (exact for sqrt; the reference's path takes none of the others in
    single precision);
  * sqrt, exp, log, log10, cos, sin and acos come from this host's C library
    (Python's math module), as the C restatement's do;
  * sum() adds in array element order from 0;
  * local variables start at zero (Fortran leaves them undefined);
  * subscripts are not checked unless the translator is built with
    check_bounds, which checks every subscript and section against its
    dimension's extent (numpy would otherwise take a negative index from the
    end without complaint);
  * MPI is one rank (MPI_SENDRECV to and from rank 0 copies the message into
    the receive buffer, MPI_REDUCE copies, barriers and broadcasts do nothing),
    or several ranks run as threads that share a World: messages go through
    mailboxes, reductions add in rank order at the root, every wait is
    bounded.
List-directed reads (read(unit,*)) take the next record of the file the unit
was opened on; list-directed writes to a file unit keep each record's values,
unformatted, under the file's name (nothing reaches the disk); writes to the
terminal and print statements do nothing.  A subroutine the sources call but do not define (PETSc) raises when
it is reached, unless the caller supplies it.
"""
import math
import os
import re
from fractions import Fraction

import numpy as np

# ----------------------------------------------------------------------------
# numbers


def f32(x):
    """Round a double to the nearest single-precision value."""
    return float(np.float32(x))


def _dec_to_f32(text):
    """A decimal literal rounded once, to nearest even, to single precision."""
    q = Fraction(text)
    c = np.float32(float(q))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        d = abs(Fraction(float(cand)) - q)
        if best is None or d < best[0] or (d == best[0] and int(np.float32(cand).view(np.int32)) % 2 == 0):
            best = (d, cand)
    return float(best[1])


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def _imod(a, b):
    return a - b * _idiv(a, b)


def _powi(x, n):
    if n == 2:
        return x * x
    if n == 3:
        return (x * x) * x
    if n == 1:
        return x
    if n == 0:
        return 1.0
    return math.pow(x, n)


def _powi4(x, n):
    """A single-precision value to a small integer power, every product rounded to single."""
    if n == 2:
        return f32(x * x)
    if n == 3:
        return f32(f32(x * x) * x)
    if n == 1:
        return x
    if n == 0:
        return 1.0
    return f32(math.pow(x, n))


def _fsum(a):
    s = 0.0
    for x in np.asarray(a).ravel(order="F"):
        s = s + float(x)
    return s


def _floor(x):
    return int(math.floor(x))


def _trunc(x):
    return int(x)


def _nint(x):
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


# ----------------------------------------------------------------------------
# arrays with Fortran bounds


class FArr:
    """A numpy array (Fortran element order) with its lower bounds o0, o1, ..."""
    __slots__ = ("a", "o0", "o1", "o2", "o3", "o4")

    def __init__(self, a, lbounds):
        self.a = a
        lb = list(lbounds) + [0] * (5 - len(lbounds))
        self.o0, self.o1, self.o2, self.o3, self.o4 = lb

    @staticmethod
    def alloc(dtype, bounds):
        shape = tuple(int(hi) - int(lo) + 1 for lo, hi in bounds)
        if any(s < 0 for s in shape):
            shape = tuple(max(s, 0) for s in shape)
        return FArr(np.zeros(shape, dtype=dtype, order="F"), [int(lo) for lo, _ in bounds])


def _ck(i, n):
    """A subscript checked against its dimension's extent."""
    if 0 <= i < n:
        return i
    raise IndexError(f"subscript {i} outside the extent {n} (counted from 0)")


def _cks(lo, hi, n):
    """A section lo:hi checked against its dimension's extent (empty sections pass)."""
    lo = 0 if lo is None else lo
    hi = n if hi is None else hi
    if hi > lo and (lo < 0 or hi > n):
        raise IndexError(f"section {lo}:{hi} outside the extent {n} (counted from 0)")
    return slice(lo, hi)


def _dummy(arg, lbounds, shape):
    """An explicit-shape dummy argument over the actual argument's storage."""
    a = arg.a if isinstance(arg, FArr) else arg
    if not isinstance(a, np.ndarray):
        raise TypeError("array dummy argument given a scalar")
    if shape is not None and tuple(a.shape) != tuple(shape):
        flat = a.reshape(-1, order="F")
        if not np.shares_memory(flat, a):
            raise ValueError("sequence association needs contiguous storage")
        n = int(np.prod(shape))
        a = flat[:n].reshape(shape, order="F")
    return FArr(a, lbounds)


def _recview(arr, idx):
    """One element of a record array as a 0-d view."""
    sl = tuple(slice(i, i + 1) for i in idx)
    return arr[sl].reshape(())


def _flat(buf):
    a = buf.a if isinstance(buf, FArr) else buf
    f = a.reshape(-1, order="F")
    if not np.shares_memory(f, a):
        raise ValueError("message buffer is not contiguous")
    return f


# ----------------------------------------------------------------------------
# list-directed reads from files (the marker templates); writes do nothing


def _io_open(G, unit, name):
    """Remember the file a unit names; it is read only if a read asks for it."""
    G.io_units[unit] = {"name": name, "lines": None}


def _io_read(G, unit, n):
    """The next record of `unit`: its first n whitespace-separated values."""
    u = G.io_units[unit]
    if u["lines"] is None:
        with open(G.io_path(u["name"])) as f:
            u["lines"] = iter(f.read().split("\n"))
    for line in u["lines"]:
        vals = line.replace(",", " ").split()
        if vals:
            if len(vals) < n:
                raise ValueError(f"record of {len(vals)} values for {n} items")
            return vals[:n]
    raise EOFError(u["name"])


def _io_close(G, unit):
    G.io_units.pop(unit, None)


def _io_write(G, unit, items):
    """A list-directed record written to a file unit: its values are kept, in
    order and unformatted, under the file's name (G.io_written); nothing is
    written to disk."""
    u = G.io_units.get(unit)
    if u is None:
        raise RuntimeError(f"write to unit {unit}, which no open names")
    rec = []
    for x in items:
        if isinstance(x, np.ndarray):
            rec.extend(v.item() for v in x.ravel(order="F"))
        elif isinstance(x, np.generic):
            rec.append(x.item())
        else:
            rec.append(x)
    G.io_written.setdefault(u["name"].strip(), []).append(rec)


def _io_internal(fmt, items):
    """An internal write of integers (and strings) into a character variable:
    list-directed (a blank and 11 columns for each default integer, a string
    as it stands) or with one Iw edit descriptor."""
    if fmt is None:
        return "".join(x if isinstance(x, str) else f" {int(x):11d}" for x in items)
    m = re.match(r"^\(\s*i(\d+)\s*\)$", fmt.strip().lower())
    if not m or len(items) != 1:
        raise NotImplementedError(f"internal write with format {fmt!r}")
    return f"{int(items[0]):{int(m.group(1))}d}"


# ----------------------------------------------------------------------------
# MPI: one rank (a state without a world), or several ranks run as threads of
# one process (states that share a World)


class World:
    """The communicator of ranks run as threads: mailboxes for point-to-point
    messages and slots for the collectives.  Every wait has a time limit."""

    def __init__(self, n, timeout=120.0):
        import threading
        self.n, self.timeout = n, timeout
        self.cv = threading.Condition()
        self.box = {}
        self.barrier = threading.Barrier(n, timeout=timeout)
        self.slots = [None] * n

    def post(self, src, dest, tag, data):
        with self.cv:
            self.box.setdefault((src, dest, tag), []).append(data)
            self.cv.notify_all()

    def take(self, src, dest, tag):
        with self.cv:
            if not self.cv.wait_for(lambda: self.box.get((src, dest, tag)), timeout=self.timeout):
                raise TimeoutError(f"rank {dest} waited for a message {tag} from rank {src}")
            return self.box[(src, dest, tag)].pop(0)


def _payload(buf, count):
    if isinstance(buf, (np.ndarray, FArr)):
        return _flat(buf)[:count].copy()
    return np.array([buf])[:count]


def _deliver(buf, data):
    if isinstance(buf, (np.ndarray, FArr)):
        _flat(buf)[:len(data)] = data
        return buf
    if len(data):
        return type(buf)(data[0]) if not isinstance(buf, np.generic) else data[0]
    return buf


def _mpi_sendrecv(G, sbuf, scount, stype, dest, stag, rbuf, rcount, rtype, src, rtag, comm, status, ierr):
    W = getattr(G, "world", None)
    data = _payload(sbuf, scount)
    if W is None:
        if dest != 0 or src != 0:
            raise RuntimeError(f"MPI_SENDRECV to {dest} from {src} on one rank")
        got = data
    else:
        W.post(G.rank, dest, stag, data)
        got = W.take(src, G.rank, rtag)
    if len(got) > rcount:
        raise RuntimeError(f"MPI_SENDRECV message of {len(got)} truncated to {rcount}")
    rbuf = _deliver(rbuf, got)
    return (sbuf, scount, stype, dest, stag, rbuf, rcount, rtype, src, rtag, comm, status, 0)


def _mpi_reduce(G, sbuf, rbuf, count, dtype, op, root, comm, ierr):
    """Sum or maximum over the ranks in rank order, at the root."""
    W = getattr(G, "world", None)
    if W is None:
        return (sbuf, _deliver(rbuf, _payload(sbuf, count)), count, dtype, op, root, comm, 0)
    W.slots[G.rank] = _payload(sbuf, count)
    W.barrier.wait()
    if G.rank == root:
        acc = W.slots[0].copy()
        for r in range(1, W.n):
            acc = acc + W.slots[r] if op == MPI_CONSTANTS["mpi_sum"] else np.maximum(acc, W.slots[r])
        rbuf = _deliver(rbuf, acc)
    W.barrier.wait()
    return (sbuf, rbuf, count, dtype, op, root, comm, 0)


def _mpi_bcast(G, buf, count, dtype, root, comm, ierr):
    W = getattr(G, "world", None)
    if W is None:
        return (buf, count, dtype, root, comm, 0)
    if G.rank == root:
        W.slots[root] = _payload(buf, count)
    W.barrier.wait()
    if G.rank != root:
        buf = _deliver(buf, W.slots[root])
    W.barrier.wait()
    return (buf, count, dtype, root, comm, 0)


def _mpi_barrier(G, comm, ierr):
    W = getattr(G, "world", None)
    if W is not None:
        W.barrier.wait()
    return (comm, 0)


def _mpi_comm_rank(G, comm, rank, ierr):
    return (comm, getattr(G, "rank", 0), 0)


BUILTIN_CALLS = {
    "mpi_sendrecv": _mpi_sendrecv,
    "mpi_reduce": _mpi_reduce,
    "mpi_bcast": _mpi_bcast,
    "mpi_barrier": _mpi_barrier,
    "mpi_comm_rank": _mpi_comm_rank,
}

MPI_CONSTANTS = {"mpi_comm_world": 0, "mpi_integer": 1, "mpi_double_precision": 2, "mpi_double": 2,
                 "mpi_sum": 3, "mpi_max": 4, "mpi_status_size": 6, "petsc_null_character": 0,
                 # names PETSc's Fortran headers define, for calls the caller supplies
                 "petsc_comm_world": 0, "petsc_decide": -1, "petsc_null_integer": 0, "petsc_copy_values": 0,
                 "matmpiaij": 0, "mat_final_assembly": 0, "insert_values": 1, "add_values": 2,
                 "scatter_forward": 0, "petsc_viewer_stdout_world": 0}

# ----------------------------------------------------------------------------
# source lines


def _strip_comment(line):
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


def _split_top(s, sep):
    """Split on `sep` outside parentheses and strings."""
    parts, depth, q, cur = [], 0, None, []
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
        elif ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    parts.append("".join(cur))
    return parts


def logical_lines(text, fname):
    """(file, line number, statement) for every statement, continuations joined."""
    out, pending, start = [], "", 0
    for n, raw in enumerate(text.split("\n"), 1):
        if raw.lstrip().startswith("#"):
            continue
        line = _strip_comment(raw).rstrip()
        if not line.strip():
            if pending:
                continue
            continue
        s = line.strip()
        if pending:
            if s.startswith("&"):
                s = s[1:]
            s = pending + " " + s
        else:
            start = n
        if s.endswith("&"):
            pending = s[:-1]
            continue
        pending = ""
        for part in _split_top(s, ";"):
            part = part.strip()
            if part:
                out.append((fname, start, _lower_outside_strings(part)))
    return out


# ----------------------------------------------------------------------------
# expressions

_TOKEN = re.compile(r"""
 (?P<ws>\s+)
|(?P<dotop>\.(?:and|or|not|eq|ne|lt|le|gt|ge|eqv|neqv|true|false)\.)
|(?P<num>(?:\d+\.\d+|\d+\.(?![a-z]{2,5}\.)|\.\d+|\d+)(?:[ed][+-]?\d+)?)
|(?P<name>[a-z_]\w*)
|(?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
|(?P<op>\*\*|//|==|/=|<=|>=|[-+*/<>=(),:%])
""", re.X)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot read {s[pos:]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        toks.append((kind, m.group()))
    toks.append(("end", ""))
    return toks


_REL = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=", ".eq.": "==", ".ne.": "!=",
        ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}


class ExprParser:
    def __init__(self, s):
        self.t = tokenize(s)
        self.i = 0

    def peek(self):
        return self.t[self.i][1]

    def kind(self):
        return self.t[self.i][0]

    def take(self, want=None):
        k, v = self.t[self.i]
        if want is not None and v != want:
            raise SyntaxError(f"expected {want!r}, got {v!r}")
        self.i += 1
        return v

    def done(self):
        return self.kind() == "end"

    def expr(self):
        e = self.or_()
        while self.peek() in (".eqv.", ".neqv."):
            op = self.take()
            e = ("rel", "==" if op == ".eqv." else "!=", e, self.or_())
        return e

    def or_(self):
        e = self.and_()
        while self.peek() == ".or.":
            self.take()
            e = ("or", e, self.and_())
        return e

    def and_(self):
        e = self.not_()
        while self.peek() == ".and.":
            self.take()
            e = ("and", e, self.not_())
        return e

    def not_(self):
        if self.peek() == ".not.":
            self.take()
            return ("not", self.not_())
        return self.rel()

    def rel(self):
        e = self.concat()
        if self.peek() in _REL:
            op = _REL[self.take()]
            e = ("rel", op, e, self.concat())
        return e

    def concat(self):
        e = self.add()
        while self.peek() == "//":
            self.take()
            e = ("cat", e, self.add())
        return e

    def add(self):
        if self.peek() in ("+", "-"):
            op = self.take()
            e = self.mul()
            if op == "-":
                e = ("neg", e)
        else:
            e = self.mul()
        while self.peek() in ("+", "-"):
            op = self.take()
            e = ("bin", op, e, self.mul())
        return e

    def mul(self):
        e = self.power()
        while self.peek() in ("*", "/"):
            op = self.take()
            e = ("bin", op, e, self.power())
        return e

    def power(self):
        b = self.primary()
        if self.peek() == "**":
            self.take()
            if self.peek() in ("+", "-"):
                op = self.take()
                x = self.power()
                return ("pow", b, ("neg", x) if op == "-" else x)
            return ("pow", b, self.power())
        return b

    def primary(self):
        k, v = self.t[self.i]
        if k == "num":
            self.i += 1
            return ("num", v)
        if k == "str":
            self.i += 1
            return ("str", v[1:-1].replace(v[0] * 2, v[0]))
        if v in (".true.", ".false."):
            self.i += 1
            return ("lit", v == ".true.")
        if v in ("+", "-"):
            self.i += 1
            x = self.power()
            return ("neg", x) if v == "-" else x
        if v == "(":
            self.i += 1
            e = self.expr()
            self.take(")")
            return ("paren", e)
        if k == "name":
            return self.designator()
        raise SyntaxError(f"unexpected {v!r}")

    def designator(self):
        parts = []
        while True:
            name = self.take()
            args = None
            if self.peek() == "(":
                self.take()
                args = self.arglist()
                self.take(")")
            parts.append((name, args))
            if self.peek() == "%":
                self.take()
                continue
            break
        return ("des", parts)

    def arglist(self):
        args = []
        if self.peek() == ")":
            return args
        while True:
            args.append(self.subscript())
            if self.peek() == ",":
                self.take()
                continue
            break
        return args

    def subscript(self):
        # keyword argument
        if self.kind() == "name" and self.t[self.i + 1][1] == "=":
            key = self.take()
            self.take("=")
            return ("kw", key, self.expr())
        lo = hi = None
        if self.peek() != ":":
            lo = self.expr()
            if self.peek() != ":":
                return lo
        self.take(":")
        if self.peek() not in (",", ")"):
            hi = self.expr()
        return ("range", lo, hi)


def parse_expr(s):
    p = ExprParser(s)
    e = p.expr()
    if not p.done():
        raise SyntaxError(f"trailing {p.peek()!r} in {s!r}")
    return e


# ----------------------------------------------------------------------------
# declarations and program units


class Sym:
    __slots__ = ("name", "kind", "tname", "dims", "param", "alloc", "where", "clen")

    def __init__(self, name, kind, tname=None, dims=None, param=None, alloc=False, where="loc"):
        self.name, self.kind, self.tname, self.dims = name, kind, tname, dims
        self.param, self.alloc, self.where, self.clen = param, alloc, where, None

    @property
    def rank(self):
        return len(self.dims) if self.dims else 0


_TYPESPEC = re.compile(r"^(integer|real\s*\*\s*8|real\s*\*\s*4|real|double\s+precision|logical|"
                       r"character\s*\(\s*len\s*=\s*(?:\d+|\*)\s*\)|character\s*\*\s*\d+|character|"
                       r"type\s*\(\s*\w+\s*\)|petscint|petscscalar|petscerrorcode)(?=\s|,|::|$)")
_OPAQUE = re.compile(r"^(ksp|mat|vec|is|vecscatter)\s+[a-z_]\w*(\s*,\s*[a-z_]\w*)*$")


def _kind_of(spec):
    spec = re.sub(r"\s+", "", spec)
    if spec in ("integer", "petscint", "petscerrorcode"):
        return "i", None
    if spec in ("real*8", "doubleprecision", "petscscalar"):
        return "r8", None
    if spec in ("real", "real*4"):
        return "r4", None
    if spec == "logical":
        return "l", None
    if spec.startswith("character"):
        return "c", None
    m = re.match(r"type\((\w+)\)", spec)
    if m:
        return "t", m.group(1)
    raise SyntaxError(spec)


def _parse_dims(text):
    """'1:3,lg1:ug1,:' -> list of (lo_ast, hi_ast) or ':' for deferred."""
    dims = []
    for d in _split_top(text, ","):
        d = d.strip()
        if d == ":":
            dims.append(":")
            continue
        halves = _split_top(d, ":")
        if len(halves) == 1:
            dims.append((("num", "1"), parse_expr(halves[0])))
        else:
            dims.append((parse_expr(halves[0]), parse_expr(halves[1])))
    return dims


def parse_decl(stmt):
    """A declaration statement -> list of (Sym, init_ast); None when `stmt` is not one."""
    if _OPAQUE.match(stmt):
        names = re.split(r"\s*,\s*", stmt.split(None, 1)[1].strip())
        return [(Sym(n, "o"), None) for n in names]
    m = _TYPESPEC.match(stmt)
    if not m:
        return None
    kind, tname = _kind_of(m.group(1))
    rest = stmt[m.end():]
    attrs, ents = [], rest
    if "::" in rest:
        a, ents = rest.split("::", 1)
        attrs = [x.strip() for x in _split_top(a, ",") if x.strip()]
    elif rest.strip().startswith(","):
        raise SyntaxError(f"attributes without '::' in {stmt!r}")
    dims, alloc, param = None, False, False
    for at in attrs:
        if at.startswith("dimension"):
            dims = _parse_dims(at[at.index("(") + 1:at.rindex(")")])
        elif at in ("allocatable", "pointer", "target"):
            alloc = True
        elif at == "parameter":
            param = True
        elif at.startswith("intent") or at == "save":
            pass
        else:
            raise SyntaxError(f"attribute {at!r}")
    out = []
    for ent in _split_top(ents, ","):
        ent = ent.strip()
        if not ent:
            continue
        init = None
        eq = _split_top(ent, "=")
        if len(eq) == 2:
            ent, init = eq[0].strip(), parse_expr(eq[1])
        mm = re.match(r"^([a-z_]\w*)\s*(\((.*)\))?\s*(\*\s*\d+)?$", ent)
        if not mm:
            raise SyntaxError(f"entity {ent!r}")
        edims = _parse_dims(mm.group(3)) if mm.group(2) else dims
        s = Sym(mm.group(1), kind, tname, edims, None, alloc or (edims is not None and ":" in edims))
        if param:
            s.param = init
            init = None
        out.append((s, init))
    return out


class Unit:
    def __init__(self, kind, name, args, fname, line):
        self.kind, self.name, self.args, self.fname, self.line = kind, name, args, fname, line
        self.syms = {}
        self.body = []
        self.implicit_none = False
        self.types = {}


def _match_paren(s, start):
    depth = 0
    for i in range(start, len(s)):
        if s[i] == "(":
            depth += 1
        elif s[i] == ")":
            depth -= 1
            if depth == 0:
                return i
    raise SyntaxError(f"unbalanced parentheses in {s!r}")


def parse_stmt(s):
    """One executable statement -> a tuple; block openers and closers included."""
    if re.match(r"^end\s*do$", s):
        return ("enddo",)
    if re.match(r"^end\s*if$", s):
        return ("endif",)
    if s == "else":
        return ("else",)
    m = re.match(r"^else\s*if\s*\(", s)
    if m:
        j = _match_paren(s, m.end() - 1)
        if s[j + 1:].strip() != "then":
            raise SyntaxError(s)
        return ("elif", parse_expr(s[m.end():j]))
    m = re.match(r"^if\s*\(", s)
    if m:
        j = _match_paren(s, m.end() - 1)
        cond = parse_expr(s[m.end():j])
        rest = s[j + 1:].strip()
        if rest == "then":
            return ("if", cond)
        return ("if1", cond, parse_stmt(rest))
    m = re.match(r"^do\s+while\s*\((.*)\)$", s)
    if m:
        return ("dowhile", parse_expr(m.group(1)))
    m = re.match(r"^do\s+([a-z_]\w*)\s*=\s*(.*)$", s)
    if m:
        b = [parse_expr(x) for x in _split_top(m.group(2), ",")]
        return ("do", m.group(1), b[0], b[1], b[2] if len(b) > 2 else None)
    m = re.match(r"^call\s+([a-z_]\w*)\s*(\((.*)\))?$", s)
    if m:
        args = []
        if m.group(2):
            p = ExprParser(m.group(3))
            if not p.done():
                args = p.arglist()
            if not p.done():
                raise SyntaxError(s)
        return ("call", m.group(1), args)
    if s in ("return", "exit", "cycle", "continue"):
        return (s,)
    if re.match(r"^stop\b", s):
        return ("stop",)
    m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", s)
    if m:
        p = ExprParser(m.group(2))
        return (m.group(1), p.arglist())
    if re.match(r"^(write|read|open|close|print|flush|format)\b", s) and not re.match(r"^\w+\s*(\(.*\))?\s*=", s):
        return ("io", s)
    if re.match(r"^(write|read|open|close)\s*\(", s):
        return ("io", s)
    parts = _split_top(s, "=")
    if len(parts) >= 2:
        # the first '=' at depth 0 that is not part of a relational operator
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
            elif ch == "=" and depth == 0 and s[i - 1] not in "=/<>" and (i + 1 >= len(s) or s[i + 1] not in "=>"):
                return ("assign", parse_expr(s[:i]), parse_expr(s[i + 1:]))
    raise SyntaxError(f"statement {s!r}")


def parse_sources(files):
    """[(fname, text)] -> (modules, subroutines) as Units."""
    modules, subs = [], {}
    cur, in_type, in_program = None, None, False
    for fname, text in files:
        for fn, line, s in logical_lines(text, fname):
            if in_program:
                if re.match(r"^end\s*program\b", s):
                    in_program = False
                continue
            m = re.match(r"^program\s+\w+$", s)
            if m:
                in_program = True
                continue
            m = re.match(r"^module\s+(\w+)$", s)
            if m:
                cur = Unit("module", m.group(1), [], fn, line)
                modules.append(cur)
                continue
            m = re.match(r"^subroutine\s+(\w+)\s*(\((.*)\))?$", s)
            if m:
                args = [a.strip() for a in (m.group(3) or "").split(",") if a.strip()]
                cur = Unit("sub", m.group(1), args, fn, line)
                if cur.name in subs:
                    raise SyntaxError(f"subroutine {cur.name} defined twice")
                subs[cur.name] = cur
                continue
            if re.match(r"^end\s*(module|subroutine)\b", s) or s == "end":
                cur = None
                continue
            if cur is None:
                raise SyntaxError(f"{fn}:{line}: statement outside a unit: {s!r}")
            if in_type is not None:
                if re.match(r"^end\s*type\b", s):
                    in_type = None
                    continue
                d = parse_decl(s)
                if d is None:
                    raise SyntaxError(f"{fn}:{line}: {s!r} in a type")
                cur.types[in_type].extend(sym for sym, _ in d)
                continue
            m = re.match(r"^type\s+(\w+)$", s) or re.match(r"^type\s*::\s*(\w+)$", s)
            if m:
                in_type = m.group(1)
                cur.types[in_type] = []
                continue
            if re.match(r"^use\b", s):
                continue
            if s == "implicit none":
                cur.implicit_none = True
                continue
            try:
                d = parse_decl(s)
            except SyntaxError as e:
                raise SyntaxError(f"{fn}:{line}: {e}") from None
            if d is not None:
                for sym, init in d:
                    cur.syms[sym.name] = sym
                    if init is not None:
                        raise SyntaxError(f"{fn}:{line}: initialised variable {sym.name}")
                continue
            try:
                cur.body.append((fn, line, parse_stmt(s)))
            except SyntaxError as e:
                raise SyntaxError(f"{fn}:{line}: {e}") from None
    return modules, subs


# ----------------------------------------------------------------------------
# translation to Python

_DTYPE = {"i": np.int32, "r8": np.float64, "r4": np.float32, "l": np.bool_, "c": object}
_ORDER = {"i": 0, "r4": 1, "r8": 2}
_INTRINSICS = {"abs", "sqrt", "dsqrt", "exp", "dexp", "log", "dlog", "log10", "cos", "dcos", "sin", "dsin",
               "acos", "dacos", "floor", "int", "nint", "dble", "real", "max", "min", "mod", "sum", "trim",
               "adjustl", "size", "sign", "dabs"}


class E:
    """A translated expression: Python code, its kind and its rank."""
    __slots__ = ("code", "kind", "rank", "tname", "const")

    def __init__(self, code, kind, rank=0, tname=None, const=None):
        self.code, self.kind, self.rank, self.tname, self.const = code, kind, rank, tname, const


class Translator:
    def __init__(self, files, param_overrides=None, check_bounds=False):
        """`check_bounds` checks every subscript and section against its
        dimension's extent (slower)."""
        self.check_bounds = check_bounds
        self.modules, self.subs = parse_sources(files)
        self.param_overrides = {k.lower(): v for k, v in (param_overrides or {}).items()}
        self.msyms, self.types, self.pvals = {}, {}, dict(MPI_CONSTANTS)
        for m in self.modules:
            for tn, fields in m.types.items():
                self.types[tn] = fields
        for m in self.modules:
            for name, s in m.syms.items():
                s.where = "mod"
                self.msyms[name] = s
        for name, s in self.msyms.items():
            if s.param is not None:
                self.pvals[name] = None
        for name, s in self.msyms.items():
            if s.param is not None:
                self.pvals[name] = self.param_overrides.get(name, self._const(s.param, s.kind))
        self.dtypes = {tn: self._record_dtype(tn) for tn in self.types}
        self.ns = None

    # constants -------------------------------------------------------------
    def _const(self, ast, kind=None):
        v = self._cval(ast)
        if kind == "i":
            return int(v)
        if kind == "r8":
            return float(v)
        if kind == "r4":
            return f32(v)
        return v

    def _cval(self, e):
        t = e[0]
        if t == "num":
            return self._num(e[1])[0]
        if t == "paren":
            return self._cval(e[1])
        if t == "neg":
            return -self._cval(e[1])
        if t == "bin":
            a, b, op = self._cval(e[2]), self._cval(e[3]), e[1]
            if op == "+":
                return a + b
            if op == "-":
                return a - b
            if op == "*":
                return a * b
            return _idiv(a, b) if isinstance(a, int) and isinstance(b, int) else a / b
        if t == "des" and len(e[1]) == 1 and e[1][0][1] is None:
            name = e[1][0][0]
            if name in self.pvals and self.pvals[name] is not None:
                return self.pvals[name]
        raise SyntaxError(f"not a constant: {e}")

    @staticmethod
    def _num(text):
        if re.match(r"^\d+$", text):
            return int(text), "i"
        if "d" in text:
            return float(text.replace("d", "e")), "r8"
        return _dec_to_f32(text), "r4"

    def _record_dtype(self, tn):
        fields = []
        for s in self.types[tn]:
            shape = ()
            if s.dims:
                shape = tuple(self._const(hi, "i") - self._const(lo, "i") + 1 for lo, hi in s.dims)
            fields.append((s.name, _DTYPE[s.kind], shape) if shape else (s.name, _DTYPE[s.kind]))
        return np.dtype(fields)

    def field(self, tn, name):
        for s in self.types[tn]:
            if s.name == name:
                return s
        raise KeyError(f"{tn}%{name}")

    # state -----------------------------------------------------------------
    def new_state(self, io_dir="."):
        """Module variables of one rank: fixed arrays allocated, scalars zero.
        Files the sources read are looked up in `io_dir`."""
        G = type("RankState", (), {})()
        G.io_units = {}
        G.io_written = {}
        G.io_path = lambda name: os.path.join(io_dir, name.strip())
        for name, s in self.msyms.items():
            if s.param is not None:
                continue
            if s.dims and not s.alloc:
                bounds = [(self._const(lo, "i"), self._const(hi, "i")) for lo, hi in s.dims]
                dt = self.dtypes[s.tname] if s.kind == "t" else _DTYPE[s.kind]
                val = FArr.alloc(dt, bounds)
            elif s.dims:
                val = None
            elif s.kind == "t":
                val = np.zeros((), dtype=self.dtypes[s.tname])
            else:
                val = {"i": 0, "r8": 0.0, "r4": 0.0, "l": False, "c": "", "o": None}[s.kind]
            setattr(G, "m_" + name, val)
        return G

    # build -----------------------------------------------------------------
    def build(self, overrides=None):
        """Translate every subroutine; `overrides` maps names to Python
        functions that replace (or supply) a subroutine."""
        src = ["import math", "import numpy as np"]
        self.outs = {name: self._outs(u) for name, u in self.subs.items()}
        for name, u in self.subs.items():
            src.append(self._translate(u))
        self.source = "\n".join(src)
        ns = {"FArr": FArr, "_dummy": _dummy, "_recview": _recview, "_idiv": _idiv, "_imod": _imod,
              "_powi": _powi, "_powi4": _powi4, "_fsum": _fsum, "_floor": _floor, "_trunc": _trunc,
              "_nint": _nint, "f32": f32, "_flat": _flat, "_missing": _missing, "_io_open": _io_open,
              "_io_read": _io_read, "_io_close": _io_close, "_io_write": _io_write, "_io_internal": _io_internal,
              "_ck": _ck, "_cks": _cks}
        for tn, dt in self.dtypes.items():
            ns["_DT_" + tn] = dt
        for k, f in BUILTIN_CALLS.items():
            ns["f_" + k] = f
        exec(compile(self.source, "<reference translation>", "exec"), ns)
        for k, f in (overrides or {}).items():
            ns["f_" + k.lower()] = f
        # a subroutine the sources call but do not define: one supplied as an override, else an error
        ns["_ext"] = lambda n: ns["f_" + n] if "f_" + n in ns else _missing(n)
        self.ns = ns
        return ns

    def call(self, G, name, *args):
        return self.ns["f_" + name.lower()](G, *args)

    # a unit ----------------------------------------------------------------
    def _outs(self, u):
        """Positions of the dummies a call may change (assigned, a loop
        variable, or passed on to another call), for the copy-out."""
        names = set()

        def base(e):
            return e[1][0][0] if e[0] == "des" else None

        def walk(st):
            t = st[0]
            if t == "assign":
                names.add(base(st[1]))
            elif t == "do":
                names.add(st[1])
            elif t == "call":
                for a in st[2]:
                    if a[0] == "des":
                        names.add(base(a))
            elif t == "if1":
                walk(st[2])
            elif t == "allocate":
                for a in st[1]:
                    names.add(base(a))

        for _, _, st in u.body:
            walk(st)
        return {k for k, a in enumerate(u.args) if a in names}

    def _translate(self, u):
        self.u = u
        self.tmp = 0
        args = ", ".join("v_" + a for a in u.args)
        self.ret = "return (" + "".join(f"v_{a}, " for a in u.args) + ")"
        body = []
        self._body(u.body, body)
        pre = []
        for name, s in u.syms.items():
            if name in u.args or s.param is not None:
                continue
            if s.dims:
                if s.alloc:
                    pre.append(f"v_{name} = None")
                else:
                    b = ", ".join(f"({self._iexpr(lo)}, {self._iexpr(hi)})" for lo, hi in s.dims)
                    dt = f"_DT_{s.tname}" if s.kind == "t" else f"np.{np.dtype(_DTYPE[s.kind]).name}"
                    pre.append(f"v_{name} = FArr.alloc({dt}, [{b}])")
            elif s.kind == "t":
                pre.append(f"v_{name} = np.zeros((), dtype=_DT_{s.tname})")
            else:
                pre.append(f"v_{name} = {self._zero(s.kind)}")
        for a in u.args:
            s = self._sym(a)
            if not s.dims:
                continue
            if ":" in s.dims:
                pre.append(f"v_{a} = _dummy(v_{a}, [{', '.join('1' for _ in s.dims)}], None)")
                continue
            lb = ", ".join(self._iexpr(lo) for lo, _ in s.dims)
            shp = ", ".join(f"({self._iexpr(hi)}) - ({self._iexpr(lo)}) + 1" for lo, hi in s.dims)
            pre.append(f"v_{a} = _dummy(v_{a}, [{lb}], ({shp},))")
        lines = [f"def f_{u.name}(G{', ' if args else ''}{args}):"]
        lines += ["    " + l for l in pre]
        lines += body
        lines.append("    " + self.ret)
        return "\n".join(lines)

    @staticmethod
    def _zero(kind):
        return {"i": "0", "r8": "0.0", "r4": "0.0", "l": "False", "c": "''", "o": "None"}[kind]

    def _sym(self, name):
        u = self.u
        if name in u.syms:
            return u.syms[name]
        if name in self.msyms:
            return self.msyms[name]
        if name in u.args or not u.implicit_none:
            kind = "i" if name[0] in "ijklmn" else "r4"
            s = Sym(name, kind)
            u.syms[name] = s
            return s
        return None

    def _ref(self, s):
        return ("G.m_" if s.where == "mod" else "v_") + s.name

    # statements ------------------------------------------------------------
    def _body(self, stmts, out):
        ind = 1
        for fn, line, st in stmts:
            try:
                ind = self._stmt(st, out, ind)
            except SyntaxError as e:
                raise SyntaxError(f"{fn}:{line}: {e}") from None
        if ind != 1:
            raise SyntaxError(f"{self.u.name}: unbalanced blocks")

    def _stmt(self, st, out, ind):
        pad = "    " * ind
        t = st[0]
        if t == "if":
            out += [pad + f"if {self._cond(st[1])}:", pad + "    pass"]
            return ind + 1
        if t == "elif":
            pad = "    " * (ind - 1)
            out += [pad + f"elif {self._cond(st[1])}:", pad + "    pass"]
            return ind
        if t == "else":
            pad = "    " * (ind - 1)
            out += [pad + "else:", pad + "    pass"]
            return ind
        if t in ("endif", "enddo"):
            return ind - 1
        if t == "if1":
            out.append(pad + f"if {self._cond(st[1])}:")
            if self._stmt(st[2], out, ind + 1) != ind + 1:
                raise SyntaxError("block statement inside a logical if")
            return ind
        if t == "dowhile":
            out += [pad + f"while {self._cond(st[1])}:", pad + "    pass"]
            return ind + 1
        if t == "do":
            var, lo, hi, step = st[1:]
            s = self._sym(var)
            if s is None or s.kind != "i" or s.dims:
                raise SyntaxError(f"loop variable {var}")
            L, H = self._iexpr(lo), self._iexpr(hi)
            if step is None:
                rng = f"range({L}, ({H}) + 1)"
            else:
                S = self._iexpr(step)
                rng = f"range({L}, ({H}) + (1 if ({S}) > 0 else -1), {S})"
            ref = self._ref(s)
            if s.where == "mod":
                out += [pad + f"for _lv in {rng}:", pad + f"    {ref} = _lv"]
            else:
                out += [pad + f"for {ref} in {rng}:", pad + "    pass"]
            return ind + 1
        if t == "assign":
            out.append(pad + self._assign(st[1], st[2]))
            return ind
        if t == "call":
            out.extend(pad + l for l in self._call(st[1], st[2]))
            return ind
        if t == "return":
            out.append(pad + self.ret)
            return ind
        if t == "exit":
            out.append(pad + "break")
            return ind
        if t == "cycle":
            out.append(pad + "continue")
            return ind
        if t == "io":
            out.extend(pad + l for l in self._io(st[1]))
            return ind
        if t == "continue":
            out.append(pad + "pass")
            return ind
        if t == "stop":
            out.append(pad + "raise RuntimeError('stop')")
            return ind
        if t == "allocate":
            for a in st[1]:
                if a[0] != "des" or len(a[1]) != 1 or a[1][0][1] is None:
                    raise SyntaxError("allocate of a non-array")
                name, subs = a[1][0]
                s = self._sym(name)
                bounds = []
                for d in subs:
                    if d[0] == "range":
                        bounds.append(f"({self._iexpr(d[1])}, {self._iexpr(d[2])})")
                    else:
                        bounds.append(f"(1, {self._iexpr(d)})")
                dt = f"_DT_{s.tname}" if s.kind == "t" else f"np.{np.dtype(_DTYPE[s.kind]).name}"
                out.append(pad + f"{self._ref(s)} = FArr.alloc({dt}, [{', '.join(bounds)}])")
            return ind
        if t == "deallocate":
            for a in st[1]:
                out.append(pad + f"{self._ref(self._sym(a[1][0][0]))} = None")
            return ind
        raise SyntaxError(f"statement {st}")

    def _io(self, s):
        """open(unit, file=...), read(unit, *) items, write(unit, *) items,
        internal writes of integers and close(unit); writes to the terminal,
        print and format statements do nothing."""
        m = re.match(r"^(open|read|close|write)\s*\(", s)
        if not m:
            return ["pass"]
        if m.group(1) == "write":
            return self._write(s, m)
        j = _match_paren(s, m.end() - 1)
        ctl = _split_top(s[m.end():j], ",")
        unit = self._ex(parse_expr(ctl[0])).code
        if m.group(1) == "open":
            files = [c.split("=", 1)[1] for c in ctl[1:] if re.match(r"^\s*file\s*=", c)]
            if not files:
                return ["pass"]
            return [f"_io_open(G, {unit}, {self._ex(parse_expr(files[0])).code})"]
        if m.group(1) == "close":
            return [f"_io_close(G, {unit})"]
        if len(ctl) != 2 or ctl[1].strip() != "*":
            raise SyntaxError(f"read other than list-directed: {s!r}")
        items = [parse_expr(x) for x in _split_top(s[j + 1:], ",") if x.strip()]
        self.tmp += 1
        v = f"_v{self.tmp}"
        out = [f"{v} = _io_read(G, {unit}, {len(items)})"]
        for k, it in enumerate(items):
            L = self._des(it, lvalue=True)
            conv = {"i": "int", "r8": "float", "r4": "f32"}.get(L.kind)
            if conv is None or L.rank:
                raise SyntaxError(f"read into {L.kind} of rank {L.rank}")
            val = f"float({v}[{k}].replace('d', 'e').replace('D', 'E'))" if conv != "int" else f"int({v}[{k}])"
            out.append(f"{L.code} = {val if conv != 'f32' else 'f32(' + val + ')'}")
        return out

    def _write(self, s, m):
        j = _match_paren(s, m.end() - 1)
        ctl = [c.strip() for c in _split_top(s[m.end():j], ",")]
        items = [parse_expr(x) for x in _split_top(s[j + 1:], ",") if x.strip()]
        if ctl[0] == "*":
            return ["pass"]
        fmt = None if len(ctl) < 2 or ctl[1] == "*" else ctl[1]
        U = self._ex(parse_expr(ctl[0]))
        if U.kind == "c":
            if fmt is not None and fmt.startswith(("'", '"')):
                fmt = self._ex(parse_expr(fmt)).code
            elif fmt is not None:
                return [f"raise NotImplementedError({('internal write: ' + s)!r})"]
            L = self._des(parse_expr(ctl[0]), lvalue=True)
            vals = ", ".join(self._ex(x).code for x in items)
            return [f"{L.code} = _io_internal({fmt}, [{vals}])"]
        if fmt is not None:
            # a formatted record to a file: an error if it is ever reached
            return [f"raise NotImplementedError({('formatted write: ' + s)!r})"]
        vals = []
        for x in items:
            X = self._ex(x)
            vals.append(X.code if X.rank == 0 else f"np.array({X.code})")
        return [f"_io_write(G, {U.code}, [{', '.join(vals)}])"]

    def _cond(self, e):
        return self._ex(e).code

    def _assign(self, lhs, rhs):
        L = self._des(lhs, lvalue=True)
        R = self._ex(rhs)
        if L.rank == 0 and R.rank == 0:
            return f"{L.code} = {self._convert(R, L.kind)}"
        if L.rank == 0 and L.kind == "t":
            return f"{L.code} = {R.code}"
        return f"{L.code}[...] = {self._convert(R, L.kind)}"

    def _convert(self, R, kind):
        if R.rank > 0 or kind == R.kind or kind in ("c", "l", "t"):
            return R.code
        if kind == "i":
            return f"_trunc({R.code})" if R.kind != "i" else R.code
        if kind == "r8":
            return f"float({R.code})" if R.kind == "i" else R.code
        if kind == "r4":
            return f"f32({R.code})"
        return R.code

    def _call(self, name, args):
        if name in self.subs:
            callee = self.subs[name]
            if len(args) != len(callee.args):
                raise SyntaxError(f"call {name}: {len(args)} arguments for {len(callee.args)}")
        fn = f"f_{name}" if (name in self.subs or name in BUILTIN_CALLS) else f"_ext('{name}')"
        outs = self.outs[name] if name in self.subs else set(range(len(args)))
        codes, backs = [], []
        for k, a in enumerate(args):
            an = a[1][0][0] if a[0] == "des" else None
            if an is not None and (an not in self.pvals or (an in self.u.syms and self.u.syms[an].param is None)) \
                    and not (an in self.u.syms and self.u.syms[an].param is not None):
                s = self._sym(a[1][0][0])
                if s is not None:
                    D = self._des(a, lvalue=False, for_arg=True)
                    codes.append(D.code)
                    if D.rank == 0 and D.kind != "t" and k in outs:
                        Lv = self._des(a, lvalue=True)
                        backs.append((k, Lv.code, D.kind))
                    continue
            X = self._ex(a)
            codes.append(X.code)
        self.tmp += 1
        r = f"_r{self.tmp}"
        out = [f"{r} = {fn}(G{''.join(', ' + c for c in codes)})"]
        for k, code, kind in backs:
            out.append(f"{code} = {r}[{k}]")
        return out

    # expressions -----------------------------------------------------------
    def _ex(self, e):
        t = e[0]
        if t == "num":
            v, k = self._num(e[1])
            return E(repr(v), k, const=v)
        if t == "str":
            return E(repr(e[1]), "c")
        if t == "lit":
            return E(repr(e[1]), "l")
        if t == "paren":
            x = self._ex(e[1])
            return E(f"({x.code})", x.kind, x.rank, x.tname)
        if t == "neg":
            x = self._ex(e[1])
            return E(f"(-{x.code})", x.kind, x.rank)
        if t == "not":
            return E(f"(not {self._ex(e[1]).code})", "l")
        if t in ("and", "or"):
            a, b = self._ex(e[1]), self._ex(e[2])
            if a.rank or b.rank:
                raise SyntaxError("array logical")
            return E(f"({a.code} {t} {b.code})", "l")
        if t == "rel":
            a, b = self._ex(e[2]), self._ex(e[3])
            if a.rank or b.rank:
                raise SyntaxError("array comparison")
            return E(f"({a.code} {e[1]} {b.code})", "l")
        if t == "cat":
            a, b = self._ex(e[1]), self._ex(e[2])
            return E(f"({a.code} + {b.code})", "c")
        if t == "bin":
            return self._bin(e[1], self._ex(e[2]), self._ex(e[3]))
        if t == "pow":
            return self._pow(self._ex(e[1]), e[2])
        if t == "des":
            return self._des_or_call(e)
        raise SyntaxError(f"expression {e}")

    def _bin(self, op, a, b):
        if a.kind not in _ORDER or b.kind not in _ORDER:
            raise SyntaxError(f"operator {op} on {a.kind}, {b.kind}")
        kind = a.kind if _ORDER[a.kind] >= _ORDER[b.kind] else b.kind
        rank = max(a.rank, b.rank)
        if rank == 0 and kind == "i" and op == "/":
            return E(f"_idiv({a.code}, {b.code})", "i")
        if rank > 0 and kind == "i" and op == "/":
            raise SyntaxError("integer array division")
        if kind == "r4" and rank == 0:
            # an integer operand is converted to single precision first
            ac = f"f32({a.code})" if a.kind == "i" else a.code
            bc = f"f32({b.code})" if b.kind == "i" else b.code
            return E(f"f32({ac} {op} {bc})", kind)
        return E(f"({a.code} {op} {b.code})", kind, rank)

    def _pow(self, b, east):
        if east[0] == "num" and re.match(r"^\d+$", east[1]):
            n = int(east[1])
            if b.rank:
                raise SyntaxError("array power")
            if b.kind == "i":
                return E(f"(({b.code}) ** {n})", "i")
            return E(f"_powi4({b.code}, {n})" if b.kind == "r4" else f"_powi({b.code}, {n})", b.kind)
        x = self._ex(east)
        if b.rank or x.rank:
            raise SyntaxError("array power")
        kind = b.kind if _ORDER[b.kind] >= _ORDER[x.kind] else x.kind
        if kind == "i":
            return E(f"(({b.code}) ** ({x.code}))", "i")
        code = f"math.pow({b.code}, {x.code})"
        return E(f"f32({code})" if kind == "r4" else code, kind)

    def _des_or_call(self, e):
        parts = e[1]
        name, args = parts[0]
        s = self._sym(name) if (name in self.u.syms or name in self.msyms) else None
        local = name in self.u.syms and self.u.syms[name].param is None
        if name in self.u.syms and self.u.syms[name].param is not None and args is None:
            ls = self.u.syms[name]
            v = self._const(ls.param, ls.kind)
            return E(repr(v), ls.kind, const=v)
        if name in self.pvals and not local and len(parts) == 1 and args is None:
            v = self.pvals[name]
            if name in self.msyms:
                kind = self.msyms[name].kind
            else:
                kind = "i"
            return E(repr(v), kind, const=v)
        if s is None and args is not None and name in _INTRINSICS and len(parts) == 1:
            return self._intrinsic(name, args)
        if s is None:
            s = self._sym(name)
            if s is None:
                raise SyntaxError(f"unknown name {name}")
        return self._des(e, lvalue=False)

    def _intrinsic(self, name, args):
        xs = [self._ex(a) for a in args]
        x = xs[0]
        real = lambda k: k in ("r8", "r4")
        if name in ("abs", "dabs"):
            return E(f"abs({x.code})" if x.rank == 0 else f"np.abs({x.code})", x.kind, x.rank)
        if name in ("sqrt", "dsqrt", "exp", "dexp", "log", "dlog", "log10", "cos", "dcos", "sin", "dsin",
                    "acos", "dacos"):
            fn = {"dsqrt": "sqrt", "dexp": "exp", "dlog": "log", "dcos": "cos", "dsin": "sin",
                  "dacos": "acos"}.get(name, name)
            if x.rank:
                raise SyntaxError(f"{name} of an array")
            arg = x.code if real(x.kind) else f"float({x.code})"
            code = f"math.{fn}({arg})"
            # a single-precision argument gives a single-precision result (the double result rounded once)
            if x.kind == "r4" and not name.startswith("d"):
                return E(f"f32({code})", "r4")
            return E(code, "r8")
        if name == "floor":
            return E(f"_floor({x.code})", "i")
        if name == "int":
            return E(f"_trunc({x.code})", "i")
        if name == "nint":
            return E(f"_nint({x.code})", "i")
        if name == "dble":
            return E(f"float({x.code})", "r8")
        if name == "real":
            return E(f"f32({x.code})", "r4")
        if name in ("max", "min"):
            kinds = {y.kind for y in xs}
            if len(kinds) != 1:
                raise SyntaxError(f"{name} of mixed kinds {kinds}")
            return E(f"{name}({', '.join(y.code for y in xs)})", x.kind)
        if name == "mod":
            y = xs[1]
            if x.kind == "i" and y.kind == "i":
                return E(f"_imod({x.code}, {y.code})", "i")
            return E(f"math.fmod({x.code}, {y.code})", "r8")
        if name == "sum":
            return E(f"_fsum({x.code})", x.kind)
        if name == "trim":
            return E(f"({x.code}).rstrip()", "c")
        if name == "adjustl":
            return E(f"({x.code}).lstrip()", "c")
        if name == "sign":
            y = xs[1]
            return E(f"math.copysign(abs({x.code}), {y.code})", x.kind)
        if name == "size":
            return E(f"({x.code}).size", "i")
        raise SyntaxError(name)

    def _index(self, s, k, a, static_lb, base, extent=None):
        """Code of one subscript of dimension k: (code, is_slice); `extent` is
        the code of the dimension's length, for the bounds checks."""
        off = str(static_lb) if static_lb is not None else f"{base}.o{k}"
        if a[0] == "range":
            lo = None if a[1] is None else f"({self._iexpr(a[1])})-{off}"
            hi = None if a[2] is None else f"({self._iexpr(a[2])})-{off}+1"
            if self.check_bounds and extent is not None:
                return f"_cks({lo}, {hi}, {extent})", True
            return f"{lo or ''}:{hi or ''}", True
        if self.check_bounds and extent is not None:
            return f"_ck(({self._iexpr(a)})-{off}, {extent})", False
        return f"({self._iexpr(a)})-{off}", False

    def _iexpr(self, a):
        x = self._ex(a)
        if x.kind != "i" or x.rank:
            raise SyntaxError(f"subscript of kind {x.kind}")
        return x.code

    def _static_lbs(self, s, dims):
        out = []
        for d in dims:
            if d == ":" or s.alloc:
                out.append(None)
                continue
            try:
                out.append(self._const(d[0], "i"))
            except SyntaxError:
                out.append(None)
        return out

    def _des(self, e, lvalue=False, for_arg=False):
        parts = e[1]
        name, args = parts[0]
        s = self._sym(name)
        if s is None:
            raise SyntaxError(f"unknown name {name}")
        base = self._ref(s)
        if s.kind == "t" and len(parts) == 2:
            comp, cargs = parts[1]
            f = self.field(s.tname, comp)
            idx, rank = [], 0
            if s.dims:
                lbs = self._static_lbs(s, s.dims)
                sub = args if args is not None else [("range", None, None)] * len(s.dims)
                for k, a in enumerate(sub):
                    c, sl = self._index(s, k, a, lbs[k], base, f"{base}.a.shape[{k}]")
                    idx.append(c)
                    rank += sl
                arr = f"{base}.a['{comp}']"
            else:
                if args is not None:
                    raise SyntaxError(f"subscripts on scalar {name}")
                arr = f"{base}['{comp}']"
            if f.dims:
                flbs = [self._const(lo, "i") for lo, _ in f.dims]
                sub = cargs if cargs is not None else [("range", None, None)] * len(f.dims)
                fext = [self._const(hi, "i") - self._const(lo, "i") + 1 for lo, hi in f.dims]
                for k, a in enumerate(sub):
                    c, sl = self._index(f, k, a, flbs[k], None, str(fext[k]))
                    idx.append(c)
                    rank += sl
            elif cargs is not None:
                raise SyntaxError(f"subscripts on scalar component {comp}")
            code = f"{arr}[{', '.join(idx)}]" if idx else (arr if rank else f"{arr}[()]")
            if not s.dims and not f.dims:
                code = arr
            return self._read(code, f.kind, rank, lvalue, scalar_0d=(not idx))
        if len(parts) > 1:
            raise SyntaxError(f"component of non-record {name}")
        if not s.dims:
            if args is not None:
                raise SyntaxError(f"{name} is not an array")
            if s.kind == "t":
                return E(base, "t", 0, s.tname)
            return E(base, s.kind, 0)
        if args is None:
            return E(f"{base}.a", s.kind, s.rank, s.tname)
        lbs = self._static_lbs(s, s.dims)
        idx, rank = [], 0
        for k, a in enumerate(args):
            c, sl = self._index(s, k, a, lbs[k], base, f"{base}.a.shape[{k}]")
            idx.append(c)
            rank += sl
        code = f"{base}.a[{', '.join(idx)}]"
        if s.kind == "t":
            if rank == 0 and for_arg:
                return E(f"_recview({base}.a, ({', '.join(idx)},))", "t", 0, s.tname)
            return E(code, "t", rank, s.tname)
        return self._read(code, s.kind, rank, lvalue)

    def _read(self, code, kind, rank, lvalue, scalar_0d=False):
        if lvalue or rank:
            if lvalue and scalar_0d and rank == 0:
                return E(code, kind, 0)
            return E(code, kind, rank)
        if kind == "i":
            return E(f"int({code})", kind)
        if kind in ("r8", "r4"):
            return E(f"float({code})", kind)
        if kind == "l":
            return E(f"bool({code})", kind)
        return E(code, kind)


def _missing(name):
    raise NotImplementedError(f"subroutine {name} is not part of the translated sources")
