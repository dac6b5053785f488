"""GAMS scalar-format (.gms) frontend: source text -> Problem.

Restates the reference's frontend (source/gams/frontend.cpp, ast.hpp,
include/cuminlp/gams.hpp) so that MINLPLib models in GAMS Convert's scalar
format reach the device path:

- lexing (frontend.cpp:92-285): column-1 `*` comments and `$` control lines,
  `$ontext`..`$offtext` blocks, case-folded identifiers, `%macro%` tokens;
- statements (frontend.cpp:415-660): variable domains, equation
  definitions, `.lo/.up/.fx/.l` attributes, the Solve statement;
- an expression AST with the reference's algebraic simplifications and
  constant folding (ast.hpp:80-330);
- objective-variable elimination from an `=E=` definition, or from a
  one-sided inequality that is tight at the optimum (frontend.cpp:839-1095);
- lowering to the DAG in the reference's node order (frontend.cpp:1100-1590),
  so the Problem this builds is node-for-node the one the reference builds.

The solver minimises: a `maximizing` model gets a negated objective and
`ParsedModel.sense == "max"`.
"""

from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

from . import _abi as A
from .problem import Expr, Problem

INF = math.inf


class ParseError(ValueError):
    """Anything the frontend cannot represent (gams.hpp:67-100); `kind` is
    one of syntax, non_scalar, discrete, unsupported_function,
    unrepresentable, io."""

    def __init__(self, line: int, message: str, kind: str = "syntax"):
        super().__init__(f"line {line}: {message}")
        self.line = line
        self.kind = kind


# -- lexer -----------------------------------------------------------------
IDENT, NUMBER, PLUS, MINUS, STAR, SLASH, POW, LPAREN, RPAREN, COMMA, SEMI, ASSIGN, REL, DOTDOT, DOT, END = range(16)
_NUM = re.compile(r"(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")


@dataclass
class Token:
    kind: int
    text: str = ""
    value: float = 0.0
    rel: str = ""
    line: int = 1


def lex(src: str) -> list[Token]:
    out: list[Token] = []
    i, line, at_start, n = 0, 1, True, len(src)

    def skip_line(j):
        while j < n and src[j] != "\n":
            j += 1
        return j

    while i < n:
        c = src[i]
        if c == "\n":
            i += 1
            line += 1
            at_start = True
            continue
        if at_start and c == "*":
            i = skip_line(i)
            continue
        if at_start and c == "$":
            begin = i
            i = skip_line(i)
            if src[begin:i].lower().startswith("$ontext"):
                while i < n:
                    i += 1
                    line += 1
                    ls = i
                    i = skip_line(i)
                    if src[ls:i].lower().startswith("$offtext"):
                        break
            continue
        if c.isspace():
            at_start = False
            i += 1
            continue
        at_start = False
        if c.isascii() and (c.isalpha() or c == "_"):
            begin = i
            while i < n and src[i].isascii() and (src[i].isalnum() or src[i] == "_"):
                i += 1
            out.append(Token(IDENT, src[begin:i].lower(), line=line))
            continue
        if c.isdigit() or (c == "." and i + 1 < n and src[i + 1].isdigit()):
            m = _NUM.match(src, i)
            if not m:
                raise ParseError(line, "malformed number")
            out.append(Token(NUMBER, value=float(m.group(0)), line=line))
            i = m.end()
            continue
        if c == "%":
            begin = i
            i += 1
            while i < n and src[i] not in "%\n":
                i += 1
            if i < n and src[i] == "%":
                i += 1
            out.append(Token(IDENT, src[begin:i].lower(), line=line))
            continue
        single = {"+": PLUS, "-": MINUS, "/": SLASH, "(": LPAREN, ")": RPAREN, ",": COMMA, ";": SEMI}
        if c in single:
            out.append(Token(single[c], line=line))
            i += 1
            continue
        if c == "*":
            if i + 1 < n and src[i + 1] == "*":
                out.append(Token(POW, line=line))
                i += 2
            else:
                out.append(Token(STAR, line=line))
                i += 1
            continue
        if c == ".":
            if i + 1 < n and src[i + 1] == ".":
                out.append(Token(DOTDOT, line=line))
                i += 2
            else:
                out.append(Token(DOT, line=line))
                i += 1
            continue
        if c == "=":
            if i + 2 < n and src[i + 1].isascii() and src[i + 1].isalpha() and src[i + 2] == "=":
                r = src[i + 1].lower()
                if r not in "elgn":
                    raise ParseError(line, "unknown relational operator")
                out.append(Token(REL, rel=r, line=line))
                i += 3
            else:
                out.append(Token(ASSIGN, line=line))
                i += 1
            continue
        if c in "'\"":
            raise ParseError(line, "quoted set element: this file has indexed identifiers and is not in GAMS scalar "
                                   "format; regenerate it with GAMS Convert", "non_scalar")
        raise ParseError(line, f"unexpected character '{c}'")
    out.append(Token(END, line=line))
    return out


# -- AST -------------------------------------------------------------------
NUM, VAR, ADD, SUB, MUL, DIV, NEG, CALL = range(8)
FUNCS = {"sqr": "sqr", "sqrt": "sqrt", "exp": "exp", "log": "log", "log10": "log10", "log2": "log2", "abs": "abs",
         "sin": "sin", "cos": "cos", "tanh": "tanh", "min": "min", "max": "max", "power": "power",
         "rpower": "power"}
UNSUPPORTED = {"tan", "arctan", "arcsin", "arccos", "errorf", "sign", "signpower", "ceil", "floor", "round", "trunc",
               "mod", "div", "centropy", "sinh", "cosh", "gamma", "loggamma", "beta", "entropy", "sigmoid", "slexp",
               "sqexp", "edist", "poly", "ifthen", "vcpower", "cvpower", "ncpcm"}
NON_SCALAR = {"set", "sets", "parameter", "parameters", "table", "alias", "scalar", "scalars", "loop", "sum", "prod",
              "smax", "smin", "abort", "display", "file", "put", "repeat", "while", "for"}


def _fmin(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return a if a <= b else b


def _fmax(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return a if a >= b else b


def _feq(a, b):
    return not (a < b) and not (b < a)


def _fold_call(f: str, a: list[float]):
    x = a[0]
    try:
        if f == "sqr":
            return x * x
        if f == "sqrt":
            return None if x < 0.0 else math.sqrt(x)
        if f == "exp":
            return math.exp(x)
        if f == "log":
            return None if x <= 0.0 else math.log(x)
        if f == "log10":
            return None if x <= 0.0 else math.log10(x)
        if f == "log2":
            return None if x <= 0.0 else math.log2(x)
        if f == "abs":
            return math.fabs(x)
        if f == "sin":
            return math.sin(x)
        if f == "cos":
            return math.cos(x)
        if f == "tanh":
            return math.tanh(x)
        if f == "min":
            return _fmin(x, a[1])
        if f == "max":
            return _fmax(x, a[1])
        if f == "power":
            e = a[1]
            if math.floor(e) < e and x <= 0.0:
                return None
            return math.pow(x, e)
    except (OverflowError, ValueError):
        return math.inf if f in ("exp", "power") else None
    return None


@dataclass
class _Node:
    kind: int
    value: float = 0.0
    sym: int = -1
    func: str = ""
    args: tuple = ()
    line: int = 0


class Ast:
    """Expression nodes in creation order (a child's index is below its
    parent's), with the builders' simplifications of ast.hpp."""

    def __init__(self):
        self.nodes: list[_Node] = []
        self._folds: list = []

    def _push(self, n: _Node) -> int:
        self.nodes.append(n)
        return len(self.nodes) - 1

    def num(self, v: float, line: int = 0) -> int:
        return self._push(_Node(NUM, value=float(v), line=line))

    def var(self, sym: int, line: int = 0) -> int:
        return self._push(_Node(VAR, sym=sym, line=line))

    def call(self, f: str, args, line: int = 0) -> int:
        return self._push(_Node(CALL, func=f, args=tuple(args), line=line))

    def as_num(self, i):
        n = self.nodes[i]
        return n.value if n.kind == NUM else None

    def neg(self, a: int) -> int:
        v = self.as_num(a)
        if v is not None:
            return self.num(-v, self.nodes[a].line)
        if self.nodes[a].kind == NEG:
            return self.nodes[a].args[0]
        return self._push(_Node(NEG, args=(a,), line=self.nodes[a].line))

    def add(self, a: int, b: int) -> int:
        va, vb = self.as_num(a), self.as_num(b)
        if va is not None and vb is not None:
            return self.num(va + vb, self.nodes[a].line)
        if vb is not None and _feq(vb, 0.0):
            return a
        if va is not None and _feq(va, 0.0):
            return b
        return self._push(_Node(ADD, args=(a, b), line=self.nodes[a].line))

    def sub(self, a: int, b: int) -> int:
        va, vb = self.as_num(a), self.as_num(b)
        if va is not None and vb is not None:
            return self.num(va - vb, self.nodes[a].line)
        if vb is not None and _feq(vb, 0.0):
            return a
        if va is not None and _feq(va, 0.0):
            return self.neg(b)
        if self.nodes[b].kind == NEG:
            return self.add(a, self.nodes[b].args[0])
        return self._push(_Node(SUB, args=(a, b), line=self.nodes[a].line))

    def mul(self, a: int, b: int) -> int:
        va, vb = self.as_num(a), self.as_num(b)
        if va is not None and vb is not None:
            return self.num(va * vb, self.nodes[a].line)
        if vb is not None and _feq(vb, 1.0):
            return a
        if va is not None and _feq(va, 1.0):
            return b
        if vb is not None and _feq(vb, -1.0):
            return self.neg(a)
        if va is not None and _feq(va, -1.0):
            return self.neg(b)
        return self._push(_Node(MUL, args=(a, b), line=self.nodes[a].line))

    def div(self, a: int, b: int) -> int:
        va, vb = self.as_num(a), self.as_num(b)
        if va is not None and vb is not None and not _feq(vb, 0.0):
            return self.num(va / vb, self.nodes[a].line)
        if vb is not None and _feq(vb, 1.0):
            return a
        if vb is not None and _feq(vb, -1.0):
            return self.neg(a)
        return self._push(_Node(DIV, args=(a, b), line=self.nodes[a].line))

    def substitute_literals(self, literal: list):
        for n in self.nodes:
            if n.kind == VAR and n.sym < len(literal) and literal[n.sym] is not None:
                n.kind, n.value, n.sym = NUM, float(literal[n.sym]), -1
        self._folds = []

    def folds(self) -> list:
        for i in range(len(self._folds), len(self.nodes)):
            self._folds.append(self._compute_fold(i))
        return self._folds

    def fold(self, i: int):
        return self.folds()[i]

    def _compute_fold(self, i: int):
        n = self.nodes[i]
        if n.kind == NUM:
            return n.value
        if n.kind == VAR:
            return None
        a = []
        for c in n.args:
            v = self._folds[c]
            if v is None:
                return None
            a.append(v)
        try:
            if n.kind == ADD:
                return a[0] + a[1]
            if n.kind == SUB:
                return a[0] - a[1]
            if n.kind == MUL:
                return a[0] * a[1]
            if n.kind == DIV:
                return None if _feq(a[1], 0.0) else a[0] / a[1]
            if n.kind == NEG:
                return -a[0]
        except OverflowError:
            return None
        if n.kind == CALL:
            return _fold_call(n.func, a)
        return None

    def contains_mask(self, sym: int) -> list:
        mask = []
        for n in self.nodes:
            found = n.kind == VAR and n.sym == sym
            if not found:
                for a in n.args:
                    if mask[a]:
                        found = True
                        break
            mask.append(found)
        return mask


# -- parser ----------------------------------------------------------------
@dataclass
class Symbol:
    name: str
    decl_line: int = 0
    lo: float = -INF
    up: float = INF
    fixed: bool = False
    fx: float = 0.0
    has_level: bool = False
    level: float = 0.0
    kind: int = A.VAR_CONTINUOUS
    integral_line: int = 0
    is_objvar: bool = False
    eliminated: bool = False


@dataclass
class Equation:
    name: str
    line: int
    rel: str = "e"
    lhs: int = -1
    rhs: int = -1
    consumed: bool = False


@dataclass
class Model:
    ast: Ast = field(default_factory=Ast)
    symbols: list = field(default_factory=list)
    symbol_index: dict = field(default_factory=dict)
    equations: list = field(default_factory=list)
    objvar: int = -1
    maximise: bool = False
    have_solve: bool = False


class _Parser:
    def __init__(self, tokens: list[Token], m: Model, warnings: list):
        self.t = tokens
        self.p = 0
        self.m = m
        self.warnings = warnings

    def cur(self) -> Token:
        return self.t[self.p]

    def peek(self, k: int = 1) -> Token:
        return self.t[min(self.p + k, len(self.t) - 1)]

    def advance(self):
        if self.p + 1 < len(self.t):
            self.p += 1

    def is_word(self, w: str) -> bool:
        return self.cur().kind == IDENT and self.cur().text == w

    def expect(self, k: int, what: str):
        if self.cur().kind != k:
            raise ParseError(self.cur().line, "expected " + what)
        self.advance()

    def skip_to_semi(self):
        while self.cur().kind not in (SEMI, END):
            self.advance()
        if self.cur().kind == SEMI:
            self.advance()

    def run(self):
        while self.cur().kind != END:
            self.statement()

    def statement(self):
        c = self.cur()
        if c.kind == SEMI:
            self.advance()
            return
        if c.kind != IDENT:
            raise ParseError(c.line, "expected the start of a statement")
        w = c.text
        if w in NON_SCALAR:
            raise ParseError(c.line, f"'{w}' means this file is not in GAMS scalar format; regenerate it with GAMS "
                                     "Convert", "non_scalar")
        if w in ("sos1", "sos2", "semicont", "semiint"):
            raise ParseError(c.line, f"'{w}' variables are not supported", "discrete")
        if w in ("free", "positive", "negative", "binary", "integer"):
            return self.declare_variables(w)
        if w in ("variables", "variable"):
            return self.declare_variables("free")
        if w in ("equations", "equation"):
            return self.declare_equations()
        if w in ("model", "models", "option", "options"):
            return self.skip_to_semi()
        if w == "solve":
            return self.solve_statement()
        if self.peek().kind == DOTDOT:
            return self.equation_definition()
        if self.peek().kind == DOT:
            return self.attribute_assignment()
        raise ParseError(c.line, f"unrecognised statement starting at '{w}'")

    def intern(self, name: str, line: int) -> int:
        if name in self.m.symbol_index:
            return self.m.symbol_index[name]
        self.m.symbols.append(Symbol(name, decl_line=line))
        idx = len(self.m.symbols) - 1
        self.m.symbol_index[name] = idx
        return idx

    def declare_variables(self, domain: str):
        line = self.cur().line
        self.advance()
        if self.is_word("variables") or self.is_word("variable"):
            self.advance()
        lo, up, kind = -INF, INF, A.VAR_CONTINUOUS
        if domain == "positive":
            lo = 0.0
        elif domain == "negative":
            up = 0.0
        elif domain == "binary":
            lo, up, kind = 0.0, 1.0, A.VAR_BINARY
        elif domain == "integer":
            lo, kind = 0.0, A.VAR_INTEGER
        while True:
            if self.cur().kind != IDENT:
                raise ParseError(self.cur().line, "variable name")
            s = self.m.symbols[self.intern(self.cur().text, line)]
            s.lo, s.up = lo, up
            if kind != A.VAR_CONTINUOUS:  # integrality is sticky across re-declarations
                s.kind = kind
                s.integral_line = line
            self.advance()
            if self.cur().kind == COMMA:
                self.advance()
                continue
            break
        self.expect(SEMI, "';' after a variable declaration")

    def declare_equations(self):
        self.advance()
        while True:
            if self.cur().kind != IDENT:
                raise ParseError(self.cur().line, "equation name")
            self.advance()
            if self.cur().kind == COMMA:
                self.advance()
                continue
            break
        self.expect(SEMI, "';' after an equation declaration")

    def equation_definition(self):
        eq = Equation(self.cur().text, self.cur().line)
        self.advance()
        self.expect(DOTDOT, "'..' after an equation name")
        eq.lhs = self.expression()
        if self.cur().kind != REL:
            raise ParseError(self.cur().line, "expected =E=, =L=, =G= or =N=")
        eq.rel = self.cur().rel
        self.advance()
        eq.rhs = self.expression()
        self.expect(SEMI, "';' after an equation definition")
        self.m.equations.append(eq)

    def attribute_assignment(self):
        line = self.cur().line
        name = self.cur().text
        self.advance()
        self.expect(DOT, "'.'")
        if self.cur().kind != IDENT:
            raise ParseError(line, "attribute name")
        attr = self.cur().text
        self.advance()
        idx = self.m.symbol_index.get(name)
        if idx is None or attr not in ("lo", "up", "fx", "l"):
            return self.skip_to_semi()  # model attributes, marginals, hints
        self.expect(ASSIGN, "'=' in an attribute assignment")
        value = self.m.ast.fold(self.expression())
        if value is None:
            raise ParseError(line, f"'{name}.{attr}' must be a constant")
        self.expect(SEMI, "';' after an attribute assignment")
        s = self.m.symbols[idx]
        if attr == "lo":
            s.lo = value
        elif attr == "up":
            s.up = value
        elif attr == "fx":
            s.fixed, s.fx = True, value
        else:
            s.has_level, s.level = True, value

    def solve_statement(self):
        line = self.cur().line
        while self.cur().kind not in (SEMI, END):
            if self.cur().kind == IDENT and self.cur().text in ("minimizing", "minimising", "maximizing", "maximising"):
                maximise = self.cur().text[1] == "a"
                self.advance()
                if self.cur().kind != IDENT:
                    raise ParseError(self.cur().line, "objective variable name after minimizing/maximizing")
                idx = self.m.symbol_index.get(self.cur().text)
                if idx is None:
                    raise ParseError(self.cur().line, f"undeclared objective variable '{self.cur().text}'")
                self.m.objvar = idx
                self.m.symbols[idx].is_objvar = True
                self.m.maximise = maximise
                self.m.have_solve = True
            self.advance()
        if self.cur().kind == SEMI:
            self.advance()
        if not self.m.have_solve:
            raise ParseError(line, "Solve statement names no objective (a feasibility-only model has no form in "
                                   "Problem)", "unrepresentable")

    # expressions: + - bind loosest, then * /, then unary sign, then **
    def expression(self) -> int:
        lhs = self.term()
        while self.cur().kind in (PLUS, MINUS):
            plus = self.cur().kind == PLUS
            self.advance()
            rhs = self.term()
            lhs = self.m.ast.add(lhs, rhs) if plus else self.m.ast.sub(lhs, rhs)
        return lhs

    def term(self) -> int:
        lhs = self.unary()
        while self.cur().kind in (STAR, SLASH):
            times = self.cur().kind == STAR
            self.advance()
            rhs = self.unary()
            lhs = self.m.ast.mul(lhs, rhs) if times else self.m.ast.div(lhs, rhs)
        return lhs

    def unary(self) -> int:
        if self.cur().kind == MINUS:
            self.advance()
            return self.m.ast.neg(self.unary())
        if self.cur().kind == PLUS:
            self.advance()
            return self.unary()
        return self.power()

    def power(self) -> int:
        base = self.atom()
        if self.cur().kind == POW:
            line = self.cur().line
            self.advance()
            exponent = self.unary()
            return self.m.ast.call("power", (base, exponent), line)
        return base

    def atom(self) -> int:
        c = self.cur()
        line = c.line
        if c.kind == NUMBER:
            self.advance()
            return self.m.ast.num(c.value, line)
        if c.kind == LPAREN:
            self.advance()
            inner = self.expression()
            self.expect(RPAREN, "')'")
            return inner
        if c.kind != IDENT:
            raise ParseError(line, "expected a number, identifier or '('")
        name = c.text
        if name == "inf":
            self.advance()
            return self.m.ast.num(INF, line)
        if name == "eps":
            self.advance()
            return self.m.ast.num(0.0, line)
        if name in ("na", "undf"):
            raise ParseError(line, f"the special value '{name}' cannot be represented", "unrepresentable")
        if self.peek().kind == LPAREN:
            f = FUNCS.get(name)
            if f is None:
                if name in UNSUPPORTED:
                    raise ParseError(line, f"function '{name}' is not supported yet", "unsupported_function")
                raise ParseError(line, f"unknown function '{name}'", "unsupported_function")
            self.advance()
            self.advance()
            args = [self.expression()]
            while self.cur().kind == COMMA:
                self.advance()
                args.append(self.expression())
            self.expect(RPAREN, "')' closing a function call")
            return self.build_call(f, args, line)
        idx = self.m.symbol_index.get(name)
        if idx is None:
            raise ParseError(line, f"undeclared identifier '{name}'")
        self.advance()
        return self.m.ast.var(idx, line)

    def build_call(self, f: str, args: list, line: int) -> int:
        if f in ("min", "max"):
            acc = args[0]
            for a in args[1:]:
                acc = self.m.ast.call(f, (acc, a), line)
            return acc
        if len(args) != (2 if f == "power" else 1):
            raise ParseError(line, "wrong number of arguments to this function")
        return self.m.ast.call(f, args, line)


# -- objective elimination --------------------------------------------------
def _split(ast: Ast, root: int, sym: int):
    """`node` as coeff * sym + rem, rem free of sym; None when not linear."""
    contains = ast.contains_mask(sym)
    table: list = [None] * (root + 1)
    for i in range(root + 1):
        if not contains[i]:
            table[i] = (0.0, i)
            continue
        n = ast.nodes[i]
        kind, args = n.kind, n.args
        if kind == VAR:
            table[i] = (1.0, ast.num(0.0))
        elif kind == NEG:
            a = table[args[0]]
            if a is not None:
                table[i] = (-a[0], ast.neg(a[1]))
        elif kind in (ADD, SUB):
            a, b = table[args[0]], table[args[1]]
            if a is not None and b is not None:
                table[i] = (a[0] + b[0], ast.add(a[1], b[1])) if kind == ADD else (a[0] - b[0], ast.sub(a[1], b[1]))
        elif kind == MUL:
            other = 1 if contains[args[0]] else 0
            if contains[args[other]]:
                continue
            k = ast.fold(args[other])
            if k is None:
                continue
            a = table[args[1 - other]]
            if a is not None:
                table[i] = (k * a[0], ast.mul(args[other], a[1]))
        elif kind == DIV:
            if contains[args[1]]:
                continue
            k = ast.fold(args[1])
            if k is None or _feq(k, 0.0):
                continue
            a = table[args[0]]
            if a is not None:
                table[i] = (a[0] / k, ast.div(a[1], args[1]))
        # anything under a function call is nonlinear in sym: stays None
    return table[root]


def _eliminate_objective(m: Model, warnings: list):
    """(objective AST index or None, from_inequality)."""
    objective, candidates = None, 0
    for eq in m.equations:
        if eq.rel != "e":
            continue
        mask = m.ast.contains_mask(m.objvar)
        if not mask[eq.lhs] and not mask[eq.rhs]:
            continue
        lhs, rhs = _split(m.ast, eq.lhs, m.objvar), _split(m.ast, eq.rhs, m.objvar)
        if lhs is None or rhs is None:
            continue
        coeff = lhs[0] - rhs[0]
        if math.fabs(coeff) < 1e-12:
            continue
        candidates += 1
        if objective is not None:
            continue
        objective = m.ast.div(m.ast.sub(rhs[1], lhs[1]), m.ast.num(coeff))
        eq.consumed = True
    if candidates > 1:
        warnings.append((0, "several equations define the objective variable; used the first"))
    if objective is not None:
        return objective, False
    for i, eq in enumerate(m.equations):
        if eq.rel not in ("l", "g"):
            continue
        mask = m.ast.contains_mask(m.objvar)
        if not mask[eq.lhs] and not mask[eq.rhs]:
            continue
        lhs, rhs = _split(m.ast, eq.lhs, m.objvar), _split(m.ast, eq.rhs, m.objvar)
        if lhs is None or rhs is None:
            continue
        coeff = lhs[0] - rhs[0]
        if math.fabs(coeff) < 1e-12:
            continue
        below = (eq.rel == "l") == (coeff < 0.0)
        if below == m.maximise:
            continue
        mask = m.ast.contains_mask(m.objvar)
        if any(j != i and e.rel != "n" and (mask[e.lhs] or mask[e.rhs]) for j, e in enumerate(m.equations)):
            continue
        out = m.ast.div(m.ast.sub(rhs[1], lhs[1]), m.ast.num(coeff))
        eq.consumed = True
        warnings.append((eq.line, f"'{m.symbols[m.objvar].name}' is defined by the inequality '{eq.name}', which is "
                                  "tight at every optimum; substituted it away rather than spending a search "
                                  "dimension on it"))
        return out, True
    return None, False


# -- lowering ---------------------------------------------------------------
@dataclass
class ParsedModel:
    problem: Problem
    sense: str = "min"
    var_names: list = field(default_factory=list)
    constraint_names: list = field(default_factory=list)
    initial_point: list = field(default_factory=list)
    warnings: list = field(default_factory=list)
    objvar_kept: bool = False


class _Lowerer:
    def __init__(self, m: Model, default_bound: float, fold_fixed: bool, out: ParsedModel):
        self.m = m
        self.default_bound = default_bound
        self.fold_fixed = fold_fixed
        self.out = out
        self.g = out.problem.graph
        self.sym_node = [None] * len(m.symbols)
        self.memo: list = []
        self.objective_expr_root = 0

    def warn(self, line, msg):
        self.out.warnings.append((line, msg))

    def create_variables(self):
        any_level = any(s.has_level for s in self.m.symbols)
        for i, s in enumerate(self.m.symbols):
            if s.eliminated or (s.fixed and self.fold_fixed):
                continue
            lo = s.fx if s.fixed else s.lo
            up = s.fx if s.fixed else s.up
            discrete = s.kind != A.VAR_CONTINUOUS
            lo_def, up_def = not math.isfinite(lo), not math.isfinite(up)
            if lo_def:
                lo = -self.default_bound
            if up_def:
                up = self.default_bound
            if discrete:
                lo, up = float(math.ceil(lo)), float(math.floor(up))
            if lo > up:
                raise ParseError(s.decl_line, f"'{s.name}' has an empty box")
            suffix = f" (integer domain size {up - lo + 1.0:f})" if discrete else ""
            if lo_def:
                self.warn(s.decl_line, f"'{s.name}' has no lower bound; using {lo:f}{suffix}")
            if up_def:
                self.warn(s.decl_line, f"'{s.name}' has no upper bound; using {up:f}{suffix}")
            kind = s.kind
            if kind == A.VAR_BINARY and (lo != 0.0 or up != 1.0):
                kind = A.VAR_INTEGER
            self.sym_node[i] = self.out.problem.var(lo, up, kind).id
            self.out.var_names.append(s.name)
            if any_level:
                start = s.level if s.has_level else min(max(0.0, lo), up)
                self.out.initial_point.append(min(max(start, lo), up))

    def set_objective(self, objective_ast: int):
        self.emit_roots([objective_ast])
        root = self.memo[objective_ast]
        if self.g.nodes[root].op == A.OP_CONST:
            raise ParseError(0, "the objective is constant", "unrepresentable")
        self.objective_expr_root = root
        if self.m.maximise:
            root = self.g.emit(A.OP_NEG, (root,))
            self.out.sense = "max"
        if self.m.objvar >= 0:
            self.sym_node[self.m.objvar] = self.objective_expr_root
        self.out.problem.set_objective(Expr(self.g, root))

    def add_constraints(self):
        pending, roots = [], []
        for eq in self.m.equations:
            if eq.consumed:
                continue
            if eq.rel == "n":
                self.warn(eq.line, f"'{eq.name}' is a =N= equation and asserts nothing; dropped")
                continue
            lhs, rhs = eq.lhs, eq.rhs
            cmp = A.CMP_EQ if eq.rel == "e" else A.CMP_LE
            if eq.rel == "g":
                lhs, rhs = rhs, lhs
            lc, rc = self.m.ast.fold(lhs), self.m.ast.fold(rhs)
            if lc is not None and rc is not None:
                holds = _feq(lc, rc) if cmp == A.CMP_EQ else lc <= rc
                self.warn(eq.line, f"'{eq.name}' has no variables and is "
                                   + ("trivially satisfied; dropped" if holds
                                      else "VIOLATED -- the model as written is infeasible"))
                continue
            roots.append(lhs)
            if rc is not None:
                pending.append((eq.name, cmp, lhs, -1, rc))
            else:
                roots.append(rhs)
                pending.append((eq.name, cmp, lhs, rhs, 0.0))
        self.emit_roots(roots)
        for name, cmp, lhs, rhs, bound in pending:
            lid = self.memo[lhs]
            root = lid if rhs < 0 else self.emit_binary(A.OP_SUB, lid, self.memo[rhs])
            self.out.problem.add_constraint(Expr(self.g, root), cmp, bound)
            self.out.constraint_names.append(name)

    def add_objective_variable_bounds(self, from_inequality: bool):
        if self.m.objvar < 0:
            return
        s = self.m.symbols[self.m.objvar]
        if not s.eliminated:
            return
        drop_lower = from_inequality and not self.m.maximise
        drop_upper = from_inequality and self.m.maximise
        if math.isfinite(s.up) and not drop_upper:
            self.out.problem.add_constraint(Expr(self.g, self.objective_expr_root), A.CMP_LE, s.up)
            self.out.constraint_names.append(s.name + ".up")
        if math.isfinite(s.lo) and not drop_lower:
            neg = self.g.emit(A.OP_NEG, (self.objective_expr_root,))
            self.out.problem.add_constraint(Expr(self.g, neg), A.CMP_LE, -s.lo)
            self.out.constraint_names.append(s.name + ".lo")
        for drop, attr in ((drop_lower and math.isfinite(s.lo), "lo"), (drop_upper and math.isfinite(s.up), "up")):
            if drop:
                self.warn(s.decl_line, f"'{s.name}.{attr}' constrains only the objective variable, which was "
                                       "substituted away; dropped")

    # DAG emission: mark live nodes backwards from the roots, emit forwards
    def emit_const(self, v: float) -> int:
        return self.g.emit(A.OP_CONST, (), constant=v)

    def emit_binary(self, op: int, a: int, b: int) -> int:
        if op == A.OP_MUL and a == b:
            return self.g.emit(A.OP_SQR, (a,))
        return self.g.emit(op, (a, b))

    def emit_roots(self, roots: list):
        if not roots:
            return
        top = max(roots)
        folds = self.m.ast.folds()
        live = [False] * (top + 1)
        for r in roots:
            live[r] = True
        for i in range(top, -1, -1):
            if not live[i] or folds[i] is not None:
                continue
            n = self.m.ast.nodes[i]
            k = 1 if (n.kind == CALL and n.func == "power" and folds[n.args[1]] is not None) else len(n.args)
            for a in n.args[:k]:
                live[a] = True
        if len(self.memo) < len(self.m.ast.nodes):
            self.memo.extend([None] * (len(self.m.ast.nodes) - len(self.memo)))
        for i in range(top + 1):
            if live[i] and self.memo[i] is None:
                self.memo[i] = self.emit_node(i)

    def emit_node(self, i: int) -> int:
        v = self.m.ast.fold(i)
        if v is not None:
            return self.emit_const(v)
        n = self.m.ast.nodes[i]

        def ins(k):
            return self.memo[n.args[k]]

        if n.kind == VAR:
            nid = self.sym_node[n.sym]
            if nid is None:
                raise ParseError(n.line, f"'{self.m.symbols[n.sym].name}' is used but has no value", "unrepresentable")
            return nid
        if n.kind == ADD:
            return self.emit_binary(A.OP_ADD, ins(0), ins(1))
        if n.kind == SUB:
            return self.emit_binary(A.OP_SUB, ins(0), ins(1))
        if n.kind == MUL:
            return self.emit_binary(A.OP_MUL, ins(0), ins(1))
        if n.kind == DIV:
            return self.emit_binary(A.OP_DIV, ins(0), ins(1))
        if n.kind == NEG:
            return self.g.emit(A.OP_NEG, (ins(0),))
        return self.emit_call(n, ins)

    def emit_call(self, n: _Node, ins) -> int:
        f = n.func
        unary = {"sqr": A.OP_SQR, "sqrt": A.OP_SQRT, "exp": A.OP_EXP, "log": A.OP_LOG, "abs": A.OP_ABS,
                 "sin": A.OP_SIN, "cos": A.OP_COS, "tanh": A.OP_TANH}
        if f in unary:
            return self.g.emit(unary[f], (ins(0),))
        if f in ("log10", "log2"):
            lg = self.g.emit(A.OP_LOG, (ins(0),))
            scale = 1.0 / (math.log(10.0) if f == "log10" else math.log(2.0))
            return self.emit_binary(A.OP_MUL, lg, self.emit_const(scale))
        if f in ("min", "max"):
            return self.emit_binary(A.OP_MIN if f == "min" else A.OP_MAX, ins(0), ins(1))
        # power
        e = self.m.ast.fold(n.args[1])
        if e is None:
            lb = self.g.emit(A.OP_LOG, (ins(0),))
            return self.g.emit(A.OP_EXP, (self.emit_binary(A.OP_MUL, lb, ins(1)),))
        if _feq(e, 0.5):
            return self.g.emit(A.OP_SQRT, (ins(0),))
        if not (math.floor(e) < e) and math.fabs(e) <= 1e9:
            return self.g.emit(A.OP_POWN, (ins(0),), int_exp=int(e))
        lb = self.g.emit(A.OP_LOG, (ins(0),))
        return self.g.emit(A.OP_EXP, (self.emit_binary(A.OP_MUL, lb, self.emit_const(e)),))


def parse(source: str, default_bound: float = 1e6, fold_fixed_to_const: bool = True,
          reject_discrete: bool = False) -> ParsedModel:
    """Parses GAMS scalar source (gams.hpp:102-133 parse)."""
    out = ParsedModel(Problem())
    m = Model()
    _Parser(lex(source), m, out.warnings).run()
    if not m.have_solve:
        raise ParseError(0, "the file has no Solve statement", "unrepresentable")
    if reject_discrete:
        for s in m.symbols:
            if s.kind != A.VAR_CONTINUOUS:
                raise ParseError(s.integral_line, f"'{s.name}' is discrete; reject_discrete is set", "discrete")
    if fold_fixed_to_const:
        literal = [s.fx if (s.fixed and i != m.objvar) else None for i, s in enumerate(m.symbols)]
        if any(v is not None for v in literal):
            m.ast.substitute_literals(literal)
    expr, from_ineq = _eliminate_objective(m, out.warnings)
    out.objvar_kept = expr is None
    if expr is not None:
        m.symbols[m.objvar].eliminated = True
    else:
        out.warnings.append((0, f"could not solve any equation for '{m.symbols[m.objvar].name}'; keeping it as a "
                                "variable, which costs one search dimension"))
        expr = m.ast.var(m.objvar, 0)
    low = _Lowerer(m, default_bound, fold_fixed_to_const, out)
    low.create_variables()
    low.set_objective(expr)
    low.add_constraints()
    low.add_objective_variable_bounds(from_ineq)
    try:
        out.problem.validate()
    except Exception as e:  # a frontend bug, not malformed input
        raise ParseError(0, str(e), "unrepresentable") from e
    return out


def parse_file(path, **options) -> ParsedModel:
    try:
        with open(path, encoding="utf-8", errors="replace") as f:
            src = f.read()
    except OSError as e:
        raise ParseError(0, f"cannot open '{path}'", "io") from e
    return parse(src, **options)
