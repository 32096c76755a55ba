"""Parser of the prtcl scheme language (``.prtcl`` files).

The language is the reference's (grammar: lua/prtcl/parser/grammar.lua;
sources: share/schemes/*.prtcl).  A file holds schemes; a scheme declares
groups (a selector over group types and tags plus the fields they carry),
global fields and procedures.  Procedure bodies are loops over the
particles of a group, over their neighbours and over the dimensions, with
``local``, ``compute`` and ``reduce`` statements, and ``solve pcg`` blocks.

Expressions fold left: ``a * b / c`` is ``((a * b) / c)`` and ``a - b + c``
is ``((a - b) + c)``, exactly as the reference's generator parenthesises
them, so the generated arithmetic has the reference's operation order.

The result is a tree of the dataclasses below; ``resolve`` (in
``prtcl_gb300.dsl.check``) binds names to their definitions.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import List, Optional, Tuple, Union


class DslError(Exception):
    """A syntax or semantic error, with the source position when known."""


# ---------------------------------------------------------------------------
# tree
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class NDType:
    """``real``, ``integer`` or ``boolean`` with zero to two extents; an
    empty extent (``real[]``) is the dimensionality N."""
    base: str
    extents: Tuple[int, ...] = ()

    @property
    def rank(self):
        return len(self.extents)

    def __str__(self):
        return self.base + "".join(f"[{e or ''}]" for e in self.extents)


@dataclass
class Select:
    kind: str  # "type" or "tag"
    name: str


@dataclass
class SelNot:
    operand: "SelExpr"


@dataclass
class SelAnd:
    operands: List["SelExpr"]


@dataclass
class SelOr:
    operands: List["SelExpr"]


SelExpr = Union[Select, SelNot, SelAnd, SelOr]


@dataclass
class FieldDef:
    kind: str  # "uniform", "varying" or "global"
    alias: str
    type: NDType
    name: str
    pos: int = 0


@dataclass
class Groups:
    name: str
    select: SelExpr
    fields: List[FieldDef]
    pos: int = 0


# expressions

@dataclass
class Literal:
    text: str
    pos: int = 0


@dataclass
class NameRef:
    name: str
    pos: int = 0
    ref: object = None  # LocalDef, FieldDef (global) or a loop (dimension index)


@dataclass
class FieldAccess:
    name: str
    frm: str
    pos: int = 0
    ref: object = None   # FieldDef
    loop: object = None  # the particle / neighbour loop or solve that binds `frm`


@dataclass
class Call:
    name: str
    type: Optional[NDType]
    args: List["Expr"]
    pos: int = 0


@dataclass
class BinOp:
    op: str
    lhs: "Expr"
    rhs: "Expr"
    pos: int = 0


@dataclass
class Neg:
    operand: "Expr"
    pos: int = 0


@dataclass
class Slice:
    subject: "Expr"
    indices: List[Union[str, NameRef]]
    pos: int = 0


Expr = Union[Literal, NameRef, FieldAccess, Call, BinOp, Neg, Slice]


# statements

@dataclass
class LocalDef:
    name: str
    type: NDType
    init: Expr
    pos: int = 0


@dataclass
class Compute:
    target: Expr
    op: str
    arg: Expr
    pos: int = 0


@dataclass
class Reduce:
    target: Expr
    op: str
    arg: Expr
    pos: int = 0


@dataclass
class ForeachParticle:
    groups: str
    index: str
    body: list
    pos: int = 0


@dataclass
class ForeachNeighbor:
    groups: Optional[str]  # None: the particle's own groups (`_`)
    index: str
    body: list
    pos: int = 0


@dataclass
class ForeachDimension:
    index: str
    body: list
    pos: int = 0


@dataclass
class SolveSetup:
    name: str   # "right_hand_side" or "guess"
    into: str
    body: list
    pos: int = 0


@dataclass
class SolveProduct:
    name: str   # "system" or "preconditioner"
    with_: str
    into: str
    body: list
    pos: int = 0


@dataclass
class SolveApply:
    with_: str
    body: list
    pos: int = 0


@dataclass
class Solve:
    solver: str
    type: NDType
    groups: str
    index: str
    parts: list
    pos: int = 0


@dataclass
class Procedure:
    name: str
    body: list
    pos: int = 0


@dataclass
class Scheme:
    name: str
    groups: List[Groups] = field(default_factory=list)
    globals: List[FieldDef] = field(default_factory=list)
    procedures: List[Procedure] = field(default_factory=list)
    source: str = ""
    pos: int = 0


# ---------------------------------------------------------------------------
# tokens
# ---------------------------------------------------------------------------

_TOKEN = re.compile(r"""
    (?P<ws>\s+|//[^\n]*|/\*.*?\*/)
  | (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?)
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op>\+=|-=|\*=|/=|[{}()\[\];:,.<>=+\-*/])
""", re.S | re.X)


@dataclass
class Tok:
    kind: str  # "num", "id", "op", "eof"
    text: str
    pos: int


def tokenize(src: str) -> List[Tok]:
    out, i = [], 0
    while i < len(src):
        m = _TOKEN.match(src, i)
        if not m:
            raise DslError(f"unexpected character {src[i]!r} at {_where(src, i)}")
        if m.lastgroup != "ws":
            out.append(Tok(m.lastgroup, m.group(), i))
        i = m.end()
    out.append(Tok("eof", "", len(src)))
    return out


def _where(src, pos):
    line = src.count("\n", 0, pos) + 1
    col = pos - (src.rfind("\n", 0, pos) + 1) + 1
    return f"line {line} column {col}"


# ---------------------------------------------------------------------------
# parser
# ---------------------------------------------------------------------------

_COMPUTE_OPS = ("=", "+=", "-=", "*=", "/=", "min=", "max=")
_REDUCE_OPS = ("+=", "-=", "*=", "min=", "max=")


class _Parser:
    def __init__(self, src):
        self.src = src
        self.toks = tokenize(src)
        self.i = 0

    # -- helpers
    @property
    def tok(self):
        return self.toks[self.i]

    def peek(self, k=1):
        return self.toks[min(self.i + k, len(self.toks) - 1)]

    def error(self, msg, tok=None):
        tok = tok or self.tok
        got = tok.text or "end of input"
        raise DslError(f"{msg} at {_where(self.src, tok.pos)} (found {got!r})")

    def accept(self, text, kind=None):
        t = self.tok
        if t.text == text and (kind is None or t.kind == kind):
            self.i += 1
            return t
        return None

    def expect(self, text, what=None):
        t = self.accept(text)
        if t is None:
            self.error(f"expected {what or repr(text)}")
        return t

    def word(self, w):
        t = self.tok
        if t.kind == "id" and t.text == w:
            self.i += 1
            return t
        self.error(f"expected {w!r}")

    def name(self):
        t = self.tok
        if t.kind != "id":
            self.error("expected a name")
        self.i += 1
        return t.text

    def is_word(self, w, k=0):
        t = self.peek(k) if k else self.tok
        return t.kind == "id" and t.text == w

    # -- file
    def parse_file(self):
        schemes = []
        while self.tok.kind != "eof":
            schemes.append(self.scheme())
        if not schemes:
            self.error("expected 'scheme'")
        return schemes

    def scheme(self):
        start = self.word("scheme").pos
        s = Scheme(self.name(), pos=start)
        self.expect("{")
        while not self.accept("}"):
            if self.is_word("groups"):
                s.groups.append(self.groups())
            elif self.is_word("global"):
                s.globals.extend(self.global_block())
            elif self.is_word("procedure"):
                s.procedures.append(self.procedure())
            else:
                self.error("expected 'groups', 'global' or 'procedure'")
        s.source = self.src[start:self.toks[self.i - 1].pos + 1]
        return s

    def groups(self):
        pos = self.word("groups").pos
        name = self.name()
        self.expect("{")
        self.word("select")
        sel = self.select_or()
        self.expect(";")
        fields = []
        while not self.accept("}"):
            t = self.tok
            kind = t.text if t.kind == "id" and t.text in ("uniform", "varying") else None
            if kind is None:
                self.error("expected 'uniform' or 'varying'")
            self.i += 1
            fields.append(self.field_rest(kind, t.pos))
        return Groups(name, sel, fields, pos)

    def select_or(self):
        ops = [self.select_and()]
        while self.is_word("or"):
            self.i += 1
            ops.append(self.select_and())
        return ops[0] if len(ops) == 1 else SelOr(ops)

    def select_and(self):
        ops = [self.select_not()]
        while self.is_word("and"):
            self.i += 1
            ops.append(self.select_not())
        return ops[0] if len(ops) == 1 else SelAnd(ops)

    def select_not(self):
        if self.is_word("not"):
            self.i += 1
            return SelNot(self.select_atom())
        return self.select_atom()

    def select_atom(self):
        if self.accept("("):
            e = self.select_or()
            self.expect(")")
            return e
        if self.is_word("type") or self.is_word("tag"):
            kind = self.tok.text
            self.i += 1
            return Select(kind, self.name())
        self.error("expected 'type', 'tag' or '('")

    def field_rest(self, kind, pos):
        self.word("field")
        alias = self.name()
        self.expect("=")
        ty = self.ndtype()
        name = self.name()
        self.expect(";")
        return FieldDef(kind, alias, ty, name, pos)

    def global_block(self):
        self.word("global")
        self.expect("{")
        out = []
        while not self.accept("}"):
            pos = self.tok.pos
            out.append(self.field_rest("global", pos))
        return out

    def ndtype(self):
        t = self.tok
        if not (t.kind == "id" and t.text in ("real", "integer", "boolean")):
            self.error("expected a type ('real', 'integer' or 'boolean')")
        self.i += 1
        ext = []
        while self.accept("["):
            if self.tok.kind == "num":
                ext.append(int(self.tok.text))
                self.i += 1
            else:
                ext.append(0)
            self.expect("]")
        return NDType(t.text, tuple(ext))

    # -- statements
    def procedure(self):
        pos = self.word("procedure").pos
        name = self.name()
        return Procedure(name, self.block(("local", "compute", "foreach_dim", "foreach_particle", "solve")), pos)

    def block(self, allowed):
        self.expect("{")
        body = []
        while not self.accept("}"):
            body.append(self.statement(allowed))
        return body

    def statement(self, allowed):
        t = self.tok
        if t.kind != "id":
            self.error("expected a statement")
        if t.text == "local" and "local" in allowed:
            return self.local_def()
        if t.text == "compute" and "compute" in allowed:
            return self.compute_like(Compute, _COMPUTE_OPS)
        if t.text == "reduce" and "reduce" in allowed:
            return self.compute_like(Reduce, _REDUCE_OPS)
        if t.text == "solve" and "solve" in allowed:
            return self.solve()
        if t.text == "foreach":
            nxt = self.peek()
            if nxt.kind == "id" and nxt.text == "dimension" and "foreach_dim" in allowed:
                return self.foreach_dimension()
            if "foreach_particle" in allowed and self.peek(2).text == "particle":
                return self.foreach_particle()
            if "foreach_neighbor" in allowed and self.peek(2).text == "neighbor":
                return self.foreach_neighbor()
        self.error("unexpected statement")

    def local_def(self):
        pos = self.word("local").pos
        name = self.name()
        self.expect(":")
        ty = self.ndtype()
        self.expect("=")
        e = self.expr()
        self.expect(";")
        return LocalDef(name, ty, e, pos)

    def compute_like(self, cls, ops):
        pos = self.tok.pos
        self.i += 1
        target = self.expr()
        op = self.assign_op(ops)
        arg = self.expr()
        self.expect(";")
        return cls(target, op, arg, pos)

    def assign_op(self, ops):
        t = self.tok
        if t.kind == "op" and t.text in ops:
            self.i += 1
            return t.text
        if t.kind == "id" and t.text in ("min", "max") and self.peek().text == "=" \
                and t.text + "=" in ops:
            self.i += 2
            return t.text + "="
        self.error("expected one of " + ", ".join(ops))

    def foreach_dimension(self):
        pos = self.word("foreach").pos
        self.word("dimension")
        self.word("index")
        idx = self.name()
        return ForeachDimension(idx, self.block(("local", "compute", "foreach_particle", "solve")), pos)

    def foreach_particle(self):
        pos = self.word("foreach").pos
        groups = self.name()
        self.word("particle")
        idx = self.name()
        return ForeachParticle(groups, idx, self.block(("local", "reduce", "compute", "foreach_neighbor")), pos)

    def foreach_neighbor(self):
        pos = self.word("foreach").pos
        groups = self.name()
        self.word("neighbor")
        idx = self.name()
        return ForeachNeighbor(None if groups == "_" else groups, idx,
                               self.block(("local", "reduce", "compute")), pos)

    def solve(self):
        pos = self.word("solve").pos
        solver = self.name()
        ty = self.ndtype()
        self.word("over")
        groups = self.name()
        self.word("particle")
        idx = self.name()
        self.expect("{")
        parts = []
        inner = ("local", "compute", "foreach_neighbor")
        while not self.accept("}"):
            t = self.tok
            if self.is_word("setup"):
                self.i += 1
                name = self.name()
                self.word("into")
                into = self.name()
                parts.append(SolveSetup(name, into, self.block(inner), t.pos))
            elif self.is_word("product"):
                self.i += 1
                name = self.name()
                self.word("with")
                w = self.name()
                self.word("into")
                into = self.name()
                parts.append(SolveProduct(name, w, into, self.block(inner), t.pos))
            elif self.is_word("apply"):
                self.i += 1
                w = self.name()
                parts.append(SolveApply(w, self.block(inner), t.pos))
            else:
                self.error("expected 'setup', 'product' or 'apply'")
        return Solve(solver, ty, groups, idx, parts, pos)

    # -- expressions (left folds, as the reference's generator brackets them)
    def expr(self):
        e = self.term()
        while self.tok.kind == "op" and self.tok.text in ("+", "-"):
            t = self.tok
            self.i += 1
            e = BinOp(t.text, e, self.term(), t.pos)
        return e

    def term(self):
        e = self.unary()
        while self.tok.kind == "op" and self.tok.text in ("*", "/"):
            t = self.tok
            self.i += 1
            e = BinOp(t.text, e, self.unary(), t.pos)
        return e

    def unary(self):
        t = self.accept("-", "op")
        if t:
            return Neg(self.slice(), t.pos)
        return self.slice()

    def slice(self):
        e = self.atom()
        if self.tok.text == "[" and self.tok.kind == "op":
            pos = self.tok.pos
            self.i += 1
            idx = [self.slice_index()]
            while self.accept(","):
                idx.append(self.slice_index())
            self.expect("]")
            e = Slice(e, idx, pos)
        return e

    def slice_index(self):
        t = self.tok
        if t.kind == "num":
            self.i += 1
            return t.text
        if t.kind == "id":
            self.i += 1
            return NameRef(t.text, t.pos)
        self.error("expected an index")

    def atom(self):
        t = self.tok
        if t.kind == "num":
            self.i += 1
            return Literal(t.text, t.pos)
        if t.kind == "op" and t.text == "(":
            self.i += 1
            e = self.expr()
            self.expect(")")
            return e
        if t.kind != "id":
            self.error("expected an expression")
        self.i += 1
        if self.tok.text == "." and self.tok.kind == "op":
            self.i += 1
            return FieldAccess(t.text, self.name(), t.pos)
        ty = None
        if self.tok.text == "<" and self.tok.kind == "op":
            self.i += 1
            ty = self.ndtype()
            self.expect(">")
            if self.tok.text != "(":
                self.error("expected '(' after a type argument")
        if self.tok.text == "(" and self.tok.kind == "op":
            self.i += 1
            args = []
            if not self.accept(")"):
                args.append(self.expr())
                while self.accept(","):
                    args.append(self.expr())
                self.expect(")")
            return Call(t.text, ty, args, t.pos)
        return NameRef(t.text, t.pos)


def parse(source: str) -> List[Scheme]:
    """All schemes of a ``.prtcl`` source text."""
    return _Parser(source).parse_file()


def parse_one(source: str, name: Optional[str] = None) -> Scheme:
    schemes = parse(source)
    if name is None:
        if len(schemes) != 1:
            raise DslError(f"the source holds {len(schemes)} schemes; name one")
        return schemes[0]
    for s in schemes:
        if s.name == name:
            return s
    raise DslError(f"no scheme {name!r} in the source")
