"""Name resolution and type inference for parsed schemes.

``resolve(scheme)`` binds every name of the scheme's procedures to its
definition and infers the type of every expression, following the
reference's resolver and generator (lua/prtcl/pst_to_ast.lua,
lua/prtcl/generate/cxx_openmp_impl_hpp.lua):

* ``x.f`` is the field with alias ``x`` of the groups that the loop binding
  ``f`` runs over: a particle loop, a neighbour loop (``_`` = the particle's
  own groups) or a ``solve`` (its ``into`` / ``with`` names then denote the
  solver's per-particle vectors).
* A bare name is a ``local`` (innermost first), a dimension index or a
  global field.
* ``reduce`` may target a global field or a local declared outside the
  particle loop only.

Locals declared outside every particle loop are procedure-level: the
generated code keeps them in device memory between the kernels of the
procedure.  Locals inside a particle loop live in registers.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional

from .parser import (BinOp, Call, Compute, DslError, FieldAccess, FieldDef, ForeachDimension, ForeachNeighbor,
                     ForeachParticle, Groups, Literal, LocalDef, NameRef, NDType, Neg, Procedure, Reduce, Scheme,
                     Slice, Solve, SolveApply, SolveProduct, SolveSetup)

REAL = NDType("real")
INTEGER = NDType("integer")
BOOLEAN = NDType("boolean")
VEC = NDType("real", (0,))
MAT = NDType("real", (0, 0))
N = 3  # dimensionality of the generated schemes (the reference's N = 3 build)


def norm_type(t: NDType) -> NDType:
    """Extents written as N (``real[3]``) are the same as ``real[]``."""
    return NDType(t.base, tuple(0 if e in (0, N) else e for e in t.extents))


@dataclass
class SolveRef:
    """``into`` / ``with`` vector of the enclosing solve part."""
    kind: str      # "into" or "with"
    solve: Solve


@dataclass
class Info:
    """What resolution learns about a scheme."""
    types: Dict[int, NDType] = field(default_factory=dict)        # id(expr) -> type
    frame_locals: Dict[int, int] = field(default_factory=dict)    # id(LocalDef) -> frame slot
    frame_slots: int = 0
    loops: List[object] = field(default_factory=list)            # particle loops and solves, in order
    reductions: Dict[int, List[Reduce]] = field(default_factory=dict)  # id(loop) -> its reduces
    uses_neighbors: Dict[int, bool] = field(default_factory=dict)


KNOWN_CALLS = {
    "kernel_h", "kernel_gradient_h", "kernel_support_radius", "dot", "norm", "norm_squared", "cabs", "max", "min",
    "reciprocal_or_zero", "unit_step_l", "unit_step_r", "outer_product", "transpose", "trace", "invert", "invert_pm",
    "smoothstep", "cross_product_matrix_from_vector", "vector_from_cross_product_matrix", "zeros", "ones",
    "identity", "positive_infinity", "negative_infinity", "aat13_cohesion_h", "aat13_adhesion_h",
}
TYPED_CALLS = {"zeros", "ones", "identity", "positive_infinity", "negative_infinity"}


class _Scope:
    def __init__(self, parent=None, loop=None):
        self.parent = parent
        self.loop = loop          # binding node when this scope is a loop body
        self.locals: Dict[str, LocalDef] = {}


class Resolver:
    def __init__(self, scheme: Scheme):
        self.s = scheme
        self.groups: Dict[str, Groups] = {}
        for g in scheme.groups:
            if g.name in self.groups:
                self.fail(f"groups {g.name!r} declared twice", g)
            names = set()
            for f in g.fields:
                if f.alias in names:
                    self.fail(f"field alias {f.alias!r} declared twice in groups {g.name!r}", f)
                names.add(f.alias)
            self.groups[g.name] = g
        self.globals: Dict[str, FieldDef] = {}
        for f in scheme.globals:
            if f.alias in self.globals:
                self.fail(f"global field alias {f.alias!r} declared twice", f)
            self.globals[f.alias] = f
        self.info = Info()

    def fail(self, msg, node=None):
        where = ""
        if node is not None and getattr(node, "pos", None) is not None and self.s.source:
            # positions are offsets in the file; report the scheme-relative line
            pos = max(0, node.pos - self.s.pos)
            line = self.s.source.count("\n", 0, pos) + 1
            where = f" (scheme {self.s.name}, line {line})"
        raise DslError(msg + where)

    # -- scopes
    def lookup_local(self, scope, name):
        while scope is not None:
            if name in scope.locals:
                return scope.locals[name]
            scope = scope.parent
        return None

    def binding(self, scope, name):
        while scope is not None:
            lp = scope.loop
            if isinstance(lp, (ForeachParticle, ForeachNeighbor, Solve)) and lp.index == name:
                return lp, scope
            if isinstance(lp, ForeachDimension) and lp.index == name:
                return lp, scope
            scope = scope.parent
        return None, None

    def enclosing(self, scope, cls):
        while scope is not None:
            if isinstance(scope.loop, cls):
                return scope.loop
            scope = scope.parent
        return None

    def in_particle_loop(self, scope):
        return self.enclosing(scope, (ForeachParticle, Solve)) is not None

    # -- procedures
    def run(self):
        names = set()
        for p in self.s.procedures:
            if p.name in names:
                self.fail(f"procedure {p.name!r} declared twice", p)
            names.add(p.name)
            self.block(p.body, _Scope())
        return self.info

    def block(self, body, scope):
        for st in body:
            self.statement(st, scope)

    def statement(self, st, scope):
        if isinstance(st, LocalDef):
            t = self.expr(st.init, scope)
            want = norm_type(st.type)
            if not assignable(want, t):
                self.fail(f"local {st.name!r} of type {want} initialised with {t}", st)
            if st.name in scope.locals:
                self.fail(f"local {st.name!r} declared twice", st)
            scope.locals[st.name] = st
            if not self.in_particle_loop(scope):
                self.info.frame_locals[id(st)] = self.info.frame_slots
                self.info.frame_slots += 1
        elif isinstance(st, (Compute, Reduce)):
            tt = self.expr(st.target, scope)
            at = self.expr(st.arg, scope)
            self.check_target(st, scope)
            if st.op in ("min=", "max="):
                if tt.rank or at.rank:
                    self.fail(f"{st.op} needs scalars", st)
            elif st.op in ("*=", "/="):
                if at.rank and not (st.op == "*=" and tt.rank == 2 and at.rank == 2):
                    self.fail(f"{st.op} needs a scalar argument", st)
            elif not assignable(tt, at):
                self.fail(f"cannot assign {at} to {tt}", st)
            if isinstance(st, Reduce):
                loop = self.enclosing(scope, ForeachParticle)
                if loop is None:
                    self.fail("reduce outside a particle loop", st)
                self.info.reductions.setdefault(id(loop), []).append(st)
        elif isinstance(st, ForeachParticle):
            if self.in_particle_loop(scope):
                self.fail("nested particle loop", st)
            if st.groups not in self.groups:
                self.fail(f"unknown groups {st.groups!r}", st)
            self.info.loops.append(st)
            self.info.uses_neighbors[id(st)] = any(isinstance(x, ForeachNeighbor) for x in st.body)
            self.block(st.body, _Scope(scope, st))
        elif isinstance(st, ForeachNeighbor):
            if st.groups is not None and st.groups not in self.groups:
                self.fail(f"unknown groups {st.groups!r}", st)
            self.block(st.body, _Scope(scope, st))
        elif isinstance(st, ForeachDimension):
            self.block(st.body, _Scope(scope, st))
        elif isinstance(st, Solve):
            self.solve(st, scope)
        else:
            self.fail(f"unsupported statement {type(st).__name__}", st)

    def solve(self, st, scope):
        if st.solver != "pcg":
            self.fail(f"unknown solver {st.solver!r}", st)
        if st.groups not in self.groups:
            self.fail(f"unknown groups {st.groups!r}", st)
        kinds = {}
        for part in st.parts:
            key = (type(part).__name__, getattr(part, "name", None))
            if key in kinds:
                self.fail("solve part declared twice", part)
            kinds[key] = part
        need = {("SolveSetup", "right_hand_side"), ("SolveSetup", "guess"), ("SolveProduct", "system"),
                ("SolveProduct", "preconditioner"), ("SolveApply", None)}
        if set(kinds) != need:
            self.fail("solve pcg needs setup right_hand_side, setup guess, product system, "
                      "product preconditioner and apply", st)
        self.info.loops.append(st)
        for part in st.parts:
            inner = _Scope(scope, st)
            inner.solve_part = part
            self.block(part.body, inner)

    # -- targets
    def check_target(self, st, scope):
        t = st.target
        if isinstance(t, Slice):
            t = t.subject
        if isinstance(st, Reduce):
            ok = (isinstance(t, NameRef) and (isinstance(t.ref, FieldDef) or
                  (isinstance(t.ref, LocalDef) and id(t.ref) in self.info.frame_locals)))
            if not ok:
                self.fail("reduce into anything but a global field or a procedure-level local", st)
            return
        if isinstance(t, FieldAccess):
            if isinstance(t.ref, SolveRef):
                if t.ref.kind != "into":
                    self.fail(f"cannot assign to the solver's {t.ref.kind} vector", st)
                return
            if isinstance(t.loop, ForeachNeighbor):
                self.fail("cannot assign to a neighbour's field", st)
            return
        if isinstance(t, NameRef) and isinstance(t.ref, (LocalDef, FieldDef)):
            if isinstance(t.ref, FieldDef) and self.in_particle_loop(scope):
                self.fail("compute into a global field inside a particle loop (use reduce)", st)
            return
        self.fail("invalid compute target", st)

    # -- expressions
    def expr(self, e, scope) -> NDType:
        t = self._expr(e, scope)
        self.info.types[id(e)] = t
        return t

    def _expr(self, e, scope) -> NDType:
        if isinstance(e, Literal):
            return REAL
        if isinstance(e, NameRef):
            loc = self.lookup_local(scope, e.name)
            if loc is not None:
                e.ref = loc
                return norm_type(loc.type)
            lp, _ = self.binding(scope, e.name)
            if isinstance(lp, ForeachDimension):
                e.ref = lp
                return INTEGER
            if e.name in self.globals:
                e.ref = self.globals[e.name]
                return norm_type(e.ref.type)
            self.fail(f"unknown name {e.name!r}", e)
        if isinstance(e, FieldAccess):
            lp, sc = self.binding(scope, e.frm)
            if lp is None or isinstance(lp, ForeachDimension):
                self.fail(f"{e.frm!r} is not a particle or neighbour index", e)
            part = self.solve_part(scope)
            if part is not None and self.enclosing(scope, Solve) is not None:
                names = {}
                if isinstance(part, SolveSetup):
                    names = {part.into: "into"}
                elif isinstance(part, SolveProduct):
                    names = {part.into: "into", part.with_: "with"}
                elif isinstance(part, SolveApply):
                    names = {part.with_: "with"}
                if e.name in names:
                    solve = self.enclosing(scope, Solve)
                    e.ref = SolveRef(names[e.name], solve)
                    e.loop = lp
                    return norm_type(solve.type)
            if isinstance(lp, ForeachNeighbor):
                gname = lp.groups
                if gname is None:
                    outer = self.enclosing(sc.parent, (ForeachParticle, Solve))
                    gname = outer.groups
            else:
                gname = lp.groups
            g = self.groups[gname]
            for f in g.fields:
                if f.alias == e.name:
                    e.ref, e.loop = f, lp
                    return norm_type(f.type)
            self.fail(f"groups {gname!r} have no field {e.name!r}", e)
        if isinstance(e, Neg):
            return self.expr(e.operand, scope)
        if isinstance(e, BinOp):
            a, b = self.expr(e.lhs, scope), self.expr(e.rhs, scope)
            return self.binop(e, a, b)
        if isinstance(e, Slice):
            t = self.expr(e.subject, scope)
            if len(e.indices) != 1:
                self.fail("a slice takes exactly one index", e)
            ix = e.indices[0]
            if isinstance(ix, NameRef):
                self.expr(ix, scope)
                if not isinstance(ix.ref, ForeachDimension):
                    self.fail("a slice index must be a dimension index or a number", e)
            if t.rank != 1:
                self.fail("only vectors can be sliced", e)
            return NDType(t.base)
        if isinstance(e, Call):
            return self.call(e, [self.expr(a, scope) for a in e.args])
        self.fail(f"unsupported expression {type(e).__name__}", e)

    def solve_part(self, scope):
        while scope is not None:
            part = getattr(scope, "solve_part", None)
            if part is not None:
                return part
            scope = scope.parent
        return None

    def binop(self, e, a, b):
        if a.base == "boolean" or b.base == "boolean":
            self.fail("arithmetic on booleans", e)
        if e.op in "+-":
            if a.rank != b.rank:
                self.fail(f"{a} {e.op} {b}", e)
            if a.rank == 0:
                return INTEGER if a.base == b.base == "integer" else REAL
            return a
        if e.op == "*":
            if a.rank == 0:
                return b if b.rank else (INTEGER if a.base == b.base == "integer" else REAL)
            if b.rank == 0:
                return a
            if a.rank == 2 and b.rank == 1:
                return VEC
            if a.rank == 2 and b.rank == 2:
                return MAT
            self.fail(f"{a} * {b} (use dot or outer_product)", e)
        if e.op == "/":
            if b.rank:
                self.fail(f"{a} / {b}", e)
            return a if a.rank else (INTEGER if a.base == b.base == "integer" else REAL)
        self.fail(f"operator {e.op}", e)

    def call(self, e, ts):
        n, k = e.name, len(ts)
        if n not in KNOWN_CALLS:
            self.fail(f"unknown function {n!r}", e)
        if n in TYPED_CALLS:
            if e.type is None or k:
                self.fail(f"{n} takes a type and no arguments: {n}<type>()", e)
            t = norm_type(e.type)
            if n == "identity" and t.rank != 2:
                self.fail("identity needs a matrix type", e)
            return t
        if e.type is not None:
            self.fail(f"{n} takes no type argument", e)

        def need(cnt, ranks=None):
            if k != cnt:
                self.fail(f"{n} takes {cnt} argument(s)", e)
            if ranks is not None:
                for t, r in zip(ts, ranks):
                    if r is not None and t.rank != r:
                        self.fail(f"argument of {n} has type {t}", e)
        if n in ("kernel_h", "kernel_gradient_h"):
            need(2, (1, 0))
            return REAL if n == "kernel_h" else VEC
        if n == "kernel_support_radius":
            need(1, (0,))
            return REAL
        if n == "dot":
            need(2, (1, 1))
            return REAL
        if n in ("norm", "norm_squared"):
            need(1)
            if ts[0].rank > 1:
                self.fail(f"{n} of a matrix is not supported", e)
            return REAL
        if n == "cabs":
            need(1)
            return ts[0]
        if n in ("max", "min"):
            if k < 2 or any(t.rank for t in ts):
                self.fail(f"{n} takes two or more scalars", e)
            return INTEGER if all(t.base == "integer" for t in ts) else REAL
        if n == "reciprocal_or_zero":
            need(2, (0, 0))
            return REAL
        if n in ("unit_step_l", "unit_step_r"):
            if k < 2 or any(t.rank for t in ts):
                self.fail(f"{n} takes two or more scalars", e)
            return REAL
        if n == "outer_product":
            need(2, (1, 1))
            return MAT
        if n in ("transpose", "invert_pm"):
            need(1, (2,))
            return MAT
        if n == "invert":
            need(1)
            if ts[0].rank == 1:
                self.fail("invert of a vector", e)
            return ts[0] if ts[0].rank else REAL
        if n == "trace":
            need(1, (2,))
            return REAL
        if n in ("aat13_cohesion_h", "aat13_adhesion_h"):
            need(2, (0, 0))
            return REAL
        if n == "smoothstep":
            need(1, (0,))
            return REAL
        if n == "cross_product_matrix_from_vector":
            need(1, (1,))
            return MAT
        if n == "vector_from_cross_product_matrix":
            need(1, (2,))
            return VEC
        self.fail(f"unsupported function {n!r}", e)


def assignable(target: NDType, value: NDType) -> bool:
    if target.rank != value.rank:
        return False
    if target.rank:
        return target.base == value.base
    return True  # scalars convert (integer <-> real) as in C++


def resolve(scheme: Scheme) -> Info:
    """Bind the names of every procedure of `scheme`; returns the types and
    storage decisions the code generator needs.  Raises DslError."""
    return Resolver(scheme).run()
