"""CUDA backend of the scheme language: a scheme -> one ``.cu`` plugin.

The reference compiles each ``.prtcl`` scheme to a C++/OpenMP header
(lua/prtcl/generate/cxx_openmp_impl_hpp.lua).  This backend emits, for the
same scheme, a CUDA source that defines a ``prtcl_gpu::Scheme`` and
registers it by full name when the plugin is loaded; the scheme is then
created, loaded and run like the hand-written ones.

Execution (one GPU stream, no host round trip inside a procedure):

* ``foreach <groups> particle i`` -> one kernel launch per model group the
  groups select (in group order, as the reference loops ``for (auto &p :
  groups)``), one thread per particle.  Statements run in order on the
  particle's fields; ``compute`` into a field of the particle reads and
  writes the field itself, as the reference's generated code does.
* ``foreach <groups> neighbor j`` -> for every selected group in order, the
  particle's neighbour list towards it (``_``: the particle's own group).
* ``reduce`` -> per-thread partials in FP64, summed per block and then in
  block order by a one-thread kernel that applies them to the target (the
  reference reduces f32 per OpenMP thread: the result agrees to rounding).
* statements outside particle loops -> one-thread kernels; their locals live
  in a small device frame, so that particle loops can read and reduce them.
* ``foreach dimension index d`` at procedure level -> a host loop over the
  N = 3 dimensions; ``d`` is a kernel argument.
* ``solve pcg`` -> per selected group, a kernel per part (guess, right-hand
  side, system and preconditioner products, apply) over the solver's
  vectors, driven by the reference's CG (solver/cg_openmp.hpp:35-215) with
  its state on the device and one 4-byte read per iteration for the stop
  decision; dots, threshold and breaks in FP64 as the hand-written WKBB18
  solver (csrc/dsl_device.cuh).

Arithmetic follows the reference's generated expressions: every binary
operation as written, folded left, with literals cast to f32 and the
operators and functions of ``csrc/dsl_device.cuh``.
"""
from __future__ import annotations

import hashlib

from .check import INTEGER, MAT, REAL, VEC, Info, SolveRef, norm_type, resolve
from .parser import (BinOp, Call, Compute, DslError, FieldAccess, FieldDef, ForeachDimension, ForeachNeighbor,
                     ForeachParticle, Literal, LocalDef, NameRef, NDType, Neg, Reduce, Scheme, Select, SelAnd, SelNot,
                     SelOr, Slice, Solve)

FULL_NAME = "prtcl::schemes::{}[T=f32, N=3, K=Cubic Spline]"


def ctype(t: NDType) -> str:
    t = norm_type(t)
    if t.base == "boolean":
        raise DslError("boolean values are not supported by the CUDA backend")
    if t.rank == 0:
        return "int" if t.base == "integer" else "float"
    if t.base != "real" or any(e not in (0,) for e in t.extents):
        raise DslError(f"unsupported type {t} (the CUDA backend takes real, real[], real[][] and integer)")
    return "f3" if t.rank == 1 else "M3"


def device_type_ok(t: NDType) -> bool:
    try:
        ctype(t)
        return True
    except DslError:
        return False


def _field_type_expr_any(t: NDType) -> str:
    """FieldType of any declared type (fields the kernels cannot read are
    still created at load, as the reference's Load does)."""
    ct = "i32" if t.base == "integer" else "f32"
    if t.rank == 0:
        return f'parse_field_type("{ct}", 0, nullptr)'
    ext = ", ".join(str(e or 3) for e in t.extents)
    return f'[] {{ static int const e[] = {{{ext}}}; return parse_field_type("{ct}", {t.rank}, e); }}()'


def _varying_member(t: NDType) -> str:
    c = ctype(t)
    return {"float": "float *", "int": "int *", "f3": "float4 *", "M3": "Planar9 "}[c]


def _small_member(t: NDType) -> str:
    return {"float": "SReal", "int": "SInt", "f3": "SVec", "M3": "SMat"}[ctype(t)]


def _field_type_expr(t: NDType) -> str:
    t = norm_type(t)
    ct = "i32" if t.base == "integer" else "f32"
    if t.rank == 0:
        return f'parse_field_type("{ct}", 0, nullptr)'
    ext = ", ".join("3" for _ in t.extents)
    return f'[] {{ static int const e[] = {{{ext}}}; return parse_field_type("{ct}", {t.rank}, e); }}()'


def _ident(s: str) -> str:
    return "".join(ch if ch.isalnum() or ch == "_" else "_" for ch in s)


class _Kernel:
    """Code of one kernel being generated."""

    def __init__(self, name, loop=None):
        self.name = name
        self.loop = loop
        self.lines = []
        self.nb_groups = []   # groups blocks walked by its neighbour loops
        self.dims = []        # dimension indices in scope (kernel arguments)
        self.reductions = []  # Reduce statements (particle kernels)


class Emitter:
    def __init__(self, scheme: Scheme, info: Info, prefix: str = "", embed_source: bool = True):
        self.s = scheme
        self.info = info
        self.prefix = prefix
        self.embed_source = embed_source
        self.full_short = prefix + scheme.name
        uid = hashlib.sha1((prefix + scheme.source).encode()).hexdigest()[:12]
        self.ns = f"gen_{_ident(scheme.name)}_{uid}"
        self.kernels = []
        self.host_procs = []
        self.groups = {g.name: g for g in scheme.groups}
        self.max_red = 0
        self.tmp = 0

    # -- names
    def fresh(self, base="t"):
        self.tmp += 1
        return f"{base}{self.tmp}_"

    def gs(self, gname):
        return f"G_{_ident(gname)}"

    # -- expressions
    def expr(self, e, ctx) -> str:
        if isinstance(e, Literal):
            return f"float({e.text})"
        if isinstance(e, NameRef):
            r = e.ref
            if isinstance(r, LocalDef):
                slot = self.info.frame_locals.get(id(r))
                if slot is not None:
                    return f"frd<{ctype(r.type)}>(fr, {slot})"
                return f"l_{_ident(r.name)}"
            if isinstance(r, FieldDef):
                self.usable(r)
                return f"rd(g.g_{_ident(r.alias)})"
            if isinstance(r, ForeachDimension):
                return f"d_{_ident(r.index)}"
            raise DslError(f"unresolved name {e.name!r}")
        if isinstance(e, FieldAccess):
            return self.field_read(e, ctx)
        if isinstance(e, Neg):
            return f"(-{self.expr(e.operand, ctx)})"
        if isinstance(e, BinOp):
            return f"({self.expr(e.lhs, ctx)} {e.op} {self.expr(e.rhs, ctx)})"
        if isinstance(e, Slice):
            return f"comp({self.expr(e.subject, ctx)}, {self.index(e.indices[0], ctx)})"
        if isinstance(e, Call):
            return self.call(e, ctx)
        raise DslError(f"unsupported expression {type(e).__name__}")

    def index(self, ix, ctx):
        if isinstance(ix, str):
            return str(int(ix))
        return self.expr(ix, ctx)

    def field_read(self, e, ctx):
        if isinstance(e.ref, SolveRef):
            _, idx = self.binding(e, ctx)
            return f"vld({e.ref.kind}_, {idx})"
        var, idx = self.binding(e, ctx)
        f = e.ref
        self.usable(f)
        if f.kind == "varying":
            return f"rd({var}.v_{_ident(f.alias)}, {idx})"
        return f"rd({var}.u_{_ident(f.alias)})"

    def usable(self, f):
        if not device_type_ok(f.type):
            raise DslError(f"field {f.name} of type {f.type} cannot be used by the CUDA backend "
                           "(it takes real, real[], real[][] and integer)")

    def binding(self, e, ctx):
        lp = e.loop
        if isinstance(lp, ForeachNeighbor):
            return "n", "j"
        return "p", "i"

    def call(self, e, ctx):
        n = e.name
        args = [self.expr(a, ctx) for a in e.args]
        if n in ("zeros", "ones", "positive_infinity", "negative_infinity"):
            return f"{n}<{ctype(e.type)}>()"
        if n == "identity":
            return "identity3()"
        if n in ("max", "min"):
            t = ctype(self.info.types[id(e)])
            return f"{n}<{t}>({', '.join(args)})"
        if n in ("unit_step_l", "unit_step_r"):
            return f"{n}({', '.join(f'float({a})' for a in args)})"
        return f"{n}({', '.join(args)})"

    # -- statements
    def stmt(self, st, k: _Kernel, ctx, ind):
        pad = "  " * ind
        out = k.lines
        if isinstance(st, LocalDef):
            slot = self.info.frame_locals.get(id(st))
            c = ctype(st.type)
            if slot is not None:
                out.append(f"{pad}fwr(fr, {slot}, {c}({self.expr(st.init, ctx)}));")
            else:
                out.append(f"{pad}{c} l_{_ident(st.name)} = {self.expr(st.init, ctx)};")
        elif isinstance(st, Compute):
            self.compute(st, k, ctx, pad)
        elif isinstance(st, Reduce):
            r = len(k.reductions)
            k.reductions.append(st)
            v = f"double({self.expr(st.arg, ctx)})"
            if st.op in ("+=", "-="):
                out.append(f"{pad}r{r}_ += {v};")
            elif st.op == "*=":
                out.append(f"{pad}r{r}_ *= {v};")
            elif st.op == "max=":
                out.append(f"{pad}{{ double v_ = {v}; r{r}_ = (r{r}_ < v_) ? v_ : r{r}_; }}")
            else:
                out.append(f"{pad}{{ double v_ = {v}; r{r}_ = (v_ < r{r}_) ? v_ : r{r}_; }}")
        elif isinstance(st, ForeachNeighbor):
            self.neighbor_loop(st, k, ctx, ind)
        else:
            raise DslError(f"unsupported statement {type(st).__name__} in a kernel")

    def compute(self, st, k, ctx, pad):
        out = k.lines
        tgt = st.target
        slice_ix = None
        if isinstance(tgt, Slice):
            slice_ix = self.index(tgt.indices[0], ctx)
            tgt = tgt.subject
        ty = ctype(self.info.types[id(tgt)])
        # read-modify-write through a temporary of the target's type
        if isinstance(tgt, FieldAccess) and isinstance(tgt.ref, SolveRef):
            read, write = "vld(into_, i)", "vst(into_, i, {});"
        elif isinstance(tgt, FieldAccess):
            var, idx = self.binding(tgt, ctx)
            f = tgt.ref
            self.usable(f)
            if f.kind == "varying":
                read, write = f"rd({var}.v_{_ident(f.alias)}, {idx})", f"wr({var}.v_{_ident(f.alias)}, {idx}, {{}});"
            else:
                read, write = f"rd({var}.u_{_ident(f.alias)})", f"wr({var}.u_{_ident(f.alias)}, {{}});"
        elif isinstance(tgt, NameRef) and isinstance(tgt.ref, LocalDef):
            slot = self.info.frame_locals.get(id(tgt.ref))
            if slot is None:
                name = f"l_{_ident(tgt.ref.name)}"
                read, write = name, name + " = {};"
            else:
                read, write = f"frd<{ty}>(fr, {slot})", f"fwr(fr, {slot}, {{}});"
        elif isinstance(tgt, NameRef) and isinstance(tgt.ref, FieldDef):
            self.usable(tgt.ref)
            name = f"g.g_{_ident(tgt.ref.alias)}"
            read, write = f"rd({name})", f"wr({name}, {{}});"
        else:
            raise DslError("invalid compute target")
        arg = self.expr(st.arg, ctx)
        t = self.fresh()
        if slice_ix is None:
            if st.op == "=":
                out.append(f"{pad}{write.format(f'{ty}({arg})')}")
                return
            op = {"+=": "add_to", "-=": "sub_from", "*=": "mul_by", "/=": "div_by"}.get(st.op)
            body = f"{op}({t}, {arg});" if op else f"{t} = {st.op[:3]}<{ty}>({t}, {arg});"
            out.append(f"{pad}{{ {ty} {t} = {read}; {body} {write.format(t)} }}")
        else:
            if ty != "f3":
                raise DslError("only vector components can be assigned")
            c = f"comp({t}, {slice_ix})"
            if st.op == "=":
                body = f"{c} = float({arg});"
            elif st.op in ("min=", "max="):
                body = f"{c} = {st.op[:3]}<float>({c}, {arg});"
            else:
                body = f"{c} = {c} {st.op[0]} {arg};"
            out.append(f"{pad}{{ f3 {t} = {read}; {body} {write.format(t)} }}")

    def neighbor_loop(self, st, k, ctx, ind):
        pad = "  " * ind
        out = k.lines
        own = st.groups is None
        gname = k.loop.groups if own else st.groups
        if own:
            out.append(f"{pad}{{ // foreach _ neighbor {st.index}")
            out.append(f"{pad}  {self.gs(gname)} const &n = p;")
            out.append(f"{pad}  NbrList nl_ = nbr_list(L, n.index);")
            out.append(f"{pad}  if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {{")
            for s in st.body:
                self.stmt(s, k, ctx, ind + 2)
            out.append(f"{pad}  }});")
            out.append(f"{pad}}}")
            return
        if gname not in k.nb_groups:
            k.nb_groups.append(gname)
        arr = f"nb_{_ident(gname)}"
        q = self.fresh("q")
        out.append(f"{pad}for (int {q} = 0; {q} < {arr}.count; ++{q}) {{ // foreach {gname} neighbor {st.index}")
        out.append(f"{pad}  {self.gs(gname)} const &n = {arr}.g[{q}];")
        out.append(f"{pad}  NbrList nl_ = nbr_list(L, n.index);")
        out.append(f"{pad}  if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {{")
        for s in st.body:
            self.stmt(s, k, ctx, ind + 2)
        out.append(f"{pad}  }});")
        out.append(f"{pad}}}")

    # -- procedures
    def procedure(self, proc):
        host = []
        self.pidx = 0
        self.body(proc, proc.body, host, [], 1)
        self.host_procs.append((proc.name, host))

    def body(self, proc, stmts, host, dims, ind):
        pad = "  " * ind
        scalar = []

        def flush():
            if not scalar:
                return
            k = _Kernel(f"k_{_ident(proc.name)}_s{self.pidx}")
            self.pidx += 1
            k.dims = list(dims)
            for st in scalar:
                self.stmt(st, k, None, 1)
            self.kernels.append(k)
            dargs = "".join(f", d_{_ident(d)}" for d in dims)
            host.append(f"{pad}{k.name}<<<1, 1, 0, s>>>(glob(), frame_{dargs});")
            host.append(f"{pad}count_launch();")
            scalar.clear()

        for st in stmts:
            if isinstance(st, ForeachParticle):
                flush()
                self.particle_loop(proc, st, host, dims, ind)
            elif isinstance(st, ForeachDimension):
                flush()
                d = _ident(st.index)
                host.append(f"{pad}for (int d_{d} = 0; d_{d} < 3; ++d_{d}) {{")
                self.body(proc, st.body, host, dims + [st.index], ind + 1)
                host.append(f"{pad}}}")
            elif isinstance(st, Solve):
                flush()
                self.solve(proc, st, host, dims, ind)
            else:
                scalar.append(st)
        flush()

    def particle_loop(self, proc, st, host, dims, ind):
        pad = "  " * ind
        k = _Kernel(f"k_{_ident(proc.name)}_p{self.pidx}", st)
        self.pidx += 1
        k.dims = list(dims)
        for s in st.body:
            self.stmt(s, k, None, 2)
        self.kernels.append(k)
        nred = len(k.reductions)
        self.max_red = max(self.max_red, nred)
        gsn = _ident(st.groups)
        needs_nb = self.info.uses_neighbors.get(id(st), False)
        nb_args = "".join(f", all_{_ident(g)}()" for g in k.nb_groups)
        dargs = "".join(f", d_{_ident(d)}" for d in dims)
        host.append(f"{pad}{{ // foreach {st.groups} particle {st.index}")
        if nred:
            host.append(f"{pad}  uint32_t off_ = 0, total_ = 0;")
            host.append(f"{pad}  for (Group *pg : sel_{gsn}) total_ += uint32_t((pg->count + kGenNT - 1) / kGenNT);")
            host.append(f"{pad}  ensure_red({nred}, total_);")
        host.append(f"{pad}  for (Group *pg : sel_{gsn}) {{")
        host.append(f"{pad}    if (pg->count == 0) continue;")
        host.append(f"{pad}    uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);")
        if needs_nb:
            host.append(f"{pad}    NbrView const &lv_ = nh.lists(pg->index, s);")
        else:
            host.append(f"{pad}    NbrView lv_{{}};")
        red_args = ", red_, red_cap_, off_" if nred else ", nullptr, 0u, 0u"
        host.append(f"{pad}    {k.name}<<<blocks_, kGenNT, 0, s>>>(mk_{gsn}(pg){nb_args}, glob(), lv_, frame_{dargs}{red_args});")
        host.append(f"{pad}    count_launch();")
        if nred:
            host.append(f"{pad}    off_ += blocks_;")
        host.append(f"{pad}  }}")
        # fields written: their versions move on, so that caches keyed on them
        # (neighbour lists on positions, packed records) are rebuilt
        for fname in self.written_fields(st):
            host.append(f'{pad}  for (Group *pg : sel_{gsn}) pg->varying.at("{fname}").version++;')
        if nred:
            fk = _Kernel(f"{k.name}_f")
            fk.dims = list(dims)
            self.finalize_kernel(fk, k)
            self.kernels.append(fk)
            host.append(f"{pad}  {fk.name}<<<1, 1, 0, s>>>(glob(), frame_, red_, red_cap_, total_{dargs});")
            host.append(f"{pad}  count_launch();")
        host.append(f"{pad}}}")

    def solve(self, proc, st, host, dims, ind):
        pad = "  " * ind
        t = norm_type(st.type)
        if t.base != "real" or t.rank > 1:
            raise DslError(f"solve pcg over {t} (the CUDA backend takes real and real[])")
        S = "float" if t.rank == 0 else "float4"
        g = self.groups[st.groups]
        aliases = {f.alias: f for f in g.fields if f.kind == "uniform"}
        for a, base in (("pcg_max_error", "real"), ("pcg_max_iters", "integer"), ("pcg_iterations", "integer")):
            if a not in aliases or norm_type(aliases[a].type) != NDType(base):
                raise DslError(f"solve pcg over groups {st.groups!r} needs a uniform field {a} of type {base}")
        parts = {}
        for part in st.parts:
            key = getattr(part, "name", "apply")
            k = _Kernel(f"k_{_ident(proc.name)}_v{self.pidx}_{key}", st)
            k.dims = list(dims)
            k.solve_storage = S
            for x in part.body:
                self.stmt(x, k, None, 2)
            self.kernels.append(k)
            parts[key] = k
        self.pidx += 1
        gsn = _ident(st.groups)
        dargs = "".join(f", d_{_ident(d)}" for d in dims)
        uses_nb = any(k.nb_groups or "nbr_list(" in "\n".join(k.lines) for k in parts.values())

        def launch(key, into, with_):
            k = parts[key]
            nb_args = "".join(f", all_{_ident(gn)}()" for gn in k.nb_groups)
            return (f"{pad}    {k.name}<<<nb_, kGenNT, 0, s>>>(pp_{nb_args}, glob(), lv_, frame_{dargs}, "
                    f"{into}, {with_});")

        h = host.append
        h(f"{pad}{{ // solve pcg {t} over {st.groups} particle {st.index}")
        h(f"{pad}  for (Group *pg : sel_{gsn}) {{")
        h(f"{pad}    {self.gs(st.groups)} pp_ = mk_{gsn}(pg);")
        h(f"{pad}    uint32_t n_ = uint32_t(pg->count);")
        h(f"{pad}    if (n_ == 0) {{ k_pcg_zero<<<1, 1, 0, s>>>(pp_.u_pcg_iterations); count_launch(); continue; }}")
        h(f"{pad}    uint32_t nb_ = (n_ + kGenNT - 1) / kGenNT;")
        h(f"{pad}    ensure_pcg(n_ * sizeof({S}), nb_);")
        h(f"{pad}    {S} *x_ = pcg_vec<{S}>(0, n_), *b_ = pcg_vec<{S}>(1, n_), *r_ = pcg_vec<{S}>(2, n_);")
        h(f"{pad}    {S} *p_ = pcg_vec<{S}>(3, n_), *q_ = pcg_vec<{S}>(4, n_), *y_ = pcg_vec<{S}>(5, n_);")
        h(f"{pad}    double *c0_ = pcg_part_, *c1_ = pcg_part_ + pcg_part_cap_, *c2_ = pcg_part_ + 2 * pcg_part_cap_;")
        if uses_nb:
            h(f"{pad}    NbrView const &lv_ = nh.lists(pg->index, s);")
        else:
            h(f"{pad}    NbrView lv_{{}};")
        h(f"{pad}    {S} *none_ = nullptr;")
        # x = guess; b = rhs; r = A x - b; y = T r; p = -y
        h(launch("guess", "x_", "none_"))
        h(launch("right_hand_side", "b_", "none_"))
        h(launch("system", "r_", "x_"))
        h(f"{pad}    k_pcg_residual<{S}><<<nb_, kPcgNT, 0, s>>>(n_, r_, b_, c0_);")
        h(launch("preconditioner", "y_", "r_"))
        h(f"{pad}    k_pcg_start<{S}><<<nb_, kPcgNT, 0, s>>>(n_, p_, y_, r_, c1_, c2_);")
        h(f"{pad}    k_pcg_begin<<<1, 1, 0, s>>>(pcg_state_, pp_.u_pcg_max_error, pp_.u_pcg_max_iters, c0_, c1_, c2_, nb_);")
        h(f"{pad}    for (int k = 0; k < 7; ++k) count_launch();")
        h(f"{pad}    for (long it_ = 0;; ++it_) {{")
        h(f"{pad}      // q = A p; alpha; x += alpha p, r += alpha q; y = T r; beta; p = -y + beta p")
        h("  " + launch("system", "q_", "p_"))
        h(f"{pad}      k_pcg_dot<{S}><<<nb_, kPcgNT, 0, s>>>(n_, p_, q_, c0_);")
        h(f"{pad}      k_pcg_step<<<1, 1, 0, s>>>(pcg_state_, c0_, nb_);")
        h(f"{pad}      k_pcg_update<{S}><<<nb_, kPcgNT, 0, s>>>(n_, x_, r_, p_, q_, pcg_state_, c1_);")
        h("  " + launch("preconditioner", "y_", "r_"))
        h(f"{pad}      k_pcg_dot<{S}><<<nb_, kPcgNT, 0, s>>>(n_, r_, y_, c2_);")
        h(f"{pad}      k_pcg_next<<<1, 1, 0, s>>>(pcg_state_, c1_, c2_, nb_);")
        h(f"{pad}      k_pcg_direction<{S}><<<nb_, kPcgNT, 0, s>>>(n_, p_, y_, pcg_state_);")
        h(f"{pad}      for (int k = 0; k < 8; ++k) count_launch();")
        h(f"{pad}      PG_CUDA(cudaMemcpyAsync(pcg_stop_h_, &pcg_state_->stop, sizeof(int), cudaMemcpyDeviceToHost, s));")
        h(f"{pad}      PG_CUDA(cudaStreamSynchronize(s));")
        h(f"{pad}      if (*pcg_stop_h_) break;")
        h(f"{pad}      if (it_ > (1L << 30)) throw Error(\"solve pcg did not stop\");")
        h(f"{pad}    }}")
        h(launch("apply", f"none_", "x_"))
        h(f"{pad}    k_pcg_end<<<1, 1, 0, s>>>(pcg_state_, pp_.u_pcg_iterations);")
        h(f"{pad}    count_launch();")
        h(f"{pad}    count_launch();")
        h(f"{pad}  }}")
        for fname in self.written_fields(st):
            h(f'{pad}  for (Group *pg : sel_{gsn}) pg->varying.at("{fname}").version++;')
        h(f"{pad}}}")
        self.uses_pcg = True

    def written_fields(self, loop):
        names = []

        def walk(stmts):
            for st in stmts:
                if hasattr(st, "body") and not isinstance(st, (ForeachNeighbor, Compute)) and \
                        type(st).__name__.startswith("Solve"):
                    walk(st.body)
                elif isinstance(st, Compute):
                    t = st.target.subject if isinstance(st.target, Slice) else st.target
                    if isinstance(t, FieldAccess) and isinstance(t.ref, FieldDef) and t.ref.kind == "varying" \
                            and t.loop is loop and t.ref.name not in names:
                        names.append(t.ref.name)
                elif isinstance(st, ForeachNeighbor):
                    walk(st.body)
        walk(loop.parts if isinstance(loop, Solve) else loop.body)
        return names

    def finalize_kernel(self, fk, k):
        out = fk.lines
        for r, st in enumerate(k.reductions):
            tgt = st.target
            ty = ctype(self.info.types[id(tgt)])
            if isinstance(tgt.ref, FieldDef):
                name = f"g.g_{_ident(tgt.ref.alias)}"
                read, write = f"rd({name})", f"wr({name}, {{}});"
            else:
                slot = self.info.frame_locals[id(tgt.ref)]
                read, write = f"frd<{ty}>(fr, {slot})", f"fwr(fr, {slot}, {{}});"
            out.append(f"  {{ // reduce {st.op}")
            out.append(f"    double const *pr_ = red + size_t({r}) * red_cap;")
            if st.op in ("+=", "-="):
                out.append("    double a_ = 0.0;")
                out.append("    for (uint32_t b = 0; b < nparts; ++b) a_ += pr_[b];")
                out.append(f"    double v_ = double({read}) {st.op[0]} a_;")
            elif st.op == "*=":
                out.append("    double a_ = 1.0;")
                out.append("    for (uint32_t b = 0; b < nparts; ++b) a_ *= pr_[b];")
                out.append(f"    double v_ = double({read}) * a_;")
            else:
                cmp = "<" if st.op == "max=" else ">"
                out.append(f"    double v_ = double({read});")
                out.append(f"    for (uint32_t b = 0; b < nparts; ++b) if (v_ {cmp} pr_[b]) v_ = pr_[b];")
            conv = "int(llrint(v_))" if ty == "int" else "float(v_)"
            out.append(f"    {write.format(conv)}")
            out.append("  }")

    # -- whole source
    def source(self) -> str:
        return HEADER + self.body_source() + init_source([self])

    def body_source(self) -> str:
        for p in self.s.procedures:
            self.procedure(p)
        L = []
        w = L.append
        w(f"// scheme {self.s.name}")
        w("namespace prtcl_gpu {")
        w(f"namespace {self.ns} {{")
        w("using namespace ::prtcl_gpu::dsl;")
        w("constexpr int kGenNT = 128;")
        w("")
        # group structs
        for g in self.s.groups:
            n = self.gs(g.name)
            w(f"struct {n} {{")
            w("  uint32_t n;")
            w("  int index;")
            for f in g.fields:
                if not device_type_ok(f.type):
                    continue  # created at load; no procedure may use it
                if f.kind == "varying":
                    w(f"  {_varying_member(f.type)}v_{_ident(f.alias)};")
                else:
                    w(f"  {_small_member(f.type)} u_{_ident(f.alias)};")
            w("};")
            w(f"struct {n}_all {{")
            w("  int count;")
            w(f"  {n} g[kMaxGroups];")
            w("};")
        w("struct Glob {")
        for f in self.s.globals:
            if device_type_ok(f.type):
                w(f"  {_small_member(f.type)} g_{_ident(f.alias)};")
        w("  int unused_;")
        w("};")
        w("")
        for k in self.kernels:
            self.emit_kernel(w, k)
        self.emit_class(w)
        w(f"}} // namespace {self.ns}")
        w("} // namespace prtcl_gpu")
        w("")
        return "\n".join(L) + "\n"

    def emit_kernel(self, w, k):
        dparams = "".join(f", int d_{_ident(d)}" for d in k.dims)
        if k.name.endswith("_f"):
            w(f"__global__ void {k.name}(Glob g, float *fr, double const *red, uint32_t red_cap, "
              f"uint32_t nparts{dparams}) {{")
            for line in k.lines:
                w(line)
            w("}")
            w("")
            return
        if k.loop is None:
            w(f"__global__ void {k.name}(Glob g, float *fr{dparams}) {{")
            for line in k.lines:
                w(line)
            w("}")
            w("")
            return
        gsn = self.gs(k.loop.groups)
        nb = "".join(f", {self.gs(gname)}_all nb_{_ident(gname)}" for gname in k.nb_groups)
        if isinstance(k.loop, Solve):
            S = k.solve_storage
            w(f"__global__ void __launch_bounds__(kGenNT) {k.name}({gsn} p{nb}, Glob g, NbrView L, float *fr{dparams}, "
              f"{S} *into_, {S} const *with_) {{")
            w("  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;")
            w("  if (i >= p.n) return;")
            w("  (void)into_;")
            w("  (void)with_;")
            for line in k.lines:
                w(line)
            w("}")
            w("")
            return
        w(f"__global__ void __launch_bounds__(kGenNT) {k.name}({gsn} p{nb}, Glob g, NbrView L, float *fr{dparams}, "
          f"double *red, uint32_t red_cap, uint32_t red_off) {{")
        w("  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;")
        for r, st in enumerate(k.reductions):
            ident = {"+=": "0.0", "-=": "0.0", "*=": "1.0", "max=": "-INFINITY", "min=": "INFINITY"}[st.op]
            w(f"  double r{r}_ = {ident};")
        w("  if (i < p.n) {")
        for line in k.lines:
            w(line)
        w("  }")
        if k.reductions:
            w("  __shared__ double sh_[32];")
            for r, st in enumerate(k.reductions):
                fn = {"+=": "block_sum", "-=": "block_sum", "max=": "block_reduce_max",
                      "min=": "block_reduce_min"}.get(st.op)
                if fn is None:
                    raise DslError("reduce *= is not supported by the CUDA backend")
                w(f"  {{ double b_ = {fn}(r{r}_, sh_); if (threadIdx.x == 0) red[size_t({r}) * red_cap + red_off + "
                  f"blockIdx.x] = b_; }}")
        w("}")
        w("")

    def emit_class(self, w):
        src = self.s.source if self.embed_source else "(scheme source text not embedded in this build)"
        w("class Scheme_ : public Scheme {")
        w("public:")
        w("  Scheme_() {")
        for name, _ in self.host_procs:
            w(f'    reg("{name}", [this](Nhood &nh, cudaStream_t s) {{ proc_{_ident(name)}(nh, s); }});')
        w("  }")
        w("  ~Scheme_() override {")
        w("    if (frame_) cudaFree(frame_);")
        w("    if (red_) cudaFree(red_);")
        w("    if (pcg_buf_) cudaFree(pcg_buf_);")
        w("    if (pcg_part_) cudaFree(pcg_part_);")
        w("    if (pcg_state_) cudaFree(pcg_state_);")
        w("    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);")
        w("  }")
        w(f'  std::string name() const override {{ return "{self.full_short}"; }}')
        delim = "prtcl_source"
        while f"){delim}\"" in src:
            delim += "_"
        w(f'  std::string source() const override {{ return R"{delim}({src}){delim}"; }}')
        w("  void load(Model &m) override {")
        for f in self.s.globals:
            w(f'    glob_{_ident(f.alias)}_ = &m.add_global("{f.name}", {_field_type_expr_any(f.type)});')
        for g in self.s.groups:
            gs = _ident(g.name)
            w(f"    sel_{gs}.clear();")
        w("    for (Group *grp : m.groups_by_index()) {")
        for g in self.s.groups:
            gs = _ident(g.name)
            w(f"      if ({self.select(g.select)}) {{")
            w(f"        if (sel_{gs}.size() == size_t(kMaxGroups)) throw Error(\"too many groups selected\");")
            w(f"        sel_{gs}.push_back(grp);")
            for f in g.fields:
                fn = "add_varying" if f.kind == "varying" else "add_uniform"
                w(f'        grp->{fn}("{f.name}", {_field_type_expr_any(f.type)});')
            w("      }")
        w("    }")
        nslots = max(1, self.info.frame_slots)
        w(f"    if (!frame_) PG_CUDA(cudaMalloc(&frame_, {nslots} * 16 * sizeof(float)));")
        w("    bind(m);")
        w("  }")
        w("  std::string source_text() const { return source(); }")
        w("")
        w("private:")
        for f in self.s.globals:
            w(f"  SmallField *glob_{_ident(f.alias)}_ = nullptr;")
        for g in self.s.groups:
            w(f"  std::vector<Group *> sel_{_ident(g.name)};")
        w("  float *frame_ = nullptr;")
        w("  double *red_ = nullptr;")
        w("  uint32_t red_cap_ = 0;")
        w("  void ensure_red(int nred, uint32_t parts) {")
        w("    if (parts <= red_cap_ && red_) return;")
        w("    if (red_) PG_CUDA(cudaFree(red_));")
        w("    red_cap_ = parts + parts / 4 + 64;")
        w(f"    PG_CUDA(cudaMalloc(&red_, size_t({max(1, self.max_red)}) * red_cap_ * sizeof(double)));")
        w("    (void)nred;")
        w("  }")
        w("  void *pcg_buf_ = nullptr;")
        w("  size_t pcg_vec_bytes_ = 0;")
        w("  double *pcg_part_ = nullptr;")
        w("  uint32_t pcg_part_cap_ = 0;")
        w("  PcgState *pcg_state_ = nullptr;")
        w("  int *pcg_stop_h_ = nullptr;")
        w("  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks")
        w("  void ensure_pcg(size_t bytes, uint32_t parts) {")
        w("    bytes = (bytes + 255) / 256 * 256;")
        w("    if (bytes > pcg_vec_bytes_) {")
        w("      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));")
        w("      pcg_vec_bytes_ = bytes + bytes / 4;")
        w("      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));")
        w("    }")
        w("    if (parts > pcg_part_cap_) {")
        w("      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));")
        w("      pcg_part_cap_ = parts + parts / 4 + 64;")
        w("      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));")
        w("    }")
        w("    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));")
        w("    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));")
        w("  }")
        w("  template <class S> S *pcg_vec(int k, uint32_t) const {")
        w("    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);")
        w("  }")
        w("  Glob glob() const {")
        w("    Glob r{};")
        for f in self.s.globals:
            if not device_type_ok(f.type):
                continue
            c = _small_member(f.type)
            base = "int" if c == "SInt" else "float"
            w(f"    r.g_{_ident(f.alias)} = {c}{{static_cast<{base} *>(model_->small_ptr(*glob_{_ident(f.alias)}_))}};")
        w("    return r;")
        w("  }")
        for g in self.s.groups:
            gs = _ident(g.name)
            n = self.gs(g.name)
            w(f"  {n} mk_{gs}(Group *grp) const {{")
            w(f"    {n} r{{}};")
            w("    r.n = uint32_t(grp->count);")
            w("    r.index = grp->index;")
            for f in g.fields:
                a = _ident(f.alias)
                if not device_type_ok(f.type):
                    continue
                if f.kind == "varying":
                    c = ctype(f.type)
                    w(f'    VaryingField &f_{a} = grp->varying.at("{f.name}");')
                    if c == "M3":
                        w(f"    r.v_{a} = Planar9{{static_cast<float *>(f_{a}.d), uint32_t(f_{a}.cap)}};")
                    else:
                        ptr = {"float": "float", "int": "int", "f3": "float4"}[c]
                        w(f"    r.v_{a} = static_cast<{ptr} *>(f_{a}.d);")
                else:
                    c = _small_member(f.type)
                    base = "int" if c == "SInt" else "float"
                    w(f'    r.u_{a} = {c}{{static_cast<{base} *>(model_->small_ptr(grp->uniform.at("{f.name}")))}};')
            w("    return r;")
            w("  }")
            w(f"  {n}_all all_{gs}() const {{")
            w(f"    {n}_all r{{}};")
            w(f"    r.count = int(sel_{gs}.size());")
            w(f"    for (int k = 0; k < r.count; ++k) r.g[k] = mk_{gs}(sel_{gs}[k]);")
            w("    return r;")
            w("  }")
        for name, host in self.host_procs:
            w(f"  void proc_{_ident(name)}(Nhood &nh, cudaStream_t s) {{")
            w("    (void)nh;")
            for line in host:
                w("  " + line)
            w("    PG_LAUNCH_CHECK();")
            w("  }")
        w("};")
        w("")

    def select(self, e) -> str:
        if isinstance(e, Select):
            if e.kind == "type":
                return f'(grp->type == "{e.name}")'
            return f'grp->has_tag("{e.name}")'
        if isinstance(e, SelNot):
            return f"(!{self.select(e.operand)})"
        if isinstance(e, SelAnd):
            return "(" + " && ".join(self.select(x) for x in e.operands) + ")"
        if isinstance(e, SelOr):
            return "(" + " || ".join(self.select(x) for x in e.operands) + ")"
        raise DslError("invalid group selector")


HEADER = """// Generated from the scheme language by prtcl_gb300.dsl.
#include "dsl_device.cuh"
#include "schemes.hpp"

#include <memory>

"""


def init_source(emitters) -> str:
    """The plugin's entry point: registers every scheme of the plugin."""
    L = ['extern "C" void prtcl_gpu_plugin_init() {']
    for e in emitters:
        L.append(f'  ::prtcl_gpu::register_scheme("{FULL_NAME.format(e.full_short)}", [] {{')
        L.append(f"    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::{e.ns}::Scheme_());")
        L.append("  });")
    L.append("}")
    return "\n".join(L) + "\n"


def generate(scheme: Scheme, prefix: str = "") -> str:
    """The CUDA source of the plugin for one scheme (raises DslError for a
    construct the backend does not support)."""
    info = resolve(scheme)
    return Emitter(scheme, info, prefix).source()


def generate_all(schemes, prefix: str = "", embed_source: bool = True) -> str:
    """One plugin source for several schemes (one nvcc run).  Without
    ``embed_source`` the schemes' GetPrtclSourceCode text is a fixed note
    instead of the ``.prtcl`` text."""
    ems = [Emitter(s, resolve(s), prefix, embed_source) for s in schemes]
    names = [e.full_short for e in ems]
    if len(set(names)) != len(names):
        raise DslError("two schemes of the same name in one plugin")
    return HEADER + "".join(e.body_source() for e in ems) + init_source(ems)


def full_name(scheme: Scheme, prefix: str = "") -> str:
    return FULL_NAME.format(prefix + scheme.name)
