"""The scheme language on the CPU: parser, name resolution and the CUDA
code generator (prtcl_gb300.dsl).  The generated plugins run in
tests/test_gpu_dsl.py."""
import os

import pytest

from prtcl_gb300.dsl.check import MAT, REAL, VEC, resolve
from prtcl_gb300.dsl.cuda import generate, generate_all
from prtcl_gb300.dsl.parser import BinOp, Compute, DslError, ForeachParticle, parse, parse_one

HERE = os.path.dirname(__file__)
TEST_SCHEMES = os.path.join(HERE, "dsl", "sph_test_schemes.prtcl")


def _reference_schemes():
    """The reference's own scheme sources, where its checkout is present
    (located by the oracle's build recipe)."""
    from oracle import ref_build
    root = ref_build.reference_root()
    return os.path.join(root, "share", "schemes") if root else ""


def _scheme(body, groups=None, glob="field hs = real smoothing_scale;"):
    groups = groups or """
      groups liquid {
        select type fluid;
        varying field pos = real[] position;
        varying field vel = real[] velocity;
        varying field dens = real density;
        varying field mass = real mass;
        varying field mat = real[][] some_matrix;
        uniform field dens0 = real rest_density;
      }"""
    return f"scheme s {{ {groups} global {{ {glob} }} procedure p {{ {body} }} }}"


def test_test_schemes_parse_resolve_and_generate():
    src = open(TEST_SCHEMES).read()
    schemes = parse(src)
    assert [s.name for s in schemes] == ["t_density", "t_volume", "t_sesph", "t_iisph", "t_motion", "t_viscosity",
                                         "t_bounds", "t_tally", "t_selectors", "t_wkbb18", "t_scalar_pcg"]
    for s in schemes:
        resolve(s)
    cu = generate_all(schemes)
    assert cu.count('register_scheme("prtcl::schemes::') == len(schemes)
    assert "extern \"C\" void prtcl_gpu_plugin_init()" in cu


def test_left_fold_and_literals():
    s = parse_one(_scheme("foreach liquid particle i { compute dens.i = mass.i * 2 / dens0.i - 0.5 + 1e-9; }"))
    resolve(s)
    comp = s.procedures[0].body[0].body[0]
    assert isinstance(comp, Compute)
    # ((((m * 2) / rho0) - 0.5) + 1e-9)
    e = comp.arg
    assert isinstance(e, BinOp) and e.op == "+"
    assert e.lhs.op == "-" and e.lhs.lhs.op == "/" and e.lhs.lhs.lhs.op == "*"
    cu = generate(s)
    assert "(((((rd(p.v_mass, i) * float(2)) / rd(p.u_dens0)) - float(0.5)) + float(1e-9))" in cu


def test_types():
    s = parse_one(_scheme("""
      foreach liquid particle i {
        local a : real[] = vel.i * 2;
        local b : real[][] = outer_product(a, pos.i) * mat.i;
        local c : real = dot(b * a, a) + trace(b) + norm(a);
        foreach liquid neighbor j {
          compute vel.i += mass.j * kernel_gradient_h(pos.i - pos.j, hs);
        }
      }"""))
    info = resolve(s)
    loop = s.procedures[0].body[0]
    assert isinstance(loop, ForeachParticle)
    types = [info.types[id(st.init)] for st in loop.body[:3]]
    assert types == [VEC, MAT, REAL]


@pytest.mark.parametrize("body,msg", [
    ("foreach liquid particle i { compute nope.i = 1; }", "no field 'nope'"),
    ("foreach liquid particle i { compute dens.i = frob(1); }", "unknown function"),
    ("foreach liquid particle i { foreach liquid neighbor j { compute dens.j = 1; } }", "neighbour's field"),
    ("foreach liquid particle i { reduce dens.i += 1; }", "reduce into anything but"),
    ("foreach liquid particle i { foreach liquid particle k { compute dens.k = 1; } }", "unexpected statement"),
    ("foreach liquid particle i { compute dens.i = pos.i; }", "cannot assign"),
    ("foreach liquid particle i { compute dens.i = vel.i * pos.i; }", "use dot or outer_product"),
    ("foreach nothing particle i { compute dens.i = 1; }", "unknown groups"),
    ("compute hs = q;", "unknown name 'q'"),
    ("foreach liquid particle i { compute hs = 1; }", "inside a particle loop"),
])
def test_errors(body, msg):
    with pytest.raises(DslError, match=msg):
        resolve(parse_one(_scheme(body)))


def test_syntax_error_position():
    with pytest.raises(DslError, match=r"line 2 column"):
        parse("scheme s {\n  procedure p { compute = ; }\n}")


def test_unsupported_field_types():
    """Declared, the field is created at load; used, it is an error."""
    groups = """
      groups liquid {
        select type fluid;
        varying field dens = real density;
        varying field cell = integer[2] some_cell;
      }"""
    s = parse_one(_scheme("foreach liquid particle i { compute dens.i = 1; }", groups=groups))
    cu = generate(s)
    assert 'add_varying("some_cell"' in cu and "v_cell" not in cu
    s = parse_one(_scheme("foreach liquid particle i { compute dens.i = cell.i[0]; }", groups=groups))
    with pytest.raises(DslError):
        generate(s)


def test_solve_pcg_needs_the_solver_fields():
    src = _scheme("""
      solve pcg real[] over liquid particle f {
        setup right_hand_side into r { compute r.f = vel.f; }
        setup guess into r { compute r.f = vel.f; }
        product preconditioner with x into r { compute r.f = x.f; }
        product system with x into r { compute r.f = x.f; }
        apply x { compute vel.f = x.f; }
      }""")
    s = parse_one(src)
    resolve(s)  # the language accepts it
    with pytest.raises(DslError, match="pcg_max_error"):
        generate(s)


def test_solve_pcg_parts_are_required():
    src = _scheme("""
      solve pcg real[] over liquid particle f {
        setup guess into r { compute r.f = vel.f; }
        apply x { compute vel.f = x.f; }
      }""")
    with pytest.raises(DslError, match="needs setup right_hand_side"):
        resolve(parse_one(src))


def test_reference_schemes():
    """Every scheme of the reference parses, resolves and generates."""
    root = _reference_schemes()
    if not os.path.isdir(root):
        pytest.skip("the reference's scheme sources are not present")
    generated = []
    for f in sorted(os.listdir(root)):
        if not f.endswith(".prtcl"):
            continue
        for s in parse(open(os.path.join(root, f)).read()):
            resolve(s)
            try:
                generate(s, prefix="gen_")
                generated.append(s.name)
            except DslError as ex:
                raise AssertionError((s.name, ex))
    assert len(generated) == 14


def test_reference_schemes_compile_and_register(gpu_lib):
    """The plugin of all 14 reference schemes compiles for sm_103a, loads and
    registers every scheme, each with the procedures of its source
    (registration and the procedure table need no device)."""
    from prtcl_gb300.core import get_scheme_names, make_scheme
    from prtcl_gb300.dsl.build import compile_scheme
    root = _reference_schemes()
    if not os.path.isdir(root):
        pytest.skip("the reference's scheme sources are not present")
    text = "\n".join(open(os.path.join(root, f)).read() for f in sorted(os.listdir(root)) if f.endswith(".prtcl"))
    names = compile_scheme(text, prefix="ref_")
    assert len(names) == 14
    registered = set(get_scheme_names())
    assert all(n in registered for n in names)
    for sc, full in zip(parse(text), names):
        assert sorted(make_scheme(full).get_procedure_names()) == sorted(p.name for p in sc.procedures), sc.name


def test_reference_scheme_fixture_is_current():
    """tests/golden/reference_schemes_plugin.cu (run on the device by
    tests/test_gpu_reference_schemes.py) is what the generator emits now
    for the reference's scheme sources."""
    import json
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_reference_schemes as mk
    from oracle import ref_build
    root = ref_build.reference_root()
    if not root or not os.path.isdir(_reference_schemes()):
        pytest.skip("the reference's scheme sources are not present")
    names, cu, meta = mk.generate(root)
    with open(mk.OUT) as f:
        assert f.read() == cu, "regenerate with tests/golden/make_reference_schemes.py"
    with open(mk.META) as f:
        assert json.load(f) == meta
