"""Known-answer tests of the CPU oracle (no GPU): the SPH kernel, the Morton
order, the grid vs brute force, permutation, the IISPH loop on a resting
block and the WKBB18 PCG vs a dense FP64 solve."""
import itertools
import math

import numpy as np
import pytest

from prtcl_gb300 import driver, scenes
from tests.helpers import point_scene


# ---- Morton order: restated comparator vs an explicit 96-bit interleave ----

def unsign(i):
    return (i + 0x7FFFFFFF) & 0xFFFFFFFF


def interleave_key(gi):
    u = [unsign(int(c)) for c in gi]
    k = 0
    for bit in range(31, -1, -1):
        for d in range(3):
            k = (k << 1) | ((u[d] >> bit) & 1)
    return k


def morton_compare(l, r):
    def less_msb(a, b):
        return a < b and a < (a ^ b)
    msd = 0
    for d in (1, 2):
        if less_msb(unsign(l[msd]) ^ unsign(r[msd]), unsign(l[d]) ^ unsign(r[d])):
            msd = d
    a, b = unsign(l[msd]), unsign(r[msd])
    return (a > b) - (a < b)


def test_morton_compare_matches_interleave():
    rng = np.random.default_rng(0)
    edge = [-2**31 + 1, -2, -1, 0, 1, 2, 2**31 - 1, 255, 256, -256, -257]
    vals = list(rng.integers(-2**31 + 1, 2**31 - 1, 300)) + list(rng.integers(-40, 40, 300)) + edge
    pts = [tuple(int(v) for v in rng.choice(vals, 3)) for _ in range(3000)]
    pts += list(itertools.product(edge[:6], repeat=3))
    for a, b in zip(pts, pts[1:] + pts[:1]):
        ka, kb = interleave_key(a), interleave_key(b)
        assert morton_compare(a, b) == (ka > kb) - (ka < kb), (a, b)


# ---- kernel ---------------------------------------------------------------

def W(r, h):
    q = abs(r) / h
    s = 1.0 / (4.0 * math.pi)
    res = 0.0
    if q < 1:
        res -= 4 * (1 - q) ** 3
    if q < 2:
        res += (2 - q) ** 3
    return s * res / h**3


def test_kernel_normalisation_and_values():
    h = 0.025
    # integral of W over its support (radial quadrature) is 1
    rs = np.linspace(0, 2 * h, 20001)
    vals = np.array([W(r, h) for r in rs])
    integral = np.trapezoid(4 * np.pi * rs**2 * vals, rs)
    assert abs(integral - 1.0) < 1e-6
    # values at q = 0, 0.5, 1, 1.5, 2 from the formula
    s = 1 / (4 * np.pi) / h**3
    for q, expect in [(0, 4 * s), (0.5, (1.5**3 - 4 * 0.5**3) * s), (1, s), (1.5, 0.5**3 * s), (2, 0.0)]:
        assert W(q * h, h) == pytest.approx(expect, rel=1e-12, abs=1e-9)


def test_oracle_density_of_lattice(oracle_mod):
    """Density at the centre of a large lattice with m = h^3 rho0 equals
    rho0 * h^3 * sum_j W(x_j) computed independently."""
    s = 0.025
    ax = (np.arange(-6, 7)) * s
    pts = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    o = oracle_mod.Scene(np.float64)
    o.add_group("f", "fluid")
    o.resize("f", len(pts))
    o.set_varying("f", "position", pts.astype(np.float64))
    o.set_varying("f", "mass", np.full(len(pts), s**3 * 1000.0))
    o.set_uniform("f", "rest_density", 1000.0)
    o.set_global("smoothing_scale", s)
    o.add_group("b", "boundary")
    o.resize("b", 0)
    o.set_radius(2 * s)
    o.update()
    o.run("density", "compute_density")
    rho = o.get_varying("f", "density")
    c = int(np.argmin((pts.astype(np.float64) ** 2).sum(1)))
    expect = sum(s**3 * 1000.0 * W(np.linalg.norm(p), s) for p in pts.astype(np.float64)
                 if np.linalg.norm(p) < 2 * s)
    assert rho[c] == pytest.approx(expect, rel=1e-12)


# ---- grid vs brute force ----------------------------------------------------

def brute(pts_by_group, q, i, r):
    x = pts_by_group[q][i].astype(np.float32)
    out = []
    for g, P in enumerate(pts_by_group):
        d = P.astype(np.float32) - x
        # float32 squared norm in the order x^2 + (y^2 + z^2)
        d2 = d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        out.append(set(np.nonzero(d2.astype(np.float64) < r * r)[0].tolist()))
    return out


def test_grid_matches_brute_force(oracle_mod):
    rng = np.random.default_rng(3)
    s = 0.02
    ax = (np.arange(-8, 8) + 0.5) * s
    lat = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    rnd = (rng.random((2000, 3)) * 0.4 - 0.2).astype(np.float32)
    o = oracle_mod.Scene(np.float32)
    point_scene(o, [("a", "fluid", lat, []), ("b", "boundary", rnd, [])], 2 * np.float64(np.float32(s)))
    o.update()
    r = 2 * np.float64(np.float32(s))
    P = [lat, rnd]
    for q, n in ((0, len(lat)), (1, len(rnd))):
        for i in rng.integers(0, n, 150):
            got = o.neighbors(q, int(i), 2)
            exp = brute(P, q, int(i), r)
            for g in range(2):
                assert set(got[g].tolist()) == exp[g]
                assert len(got[g]) == len(exp[g])
    # grid structure: ranges partition the sorted handles, cells in Morton order
    g = o.grid()
    assert (g["cell_range"][1:, 0] == g["cell_range"][:-1, 1]).all()
    keys = [interleave_key(c) for c in g["cell_gi"]]
    assert keys == sorted(keys) and len(set(keys)) == len(keys)


def test_permute_reorders_into_cell_order(oracle_mod):
    rng = np.random.default_rng(9)
    pts = rng.random((5000, 3)).astype(np.float32)
    tag = np.arange(5000, dtype=np.float32)
    o = oracle_mod.Scene(np.float32)
    point_scene(o, [("a", "fluid", pts, [])], 0.05)
    o.set_varying("a", "tag", tag)
    o.update()
    o.permute()
    t = o.get_varying("a", "tag")
    x = o.get_varying("a", "position", 3)
    assert np.array_equal(pts[t.astype(np.int64)], x)
    g = o.grid()
    assert np.array_equal(g["sorted"] & 0x0FFFFFFF, np.arange(5000, dtype=np.uint32))


# ---- IISPH on a resting block; PCG vs dense solve ---------------------------

def test_iisph_resting_block_converges(oracle_mod):
    sc = scenes.dam_break(fluid_cells=(10, 10, 10), spacing=0.025, box=(0.25, 0.25, 0.25))
    p = dict(driver.DAM_BREAK_27K)
    o = oracle_mod.Scene(np.float32)
    driver.setup_dam_break(o, sc, p)
    loop = driver.StepLoop(o, p)
    for _ in range(5):
        st = loop.step()
    assert st["relative_aprde"] < p["eta"] or st["jacobi_iterations"] == p["max_iters"]
    assert (o.get_varying("f", "pressure") >= 0).all()


def test_pcg_matches_dense_solve(oracle_mod):
    sc = scenes.dam_break(fluid_cells=(6, 6, 6), spacing=0.025, box=(0.2, 0.2, 0.2))
    p = dict(driver.DAM_BREAK_27K, viscosity=True, wkbb18_maximum_error=1e-7, wkbb18_maximum_iterations=200)
    o = oracle_mod.Scene(np.float64)
    driver.setup_dam_break(o, sc, p)
    rng = np.random.default_rng(2)
    nf = len(sc["fluid"])
    v = rng.standard_normal((nf, 3))
    o.set_varying("f", "velocity", v)
    o.update()
    o.run("density", "compute_density")
    o.run("wkbb18", "compute_diagonal")
    o.run("wkbb18", "accumulate_acceleration")
    x = v + o.get_varying("f", "wkbb18_velocity_delta", 3)
    # dense system A x = v of wkbb18.accumulate_acceleration
    h, dt, mu, mub, rho0 = float(np.float32(0.025)), float(np.float32(1e-3)), 10.0, 10.0, 1000.0
    X = o.get_varying("f", "position", 3)
    XB = o.get_varying("b", "position", 3)
    VB = o.get_varying("b", "volume")
    m = o.get_varying("f", "mass")
    rho = o.get_varying("f", "density")
    A = np.eye(3 * nf)

    def gradW(d):
        r = np.linalg.norm(d)
        if r < np.sqrt(np.finfo(np.float64).eps):
            return np.zeros(3)
        q = r / h
        s = 1 / (4 * np.pi)
        dq = 0.0
        if q < 1:
            dq += 12 * (1 - q) ** 2
        if q < 2:
            dq -= 3 * (2 - q) ** 2
        return (-abs(s * dq / h**4) / r) * d
    for i in range(nf):
        for j in range(nf):
            d = X[i] - X[j]
            if d @ d >= (2 * h) ** 2:
                continue
            c = 10 * (mu / rho[i]) * (m[j] / rho[j]) / (d @ d + 0.01 * h * h)
            blk = dt * c * np.outer(gradW(d), d)
            A[3 * i:3 * i + 3, 3 * i:3 * i + 3] -= blk
            A[3 * i:3 * i + 3, 3 * j:3 * j + 3] += blk
        for j in range(len(XB)):
            d = X[i] - XB[j]
            if d @ d >= (2 * h) ** 2:
                continue
            c = 10 * (mub / rho[i]) * (rho0 * VB[j] / rho[i]) / (d @ d + 0.01 * h * h)
            A[3 * i:3 * i + 3, 3 * i:3 * i + 3] -= dt * c * np.outer(gradW(d), d)
    xs = np.linalg.solve(A, v.reshape(-1)).reshape(nf, 3)
    # the PCG stops at |r|^2 < tol^2 |b|^2: its iterate satisfies the dense
    # system to that residual and is close to the dense solution
    res = np.linalg.norm(A @ x.reshape(-1) - v.reshape(-1)) / np.linalg.norm(v)
    assert res < 1e-6
    assert np.abs(x - xs).max() < 1e-4 * max(1.0, np.abs(xs).max())
    assert int(o.get_uniform("f", "wkbb18_iterations")) >= 1


def test_pseudo_inverse_matches_numpy(oracle_mod):
    """The 3x3 pseudo-inverse standing in for invert_pm (Eigen's complete
    orthogonal decomposition): full rank, rank 2, rank 1 and zero matrices
    against numpy's SVD-based pinv in float64."""
    rng = np.random.default_rng(8)
    full = rng.standard_normal((200, 3, 3))
    u = rng.standard_normal((100, 3, 2))
    r2 = u @ rng.standard_normal((100, 2, 3))
    r1 = rng.standard_normal((50, 3, 1)) @ rng.standard_normal((50, 1, 3))
    mats = np.concatenate([full, r2, r1, np.zeros((2, 3, 3)), np.eye(3)[None] * 1e-3]).astype(np.float32)
    got = oracle_mod.pinv3(mats).astype(np.float64)
    ref = np.linalg.pinv(mats.astype(np.float64), rcond=1e-5)
    scale = np.maximum(np.abs(ref).max(axis=(1, 2)), 1e-30)
    cond = np.linalg.cond(mats.astype(np.float64)[:200])
    err = np.abs(got - ref).max(axis=(1, 2)) / scale
    assert (err[:200] <= 2e-6 * np.maximum(cond, 1.0)).all()
    assert (err[200:] <= 1e-4).all()
    assert not got[350:352].any()  # pinv(0) = 0
    # Moore-Penrose conditions A A+ A = A and A+ A A+ = A+
    a = mats.astype(np.float64)
    np.testing.assert_allclose(a @ got @ a, a, atol=1e-4 * np.abs(a).max())
    np.testing.assert_allclose(got @ a @ got, got, atol=1e-3 * np.abs(got).max())
