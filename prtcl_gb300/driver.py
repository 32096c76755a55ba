"""Scene set-up and the dam-break step loop over the flat model API.

The step loop restates the driver script of the reference
(share/scripts/prtcl-lua.example.lua:363-461): grid update (with a permute
every 8 steps), density, gravity, velocity integration, IISPH set-up and the
relaxed-Jacobi pressure loop with its host-side convergence test, velocity
integration, optional WKBB18 implicit viscosity, position integration.

``setup_dam_break`` mirrors the scene set-up of the same script
(:122-186, :196-207, :288-316): fluid group ``f`` (type fluid, tag dynamic),
boundary group ``b`` (type boundary), mass = h^3 * rho0, search radius 2h,
update + permute, then ``aiast12.compute_volume`` for the wall volumes.

Any object with the flat API (``add_group``, ``add_tag``, ``resize``,
``set_varying``, ``get_varying``, ``set_uniform``, ``set_global``,
``get_global``, ``set_radius``, ``update``, ``permute``, ``run``) can be
driven: the device model of this package and the CPU oracle both provide it.
"""
from __future__ import annotations

import numpy as np

# 27,000 fluid particle dam break: spacing 0.025 m, smoothing scale = spacing,
# support / search radius = 2 * smoothing scale, rest density 1000 kg/m^3,
# gravity -9.81 m/s^2 along y, dt 1e-3 s, relaxation 0.5, stop at 0.1 %
# average density error or 100 Jacobi iterations.
DAM_BREAK_27K = dict(
    smoothing_scale=0.025,
    time_step=1e-3,
    rest_density=1000.0,
    gravity=(0.0, -9.81, 0.0),
    iisph_relaxation=0.5,
    eta=1e-3,
    max_iters=100,
    # particles are born before t = 0 with no fade-in, so the hard fade of the
    # velocity integration is open from the first step
    fade_duration=0.0,
    time_of_birth=-1.0,
    viscosity=False,
    dynamic_viscosity=10.0,
    boundary_dynamic_viscosity=10.0,
    wkbb18_maximum_error=1e-4,
    wkbb18_maximum_iterations=100,
    permute_every=8,
)

# 1,000,000 fluid particle dam break with WKBB18 implicit viscosity:
# kinematic viscosity 1e-2 m^2/s -> dynamic viscosity 10 Pa s, PCG tolerance
# 1e-4, at most 100 PCG iterations, dt 5e-4 s.
DAM_BREAK_1M = dict(DAM_BREAK_27K, smoothing_scale=0.0075, time_step=5e-4, viscosity=True)


def setup_dam_break(m, scene, p):
    """Create groups and fields of a dam-break scene on model ``m``."""
    nf, nb = len(scene["fluid"]), len(scene["boundary"])
    m.add_group("f", "fluid")
    m.add_tag("f", "dynamic")
    m.add_group("b", "boundary")
    m.resize("f", nf)
    m.resize("b", nb)
    h = np.float32(p["smoothing_scale"])
    rho0 = np.float32(p["rest_density"])
    m.set_global("smoothing_scale", float(h))
    m.set_global("time_step", float(np.float32(p["time_step"])))
    m.set_global("gravity", np.asarray(p["gravity"], np.float32).astype(np.float64))
    m.set_global("iisph_relaxation", float(np.float32(p["iisph_relaxation"])))
    m.set_global("fade_duration", float(np.float32(p["fade_duration"])))
    m.set_global("current_time", 0.0)
    m.set_global("maximum_speed", 0.0)
    # parameters of the device-side relaxed-Jacobi loop (iisph.solve_pressure)
    m.set_global("iisph_maximum_iterations", int(p["max_iters"]))
    m.set_global("iisph_maximum_density_error", float(np.float32(p["eta"])))
    m.set_global("iisph_iterations", 0)
    m.set_uniform("f", "rest_density", float(rho0))
    m.set_uniform("f", "dynamic_viscosity", float(np.float32(p["dynamic_viscosity"])))
    m.set_uniform("f", "wkbb18_maximum_error", float(np.float32(p["wkbb18_maximum_error"])))
    m.set_uniform("f", "wkbb18_maximum_iterations", int(p["wkbb18_maximum_iterations"]))
    m.set_uniform("b", "dynamic_viscosity", float(np.float32(p["boundary_dynamic_viscosity"])))
    m.set_varying("f", "position", scene["fluid"])
    m.set_varying("f", "velocity", np.zeros((nf, 3), np.float32))
    m.set_varying("f", "acceleration", np.zeros((nf, 3), np.float32))
    # mass = h * h * h * rho0 (the script computes it in double, stores f32)
    mass = np.float32(float(h) * float(h) * float(h) * float(rho0))
    m.set_varying("f", "mass", np.full(nf, mass, np.float32))
    m.set_varying("f", "time_of_birth", np.full(nf, np.float32(p["time_of_birth"]), np.float32))
    m.set_varying("b", "position", scene["boundary"])
    m.set_varying("b", "volume", np.zeros(nb, np.float32))
    m.set_radius(2.0 * float(h))
    m.update()
    m.permute()
    m.run("aiast12", "compute_volume")


class StepLoop:
    """The reference driver loop; ``t`` is kept in double like the script's
    virtual clock and written to ``current_time`` each step.

    ``device_loop=False`` runs the relaxed-Jacobi loop on the host exactly as
    the script does (iteration_pressure_acceleration + iteration_pressure,
    reading aprde after every iteration); ``device_loop=True`` runs the same
    loop as one procedure, ``iisph.solve_pressure``, on the device."""

    def __init__(self, m, p, device_loop=False):
        self.m, self.p = m, p
        self.device_loop = device_loop
        self.t = 0.0
        self.steps_since_permute = 0
        self.dt = float(np.float32(p["time_step"]))

    def step(self, quiet=False):
        """One step.  ``quiet`` (device loop only) reads nothing back: the
        step is queued without a host round trip and the returned counts are
        None (the device-loop statistics of the model hold them)."""
        m, p = self.m, self.p
        if quiet and self.device_loop:
            return self._quiet_step()
        self.steps_since_permute += 1
        m.set_global("current_time", float(np.float32(self.t)))
        m.update()
        if self.steps_since_permute >= p["permute_every"]:
            m.permute()
            self.steps_since_permute = 0
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("iisph", "setup")
        nprde = m.get_global("iisph_nprde")
        it, rel = 0, 0.0
        if self.device_loop:
            m.run("iisph", "solve_pressure")
            it = int(m.get_global("iisph_iterations"))
            rel = m.get_global("iisph_aprde") / nprde if nprde >= 1 else 0.0
        elif nprde >= 1:
            for it in range(1, p["max_iters"] + 1):
                m.set_global("iisph_aprde", 0.0)
                m.run("iisph", "iteration_pressure_acceleration")
                m.run("iisph", "iteration_pressure")
                rel = m.get_global("iisph_aprde") / nprde
                if it >= 2 and rel < p["eta"]:
                    break
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        pcg = -1
        if p.get("viscosity"):
            m.run("wkbb18", "compute_diagonal")
            m.run("wkbb18", "accumulate_acceleration")
            pcg = int(m.get_uniform("f", "wkbb18_iterations"))
            m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("symplectic_euler", "integrate_position")
        self.t += self.dt
        return {"jacobi_iterations": it, "relative_aprde": rel, "pcg_iterations": pcg}

    def _quiet_step(self):
        m, p = self.m, self.p
        self.steps_since_permute += 1
        m.set_global("current_time", float(np.float32(self.t)), asynchronous=True)
        m.update()
        if self.steps_since_permute >= p["permute_every"]:
            m.permute()
            self.steps_since_permute = 0
        m.run("density", "compute_density")
        m.run("gravity", "initialize_acceleration")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("iisph", "setup")
        m.run("iisph", "solve_pressure")
        m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        if p.get("viscosity"):
            m.run("wkbb18", "compute_diagonal")
            m.run("wkbb18", "accumulate_acceleration")
            m.run("symplectic_euler", "integrate_velocity_with_hard_fade")
        m.run("symplectic_euler", "integrate_position")
        self.t += self.dt
        return {"jacobi_iterations": None, "relative_aprde": None, "pcg_iterations": None}
