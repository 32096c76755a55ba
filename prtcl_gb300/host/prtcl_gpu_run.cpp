// prtcl_gpu_run: a native driver of the GPU library, written against the C++
// facade (include/prtcl_gpu.hpp) the way prtcl's own drivers are written
// against prtcl::Model / Neighborhood / SchemeBase.
//
//   prtcl_gpu_run <model.bin> <steps> <out.bin> [--viscosity] [--vtk-every K --vtk-prefix P]
//
// Loads a model archive in the reference's native binary format (one written
// by prtcl itself or by prtcl_gb300's Model.save), runs `steps` steps of the
// step loop of the reference's driver script
// (share/scripts/prtcl-lua.example.lua:363-461) and saves the final model:
// grid update with a permute every 8 steps, density, gravity, velocity
// integration, IISPH set-up and the relaxed-Jacobi loop (on the device:
// iisph.solve_pressure, with the globals iisph_maximum_iterations and
// iisph_maximum_density_error), velocity integration, optionally the WKBB18
// implicit viscosity, position integration.  The clock starts at the
// archive's current_time and advances by time_step, kept in double like the
// script's.  Prints one line per step with the Jacobi and PCG iterations.
#include "prtcl_gpu.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

using namespace prtcl_gpu;

namespace {
std::string full(char const *name) { return std::string("prtcl::schemes::") + name + "[T=f32, N=3, K=Cubic Spline]"; }

int usage() {
  std::fprintf(stderr,
               "usage: prtcl_gpu_run <model.bin> <steps> <out.bin> [--viscosity] [--vtk-every K --vtk-prefix P]\n");
  return 2;
}
} // namespace

int main(int argc, char **argv) {
  if (argc < 4) return usage();
  std::string in = argv[1], out = argv[3];
  int steps = std::atoi(argv[2]);
  bool viscosity = false;
  int vtk_every = 0;
  std::string vtk_prefix = "frame";
  for (int k = 4; k < argc; ++k) {
    if (!std::strcmp(argv[k], "--viscosity")) viscosity = true;
    else if (!std::strcmp(argv[k], "--vtk-every") && k + 1 < argc) vtk_every = std::atoi(argv[++k]);
    else if (!std::strcmp(argv[k], "--vtk-prefix") && k + 1 < argc) vtk_prefix = argv[++k];
    else return usage();
  }
  if (steps < 0) return usage();
  try {
    Model model;
    model.Load(in);
    auto density = SchemeRegistry::NewScheme(full("density"));
    auto gravity = SchemeRegistry::NewScheme(full("gravity"));
    auto euler = SchemeRegistry::NewScheme(full("symplectic_euler"));
    auto iisph = SchemeRegistry::NewScheme(full("iisph"));
    auto wkbb18 = SchemeRegistry::NewScheme(full("wkbb18"));
    for (auto *s : {density.get(), gravity.get(), euler.get(), iisph.get(), wkbb18.get()}) s->Load(model);
    float h = 0.0f, dt = 0.0f, t0 = 0.0f;
    model.GetGlobal("smoothing_scale", &h);
    model.GetGlobal("time_step", &dt);
    model.GetGlobal("current_time", &t0);
    Neighborhood nhood;
    nhood.Load(model);
    nhood.SetRadius(2.0 * double(h));
    double t = double(t0);
    int since_permute = 0;
    for (int step = 0; step < steps; ++step) {
      float tf = float(t);
      model.SetGlobal("current_time", &tf);
      nhood.Update();
      if (++since_permute >= 8) {
        nhood.Permute(model);
        since_permute = 0;
      }
      density->RunProcedure("compute_density", nhood);
      gravity->RunProcedure("initialize_acceleration", nhood);
      euler->RunProcedure("integrate_velocity_with_hard_fade", nhood);
      iisph->RunProcedure("setup", nhood);
      iisph->RunProcedure("solve_pressure", nhood);
      euler->RunProcedure("integrate_velocity_with_hard_fade", nhood);
      int pcg = -1;
      if (viscosity) {
        wkbb18->RunProcedure("compute_diagonal", nhood);
        wkbb18->RunProcedure("accumulate_acceleration", nhood);
        model.GetGroup("f").GetUniform("wkbb18_iterations", &pcg);
        euler->RunProcedure("integrate_velocity_with_hard_fade", nhood);
      }
      euler->RunProcedure("integrate_position", nhood);
      t += double(dt);
      int jac = 0;
      model.GetGlobal("iisph_iterations", &jac);
      std::printf("step %d t %.6f jacobi %d pcg %d\n", step + 1, t, jac, pcg);
      if (vtk_every > 0 && (step + 1) % vtk_every == 0)
        for (auto const &g : model.GetGroupNames())
          model.GetGroup(g).SaveVTK(vtk_prefix + "." + g + "." + std::to_string(step + 1) + ".vtk");
    }
    model.Save(out);
  } catch (std::exception const &e) {
    std::fprintf(stderr, "prtcl_gpu_run: %s\n", e.what());
    return 1;
  }
  return 0;
}
