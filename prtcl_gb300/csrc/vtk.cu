// Frame output of a group as a legacy ASCII VTK polydata file, the format
// of the reference's SaveVTK (util/save_vtk.cpp:57-128): the header, POINTS
// from "position", then POINT_DATA with the vectors velocity and
// acceleration, the scalar _index, the scalars mass, volume, density,
// pressure, time_of_birth and implicit_function, and the vector
// implicit_function_gradient, each present field in that order.  Values are
// printed as std::fixed with the default precision 6 ("%f"); the index as an
// integer.
#include "model.hpp"

#include <cstdio>
#include <vector>

namespace prtcl_gpu {

namespace {

struct File {
  std::FILE *f;
  explicit File(std::string const &path) : f(std::fopen(path.c_str(), "w")) {
    if (!f) throw Error("vtk: cannot write " + path);
  }
  ~File() {
    if (f) std::fclose(f);
  }
};

void write_field(std::FILE *f, VaryingField const &v, size_t count, cudaStream_t s) {
  if (v.type.ctype != CType::F32 || v.type.rank > 1) throw Error("vtk: only real and real[N] fields are written");
  size_t comps = v.type.comps();
  std::vector<float> buf(count * comps);
  download_varying(v, count, buf.data(), count, s);
  for (size_t i = 0; i < count; ++i) {
    for (size_t c = 0; c < comps; ++c) std::fprintf(f, c ? " %f" : "%f", double(buf[i * comps + c]));
    std::fputc('\n', f);
  }
}

} // namespace

void save_vtk(Group &g, std::string const &path, cudaStream_t s) {
  File out(path);
  std::FILE *f = out.f;
  size_t n = g.count;
  auto field = [&](char const *name) { return g.find_varying(name); };
  std::fprintf(f, "# vtk DataFile Version 2.0\n%s %s\nASCII\nDATASET POLYDATA\n", g.name.c_str(), g.type.c_str());
  VaryingField *x = field("position");
  if (!x) throw Error("vtk: group '" + g.name + "' has no position field");
  std::fprintf(f, "POINTS %zu float\n", n);
  write_field(f, *x, n, s);
  std::fprintf(f, "POINT_DATA %zu\n", n);
  for (char const *name : {"velocity", "acceleration"})
    if (VaryingField *v = field(name)) {
      std::fprintf(f, "VECTORS %s float\n", name);
      write_field(f, *v, n, s);
    }
  std::fprintf(f, "SCALARS _index float 1\nLOOKUP_TABLE default\n");
  for (size_t i = 0; i < n; ++i) std::fprintf(f, "%zu\n", i);
  for (char const *name : {"mass", "volume", "density", "pressure", "time_of_birth", "implicit_function"})
    if (VaryingField *v = field(name)) {
      std::fprintf(f, "SCALARS %s float 1\nLOOKUP_TABLE default\n", name);
      write_field(f, *v, n, s);
    }
  if (VaryingField *v = field("implicit_function_gradient")) {
    std::fprintf(f, "VECTORS implicit_function_gradient float\n");
    write_field(f, *v, n, s);
  }
  if (std::fflush(f) != 0) throw Error("vtk: write failed");
}

} // namespace prtcl_gpu
