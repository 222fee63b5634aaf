// Writes every dump kind of vtk_dump.hpp from fixed synthetic data into the
// directory argv[1] (test driver of tests/test_vtk_dump.py).
#include <string>
#include <vector>

#include "vtk_dump.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  const int n = 5;
  std::vector<double> x(3 * n), ux(3 * n), f(3 * n);
  std::vector<int> img(n), tags(n), mols(n), types(n);
  for (int i = 0; i < 3 * n; ++i) {
    x[i] = -3.25 + 1.0 / 3.0 * i;
    ux[i] = 100.0 * x[i] + 1e-7 * i;
    f[i] = (i % 2 ? -1 : 1) * 1.2345678901e-5 * (i + 1);
  }
  for (int i = 0; i < n; ++i) {
    img[i] = 512 * 512 * (i % 3) + i;
    tags[i] = i + 1;
    mols[i] = i / 3;
    types[i] = i % 2;
  }
  phafd_dump::Atoms a;
  a.n = n;
  a.x = x.data(); a.ux = ux.data(); a.f = f.data(); a.images = img.data();
  a.tags = tags.data(); a.mols = mols.data(); a.types = types.data();
  for (int k = 0; k < 3; ++k) { a.boxlo[k] = -16.0; a.boxhi[k] = 16.0 + k; }
  const int nx = 3, ny = 4, nz = 5;
  std::vector<double> phi(nx * ny * nz), mu(nx * ny * nz);
  for (int i = 0; i < nx * ny * nz; ++i) { phi[i] = 0.5 + 0.01 * i; mu[i] = -1.0 / (i + 1); }
  phafd_dump::Grid g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.boxlo[0] = -1.5; g.boxlo[1] = -2.0; g.boxlo[2] = -2.5;
  g.spacing[0] = 1.0; g.spacing[1] = 1.0; g.spacing[2] = 1.0;
  g.fields["phi"] = phi.data();
  g.fields["chempot"] = mu.data();
  // an ftgrid file: the half spectrum [ky][kz][kx] of a 6 (x) x 4 (y) x 5 (z)
  // grid, spacing dq (x, then the z and y periods), origin 0
  std::vector<double> sk(4 * 5 * 4);
  for (size_t i = 0; i < sk.size(); ++i) sk[i] = 1.0 / (i + 3);
  phafd_dump::Grid ft;
  ft.nx = 4; ft.ny = 5; ft.nz = 4;
  ft.spacing[0] = 2 * 3.141592 / 12.0; ft.spacing[1] = 2 * 3.141592 / 10.0; ft.spacing[2] = 2 * 3.141592 / 8.0;
  ft.fields["c_sk"] = sk.data();
  using V = std::vector<std::string>;
  const std::vector<V> specs = {
      {"a1", "atom/owned", dir + "/sub/atoms", "10", "attributes", "8", "x", "ux", "F", "ix", "ID", "molID", "type", "label"},
      {"a2", "atom/all", dir + "/atoms2", "5", "attributes", "2", "x", "F", "decimalplaces", "4", "fmt", "e"},
      {"a3", "atom/owned", dir + "/atoms3", "5", "attributes", "1", "x", "decimalplaces", "3"},
      {"a4", "atom/owned", dir + "/atoms4", "5", "attributes", "1", "x", "fmt", "e"},
      {"g1", "grid", dir + "/grid", "5", "attributes", "2", "phi", "chempot"},
      {"l1", "lammpsatom", dir + "/lmp", "5", "attributes", "4", "ID", "type", "x", "F"},
  };
  for (auto& v : specs) {
    const phafd_dump::Spec s = phafd_dump::parse(v);
    phafd_dump::collection_header(s);
    phafd_dump::write_step(s, 0, 1e-3, &a, &g);
    phafd_dump::write_step(s, 10, 1e-3, &a, &g);
    phafd_dump::collection_footer(s);
  }
  const phafd_dump::Spec fs = phafd_dump::parse(V{"s1", "ftgrid", dir + "/spec", "5", "attributes", "1", "c_sk"});
  phafd_dump::collection_header(fs);
  phafd_dump::write_step(fs, 5, 1e-3, &a, &ft);
  phafd_dump::collection_footer(fs);
  return 0;
}
