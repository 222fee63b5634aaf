// Driver of the reference's own code, built against the stand-ins under
// include/ (test infrastructure: it produces reference outputs that pin the
// oracle; nothing in the product runs it).
//
//   phafd_ref -in SCRIPT [-var NAME VALUE ...]
//
// runs SCRIPT through the reference's Input::read, exactly as its main()
// does, then writes the final state to the file named by the environment
// variable REFPIN_OUT as a sequence of records:
//   char name[32] (NUL padded), int32 dtype (0 float64, 1 int32, 2 int64),
//   int32 ndim, int64 dims[ndim], raw little-endian data.
// Grid fields are written over their logical extents ([z][y][x]; spectra
// [ky][kz][kx] as (re, im) pairs), beads over every copy the atom arrays hold
// (owned, then gathered local and ghost copies), each compute's array as
// last evaluated, neighbor lists as (ilist, numneigh, concatenated
// neighbors) per list.
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <fftw3-mpi.h>
#include <mpi.h>

#include "atom.hpp"
#include "compute.hpp"
#include "fix.hpp"
#include "fixgrid_floryhuggins.hpp"
#include "fftw_arr/array3d.hpp"
#include "grid.hpp"
#include "input.hpp"
#include "integrate.hpp"
#include "neigh_list.hpp"
#include "neighbor.hpp"
#include "phafd.hpp"

namespace {

struct Writer {
  std::ofstream f;
  explicit Writer(const char* path) : f(path, std::ios::binary) {}
  void head(const std::string& name, int32_t dtype, const std::vector<int64_t>& dims) {
    char nm[32] = {0};
    std::strncpy(nm, name.c_str(), 31);
    f.write(nm, 32);
    f.write(reinterpret_cast<const char*>(&dtype), 4);
    const int32_t nd = (int32_t)dims.size();
    f.write(reinterpret_cast<const char*>(&nd), 4);
    f.write(reinterpret_cast<const char*>(dims.data()), 8 * dims.size());
  }
  void f64(const std::string& name, const std::vector<double>& v, std::vector<int64_t> dims) {
    head(name, 0, dims);
    f.write(reinterpret_cast<const char*>(v.data()), 8 * v.size());
  }
  void i32(const std::string& name, const std::vector<int>& v, std::vector<int64_t> dims) {
    head(name, 1, dims);
    f.write(reinterpret_cast<const char*>(v.data()), 4 * v.size());
  }
  void i64(const std::string& name, const std::vector<int64_t>& v) {
    head(name, 2, {(int64_t)v.size()});
    f.write(reinterpret_cast<const char*>(v.data()), 8 * v.size());
  }
};

void real_field(Writer& w, const std::string& name, fftwArr::array3D<double>* a) {
  if (!a) return;
  std::vector<double> v;
  v.reserve((size_t)a->Nx() * a->Ny() * a->Nz());
  for (int i = 0; i < a->Nz(); ++i)
    for (int j = 0; j < a->Ny(); ++j)
      for (int k = 0; k < a->Nx(); ++k) v.push_back((*a)(i, j, k));
  w.f64(name, v, {a->Nz(), a->Ny(), a->Nx()});
}

void complex_field(Writer& w, const std::string& name, fftwArr::array3D<std::complex<double>>* a) {
  if (!a) return;
  std::vector<double> v;
  for (int i = 0; i < a->Nz(); ++i)
    for (int j = 0; j < a->Ny(); ++j)
      for (int k = 0; k < a->Nx(); ++k) {
        v.push_back((*a)(i, j, k).real());
        v.push_back((*a)(i, j, k).imag());
      }
  w.f64(name, v, {a->Nz(), a->Ny(), a->Nx(), 2});
}

void write_state(PHAFD_NS::PHAFD* p, const char* path) {
  Writer w(path);
  auto& g = p->grid;
  if (g && g->gridset) {
    real_field(w, "phi", g->phi.get());
    real_field(w, "chempot", g->chempot.get());
    real_field(w, "gradx", g->gradphi[0].get());
    real_field(w, "grady", g->gradphi[1].get());
    real_field(w, "gradz", g->gradphi[2].get());
    complex_field(w, "ft_phi", g->ft_phi.get());
    complex_field(w, "ft_chempot", g->ft_chempot.get());
  }
  auto& a = p->atoms;
  const int64_t n = a->xs.cols();
  std::vector<double> x(a->xs.data(), a->xs.data() + 3 * n);
  w.f64("x", x, {n, 3});
  const int64_t nu = a->uxs.cols();
  w.f64("ux", std::vector<double>(a->uxs.data(), a->uxs.data() + 3 * nu), {nu, 3});
  const int64_t nf = a->Fs.cols();
  w.f64("f", std::vector<double>(a->Fs.data(), a->Fs.data() + 3 * nf), {nf, 3});
  w.i32("tags", std::vector<int>(a->tags.begin(), a->tags.begin() + n), {n});
  w.i32("types", std::vector<int>(a->types.begin(), a->types.begin() + n), {n});
  w.i32("images", std::vector<int>(a->images.begin(), a->images.begin() + a->nowned), {a->nowned});
  w.i32("labels", std::vector<int>(a->labels.begin(), a->labels.begin() + n), {n});
  std::vector<int64_t> counters = {(int64_t)a->nowned, (int64_t)p->integrate->timestep,
                                   (int64_t)p->neighbor->get_ncalls()};
  int64_t less = 0, great = 0;
  for (auto& fx : p->fixes)
    if (auto* fh = dynamic_cast<PHAFD_NS::FixGridFloryHuggins*>(fx.get())) {
      less += fh->num_less_zero;
      great += fh->num_great_zero;
    }
  counters.push_back(less);
  counters.push_back(great);
  w.i64("counters", counters);  // nowned, timestep, neighbor calls, FH reflections (phi <= 0, phi >= 1)
  for (auto& c : p->computes)  // each compute's array as last evaluated
    w.f64("compute_" + c->name, c->array, {(int64_t)c->array.size()});
  auto& lists = p->neighbor->neigh_lists;
  for (size_t l = 0; l < lists.size(); ++l) {
    auto& L = *lists[l];
    std::vector<int> flat;
    for (size_t ii = 0; ii < L.ilist.size(); ++ii)
      for (int jj = 0; jj < L.numneigh[ii]; ++jj) flat.push_back(L.firstneigh[ii][jj]);
    const std::string tag = "list" + std::to_string(l) + "_";
    w.i32(tag + "ilist", L.ilist, {(int64_t)L.ilist.size()});
    w.i32(tag + "numneigh", L.numneigh, {(int64_t)L.numneigh.size()});
    w.i32(tag + "neigh", flat, {(int64_t)flat.size()});
    w.i32(tag + "kind", std::vector<int>{L.list_type, L.list_style}, {2});
  }
}

}  // namespace

int main(int argc, char** argv) {
  MPI_Init(nullptr, nullptr);
  fftw_mpi_init();
  int rc = 0;
  try {
    auto* phafd = new PHAFD_NS::PHAFD(MPI_COMM_WORLD, argc, argv);
    phafd->input->read();
    const char* out = std::getenv("REFPIN_OUT");
    if (out) write_state(phafd, out);
    delete phafd;
  } catch (const std::exception& e) {
    std::cerr << "reference error: " << e.what() << std::endl;
    rc = 1;
  }
  fftw_mpi_cleanup();
  MPI_Finalize();
  return rc;
}
