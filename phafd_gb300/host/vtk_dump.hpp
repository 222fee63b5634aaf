// VTK and LAMMPS-style dump writers of the phafd_gpu interpreter
// (dump.cpp:28-152 for the command, :235-309 collection, :343-480 atoms,
// :484-668 LAMMPS style, :681-867 grid, :870-1090 attributes, :1135-1254
// appended data).  The text is produced with the same ostream settings as the
// reference, so a one-rank run writes the same bytes.  The grid files
// describe the one periodic domain: extent 0 .. Nz-1 and Nx*Ny*Nz doubles per
// array.  (The reference's one-rank grid dump cannot run: its plane exchange
// addresses rank 1 and its length header counts Nz + 1 planes.)
#pragma once
#include <cstdint>
#include <fstream>
#include <iomanip>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace phafd_dump {

struct Spec {
  std::string name, type, which_atoms, base_name, nopath_base, fext;
  long long every = 1;
  std::vector<std::string> attributes;
  int precision = -1;
  std::string fmt = "lf";
};

// Dump::init (dump.cpp:28-152)
inline Spec parse(const std::vector<std::string>& v) {
  Spec s;
  s.name = v.at(0);
  s.type = v.at(1);
  if (s.type.rfind("atom", 0) == 0) {
    s.which_atoms = s.type.size() > 5 ? s.type.substr(5) : std::string();
    s.type = "atom";
  }
  if (s.type == "atom") s.fext = "vtp";
  else if (s.type == "lammpsatom") s.fext = "lmmpstrj";
  else if (s.type == "grid" || s.type == "ftgrid") s.fext = "vti";
  else throw std::runtime_error("Invalid dump type (must be atom or grid or ftgrid).");
  s.base_name = v.at(2);
  s.nopath_base = s.base_name;
  const size_t slash = s.base_name.find_last_of("\\/");
  if (slash != std::string::npos) s.nopath_base = s.base_name.substr(slash + 1);
  s.every = std::stoll(v.at(3));
  size_t it = 4;
  while (it < v.size()) {
    if (v[it] == "attributes") {
      ++it;
      const int na = std::stoi(v.at(it));
      ++it;
      for (int i = 0; i < na; i++) {
        if (it >= v.size()) throw std::invalid_argument("Incorrect number of attributes in dump file.");
        s.attributes.push_back(v[it]);
        ++it;
      }
    } else if (v[it] == "decimalplaces") {
      ++it;
      s.precision = std::stoi(v.at(it));
      ++it;
      if (s.precision <= 0) throw std::invalid_argument("Dump precision must be greater than or equal to zero.");
    } else if (v[it] == "fmt") {
      ++it;
      s.fmt = v.at(it);
      ++it;
      if (s.fmt != "lf" && s.fmt != "e") throw std::invalid_argument("Dump fmt must be either lf or e.");
    } else {
      throw std::invalid_argument("Invalid dump command.");
    }
  }
  if (s.attributes.empty()) throw std::invalid_argument("Need attributes to write dump files.");
  return s;
}

// owned beads of the one domain (labels are all OWNED = 0)
struct Atoms {
  int n = 0;
  const double *x = nullptr, *ux = nullptr, *f = nullptr;
  const int *images = nullptr, *tags = nullptr, *mols = nullptr, *types = nullptr;
  double boxlo[3] = {0, 0, 0}, boxhi[3] = {0, 0, 0};
  // per-atom compute arrays by attribute name (c_NAME): 3 components per
  // bead (compute pair, compute_pair.cpp:9-10)
  std::map<std::string, const double*> computes;
};

// real fields [z][y][x] of the one domain, by attribute name (c_NAME for per-grid computes)
struct Grid {
  int nx = 0, ny = 0, nz = 0;
  double boxlo[3] = {0, 0, 0}, spacing[3] = {1, 1, 1};
  std::map<std::string, const double*> fields;
};

inline std::string instance_name(const Spec& s, long long timestep) {
  return s.base_name + "_p0_" + std::to_string(timestep) + "." + s.fext;
}
inline std::string pinstance_name(const Spec& s, long long timestep) {
  return s.base_name + "_" + std::to_string(timestep) + ".p" + s.fext;
}
inline std::string pnopath_instance_name(const Spec& s, long long timestep) {
  return s.nopath_base + "_" + std::to_string(timestep) + ".p" + s.fext;
}

inline std::fstream open(const std::string& name, std::ios::openmode mode) {
  std::fstream f(name, mode);
  if (!f.is_open()) throw std::runtime_error(std::string("Cannot open file ") + name);
  return f;
}

// dump.cpp:235-259
inline void collection_header(const Spec& s) {
  if (s.type == "lammpsatom") {
    open(s.base_name + "_p0." + s.fext, std::ios::out);  // create_lammps_style_file, dump.cpp:332-341
    return;
  }
  auto f = open(s.base_name + ".pvd", std::ios::out);
  f << "<?xml version=\"1.0\"?>" << std::endl
    << "<VTKFile type=\"Collection\"  version=\"1.0\"" << " byte_order=\"LittleEndian\">" << std::endl
    << "<Collection>" << std::endl;
}

// dump.cpp:264-277
inline void collection_footer(const Spec& s) {
  if (s.type == "lammpsatom") return;
  auto f = open(s.base_name + ".pvd", std::ios::out | std::ios::app);
  f << "</Collection>" << std::endl << "</VTKFile>";
}

inline void number_format(std::ostream& f, const Spec& s) {
  if (s.precision > 0 && s.fmt == "lf") f << std::fixed << std::setprecision(s.precision);
  else if (s.precision > 0 && s.fmt == "e") f << std::scientific << std::setprecision(s.precision);
  else if (s.fmt == "e") f << std::scientific;
}

// write_ascii_data (dump.cpp:991-1090) for the owned beads
inline void ascii3(std::ostream& f, const std::string& name, const double* a, int n, bool pv) {
  if (pv) {
    f << "<PDataArray Name=\"" << name << "\" " << "type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\"/>"
      << std::endl;
    return;
  }
  f << "<DataArray Name=\"" << name << "\" " << "type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">"
    << std::endl;
  for (int i = 0; i < n; i++) f << a[3 * i] << " " << a[3 * i + 1] << " " << a[3 * i + 2] << " ";
  f << std::endl << "</DataArray>" << std::endl;
}
inline void ascii1(std::ostream& f, const std::string& name, const int* a, int n, bool pv) {
  if (pv) {
    f << "<PDataArray Name=\"" << name << "\" " << "type=\"Int64\" NumberOfComponents=\"" << 1
      << "\" format=\"ascii\"/>" << std::endl;
    return;
  }
  f << "<DataArray Name=\"" << name << "\" " << "type=\"Int64\" NumberOfComponents=\"" << 1
    << "\" format=\"ascii\">" << std::endl;
  for (int i = 0; i < n; i++) f << (a ? a[i] : 0) << " ";
  f << std::endl << "</DataArray>" << std::endl;
}

// process_attribute_name for beads (dump.cpp:956-977)
inline void atom_attribute(std::ostream& f, const std::string& w, const Atoms& a, bool pv) {
  if (w == "F") ascii3(f, w, a.f, a.n, pv);
  else if (w == "ux") ascii3(f, w, a.ux, a.n, pv);
  else if (w == "ix") ascii1(f, w, a.images, a.n, pv);
  else if (w == "ID") ascii1(f, w, a.tags, a.n, pv);
  else if (w == "molID") ascii1(f, w, a.mols, a.n, pv);
  else if (w == "type") ascii1(f, w, a.types, a.n, pv);
  else if (w == "label") ascii1(f, w, nullptr, a.n, pv);  // every bead of the one domain is OWNED (0)
  else if (a.computes.count(w)) ascii3(f, w, a.computes.at(w), a.n, pv);  // write_ascii_data, 3 components
  else throw std::runtime_error("Invalid per atom quantity in dump file.");
}

// the errors dump.cpp:369-409 and :956-977 raise at the first write, raised
// when the command is read (the LAMMPS style writes the owned beads, :503)
inline void check_atoms(const Spec& s) {
  if (s.type == "atom" && s.which_atoms != "owned" && s.which_atoms != "all")
    throw std::runtime_error("need atoms to be dumped to be owned, all, local, or ghost");
  bool hasx = false;
  for (auto& w : s.attributes) {
    hasx = hasx || w == "x";
    if (w != "x" && w != "F" && w != "ux" && w != "ix" && w != "ID" && w != "molID" && w != "type" && w != "label" &&
        w.rfind("c_", 0) != 0)
      throw std::runtime_error("Invalid per atom quantity in dump file.");
  }
  if (s.type == "atom" && !hasx) throw std::runtime_error("Atom dump must contain positions.");
}

// write_atom_timestep + write_atom_timestep_pvtp (dump.cpp:343-480); with one
// domain "all" and "owned" hold the same beads (the gathered and ghost copies
// are internal to the GPU lists)
inline void write_atoms(const Spec& s, long long timestep, const Atoms& a) {
  check_atoms(s);
  bool hasx = false;
  for (auto& w : s.attributes) hasx = hasx || w == "x";
  if (!hasx) throw std::runtime_error("Atom dump must contain positions.");
  {
    auto f = open(instance_name(s, timestep), std::ios::out);
    number_format(f, s);
    f << "<?xml version=\"1.0\"?>" << std::endl
      << "<VTKFile type=\"PolyData\"  version=\"1.0\"" << " byte_order=\"LittleEndian\">" << std::endl
      << "<PolyData>" << std::endl
      << "<Piece NumberOfPoints=\"" << a.n << "\" NumberOfLines=\"1\">" << std::endl;
    f << "<Points>" << std::endl;
    ascii3(f, "x", a.x, a.n, false);
    f << "</Points>" << std::endl;
    f << "<PointData>" << std::endl;
    for (auto& w : s.attributes)
      if (w != "x") atom_attribute(f, w, a, false);
    f << "</PointData>" << std::endl;
    f << "</Piece>" << std::endl << "</PolyData>" << std::endl << "</VTKFile>" << std::endl;
  }
  auto f = open(pinstance_name(s, timestep), std::ios::out);
  f << "<?xml version=\"1.0\"?>" << std::endl
    << "<VTKFile type=\"PPolyData\"  version=\"1.0\"" << " byte_order=\"LittleEndian\">" << std::endl
    << "<PPolyData GhostLevel=\"0\">" << std::endl
    << "<PPoints>" << std::endl;
  ascii3(f, "x", a.x, a.n, true);
  f << "</PPoints>" << std::endl;
  f << "<PPointData>" << std::endl;
  for (auto& w : s.attributes)
    if (w != "x") atom_attribute(f, w, a, true);
  f << "</PPointData>" << std::endl;
  f << "<Piece Source=\"" + s.nopath_base + "_p0_" + std::to_string(timestep) + "." + s.fext + "\"/>" << std::endl;
  f << "</PPolyData>" << std::endl << "</VTKFile>" << std::endl;
}

// write_lammps_dump (dump.cpp:484-668), owned beads
inline void write_lammps(const Spec& s, long long timestep, const Atoms& a) {
  auto f = open(s.base_name + "_p0." + s.fext, std::ios::out | std::ios::app);
  number_format(f, s);
  f << "ITEM: TIMESTEP" << std::endl << timestep << std::endl;
  f << "ITEM: NUMBER OF ATOMS" << std::endl << a.n << std::endl;
  f << "ITEM: BOX BOUNDS pp pp pp" << std::endl
    << a.boxlo[0] << " " << a.boxhi[0] << std::endl
    << a.boxlo[1] << " " << a.boxhi[1] << std::endl
    << a.boxlo[2] << " " << a.boxhi[2] << std::endl;
  f << "ITEM: ATOMS ";
  for (auto& w : s.attributes) {
    if (w == "x") f << "x y z ";
    else if (w == "F") f << "Fx Fy Fz ";
    else if (w == "ux") f << "ux uy uz ";
    else if (a.computes.count(w)) f << w << "_0 " << w << "_1 " << w << "_2 ";  // one column per component
    else f << w << " ";
  }
  f << std::endl;
  for (int p = 0; p < a.n; p++) {
    for (auto& w : s.attributes) {
      if (w == "x") f << a.x[3 * p] << " " << a.x[3 * p + 1] << " " << a.x[3 * p + 2] << " ";
      else if (w == "F") f << a.f[3 * p] << " " << a.f[3 * p + 1] << " " << a.f[3 * p + 2] << " ";
      else if (w == "ux") f << a.ux[3 * p] << " " << a.ux[3 * p + 1] << " " << a.ux[3 * p + 2] << " ";
      else if (w == "ix") f << a.images[p] << " ";
      else if (w == "ID") f << a.tags[p] << " ";
      else if (w == "molID") f << a.mols[p] << " ";
      else if (w == "type") f << a.types[p] << " ";
      else if (w == "label") f << 0 << " ";
      else if (a.computes.count(w)) {
        const double* c = a.computes.at(w);
        f << c[3 * p] << " " << c[3 * p + 1] << " " << c[3 * p + 2] << " ";
      } else throw std::runtime_error("Invalid per atom quantity in dump file.");
    }
    f << std::endl;
  }
}

// write_grid_timestep + write_grid_timestep_pvti (dump.cpp:681-867) for the one domain
inline void write_grid(const Spec& s, long long timestep, const Grid& g) {
  const unsigned int bytelength = (unsigned int)((size_t)g.nx * g.ny * g.nz * sizeof(double));
  const int zstart = 0, zend = g.nz - 1;
  for (auto& w : s.attributes)
    if (!g.fields.count(w)) throw std::runtime_error("Dump error: Attribute does not exist.");
  {
    auto f = open(instance_name(s, timestep), std::ios::out | std::ios::binary);
    f << "<?xml version=\"1.0\"?>" << std::endl
      << "<VTKFile type=\"ImageData\"  version=\"1.0\"" << " byte_order=\"LittleEndian\">" << std::endl
      << "<ImageData WholeExtent=\"0 " << g.nx - 1 << " 0 " << g.ny - 1 << " " << zstart << "  " << zend << "\" "
      << "Origin=\"" << g.boxlo[0] << " " << g.boxlo[1] << " " << g.boxlo[2] << " \" "
      << "Spacing=\"" << g.spacing[0] << " " << g.spacing[1] << " " << g.spacing[2] << " " << "\">" << std::endl
      << "<Piece Extent=\"0 " << g.nx - 1 << " 0 " << g.ny - 1 << " " << zstart << " " << zend << "\">"
      << std::endl
      << "<PointData Scalars=\"scalars\">" << std::endl;
    int counter = 0;
    for (auto& w : s.attributes) {
      const int offset = counter * (int)(bytelength + sizeof(bytelength));
      f << "<DataArray Name=\"" << w << "\" type=\"Float64\" format=\"appended\" " << "offset=\"" << offset
        << "\"/>" << std::endl;
      counter++;
    }
    f << "</PointData>" << std::endl
      << "</Piece>" << std::endl
      << "</ImageData>" << std::endl
      << "<AppendedData encoding=\"raw\">" << std::endl
      << "_";
    for (auto& w : s.attributes) {
      f.write(reinterpret_cast<const char*>(&bytelength), sizeof(bytelength));
      f.write(reinterpret_cast<const char*>(g.fields.at(w)), bytelength);
    }
    f << std::endl << "</AppendedData>" << std::endl << "</VTKFile>" << std::endl;
  }
  auto f = open(pinstance_name(s, timestep), std::ios::out | std::ios::binary);
  f << "<?xml version=\"1.0\"?>" << std::endl
    << "<VTKFile type=\"PImageData\"  version=\"1.0\"" << " byte_order=\"LittleEndian\">" << std::endl
    << "<PImageData WholeExtent=\"0 " << g.nx - 1 << " 0 " << g.ny - 1 << " " << " 0 " << g.nz - 1 << "\" "
    << "Origin=\"" << g.boxlo[0] << " " << g.boxlo[1] << " " << g.boxlo[2] << " \" "
    << "Spacing=\"" << g.spacing[0] << " " << g.spacing[1] << " " << g.spacing[2] << "\"" << " GhostLevel=\"1\">"
    << std::endl
    << "<PPointData Scalars=\"scalars\">" << std::endl;
  for (auto& w : s.attributes) f << "<PDataArray Name=\"" << w << "\" type=\"Float64\"/>" << std::endl;
  f << "</PPointData>" << std::endl;
  f << "<Piece Extent=\"0 " << g.nx << " 0 " << g.ny << " " << zstart << " " << zend << "\" Source=\""
    << s.nopath_base + "_p0_" + std::to_string(timestep) + "." + s.fext << "\"/>" << std::endl;
  f << std::endl << "</PImageData>" << std::endl << "</VTKFile>" << std::endl;
}

// write_collection_middle (dump.cpp:282-309): the .pvd entry, then the files
inline void write_step(const Spec& s, long long timestep, double dt, const Atoms* a, const Grid* g) {
  if (s.type != "lammpsatom") {
    const double time = timestep * dt;
    auto f = open(s.base_name + ".pvd", std::ios::out | std::ios::app);
    f << "<DataSet timestep=\"" << time << "\" group=\"\" part=\"0\"" << " file=\""
      << pnopath_instance_name(s, timestep) << "\"/>" << std::endl;
  }
  if (s.type == "atom") write_atoms(s, timestep, *a);
  else if (s.type == "lammpsatom") write_lammps(s, timestep, *a);
  else write_grid(s, timestep, *g);
}

}  // namespace phafd_dump
