// Restart input of the phafd_gpu interpreter: `grid_populate read_dump` and
// `atom_populate read_dump` (read_dump.cpp:21-394, grid.cpp:168-176,
// atom.cpp:125-134) for one rank.  The grid reader takes the .vti layout the
// dump writer produces for one domain: each appended array holds
// Nx*Ny*Nz doubles (read_dump.cpp:336-346 with rank 0 also the last rank).
#pragma once
#include <cstdint>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace phafd_dump {

struct ReadSpec {
  std::string type, filename;
  std::vector<std::string> attributes;
  bool no_padding = false;
};

// ReadDump::init (read_dump.cpp:21-60); v = {"grid"|"atom", FILE, options...}
inline ReadSpec parse_read(const std::vector<std::string>& v) {
  ReadSpec s;
  s.type = v.at(0);
  s.filename = v.at(1);
  size_t it = 2;
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
    } else if (v[it] == "no_padding") {
      s.no_padding = true;
      ++it;
    } else {
      throw std::invalid_argument("Third word in dump must be 'attributes'.");
    }
  }
  if (s.attributes.empty()) throw std::invalid_argument("Need attributes to read dump files.");
  for (auto& w : s.attributes)
    if (w.rfind("c_", 0) == 0 || w.rfind("f_", 0) == 0) throw std::runtime_error("Cannot read computes from dump");
  if (s.type != "grid" && s.type != "atom") throw std::runtime_error("Can only read atoms or grid from dump file.");
  return s;
}

inline bool has(const std::vector<std::string>& v, const std::string& w) {
  for (auto& a : v)
    if (a == w) return true;
  return false;
}

// The arrays of a grid dump (.vti, raw appended data): the XML header is
// parsed once into a table of DataArray name -> offset into the appended
// block; each requested array is then read at its offset, as a 4-byte length
// followed by Nx*Ny*Nz doubles [z][y][x].  The checks and their messages are
// those of ReadDump::process_grid_attributes (read_dump.cpp:90-185).
struct VtiTable {
  std::map<std::string, uint64_t> offset;  // name -> offset after the '_' marker
  std::streampos data = 0;                 // file position of the first appended byte
};

// the attribute value NAME="..." of an XML element line, if present
inline bool xml_attr(const std::string& line, const std::string& name, std::string& value) {
  const std::string key = name + "=\"";
  const size_t at = line.find(key);
  if (at == std::string::npos) return false;
  const size_t start = at + key.size();
  const size_t end = line.find('"', start);
  if (end == std::string::npos) return false;
  value = line.substr(start, end - start);
  return true;
}

inline VtiTable vti_table(std::ifstream& f) {
  VtiTable t;
  std::string line;
  while (std::getline(f, line)) {
    if (line.rfind("<AppendedData", 0) == 0) {
      char marker = 0;
      f.read(&marker, 1);  // the raw block starts after '_'
      t.data = f.tellg();
      return t;
    }
    std::string name, off;
    if (line.rfind("<DataArray ", 0) == 0 && xml_attr(line, "Name", name) && xml_attr(line, "offset", off))
      t.offset[name] = std::stoull(off);
  }
  t.data = -1;
  return t;
}

inline std::map<std::string, std::vector<double>> read_grid(const ReadSpec& s, int nx, int ny, int nz) {
  std::ifstream f(s.filename, std::ios::in | std::ios::binary);
  if (!f) {
    std::cerr << "could not open file " << s.filename << std::endl;
    throw std::runtime_error("file not found.");
  }
  if (!has(s.attributes, "phi")) throw std::runtime_error("Read dump needs attribute phi.");
  const VtiTable t = vti_table(f);
  bool all = t.data != std::streampos(-1);
  for (auto& w : s.attributes) all = all && t.offset.count(w);
  if (!all) {
    std::string msg = "Not all attributes requested in read_dump command are in " + s.filename +
                      ". List of attributes in file are:";
    for (auto& w : s.attributes) msg += " " + w;
    throw std::runtime_error(msg + ".");
  }
  const uint64_t want = (uint64_t)nx * ny * nz * sizeof(double);  // one domain: no neighbour planes
  std::map<std::string, std::vector<double>> out;
  for (auto& w : s.attributes) {
    if (w != "phi" && w != "chempot" && w != "gradphi_x" && w != "gradphi_y" && w != "gradphi_z")
      throw std::runtime_error("ReadDump error: Attribute does not exist.");
    f.clear();
    f.seekg(t.data + (std::streamoff)t.offset.at(w));
    uint32_t bytelength = 0;
    f.read(reinterpret_cast<char*>(&bytelength), sizeof(bytelength));
    if (!f || bytelength != want) throw std::runtime_error("incorrect size " + w + " in file.");
    std::vector<double> a((size_t)nx * ny * nz);
    f.read(reinterpret_cast<char*>(a.data()), (std::streamsize)want);
    if (!f) throw std::runtime_error("incorrect size " + w + " in file.");
    out[w] = std::move(a);
  }
  return out;
}

struct ReadAtoms {
  std::vector<double> x, ux, F;
  std::vector<int> images, tags, mols, types, labels;
};

// ReadDump::read_ascii_data: values from the one line after the header;
// entries the line does not hold keep their previous value
inline void read_line(const std::string& line, std::vector<double>& a) {
  std::stringstream ss(line);
  for (auto& v : a) ss >> v;
}
inline void read_line(const std::string& line, std::vector<int>& a) {
  std::stringstream ss(line);
  for (auto& v : a) ss >> v;
}

// ReadDump::process_atom_attributes (read_dump.cpp:188-286) for natoms beads
inline ReadAtoms read_atoms(const ReadSpec& s, int natoms, bool molecule_flag) {
  std::ifstream f(s.filename);
  if (!f) {
    std::cerr << "could not open file " << s.filename << std::endl;
    throw std::runtime_error("file not found.");
  }
  std::vector<std::string> necessary = {"x", "type", "ID"};
  if (molecule_flag) {
    necessary.push_back("molID");
    necessary.push_back("ix");
  }
  for (auto& w : necessary)
    if (!has(s.attributes, w)) throw std::runtime_error("Read dump needs attribute " + w + ".");
  ReadAtoms r;
  const size_t n = (size_t)natoms;
  r.x.assign(3 * n, 0.0); r.ux.assign(3 * n, 0.0); r.F.assign(3 * n, 0.0);
  r.images.assign(n, 0); r.tags.assign(n, 0); r.mols.assign(n, 0); r.types.assign(n, 0); r.labels.assign(n, 0);
  std::vector<std::string> found;
  std::string line;
  while (std::getline(f, line)) {
    for (auto& w : s.attributes) {
      if (line == "<DataArray Name=\"" + w + "\" type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">") {
        std::getline(f, line);
        if (w == "x") read_line(line, r.x);
        else if (w == "F") read_line(line, r.F);
        else if (w == "ux") read_line(line, r.ux);
        else throw std::runtime_error("Attribute " + w + " not recognised.");
        found.push_back(w);
        break;
      } else if (line == "<DataArray Name=\"" + w + "\" type=\"Int64\" NumberOfComponents=\"1\" format=\"ascii\">") {
        std::getline(f, line);
        if (w == "ix") read_line(line, r.images);
        else if (w == "ID") read_line(line, r.tags);
        else if (w == "molID") read_line(line, r.mols);
        else if (w == "type") read_line(line, r.types);
        else if (w == "label") read_line(line, r.labels);
        else throw std::runtime_error("Attribute " + w + " not recognised.");
        found.push_back(w);
        break;
      }
    }
  }
  if (found.size() != s.attributes.size()) {
    std::string e = "Only found attributes ";
    for (auto& w : found) e += w + ", ";
    throw std::runtime_error(e);
  }
  return r;
}

}  // namespace phafd_dump
