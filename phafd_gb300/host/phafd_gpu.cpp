// phafd_gpu: the PHAFD input-script interpreter on top of libphafd_gpu.
//
// Same command line as the reference's phafd (phafd.cpp:30-93):
//   phafd_gpu -in script [-var name value ...] [-sf gpu] [-dry-run]
// and the same commands, in the same order rules, as Input::read
// (input.cpp:48-299).  Pair and fix styles resolve to the GPU
// implementations when their name carries the "/gpu" suffix, or for every
// style once "-sf gpu" is on the command line or "suffix gpu" is in the
// script, so an unchanged reference script runs with -sf gpu.
//
// GPU-only settings come from one extra command (ignored by nothing else):
//   package gpu [precision 32|64] [schedule resident|reference]
//               [zghost periodic|rank1] [noise philox|reference|off]
//               [device N] [plane on|off]
// and one output command for raw fields:
//   write_field phi|chempot|gradx|grady|gradz FILE   (raw float64, [z][y][x])
// Dumps (atom, lammpsatom, grid, ftgrid) are written as the reference writes
// them (vtk_dump.hpp); per-grid attributes are phi, chempot, gradphi_x/y/z
// and c_NAME of compute grid/cluster, per-atom attributes include c_NAME of
// compute pair, per-ftgrid ones c_NAME of compute complex.
// "-dry-run" parses and checks the script without touching a GPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "phafd_gpu.h"
#include "read_dump.hpp"
#include "vtk_dump.hpp"

namespace {

using Words = std::vector<std::string>;

// utility.cpp:11-45: split on whitespace after dropping a trailing # comment
Words split_line(std::string line) {
  line = line.substr(0, line.find('#'));
  Words out;
  std::istringstream is(line);
  std::string w;
  while (is >> w) out.push_back(w);
  return out;
}

// utility.cpp:77-139: ${name} substitution from -var
void convert_variables(std::string& raw, const std::map<std::string, std::string>& vars) {
  for (;;) {
    auto a = raw.find("${");
    if (a == std::string::npos) return;
    auto b = raw.find('}', a + 2);
    if (b == std::string::npos) throw std::runtime_error("Missing '}' in input script.");
    std::string key = raw.substr(a + 2, b - a - 2);
    if (key.empty()) throw std::runtime_error("No content ('${}') in input file.");
    auto it = vars.find(key);
    if (it == vars.end()) throw std::runtime_error("No such command line variable " + key);
    raw.replace(a, b - a + 1, it->second);
  }
}

// utility.cpp:49-75: % -> MPI rank (always 0 here)
void replace_percentages(std::string& raw) {
  for (auto p = raw.find('%'); p != std::string::npos; p = raw.find('%')) raw.replace(p, 1, "0");
}

double num(const std::string& s) { return std::stod(s); }
int inum(const std::string& s) { return std::stoi(s); }

struct Range { int start, end; };

class Interpreter {
 public:
  Interpreter(bool dry, bool suffix) : dry_(dry), suffix_gpu_(suffix) {}
  ~Interpreter() {
    if (ctx_) phafd_ctx_destroy(ctx_);
  }

  void run_file(std::istream& in, const std::map<std::string, std::string>& vars) {
    std::string line;
    std::vector<std::string> lines;
    while (std::getline(in, line)) lines.push_back(line);
    // mu survives a step only when kept from the start: a later
    // `write_field chempot` asks for it before the first run
    for (auto& l : lines) {
      const Words w = split_line(l);
      if (w.size() >= 2 && w[0] == "write_field" && w[1] == "chempot") want_chempot_ = true;
    }
    for (size_t li = 0; li < lines.size(); ++li) {
      std::string l = lines[li];
      convert_variables(l, vars);
      replace_percentages(l);
      Words w = split_line(l);
      if (w.empty()) continue;
      std::string cmd = w[0];
      w.erase(w.begin());
      if (cmd == "pair") {
        command_pair(w);
        // pairCoeffs lines directly follow their pair (input.cpp:133-153)
        while (li + 1 < lines.size()) {
          std::string n = lines[li + 1];
          convert_variables(n, vars);
          Words nw = split_line(n);
          if (nw.empty()) { ++li; continue; }
          if (nw[0] != "pairCoeffs") break;
          nw.erase(nw.begin());
          command_pair_coeff(nw);
          ++li;
        }
      } else {
        command(cmd, w);
      }
    }
  }

 private:
  bool dry_, suffix_gpu_;
  phafd_ctx* ctx_ = nullptr;
  int precision_ = PHAFD_FP32, schedule_ = PHAFD_SCHEDULE_RESIDENT, zghost_ = PHAFD_ZGHOST_PERIODIC;
  int noise_ = PHAFD_NOISE_PHILOX, device_ = 0, plane_ = 0;
  bool boxset_ = false, gridset_ = false, populated_ = false, atomset_ = false, atoms_made_ = false;
  double boxlo_[3] = {0, 0, 0}, period_[3] = {0, 0, 0};
  int grid_n_[3] = {0, 0, 0};
  int natoms_ = 0, ntypes_ = 0;
  bool molecule_flag_ = false;
  std::vector<int> tags_, mols_, types_;
  std::vector<double> xs_;
  std::map<std::string, std::vector<Range>> groups_;
  std::set<std::string> fix_names_;
  int last_gridatom_ = PHAFD_GRIDATOM_NONE;
  int npairs_ = 0;
  bool neighbor_set_ = false;
  double dt_ = 0.0;
  long long timestep_ = 0;
  std::vector<std::pair<std::string, bool>> fh_fixes_;  // names of grid/floryhuggins fixes
  bool conj_set_ = false;                                // a grid/conjugate/volfrac fix exists
  bool want_chempot_ = false;                            // the script writes chempot after a run
  std::vector<phafd_dump::Spec> dumps_;
  struct Cluster { double threshold; bool greater; };
  std::map<std::string, Cluster> clusters_;  // compute grid/cluster NAME phi THRESHOLD lt|gt
  struct Complex {
    int field, quant;
  };
  std::map<std::string, Complex> complexes_;  // compute complex NAME ft_phi|ft_chempot real|imag|modulus|norm
  std::map<std::string, int> pair_computes_;  // compute pair NAME PAIRSTYLE -> PHAFD_PAIR_*
  std::set<std::string> pair_names_;          // pair styles created (their reference names)
  std::map<std::string, std::vector<double>> compute_cache_;  // each compute's array as last computed
  std::set<std::string> compute_names_;

  void check(int rc) {
    if (rc != PHAFD_OK) throw std::runtime_error(ctx_ ? phafd_last_error(ctx_) : "libphafd_gpu call failed");
  }

  phafd_ctx* ctx() {
    if (dry_) return nullptr;
    if (!ctx_) {
      int rc = phafd_ctx_create(&ctx_, device_, precision_);
      if (rc) throw std::runtime_error("cannot create a GPU context on device " + std::to_string(device_));
      check(phafd_set_schedule(ctx_, schedule_));
      check(phafd_set_zghost(ctx_, zghost_));
      check(phafd_set_plane_fusion(ctx_, plane_));
      if (want_chempot_) check(phafd_set_keep_chempot(ctx_, 1));
    }
    return ctx_;
  }

  // a style name resolves to the GPU implementation with "/gpu" or an active suffix
  std::string gpu_style(const std::string& name) {
    const std::string sfx = "/gpu";
    if (name.size() > sfx.size() && name.compare(name.size() - sfx.size(), sfx.size(), sfx) == 0)
      return name.substr(0, name.size() - sfx.size());
    if (suffix_gpu_) return name;
    throw std::invalid_argument("style " + name + " has no CPU implementation in phafd_gpu: use " + name +
                                "/gpu, 'suffix gpu' or -sf gpu");
  }

  void command(const std::string& cmd, Words& w) {
    if (cmd == "suffix") {
      if (w.size() != 1 || (w[0] != "gpu" && w[0] != "off")) throw std::invalid_argument("suffix gpu|off");
      suffix_gpu_ = w[0] == "gpu";
    } else if (cmd == "package") {
      command_package(w);
    } else if (cmd == "domain") {
      command_domain(w);
    } else if (cmd == "grid_style") {
      if (!boxset_) throw std::invalid_argument("CAnnot use command grid_style before domain box is set.");
      if (w.size() < 4 || w[3] != "concentration") throw std::invalid_argument("Incompatible style type in grid_style.");
      for (int d = 0; d < 3; ++d) grid_n_[d] = inum(w[d]);
      if (!dry_) check(phafd_grid_style(ctx(), grid_n_[0], grid_n_[1], grid_n_[2]));
      gridset_ = true;
    } else if (cmd == "grid_populate") {
      if (!gridset_) throw std::invalid_argument("CAnnot use command grid_populate before grid_style is set.");
      if (w.size() >= 5 && w[0] == "constant" && w[1] == "concentration") {
        if (!dry_) check(phafd_grid_populate_constant(ctx(), num(w[2]), num(w[3]), inum(w[4])));
      } else if (w.size() >= 7 && w[0] == "flat_interface" && w[1] == "concentration") {  // grid.cpp:136-151
        if (!dry_)
          check(phafd_grid_populate_flat_interface(ctx(), num(w[2]), num(w[3]), num(w[4]), num(w[5]), inum(w[6])));
      } else if (w.size() >= 6 && w[0] == "sphere" && w[1] == "concentration") {  // grid.cpp:153-166
        if (!dry_) check(phafd_grid_populate_sphere(ctx(), num(w[2]), std::sqrt(num(w[3])), num(w[4]), num(w[5])));
      } else if (!w.empty() && w[0] == "read_dump") {
        grid_read_dump(w);
      } else {
        throw std::runtime_error("grid_populate " + (w.empty() ? std::string() : w[0]) +
                                 " is not supported by phafd_gpu (constant, flat_interface or sphere "
                                 "concentration, or read_dump)");
      }
      populated_ = true;
    } else if (cmd == "atom_style") {
      command_atom_style(w);
    } else if (cmd == "atom_populate") {
      if (!atomset_) throw std::invalid_argument("CAnnot use command atom_populate before atom_style is set.");
      if (w.size() >= 2 && w[0] == "read_atoms") read_atoms(w[1]);
      else if (w.size() >= 2 && w[0] == "read_dump") atom_read_dump(w);
      else throw std::runtime_error("Invalid atom_populate command.");
    } else if (cmd == "neighbor") {
      if (npairs_ == 0 && ntypes_ > 0) throw std::runtime_error("Must call neighbor after pairs are given.");
      if (!gridset_) throw std::runtime_error("Must call neighbor after subboxes are set (via grid style).");
      if (!dry_) check(phafd_neighbor(ctx(), num(w.at(0))));
      neighbor_set_ = true;
    } else if (cmd == "group") {
      command_group(w);
    } else if (cmd == "fix") {
      command_fix(w);
    } else if (cmd == "compute") {
      command_compute(w);
    } else if (cmd == "dump") {
      command_dump(w);
    } else if (cmd == "timestep") {
      timestep_ = std::stoll(w.at(0));
      if (!dry_) check(phafd_set_timestep(ctx(), timestep_));
    } else if (cmd == "dt") {
      dt_ = num(w.at(0));
      if (!dry_) check(phafd_set_dt(ctx(), dt_));
    } else if (cmd == "run") {
      if (dt_ <= 0.0) throw std::runtime_error("Cannot run simulation without setting dt > 0.");
      run(std::stoll(w.at(0)));
    } else if (cmd == "write_field") {
      write_field(w.at(0), w.at(1));
    } else if (cmd == "write_noise_state" || cmd == "read_noise_state") {
      noise_state(cmd == "write_noise_state", w.at(0));
    } else if (cmd == "run_until_touching") {  // input.cpp:274-295
      if (dt_ <= 0.0) throw std::runtime_error("Cannot run simulation without setting dt > 0.");
      const long long nsteps = std::stoll(w.at(0));
      if (w.size() < 2) throw std::runtime_error("Must provide a size at which atoms are considered touching.");
      if (w.size() < 3) throw std::runtime_error("Must say whether to continue simulation after touching occurs.");
      if (w[2] == "continue") {
        if (w.size() < 4) throw std::runtime_error("Must say delay to mention new cyclisation events.");
        run_until_touching(nsteps, num(w[1]), true, (int)num(w[3]));
      } else if (w[2] == "stop") {
        run_until_touching(nsteps, num(w[1]), false, 0);
      } else {
        throw std::runtime_error("Must say whether to continue simulation after touching occurs.");
      }
    } else {
      throw std::invalid_argument("Unknown command: " + cmd);
    }
  }

  void command_package(Words& w) {
    if (w.empty() || w[0] != "gpu") throw std::invalid_argument("package gpu ...");
    for (size_t i = 1; i + 1 < w.size(); i += 2) {
      const std::string& k = w[i];
      const std::string& v = w[i + 1];
      if (ctx_) throw std::runtime_error("package gpu must come before domain / grid_style");
      if (k == "precision") {
        precision_ = inum(v);
        if (precision_ != 32 && precision_ != 64) throw std::invalid_argument("package gpu precision 32|64");
      } else if (k == "schedule") {
        schedule_ = v == "reference" ? PHAFD_SCHEDULE_REFERENCE : PHAFD_SCHEDULE_RESIDENT;
      } else if (k == "zghost") {
        zghost_ = v == "rank1" ? PHAFD_ZGHOST_RANK1 : PHAFD_ZGHOST_PERIODIC;
      } else if (k == "noise") {
        noise_ = v == "reference" ? PHAFD_NOISE_REFERENCE : v == "off" ? PHAFD_NOISE_OFF : PHAFD_NOISE_PHILOX;
      } else if (k == "device") {
        device_ = inum(v);
      } else if (k == "plane") {
        plane_ = v == "on";
      } else {
        throw std::invalid_argument("unknown package gpu keyword " + k);
      }
    }
  }

  void command_domain(Words& w) {  // domain.cpp:30-76
    bool pf = false, of = false;
    size_t i = 0;
    while (i < w.size()) {
      if (w[i] == "boxdims" && i + 3 < w.size()) {
        for (int d = 0; d < 3; ++d) period_[d] = num(w[i + 1 + d]);
        pf = true;
        i += 4;
      } else if (w[i] == "boxorigin" && i + 3 < w.size()) {
        for (int d = 0; d < 3; ++d) boxlo_[d] = num(w[i + 1 + d]);
        of = true;
        i += 4;
      } else {
        throw std::invalid_argument("Bad arguments for domain_setup.");
      }
    }
    if (!pf) throw std::runtime_error("need to set box dimensions.");
    if (!of) throw std::runtime_error("need to set box origin.");
    if (!dry_) check(phafd_domain(ctx(), boxlo_, period_));
    boxset_ = true;
  }

  void command_atom_style(Words& w) {  // atom.cpp:26-110, one rank
    size_t i = 0;
    while (i < w.size() && w[i] != "natoms") {
      if (w[i] == "polymer") molecule_flag_ = true;
      else if (w[i] == "sphere") throw std::runtime_error("atom_style sphere is not supported by phafd_gpu");
      else throw std::runtime_error("Unrecognised atom style.");
      ++i;
    }
    if (i + 1 >= w.size()) throw std::runtime_error("atom_style needs natoms N");
    std::string n = w[i + 1];
    auto star = n.find('*');
    natoms_ = star == std::string::npos ? inum(n) : inum(n.substr(0, star));
    atomset_ = true;
  }

  void read_atoms(const std::string& fname) {  // read_atoms.cpp:58-97, atom.cpp:219-252
    std::ifstream f(fname);
    if (!f) throw std::runtime_error("Could not read data atom file. ");
    std::string line;
    while (std::getline(f, line)) {
      if (line.empty() || line[0] == '#') continue;
      Words w = split_line(line);
      if (w.empty()) continue;
      size_t k = 0;
      tags_.push_back(inum(w.at(k++)));
      mols_.push_back(molecule_flag_ ? inum(w.at(k++)) : 0);
      types_.push_back(inum(w.at(k++)));
      for (int d = 0; d < 3; ++d) xs_.push_back(num(w.at(k++)));
    }
    if ((int)tags_.size() != natoms_) throw std::runtime_error("Could not read data atom file. ");
    std::set<int> ts(tags_.begin(), tags_.end());
    if (ts.size() != tags_.size()) throw std::runtime_error("duplicate IDs found on processor(s).");
    ntypes_ = types_.empty() ? 0 : *std::max_element(types_.begin(), types_.end()) + 1;
    groups_["all"] = {{0, natoms_}};
    if (!dry_) check(phafd_atoms_create(ctx(), natoms_, tags_.data(), mols_.data(), types_.data(), xs_.data()));
    atoms_made_ = true;
  }

  // grid_populate read_dump FILE attributes N ... (grid.cpp:168-176): phi is
  // uploaded; chempot and the gradient are rebuilt from phi by every step, so
  // the arrays read for them only pass the reference's checks
  void grid_read_dump(const Words& w) {
    Words v(w);
    v[0] = "grid";
    const auto s = phafd_dump::parse_read(v);
    const auto fields = phafd_dump::read_grid(s, grid_n_[0], grid_n_[1], grid_n_[2]);
    if (!dry_) check(phafd_grid_set(ctx(), PHAFD_FIELD_PHI, fields.at("phi").data()));
  }

  // atom_populate read_dump FILE attributes N ... (atom.cpp:125-134)
  void atom_read_dump(const Words& w) {
    Words v(w);
    v[0] = "atom";
    const auto s = phafd_dump::parse_read(v);
    const auto r = phafd_dump::read_atoms(s, natoms_, molecule_flag_);
    tags_ = r.tags;
    mols_ = molecule_flag_ ? r.mols : std::vector<int>(natoms_, 0);
    types_ = r.types;
    xs_ = r.x;
    std::set<int> ts(tags_.begin(), tags_.end());
    if (ts.size() != tags_.size()) throw std::runtime_error("duplicate IDs found on processor(s).");
    ntypes_ = types_.empty() ? 0 : *std::max_element(types_.begin(), types_.end()) + 1;
    groups_["all"] = {{0, natoms_}};
    if (!dry_) {
      check(phafd_atoms_create(ctx(), natoms_, tags_.data(), mols_.data(), types_.data(), xs_.data()));
      if (phafd_dump::has(s.attributes, "ix")) check(phafd_atoms_set_images(ctx(), r.images.data()));
    }
    atoms_made_ = true;
  }

  void command_pair(Words& w) {  // input.cpp:99-131
    if (ntypes_ <= 0) throw std::runtime_error("Cannot create pair style before atoms are made.");
    const std::string style = gpu_style(w.at(0));
    if (style == "gridatom/gaussian" || style == "gridatom/LJish" || style == "gridatom/LJish/linear") {
      last_gridatom_ = style == "gridatom/gaussian" ? PHAFD_GRIDATOM_GAUSSIAN
                     : style == "gridatom/LJish" ? PHAFD_GRIDATOM_LJISH : PHAFD_GRIDATOM_LJISH_LINEAR;
      if (!dry_) check(phafd_pair_gridatom(ctx(), last_gridatom_, num(w.at(1))));
      pair_names_.insert(style);
    } else if (style == "lj/cut") {
      pair_names_.insert(style);
      last_gridatom_ = PHAFD_GRIDATOM_NONE;
      if (!dry_) check(phafd_pair_lj_cut(ctx(), num(w.at(1)), num(w.at(2)), num(w.at(3))));
    } else {
      throw std::invalid_argument("Unrecognised pair style.");
    }
    ++npairs_;
  }

  void command_pair_coeff(Words& w) {  // pair_gridatom_gaussian.cpp:145-181 (lj/cut takes none)
    if (last_gridatom_ == PHAFD_GRIDATOM_NONE) return;
    const int type = inum(w.at(0));
    if (type > ntypes_ || type < 0) throw std::runtime_error("Pair grid/atom atom type out of range.");
    if (w.size() - 1 > 6) throw std::runtime_error("Pair grid/atom invalid coeffs.");
    int he = 0, hw = 0, hp = 0;
    double e = 0, wd = 0, p = 0;
    for (size_t i = 1; i + 1 < w.size(); i += 2) {
      if (w[i] == "epsilon") { he = 1; e = num(w[i + 1]); }
      else if (w[i] == "nucwidth") { hw = 1; wd = num(w[i + 1]); }
      else if (w[i] == "phi") { hp = 1; p = num(w[i + 1]); }
      else throw std::runtime_error("Pair grid/atom invalid coeffs.");
    }
    if (!dry_) check(phafd_pair_gridatom_coeff(ctx(), type, he, e, hw, wd, hp, p));
  }

  void command_group(Words& w) {  // group.cpp:31-207
    if (ntypes_ <= 0) throw std::runtime_error("Must call group after atoms have been read in (via read_atoms).");
    const std::string name = w.at(0);
    if (name == "all" || groups_.count(name)) throw std::runtime_error("Error: Duplicate of group " + name + ".");
    const std::string style = w.at(1);
    std::vector<Range> ranges;
    if (style == "molecule") {
      std::set<int> mols;
      if (w.at(2) == "<>") for (int m = inum(w.at(3)); m <= inum(w.at(4)); ++m) mols.insert(m);
      else for (size_t i = 2; i < w.size(); ++i) mols.insert(inum(w[i]));
      for (int m : mols) {
        int start = -1, last = -1;
        for (int i = 0; i < natoms_; ++i)
          if (mols_[i] == m) {
            if (start < 0) start = i;
            else if (last != i - 1) throw std::runtime_error("atoms of the same molecule must be adjacently owned.");
            last = i;
          }
        if (start < 0) throw std::runtime_error("Group error: Molecule " + std::to_string(m) + " does not exist on any processor.");
        ranges.push_back({start, last + 1});
      }
    } else if (style == "atom") {
      if (w.at(2) != "<>") throw std::invalid_argument("Group atom requires '<>' style parameters.");
      const int t0 = inum(w.at(3)), t1 = inum(w.at(4));
      int i = 0;
      while (i < natoms_ && tags_[i] < t0) ++i;
      const int s = i;
      for (int t = t0; t <= t1 && i < natoms_; ++t, ++i)
        if (tags_[i] != t) throw std::invalid_argument("atoms of the same group must be adjacently owned.");
      if (i == s) throw std::runtime_error("atoms do not exist on any processor.");
      ranges.push_back({s, i});
    } else {
      throw std::invalid_argument("Group must be of style molecule or atom.");
    }
    groups_[name] = ranges;
  }

  const std::vector<Range>& group(const std::string& g) {
    auto it = groups_.find(g);
    if (it == groups_.end()) throw std::runtime_error("Group " + g + " does not exist.");
    return it->second;
  }

  void command_fix(Words& w) {  // input.cpp:177-229
    const std::string style = gpu_style(w.at(0));
    w.erase(w.begin());
    const std::string name = w.at(0);
    if (fix_names_.count(name)) throw std::runtime_error("Error: Duplicate of fix " + name + ".");
    fix_names_.insert(name);
    if (style == "grid/conjugate/volfrac") {  // fixgrid_conjugate.cpp:21-45, conjugate_volfrac.cpp:29-70
      if (!populated_) throw std::runtime_error("Fix requires grid to be populated.");
      const int seed = inum(w.at(1));
      double M = 1, T = 1, v = 1, g = 1;
      for (size_t i = 2; i < w.size(); i += 2) {
        if (i + 1 >= w.size()) throw std::runtime_error("Error: invalid conjugate/volfrac command");
        if (w[i] == "mobility") M = num(w[i + 1]);
        else if (w[i] == "temp") T = num(w[i + 1]);
        else if (w[i] == "volFH") v = num(w[i + 1]);
        else if (w[i] == "gamma") g = num(w[i + 1]);
        else throw std::runtime_error("Error: invalid conjugate/volfrac command");
      }
      if (!dry_) check(phafd_fix_conjugate_volfrac(ctx(), seed, M, T, v, g, noise_));
      conj_set_ = true;
    } else if (style == "grid/floryhuggins") {  // fixgrid_floryhuggins.cpp:22-56
      if (!populated_) throw std::runtime_error("Fix requires grid to be populated.");
      double T = 1, v = 1, chi = 1;
      for (size_t i = 1; i < w.size(); i += 2) {
        if (i + 1 >= w.size()) throw std::runtime_error("Error: invalid fixgrid/floryhuggins command");
        if (w[i] == "temp") T = num(w[i + 1]);
        else if (w[i] == "volFH") v = num(w[i + 1]);
        else if (w[i] == "chi") chi = num(w[i + 1]);
        else throw std::runtime_error("Error: invalid fixgrid/floryhuggins command");
      }
      if (!dry_) check(phafd_fix_floryhuggins(ctx(), T, v, chi));
      fh_fixes_.push_back({name, true});
    } else if (style == "grid/gradphi") {
      if (!populated_) throw std::runtime_error("Fix requires grid to be populated.");
      const bool once = w.size() > 1 && w[1] == "once";
      if (!dry_) check(phafd_fix_gradphi(ctx(), once));
    } else if (style == "atom/drag") {  // fixatom_drag.cpp:24-33
      if (ntypes_ <= 0) throw std::runtime_error("Fix requires atoms to be created.");
      const auto& rg = group(w.at(1));
      std::vector<int> s, e;
      for (auto& r : rg) { s.push_back(r.start); e.push_back(r.end); }
      if (!dry_) check(phafd_fix_drag(ctx(), (int)s.size(), s.data(), e.data(), num(w.at(2))));
    } else if (style == "atom/semiflexible/notether") {  // fixatom_semiflexible.cpp:27-82
      if (ntypes_ <= 0) throw std::runtime_error("Fix requires atoms to be created.");
      const auto& rg = group(w.at(1));
      phafd_semiflexible_params p{};
      p.bondlength = 1.0; p.zeta_para = 1.0; p.zeta_perp = 1.0; p.bending = 0.0; p.temp = 0.0; p.kbond = 100.0;
      p.seed = inum(w.at(2));
      for (size_t i = 3; i + 1 < w.size(); i += 2) {
        const std::string& k = w[i];
        const double v = num(w[i + 1]);
        if (k == "bondlength") p.bondlength = v;
        else if (k == "zeta_para") p.zeta_para = v;
        else if (k == "zeta_perp") p.zeta_perp = v;
        else if (k == "bending") p.bending = v;
        else if (k == "temp") p.temp = v;
        else if (k == "kbond" || k == "springK") p.kbond = v;
        else throw std::runtime_error("invalid atom/semiflexible keyword " + k);
      }
      p.noise = p.temp > 0 ? PHAFD_NOISE_PHILOX : PHAFD_NOISE_OFF;
      std::vector<int> s, e;
      for (auto& r : rg) { s.push_back(r.start); e.push_back(r.end); }
      if (!dry_) check(phafd_fix_semiflexible(ctx(), (int)s.size(), s.data(), e.data(), &p));
    } else if (style == "atom/semiflexible/singletether" || style == "atom/semiflexible/doubletether" ||
               style == "grid/ave") {
      throw std::runtime_error("fix " + style + " is not supported by phafd_gpu");
    } else {
      throw std::runtime_error("Invalid fix.");
    }
  }

  // Compute::init + ComputeGridClusters::init / ComputeComplex::init /
  // ComputePair::init (compute.cpp:13-27, compute_grid_clusters.cpp:23-64,
  // compute_complex.cpp:14-41, compute_pair.cpp:15-35)
  void command_compute(const Words& w) {  // compute STYLE NAME args (input.cpp:234-254)
    std::string style = w.at(0);
    if (style.size() > 4 && style.compare(style.size() - 4, 4, "/gpu") == 0) style.resize(style.size() - 4);
    if (style != "complex" && style != "pair" && style != "grid/cluster") throw std::runtime_error("Invalid compute.");
    const std::string name = w.at(1);  // Compute::init, compute.cpp:13-27
    if (compute_names_.count(name)) throw std::runtime_error("Error: Duplicate of compute " + name + std::string("."));
    compute_names_.insert(name);
    if (style == "grid/cluster") {  // compute_grid_clusters.cpp:23-64
      if (w.at(2) != "phi") throw std::runtime_error("Must use phi as array for clustering.");
      const double thr = num(w.at(3));
      const std::string cond = w.at(4);
      if (cond != "lt" && cond != "gt") throw std::runtime_error("Must specify lt or gt for compute grid cluster.");
      clusters_[name] = Cluster{thr, cond == "gt"};
    } else if (style == "complex") {  // compute_complex.cpp:14-41
      const std::string arr = w.at(2);
      int field;
      if (arr == "ft_phi") field = PHAFD_FIELD_FT_PHI_STEP_START;  // what the reference sees inside the step
      else if (arr == "ft_chempot") field = PHAFD_FIELD_FT_CHEMPOT;
      else throw std::runtime_error("Invalid array to compute in compute modulus.");
      const std::string q = w.at(3);
      const int quant = q == "real" ? PHAFD_COMPLEX_REAL : q == "imag" ? PHAFD_COMPLEX_IMAG
                      : q == "modulus" ? PHAFD_COMPLEX_MODULUS : q == "norm" ? PHAFD_COMPLEX_NORM : -1;
      if (quant < 0) throw std::runtime_error("Invalid argument in compute complex.");
      if (field == PHAFD_FIELD_FT_CHEMPOT && !dry_) check(phafd_set_keep_chempot(ctx(), 1));
      complexes_[name] = Complex{field, quant};
    } else {  // compute pair NAME PAIRSTYLE (compute_pair.cpp:15-35)
      const std::string pairname = gpu_style(w.at(2));
      if (!pair_names_.count(pairname))
        throw std::invalid_argument("Cannot compute pair style " + pairname + ", it hasn't been created!");
      pair_computes_[name] = pairname == "lj/cut" ? PHAFD_PAIR_LJ_CUT : PHAFD_PAIR_GRIDATOM;
      if (!dry_) check(phafd_set_pair_snapshot(ctx(), 1));  // each step keeps its pair-stage positions
    }
  }

  // Dump::init + Dump::setup checks (dump.cpp:28-233)
  void command_dump(const Words& w) {
    phafd_dump::Spec d = phafd_dump::parse(w);
    for (auto& o : dumps_)
      if (o.name == d.name) throw std::runtime_error("Error: Duplicate of dump " + d.name + std::string("."));
    // process_attribute_name's checks (dump.cpp:870-990), made when the command is read
    auto compute_attr = [&](const std::string& a, bool ft) {
      const std::string cid = a.substr(2);
      if (!compute_names_.count(cid))
        throw std::runtime_error("Cannot write dump, compute ID " + cid + std::string("doesn't exist."));
      if (ft ? !complexes_.count(cid) : !clusters_.count(cid))
        throw std::runtime_error("Cannot write dump, compute ID " + cid +
                                 std::string(ft ? "is not a per_ftgrid quantity." : "is not a per_grid quantity."));
    };
    if (d.type == "ftgrid") {
      if (!gridset_) throw std::runtime_error("ft_phi does not exist, but needed to save dump.");
      for (auto& a : d.attributes) {
        if (a.rfind("c_", 0) == 0) compute_attr(a, true);
        else if (a.rfind("f_", 0) == 0) throw std::runtime_error("Cannot write dump, fix ID " + a.substr(2) +
                                                                 std::string("is not a per_ftgrid quantity."));
        else throw std::runtime_error("Something wrong, should not get here. ");
      }
    } else if (d.type == "grid") {
      if (!gridset_) throw std::runtime_error("phi does not exist, but needed to save dump.");
      for (auto& a : d.attributes) {
        if (a.rfind("c_", 0) == 0) {
          compute_attr(a, false);
        } else if (a == "gradphi_x" || a == "gradphi_y" || a == "gradphi_z") {
          // the gradient of the step's starting phi, which the reference's
          // arrays hold at a dump (dump.cpp:976-981)
        } else if (a == "chempot") {
          if (!dry_) check(phafd_set_keep_chempot(ctx(), 1));
        } else if (a != "phi") {
          throw std::runtime_error("Dump error: Attribute does not exist.");
        }
      }
    } else {
      phafd_dump::check_atoms(d);
      for (auto& a : d.attributes) {  // per-atom computes (dump.cpp:930-950)
        if (a.rfind("c_", 0) != 0) continue;
        const std::string cid = a.substr(2);
        if (!compute_names_.count(cid))
          throw std::runtime_error("Cannot write dump, compute ID " + cid + std::string("doesn't exist."));
        if (!pair_computes_.count(cid))
          throw std::runtime_error("Cannot write dump, compute ID " + cid + std::string("is not a per_atom quantity."));
      }
    }
    dumps_.push_back(d);
  }

  // a compute's array at a dump: computed on dump steps inside a run; the
  // dump a run writes at its start gets the array as the compute last left
  // it, zeros before any step (integrate.cpp:62-64)
  const std::vector<double>& compute_array(const std::string& cid, bool start_of_run) {
    std::vector<double>& a = compute_cache_[cid];
    const size_t n = complexes_.count(cid) ? ncplx()
                   : pair_computes_.count(cid) ? 3 * (size_t)natoms_ : (size_t)grid_n_[0] * grid_n_[1] * grid_n_[2];
    if (a.size() != n) a.assign(n, 0.0);
    if (start_of_run) return a;
    if (pair_computes_.count(cid)) {
      // the style's forces after the step; like the reference's compute it
      // also adds the style's deposit to chempot (compute_pair.cpp:52-68)
      if (natoms_ > 0) check(phafd_compute_pair(ctx(), pair_computes_.at(cid), 1, a.data()));
    } else if (complexes_.count(cid)) {
      const Complex& c = complexes_.at(cid);
      check(phafd_compute_complex(ctx(), c.field, c.quant, a.data()));
    } else {
      const Cluster& c = clusters_.at(cid);
      std::vector<int> lab(n);
      check(phafd_compute_grid_clusters(ctx(), c.threshold, c.greater ? 1 : 0, lab.data(), nullptr));
      for (size_t k = 0; k < n; ++k) a[k] = lab[k];
    }
    return a;
  }
  size_t ncplx() const { return (size_t)(grid_n_[0] / 2 + 1) * grid_n_[1] * grid_n_[2]; }

  void write_dumps(bool force_all, bool start_of_run) {
    bool any = false;
    for (auto& d : dumps_) any = any || force_all || timestep_ % d.every == 0;
    if (!any) return;
    std::cout << "Saving on step " << timestep_ << std::endl;
    const size_t nr = (size_t)grid_n_[0] * grid_n_[1] * grid_n_[2];
    std::vector<double> x, ux, f;
    std::vector<int> img;
    std::map<std::string, std::vector<double>> fields;
    std::set<std::string> done;  // computes evaluated at this step
    // compute pair runs after every step of the reference, before its dumps
    // read chempot (integrate.cpp:172-183): evaluate it first
    for (auto& pc : pair_computes_) {
      compute_array(pc.first, start_of_run);
      done.insert(pc.first);
    }
    for (auto& d : dumps_) {
      if (!force_all && timestep_ % d.every != 0) continue;
      phafd_dump::Atoms a;
      phafd_dump::Grid g;
      if (d.type == "grid" || d.type == "ftgrid") {
        if (d.type == "grid") {
          g.nx = grid_n_[0]; g.ny = grid_n_[1]; g.nz = grid_n_[2];
          for (int k = 0; k < 3; ++k) {
            g.boxlo[k] = boxlo_[k];
            g.spacing[k] = period_[k] / grid_n_[k];
          }
        } else {  // the transposed half spectrum [ky][kz][kx] (grid.cpp:212-225), spacing dq (domain.cpp:206-208)
          g.nx = grid_n_[0] / 2 + 1; g.ny = grid_n_[2]; g.nz = grid_n_[1];
          g.spacing[0] = 2 * 3.141592 / period_[0];
          g.spacing[1] = 2 * 3.141592 / period_[2];
          g.spacing[2] = 2 * 3.141592 / period_[1];
        }
        for (auto& att : d.attributes) {
          if (att.rfind("c_", 0) == 0) {
            const std::string cid = att.substr(2);
            g.fields[att] = done.count(cid) ? compute_cache_[cid].data() : compute_array(cid, start_of_run).data();
            done.insert(cid);
            continue;
          }
          if (!fields.count(att)) {
            std::vector<double> buf(nr);
            const int field = att == "phi" ? PHAFD_FIELD_PHI : att == "chempot" ? PHAFD_FIELD_CHEMPOT
                            : att == "gradphi_x" ? PHAFD_FIELD_GRADX_STEP_START
                            : att == "gradphi_y" ? PHAFD_FIELD_GRADY_STEP_START : PHAFD_FIELD_GRADZ_STEP_START;
            check(phafd_grid_get(ctx(), field, buf.data()));
            fields[att] = std::move(buf);
          }
          g.fields[att] = fields[att].data();
        }
      } else {
        if (x.empty()) {
          x.resize(3 * (size_t)natoms_); ux.resize(x.size()); f.resize(x.size()); img.resize(natoms_);
          check(phafd_atoms_get(ctx(), x.data(), ux.data(), f.data(), img.data()));
        }
        a.n = natoms_;
        a.x = x.data(); a.ux = ux.data(); a.f = f.data(); a.images = img.data();
        a.tags = tags_.data(); a.mols = mols_.data(); a.types = types_.data();
        for (auto& att : d.attributes)
          if (att.rfind("c_", 0) == 0) a.computes[att] = compute_cache_[att.substr(2)].data();
        for (int k = 0; k < 3; ++k) {
          a.boxlo[k] = boxlo_[k];
          a.boxhi[k] = boxlo_[k] + period_[k];
        }
      }
      phafd_dump::write_step(d, timestep_, dt_, &a, &g);
    }
  }


  // the reference-noise generator's state for a restart (an extension:
  // the reference keeps no generator state across runs)
  void noise_state(bool write, const std::string& fname) {
    if (!conj_set_) throw std::runtime_error("noise state needs fix grid/conjugate/volfrac");
    if (write) {
      if (dry_) return;
      int n = 0;
      check(phafd_noise_state_get(ctx(), nullptr, 0, &n));
      std::vector<char> buf(n);
      check(phafd_noise_state_get(ctx(), buf.data(), n, &n));
      std::ofstream f(fname);
      if (!f) throw std::runtime_error("cannot open " + fname);
      f << buf.data();
    } else {
      std::ifstream f(fname);
      if (!f) throw std::runtime_error("Cannot open file " + fname);
      std::stringstream ss;
      ss << f.rdbuf();
      if (!dry_) check(phafd_noise_state_set(ctx(), ss.str().c_str()));
    }
  }

  void write_field(const std::string& field, const std::string& fname) {
    const std::map<std::string, int> ids = {{"phi", PHAFD_FIELD_PHI}, {"chempot", PHAFD_FIELD_CHEMPOT},
                                            {"gradx", PHAFD_FIELD_GRADX}, {"grady", PHAFD_FIELD_GRADY},
                                            {"gradz", PHAFD_FIELD_GRADZ}};
    auto it = ids.find(field);
    if (it == ids.end()) throw std::invalid_argument("write_field phi|chempot|gradx|grady|gradz FILE");
    if (dry_) return;
    std::vector<double> buf((size_t)grid_n_[0] * grid_n_[1] * grid_n_[2]);
    check(phafd_grid_get(ctx(), it->second, buf.data()));
    std::ofstream f(fname, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + fname);
    f.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(double)));
  }

  // integrate.cpp:221-415: the events come back from the device in order and
  // are printed with the reference's text after the run
  void run_until_touching(long long nsteps, double touch, bool cont, int delay) {
    if (!dumps_.empty()) throw std::runtime_error("phafd_gpu writes no dumps during run_until_touching");
    std::cout << "Running simulation of solution." << std::endl;
    if (dry_) {
      std::cout << "dry run: " << nsteps << " steps parsed" << std::endl;
      return;
    }
    check(phafd_setup(ctx()));
    auto t0 = std::chrono::steady_clock::now();
    const int maxev = 1024;
    std::vector<long long> steps(maxev);
    std::vector<int> kinds(maxev);
    long long done = 0;
    int nev = 0;
    check(phafd_run_until_touching(ctx(), nsteps, touch, cont ? 1 : 0, delay, &done, maxev, steps.data(),
                                   kinds.data(), &nev));
    auto t1 = std::chrono::steady_clock::now();
    for (int k = 0; k < std::min(nev, maxev); ++k)
      std::cout << (kinds[k] == 0 ? "cyclisation occured at step " : "cyclisation interval ended at step ")
                << steps[k] << std::endl;
    if (nev > maxev) std::cout << "(" << nev - maxev << " further events not kept)" << std::endl;
    phafd_counters c{};
    check(phafd_counters_get(ctx(), &c));
    std::cout << "number of neighbor calls = " << c.neighbor_calls << std::endl;
    std::cout << "other flags:" << std::endl;
    for (auto& f : fh_fixes_)  // Integrate::finalise, integrate.cpp:418-443
      std::cout << f.first << " had phi < 0 " << c.num_less_zero << " times, and phi > 1 " << c.num_great_zero
                << "times." << std::endl;
    std::cout << "Run time = " << std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count() / 1e6
              << "seconds." << std::endl;
  }

  void run(long long nsteps) {  // integrate.cpp:90-219
    std::cout << "Running simulation of solution." << std::endl;
    if (dry_) {
      std::cout << "dry run: " << nsteps << " steps parsed" << std::endl;
      return;
    }
    check(phafd_setup(ctx()));
    // Integrate::setup (integrate.cpp:47-84): collection headers, then the
    // dumps of the starting step
    for (auto& d : dumps_) phafd_dump::collection_header(d);
    write_dumps(false, true);
    auto t0 = std::chrono::steady_clock::now();
    const long long chunk = 1000;
    for (long long s = 0; s < nsteps;) {
      long long n = std::min(chunk, nsteps - s);
      for (auto& d : dumps_) n = std::min(n, d.every - timestep_ % d.every);  // stop at the next dump step
      check(phafd_run(ctx(), (int)n));
      s += n;
      timestep_ += n;
      write_dumps(false, false);  // integrate.cpp:179-186
    }
    auto t1 = std::chrono::steady_clock::now();
    for (auto& d : dumps_) phafd_dump::collection_footer(d);
    phafd_counters c{};
    check(phafd_counters_get(ctx(), &c));
    for (auto& f : fh_fixes_)  // Integrate::finalise, integrate.cpp:418-443
      std::cout << f.first << " had phi < 0 " << c.num_less_zero << " times, and phi > 1 " << c.num_great_zero
                << "times." << std::endl;
    std::cout << "Run time = " << std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count() / 1e6
              << "seconds." << std::endl;
  }
};

}  // namespace

int main(int argc, char** argv) {
  std::string infile;
  std::map<std::string, std::string> vars;
  bool dry = false, sf = false;
  try {
    for (int i = 1; i < argc;) {  // phafd.cpp:30-93
      std::string a = argv[i];
      if (a == "-in") {
        if (i + 1 >= argc) throw std::invalid_argument("Error: input flag '-in' specified, but no file given.");
        infile = argv[i + 1];
        i += 2;
      } else if (a == "-var") {
        if (i + 2 >= argc) throw std::invalid_argument("Error: invalid command line variable specification.");
        std::string v = argv[i + 2];
        int used = 3;
        if (!v.empty() && v[0] == '"') {
          v.erase(v.begin());
          if (!v.empty() && v.back() == '"') {
            v.pop_back();
          } else {
            int k = i + 3;
            for (; k < argc; ++k) {
              v += std::string(" ") + argv[k];
              if (v.back() == '"') { v.pop_back(); break; }
            }
            if (k >= argc) throw std::invalid_argument("Error: open double quotes in command line variable specification.");
            used = k - i + 1;
          }
        }
        vars[argv[i + 1]] = v;
        i += used;
      } else if (a == "-sf" && i + 1 < argc) {
        sf = std::string(argv[i + 1]) == "gpu";
        i += 2;
      } else if (a == "-dry-run") {
        dry = true;
        i += 1;
      } else {
        throw std::invalid_argument("Error: invalid command line variable specification.");
      }
    }
    if (infile.empty()) throw std::runtime_error("Error: need to specify input file.");
    std::ifstream in(infile);
    if (!in) throw std::runtime_error("Error: need to specify input file.");
    Interpreter interp(dry, sf);
    interp.run_file(in, vars);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
