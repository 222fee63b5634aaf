// Stand-in for the external beadrodpmer library's chain integrators (test
// infrastructure for the oracle's parity pin; not part of the product).  The
// library is not vendored and its model is not published with the
// reference, so these classes only satisfy the interface that
// fixatom_semiflexible.cpp instantiates: constructing one (a script that
// uses fix atom/semiflexible/...) raises std::runtime_error.  Parity
// scenarios move beads with fix atom/drag instead.
#ifndef PHAFD_REFPIN_BEADRODPMER_STANDIN_HPP
#define PHAFD_REFPIN_BEADRODPMER_STANDIN_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include <Eigen/Core>

namespace BeadRodPmer {

class ChainStandIn {
 public:
  explicit ChainStandIn(const std::vector<std::string>&) {
    throw std::runtime_error("beadrodpmer (the external chain integrator) is not part of the reference checkout");
  }
  void setup(const Eigen::ColsView&) {}
  void first_step(const Eigen::ColsView&, const Eigen::ColsView&, double) {}
  int second_step(const Eigen::ColsView&, const Eigen::ColsView&, double, int) { return 0; }
  double get_bondlength() const { return 0.0; }
};

class NoTether : public ChainStandIn {
 public:
  using ChainStandIn::ChainStandIn;
};
class SingleTether : public ChainStandIn {
 public:
  using ChainStandIn::ChainStandIn;
};
class DoubleTether : public ChainStandIn {
 public:
  using ChainStandIn::ChainStandIn;
};

}  // namespace BeadRodPmer

#endif
