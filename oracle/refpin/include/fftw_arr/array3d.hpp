// Stand-in for the fftw_arr library's array3D (test infrastructure for the
// oracle's parity pin; not part of the product).  The library is not
// vendored; its semantics here follow its call sites in the reference:
//   * array3D<double>(comm, name, Nx, Ny, Nz): a real field indexed (i, j, k)
//     = (z, y, x), x fastest, each x row padded to 2 (Nx/2 + 1) doubles (the
//     FFTW-MPI r2c layout; the reference writes rows one by one because of
//     it); Nx(), Ny(), Nz() are the logical extents;
//   * array3D<std::complex<double>>(comm, name, Nx, A, B): the transposed
//     half spectrum, indexed (i, j, k) with k over Nx/2 + 1 modes fastest;
//     Nx() is Nx/2 + 1, Ny() is A and Nz() is B;
//   * one rank owns every slow index: get_local0start() is 0;
//   * reverseFlat(n, i, j, k) inverts n = (i Ny + j) Nx + k over the logical
//     extents; xysize() is the storage of one slow index; size() the
//     storage of the whole array; operator/= scales every element and setZero()
//     clears it.
#ifndef PHAFD_REFPIN_ARRAY3D_HPP
#define PHAFD_REFPIN_ARRAY3D_HPP

#include <complex>
#include <cstddef>
#include <string>
#include <type_traits>
#include <vector>

#include <mpi.h>

namespace fftwArr {

template <typename T>
class array3D {
  static constexpr bool kComplex = std::is_same<T, std::complex<double>>::value;

 public:
  array3D(MPI_Comm, const std::string& name, ptrdiff_t nx, ptrdiff_t ny, ptrdiff_t nz)
      : name_(name), ny_(ny), nz_(nz) {
    if (kComplex) {
      nx_ = nx / 2 + 1;
      row_ = nx_;
    } else {
      nx_ = nx;
      row_ = 2 * (nx / 2 + 1);
    }
    v_.assign((size_t)(row_ * ny_ * nz_), T(0));
  }

  T& operator()(ptrdiff_t i, ptrdiff_t j, ptrdiff_t k) { return v_[(size_t)((i * ny_ + j) * row_ + k)]; }
  const T& operator()(ptrdiff_t i, ptrdiff_t j, ptrdiff_t k) const {
    return v_[(size_t)((i * ny_ + j) * row_ + k)];
  }

  int Nx() const { return (int)nx_; }
  int Ny() const { return (int)ny_; }
  int Nz() const { return (int)nz_; }
  ptrdiff_t get_local0start() const { return 0; }
  ptrdiff_t xysize() const { return row_ * ny_; }
  ptrdiff_t size() const { return (ptrdiff_t)v_.size(); }
  std::string get_name() const { return name_; }
  T* data() { return v_.data(); }
  const T* data() const { return v_.data(); }

  void reverseFlat(int n, int& i, int& j, int& k) const {
    k = n % (int)nx_;
    j = (n / (int)nx_) % (int)ny_;
    i = n / ((int)nx_ * (int)ny_);
  }

  void setZero() {
    for (auto& x : v_) x = T(0);
  }
  array3D& operator/=(T s) {
    for (auto& x : v_) x /= s;
    return *this;
  }
  array3D& operator*=(T s) {
    for (auto& x : v_) x *= s;
    return *this;
  }

 private:
  std::string name_;
  ptrdiff_t nx_ = 0, ny_ = 0, nz_ = 0, row_ = 0;
  std::vector<T> v_;
};

}  // namespace fftwArr

#endif
