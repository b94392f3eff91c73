// Stand-in for exaNBody's cell grid: cells()[c][field::x][p], the grid
// dimensions and ghost layers, GRID_FOR_BEGIN / GRID_FOR_END over a box of
// cells, grid_ijk_to_index, and a compile-time field test.
#pragma once
#include <cstddef>
#include <cstdint>
#include <sys/types.h>
#include "domain.h"

namespace exanb {
struct IJK {
  ssize_t i = 0, j = 0, k = 0;
};
inline IJK operator-(IJK a, ssize_t b) { return {a.i - b, a.j - b, a.k - b}; }
inline IJK operator+(IJK a, ssize_t b) { return {a.i + b, a.j + b, a.k + b}; }
inline size_t grid_ijk_to_index(IJK dims, IJK loc) { return (size_t)((loc.k * dims.j + loc.j) * dims.i + loc.i); }

namespace field {
struct _rx {}; struct _ry {}; struct _rz {}; struct _vx {}; struct _vy {}; struct _vz {};
struct _fx {}; struct _fy {}; struct _fz {}; struct _ep {}; struct _type {}; struct _id {}; struct _virial {};
constexpr _rx rx{}; constexpr _ry ry{}; constexpr _rz rz{}; constexpr _vx vx{}; constexpr _vy vy{};
constexpr _vz vz{}; constexpr _fx fx{}; constexpr _fy fy{}; constexpr _fz fz{}; constexpr _ep ep{};
constexpr _type type{}; constexpr _id id{}; constexpr _virial virial{};
}  // namespace field

// A cell of particles (SoA); field access returns the field's array.
template <bool VIRIAL>
struct StubCell {
  double* r[10];
  uint8_t* t;
  uint64_t* i;
  Mat3d* v;
  size_t size() const;
  double* operator[](field::_rx) const { return r[0]; }
  double* operator[](field::_ry) const { return r[1]; }
  double* operator[](field::_rz) const { return r[2]; }
  double* operator[](field::_vx) const { return r[3]; }
  double* operator[](field::_vy) const { return r[4]; }
  double* operator[](field::_vz) const { return r[5]; }
  double* operator[](field::_fx) const { return r[6]; }
  double* operator[](field::_fy) const { return r[7]; }
  double* operator[](field::_fz) const { return r[8]; }
  double* operator[](field::_ep) const { return r[9]; }
  uint8_t* operator[](field::_type) const { return t; }
  uint64_t* operator[](field::_id) const { return i; }
  Mat3d* operator[](field::_virial) const { return v; }
};

template <bool VIRIAL>
class StubGrid {
 public:
  using CellT = StubCell<VIRIAL>;
  size_t number_of_cells() const;
  IJK dimension() const;
  ssize_t ghost_layers() const;
  CellT* cells();
  const CellT* cells() const;
};

template <class GridT, class FieldT>
struct GridHasField;
template <bool V, class FieldT>
struct GridHasField<StubGrid<V>, FieldT> {
  static constexpr bool value = true;
};
template <bool V>
struct GridHasField<StubGrid<V>, field::_virial> {
  static constexpr bool value = V;
};

struct GridParticleLocks {};
}  // namespace exanb

#define GRID_FOR_BEGIN(dims, idx, loc)              \
  for (ssize_t k_ = 0; k_ < (dims).k; ++k_)         \
    for (ssize_t j_ = 0; j_ < (dims).j; ++j_)       \
      for (ssize_t i_ = 0; i_ < (dims).i; ++i_) {   \
        const ::exanb::IJK loc{i_, j_, k_};
#define GRID_FOR_END }
