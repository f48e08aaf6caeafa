// Coordinates and points of the GB300 sparse grid, with the names and meaning
// of the reference's bonxai_core/include/bonxai/grid_coord.hpp so that caller
// code compiles unchanged:
//   CoordT     int32 cell index {x, y, z}                       (grid_coord.hpp:62-78)
//   Point3D    double point {x, y, z}                           (grid_coord.hpp:32-60)
//   ConvertPoint<Out>(in)  any xyz type: .x/.y/.z members, .x()/.y()/.z()
//                          methods, or [0]/[1]/[2]              (grid_coord.hpp:134-162)
//   PosToCoord / CoordToPos  floor(p * inv_resolution) / c * resolution in
//                            double                             (grid_coord.hpp:80-91)
//   std::hash<CoordT>       for host-side containers            (grid_coord.hpp:209-220)
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace Bonxai {

template <typename PointOut, typename PointIn>
PointOut ConvertPoint(const PointIn& v);

struct Point3D {
  double x = 0;
  double y = 0;
  double z = 0;

  Point3D() = default;
  Point3D(const Point3D&) = default;
  Point3D(Point3D&&) = default;
  Point3D& operator=(const Point3D&) = default;
  Point3D& operator=(Point3D&&) = default;
  Point3D(double x_, double y_, double z_) : x(x_), y(y_), z(z_) {}

  template <typename T, typename = std::enable_if_t<!std::is_same_v<std::decay_t<T>, Point3D>>>
  Point3D(const T& v) {
    *this = ConvertPoint<Point3D>(v);
  }
  template <typename T, typename = std::enable_if_t<!std::is_same_v<std::decay_t<T>, Point3D>>>
  Point3D& operator=(const T& v) {
    *this = ConvertPoint<Point3D>(v);
    return *this;
  }

  double& operator[](size_t i) {
    if (i == 0) return x;
    if (i == 1) return y;
    if (i == 2) return z;
    throw std::runtime_error("out of bound index");
  }
};

struct CoordT {
  int32_t x;
  int32_t y;
  int32_t z;

  int32_t& operator[](size_t i) {
    if (i == 0) return x;
    if (i == 1) return y;
    if (i == 2) return z;
    throw std::runtime_error("out of bound index");
  }
  bool operator==(const CoordT& o) const { return x == o.x && y == o.y && z == o.z; }
  bool operator!=(const CoordT& o) const { return !(*this == o); }
  CoordT operator+(const CoordT& o) const { return {x + o.x, y + o.y, z + o.z}; }
  CoordT operator-(const CoordT& o) const { return {x - o.x, y - o.y, z - o.z}; }
  CoordT& operator+=(const CoordT& o) {
    x += o.x;
    y += o.y;
    z += o.z;
    return *this;
  }
  CoordT& operator-=(const CoordT& o) {
    x -= o.x;
    y -= o.y;
    z -= o.z;
    return *this;
  }
};
static_assert(sizeof(CoordT) == 12, "CoordT must be three packed int32");

// The device computes the same single IEEE multiply and floor.
inline CoordT PosToCoord(const Point3D& p, double inv_resolution) {
  return {static_cast<int32_t>(std::floor(p.x * inv_resolution)),
          static_cast<int32_t>(std::floor(p.y * inv_resolution)),
          static_cast<int32_t>(std::floor(p.z * inv_resolution))};
}

inline Point3D CoordToPos(const CoordT& c, double resolution) {
  return {static_cast<double>(c.x) * resolution, static_cast<double>(c.y) * resolution,
          static_cast<double>(c.z) * resolution};
}

namespace detail {
template <class T, class = void>
struct has_method_x : std::false_type {};
template <class T>
struct has_method_x<T, std::void_t<decltype(std::declval<const T&>().x())>> : std::true_type {};

template <class T, class = void>
struct has_member_x : std::false_type {};
template <class T>
struct has_member_x<T, std::void_t<decltype(T::x)>> : std::true_type {};

template <class T>
struct is_indexable3 : std::false_type {};
template <class T, class A>
struct is_indexable3<std::vector<T, A>> : std::true_type {};
template <class T>
struct is_indexable3<std::array<T, 3>> : std::true_type {};

// Scalar type of an xyz point type (float for pcl::PointXYZ / Vector3f, ...).
template <class P>
auto scalar_of(const P& p) {
  if constexpr (has_method_x<P>::value) {
    return p.x();
  } else if constexpr (has_member_x<P>::value) {
    return p.x;
  } else {
    return p[0];
  }
}
template <class P>
using scalar_t = std::decay_t<decltype(scalar_of(std::declval<const P&>()))>;
}  // namespace detail

template <typename PointOut, typename PointIn>
inline PointOut ConvertPoint(const PointIn& v) {
  if constexpr (std::is_same_v<PointIn, PointOut>) {
    return v;
  } else if constexpr (detail::has_method_x<PointIn>::value) {
    return {v.x(), v.y(), v.z()};
  } else if constexpr (detail::has_member_x<PointIn>::value) {
    return {v.x, v.y, v.z};
  } else {
    static_assert(detail::is_indexable3<PointIn>::value, "Can't convert from the specified type");
    return {v[0], v[1], v[2]};
  }
}

}  // namespace Bonxai

namespace std {
template <>
struct hash<Bonxai::CoordT> {
  size_t operator()(const Bonxai::CoordT& c) const {
    uint64_t h = uint64_t(uint32_t(c.x)) * 0x9E3779B97F4A7C15ull;
    h ^= uint64_t(uint32_t(c.y)) * 0xC2B2AE3D27D4EB4Full + (h >> 29);
    h ^= uint64_t(uint32_t(c.z)) * 0x165667B19E3779F9ull + (h >> 31);
    return size_t(h ^ (h >> 32));
  }
};
}  // namespace std
