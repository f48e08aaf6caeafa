// Serialization of a device grid in the reference's byte format, with the
// interface of bonxai_core/include/bonxai/serialization.hpp:
//   Serialize(std::ostream&, const VoxelGrid<T>&)
//   GetHeaderInfo(std::string header line)
//   Deserialize<T>(std::istream&, HeaderInfo)   (header line already read)
// Streams written here are read by the reference and vice versa; roots are
// written in ascending key order (the reference writes its unordered_map's
// order -- the format does not fix one).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <istream>
#include <iterator>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <typeinfo>
#include <vector>

#include "bonxai/bonxai.hpp"

#ifdef __GNUG__
#include <cxxabi.h>

#include <cstdlib>
#endif

namespace Bonxai {

struct HeaderInfo {
  std::string type_name;
  int inner_bits = 0;
  int leaf_bits = 0;
  double resolution = 0;
};

namespace details {
inline std::string demangle(const char* name) {
#ifdef __GNUG__
  int status = -4;
  std::unique_ptr<char, void (*)(void*)> res{abi::__cxa_demangle(name, nullptr, nullptr, &status),
                                             std::free};
  return status == 0 ? std::string(res.get()) : std::string(name);
#else
  return name;
#endif
}
}  // namespace details

template <typename DataT>
inline void Serialize(std::ostream& out, const VoxelGrid<DataT>& grid) {
  const std::string type_name = details::demangle(typeid(DataT).name());
  size_t n = 0;
  int st = bxg_grid_serialize(grid.handle(), type_name.c_str(), nullptr, 0, &n);
  if (st != BXG_OK && st != BXG_ERR_CAPACITY) detail::check(st, grid.handle());
  std::vector<char> buf(n);
  detail::check(bxg_grid_serialize(grid.handle(), type_name.c_str(), buf.data(), n, &n),
                grid.handle());
  out.write(buf.data(), std::streamsize(n));
}

// Parses "Bonxai::VoxelGrid<type,inner_bits,leaf_bits>(resolution)".
inline HeaderInfo GetHeaderInfo(std::string header) {
  const std::string prefix = "Bonxai::VoxelGrid<";
  if (header.rfind(prefix, 0) != 0) throw std::runtime_error("Header wasn't recognized");
  const size_t lt = header.rfind('>');
  const size_t c2 = header.rfind(',', lt);
  const size_t c1 = header.rfind(',', c2 - 1);
  const size_t lp = header.find('(', lt);
  const size_t rp = header.find(')', lp);
  if (lt == std::string::npos || c1 == std::string::npos || c2 == std::string::npos ||
      lp == std::string::npos || rp == std::string::npos)
    throw std::runtime_error("Header wasn't recognized");
  HeaderInfo info;
  info.type_name = header.substr(prefix.size(), c1 - prefix.size());
  info.inner_bits = std::stoi(header.substr(c1 + 1, c2 - c1 - 1));
  info.leaf_bits = std::stoi(header.substr(c2 + 1, lt - c2 - 1));
  info.resolution = std::stod(header.substr(lp + 1, rp - lp - 1));
  return info;
}

template <typename DataT>
inline VoxelGrid<DataT> Deserialize(std::istream& input, HeaderInfo info) {
  if (details::demangle(typeid(DataT).name()) != info.type_name)
    throw std::runtime_error("DataT does not match");
  VoxelGrid<DataT> grid(info.resolution, uint8_t(info.inner_bits), uint8_t(info.leaf_bits));
  char header[256];
  std::snprintf(header, sizeof(header), "Bonxai::VoxelGrid<%s,%d,%d>(%lf)\n",
                info.type_name.c_str(), info.inner_bits, info.leaf_bits, info.resolution);
  std::vector<char> bytes(header, header + std::strlen(header));
  // Read exactly this grid's bytes (serialization.hpp:164-196), leaving the
  // stream after it as the reference does.
  auto take = [&](size_t k) -> const char* {
    const size_t at = bytes.size();
    bytes.resize(at + k);
    if (!input.read(bytes.data() + at, std::streamsize(k)))
      throw std::runtime_error("truncated stream");
    return bytes.data() + at;
  };
  const size_t iwords = std::max<size_t>((size_t(1) << (3 * info.inner_bits)) / 64, 1);
  const size_t lwords = std::max<size_t>((size_t(1) << (3 * info.leaf_bits)) / 64, 1);
  const size_t vbytes = detail::value_bytes<DataT>();
  uint32_t nroots = 0;
  std::memcpy(&nroots, take(4), 4);
  for (uint32_t r = 0; r < nroots; r++) {
    take(12);
    std::vector<uint64_t> inner(iwords);
    std::memcpy(inner.data(), take(iwords * 8), iwords * 8);
    for (uint64_t w : inner) {
      for (; w; w &= w - 1) {
        std::vector<uint64_t> leaf(lwords);
        std::memcpy(leaf.data(), take(lwords * 8), lwords * 8);
        size_t on = 0;
        for (uint64_t lw : leaf) on += size_t(__builtin_popcountll(lw));
        take(on * vbytes);
      }
    }
  }
  detail::check(bxg_grid_deserialize(grid.handle(), bytes.data(), bytes.size()), grid.handle());
  return grid;
}

}  // namespace Bonxai
