// Caller code written against the reference's C++ API, compiled unchanged
// against include/bonxai/bonxai.hpp and include/bonxai_map/probabilistic_map.hpp
// (the GPU library). It follows the calls of the reference's
// examples/tutorial.cpp and a LiDAR-style insertPointCloud loop, and writes
// its results to text/binary files that tests/test_dropin_cpp.py compares with
// the CPU oracle.
//
// usage: dropin_main <scans.bin> <out_dir>
//   scans.bin: int32 n_scans, int32 n_points, double resolution, double max_range,
//              then per scan: float origin[3], float xyz[n_points*3]
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <algorithm>
#include <cmath>
#include <sstream>
#include <tuple>

#include "bonxai/bonxai.hpp"
#include "bonxai/serialization.hpp"
#include "bonxai_map/probabilistic_map.hpp"

struct PointXYZ {  // pcl::PointXYZ layout: x, y, z and padding
  float x, y, z, pad;
  PointXYZ() = default;
  PointXYZ(float a, float b, float c) : x(a), y(b), z(c), pad(1.0f) {}
};

static int tutorial(const std::string& out) {
  std::ofstream f(out);
  const double VOXEL_RESOLUTION = 0.1;
  Bonxai::VoxelGrid<long> grid(VOXEL_RESOLUTION);
  Bonxai::BinaryVoxelGrid binaryGrid(VOXEL_RESOLUTION);
  auto accessor = grid.createAccessor();
  auto binaryAccessor = binaryGrid.createAccessor();
  // the reference's tutorial fills this cube one scalar call at a time; the
  // batch calls do the same writes in one pass each
  std::vector<Bonxai::CoordT> coords;
  std::vector<long> vals;
  int count = 0;
  for (double x = -1.0; x < 1.0; x += VOXEL_RESOLUTION) {
    for (double y = -1.0; y < 1.0; y += VOXEL_RESOLUTION) {
      for (double z = -1.0; z < 1.0; z += VOXEL_RESOLUTION) {
        coords.push_back(grid.posToCoord(x, y, z));
        vals.push_back(count++);
      }
    }
  }
  grid.setValues(coords, vals);
  binaryGrid.setCellsOn(coords);
  // a few scalar calls too
  accessor.setValue(grid.posToCoord(0.55, 0.55, 0.55), 77);
  binaryAccessor.setCellOn(grid.posToCoord(0.55, 0.55, 0.55));
  f << "cells " << grid.activeCellsCount() << " " << binaryGrid.activeCellsCount() << "\n";

  auto* origin_ptr = accessor.value(grid.posToCoord(0, 0, 0));
  *origin_ptr = 500;
  f << "origin " << *origin_ptr << "\n";
  auto* far_voxel = accessor.value(grid.posToCoord(10, 10, 10), true);
  (*far_voxel)++;
  f << "far " << *far_voxel << "\n";

  auto mutableVisitor = [&grid, &accessor](auto& value, const Bonxai::CoordT& coord) {
    Bonxai::Point3D pos = grid.coordToPos(coord);
    if (pos.z < -0.1) {
      accessor.setCellOff(coord);
    } else {
      value = 1;
    }
  };
  grid.forEachCell(mutableVisitor);

  long sum = 0;
  grid.forEachCell([&sum](const long& v, const Bonxai::CoordT&) { sum += v; });
  f << "after_visit " << grid.activeCellsCount() << " sum " << sum << "\n";

  auto constAccessor = grid.createConstAccessor();
  const auto* cell = constAccessor.value(grid.posToCoord(0, 0, 0));
  f << "const_origin " << (cell ? std::to_string(*cell) : std::string("nullptr")) << "\n";
  cell = constAccessor.value(grid.posToCoord(0, 0, -0.2));
  f << "const_below " << (cell ? std::to_string(*cell) : std::string("nullptr")) << "\n";
  f << "binary_on " << binaryGrid.createConstAccessor().isCellOn(grid.posToCoord(0.55, 0.55, 0.55))
    << "\n";

  // serialization round trip (the reference's examples/test_serialization.cpp
  // flow): Serialize, read the header line, GetHeaderInfo, Deserialize
  std::ostringstream ofile(std::ios::binary);
  Bonxai::Serialize(ofile, grid);
  Bonxai::Serialize(ofile, grid);  // two grids in one stream
  std::istringstream ifile(ofile.str(), std::ios::binary);
  char header[256];
  ifile.getline(header, 256);
  Bonxai::HeaderInfo info = Bonxai::GetHeaderInfo(header);
  auto new_grid = Bonxai::Deserialize<long>(ifile, info);
  ifile.getline(header, 256);
  auto third = Bonxai::Deserialize<long>(ifile, Bonxai::GetHeaderInfo(header));
  bool same = new_grid.activeCellsCount() == grid.activeCellsCount() &&
              third.activeCellsCount() == grid.activeCellsCount();
  auto na = new_grid.createConstAccessor();
  grid.forEachCell([&](const long& v, const Bonxai::CoordT& c) {
    const long* p = na.value(c);
    if (!p || *p != v) same = false;
  });
  f << "serialization " << info.type_name << " " << info.inner_bits << " " << info.leaf_bits
    << " " << (same ? "round_trip_ok" : "round_trip_bad") << "\n";
  return 0;
}

// Walks the tree the way the reference's Serialize does
// (bonxai_core/include/bonxai/serialization.hpp:91-113): rootMap(), the inner
// masks, each leaf's mask and on-cell values. Checks the walk against
// activeCellsCount / forEachCell, getLeafGrid copies against the walk, pointer
// stability of value(), and writes through getLeafGrid and value() pointers.
static int tree(const std::string& out) {
  std::ofstream f(out);
  Bonxai::VoxelGrid<int32_t> grid(0.05);
  std::vector<Bonxai::CoordT> coords;
  std::vector<int32_t> vals;
  for (int i = 0; i < 3000; i++) {
    coords.push_back({(i * 37) % 211 - 100, (i * 53) % 97 - 40, (i * 11) % 61 - 30});
    vals.push_back(i * 7 + 1);
  }
  grid.setValues(coords, vals);
  size_t roots = 0, leaves = 0, cells = 0;
  long long vsum = 0;
  bool leaf_copies_match = true;
  auto ca = grid.createConstAccessor();
  for (const auto& it : grid.rootMap()) {
    const Bonxai::CoordT& root = it.first;
    const auto& inner_grid = it.second;
    roots++;
    for (auto inner = inner_grid.mask().beginOn(); inner; ++inner) {
      const uint32_t ii = *inner;
      const auto& leaf_grid = *(inner_grid.cell(ii));
      leaves++;
      const int lb = int(grid.leafBits()), ib = int(grid.innetBits());
      const int32_t im = (1 << ib) - 1;
      const Bonxai::CoordT lc{root.x | int32_t((ii & im) << lb),
                              root.y | int32_t(((ii >> ib) & im) << lb),
                              root.z | int32_t(((ii >> (2 * ib)) & im) << lb)};
      const auto* copy = ca.getLeafGrid(lc);
      if (!copy || copy != ca.lastLeafGrid() || !ca.lastInnerGrid() ||
          !(copy->mask() == leaf_grid.mask()) ||
          !ca.lastInnerGrid()->mask().isOn(ii))
        leaf_copies_match = false;
      for (auto leaf = leaf_grid.mask().beginOn(); leaf; ++leaf) {
        cells++;
        vsum += leaf_grid.cell(*leaf);
        if (copy && copy->cell(*leaf) != leaf_grid.cell(*leaf)) leaf_copies_match = false;
      }
      ca.releasePointers();  // one leaf copy at a time: the accessor caps live copies
    }
  }
  long long fsum = 0;
  grid.forEachCell([&fsum](const int32_t& v, const Bonxai::CoordT&) { fsum += v; });
  f << "walk " << (cells == grid.activeCellsCount() && vsum == fsum ? "same" : "differs") << " "
    << roots << " " << leaves << " " << cells << "\n";
  f << "leaf_copies " << (leaf_copies_match ? "same" : "differs") << "\n";
  f << "missing_leaf " << (ca.getLeafGrid({5000, 5000, 5000}) == nullptr ? "nullptr" : "found")
    << "\n";

  // value(): one pointer per cell, all of them live at once
  auto acc = grid.createAccessor();
  std::vector<int32_t*> ptrs;
  for (int i = 0; i < 40; i++) ptrs.push_back(acc.value(coords[i]));
  bool stable = acc.value(coords[3]) == ptrs[3];
  for (int i = 0; i < 40; i++) *ptrs[i] = -i - 1;
  acc.flush();
  std::vector<int32_t> got;
  std::vector<uint8_t> found;
  std::vector<Bonxai::CoordT> first(coords.begin(), coords.begin() + 40);
  grid.values(first, got, found);
  bool written = true;
  for (int i = 0; i < 40; i++) written = written && found[i] && got[i] == -i - 1;
  f << "pointers " << (stable ? "stable" : "moved") << " " << (written ? "stored" : "lost") << "\n";

  // getLeafGrid(create): a new, empty leaf; a cell turned on through it
  const Bonxai::CoordT far{4000, -4000, 800};
  const size_t before_cells = grid.activeCellsCount();
  auto* lg = acc.getLeafGrid(far, true);
  const bool empty_leaf = lg && lg->mask().countOn() == 0 && grid.activeCellsCount() == before_cells;
  const uint32_t li = grid.getLeafIndex(far);
  lg->mask().setOn(li);
  lg->cell(li) = 4242;
  acc.flush();
  const int32_t* pv = ca.value(far);
  f << "leaf_create " << (empty_leaf ? "empty" : "not_empty") << " "
    << (pv ? std::to_string(*pv) : std::string("nullptr")) << "\n";
  acc.releasePointers();
  return 0;
}

static int lidar(const std::string& in, const std::string& outdir) {
  std::ifstream f(in, std::ios::binary);
  int32_t n_scans = 0, n_points = 0;
  double res = 0, max_range = 0;
  f.read(reinterpret_cast<char*>(&n_scans), 4);
  f.read(reinterpret_cast<char*>(&n_points), 4);
  f.read(reinterpret_cast<char*>(&res), 8);
  f.read(reinterpret_cast<char*>(&max_range), 8);
  Bonxai::ProbabilisticMap map(res);
  // the ROS node's flow: sensor-frame clouds + pose (identity rotation here),
  // against insertPointCloud of the same world points
  Bonxai::ProbabilisticMap node_map(res), plain_map(res);
  struct Pose {
    float m[3][4];
    float operator()(int r, int c) const { return m[r][c]; }
  };
  std::vector<float> buf(size_t(n_points) * 3);
  for (int s = 0; s < n_scans; s++) {
    float o[3];
    f.read(reinterpret_cast<char*>(o), 12);
    f.read(reinterpret_cast<char*>(buf.data()), buf.size() * 4);
    std::vector<PointXYZ> cloud, sensor, world;
    cloud.reserve(n_points);
    for (int i = 0; i < n_points; i++) {
      cloud.emplace_back(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]);
      sensor.emplace_back(buf[3 * i] - o[0], buf[3 * i + 1] - o[1], buf[3 * i + 2] - o[2]);
      world.emplace_back(sensor.back().x + o[0], sensor.back().y + o[1], sensor.back().z + o[2]);
    }
    sensor.emplace_back(std::nanf(""), 0.f, 0.f);  // dropped by the ingest
    map.insertPointCloud(cloud, PointXYZ(o[0], o[1], o[2]), max_range);
    const Pose pose{{{1, 0, 0, o[0]}, {0, 1, 0, o[1]}, {0, 0, 1, o[2]}}};
    node_map.insertSensorCloud(sensor, pose, max_range);
    plain_map.insertPointCloud(world, PointXYZ(o[0], o[1], o[2]), max_range);
  }
  {
    std::vector<Bonxai::CoordT> a, b;
    node_map.getOccupiedVoxels(a);
    plain_map.getOccupiedVoxels(b);
    auto key = [](const Bonxai::CoordT& c) { return std::make_tuple(c.x, c.y, c.z); };
    auto less = [&](const Bonxai::CoordT& l, const Bonxai::CoordT& r) { return key(l) < key(r); };
    std::sort(a.begin(), a.end(), less);
    std::sort(b.begin(), b.end(), less);
    bool same = a.size() == b.size() && node_map.grid().activeCellsCount() ==
                                            plain_map.grid().activeCellsCount();
    for (size_t i = 0; same && i < a.size(); i++) same = key(a[i]) == key(b[i]);
    // the export: float corner positions of the occupied cells
    std::vector<float> pos(node_map.countOccupied(-1e30, 1e30) * 3);
    const size_t n_exp = node_map.exportOccupied(pos.data(), pos.size() / 3, -1e30, 1e30);
    std::vector<Bonxai::Point3D> want;
    node_map.getOccupiedVoxels(want);
    std::vector<std::tuple<float, float, float>> pe, pw;
    for (size_t i = 0; i < n_exp; i++) pe.emplace_back(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    for (const auto& p : want) pw.emplace_back(float(p.x), float(p.y), float(p.z));
    std::sort(pe.begin(), pe.end());
    std::sort(pw.begin(), pw.end());
    std::ofstream fn(outdir + "/node.txt");
    fn << "ingest " << (same ? "same" : "differs") << " export "
       << (pe == pw && n_exp > 0 ? "same" : "differs") << "\n";
  }
  // hit and miss points by hand, then the free-space rays
  for (int i = 0; i < 200; i++) {
    const double a = 0.01 * i;
    map.addHitPoint(Bonxai::Point3D{1.0 + a, -0.5 + 0.3 * a, 0.8});
    if (i % 3 == 0) map.addMissPoint(Bonxai::Point3D{-2.0 - a, 0.5, 1.2 + 0.1 * a});
  }
  map.updateFreeCells(Bonxai::Point3D{0.05, 0.05, 1.0});

  std::vector<Bonxai::CoordT> occ;
  map.getOccupiedVoxels(occ);
  std::ofstream fo(outdir + "/occupied.bin", std::ios::binary);
  fo.write(reinterpret_cast<const char*>(occ.data()), occ.size() * sizeof(Bonxai::CoordT));

  std::ofstream fc(outdir + "/cells.bin", std::ios::binary);
  map.grid().forEachCell([&fc](const Bonxai::ProbabilisticMap::CellT& c, const Bonxai::CoordT& p) {
    int32_t w;
    std::memcpy(&w, &c, 4);
    fc.write(reinterpret_cast<const char*>(&p), 12);
    fc.write(reinterpret_cast<const char*>(&w), 4);
  });
  std::vector<Bonxai::CoordT> probe(occ.begin(), occ.begin() + std::min<size_t>(occ.size(), 50));
  int n_occ = 0;
  for (const auto& c : probe) n_occ += map.isOccupied(c);
  std::ofstream ft(outdir + "/summary.txt");
  ft << "occupied " << occ.size() << " probe_occ " << n_occ << " probe " << probe.size() << "\n";
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: dropin_main <scans.bin> <out_dir>\n";
    return 2;
  }
  try {
    tutorial(std::string(argv[2]) + "/tutorial.txt");
    tree(std::string(argv[2]) + "/tree.txt");
    lidar(argv[1], argv[2]);
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
