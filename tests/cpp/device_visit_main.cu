// A caller of the device-side forEachCell (include/bonxai/device_visit.cuh):
// a functor doubles every value and accumulates a count and a coordinate
// checksum with atomics; the host API then checks the values.
#include <cstdio>
#include <vector>

#include "bonxai/bonxai.hpp"
#include "bonxai/device_visit.cuh"

struct Visit {
  unsigned long long* count;
  long long* checksum;
  __device__ void operator()(float& v, const Bonxai::CoordT& c) const {
    v *= 2.0f;
    atomicAdd(count, 1ull);
    atomicAdd(reinterpret_cast<unsigned long long*>(checksum),
              static_cast<unsigned long long>(static_cast<long long>(c.x) * 3 + c.y * 5 + c.z * 7));
  }
};

int main() {
  Bonxai::VoxelGrid<float> grid(0.05);
  std::vector<Bonxai::CoordT> coords;
  std::vector<float> values;
  long long want_sum = 0;
  for (int x = -20; x < 20; x += 3)
    for (int y = -9; y < 31; y += 2)
      for (int z = -5; z < 6; z++) {
        coords.push_back({x, y, z});
        values.push_back(float(x + 2 * y + 3 * z));
        want_sum += static_cast<long long>(x) * 3 + y * 5 + z * 7;
      }
  grid.setValues(coords, values);
  unsigned long long* d_count;
  long long* d_sum;
  cudaMalloc(&d_count, 8);
  cudaMalloc(&d_sum, 8);
  cudaMemset(d_count, 0, 8);
  cudaMemset(d_sum, 0, 8);
  Bonxai::device::forEachCell<float>(grid.handle(), Visit{d_count, d_sum});
  unsigned long long count = 0;
  long long sum = 0;
  cudaMemcpy(&count, d_count, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(&sum, d_sum, 8, cudaMemcpyDeviceToHost);
  bool ok = count == coords.size() && sum == want_sum;
  auto acc = grid.createConstAccessor();
  for (size_t i = 0; i < coords.size(); i++) {
    const float* p = acc.value(coords[i]);
    if (!p || *p != 2.0f * values[i]) ok = false;
  }
  std::printf("device_visit %s %llu %lld %lld\n", ok ? "ok" : "bad", count, sum, want_sum);
  cudaFree(d_count);
  cudaFree(d_sum);
  return ok ? 0 : 1;
}
