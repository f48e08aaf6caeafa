// Device-side forEachCell: the visitor runs on the GPU, one call per active
// cell, with the cell's value by reference and its coordinate -- the
// signature of VoxelGrid::forEachCell (bonxai_core/include/bonxai/bonxai.hpp:
// 194-207, 703-743) with a __device__ functor instead of a host lambda.
//
//   Bonxai::device::forEachCell<float>(grid.handle(),
//       [] __device__(float& v, const Bonxai::CoordT& c) { v *= 2.f; });
//
// (an extended __device__ lambda needs nvcc --extended-lambda; a functor
// struct with a __device__ operator() needs nothing). Compile the caller with
// nvcc. Visits run concurrently in unspecified order, as the reference's order
// is unspecified; a visitor that combines results uses atomics. The call
// returns after the visit has finished on the grid's stream.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "bonxai/grid_coord.hpp"
#include "bonxai_gb300.h"

namespace Bonxai {
namespace device {

// One thread per leaf mask word; each on bit is one visit.
template <typename T, typename F>
__global__ void for_each_cell_kernel(bxg_device_view v, F f) {
  const int lb = v.leaf_bits;
  const unsigned lsize = 1u << (3 * lb);
  const unsigned words = lsize >= 64 ? lsize / 64 : 1;
  const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (t >= size_t(v.n_leaves) * words) return;
  const unsigned leaf = unsigned(t / words), wi = unsigned(t % words);
  if (v.leaf_key[4 * size_t(leaf) + 3] == -1) return;  // free slot
  unsigned long long w = v.leaf_mask[t];
  const int kx = v.leaf_key[4 * size_t(leaf)], ky = v.leaf_key[4 * size_t(leaf) + 1],
            kz = v.leaf_key[4 * size_t(leaf) + 2];
  T* cells = reinterpret_cast<T*>(v.leaf_data) + size_t(leaf) * lsize;
  const int lm = (1 << lb) - 1;
  while (w) {
    const unsigned b = unsigned(__ffsll(static_cast<long long>(w)) - 1);
    w &= w - 1;
    const unsigned ci = wi * 64 + b;
    const CoordT c{kx | int(ci & lm), ky | int((ci >> lb) & lm), kz | int((ci >> (2 * lb)) & lm)};
    f(cells[ci], c);
  }
}

template <typename T, typename F>
inline void forEachCell(bxg_grid grid, F f) {
  bxg_device_view v;
  const int st = bxg_grid_device_view(grid, &v);
  if (st != BXG_OK) throw std::runtime_error(bxg_last_error(grid));
  if (v.value_bytes != int(sizeof(T)))
    throw std::runtime_error("forEachCell: sizeof(T) differs from the grid's value size");
  const unsigned lsize = 1u << (3 * v.leaf_bits);
  const size_t threads = size_t(v.n_leaves) * (lsize >= 64 ? lsize / 64 : 1);
  if (!threads) return;
  cudaStream_t s = static_cast<cudaStream_t>(v.stream);
  for_each_cell_kernel<T, F><<<unsigned((threads + 255) / 256), 256, 0, s>>>(v, f);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("forEachCell: ") + cudaGetErrorString(e));
}

}  // namespace device
}  // namespace Bonxai
