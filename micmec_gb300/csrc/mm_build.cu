// Topology of a micromechanical system built on the device from its grid of cell
// types: the tables of build_system (micmec/utils.py:164-263) and Grid._get_nodes
// (utils.py:113-136) without the reference's per-cell node search.
//
// Orderings follow the reference: cells and nodes are numbered lexicographically over
// their grid coordinates (last index fastest), keeping only occupied cells and nodes
// that touch an occupied cell; corner k of a cell is neighbor_nodes[k] (utils.py:43-52);
// a node's mass is the sum of 1/8 of its cells' type masses, added in increasing cell
// order (utils.py:217-218). Numbering is a stream compaction: an exclusive prefix sum
// of the occupancy flags over tiles of 8,192 grid points (per-tile counts, one block
// scanning the tile counts, then per-tile block scans), all integer, so the tables are
// bit-identical to the host builder's. Every kernel is a streaming pass over the grid:
// HBM-bound integer work (int64 tables of 8 entries per cell and per node dominate).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "../../include/micmec_gb300.h"
#include "mm_handle.h"

namespace {

constexpr int kScanThreads = 1024;
constexpr int kItems = 8;
constexpr int kTile = kScanThreads * kItems;
constexpr int kMaxTypeIds = 256;

// corner offsets of a cell (neighbor_nodes, utils.py:43-52)
__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                   {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

struct Geo {
  int nx, ny, nz;     // cells per axis
  int nnx, nny, nnz;  // node grid per axis: n (periodic) or n + 1
  int px, py, pz;     // periodic axes
  int ntypes;         // type ids are 0 (vacancy) .. ntypes - 1
  long long ncell_grid, nnode_grid;
  int* err;           // set when a type id is out of range
};

__device__ __forceinline__ long long cell_at(const Geo& g, int x, int y, int z) {
  return ((long long)x * g.ny + y) * g.nz + z;
}

// Grid cell that has node (k, l, m) as its corner c, or -1 outside a non-periodic grid.
__device__ __forceinline__ long long cell_of_corner(const Geo& g, int k, int l, int m, int c) {
  int x = k - c_corner[c][0], y = l - c_corner[c][1], z = m - c_corner[c][2];
  if (x < 0) {
    if (!g.px) return -1;
    x += g.nx;
  }
  if (y < 0) {
    if (!g.py) return -1;
    y += g.ny;
  }
  if (z < 0) {
    if (!g.pz) return -1;
    z += g.nz;
  }
  if (x >= g.nx || y >= g.ny || z >= g.nz) return -1;
  return cell_at(g, x, y, z);
}

__device__ __forceinline__ void node_coords(const Geo& g, long long n, int& k, int& l, int& m) {
  m = (int)(n % g.nnz);
  const long long r = n / g.nnz;
  l = (int)(r % g.nny);
  k = (int)(r / g.nny);
}

// SRC 0: cell occupied; SRC 1: node touches an occupied cell (Grid._get_nodes)
template <int SRC>
__device__ __forceinline__ int flag_of(const int32_t* __restrict__ grid, const Geo& g, long long i) {
  if (SRC == 0) return (i < g.ncell_grid && grid[i] != 0) ? 1 : 0;
  if (i >= g.nnode_grid) return 0;
  int k, l, m;
  node_coords(g, i, k, l, m);
  for (int c = 0; c < 8; ++c) {
    const long long cell = cell_of_corner(g, k, l, m, c);
    if (cell >= 0 && grid[cell] != 0) return 1;
  }
  return 0;
}

// exclusive block scan of one count per thread; returns the prefix, *total the block sum
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < nw) warp_sums[lane] = w;  // inclusive warp-total prefix
  }
  __syncthreads();
  const int before = warp > 0 ? warp_sums[warp - 1] : 0;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  return before + x - v;
}

// per-tile flag counts
template <int SRC>
__global__ void __launch_bounds__(kScanThreads) k_tile_counts(const int32_t* __restrict__ grid, Geo g,
                                                             long long n, long long* __restrict__ tile_count) {
  __shared__ int ws[32];
  const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < kItems; ++j)
    if (base + j < n) {
      cnt += flag_of<SRC>(grid, g, base + j);
      if (SRC == 0 && (grid[base + j] < 0 || grid[base + j] >= g.ntypes)) atomicExch(g.err, 1);
    }
  int total;
  block_exclusive_scan(cnt, ws, &total);
  if (threadIdx.x == 0) tile_count[blockIdx.x] = total;
}

// exclusive scan of the tile counts in one block; tile_count[ntiles] = grand total
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(long long* __restrict__ tile_count, int ntiles) {
  __shared__ long long carry_s;
  __shared__ long long ws[32];
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int start = 0; start < ntiles; start += kScanThreads) {
    const int i = start + threadIdx.x;
    const long long v = i < ntiles ? tile_count[i] : 0;
    long long x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
      long long w = ws[lane];
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, w, off);
        if (lane >= off) w += y;
      }
      ws[lane] = w;
    }
    __syncthreads();
    const long long carry = carry_s;
    const long long excl = carry + (warp > 0 ? ws[warp - 1] : 0) + x - v;
    if (i < ntiles) tile_count[i] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = carry + ws[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_count[ntiles] = carry_s;
}

// index[i] = rank of i among the flagged points, -1 where unflagged
template <int SRC>
__global__ void __launch_bounds__(kScanThreads) k_tile_index(const int32_t* __restrict__ grid, Geo g, long long n,
                                                            const long long* __restrict__ tile_offset,
                                                            long long* __restrict__ index) {
  __shared__ int ws[32];
  const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
  int f[kItems];
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    f[j] = (base + j < n) ? flag_of<SRC>(grid, g, base + j) : 0;
    cnt += f[j];
  }
  int total;
  long long r = tile_offset[blockIdx.x] + block_exclusive_scan(cnt, ws, &total);
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    if (base + j < n) index[base + j] = f[j] ? r : -1;
    r += f[j];
  }
}

// surrounding_nodes and types of every occupied cell
__global__ void k_cells_out(const int32_t* __restrict__ grid, Geo g, const long long* __restrict__ cell_index,
                            const long long* __restrict__ node_index, int64_t* __restrict__ snodes,
                            int32_t* __restrict__ types) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g.ncell_grid;
       i += (long long)gridDim.x * blockDim.x) {
    const long long ci = cell_index[i];
    if (ci < 0) continue;
    const int z = (int)(i % g.nz);
    const long long r = i / g.nz;
    const int y = (int)(r % g.ny), x = (int)(r / g.ny);
    long long nd[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int k = (x + c_corner[c][0]) % g.nnx, l = (y + c_corner[c][1]) % g.nny, m = (z + c_corner[c][2]) % g.nnz;
      nd[c] = node_index[((long long)k * g.nny + l) * g.nnz + m];
    }
    longlong2* row = reinterpret_cast<longlong2*>(snodes + ci * 8);
#pragma unroll
    for (int q = 0; q < 4; ++q) row[q] = make_longlong2(nd[2 * q], nd[2 * q + 1]);
    types[ci] = grid[i];
  }
}

// compare-exchange of (key, type) pairs in registers
__device__ __forceinline__ void cswap(long long& a, int& ta, long long& b, int& tb) {
  if (b < a) {
    const long long k = a;
    a = b;
    b = k;
    const int t = ta;
    ta = tb;
    tb = t;
  }
}

// surrounding_cells, masses, positions and boundary flags of every node. The node's
// cells are put in increasing index order by Batcher's odd-even merge network for
// eight keys (19 comparators on registers; absent cells sort last) before their masses
// are added.
__global__ void k_nodes_out(const int32_t* __restrict__ grid, Geo g, const long long* __restrict__ cell_index,
                            const long long* __restrict__ node_index, const double* __restrict__ cell_mass,
                            double dx, double dy, double dz, int64_t* __restrict__ scells,
                            double* __restrict__ masses, double* __restrict__ pos, uint8_t* __restrict__ boundary) {
  constexpr long long kAbsent = 0x7fffffffffffffffLL;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < g.nnode_grid;
       n += (long long)gridDim.x * blockDim.x) {
    const long long ni = node_index[n];
    if (ni < 0) continue;
    int k, l, m;
    node_coords(g, n, k, l, m);
    long long ci[8], key[8];
    int ty[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const long long cell = cell_of_corner(g, k, l, m, c);
      ci[c] = cell >= 0 ? cell_index[cell] : -1;
      key[c] = ci[c] >= 0 ? ci[c] : kAbsent;
      ty[c] = ci[c] >= 0 ? grid[cell] : 0;
    }
    longlong2* row = reinterpret_cast<longlong2*>(scells + ni * 8);
#pragma unroll
    for (int q = 0; q < 4; ++q) row[q] = make_longlong2(ci[2 * q], ci[2 * q + 1]);
    // Batcher odd-even merge sort, n = 8
    cswap(key[0], ty[0], key[1], ty[1]); cswap(key[2], ty[2], key[3], ty[3]);
    cswap(key[4], ty[4], key[5], ty[5]); cswap(key[6], ty[6], key[7], ty[7]);
    cswap(key[0], ty[0], key[2], ty[2]); cswap(key[1], ty[1], key[3], ty[3]);
    cswap(key[4], ty[4], key[6], ty[6]); cswap(key[5], ty[5], key[7], ty[7]);
    cswap(key[1], ty[1], key[2], ty[2]); cswap(key[5], ty[5], key[6], ty[6]);
    cswap(key[0], ty[0], key[4], ty[4]); cswap(key[1], ty[1], key[5], ty[5]);
    cswap(key[2], ty[2], key[6], ty[6]); cswap(key[3], ty[3], key[7], ty[7]);
    cswap(key[2], ty[2], key[4], ty[4]); cswap(key[3], ty[3], key[5], ty[5]);
    cswap(key[1], ty[1], key[2], ty[2]); cswap(key[3], ty[3], key[4], ty[4]);
    cswap(key[5], ty[5], key[6], ty[6]);
    double mass = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (key[j] != kAbsent) mass += cell_mass[min(max(ty[j], 0), kMaxTypeIds - 1)];
    masses[ni] = mass;
    pos[ni * 3 + 0] = k * dx;
    pos[ni * 3 + 1] = l * dy;
    pos[ni * 3 + 2] = m * dz;
    boundary[ni] = (k == 0 || k == g.nnx - 1 || l == 0 || l == g.nny - 1 || m == 0 || m == g.nnz - 1) ? 1 : 0;
  }
}

template <int SRC>
cudaError_t compact(const int32_t* grid, const Geo& g, long long n, long long* tiles, long long* index,
                    cudaStream_t st) {
  const int ntiles = (int)((n + kTile - 1) / kTile);
  k_tile_counts<SRC><<<ntiles, kScanThreads, 0, st>>>(grid, g, n, tiles);
  k_scan_tiles<<<1, kScanThreads, 0, st>>>(tiles, ntiles);
  k_tile_index<SRC><<<ntiles, kScanThreads, 0, st>>>(grid, g, n, tiles, index);
  return cudaGetLastError();
}

}  // namespace

extern "C" mm_status mm_build_topology(const int32_t* grid, int nx, int ny, int nz, const int32_t* pbc,
                                       const double* type_mass, int ntype_ids, const double* cell_size,
                                       int64_t* surrounding_nodes, int64_t* surrounding_cells, double* masses,
                                       double* pos, int32_t* types, uint8_t* boundary, int64_t* counts,
                                       void* stream) {
  if (!grid || nx < 1 || ny < 1 || nz < 1 || !pbc || !type_mass || ntype_ids < 1 || ntype_ids > kMaxTypeIds ||
      !cell_size || !surrounding_nodes || !surrounding_cells || !masses || !pos || !types || !boundary || !counts) {
    mm::set_error("mm_build_topology: bad argument");
    return MM_ERR_ARG;
  }
  if (((uintptr_t)surrounding_nodes | (uintptr_t)surrounding_cells) & 15u) {
    mm::set_error("mm_build_topology: the surrounding tables must be 16-byte aligned");
    return MM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  Geo g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.px = pbc[0] != 0;
  g.py = pbc[1] != 0;
  g.pz = pbc[2] != 0;
  g.nnx = nx + 1 - g.px;
  g.nny = ny + 1 - g.py;
  g.nnz = nz + 1 - g.pz;
  g.ntypes = ntype_ids;
  g.ncell_grid = (long long)nx * ny * nz;
  g.nnode_grid = (long long)g.nnx * g.nny * g.nnz;
  const long long ntiles = (std::max(g.ncell_grid, g.nnode_grid) + kTile - 1) / kTile;
  // scratch: cell and node index maps, tile offsets (+ grand total), error flag; cell masses
  const size_t nscratch = (size_t)(g.ncell_grid + g.nnode_grid + ntiles + 2);
  long long* scratch = nullptr;
  double* cmass = nullptr;
  cudaError_t e = cudaMalloc((void**)&scratch, nscratch * sizeof(long long));
  if (e == cudaSuccess) e = cudaMalloc((void**)&cmass, kMaxTypeIds * sizeof(double));
  double hmass[kMaxTypeIds] = {0.0};
  for (int t = 0; t < ntype_ids; ++t) hmass[t] = 0.125 * type_mass[t];
  long long* cell_index = scratch;
  long long* node_index = scratch + g.ncell_grid;
  long long* tiles = node_index + g.nnode_grid;
  g.err = (int*)(tiles + ntiles + 1);
  long long tot[2] = {0, 0};
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(g.err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cmass, hmass, sizeof(hmass), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = compact<0>(grid, g, g.ncell_grid, tiles, cell_index, st);
  if (e == cudaSuccess) {
    const int nt = (int)((g.ncell_grid + kTile - 1) / kTile);
    e = cudaMemcpyAsync(&tot[0], tiles + nt, sizeof(long long), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = compact<1>(grid, g, g.nnode_grid, tiles, node_index, st);
  if (e == cudaSuccess) {
    const int nt = (int)((g.nnode_grid + kTile - 1) / kTile);
    e = cudaMemcpyAsync(&tot[1], tiles + nt, sizeof(long long), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) {
    const int nsm = 152;
    k_cells_out<<<nsm * 8, 256, 0, st>>>(grid, g, cell_index, node_index, surrounding_nodes, types);
    k_nodes_out<<<nsm * 8, 256, 0, st>>>(grid, g, cell_index, node_index, cmass, cell_size[0], cell_size[1],
                                        cell_size[2], surrounding_cells, masses, pos, boundary);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, g.err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (scratch) cudaFree(scratch);
  if (cmass) cudaFree(cmass);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_build_topology: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  if (herr) {
    mm::set_error("mm_build_topology: a cell type id is outside 0 .. ntype_ids - 1");
    return MM_ERR_ARG;
  }
  counts[0] = tot[0];
  counts[1] = tot[1];
  return MM_OK;
}
