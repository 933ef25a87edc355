// Force evaluation and fused velocity-Verlet / Langevin steps for one lattice
// spread over the whole GPU.
//
// Per force evaluation two kernels run:
//   k_cells  : one thread per nanocell. Gathers its 8 corner displacements
//              (SoA, coalesced along the fastest lattice direction), evaluates
//              every metastable state and the -kT log-sum-exp combination
//              (mm_device.cuh), writes the 8x3 corner gradient to a corner-major
//              SoA buffer G[(corner*3+xyz)*M + cell], and reduces energy and
//              virial per block in FP64 (deterministic tree).
//   k_gather / k_md_nodes : one thread per node. Sums the <=8 corner gradients
//              of its incident cells in corner order (no atomics; the order of
//              micmec/pes/mmff.py:303-318), then either adds the result to the
//              caller's gradient (ForcePart.compute) or performs the
//              velocity-Verlet kick/drift and Langevin updates in FP64.
// Grid-wide totals use a "last block" pattern: every block writes a partial,
// an integer ticket picks the last block, and that block sums the partials in
// block order, so results are bit-reproducible run to run.
//
// Periodic lattices whose cells fill the grid (N == M, node index == cell
// index) use implicit topology (STRUCT = true): no index tables are read.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/micmec_gb300.h"
#include "mm_device.cuh"
#include "mm_handle.h"

using namespace mm;

namespace {

constexpr int kCellThreads = 128;
constexpr int kNodeThreads = 256;
constexpr int kMDThreads = 1024;  // node-update blocks: one resident block per SM, few partials
// FP32 node update: per-thread staging slots for 24 gradient floats, v and u (3 doubles each)
// and the mass data (one float4)
constexpr size_t kMDStageBytes = (size_t)kMDThreads * (24 * 4 + 6 * 8 + 16);
constexpr int kCellPart = 10;  // energy + virial(9)
constexpr int kNodePart = 9;   // ekin_a, ekin_b, ekin_c, ktens(6)

struct Topo {
  int N, M, structured, nx, ny, nz;
  FastDiv div_nyz, div_nz;  // / (ny nz), / nz for the implicit lattice index
  const int32_t* cell_nodes;  // [8][M]
  const int32_t* node_cells;  // [8][N]
  const int32_t* node_lat;    // [3][N]
  const uint8_t* cell_type;   // [M]
};

// (i, j, k) of a node or cell index of the implicit lattice (lexicographic, k fastest)
__device__ __forceinline__ void split_index(const Topo& t, int n, int& i, int& j, int& k) {
  i = fdiv(n, t.div_nyz);
  const int r = n - i * (t.ny * t.nz);
  j = fdiv(r, t.div_nz);
  k = r - j * t.nz;
}

__device__ __forceinline__ void lattice_of(const Topo& t, int n, int& a, int& b, int& c) {
  if (t.structured) {
    split_index(t, n, a, b, c);
  } else {
    a = t.node_lat[n];
    b = t.node_lat[t.N + n];
    c = t.node_lat[2 * t.N + n];
  }
}

// node index of corner (bits) of cell `cell` in the implicit periodic lattice
__device__ __forceinline__ int struct_corner_node(const Topo& t, int i, int j, int k, int bits) {
  int a = i + (bits & 1), b = j + ((bits >> 1) & 1), c = k + (bits >> 2);
  a = (a == t.nx) ? 0 : a;
  b = (b == t.ny) ? 0 : b;
  c = (c == t.nz) ? 0 : c;
  return (a * t.ny + b) * t.nz + c;
}

// cell that has node (i,j,k) as corner with offset bits
__device__ __forceinline__ int struct_corner_cell(const Topo& t, int i, int j, int k, int bits) {
  int a = i - (bits & 1), b = j - ((bits >> 1) & 1), c = k - (bits >> 2);
  a = (a < 0) ? t.nx - 1 : a;
  b = (b < 0) ? t.ny - 1 : b;
  c = (c < 0) ? t.nz - 1 : c;
  return (a * t.ny + b) * t.nz + c;
}

// Asynchronous global -> shared copies (cp.async, no registers held while in flight);
// each thread waits for its own copies only.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Build the per-block parameter table in precision T from the FP64 table and
// the current lattice matrix L: B = L - h0 is formed in FP64, then rounded.
template <typename T>
__device__ void load_params(TypeParams<T>* tp, const TypeTable* tt, int ntypes, const double* box) {
  fill_params_block<T>(tp, tt, ntypes, box);
}

// ------------------------------------------------------------------ kernels

template <typename T>
__global__ void k_pos_to_state(Topo t, const double* __restrict__ pos, const double* __restrict__ box,
                               double* __restrict__ u, T* __restrict__ disp) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
  int a, b, c;
  lattice_of(t, n, a, b, c);
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    const double X = a * box[x] + b * box[3 + x] + c * box[6 + x];
    const double val = pos[3 * n + x] - X;
    u[x * t.N + n] = val;
    disp[x * t.N + n] = (T)val;
  }
}

__global__ void k_state_to_pos(Topo t, const double* __restrict__ u, const double* __restrict__ box,
                               double* __restrict__ pos) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
  int a, b, c;
  lattice_of(t, n, a, b, c);
#pragma unroll
  for (int x = 0; x < 3; ++x) pos[3 * n + x] = (a * box[x] + b * box[3 + x] + c * box[6 + x]) + u[x * t.N + n];
}

__global__ void k_aos_to_soa(int N, const double* __restrict__ a, double* __restrict__ s) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
#pragma unroll
  for (int x = 0; x < 3; ++x) s[x * N + n] = a[3 * n + x];
}

__global__ void k_soa_to_aos(int N, const double* __restrict__ s, double* __restrict__ a) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
#pragma unroll
  for (int x = 0; x < 3; ++x) a[3 * n + x] = s[x * N + n];
}

template <typename T, int MODEL, bool STRUCT>
__global__ void __launch_bounds__(kCellThreads) k_cells(Topo t, const TypeTable* __restrict__ tt, int ntypes,
                                                        const double* __restrict__ box, const T* __restrict__ disp,
                                                        T* __restrict__ G, double* __restrict__ ecell,
                                                        double* __restrict__ cpart) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TypeParams<T>* tp = reinterpret_cast<TypeParams<T>*>(smem_raw);
  double* red = reinterpret_cast<double*>(smem_raw + ((sizeof(TypeParams<T>) * ntypes + 15) / 16) * 16);
  __shared__ T Ls[9];
  load_params<T>(tp, tt, ntypes, box);
  if (threadIdx.x < 9) Ls[threadIdx.x] = (T)box[threadIdx.x];
  __syncthreads();

  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[kCellPart];
#pragma unroll
  for (int i = 0; i < kCellPart; ++i) acc[i] = 0.0;
  if (cell < t.M) {
    T du[8][3];
    if (STRUCT) {
      int i, j, k;
      split_index(t, cell, i, j, k);
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int node = struct_corner_node(t, i, j, k, b);
#pragma unroll
        for (int x = 0; x < 3; ++x) du[b][x] = disp[x * t.N + node];
      }
    } else {
#pragma unroll
      for (int kc = 0; kc < 8; ++kc) {
        const int node = t.cell_nodes[kc * t.M + cell];
        const int b = corner_to_bits(kc);
#pragma unroll
        for (int x = 0; x < 3; ++x) du[b][x] = disp[x * t.N + node];
      }
    }
    const int ty = t.cell_type[cell];
    T g[8][3];
    const double E = cell_eval<T, MODEL>(du, tp[ty], g);
#pragma unroll
    for (int kc = 0; kc < 8; ++kc) {
      const int b = corner_to_bits(kc);
#pragma unroll
      for (int x = 0; x < 3; ++x) G[(kc * 3 + x) * (size_t)t.M + cell] = g[b][x];
    }
    if (ecell) ecell[cell] = E;
    acc[0] = E;
    // virial: sum_b g_b (x) (r_b - r_0), r_b - r_0 = offset(b) . L + du_b - du_0
    T vt[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) vt[i] = T(0);
#pragma unroll
    for (int b = 1; b < 8; ++b) {
      T rel[3];
#pragma unroll
      for (int y = 0; y < 3; ++y) {
        T r = du[b][y] - du[0][y];
        if (b & 1) r += Ls[0 * 3 + y];
        if (b & 2) r += Ls[1 * 3 + y];
        if (b & 4) r += Ls[2 * 3 + y];
        rel[y] = r;
      }
#pragma unroll
      for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) vt[x * 3 + y] += g[b][x] * rel[y];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[1 + i] = (double)vt[i];
  }
  if constexpr (sizeof(T) == 8) {
    block_sum<kCellPart>(acc, red);
    if (threadIdx.x == 0)
#pragma unroll
      for (int i = 0; i < kCellPart; ++i) cpart[i * gridDim.x + blockIdx.x] = acc[i];
  } else {
    F2 f[kCellPart];
#pragma unroll
    for (int i = 0; i < kCellPart; ++i) {
      const float hi = (float)acc[i];
      f[i] = F2{hi, i == 0 ? (float)(acc[i] - (double)hi) : 0.0f};
    }
    block_sum_f2_pairs<kCellPart>(f, red);
    if (threadIdx.x == 0)
#pragma unroll
      for (int i = 0; i < kCellPart; ++i) store_pair(cpart + i * gridDim.x + blockIdx.x, f[i]);
  }
}

// Eight lanes per cell for the eight-corner-matrix model: lane a (offset bits of
// corner a) evaluates corner matrix a for every state. The three edges of matrix a
// join vertex a to its neighbours a^1, a^2, a^4, whose displacements come from
// xor-shuffles inside the 8-lane group; state energies are summed with three
// xor-shuffles; vertex a's gradient collects, for each direction d, the row-d
// gradient of matrix a and of matrix a^(1<<d) (the same edge). Corner gradients and
// vertex offsets are staged in shared memory; the gradients are written as
// contiguous runs of the corner-major layout, and the per-cell virial components
// sum_a g_a (x) (r_a - r_0) and energies are formed from the staged tiles by one warp
// per component (warp w: component w; warps 0, 1 also components 8 and 9), so each
// thread carries one or two running sums (compensated FP32 for FP32 cells) and a
// block's partial of a component is one warp sum.
constexpr int kCell8Threads = 256;
constexpr int kCell8Cells = kCell8Threads / 8;
// Row stride of the staging tiles ([24 rows = corner x component][cell slot]). A warp's
// staging store writes one row per corner (8 corners x 4 cell slots): with stride 44
// (3 x 44 = 4 mod 32) those 32 words fall in 32 different banks; with stride 32 the eight
// corners of a cell shared a bank (8-way conflicts on every store).
constexpr int kTileStride = 44;
constexpr int kTileElems = (2 * 24) * kTileStride + kCell8Cells;  // tile, relt, et
static_assert(kCell8Threads == 256 && kCellPart == 10, "component ownership assumes 8 warps and 10 components");

// Programmatic dependent launch of the step kernels (k_cells8, k_md_nodes; launch_pdl):
// such a grid may be scheduled while the kernel before it on the stream is still running.
// Every thread first waits until that kernel has completed and its writes are visible
// (griddepcontrol.wait), before any global access, so the order of reads and writes is
// that of a plain launch; it then lets the next kernel's blocks be scheduled. Launched
// without the attribute, both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

template <typename T, bool STRUCT, bool SIMPLE>
__global__ void __launch_bounds__(kCell8Threads, sizeof(T) == 4 ? 3 : 2) k_cells8(Topo t, const TypeTable* __restrict__ tt, int ntypes,
                                                          const double* __restrict__ box, const T* __restrict__ disp,
                                                          T* __restrict__ G, double* __restrict__ ecell,
                                                          double* __restrict__ cpart) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TypeParams<T>* tp = reinterpret_cast<TypeParams<T>*>(smem_raw);
  const size_t tp_bytes = ((sizeof(TypeParams<T>) * ntypes + 15) / 16) * 16;
  // two buffers (alternating groups), so one barrier per group suffices
  T* const buf0 = reinterpret_cast<T*>(smem_raw + tp_bytes);
  constexpr int kBuf = kTileElems;
  __shared__ T Ls[9];
  pdl_enter();
  load_params<T>(tp, tt, ntypes, box);
  if (threadIdx.x < 9) Ls[threadIdx.x] = (T)box[threadIdx.x];
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int a = threadIdx.x & 7;
  const int cl = threadIdx.x >> 3;
  const int ngroups = (t.M + kCell8Cells - 1) / kCell8Cells;
  // components owned by this warp: c0 = warp (virial x = c0 / 3, y = c0 % 3), and for
  // warps 0, 1 also c1 = 8 (virial zz) / 9 (energy)
  const int c0x = warp / 3, c0y = warp % 3;
  // lattice offset of vertex a, offset(a) . L (the same in every group)
  T loff[3];
#pragma unroll
  for (int x = 0; x < 3; ++x)
    loff[x] = ((a & 1) ? Ls[x] : T(0)) + ((a & 2) ? Ls[3 + x] : T(0)) + ((a & 4) ? Ls[6 + x] : T(0));
  typedef typename std::conditional<sizeof(T) == 8, double, F2>::type Acc;
  Acc acc0{}, acc1{};
  int parity = 0;
  // software pipelining (FP32 cells): the next group's corner displacements and cell type
  // are loaded before the current group is evaluated (FP64: no spare registers, loaded in turn)
  constexpr bool kPrefetch = sizeof(T) == 4;
  T du_n[3];
  int ty_n;
  auto load_group = [&](int gg) {
    const int cc = gg * kCell8Cells + cl;
    du_n[0] = du_n[1] = du_n[2] = T(0);
    ty_n = 0;
    if (gg < ngroups && cc < t.M) {
      int node;
      if (STRUCT) {
        int i, j, k;
        split_index(t, cc, i, j, k);
        node = struct_corner_node(t, i, j, k, a);
      } else {
        node = t.cell_nodes[bits_to_corner(a) * t.M + cc];
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) du_n[x] = disp[x * t.N + node];
      ty_n = t.cell_type[cc];
    }
  };
  if constexpr (kPrefetch) load_group(blockIdx.x);
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x, parity ^= 1) {
  T* tile = buf0 + parity * kBuf;      // [24][kTileStride] corner gradients
  T* relt = tile + 24 * kTileStride;   // [24][kTileStride] vertex offsets r_a - r_0
  T* et = relt + 24 * kTileStride;     // [kCell8Cells] cell energies
  const int cell = grp * kCell8Cells + cl;
  const bool valid = cell < t.M;
  if constexpr (!kPrefetch) load_group(grp);
  T du[3] = {du_n[0], du_n[1], du_n[2]};
  const int ty = ty_n;
  if constexpr (kPrefetch) load_group(grp + gridDim.x);
  T g[3];
  const T Ecell = cell8_eval<T, SIMPLE>(du, a, tp[ty], valid, g);
  // stage corner gradients and vertex offsets r_a - r_0 = offset(a) . L + du_a - du_0
  const int corner = bits_to_corner(a);
  const int src0 = lane & ~7;
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    tile[(corner * 3 + x) * kTileStride + cl] = valid ? g[x] : T(0);
    const T d0 = __shfl_sync(0xffffffffu, du[x], src0);
    relt[(corner * 3 + x) * kTileStride + cl] = (du[x] - d0) + loff[x];
  }
  if (a == 0) et[cl] = valid ? Ecell : T(0);
  if (valid && a == 0 && ecell) ecell[cell] = (double)Ecell;
  __syncthreads();
  {
    // component c0 of cell slot `lane`, corners in reference order
    T v = T(0);
#pragma unroll
    for (int k = 0; k < 8; ++k) v += tile[(k * 3 + c0x) * kTileStride + lane] * relt[(k * 3 + c0y) * kTileStride + lane];
    if constexpr (sizeof(T) == 8) acc0 += v;
    else acc0 = f2_add(acc0, F2{v, 0.0f});
    if (warp < 2) {
      T w = T(0);
      if (warp == 0) {
#pragma unroll
        for (int k = 0; k < 8; ++k) w += tile[(k * 3 + 2) * kTileStride + lane] * relt[(k * 3 + 2) * kTileStride + lane];
      } else {
        w = et[lane];
      }
      if constexpr (sizeof(T) == 8) acc1 += w;
      else acc1 = f2_add(acc1, F2{w, 0.0f});
    }
  }
  // corner-gradient rows: warp w writes rows w, w + 8, w + 16 (one 128-byte run each)
  {
    const int c = grp * kCell8Cells + lane;
    if (c < t.M)
#pragma unroll
      for (int r = warp; r < 24; r += 8) G[r * (size_t)t.M + c] = tile[r * kTileStride + lane];
  }
  }  // groups
  // block partials: slot 0 energy, slot 1 + 3x + y virial; component c -> slot (c == 9 ? 0 : 1 + c)
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      acc0 += __shfl_down_sync(0xffffffffu, acc0, off);
      acc1 += __shfl_down_sync(0xffffffffu, acc1, off);
    }
    if (lane == 0) {
      cpart[(1 + warp) * gridDim.x + blockIdx.x] = acc0;
      if (warp < 2) cpart[(warp == 0 ? 9 : 0) * gridDim.x + blockIdx.x] = acc1;
    }
  } else {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      acc0 = f2_add(acc0, F2{__shfl_down_sync(0xffffffffu, acc0.hi, off), __shfl_down_sync(0xffffffffu, acc0.lo, off)});
      acc1 = f2_add(acc1, F2{__shfl_down_sync(0xffffffffu, acc1.hi, off), __shfl_down_sync(0xffffffffu, acc1.lo, off)});
    }
    if (lane == 0) {
      store_pair(cpart + (1 + warp) * gridDim.x + blockIdx.x, acc0);
      if (warp < 2) store_pair(cpart + (warp == 0 ? 9 : 0) * gridDim.x + blockIdx.x, acc1);
    }
  }
}

// One thread per cell (cell1_eval), both energy models: the thread gathers its cell's eight
// corner displacements and evaluates the cell itself (eight corner matrices or the averaged
// one), so there are no lane exchanges, no per-corner index arithmetic and no staging of
// virial terms (the cell's gradient and vertex offsets stay in registers). Corner gradients are written
// as in k_cells8 (corner-major, coalesced across the threads of a warp). A thread's few
// cells are summed in the cell precision; the per-block sums are compensated FP32 pairs
// (FP32 cells) or doubles, value-major: slot 0 energy, 1 + 3x + y virial.
constexpr int kCell1Threads = 128;
#ifndef MM_CELL1_MINB
#define MM_CELL1_MINB 3
#endif
constexpr int kCell1MinBlocks = MM_CELL1_MINB;  // FP32: resident blocks per SM the registers are sized for

template <typename T, int MODEL, bool STRUCT, bool SIMPLE>
__global__ void __launch_bounds__(kCell1Threads, sizeof(T) == 4 ? kCell1MinBlocks : 2)
    k_cells1(Topo t, const TypeTable* __restrict__ tt, int ntypes, const double* __restrict__ box,
             const T* __restrict__ disp, T* __restrict__ G, double* __restrict__ ecell, double* __restrict__ cpart) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TypeParams<T>* tp = reinterpret_cast<TypeParams<T>*>(smem_raw);
  double* red = reinterpret_cast<double*>(smem_raw + ((sizeof(TypeParams<T>) * ntypes + 15) / 16) * 16);
  __shared__ T Ls[9];
  // Averaged-matrix model, FP32, structured lattice: the next cell's 24 corner displacements
  // are copied into this thread's slots of two alternating buffers (cp.async) while the
  // current cell is evaluated. 64^3 launch: 20.5 -> 19.1 us. The eight-matrix model's
  // longer arithmetic already hides the loads: 27.4 -> 28.7 us with these copies, and the
  // same with only the first cell's corners copied while the block builds its parameter
  // table (the staging buffer's shared memory costs more than the hidden latency gains),
  // so it loads directly.
  constexpr bool kPrefetch = STRUCT && sizeof(T) == 4 && MODEL == 0;
  __shared__ __align__(16) float pre[kPrefetch ? 2 : 1][kPrefetch ? 24 : 1][kPrefetch ? kCell1Threads : 1];
  auto prefetch = [&](int c, int buf) {
    int i, j, k;
    split_index(t, c, i, j, k);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int node = struct_corner_node(t, i, j, k, b);
#pragma unroll
      for (int x = 0; x < 3; ++x) cp_async4(&pre[buf][b * 3 + x][threadIdx.x], disp + x * t.N + node);
    }
    cp_async_commit();
  };
  // FP32 cubic form: block b owns the 32-cell chunks [C b / nb, C (b + 1) / nb) of the
  // C = ceil(M / 32): every SM's resident blocks get the same number of warp passes (+-1)
  // whatever the number of passes per thread, and each warp's cells start on a chunk
  // boundary (64^3 launch 27.4 -> 26.7 us). The other forms grid-stride: the general FP32
  // form, at its register limit with spills, ran 58.7 -> 65.9 us per 64^3 step with the
  // chunked ranges.
  constexpr bool kChunked = SIMPLE && sizeof(T) == 4;
  int c_begin, c_end, stride;
  if constexpr (kChunked) {
    const int nchunk = (t.M + 31) / 32;
    c_begin = (int)(((long long)nchunk * blockIdx.x) / gridDim.x) * 32;
    c_end = min(t.M, (int)(((long long)nchunk * (blockIdx.x + 1)) / gridDim.x) * 32);
    stride = blockDim.x;
  } else {
    c_begin = blockIdx.x * blockDim.x;
    c_end = t.M;
    stride = gridDim.x * blockDim.x;
  }
  pdl_enter();
  if constexpr (kPrefetch) {
    const int c0 = c_begin + threadIdx.x;
    if (c0 < c_end) prefetch(c0, 0);
  }
  load_params<T>(tp, tt, ntypes, box);
  if (threadIdx.x < 9) Ls[threadIdx.x] = (T)box[threadIdx.x];
  __syncthreads();
  T acc[kCellPart];
#pragma unroll
  for (int i = 0; i < kCellPart; ++i) acc[i] = T(0);
  F2 eacc{0.0f, 0.0f};  // FP32 cells: a thread's cell energies summed with compensation
  int buf = 0;
  for (int cell = c_begin + threadIdx.x; cell < c_end; cell += stride) {
    T du[8][3];
    if constexpr (kPrefetch) {
      cp_async_wait_all();
#pragma unroll
      for (int b = 0; b < 8; ++b)
#pragma unroll
        for (int x = 0; x < 3; ++x) du[b][x] = pre[buf][b * 3 + x][threadIdx.x];
      buf ^= 1;
      if (cell + stride < c_end) prefetch(cell + stride, buf);
    } else if (STRUCT) {
      int i, j, k;
      split_index(t, cell, i, j, k);
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int node = struct_corner_node(t, i, j, k, b);
#pragma unroll
        for (int x = 0; x < 3; ++x) du[b][x] = disp[x * t.N + node];
      }
    } else {
#pragma unroll
      for (int kc = 0; kc < 8; ++kc) {
        const int node = t.cell_nodes[kc * t.M + cell];
#pragma unroll
        for (int x = 0; x < 3; ++x) du[corner_to_bits(kc)][x] = disp[x * t.N + node];
      }
    }
    T g[8][3];
    const T Ecell = cell1_eval<T, SIMPLE, MODEL>(du, tp[t.cell_type[cell]], g);
#pragma unroll
    for (int kc = 0; kc < 8; ++kc)
#pragma unroll
      for (int x = 0; x < 3; ++x) G[(kc * 3 + x) * (size_t)t.M + cell] = g[corner_to_bits(kc)][x];
    if (ecell) ecell[cell] = (double)Ecell;
    if constexpr (sizeof(T) == 4) eacc = f2_add(eacc, F2{(float)Ecell, 0.0f});
    else acc[0] += Ecell;
    // virial: sum_b g_b (x) (r_b - r_0), r_b - r_0 = offset(b) . L + du_b - du_0
#pragma unroll
    for (int b = 1; b < 8; ++b) {
      T rel[3];
#pragma unroll
      for (int y = 0; y < 3; ++y) {
        T r = du[b][y] - du[0][y];
        if (b & 1) r += Ls[0 * 3 + y];
        if (b & 2) r += Ls[1 * 3 + y];
        if (b & 4) r += Ls[2 * 3 + y];
        rel[y] = r;
      }
#pragma unroll
      for (int x = 0; x < 3; ++x)
#pragma unroll
        for (int y = 0; y < 3; ++y) acc[1 + x * 3 + y] += g[b][x] * rel[y];
    }
  }
  if constexpr (sizeof(T) == 8) {
    double v[kCellPart];
#pragma unroll
    for (int i = 0; i < kCellPart; ++i) v[i] = acc[i];
    block_sum<kCellPart>(v, red);
    if (threadIdx.x == 0)
#pragma unroll
      for (int i = 0; i < kCellPart; ++i) cpart[i * gridDim.x + blockIdx.x] = v[i];
  } else {
    // values 0..7 as a reduce-scatter (the owning warps store them), 8 and 9 by thread 0;
    // the consumer is the next kernel, so no fence
    static_assert(kCellPart == 10, "energy + 9 virial components");
    F2 f8[8], f2[2];
    f8[0] = eacc;
#pragma unroll
    for (int i = 1; i < 8; ++i) f8[i] = F2{(float)acc[i], 0.0f};
    f2[0] = F2{(float)acc[8], 0.0f};
    f2[1] = F2{(float)acc[9], 0.0f};
    block_scatter_sum8(f8, red, [&](int i, F2 t) { store_pair(cpart + i * gridDim.x + blockIdx.x, t); });
    block_sum_f2_pairs<2>(f2, red + 8 * (kCell1Threads / 32));
    if (threadIdx.x == 0)
#pragma unroll
      for (int i = 0; i < 2; ++i) store_pair(cpart + (8 + i) * gridDim.x + blockIdx.x, f2[i]);
  }
}

template <typename T, bool STRUCT>
__device__ __forceinline__ void gather_node(const Topo& t, const T* __restrict__ G, int n, T (&s)[3]) {
  s[0] = s[1] = s[2] = T(0);
  if (STRUCT) {
    int i, j, k;
    split_index(t, n, i, j, k);
#pragma unroll
    for (int kc = 0; kc < 8; ++kc) {
      const int cell = struct_corner_cell(t, i, j, k, corner_to_bits(kc));
#pragma unroll
      for (int x = 0; x < 3; ++x) s[x] += G[(kc * 3 + x) * (size_t)t.M + cell];
    }
  } else {
#pragma unroll
    for (int kc = 0; kc < 8; ++kc) {
      const int cell = t.node_cells[kc * t.N + n];
      if (cell < 0) continue;
#pragma unroll
      for (int x = 0; x < 3; ++x) s[x] += G[(kc * 3 + x) * (size_t)t.M + cell];
    }
  }
}

template <typename T, bool STRUCT>
__global__ void k_gather(Topo t, const T* __restrict__ G, double* __restrict__ gpos, int* __restrict__ flag) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
  T s[3];
  gather_node<T, STRUCT>(t, G, n, s);
  bool bad = false;
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    const double v = (double)s[x];
    bad |= isnan(v);
    gpos[3 * n + x] += v;
  }
  if (bad && flag) atomicOr(flag, 1);
}

// Sum the per-block partials in block order: energy written, virial added.
template <bool PAIRS>
__global__ void k_finalize(const double* __restrict__ cpart, int nblk, double* __restrict__ energy,
                           double* __restrict__ vtens, int* __restrict__ flag) {
  __shared__ double acc[kCellPart];
  sum_partials_by_warp<kCellPart, 0, PAIRS>(cpart, nblk, nullptr, 0, acc);
  if (threadIdx.x == 0) {
    *energy = acc[0];
    bool bad = isnan(acc[0]);
    if (vtens) {
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        bad |= isnan(acc[1 + i]);
        vtens[i] += acc[1 + i];
      }
    }
    if (bad && flag) atomicOr(flag, 1);
  }
}

struct MDArgs {
  double dt;
  double c1;            // Langevin exp(-dt / (2 timecon))
  double cv;            // velocity factor of the step part run (FP32-cell path): c1^2, c1 or 1
  float hf, c1f;        // dt / 2 and the thermostat factor (1 without one) in FP32
  uint64_t seed;
  int64_t step;         // step being finished (1-based); the next one is step+1
  int64_t noise_step0;  // step index of noise[0]
  int finish;           // kick + post thermostat of `step`
  int start;            // pre thermostat + kick + drift of `step + 1`
};

// The block that arrives last: totals of the nb node-block partials and of the cell
// totals, the step record and the conserved-energy carry. Deterministic (fixed order).
template <typename T>
__device__ __forceinline__ void md_nodes_final(const MDArgs& p, const double* npart, int nb, const double* cell_tot,
                                               unsigned* ticket, double* carry, double* record) {
  __shared__ double tn[kNodePart];
  __shared__ double tc[kCellPart + 1];  // cell totals, then the conserved-energy carry
  __threadfence();
  // warps 0 .. kNodePart-1 sum the node partials; warp kNodePart loads the cell totals and
  // the carry meanwhile (the block has 32 warps)
  static_assert(kNodePart < kMDThreads / 32 && kCellPart < 32, "one idle warp loads the totals");
  if ((int)(threadIdx.x >> 5) == kNodePart) {
    const int lane = threadIdx.x & 31;
    if (lane < kCellPart) tc[lane] = __ldcg(cell_tot + lane);
    else if (lane == kCellPart) tc[kCellPart] = __ldcg(carry);
  }
  sum_partials_by_warp<kNodePart, 0, sizeof(T) == 4>(npart, nb, nullptr, 0, tn);
  if (threadIdx.x == 0) {
    const double ek = (sizeof(T) == 4) ? 0.5 * (tn[3] + tn[4] + tn[5]) : tn[1];
    *ticket = 0u;
    if (record) {
      record[MM_REC_EPOT] = tc[0];
      record[MM_REC_EKIN] = ek;
      record[MM_REC_DECONS] = (p.finish ? (tn[0] - ek) : 0.0) + (p.finish ? tc[kCellPart] : 0.0);
#pragma unroll
      for (int i = 0; i < 9; ++i) record[MM_REC_VTENS + i] = tc[1 + i];
      const double k[9] = {tn[3], tn[8], tn[7], tn[8], tn[4], tn[6], tn[7], tn[6], tn[5]};
#pragma unroll
      for (int i = 0; i < 9; ++i) record[MM_REC_KTENS + i] = k[i];
    }
    carry[0] = p.start ? (ek - tn[2]) : 0.0;
    carry[1] = tc[0];
  }
}

// One thread per node: gather, kick, thermostat, drift, and per-step observables.
template <typename T, bool STRUCT, int THERMO>
__global__ void __launch_bounds__(kMDThreads, 1) k_md_nodes(Topo t, MDArgs p, const T* __restrict__ G,
                                                           double* __restrict__ u, double* __restrict__ v,
                                                           T* __restrict__ disp, const double* __restrict__ mass,
                                                           const double* __restrict__ invm, const double* __restrict__ c2,
                                                           const double* __restrict__ noise, double* __restrict__ npart,
                                                           const double* __restrict__ cpart, int ncblk,
                                                           unsigned* __restrict__ ticket, double* __restrict__ carry,
                                                           double* __restrict__ record, double* __restrict__ gpos_out,
                                                           const float4* __restrict__ nodef) {
  __shared__ double red[kNodePart * (kMDThreads / 32)];
  __shared__ double ctot[kCellPart];
  __shared__ bool last;
  extern __shared__ __align__(16) float md_stage[];  // FP32 cells: per-thread input slots (kMDStageBytes)
  pdl_enter();
  // blocks 0 .. nb-1 update the nodes; block nb (the last one) sums the cell kernel's
  // partials meanwhile, so the block that finishes last has only nb node partials left
  const int nb = gridDim.x - 1;
  double* const cell_tot = npart + (size_t)kNodePart * nb;  // cell totals (FP64), after the node partials
  if (blockIdx.x == nb) {
    sum_partials_by_warp<kCellPart, 0, sizeof(T) == 4>(cpart, ncblk, nullptr, 0, ctot);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int i = 0; i < kCellPart; ++i) cell_tot[i] = ctot[i];
      __threadfence();
      last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last) md_nodes_final<T>(p, npart, nb, cell_tot, ticket, carry, record);
    return;
  }
  // per-node observables: FP64 for an FP64 handle; for an FP32 handle in FP32, summed
  // per warp with compensated FP32 and per block in FP64
  typedef typename std::conditional<sizeof(T) == 8, double, float>::type R;
  typedef typename std::conditional<sizeof(T) == 8, double, F2>::type Acc;
  Acc accum[kNodePart];
#pragma unroll
  for (int i = 0; i < kNodePart; ++i) accum[i] = Acc{};
  // block b owns the 32-node chunks [C b / nb, C (b + 1) / nb) of the C = ceil(N / 32):
  // equal shares for all SMs (+-1 chunk), each warp's nodes starting on a chunk boundary;
  // its threads stride through them
  const int nchunk = (t.N + 31) / 32;
  const int n_begin = (int)(((long long)nchunk * blockIdx.x) / nb) * 32;
  const int n_end = min(t.N, (int)(((long long)nchunk * (blockIdx.x + 1)) / nb) * 32);
  const int n_first_end = n_begin + (int)blockDim.x;  // first pass
  for (int n = n_begin + threadIdx.x; n < n_end; n += blockDim.x) {
  R obs[kNodePart];
#pragma unroll
  for (int i = 0; i < kNodePart; ++i) obs[i] = R(0);
  if constexpr (sizeof(T) == 4) {
    // FP32 cells: the velocity and position increments of the whole step are formed in
    // FP32, the state update itself is FP64:
    //   v' = cv v + q,  u' = u + dt v'
    // with (finish and start) cv = c1^2, q = (c1^2 + 1) h a + c1 n1 + n2; (finish only)
    // cv = c1, q = c1 h a + n1; (start only) cv = c1, q = h a + n2; h = dt/2, a = -g/m,
    // n1/n2 the post/pre thermostat noise terms (c1 = 1, n = 0 without a thermostat).
    // The observables come from an FP32 copy of the same velocity sequence.
    // The node's inputs (24 corner-gradient values, v, u, mass data) are staged in this
    // thread's shared-memory slots with asynchronous copies; the Langevin draws are
    // computed while they are in flight.
    // regions (bases, then this thread's slot in each): gradients [24][kMDThreads] floats,
    // v [3][kMDThreads] and u [3][kMDThreads] doubles, mass data [kMDThreads] float4
    double* const v_base = reinterpret_cast<double*>(md_stage + 24 * kMDThreads);
    double* const u_base = v_base + 3 * kMDThreads;
    float4* const nf_base = reinterpret_cast<float4*>(u_base + 3 * kMDThreads);
    float* const sg = md_stage + threadIdx.x;
    double* const sv = v_base + threadIdx.x;
    double* const su = u_base + threadIdx.x;
    float4* const snf = nf_base + threadIdx.x;
    {
      int ci = 0, cj = 0, ck = 0;
      if (STRUCT) split_index(t, n, ci, cj, ck);
#pragma unroll
      for (int kc = 0; kc < 8; ++kc) {
        const int cell = STRUCT ? struct_corner_cell(t, ci, cj, ck, corner_to_bits(kc)) : t.node_cells[kc * t.N + n];
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          float* dst = sg + (kc * 3 + x) * kMDThreads;
          if (cell >= 0) cp_async4(dst, G + (kc * 3 + x) * (size_t)t.M + cell);
          else *dst = 0.0f;
        }
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        cp_async8(sv + x * kMDThreads, v + x * (size_t)t.N + n);
        if (p.start) cp_async8(su + x * kMDThreads, u + x * (size_t)t.N + n);
      }
      cp_async16(snf, nodef + n);
      cp_async_commit();
    }
    float z1[3] = {0.f, 0.f, 0.f}, z2[3] = {0.f, 0.f, 0.f};
    if (THERMO == MM_THERMO_LANGEVIN) {
      if (p.finish) {
        if (noise) {
          const size_t base = ((size_t)(p.step - p.noise_step0) * 2 + 1) * (size_t)t.N * 3;
#pragma unroll
          for (int x = 0; x < 3; ++x) z1[x] = d2f_rn(noise[base + 3 * n + x]);
        } else {
          normal3(p.seed, (uint32_t)n, (uint32_t)p.step, 1u, z1);
        }
      }
      if (p.start) {
        if (noise) {
          const size_t base = ((size_t)(p.step + 1 - p.noise_step0) * 2 + 0) * (size_t)t.N * 3;
#pragma unroll
          for (int x = 0; x < 3; ++x) z2[x] = d2f_rn(noise[base + 3 * n + x]);
        } else {
          normal3(p.seed, (uint32_t)n, (uint32_t)(p.step + 1), 0u, z2);
        }
      }
    }
    cp_async_wait_all();
    T s[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int kc = 0; kc < 8; ++kc)
#pragma unroll
      for (int x = 0; x < 3; ++x) s[x] += sg[(kc * 3 + x) * kMDThreads];
    const float4 nf = *snf;  // mass, 1/mass, Langevin amplitude
    const float hf = p.hf;
    float af[3], n1[3], n2[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      af[x] = -(float)s[x] * nf.y;
      n1[x] = nf.z * z1[x];
      n2[x] = nf.z * z2[x];
    }
    if (gpos_out)
#pragma unroll
      for (int x = 0; x < 3; ++x) gpos_out[3 * n + x] = f2d(s[x]);
    const float c1 = (THERMO == MM_THERMO_LANGEVIN) ? p.c1f : 1.0f;
    double vv[3];
    float vf[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      vv[x] = sv[x * kMDThreads];
      vf[x] = d2f_rn(vv[x]);
    }
    const float mf = nf.x;
    if (p.finish) {
#pragma unroll
      for (int x = 0; x < 3; ++x) vf[x] += hf * af[x];
      obs[0] = 0.5f * mf * (vf[0] * vf[0] + vf[1] * vf[1] + vf[2] * vf[2]);
#pragma unroll
      for (int x = 0; x < 3; ++x) vf[x] = c1 * vf[x] + n1[x];
    }
    // obs[1] (kinetic energy between the two halves) is 0.5 * (obs[3] + obs[4] + obs[5])
    // and is formed from those totals in the block sum below
    obs[3] = mf * vf[0] * vf[0];
    obs[4] = mf * vf[1] * vf[1];
    obs[5] = mf * vf[2] * vf[2];
    obs[6] = mf * vf[1] * vf[2];
    obs[7] = mf * vf[0] * vf[2];
    obs[8] = mf * vf[0] * vf[1];
    if (p.start) {
#pragma unroll
      for (int x = 0; x < 3; ++x) vf[x] = c1 * vf[x] + n2[x];
      obs[2] = 0.5f * mf * (vf[0] * vf[0] + vf[1] * vf[1] + vf[2] * vf[2]);
    }
    if (p.finish || p.start) {
      const double cv = p.cv;
      float q[3];
      if (p.finish && p.start) {
        const float cc = c1 * c1;
#pragma unroll
        for (int x = 0; x < 3; ++x) q[x] = (cc + 1.0f) * hf * af[x] + c1 * n1[x] + n2[x];
      } else if (p.finish) {
#pragma unroll
        for (int x = 0; x < 3; ++x) q[x] = c1 * hf * af[x] + n1[x];
      } else {
#pragma unroll
        for (int x = 0; x < 3; ++x) q[x] = hf * af[x] + n2[x];
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        vv[x] = fma(cv, vv[x], f2d(q[x]));
        v[x * t.N + n] = vv[x];
      }
      if (p.start)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const double un = fma(p.dt, vv[x], su[x * kMDThreads]);
          u[x * t.N + n] = un;
          disp[x * t.N + n] = d2f_rn(un);
        }
    }
  } else {
    T s[3];
    gather_node<T, STRUCT>(t, G, n, s);
    const double m = mass[n], im = invm[n];
    const R mf = (R)m;
    double vv[3], a[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      vv[x] = v[x * t.N + n];
      a[x] = -(double)s[x] * im;
    }
    if (gpos_out)
#pragma unroll
      for (int x = 0; x < 3; ++x) gpos_out[3 * n + x] = (double)s[x];
    if (p.finish) {
#pragma unroll
      for (int x = 0; x < 3; ++x) vv[x] += 0.5 * a[x] * p.dt;
      {
        const R v0 = (R)vv[0], v1 = (R)vv[1], v2 = (R)vv[2];
        obs[0] = R(0.5) * mf * (v0 * v0 + v1 * v1 + v2 * v2);
      }
      if (THERMO == MM_THERMO_LANGEVIN) {
        double z[3];
        if (noise) {
          const size_t base = ((size_t)(p.step - p.noise_step0) * 2 + 1) * (size_t)t.N * 3;
#pragma unroll
          for (int x = 0; x < 3; ++x) z[x] = noise[base + 3 * n + x];
        } else {
          float zf[3];
          normal3(p.seed, (uint32_t)n, (uint32_t)p.step, 1u, zf);
#pragma unroll
          for (int x = 0; x < 3; ++x) z[x] = zf[x];
        }
        const double amp = c2[n];
#pragma unroll
        for (int x = 0; x < 3; ++x) vv[x] = p.c1 * vv[x] + amp * z[x];
      }
    }
    {
      const R v0 = (R)vv[0], v1 = (R)vv[1], v2 = (R)vv[2];
      obs[1] = R(0.5) * mf * (v0 * v0 + v1 * v1 + v2 * v2);
      obs[3] = mf * v0 * v0;
      obs[4] = mf * v1 * v1;
      obs[5] = mf * v2 * v2;
      obs[6] = mf * v1 * v2;
      obs[7] = mf * v0 * v2;
      obs[8] = mf * v0 * v1;
    }
    if (p.start) {
      if (THERMO == MM_THERMO_LANGEVIN) {
        double z[3];
        if (noise) {
          const size_t base = ((size_t)(p.step + 1 - p.noise_step0) * 2 + 0) * (size_t)t.N * 3;
#pragma unroll
          for (int x = 0; x < 3; ++x) z[x] = noise[base + 3 * n + x];
        } else {
          float zf[3];
          normal3(p.seed, (uint32_t)n, (uint32_t)(p.step + 1), 0u, zf);
#pragma unroll
          for (int x = 0; x < 3; ++x) z[x] = zf[x];
        }
        const double amp = c2[n];
#pragma unroll
        for (int x = 0; x < 3; ++x) vv[x] = p.c1 * vv[x] + amp * z[x];
      }
      {
        const R v0 = (R)vv[0], v1 = (R)vv[1], v2 = (R)vv[2];
        obs[2] = R(0.5) * mf * (v0 * v0 + v1 * v1 + v2 * v2);
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        vv[x] += 0.5 * a[x] * p.dt;
        const double un = u[x * t.N + n] + p.dt * vv[x];
        u[x * t.N + n] = un;
        disp[x * t.N + n] = (T)un;
      }
    }
#pragma unroll
    for (int x = 0; x < 3; ++x) v[x * t.N + n] = vv[x];
  }
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int i = 0; i < kNodePart; ++i) accum[i] += obs[i];
  } else {
    // obs[1] is not summed for FP32 cells (formed from the kinetic tensor's diagonal); a
    // thread's first node starts the compensated sums (exactly what adding it to zero gives)
    if (n < n_first_end) {
#pragma unroll
      for (int i = 0; i < kNodePart; ++i)
        if (i != 1) accum[i] = F2{(float)obs[i], 0.0f};
    } else {
#pragma unroll
      for (int i = 0; i < kNodePart; ++i)
        if (i != 1) accum[i] = f2_add(accum[i], F2{(float)obs[i], 0.0f});
    }
  }
  }  // nodes
  double tot[kNodePart];
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int i = 0; i < kNodePart; ++i) tot[i] = accum[i];
    block_sum<kNodePart>(tot, red);
  } else {
    // accum[1] is not summed: the final sum forms it from the kinetic tensor's diagonal.
    // Warp j stores the block total of value j (observable j, or j + 1 from j = 1 on) and
    // fences its own store before the barrier that precedes the ticket.
    static_assert(kNodePart - 1 == 8, "eight compensated node observables");
    F2 acc[kNodePart - 1];
    acc[0] = accum[0];
#pragma unroll
    for (int i = 2; i < kNodePart; ++i) acc[i - 1] = accum[i];
    block_scatter_sum8(acc, red, [&](int j, F2 tj) {
      store_pair(npart + (j == 0 ? 0 : j + 1) * nb + blockIdx.x, tj);
      if (j == 0) store_pair(npart + 1 * nb + blockIdx.x, F2{0.0f, 0.0f});
      __threadfence();
    });
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if constexpr (sizeof(T) == 8) {
#pragma unroll
      for (int i = 0; i < kNodePart; ++i) npart[i * nb + blockIdx.x] = tot[i];
    }
    __threadfence();
    const unsigned prev = atomicAdd(ticket, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last) md_nodes_final<T>(p, npart, nb, cell_tot, ticket, carry, record);
}

// Host-buffer step, first half in one pass: u = pos - X(L) and v from the caller's
// AoS arrays, then the "pre" thermostat, kick with the caller's gradient, and drift
// (u as k_pos_to_state forms it, then the arithmetic of the host step's first half);
// pos / vel / gpos are the device copies of the caller's arrays. The step's final
// positions X(L) + u are known after the drift: each thread writes them over its own
// entries of pos, so their copy to the host overlaps the force evaluation.
template <typename T, int THERMO>
__global__ void k_md_host_begin(Topo t, MDArgs p, double* pos, const double* __restrict__ vel,
                                const double* __restrict__ gpos, const double* __restrict__ box,
                                double* __restrict__ u, double* __restrict__ v, T* __restrict__ disp,
                                const double* __restrict__ invm, const double* __restrict__ c2,
                                const float4* __restrict__ nodef) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
  int la, lb, lc;
  lattice_of(t, n, la, lb, lc);
  if constexpr (sizeof(T) == 4) {
    // FP32 cells: the start half of k_md_nodes' update. The half step's velocity increment
    // is formed in FP32 (v' = c1 v + q, q = (dt/2) a + amp z, a = -g / m; c1 = 1 and z = 0
    // without a thermostat) and added to the FP64 state; the FP32 displacement is rounded on
    // the integer pipe. FP64 work per component: the lattice site X, u = pos - X, v', u' and
    // the output position X + u' (the FP64 pipe of this part bounds the kernel otherwise).
    const float4 nf = nodef[n];  // mass, 1/mass, Langevin amplitude
    float z[3] = {0.f, 0.f, 0.f};
    if (THERMO == MM_THERMO_LANGEVIN) normal3(p.seed, (uint32_t)n, (uint32_t)p.step, 0u, z);
    const double cv = (THERMO == MM_THERMO_LANGEVIN) ? p.c1 : 1.0;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const double X = la * box[x] + lb * box[3 + x] + lc * box[6 + x];
      const double uu = pos[3 * n + x] - X;
      const float q = p.hf * (-d2f_rn(gpos[3 * n + x]) * nf.y) + nf.z * z[x];
      const double vv = fma(cv, vel[3 * n + x], f2d(q));
      const double un = fma(p.dt, vv, uu);
      u[x * t.N + n] = un;
      disp[x * t.N + n] = d2f_rn(un);
      v[x * t.N + n] = vv;
      pos[3 * n + x] = X + un;
    }
    return;
  }
  double uu[3], vv[3], gg[3];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    uu[x] = pos[3 * n + x] - (la * box[x] + lb * box[3 + x] + lc * box[6 + x]);
    vv[x] = vel[3 * n + x];
    gg[x] = gpos[3 * n + x];
  }
  if (THERMO == MM_THERMO_LANGEVIN) {
    float zf[3];
    normal3(p.seed, (uint32_t)n, (uint32_t)p.step, 0u, zf);
    const double amp = c2[n];
#pragma unroll
    for (int x = 0; x < 3; ++x) vv[x] = p.c1 * vv[x] + amp * (double)zf[x];
  }
  const double im = invm[n];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    vv[x] += 0.5 * (-gg[x] * im) * p.dt;
    const double un = uu[x] + p.dt * vv[x];
    u[x * t.N + n] = un;
    disp[x * t.N + n] = (T)un;
    v[x * t.N + n] = vv[x];
    pos[3 * n + x] = (la * box[x] + lb * box[3 + x] + lc * box[6 + x]) + un;
  }
}

// Host-buffer step, output: vel in AoS (the arithmetic of k_soa_to_aos), into the device
// buffer copied back to the caller (positions come from k_md_host_begin).
__global__ void k_md_host_end(Topo t, const double* __restrict__ v, double* __restrict__ vel) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
#pragma unroll
  for (int x = 0; x < 3; ++x) vel[3 * n + x] = v[x * t.N + n];
}

}  // namespace

// ------------------------------------------------------------------ host side

namespace mm {

static thread_local std::string g_last_error;

void set_error(const std::string& s) { g_last_error = s; }
const char* last_error() { return g_last_error.c_str(); }

static void topo_of(const mm_handle* h, Topo& t) {
  t.N = h->N;
  t.M = h->M;
  t.structured = h->structured;
  t.nx = h->nn[0];
  t.ny = h->nn[1];
  t.nz = h->nn[2];
  t.div_nyz = make_fastdiv((uint32_t)(t.ny * t.nz > 0 ? t.ny * t.nz : 1));
  t.div_nz = make_fastdiv((uint32_t)(t.nz > 0 ? t.nz : 1));
  t.cell_nodes = h->d_cell_nodes;
  t.node_cells = h->d_node_cells;
  t.node_lat = h->d_node_lat;
  t.cell_type = h->d_cell_type;
}

static size_t cell_smem(const mm_handle* h) {
  const size_t esz = h->prec == MM_PREC_FP32 ? sizeof(float) : sizeof(double);
  const size_t tp = (h->prec == MM_PREC_FP32 ? sizeof(TypeParams<float>) : sizeof(TypeParams<double>)) * h->ntypes;
  if (h->cell_kernel == 1) return ((tp + 15) / 16) * 16 + sizeof(double) * kCellPart * (kCell1Threads / 32);
  if (h->model == MM_MODEL_NANOCELL) return ((tp + 15) / 16) * 16 + 2 * esz * kTileElems;
  return ((tp + 15) / 16) * 16 + sizeof(double) * kCellPart * (kCellThreads / 32);
}

template <typename K>
static int occupancy_of(K kern, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem) != cudaSuccess || nb < 1) {
    (void)cudaGetLastError();
    nb = 1;
  }
  return nb;
}

template <typename T, bool STRUCT>
static int cell8_occupancy(const mm_handle* h) {
  if (h->cell_kernel == 1) {
    if (h->model == MM_MODEL_ORIGINAL)
      return h->simple ? occupancy_of(k_cells1<T, 0, STRUCT, true>, kCell1Threads, cell_smem(h))
                       : occupancy_of(k_cells1<T, 0, STRUCT, false>, kCell1Threads, cell_smem(h));
    return h->simple ? occupancy_of(k_cells1<T, 1, STRUCT, true>, kCell1Threads, cell_smem(h))
                     : occupancy_of(k_cells1<T, 1, STRUCT, false>, kCell1Threads, cell_smem(h));
  }
  return h->simple ? occupancy_of(k_cells8<T, STRUCT, true>, kCell8Threads, cell_smem(h))
                   : occupancy_of(k_cells8<T, STRUCT, false>, kCell8Threads, cell_smem(h));
}

template <typename T, int MODEL, bool STRUCT>
static void launch_cells_t(mm_handle* h, cudaStream_t st, double* ecell) {
  Topo t;
  topo_of(h, t);
  const int nblk = cell_grid(h);
  if (h->cell_kernel == 1) {
    if (h->simple)
      launch_pdl(k_cells1<T, MODEL, STRUCT, true>, nblk, kCell1Threads, cell_smem(h), st, t,
                 (const TypeTable*)h->d_tt, h->ntypes, (const double*)h->d_box, (const T*)h->d_disp, (T*)h->d_G,
                 ecell, h->d_cpart);
    else
      launch_pdl(k_cells1<T, MODEL, STRUCT, false>, nblk, kCell1Threads, cell_smem(h), st, t,
                 (const TypeTable*)h->d_tt, h->ntypes, (const double*)h->d_box, (const T*)h->d_disp, (T*)h->d_G,
                 ecell, h->d_cpart);
  } else if constexpr (MODEL == 1) {
    if (h->simple)
      launch_pdl(k_cells8<T, STRUCT, true>, nblk, kCell8Threads, cell_smem(h), st, t, (const TypeTable*)h->d_tt,
                 h->ntypes, (const double*)h->d_box, (const T*)h->d_disp, (T*)h->d_G, ecell, h->d_cpart);
    else
      launch_pdl(k_cells8<T, STRUCT, false>, nblk, kCell8Threads, cell_smem(h), st, t, (const TypeTable*)h->d_tt,
                 h->ntypes, (const double*)h->d_box, (const T*)h->d_disp, (T*)h->d_G, ecell, h->d_cpart);
  } else {
    k_cells<T, MODEL, STRUCT><<<nblk, kCellThreads, cell_smem(h), st>>>(
        t, h->d_tt, h->ntypes, h->d_box, (const T*)h->d_disp, (T*)h->d_G, ecell, h->d_cpart);
  }
}

template <typename T>
static void launch_cells_p(mm_handle* h, cudaStream_t st, double* ecell) {
  if (h->model == MM_MODEL_ORIGINAL) {
    if (h->structured) launch_cells_t<T, 0, true>(h, st, ecell);
    else launch_cells_t<T, 0, false>(h, st, ecell);
  } else {
    if (h->structured) launch_cells_t<T, 1, true>(h, st, ecell);
    else launch_cells_t<T, 1, false>(h, st, ecell);
  }
}

void launch_cells(mm_handle* h, cudaStream_t st, double* ecell) {
  if (h->prec == MM_PREC_FP32) launch_cells_p<float>(h, st, ecell);
  else launch_cells_p<double>(h, st, ecell);
}

// Resident blocks per SM at most: eight-lane kernel (256 threads) 4, one-thread kernel
// (128 threads) 16.
constexpr int kCell8MaxPerSM = 4, kCell1MaxPerSM = 16;

int cell_blocks(const mm_handle* h) {
  // one-thread kernel: at most kCell1MaxPerSM resident blocks per SM, each owning a run of
  // 32-cell chunks
  const int sms = h->num_sms > 0 ? h->num_sms : 152;
  const int g1 = std::min((h->M + kCell1Threads - 1) / kCell1Threads, sms * kCell1MaxPerSM);
  if (h->model == MM_MODEL_NANOCELL)  // or the eight-lane kernel: grid-stride over groups of cells
    return std::max(g1, std::min((h->M + kCell8Cells - 1) / kCell8Cells, sms * kCell8MaxPerSM));
  return std::max(g1, (h->M + kCellThreads - 1) / kCellThreads);  // or one block per kCellThreads cells
}
int node_blocks(const mm_handle* h) { return (h->N + kNodeThreads - 1) / kNodeThreads; }

// The one-thread cell kernel (each block a run of 32-cell chunks) and the eight-lane kernel
// (grid-stride over groups of cells) run exactly as many blocks as fit on the GPU at once
// (so no partial second wave), at most 16 and 4 per SM.
int cell_grid(mm_handle* h) {
  if (h->model != MM_MODEL_NANOCELL && h->cell_kernel != 1) return (h->M + kCellThreads - 1) / kCellThreads;
  int& occ = h->cell_occ[h->simple ? 1 : 0];
  if (occ == 0) {
    if (h->prec == MM_PREC_FP32) occ = h->structured ? cell8_occupancy<float, true>(h) : cell8_occupancy<float, false>(h);
    else occ = h->structured ? cell8_occupancy<double, true>(h) : cell8_occupancy<double, false>(h);
  }
  const int sms = h->num_sms > 0 ? h->num_sms : 152;
  if (h->cell_kernel == 1)
    return std::min((h->M + kCell1Threads - 1) / kCell1Threads, sms * std::min(occ, kCell1MaxPerSM));
  const int groups = (h->M + kCell8Cells - 1) / kCell8Cells;
  const int cap = sms * (occ < kCell8MaxPerSM ? occ : kCell8MaxPerSM);
  return groups < cap ? groups : cap;
}

void launch_pos_to_state(mm_handle* h, const double* pos, cudaStream_t st) {
  Topo t;
  topo_of(h, t);
  const int nb = node_blocks(h);
  if (h->prec == MM_PREC_FP32)
    k_pos_to_state<float><<<nb, kNodeThreads, 0, st>>>(t, pos, h->d_box, h->d_u, (float*)h->d_disp);
  else
    k_pos_to_state<double><<<nb, kNodeThreads, 0, st>>>(t, pos, h->d_box, h->d_u, (double*)h->d_disp);
}

void launch_state_to_pos(mm_handle* h, double* pos, cudaStream_t st) {
  Topo t;
  topo_of(h, t);
  k_state_to_pos<<<node_blocks(h), kNodeThreads, 0, st>>>(t, h->d_u, h->d_box, pos);
}

void launch_gather(mm_handle* h, double* gpos, int* flag, cudaStream_t st) {
  Topo t;
  topo_of(h, t);
  const int nb = node_blocks(h);
  if (h->prec == MM_PREC_FP32) {
    if (h->structured) k_gather<float, true><<<nb, kNodeThreads, 0, st>>>(t, (const float*)h->d_G, gpos, flag);
    else k_gather<float, false><<<nb, kNodeThreads, 0, st>>>(t, (const float*)h->d_G, gpos, flag);
  } else {
    if (h->structured) k_gather<double, true><<<nb, kNodeThreads, 0, st>>>(t, (const double*)h->d_G, gpos, flag);
    else k_gather<double, false><<<nb, kNodeThreads, 0, st>>>(t, (const double*)h->d_G, gpos, flag);
  }
}

void launch_finalize(mm_handle* h, double* energy, double* vtens, int* flag, cudaStream_t st) {
  if (h->prec == MM_PREC_FP32) k_finalize<true><<<1, 256, 0, st>>>(h->d_cpart, cell_grid(h), energy, vtens, flag);
  else k_finalize<false><<<1, 256, 0, st>>>(h->d_cpart, cell_grid(h), energy, vtens, flag);
}

__global__ void k_selftest_convert(const double* din, float* dout, const float* fin, double* fout, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dout[i] = d2f_rn(din[i]);
  fout[i] = f2d(fin[i]);
}
void launch_selftest_convert(const double* din, float* dout, const float* fin, double* fout, int n, cudaStream_t st) {
  if (n > 0) k_selftest_convert<<<(n + 255) / 256, 256, 0, st>>>(din, dout, fin, fout, n);
}

void launch_aos_to_soa(int N, const double* a, double* s, cudaStream_t st) {
  k_aos_to_soa<<<(N + kNodeThreads - 1) / kNodeThreads, kNodeThreads, 0, st>>>(N, a, s);
}
void launch_soa_to_aos(int N, const double* s, double* a, cudaStream_t st) {
  k_soa_to_aos<<<(N + kNodeThreads - 1) / kNodeThreads, kNodeThreads, 0, st>>>(N, s, a);
}

template <typename T, bool STRUCT, int THERMO>
static void launch_md_nodes_t(mm_handle* h, const MDArgs& a, const double* noise, double* record, double* gpos_out,
                              cudaStream_t st) {
  Topo t;
  topo_of(h, t);
  const size_t smem = sizeof(T) == 4 ? kMDStageBytes : 0;
  int& occ = h->node_occ[THERMO == MM_THERMO_LANGEVIN ? 1 : 0];
  if (occ == 0) {
    if (smem) cudaFuncSetAttribute(k_md_nodes<T, STRUCT, THERMO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    occ = occupancy_of(k_md_nodes<T, STRUCT, THERMO>, kMDThreads, smem);
  }
  launch_pdl(k_md_nodes<T, STRUCT, THERMO>, node_grid(h, THERMO) + 1, kMDThreads, smem, st, t, a, (const T*)h->d_G,
             h->d_u, h->d_v, (T*)h->d_disp, (const double*)h->d_mass, (const double*)h->d_invm,
             (const double*)h->d_c2, noise, h->d_npart, (const double*)h->d_cpart, cell_grid(h), h->d_ticket,
             h->d_carry, record, gpos_out, (const float4*)h->d_nodef);
}

// Node-update grid: at most one block per kMDThreads nodes, and one block fewer than fit
// on the GPU at once: the kernel adds one block for the cell partials, which must be
// resident together with the node blocks (else it would start only when a node block
// retires, and the step would end one reduction later).
int node_grid(mm_handle* h, int thermo) {
  const int occ = h->node_occ[thermo == MM_THERMO_LANGEVIN ? 1 : 0];
  const int nb = (h->N + kMDThreads - 1) / kMDThreads;
  if (occ <= 0) return nb;
  int cap = (h->num_sms > 0 ? h->num_sms : 152) * occ - 1;
  if (cap < 1) cap = 1;
  return nb < cap ? nb : cap;
}

template <typename T>
static void launch_md_nodes_p(mm_handle* h, const MDArgs& a, int thermo, const double* noise, double* record,
                              double* gpos_out, cudaStream_t st) {
  if (thermo == MM_THERMO_LANGEVIN) {
    if (h->structured) launch_md_nodes_t<T, true, MM_THERMO_LANGEVIN>(h, a, noise, record, gpos_out, st);
    else launch_md_nodes_t<T, false, MM_THERMO_LANGEVIN>(h, a, noise, record, gpos_out, st);
  } else {
    if (h->structured) launch_md_nodes_t<T, true, MM_THERMO_NONE>(h, a, noise, record, gpos_out, st);
    else launch_md_nodes_t<T, false, MM_THERMO_NONE>(h, a, noise, record, gpos_out, st);
  }
}

void launch_md_nodes(mm_handle* h, double dt, double c1, uint64_t seed, int64_t step, int64_t noise_step0, int finish,
                     int start, int thermo, const double* noise, double* record, double* gpos_out, cudaStream_t st) {
  MDArgs a;
  a.dt = dt;
  a.c1 = c1;
  a.seed = seed;
  a.step = step;
  a.noise_step0 = noise_step0;
  a.finish = finish;
  a.start = start;
  const bool lang = thermo == MM_THERMO_LANGEVIN;
  a.cv = lang ? ((finish && start) ? c1 * c1 : c1) : 1.0;
  a.hf = (float)(0.5 * dt);
  a.c1f = lang ? (float)c1 : 1.0f;
  if (h->prec == MM_PREC_FP32) launch_md_nodes_p<float>(h, a, thermo, noise, record, gpos_out, st);
  else launch_md_nodes_p<double>(h, a, thermo, noise, record, gpos_out, st);
}

void launch_md_host_begin(mm_handle* h, double dt, double c1, uint64_t seed, int64_t step, int thermo,
                          double* pos, const double* vel, const double* gpos, cudaStream_t st) {
  Topo t;
  topo_of(h, t);
  MDArgs a;
  a.dt = dt;
  a.c1 = c1;
  a.seed = seed;
  a.step = step;
  a.noise_step0 = step;
  a.finish = 0;
  a.start = 1;
  const bool lang = thermo == MM_THERMO_LANGEVIN;
  a.hf = (float)(0.5 * dt);
  a.c1f = lang ? (float)c1 : 1.0f;
  a.cv = lang ? c1 : 1.0;
  const int nb = node_blocks(h);
  const float4* nf = (const float4*)h->d_nodef;
  if (h->prec == MM_PREC_FP32) {
    if (lang)
      k_md_host_begin<float, MM_THERMO_LANGEVIN><<<nb, kNodeThreads, 0, st>>>(t, a, pos, vel, gpos, h->d_box, h->d_u, h->d_v, (float*)h->d_disp, h->d_invm, h->d_c2, nf);
    else
      k_md_host_begin<float, MM_THERMO_NONE><<<nb, kNodeThreads, 0, st>>>(t, a, pos, vel, gpos, h->d_box, h->d_u, h->d_v, (float*)h->d_disp, h->d_invm, h->d_c2, nf);
  } else {
    if (lang)
      k_md_host_begin<double, MM_THERMO_LANGEVIN><<<nb, kNodeThreads, 0, st>>>(t, a, pos, vel, gpos, h->d_box, h->d_u, h->d_v, (double*)h->d_disp, h->d_invm, h->d_c2, nf);
    else
      k_md_host_begin<double, MM_THERMO_NONE><<<nb, kNodeThreads, 0, st>>>(t, a, pos, vel, gpos, h->d_box, h->d_u, h->d_v, (double*)h->d_disp, h->d_invm, h->d_c2, nf);
  }
}

void launch_md_host_end(mm_handle* h, double* vel, cudaStream_t st) {
  Topo t;
  topo_of(h, t);
  k_md_host_end<<<node_blocks(h), kNodeThreads, 0, st>>>(t, h->d_v, vel);
}

}  // namespace mm
