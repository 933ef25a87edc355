// Batched systems: hundreds of independent periodic lattices of uneven size
// (defect configurations, strain-scan points, replicas) in one persistent launch.
//
// Each CTA owns a list of whole systems (longest-first, balanced on the host) and
// runs every step of a system before moving on, so a step needs only CTA-wide
// barriers: force evaluation (cells, then the per-node gather), kicks, drifts,
// Langevin / Nose-Hoover-chain thermostats and the MTK barostat. The barostat's
// 3x3 algebra (matrix exponentials by scaling and squaring of the Taylor series) runs
// on one thread in FP64. The step order is that of the reference's Verlet step with
// its hooks (micmec/sampling/verlet.py:140-166; TBCombination, npt.py:99-148;
// MTKBarostat.baro, npt.py:653-736; NHChain, nvt.py:410-458; Langevin, nvt.py:196-218).
// A second persistent kernel relaxes every system with nonlinear conjugate
// gradients (Polak-Ribiere+, secant line search).
//
// This header holds the device code; mm_batch_md_*.cu (one per cell precision and
// model) and mm_batch_relax.cu instantiate the two kernels (separate translation units
// compile in parallel), mm_batch_md.cu dispatches, and mm_batch.cu holds the host API.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/micmec_gb300.h"
#include "mm_device.cuh"
#include "mm_handle.h"
#include "mm_control.cuh"

namespace mmb {

using namespace mm;
using namespace mmc;

struct BSys {
  int nx, ny, nz, M;
  long long off;  // first node / cell in the concatenated arrays
  FastDiv div_nyz, div_nz;  // cell / node index -> grid coordinates
};

// grid coordinates (i, j, k) of cell or node index n of system s
__device__ __forceinline__ void grid_coords(const BSys& s, int n, int& i, int& j, int& k) {
  i = fdiv(n, s.div_nyz);
  const int r = n - i * (s.ny * s.nz);
  j = fdiv(r, s.div_nz);
  k = r - j * s.nz;
}

struct BArgs {
  const BSys* sys;
  int nsys;
  const int* work;       // system indices, grouped by CTA
  const int* work_off;   // [nCTA + 1]
  const TypeTable* tt;
  int ntypes;
  const uint8_t* ctype;
  const double* mass;
  const double* invm;
  double* u;             // [3][Ntot]
  double* v;             // [3][Ntot]
  void* disp;            // [3][Ntot] cell precision
  void* G;               // per system 24*M at 24*off
  double* gpos;          // [3][Ntot]
  double* ctl;           // [nsys][C_LEN]
  double* cgd;           // [3][Ntot] CG direction
  double* cgu;           // [3][Ntot] CG saved positions
  double* cgg;           // [3][Ntot] CG previous gradient
  long long Ntot;
};

// Launch configuration of the persistent kernels.
struct BatchLaunch {
  BArgs a;
  int bt;      // CTA size (128 or 256)
  int nctas;   // persistent CTAs
  int prec, model, simple;
};
void launch_md(const BatchLaunch& L, const BMD& p, cudaStream_t st);                     // mm_batch_md.cu
void launch_relax(const BatchLaunch& L, int max_iter, double gtol, cudaStream_t st);    // mm_batch_relax.cu
// Relaxation of positions and domain (k_batch_relax_cell).
struct CellRelax {
  int max_iter;
  double gtol, stol, press;
  int full;  // 1: FullCellDOF, 0: StrainCellDOF
};
void launch_relax_cell(const BatchLaunch& L, const CellRelax& r, cudaStream_t st);       // mm_batch_relax_cell.cu
// MD launch of one (cell precision, model) pair: each is instantiated in its own
// translation unit (mm_batch_md_<precision><model>.cu) so that they compile in parallel.
template <typename T, int MODEL>
void launch_md_t(const BatchLaunch& L, const BMD& p, cudaStream_t st);
template <> void launch_md_t<float, 0>(const BatchLaunch&, const BMD&, cudaStream_t);
template <> void launch_md_t<float, 1>(const BatchLaunch&, const BMD&, cudaStream_t);
template <> void launch_md_t<float, 2>(const BatchLaunch&, const BMD&, cudaStream_t);
template <> void launch_md_t<double, 0>(const BatchLaunch&, const BMD&, cudaStream_t);
template <> void launch_md_t<double, 1>(const BatchLaunch&, const BMD&, cudaStream_t);

namespace {


// systems with at least this many cells per thread evaluate them one thread per cell
// (cell1_eval); smaller ones use eight lanes per cell (cell8_eval)
#ifndef MM_BATCH_CELL1_MIN
#define MM_BATCH_CELL1_MIN 1
#endif
constexpr int kCell1MinCellsPerThread = MM_BATCH_CELL1_MIN;
constexpr int kMaxBT = 256;  // largest CTA size; the kernels are instantiated for 128 and 256
constexpr int kMaxNW = kMaxBT / 32;

// ------------------------------------------------------------ CTA-wide building blocks

template <typename T>
struct Shared {
  TypeParams<T> tp[MM_MAX_TYPES];
  T L[9];
  double red[20 * kMaxNW];
  double ctl[C_LEN];
  double mat[9];
  double scal[4];
};

template <typename T>
__device__ void load_tables(Shared<T>& sh, const TypeTable* tt, int ntypes, const double* L) {
  fill_params_block<T>(sh.tp, tt, ntypes, L);
  if (threadIdx.x < 9) sh.L[threadIdx.x] = (T)L[threadIdx.x];
}

// new lattice matrix: refresh B = L - h0 and L in the cell precision
template <typename T>
__device__ void refresh_B(Shared<T>& sh, const TypeTable* tt, int ntypes, const double* L) {
  for (int idx = threadIdx.x; idx < ntypes * MM_MAX_STATES * 9; idx += blockDim.x) {
    const int i = idx % 9, s = (idx / 9) % MM_MAX_STATES, ty = idx / (9 * MM_MAX_STATES);
    sh.tp[ty].s[s].B[i] = (T)(L[i] - tt[ty].s[s].h0[i]);
  }
  if (threadIdx.x < 9) sh.L[threadIdx.x] = (T)L[threadIdx.x];
}

template <int NV>
__device__ void cta_sum(double (&v)[NV], double* red) {
  block_sum<NV>(v, red);
}

__device__ __forceinline__ int wrap_node(const BSys& s, int i, int j, int k) {
  i = (i >= s.nx) ? i - s.nx : i;
  j = (j >= s.ny) ? j - s.ny : j;
  k = (k >= s.nz) ? k - s.nz : k;
  return (i * s.ny + j) * s.nz + k;
}
__device__ __forceinline__ int wrap_cell(const BSys& s, int i, int j, int k) {
  i = (i < 0) ? i + s.nx : i;
  j = (j < 0) ? j + s.ny : j;
  k = (k < 0) ? k + s.nz : k;
  return (i * s.ny + j) * s.nz + k;
}

__device__ __forceinline__ double to_double(float x) { return f2d(x); }
__device__ __forceinline__ double to_double(double x) { return x; }
template <typename T>
__device__ __forceinline__ T from_double(double x) {
  if constexpr (sizeof(T) == 4) return d2f_rn(x);
  else return x;
}

// Totals of block_sum_f2_pairs (held by thread 0) in FP64, lane l < NV of warp 0 forming
// total l (one FP64 add for all of them; the conversions are exact integer-pipe ones).
// Called by all 32 lanes of warp 0.
template <int NV>
__device__ __forceinline__ double f2_total_of_lane(const F2 (&v)[NV]) {
  const int l = threadIdx.x & 31;
  float hi = 0.0f, lo = 0.0f;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const float h = __shfl_sync(0xffffffffu, v[i].hi, 0), w = __shfl_sync(0xffffffffu, v[i].lo, 0);
    if (l == i) {
      hi = h;
      lo = w;
    }
  }
  return f2d(hi) + f2d(lo);
}

// Energy, virial (into sh.ctl) and node gradient (a.gpos) of system sy. Not inlined: a step
// evaluates the forces at up to four places (MTK half steps, the Verlet step, the Berendsen
// barostat), and one copy of this code keeps the kernel smaller in the instruction cache.
#ifndef MM_FORCES_INLINE
#define MM_FORCES_INLINE __noinline__
#endif
template <typename T, int MODEL>
__device__ MM_FORCES_INLINE void forces(const BArgs& a, Shared<T>& sh, const BSys& sy) {
  const T* disp = (const T*)a.disp;
  T* G = (T*)a.G + 24 * sy.off;
  const long long N3 = a.Ntot;
  const int M = sy.M;
  double acc[10];
  for (int i = 0; i < 10; ++i) acc[i] = 0.0;
  // FP32 cells: energy and virial terms summed in compensated FP32 (the FP64 pipe is
  // narrow), converted once per system in the CTA sum
  F2 facc[10];
  for (int i = 0; i < 10; ++i) facc[i] = F2{0.0f, 0.0f};
  if (MODEL == 0 || M >= kCell1MinCellsPerThread * (int)blockDim.x) {
    // one thread per cell: the averaged-matrix model always, the eight-corner-matrix model
    // for systems with at least a cell per thread; a thread's few cells are summed in the
    // cell precision, then join the CTA sums below
    T vs[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) vs[q] = T(0);
    for (int cell = threadIdx.x; cell < M; cell += blockDim.x) {
      int i, j, k;
      grid_coords(sy, cell, i, j, k);
      T du[8][3];
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int node = wrap_node(sy, i + (b & 1), j + ((b >> 1) & 1), k + (b >> 2));
#pragma unroll
        for (int x = 0; x < 3; ++x) du[b][x] = disp[x * N3 + sy.off + node];
      }
      T g[8][3];
      const T E = cell1_eval<T, MODEL == 2, (MODEL == 0 ? 0 : 1)>(du, sh.tp[a.ctype[sy.off + cell]], g);
#pragma unroll
      for (int kc = 0; kc < 8; ++kc)
#pragma unroll
        for (int x = 0; x < 3; ++x) G[(kc * 3 + x) * (size_t)M + cell] = g[corner_to_bits(kc)][x];
      vs[0] += E;
#pragma unroll
      for (int b = 1; b < 8; ++b)
#pragma unroll
        for (int y = 0; y < 3; ++y) {
          T r = du[b][y] - du[0][y];
          if (b & 1) r += sh.L[0 * 3 + y];
          if (b & 2) r += sh.L[1 * 3 + y];
          if (b & 4) r += sh.L[2 * 3 + y];
#pragma unroll
          for (int x = 0; x < 3; ++x) vs[1 + x * 3 + y] += g[b][x] * r;
        }
    }
#pragma unroll
    for (int q = 0; q < 10; ++q) {
      if constexpr (sizeof(T) == 4) facc[q] = F2{vs[q], 0.0f};
      else acc[q] = (double)vs[q];
    }
  } else {  // eight lanes per cell (small systems); MODEL 2: diagonal h0, cubic stress maps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, av = threadIdx.x & 7;
    const int ngroups = (M + 3) / 4;
    const int nw = blockDim.x >> 5;
    for (int grp = warp; grp < ngroups; grp += nw) {
      const int cell = grp * 4 + (lane >> 3);
      const bool valid = cell < M;
      T du[3] = {T(0), T(0), T(0)};
      int ty = 0;
      if (valid) {
        int i, j, k;
        grid_coords(sy, cell, i, j, k);
        const int node = wrap_node(sy, i + (av & 1), j + ((av >> 1) & 1), k + (av >> 2));
        for (int x = 0; x < 3; ++x) du[x] = disp[x * N3 + sy.off + node];
        ty = a.ctype[sy.off + cell];
      }
      T g[3];
      const T E = cell8_eval<T, MODEL == 2>(du, av, sh.tp[ty], valid, g);
      T d0[3];
      for (int y = 0; y < 3; ++y) d0[y] = __shfl_sync(0xffffffffu, du[y], lane & ~7);  // all lanes
      if (valid) {
        const int corner = bits_to_corner(av);
        for (int x = 0; x < 3; ++x) G[(corner * 3 + x) * (size_t)M + cell] = g[x];
        T rel[3];
        for (int y = 0; y < 3; ++y) {
          T r = du[y] - d0[y];
          if (av & 1) r += sh.L[0 * 3 + y];
          if (av & 2) r += sh.L[1 * 3 + y];
          if (av & 4) r += sh.L[2 * 3 + y];
          rel[y] = r;
        }
        if constexpr (sizeof(T) == 4) {
          if (av == 0) facc[0] = f2_add(facc[0], F2{E, 0.0f});
          for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) facc[1 + x * 3 + y] = f2_add(facc[1 + x * 3 + y], F2{g[x] * rel[y], 0.0f});
        } else {
          if (av == 0) acc[0] += (double)E;
          for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) acc[1 + x * 3 + y] += (double)(g[x] * rel[y]);
        }
      }
    }
  }
  // (the CTA sum's barrier also orders every corner-gradient write before the gather)
  if constexpr (sizeof(T) == 4) {
    block_sum_f2_pairs<10>(facc, sh.red);
    if (threadIdx.x < 32) {
      const double t = f2_total_of_lane<10>(facc);
      if (threadIdx.x < 10) sh.ctl[threadIdx.x == 0 ? C_EPOT : C_VT + threadIdx.x - 1] = t;
    }
  } else {
    cta_sum<10>(acc, sh.red);
    if (threadIdx.x == 0) {
      sh.ctl[C_EPOT] = acc[0];
      for (int i = 0; i < 9; ++i) sh.ctl[C_VT + i] = acc[1 + i];
    }
  }
  for (int n = threadIdx.x; n < M; n += blockDim.x) {
    int i, j, k;
    grid_coords(sy, n, i, j, k);
    T s[3] = {T(0), T(0), T(0)};
    for (int kc = 0; kc < 8; ++kc) {
      const int b = corner_to_bits(kc);
      const int cell = wrap_cell(sy, i - (b & 1), j - ((b >> 1) & 1), k - (b >> 2));
      for (int x = 0; x < 3; ++x) s[x] += G[(kc * 3 + x) * (size_t)M + cell];
    }
    for (int x = 0; x < 3; ++x) a.gpos[x * N3 + sy.off + n] = to_double(s[x]);
  }
  __syncthreads();
}

// Per-node velocity updates that a kinetic-energy sum follows directly (fused into one
// pass over the system's nodes; the thread that updates a node also sums it):
enum { KV_NONE = 0, KV_SCALE = 1, KV_KICK = 2 };

// v <- v R (row vector times a 3x3 matrix). FP32 cells: R = I + (R - I) with R - I small
// (the exponential of a barostat half step); the increment v (R - I) is formed in FP32
// and added to the FP64 state.
template <typename T>
__device__ __forceinline__ void rows_times(double& x, double& y, double& z, const double* R) {
  if constexpr (sizeof(T) == 4) {
    const float xf = d2f_rn(x), yf = d2f_rn(y), zf = d2f_rn(z);
    const float d0 = (float)(R[0] - 1.0), d4 = (float)(R[4] - 1.0), d8 = (float)(R[8] - 1.0);
    const double nx = x + f2d(xf * d0 + yf * (float)R[3] + zf * (float)R[6]);
    const double ny = y + f2d(xf * (float)R[1] + yf * d4 + zf * (float)R[7]);
    const double nz = z + f2d(xf * (float)R[2] + yf * (float)R[5] + zf * d8);
    x = nx;
    y = ny;
    z = nz;
  } else {
    const double nx = x * R[0] + y * R[3] + z * R[6];
    const double ny = x * R[1] + y * R[4] + z * R[7];
    const double nz = x * R[2] + y * R[5] + z * R[8];
    x = nx;
    y = ny;
    z = nz;
  }
}

// Velocity-Verlet half kick v += -g/m dt/2 of one component. FP32 cells: the increment
// in FP32, added to the FP64 state.
template <typename T>
__device__ __forceinline__ double half_kick(double v, double g, double im, double dt) {
  if constexpr (sizeof(T) == 4) return v + f2d((float)(0.5 * dt) * (-d2f_rn(g) * d2f_rn(im)));
  else return v + 0.5 * (-g * im) * dt;
}

// Optional velocity update (op, see KV_*), then ekin and the kinetic tensor into ctl.
// FP32 cells: from an FP32 copy of the velocities, summed in compensated FP32
// (observables at the precision of the forces).
template <typename T>
__device__ void kinetic(const BArgs& a, double* ctl, double* red, const BSys& sy, int op = KV_NONE,
                        const double* R = nullptr, double dt = 0.0) {
  double acc[7];
  const long long N3 = a.Ntot;
  typedef typename std::conditional<sizeof(T) == 4, F2, double>::type Acc;
  Acc f[6];
  for (int i = 0; i < 6; ++i) f[i] = Acc{};
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    double w0 = a.v[g], w1 = a.v[N3 + g], w2 = a.v[2 * N3 + g];
    if (op == KV_SCALE) {
      rows_times<T>(w0, w1, w2, R);
    } else if (op == KV_KICK) {
      const double im = a.invm[g];
      w0 = half_kick<T>(w0, a.gpos[g], im, dt);
      w1 = half_kick<T>(w1, a.gpos[N3 + g], im, dt);
      w2 = half_kick<T>(w2, a.gpos[2 * N3 + g], im, dt);
    }
    if (op != KV_NONE) {
      a.v[g] = w0;
      a.v[N3 + g] = w1;
      a.v[2 * N3 + g] = w2;
    }
    if constexpr (sizeof(T) == 4) {
      const float m = d2f_rn(a.mass[g]), v0 = d2f_rn(w0), v1 = d2f_rn(w1), v2 = d2f_rn(w2);
      f[0] = f2_add(f[0], F2{m * v0 * v0, 0.0f});
      f[1] = f2_add(f[1], F2{m * v1 * v1, 0.0f});
      f[2] = f2_add(f[2], F2{m * v2 * v2, 0.0f});
      f[3] = f2_add(f[3], F2{m * v1 * v2, 0.0f});
      f[4] = f2_add(f[4], F2{m * v0 * v2, 0.0f});
      f[5] = f2_add(f[5], F2{m * v0 * v1, 0.0f});
    } else {
      const double m = a.mass[g];
      f[0] += m * w0 * w0;
      f[1] += m * w1 * w1;
      f[2] += m * w2 * w2;
      f[3] += m * w1 * w2;
      f[4] += m * w0 * w2;
      f[5] += m * w0 * w1;
    }
  }
  if constexpr (sizeof(T) == 4) {
    block_sum_f2_pairs<6>(f, red);
    if (threadIdx.x < 32) {
      // lane l < 6 converts total l; lane l < 9 writes kinetic-tensor entry l
      // (xx yy zz yz xz xy -> row-major 3x3: source totals 0 5 4 5 1 3 4 3 2)
      const int l = threadIdx.x;
      const double t = f2_total_of_lane<6>(f);
      const int src = (int)((0x234315450ull >> (4 * (l < 9 ? l : 0))) & 15u);
      const double kv = __shfl_sync(0xffffffffu, t, src);
      const double ek = 0.5 * (__shfl_sync(0xffffffffu, t, 0) + __shfl_sync(0xffffffffu, t, 1) +
                               __shfl_sync(0xffffffffu, t, 2));
      if (l < 9) ctl[C_KT + l] = kv;
      if (l == 0) ctl[C_EKIN] = ek;
    }
  } else {
    double t6[6];
    for (int i = 0; i < 6; ++i) t6[i] = f[i];
    block_sum<6>(t6, red);
    if (threadIdx.x == 0) {
      acc[0] = 0.5 * (t6[0] + t6[1] + t6[2]);
      for (int i = 0; i < 6; ++i) acc[1 + i] = t6[i];
      ctl[C_EKIN] = acc[0];
      const double k[9] = {acc[1], acc[6], acc[5], acc[6], acc[2], acc[4], acc[5], acc[4], acc[3]};
      for (int i = 0; i < 9; ++i) ctl[C_KT + i] = k[i];
    }
  }
  __syncthreads();
}

// Positions: u <- u R (barostat scaling), or the first half kick and drift
// (v += -g/m dt/2, u += dt v); then the cell-precision copy of u, in one pass.
// FP32 cells: increments formed in FP32 and added to the FP64 state.
template <typename T>
__device__ void positions(const BArgs& a, const BSys& sy, const double* R, double dt) {
  T* disp = (T*)a.disp;
  const long long N3 = a.Ntot;
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    double x = a.u[g], y = a.u[N3 + g], z = a.u[2 * N3 + g];
    if (R) {
      rows_times<T>(x, y, z, R);
    } else {
      const double im = a.invm[g];
      double* uu[3] = {&x, &y, &z};
      for (int c = 0; c < 3; ++c) {
        const double vv = half_kick<T>(a.v[c * N3 + g], a.gpos[c * N3 + g], im, dt);
        a.v[c * N3 + g] = vv;
        if constexpr (sizeof(T) == 4) *uu[c] += f2d((float)dt * d2f_rn(vv));
        else *uu[c] += dt * vv;
      }
    }
    a.u[g] = x;
    a.u[N3 + g] = y;
    a.u[2 * N3 + g] = z;
    disp[g] = from_double<T>(x);
    disp[N3 + g] = from_double<T>(y);
    disp[2 * N3 + g] = from_double<T>(z);
  }
}

template <typename T>
__device__ void write_disp(const BArgs& a, const BSys& sy) {
  T* disp = (T*)a.disp;
  const long long N3 = a.Ntot;
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
    for (int x = 0; x < 3; ++x) disp[x * N3 + sy.off + n] = from_double<T>(a.u[x * N3 + sy.off + n]);
}

__device__ __forceinline__ void langevin_noise(const BMD& p, const BArgs& a, long long g, long long step,
                                               unsigned call, double (&z)[3]) {
  if (p.noise) {
    const size_t base = ((size_t)(step - p.step0 - 1) * 2 + call) * (size_t)a.Ntot * 3;
    for (int x = 0; x < 3; ++x) z[x] = p.noise[base + 3 * g + x];
  } else {
    float zf[3];
    normal3(p.seed, (uint32_t)g, (uint32_t)step, call, zf);
    for (int x = 0; x < 3; ++x) z[x] = zf[x];
  }
}

// thermostat pre/post (THERMO: TH_LANGEVIN, TH_NHC; TH_BERENDSEN and TH_CSVR act in pre only)
template <typename T, int THERMO>
__device__ void thermostat(const BArgs& a, Shared<T>& sh, const BSys& sy, const BMD& p, long long step,
                           unsigned call, bool g1, double kT, unsigned sys) {
  double* c = sh.ctl;
  double* red = sh.red;
  const long long N3 = a.Ntot;
  if (THERMO == TH_LANGEVIN) {
    const double c1 = exp(-p.dt / p.timecon / 2);
    const double ekin0 = c[C_EKIN];
    __syncthreads();
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
      const long long g = sy.off + n;
      const double c2 = sqrt((1.0 - c1 * c1) * kT * a.invm[g]);
      double z[3];
      langevin_noise(p, a, g, step, call, z);
      for (int x = 0; x < 3; ++x) a.v[x * N3 + g] = c1 * a.v[x * N3 + g] + c2 * z[x];
    }
    __syncthreads();
    kinetic<T>(a, c, red, sy);
    if (threadIdx.x == 0) c[C_ECT] += ekin0 - c[C_EKIN];
    __syncthreads();
  } else if (THERMO == TH_NHC || THERMO == TH_CSVR) {
    // one scale factor for all velocities; ekin and the kinetic tensor scale by its square
    // (NHChain.__call__, nvt.py:441-446; CSVRThermostat.pre, nvt.py:267-270)
    if (threadIdx.x == 0) {
      if (THERMO == TH_NHC) {
        double G1 = 0.0;
        if (g1) G1 = 2 * ekin_baro(c) - c[C_BNDOF] * kT;
        const double f = nhc_call(c, p, g1, G1, kT);
        for (int i = 0; i < 9; ++i) c[C_KT + i] *= f * f;
        if (call == 1) c[C_ECT] = nhc_econs(c, p, kT);
        sh.scal[0] = f;
      } else {
        sh.scal[0] = csvr_call(c, p, sys, a.nsys, step);
      }
    }
    __syncthreads();
    const double f = sh.scal[0];
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
      for (int x = 0; x < 3; ++x) a.v[x * N3 + sy.off + n] *= f;
    __syncthreads();
  } else if (THERMO == TH_BERENDSEN) {
    // v <- f v, ekin from the scaled velocities, correction (1 - f^2) ekin_before (nvt.py:152-159)
    if (threadIdx.x == 0) {
      const double f = berendsen_factor(c, p);
      c[C_SAVE] = c[C_EKIN];
      sh.scal[0] = f;
      for (int i = 0; i < 9; ++i) sh.mat[i] = (i % 4 == 0) ? f : 0.0;
    }
    __syncthreads();
    kinetic<T>(a, c, red, sy, KV_SCALE, sh.mat);
    if (threadIdx.x == 0) c[C_ECT] += (1 - sh.scal[0] * sh.scal[0]) * c[C_SAVE];
    __syncthreads();
  }
}

// ---- 3x3 algebra of the barostats on warp 0. On this part an FP64 instruction takes the
// same issue time on its SM sub-partition (~64 cycles) whether one lane or 32 are active,
// so a one-thread 3x3 product costs 27 such instructions and the CTA waits at the next
// barrier meanwhile. Here lane e < 9 forms entry e = 3 i + j of each 3x3 result (the
// expressions of the one-thread forms in mm_control.cuh; the matrix exponential with the
// same explicitly fused steps, so its two forms agree bit for bit), and scalars are formed
// redundantly by every lane. All 32 lanes of warp 0 call these.

__device__ __forceinline__ int wentry() {
  const int l = threadIdx.x & 31;
  return l < 9 ? l : 0;
}

// (A B)[e] from one entry per lane (a = A[e], b = B[e]).
__device__ __forceinline__ double wmatmul3(double a, double b) {
  const int e = wentry(), i = e / 3, j = e % 3;
  const double a0 = __shfl_sync(0xffffffffu, a, 3 * i), a1 = __shfl_sync(0xffffffffu, a, 3 * i + 1),
               a2 = __shfl_sync(0xffffffffu, a, 3 * i + 2);
  const double b0 = __shfl_sync(0xffffffffu, b, j), b1 = __shfl_sync(0xffffffffu, b, 3 + j),
               b2 = __shfl_sync(0xffffffffu, b, 6 + j);
  return fma(a2, b2, fma(a1, b1, __dmul_rn(a0, b0)));  // the rounding steps of matmul3
}

// norm1_3 (largest column sum of |A|) from one entry per lane; every lane gets it. The
// column sums are non-negative, so their largest is taken on the bit patterns.
__device__ __forceinline__ double wnorm1(double a) {
  const int l = threadIdx.x & 31, cj = l < 3 ? l : 0;
  const double x = fabs(a);
  const double col = __shfl_sync(0xffffffffu, x, cj) + __shfl_sync(0xffffffffu, x, 3 + cj) +
                     __shfl_sync(0xffffffffu, x, 6 + cj);
  const long long b = __double_as_longlong(col);
  const long long b0 = __shfl_sync(0xffffffffu, b, 0), b1 = __shfl_sync(0xffffffffu, b, 1),
                  b2 = __shfl_sync(0xffffffffu, b, 2);
  return __longlong_as_double(max(b0, max(b1, b2)));
}

// Entry e of exp(f S) from s = S[e] (sym_exp: scaling and squaring of the Taylor series).
__device__ __forceinline__ double wsym_exp(double s, double f) {
  const int e = wentry();
  double A = f * s;
  int k = 0;
  double nrm = wnorm1(A);
  while (nrm > 0.125 && k < 64) {
    A *= 0.5;
    nrm *= 0.5;
    ++k;
  }
  double term = (e % 4 == 0) ? 1.0 : 0.0, r = term;
  double bound = 1.0;
  for (int n = 1; n <= 20; ++n) {
    const double t = wmatmul3(term, A);
    const double inv = kInvN[n];
    term = __dmul_rn(t, inv);
    r = __dadd_rn(r, term);
    bound = __dmul_rn(__dmul_rn(bound, nrm), inv);
    if (bound <= 5e-19) break;
  }
  for (int q = 0; q < k; ++q) r = wmatmul3(r, r);
  return r;
}

// update_baro_vel with lane e updating c[C_VP + e].
__device__ __forceinline__ void wupdate_baro_vel(double* c, const BMD& p, bool chain, double cv0, const double* z6) {
  const int l = threadIdx.x & 31, e = wentry(), i = e / 3, j = e % 3;
  const double dt = p.dt;
  double vp = c[C_VP + e];
  const double fric = z6 ? exp_small(-dt / (8 * c[C_BTAU])) : 1.0;
  const double cfac = chain ? exp_small(-dt * cv0 / 8) : 1.0;
  const double inv_mass = 1.0 / c[C_MPRESS];
  if (z6) vp *= fric;
  if (chain) vp *= cfac;
  const double pt_ij = c[C_KT + e] - c[C_VT + e];
  const double pt_ji = c[C_KT + j * 3 + i] - c[C_VT + j * 3 + i];
  const double ps = 0.5 * (pt_ji + pt_ij);
  const double diag = 2.0 * c[C_EKIN] / c[C_NDOF] - p.press * c[C_VOL];
  double R = 0.0;
  if (z6) {
    const double sc = sqrt(2 * c[C_MPRESS] * kBoltzmannHa * c[C_BTEMP] / (dt * c[C_BTAU]));
    const int mx = i > j ? i : j, mn = i > j ? j : i, tri = mx * (mx + 1) / 2 + mn;  // lower-triangle slot
    double z = z6[0];
#pragma unroll
    for (int t = 1; t < 6; ++t)
      if (tri == t) z = z6[t];
    R = z * sc;
  }
  double Gi = (ps + ((e % 4 == 0) ? diag : 0.0)) * inv_mass;
  if (p.bflags & (BF_ISO | BF_VOLC)) {
    const double t = __shfl_sync(0xffffffffu, Gi, 0) + __shfl_sync(0xffffffffu, Gi, 4) +
                     __shfl_sync(0xffffffffu, Gi, 8);
    const double tr = __shfl_sync(0xffffffffu, R, 0) + __shfl_sync(0xffffffffu, R, 4) +
                      __shfl_sync(0xffffffffu, R, 8);
    if (p.bflags & BF_ISO) {  // one number: the trace of G, the first entry of R
      Gi = (e == 0) ? t : 0.0;
      R = (e == 0) ? R : 0.0;
    } else if (e % 4 == 0) {  // traceless
      Gi -= t / 3;
      R -= tr / 3;
    }
  }
  if (z6) vp += (Gi - R * inv_mass) * dt / 4;
  else vp += Gi * dt / 4;
  if (z6) vp *= fric;
  if (chain) vp *= cfac;
  __syncwarp();
  if (l < 9) c[C_VP + e] = vp;
  __syncwarp();
}

// berendsen_mu, entry e on lane e.
__device__ __forceinline__ double wberendsen_mu(const double* c, const BMD& p) {
  const int e = wentry(), i = e / 3, j = e % 3;
  auto dm = [&](int k) {
    const double ptens = (c[C_KT + k] - c[C_VT + k]) / c[C_VOL];
    return p.dt / c[C_MPRESS] * (((k % 4 == 0) ? p.press : 0.0) - ptens);
  };
  double d_ij = dm(i * 3 + j), d_ji = dm(j * 3 + i);
  if (p.bflags & BF_VOLC) {  // traceless increment (the trace formed redundantly by every lane)
    const double t3 = (dm(0) + dm(4) + dm(8)) / 3;
    if (i == j) {
      d_ij -= t3;
      d_ji -= t3;
    }
  }
  const double mu = 0.5 * ((((i == j) ? 1.0 : 0.0) - d_ij) + (((i == j) ? 1.0 : 0.0) - d_ji));
  if (p.bflags & BF_ISO) {  // the cube root of the mean diagonal, times the identity
    const double tr = __shfl_sync(0xffffffffu, mu, 0) + __shfl_sync(0xffffffffu, mu, 4) +
                      __shfl_sync(0xffffffffu, mu, 8);
    return (i == j) ? cbrt(tr / 3.0) : 0.0;
  }
  return mu;
}

// scale_domain: L <- L M, rv <- rv M (lane e: entry e), volume from the new rv.
__device__ __forceinline__ void wscale_domain(double* c, const double* M) {
  const int l = threadIdx.x & 31, e = wentry(), i = e / 3, j = e % 3;
  double sl = 0.0, sr = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    sl += c[C_L + i * 3 + k] * M[k * 3 + j];
    sr += c[C_RV + i * 3 + k] * M[k * 3 + j];
  }
  __syncwarp();
  if (l < 9) {
    c[C_L + e] = sl;
    c[C_RV + e] = sr;
  }
  __syncwarp();
  const double* r = c + C_RV;
  const double vol = fabs(r[0] * (r[4] * r[8] - r[5] * r[7]) + r[1] * (r[5] * r[6] - r[3] * r[8]) +
                          r[2] * (r[3] * r[7] - r[4] * r[6]));
  __syncwarp();
  if (l == 0) c[C_VOL] = vol;
  __syncwarp();
}

// Self-test of exp_small: out[i] = exp_small(x[i]).
__global__ void k_selftest_exp_small(const double* x, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = exp_small(x[i]);
}

// Self-test of the warp form: exp(f S) of n 3x3 matrices (row-major, 9 doubles each) by
// sym_exp on one thread (r_thread) and by wsym_exp on the warp (r_warp); one 32-thread
// block per matrix (mm_selftest_sym_exp).
__global__ void k_selftest_sym_exp(const double* S, int n, double f, double* r_thread, double* r_warp) {
  const int m = blockIdx.x;
  if (m >= n) return;
  if (threadIdx.x == 0) sym_exp(S + 9 * m, f, r_thread + 9 * m);
  const double r = wsym_exp(S[9 * m + wentry()], f);
  if (threadIdx.x < 9) r_warp[9 * m + threadIdx.x] = r;
}

// MTK half step (MTKBarostat.baro, npt.py:653-736): barostat velocity, position and
// domain scaling, force evaluation, velocity scaling, barostat velocity again. With
// BA_LANGEVIN the barostat-velocity updates carry the Langevin barostat's friction and
// random force (LangevinBarostat.baro, npt.py:402-486; draws `call0`, `call0 + 1`).
template <typename T, int MODEL>
__device__ void baro_half(const BArgs& a, Shared<T>& sh, const BSys& sy, const BMD& p, bool chain, double* cv0p,
                          unsigned sys, long long step, int call0) {
  double* c = sh.ctl;
  const long long N3 = a.Ntot;
  const bool lang = p.baro == BA_LANGEVIN;
  if (threadIdx.x < 32) {
    double z6[6];
    if (lang) lbaro_draws(p, sys, a.nsys, step, call0, z6);
    wupdate_baro_vel(c, p, chain, chain ? *cv0p : 0.0, lang ? z6 : nullptr);
    double r;
    if (p.bflags & BF_ISO) {
      const double f = exp_small(c[C_VP + 0] * p.dt / 2);
      r = (wentry() % 4 == 0) ? f : 0.0;
    } else {
      r = wsym_exp(c[C_VP + wentry()], p.dt / 2);
    }
    if (threadIdx.x < 9) sh.mat[threadIdx.x] = r;
    __syncwarp();
    wscale_domain(c, sh.mat);
  }
  __syncthreads();
  positions<T>(a, sy, sh.mat, 0.0);
  refresh_B<T>(sh, a.tt, a.ntypes, c + C_L);
  __syncthreads();
  forces<T, MODEL>(a, sh, sy);
  if (threadIdx.x < 32) {
    // mtk_vel_scaling, entry e on lane e
    const int e = wentry();
    double r;
    if (p.bflags & BF_ISO) {
      const double f = exp_small(-((1.0 + 3.0 / c[C_NDOF]) * c[C_VP + 0]) * p.dt / 2);
      r = (e % 4 == 0) ? f : 0.0;
    } else {
      const double tr = (p.bflags & BF_VOLC) ? 0.0 : c[C_VP + 0] + c[C_VP + 4] + c[C_VP + 8];
      r = wsym_exp(c[C_VP + e] + ((e % 4 == 0) ? tr / c[C_NDOF] : 0.0), -p.dt / 2);
    }
    if (threadIdx.x < 9) sh.mat[threadIdx.x] = r;
  }
  __syncthreads();
  // v <- v R; the kinetic tensor follows as R^T K R (no second sum over the nodes)
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    double x = a.v[g], y = a.v[N3 + g], z = a.v[2 * N3 + g];
    rows_times<T>(x, y, z, sh.mat);
    a.v[g] = x;
    a.v[N3 + g] = y;
    a.v[2 * N3 + g] = z;
  }
  if (threadIdx.x < 32) {
    // K <- sym(R^T (K R)), entry e on lane e
    const int e = wentry(), i = e / 3, j = e % 3;
    const double* R = sh.mat;
    const double KR = wmatmul3(c[C_KT + e], R[e]);
    const double K2 = wmatmul3(R[j * 3 + i], KR);
    const double kt = 0.5 * (K2 + __shfl_sync(0xffffffffu, K2, j * 3 + i));
    __syncwarp();
    if (threadIdx.x < 9) c[C_KT + e] = kt;
    __syncwarp();
    const double ek = 0.5 * (c[C_KT + 0] + c[C_KT + 4] + c[C_KT + 8]);
    __syncwarp();
    if (threadIdx.x == 0) c[C_EKIN] = ek;
    __syncwarp();
    double z6[6];
    if (lang) lbaro_draws(p, sys, a.nsys, step, call0 + 1, z6);
    wupdate_baro_vel(c, p, chain, chain ? *cv0p : 0.0, lang ? z6 : nullptr);
  }
  __syncthreads();
}

// Berendsen barostat post call (BerendsenBarostat.post, npt.py:262-292): positions and
// domain times mu, forces again, correction += epot before - epot after.
template <typename T, int MODEL>
__device__ void berendsen_baro(const BArgs& a, Shared<T>& sh, const BSys& sy, const BMD& p) {
  double* c = sh.ctl;
  if (threadIdx.x < 32) {
    const double mu = wberendsen_mu(c, p);
    if (threadIdx.x == 0) c[C_SAVE] = c[C_EPOT];
    if (threadIdx.x < 9) sh.mat[threadIdx.x] = mu;
    __syncwarp();
    wscale_domain(c, sh.mat);
  }
  __syncthreads();
  positions<T>(a, sy, sh.mat, 0.0);
  refresh_B<T>(sh, a.tt, a.ntypes, c + C_L);
  __syncthreads();
  forces<T, MODEL>(a, sh, sy);
  if (threadIdx.x == 0) c[C_ECB] += c[C_SAVE] - c[C_EPOT];
  __syncthreads();
}

// Barostat pre/post call of the MTK or Langevin barostat (the Berendsen barostat acts in
// post only). The Langevin barostat adds the change of epot + ekin over its call to its
// correction (npt.py:375-395); the MTK barostat sets its correction after post. An MTK
// barostat with its own chain runs that chain after the half step in pre and before it in
// post, and its barostat velocity feels that chain's first velocity (npt.py:616-651).
template <typename T, int MODEL>
__device__ void baro_call(const BArgs& a, Shared<T>& sh, const BSys& sy, const BMD& p, double* cv0p,
                          unsigned sys, long long step, int call0) {
  double* c = sh.ctl;
  const bool bch = p.bflags & BF_CHAIN;
  const bool chain = p.thermo == TH_NHC || bch;
  if (threadIdx.x == 0) {
    if (bch && call0 != 0) mtk_chain_step(c, p);
    *cv0p = bch ? c[C_BCVEL + 0] : c[C_CVEL + 0];
    c[C_SAVE] = c[C_EPOT] + c[C_EKIN];
  }
  __syncthreads();
  baro_half<T, MODEL>(a, sh, sy, p, chain, cv0p, sys, step, call0);
  if (threadIdx.x == 0) {
    if (bch && call0 == 0) mtk_chain_step(c, p);
    if (p.baro == BA_LANGEVIN) c[C_ECB] += c[C_SAVE] - c[C_EPOT] - c[C_EKIN];
    else if (call0 != 0) c[C_ECB] = mtk_econs(c, p);
  }
  __syncthreads();
}

template <typename T, int MODEL, int BT>
__global__ void __launch_bounds__(BT, (sizeof(T) == 4 && MODEL >= 1) ? 512 / BT : 1) k_batch_md(BArgs a, BMD p) {
  const int THERMO = p.thermo, BARO = p.baro;
  __shared__ Shared<T> sh;
  __shared__ double cv0;
  for (int w = a.work_off[blockIdx.x]; w < a.work_off[blockIdx.x + 1]; ++w) {
    const int b = a.work[w];
    const BSys sy = a.sys[b];
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) sh.ctl[i] = a.ctl[(size_t)b * C_LEN + i];
    __syncthreads();
    double* c = sh.ctl;
    load_tables<T>(sh, a.tt, a.ntypes, c + C_L);
    __syncthreads();
    const double kT = kBoltzmannHa * p.temp;
    write_disp<T>(a, sy);
    __syncthreads();
    forces<T, MODEL>(a, sh, sy);
    kinetic<T>(a, c, sh.red, sy);
    for (int st = 1; st <= p.nsteps; ++st) {
      const long long step = p.step0 + st;
      // ---- pre hooks: barostat, then thermostat (TBCombination.pre)
      if (BARO == BA_MTK || BARO == BA_LANGEVIN) baro_call<T, MODEL>(a, sh, sy, p, &cv0, b, step, 0);
      if (THERMO == TH_LANGEVIN) thermostat<T, TH_LANGEVIN>(a, sh, sy, p, step, 0u, false, kT, b);
      if (THERMO == TH_NHC) thermostat<T, TH_NHC>(a, sh, sy, p, step, 0u, mtk_couples_chain(p), kT, b);
      if (THERMO == TH_BERENDSEN) thermostat<T, TH_BERENDSEN>(a, sh, sy, p, step, 0u, false, kT, b);
      if (THERMO == TH_CSVR) thermostat<T, TH_CSVR>(a, sh, sy, p, step, 0u, false, kT, b);
      // ---- velocity Verlet
      positions<T>(a, sy, nullptr, p.dt);
      __syncthreads();
      forces<T, MODEL>(a, sh, sy);
      kinetic<T>(a, c, sh.red, sy, KV_KICK, nullptr, p.dt);
      // ---- post hooks: thermostat, then barostat
      if (THERMO == TH_LANGEVIN) thermostat<T, TH_LANGEVIN>(a, sh, sy, p, step, 1u, false, kT, b);
      if (THERMO == TH_NHC) thermostat<T, TH_NHC>(a, sh, sy, p, step, 1u, mtk_couples_chain(p), kT, b);
      if (BARO == BA_MTK || BARO == BA_LANGEVIN) baro_call<T, MODEL>(a, sh, sy, p, &cv0, b, step, 2);
      if (BARO == BA_BERENDSEN) berendsen_baro<T, MODEL>(a, sh, sy, p);
      if (threadIdx.x == 0 && p.rec) {
        double* r = p.rec + ((size_t)b * p.nsteps + (st - 1)) * BR_LEN;
        double corr = c[C_ECT] + c[C_ECB];
        if (THERMO == TH_NHC && BARO != BA_NONE && !(p.bflags & BF_CHAIN)) corr += c[C_BNDOF] * kT * c[C_CPOS + 0];
        r[BR_EPOT] = c[C_EPOT];
        r[BR_EKIN] = c[C_EKIN];
        r[BR_ECORR] = corr;
        r[BR_VOL] = c[C_VOL];
        for (int i = 0; i < 9; ++i) {
          r[BR_VT + i] = c[C_VT + i];
          r[BR_KT + i] = c[C_KT + i];
          r[BR_RV + i] = c[C_RV + i];
        }
      }
      __syncthreads();
    }
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) a.ctl[(size_t)b * C_LEN + i] = sh.ctl[i];
    __syncthreads();
  }
}

// Relaxation of every system with Polak-Ribiere+ conjugate gradients and a secant
// line search along each direction, until the largest node gradient is below gtol
// or max_iter iterations have run. Positions only (the domain is fixed).
template <typename T, int MODEL, int BT>
__global__ void __launch_bounds__(BT) k_batch_relax(BArgs a, int max_iter, double gtol) {
  __shared__ Shared<T> sh;
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done;
  const long long N3 = a.Ntot;
  for (int w = a.work_off[blockIdx.x]; w < a.work_off[blockIdx.x + 1]; ++w) {
    const int b = a.work[w];
    const BSys sy = a.sys[b];
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) sh.ctl[i] = a.ctl[(size_t)b * C_LEN + i];
    __syncthreads();
    double* c = sh.ctl;
    load_tables<T>(sh, a.tt, a.ntypes, c + C_L);
    __syncthreads();
    write_disp<T>(a, sy);
    __syncthreads();
    forces<T, MODEL>(a, sh, sy);
    // d = -g ; keep g
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
      for (int x = 0; x < 3; ++x) {
        const long long g = x * N3 + sy.off + n;
        a.cgd[g] = -a.gpos[g];
        a.cgg[g] = a.gpos[g];
      }
    if (threadIdx.x == 0) {
      s_done = 0;
      if (!(c[C_ALPHA] > 0.0)) c[C_ALPHA] = 1e-3;
    }
    __syncthreads();
    int it = 0;
    for (; it < max_iter; ++it) {
      // convergence and directional derivative s0 = g.d, gmax
      double acc[3] = {0.0, 0.0, 0.0};
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
        double gn = 0.0;
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          acc[0] += a.gpos[g] * a.cgd[g];
          acc[1] += a.gpos[g] * a.gpos[g];
          gn += a.gpos[g] * a.gpos[g];
        }
        acc[2] = fmax(acc[2], gn);
      }
      // max via a separate block reduction of a value stored as the largest element
      __shared__ double gm[BT];
      gm[threadIdx.x] = acc[2];
      acc[2] = 0.0;
      block_sum<3>(acc, sh.red);
      for (int off = BT / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) gm[threadIdx.x] = fmax(gm[threadIdx.x], gm[threadIdx.x + off]);
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        c[C_GMAX] = sqrt(gm[0]);
        s_done = (c[C_GMAX] < gtol) ? 1 : 0;
        sh.scal[0] = acc[0];  // s0
        sh.scal[1] = acc[1];  // g.g
      }
      __syncthreads();
      if (s_done) break;
      if (sh.scal[0] >= 0.0) {  // not a descent direction: restart with steepest descent
        for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
          for (int x = 0; x < 3; ++x) a.cgd[x * N3 + sy.off + n] = -a.gpos[x * N3 + sy.off + n];
        if (threadIdx.x == 0) sh.scal[0] = -sh.scal[1];
        __syncthreads();
      }
      const double s0 = sh.scal[0], e0 = c[C_EPOT];
      // save positions and gradient
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          a.cgu[g] = a.u[g];
          a.cgg[g] = a.gpos[g];
        }
      __syncthreads();
      // line search on phi'(alpha) = g(x + alpha d) . d (gradient-based, so that it also
      // works when energy differences are below the cell precision's resolution):
      // bracketed (phi' >= 0) -> secant root; enough slope decrease -> accept; still
      // steep -> extrapolate; energy above e0 + noise -> backtrack.
      const double noise = (sizeof(T) == 4 ? 1e-6 : 1e-12) * fabs(e0);
      double alpha = c[C_ALPHA];
      bool accepted = false;
      __shared__ int s_mode;
      for (int ls = 0; ls < 16 && !accepted; ++ls) {
        for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
          for (int x = 0; x < 3; ++x) {
            const long long g = x * N3 + sy.off + n;
            a.u[g] = a.cgu[g] + alpha * a.cgd[g];
          }
        __syncthreads();
        write_disp<T>(a, sy);
        __syncthreads();
        forces<T, MODEL>(a, sh, sy);
        double s1v[1] = {0.0};
        for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
          for (int x = 0; x < 3; ++x) s1v[0] += a.gpos[x * N3 + sy.off + n] * a.cgd[x * N3 + sy.off + n];
        block_sum<1>(s1v, sh.red);
        if (threadIdx.x == 0) {
          const double s1 = s1v[0], e1 = c[C_EPOT];
          int mode = 0;
          double anew = alpha;
          if (e1 > e0 + noise && s1 < 0.0) {
            anew = 0.25 * alpha;
          } else if (s1 >= 0.0) {
            anew = alpha * (-s0) / (s1 - s0);  // root of the secant through (0, s0), (alpha, s1)
            mode = 2;
          } else if (fabs(s1) <= 0.5 * fabs(s0)) {
            mode = 1;
          } else {
            anew = (s1 > s0) ? fmin(alpha * (-s0) / (s1 - s0), 8.0 * alpha) : 4.0 * alpha;
          }
          s_alpha = anew;
          s_mode = mode;
        }
        __syncthreads();
        if (s_mode == 1) {
          accepted = true;
          if (threadIdx.x == 0) c[C_ALPHA] = alpha;
        } else if (s_mode == 2) {
          const double as = s_alpha;
          for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
            for (int x = 0; x < 3; ++x) {
              const long long g = x * N3 + sy.off + n;
              a.u[g] = a.cgu[g] + as * a.cgd[g];
            }
          __syncthreads();
          write_disp<T>(a, sy);
          __syncthreads();
          forces<T, MODEL>(a, sh, sy);
          accepted = true;
          if (threadIdx.x == 0) c[C_ALPHA] = as;
        } else {
          alpha = s_alpha;
        }
        __syncthreads();
      }
      if (!accepted) {  // restore and stop: no progress possible along d
        for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
          for (int x = 0; x < 3; ++x) {
            const long long g = x * N3 + sy.off + n;
            a.u[g] = a.cgu[g];
          }
        __syncthreads();
        write_disp<T>(a, sy);
        __syncthreads();
        forces<T, MODEL>(a, sh, sy);
        break;
      }
      // Polak-Ribiere+: beta = max(0, g.(g - g_old) / g_old.g_old)
      double bb[2] = {0.0, 0.0};
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          bb[0] += a.gpos[g] * (a.gpos[g] - a.cgg[g]);
          bb[1] += a.cgg[g] * a.cgg[g];
        }
      block_sum<2>(bb, sh.red);
      if (threadIdx.x == 0) s_beta = fmax(0.0, bb[0] / fmax(bb[1], 1e-300));
      __syncthreads();
      const double beta = s_beta;
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          a.cgd[g] = -a.gpos[g] + beta * a.cgd[g];
        }
      __syncthreads();
    }
    if (threadIdx.x == 0) c[C_ITER] = it;
    __syncthreads();
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) a.ctl[(size_t)b * C_LEN + i] = sh.ctl[i];
    __syncthreads();
  }
}

// ------------------------------------------------------------ relaxation with cell DOFs
// Positions and domain together, as the reference's BaseCellDOF does (dof.py:199-470):
// x = (cell variables, fractional coordinates). StrainCellDOF (dof.py:522-697): six
// variables [A00, A11, A22, 2 A12, 2 A20, 2 A01] of a symmetric A, rvecs = A rvecs0;
// FullCellDOF (dof.py:492-519): the nine components of rvecs / V0^(1/3). The gradient is
// (J^T grvecs, gpos rvecs^T) with grvecs = gvecs (vtens + P V I) (dof.py:370-384; the
// pressure term is ForcePartPressure's E = P V). Polak-Ribiere+ CG with the secant line
// search of k_batch_relax along the joint direction; converged when the largest node
// gradient is below gtol and the largest residual stress component |vtens / V + P I| is
// below stol. Fractional displacements w (pos = (grid fraction + w) rvecs) are the
// position variables; u = w rvecs is rebuilt at every evaluation.
__device__ inline void inv3(const double* m, double* r) {
  const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
  const double id = 1.0 / (m[0] * c00 + m[1] * c01 + m[2] * c02);
  r[0] = c00 * id;
  r[1] = (m[2] * m[7] - m[1] * m[8]) * id;
  r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  r[3] = c01 * id;
  r[4] = (m[0] * m[8] - m[2] * m[6]) * id;
  r[5] = (m[2] * m[3] - m[0] * m[5]) * id;
  r[6] = c02 * id;
  r[7] = (m[1] * m[6] - m[0] * m[7]) * id;
  r[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

// rvecs from the cell variables (thread 0)
__device__ inline void cell_to_rvecs(const double* xc, const double* rv0, double scale, int full, double* rv) {
  if (full) {
    for (int i = 0; i < 9; ++i) rv[i] = xc[i] * scale;
  } else {
    const double A[9] = {xc[0], 0.5 * xc[5], 0.5 * xc[4], 0.5 * xc[5], xc[1], 0.5 * xc[3],
                         0.5 * xc[4], 0.5 * xc[3], xc[2]};
    matmul3(A, rv0, rv);
  }
}

// gradient of the cell variables from grvecs (thread 0): J^T grvecs
__device__ inline void cell_gradient(const double* grv, const double* rv0, double scale, int full, double* gx) {
  if (full) {
    for (int i = 0; i < 9; ++i) gx[i] = grv[i] * scale;
  } else {
    double gA[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        gA[i * 3 + j] = grv[i * 3] * rv0[j * 3] + grv[i * 3 + 1] * rv0[j * 3 + 1] + grv[i * 3 + 2] * rv0[j * 3 + 2];
    gx[0] = gA[0];
    gx[1] = gA[4];
    gx[2] = gA[8];
    gx[3] = 0.5 * (gA[5] + gA[7]);
    gx[4] = 0.5 * (gA[6] + gA[2]);
    gx[5] = 0.5 * (gA[1] + gA[3]);
  }
}

struct CellShared {
  double rv0[9], rv[9], xc0[9], dc[9], gc[9], gco[9];
  double scale;
  double s, gg, gmax;  // reduction results of the last evaluation
  double alpha, beta;
  int mode, done, ncv;
};

// One evaluation at x0 + alpha d: domain, displacements, forces, gradients in x space
// (node part written over gpos), node max |gpos|^2, g.d and g.g (cell parts included).
template <typename T, int MODEL, int BT>
__device__ __noinline__ void cell_eval(const BArgs& a, Shared<T>& sh, CellShared& cs, const BSys& sy, const CellRelax& r,
                          double alpha, double* gm) {
  double* c = sh.ctl;
  const long long N3 = a.Ntot;
  if (threadIdx.x == 0) {
    double xc[9];
    for (int i = 0; i < cs.ncv; ++i) xc[i] = cs.xc0[i] + alpha * cs.dc[i];
    cell_to_rvecs(xc, cs.rv0, cs.scale, r.full, cs.rv);
    const int n[3] = {sy.nx, sy.ny, sy.nz};
    for (int d = 0; d < 3; ++d)
      for (int x = 0; x < 3; ++x) {
        c[C_RV + 3 * d + x] = cs.rv[3 * d + x];
        c[C_L + 3 * d + x] = cs.rv[3 * d + x] / n[d];
      }
    const double* q = cs.rv;
    c[C_VOL] = fabs(q[0] * (q[4] * q[8] - q[5] * q[7]) + q[1] * (q[5] * q[6] - q[3] * q[8]) +
                    q[2] * (q[3] * q[7] - q[4] * q[6]));
  }
  __syncthreads();
  refresh_B<T>(sh, a.tt, a.ntypes, c + C_L);
  T* disp = (T*)a.disp;
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    double w[3];
    for (int x = 0; x < 3; ++x) w[x] = a.cgu[x * N3 + g] + alpha * a.cgd[x * N3 + g];
    for (int x = 0; x < 3; ++x) {
      const double ux = w[0] * cs.rv[x] + w[1] * cs.rv[3 + x] + w[2] * cs.rv[6 + x];
      a.u[x * N3 + g] = ux;
      disp[x * N3 + g] = from_double<T>(ux);
    }
  }
  __syncthreads();
  forces<T, MODEL>(a, sh, sy);
  // node gradient in fractional coordinates gw = gpos rvecs^T, with max |gpos|^2, gw.d, gw.gw
  double acc[2] = {0.0, 0.0};
  double gmx = 0.0;
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    const double gp[3] = {a.gpos[g], a.gpos[N3 + g], a.gpos[2 * N3 + g]};
    gmx = fmax(gmx, gp[0] * gp[0] + gp[1] * gp[1] + gp[2] * gp[2]);
    for (int i = 0; i < 3; ++i) {
      const double gw = gp[0] * cs.rv[3 * i] + gp[1] * cs.rv[3 * i + 1] + gp[2] * cs.rv[3 * i + 2];
      a.gpos[i * N3 + g] = gw;
      acc[0] += gw * a.cgd[i * N3 + g];
      acc[1] += gw * gw;
    }
  }
  gm[threadIdx.x] = gmx;
  block_sum<2>(acc, sh.red);
  for (int off = BT / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) gm[threadIdx.x] = fmax(gm[threadIdx.x], gm[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // cell gradient: grvecs = gvecs (vtens + P V I), gvecs = rvecs^-T
    double vt[9], inv[9], gv[9], grv[9];
    double smax = 0.0;
    for (int i = 0; i < 9; ++i) {
      vt[i] = c[C_VT + i] + ((i % 4 == 0) ? r.press * c[C_VOL] : 0.0);
      smax = fmax(smax, fabs(vt[i]) / c[C_VOL]);
    }
    inv3(cs.rv, inv);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) gv[i * 3 + j] = inv[j * 3 + i];
    matmul3(gv, vt, grv);
    cell_gradient(grv, cs.rv0, cs.scale, r.full, cs.gc);
    double sd = acc[0], g2 = acc[1];
    for (int i = 0; i < cs.ncv; ++i) {
      sd += cs.gc[i] * cs.dc[i];
      g2 += cs.gc[i] * cs.gc[i];
    }
    cs.s = sd;
    cs.gg = g2;
    cs.gmax = sqrt(gm[0]);
    c[C_GMAX] = cs.gmax;
    c[C_SRES] = smax;
  }
  __syncthreads();
}

template <typename T, int MODEL, int BT>
__global__ void __launch_bounds__(BT) k_batch_relax_cell(BArgs a, CellRelax r) {
  __shared__ Shared<T> sh;
  __shared__ CellShared cs;
  __shared__ double gm[BT];
  const long long N3 = a.Ntot;
  for (int w = a.work_off[blockIdx.x]; w < a.work_off[blockIdx.x + 1]; ++w) {
    const int b = a.work[w];
    const BSys sy = a.sys[b];
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) sh.ctl[i] = a.ctl[(size_t)b * C_LEN + i];
    __syncthreads();
    double* c = sh.ctl;
    load_tables<T>(sh, a.tt, a.ntypes, c + C_L);
    if (threadIdx.x == 0) {
      for (int i = 0; i < 9; ++i) cs.rv0[i] = c[C_RV + i];
      cs.scale = cbrt(c[C_VOL]);
      cs.ncv = r.full ? 9 : 6;
      if (r.full) {
        for (int i = 0; i < 9; ++i) cs.xc0[i] = cs.rv0[i] / cs.scale;
      } else {
        const double x0[6] = {1.0, 1.0, 1.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < 6; ++i) cs.xc0[i] = x0[i];
      }
      for (int i = 0; i < 9; ++i) cs.dc[i] = 0.0;
      inv3(cs.rv0, sh.mat);
      cs.done = 0;
      if (!(c[C_ALPHA] > 0.0)) c[C_ALPHA] = 1e-3;
    }
    __syncthreads();
    // fractional displacements w = u rvecs^-1 (saved point), zero direction
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
      const long long g = sy.off + n;
      const double u[3] = {a.u[g], a.u[N3 + g], a.u[2 * N3 + g]};
      for (int x = 0; x < 3; ++x) {
        a.cgu[x * N3 + g] = u[0] * sh.mat[x] + u[1] * sh.mat[3 + x] + u[2] * sh.mat[6 + x];
        a.cgd[x * N3 + g] = 0.0;
      }
    }
    __syncthreads();
    cell_eval<T, MODEL, BT>(a, sh, cs, sy, r, 0.0, gm);
    // d = -g
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
      for (int x = 0; x < 3; ++x) a.cgd[x * N3 + sy.off + n] = -a.gpos[x * N3 + sy.off + n];
    if (threadIdx.x == 0) {
      for (int i = 0; i < cs.ncv; ++i) cs.dc[i] = -cs.gc[i];
      cs.s = -cs.gg;
    }
    __syncthreads();
    int it = 0;
    for (; it < r.max_iter; ++it) {
      if (threadIdx.x == 0) cs.done = (cs.gmax < r.gtol && c[C_SRES] < r.stol) ? 1 : 0;
      __syncthreads();
      if (cs.done) break;
      if (cs.s >= 0.0) {  // not a descent direction: steepest descent
        for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
          for (int x = 0; x < 3; ++x) a.cgd[x * N3 + sy.off + n] = -a.gpos[x * N3 + sy.off + n];
        if (threadIdx.x == 0) {
          for (int i = 0; i < cs.ncv; ++i) cs.dc[i] = -cs.gc[i];
          cs.s = -cs.gg;
        }
        __syncthreads();
      }
      const double s0 = cs.s, e0 = c[C_EPOT] + r.press * c[C_VOL];
      // keep the gradient at the line-search start (cgg, gco)
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) a.cgg[x * N3 + sy.off + n] = a.gpos[x * N3 + sy.off + n];
      if (threadIdx.x == 0)
        for (int i = 0; i < cs.ncv; ++i) cs.gco[i] = cs.gc[i];
      __syncthreads();
      const double noise = (sizeof(T) == 4 ? 1e-6 : 1e-12) * fabs(e0);
      double alpha = c[C_ALPHA];
      bool accepted = false;
      for (int ls = 0; ls < 16 && !accepted; ++ls) {
        cell_eval<T, MODEL, BT>(a, sh, cs, sy, r, alpha, gm);
        if (threadIdx.x == 0) {
          const double s1 = cs.s, e1 = c[C_EPOT] + r.press * c[C_VOL];
          int mode = 0;
          double anew = alpha;
          if (e1 > e0 + noise && s1 < 0.0) {
            anew = 0.25 * alpha;
          } else if (s1 >= 0.0) {
            anew = alpha * (-s0) / (s1 - s0);
            mode = 2;
          } else if (fabs(s1) <= 0.5 * fabs(s0)) {
            mode = 1;
          } else {
            anew = (s1 > s0) ? fmin(alpha * (-s0) / (s1 - s0), 8.0 * alpha) : 4.0 * alpha;
          }
          cs.alpha = anew;
          cs.mode = mode;
        }
        __syncthreads();
        if (cs.mode == 1) {
          accepted = true;
        } else if (cs.mode == 2) {
          alpha = cs.alpha;
          cell_eval<T, MODEL, BT>(a, sh, cs, sy, r, alpha, gm);
          accepted = true;
        } else {
          alpha = cs.alpha;
        }
        __syncthreads();
      }
      if (!accepted) {  // restore the start point and stop
        cell_eval<T, MODEL, BT>(a, sh, cs, sy, r, 0.0, gm);
        break;
      }
      // move the saved point to the accepted one: w0 += alpha d, xc0 += alpha dc
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          a.cgu[g] += alpha * a.cgd[g];
        }
      // Polak-Ribiere+: beta = max(0, g.(g - g_old) / g_old.g_old)
      double bb[2] = {0.0, 0.0};
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          bb[0] += a.gpos[g] * (a.gpos[g] - a.cgg[g]);
          bb[1] += a.cgg[g] * a.cgg[g];
        }
      block_sum<2>(bb, sh.red);
      if (threadIdx.x == 0) {
        c[C_ALPHA] = alpha;
        for (int i = 0; i < cs.ncv; ++i) {
          cs.xc0[i] += alpha * cs.dc[i];
          bb[0] += cs.gc[i] * (cs.gc[i] - cs.gco[i]);
          bb[1] += cs.gco[i] * cs.gco[i];
        }
        cs.beta = fmax(0.0, bb[0] / fmax(bb[1], 1e-300));
      }
      __syncthreads();
      const double beta = cs.beta;
      double sv[1] = {0.0};
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
        for (int x = 0; x < 3; ++x) {
          const long long g = x * N3 + sy.off + n;
          const double d = -a.gpos[g] + beta * a.cgd[g];
          a.cgd[g] = d;
          sv[0] += a.gpos[g] * d;
        }
      block_sum<1>(sv, sh.red);
      if (threadIdx.x == 0) {
        double sd = sv[0];
        for (int i = 0; i < cs.ncv; ++i) {
          cs.dc[i] = -cs.gc[i] + beta * cs.dc[i];
          sd += cs.gc[i] * cs.dc[i];
        }
        cs.s = sd;
      }
      __syncthreads();
    }
    // positions gradient back to Cartesian (gpos = gw rvecs^-T) for the caller
    if (threadIdx.x == 0) {
      c[C_ITER] = it;
      inv3(cs.rv, sh.mat);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
      const long long g = sy.off + n;
      const double gw[3] = {a.gpos[g], a.gpos[N3 + g], a.gpos[2 * N3 + g]};
      for (int x = 0; x < 3; ++x)
        a.gpos[x * N3 + g] = gw[0] * sh.mat[x * 3] + gw[1] * sh.mat[x * 3 + 1] + gw[2] * sh.mat[x * 3 + 2];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) a.ctl[(size_t)b * C_LEN + i] = sh.ctl[i];
    __syncthreads();
  }
}

}  // namespace
}  // namespace mmb
