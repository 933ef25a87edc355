// Device-side building blocks of the MicMec force path for sm_103a.
//
// One nanocell is a hexahedron with 8 corner nodes. Corner k of a cell sits at
// lattice offset CORNER_OFF[k] from the cell's origin node, in the order of
// micmec/utils.py:43-52. Inside the kernels the corners are addressed by their
// offset bits (x | y<<1 | z<<2), which makes "the edge along d touching corner
// b" a bit flip; BITS_TO_CORNER / CORNER_TO_BITS convert between the two.
//
// Node displacements: every node has a lattice site X = kk*L0 + ll*L1 + mm*L2,
// with L the lattice matrix (rows L_d = rvecs_d / n_d for a periodic domain).
// Kernels work with u = pos - X. The edge along d between corners lo and hi is
// then exactly L_d + u_hi - u_lo, including edges that cross the periodic
// boundary (the reference's minimum-image shift, micmec/pes/mmff.py:334-371),
// and the deviation of a corner matrix from a rest matrix h0 is
// W = (L - h0) + dU: a small number in every precision.
#pragma once

#include <cstddef>
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#define MM_MAX_TYPES 8
#define MM_MAX_STATES 4

namespace mm {

// corner index (reference order) <-> offset bits
__host__ __device__ constexpr int bits_to_corner(int b) {
  // (0,0,0)0 (1,0,0)1 (0,1,0)2 (1,1,0)4 (0,0,1)3 (1,0,1)5 (0,1,1)6 (1,1,1)7
  return b == 3 ? 4 : (b == 4 ? 3 : b);
}
__host__ __device__ constexpr int corner_to_bits(int k) { return k == 3 ? 4 : (k == 4 ? 3 : k); }

// Per (type, state) parameters in the precision T of the cell arithmetic. The first
// 20 values are what the cubic form reads (16-byte aligned, vector loads).
template <typename T>
struct __align__(16) StateParams {
  T B[9];      // L - h0 (rows), for the current lattice matrix L
  T v0;        // det(h0)
  T df;        // state free energy
  T hd[3];     // diagonal of h0^-1 (cubic form)
  T cub[3];    // A00 - A01, A01, A33 (cubic form)
  T pad0[3];
  T A[36];     // 6x6: symmetric stress (Voigt 00,11,22,12,02,01) = A . strain
  T hinv[9];   // h0^-1, row-major
  T pad1[3];
};

template <typename T>
struct TypeParams {
  StateParams<T> s[MM_MAX_STATES];
  T kT;        // boltzmann * effective temperature
  T lkT;       // log2(e) / kT
  int nstates;
};

// Host-side FP64 table (uploaded once); B is derived per launch from L.
struct StateTable {
  double h0[9];
  double hinv[9];
  double A[36];
  double v0;
  double df;
};
struct TypeTable {
  StateTable s[MM_MAX_STATES];
  double kT;
  int nstates;
  int pad;
};

template <typename T>
__device__ __forceinline__ void fill_type_scalars(TypeParams<T>& dst, const TypeTable& src) {
  dst.kT = (T)src.kT;
  dst.lkT = (T)(1.4426950408889634 / src.kT);
  dst.nstates = src.nstates;
}

// Cell-precision copy of one (type, state) entry for the lattice matrix L. Entry e of
// StateParams (in its field order) is (T)(x - y), formed in FP64 and then rounded: B = L - h0,
// cub[0] = A00 - A01, and y = 0 for the others (x - 0.0 is x exactly): v0, df, hd = diagonal
// of h0^-1, cub[1] = A01, cub[2] = A33, A, hinv; the pads are 0.
constexpr int kStateParamElems = 68;
static_assert(sizeof(StateParams<float>) == kStateParamElems * sizeof(float), "StateParams<float> layout");
static_assert(sizeof(StateParams<double>) == kStateParamElems * sizeof(double), "StateParams<double> layout");
__device__ __forceinline__ void state_param_source(const StateTable& src, const double* L, int e, double& x,
                                                   double& y) {
  x = 0.0;
  y = 0.0;
  if (e < 9) {  // B
    x = L[e];
    y = src.h0[e];
  } else if (e == 9) {
    x = src.v0;
  } else if (e == 10) {
    x = src.df;
  } else if (e < 14) {  // hd
    x = src.hinv[4 * (e - 11)];
  } else if (e == 14) {  // cub
    x = src.A[0];
    y = src.A[1];
  } else if (e == 15) {
    x = src.A[1];
  } else if (e == 16) {
    x = src.A[21];
  } else if (e >= 20 && e < 56) {  // A (pad0 is 17..19)
    x = src.A[e - 20];
  } else if (e >= 56 && e < 65) {  // hinv (pad1 is 65..67)
    x = src.hinv[e - 56];
  }
}

// The block's copy of the parameter tables for lattice matrix L, every state of every type:
// entries spread over all threads, each thread's loads issued before its conversions
// (FP64 operations are slow and unpipelined per warp on this part, so a routine that
// gives one thread a whole (type, state) entry keeps the block waiting thousands of
// cycles). The type scalars (one FP64 division each) go to the last threads.
template <typename T>
__device__ void fill_params_block(TypeParams<T>* tp, const TypeTable* __restrict__ tt, int ntypes,
                                  const double* __restrict__ L) {
  constexpr int kPer = MM_MAX_STATES * kStateParamElems, kBatch = 8;
  const int total = ntypes * kPer;
  for (int base = threadIdx.x; base < total; base += kBatch * blockDim.x) {
    double x[kBatch], y[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      const int idx = base + k * blockDim.x;
      x[k] = y[k] = 0.0;
      if (idx < total) {
        const int ty = idx / kPer, r = idx - ty * kPer, s = r / kStateParamElems;
        state_param_source(tt[ty].s[s], L, r - s * kStateParamElems, x[k], y[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      const int idx = base + k * blockDim.x;
      if (idx < total) {
        const int ty = idx / kPer, r = idx - ty * kPer;
        reinterpret_cast<T*>(tp[ty].s)[r] = (T)(x[k] - y[k]);
      }
    }
  }
  for (int ty = (int)(blockDim.x - 1 - threadIdx.x); ty < ntypes; ty += blockDim.x) fill_type_scalars<T>(tp[ty], tt[ty]);
}

// Elastic energy of one state (state_energy, which also returns D and the stress s) and
// its gradient with respect to the rows of W (state_gradient, from D and s).
// W = M - h0 (rows: edge deviations). F = M^T h0^-T = I + D with
// D[i][k] = sum_j W[j][i] hinv[k][j]; eps = (D + D^T + D^T D)/2;
// s = A eps; E = scale * eps:s / 2; dE/dW[j][i] = scale * sum_k (F S)[i][k] hinv[k][j].
// This is the energy of nanocell_original.py:46-82 / nanocell.py:40-77 and the
// gradient form of nanocell.py:98-132 (stress C_ijkl eps_kl against the
// symmetric strain derivative).
// SIMPLE: every rest matrix is diagonal and every stress map has cubic form
// (A00 = A11 = A22, A01 = A02 = A12 and symmetric, A33 = A44 = A55, all else 0); the
// products with h0^-1 and A then reduce to scalings (detected exactly on the host).
template <typename T, bool SIMPLE = false, typename P = StateParams<T>>
__device__ __forceinline__ T state_energy(const T* __restrict__ W, const P& p, T scale, T (&D)[9], T (&s)[6]) {
  if constexpr (SIMPLE) {
    const T h[3] = {p.hd[0], p.hd[1], p.hd[2]};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) D[i * 3 + k] = W[k * 3 + i] * h[k];
  } else {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      D[i * 3 + k] = W[0 * 3 + i] * p.hinv[k * 3 + 0] + W[1 * 3 + i] * p.hinv[k * 3 + 1] + W[2 * 3 + i] * p.hinv[k * 3 + 2];
  }
  const T h = T(0.5);
  T e[6];
  e[0] = D[0] + h * (D[0] * D[0] + D[3] * D[3] + D[6] * D[6]);
  e[1] = D[4] + h * (D[1] * D[1] + D[4] * D[4] + D[7] * D[7]);
  e[2] = D[8] + h * (D[2] * D[2] + D[5] * D[5] + D[8] * D[8]);
  e[3] = h * (D[5] + D[7] + D[1] * D[2] + D[4] * D[5] + D[7] * D[8]);
  e[4] = h * (D[2] + D[6] + D[0] * D[2] + D[3] * D[5] + D[6] * D[8]);
  e[5] = h * (D[1] + D[3] + D[0] * D[1] + D[3] * D[4] + D[6] * D[7]);
  if constexpr (SIMPLE) {
    const T amb = p.cub[0], b = p.cub[1], c = p.cub[2];
    const T tr = e[0] + e[1] + e[2];
    s[0] = amb * e[0] + b * tr;
    s[1] = amb * e[1] + b * tr;
    s[2] = amb * e[2] + b * tr;
    s[3] = c * e[3];
    s[4] = c * e[4];
    s[5] = c * e[5];
  } else {
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    T acc = T(0);
#pragma unroll
    for (int r = 0; r < 6; ++r) acc += p.A[q * 6 + r] * e[r];
    s[q] = acc;
  }
  }
  const T dens = e[0] * s[0] + e[1] * s[1] + e[2] * s[2] + T(2) * (e[3] * s[3] + e[4] * s[4] + e[5] * s[5]);
  return h * scale * dens;
}

// Gradient with respect to the rows of W from the D and stress s of state_energy.
template <typename T, bool SIMPLE = false, typename P = StateParams<T>>
__device__ __forceinline__ void state_gradient(const T (&D)[9], const T (&s)[6], const P& p, T scale,
                                               T* __restrict__ GW) {
  // S symmetric 3x3 from s
  const T S[9] = {s[0], s[5], s[4], s[5], s[1], s[3], s[4], s[3], s[2]};
  // GF = (I + D) S
  T GF[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int l = 0; l < 3; ++l)
      GF[i * 3 + l] = S[i * 3 + l] + D[i * 3 + 0] * S[0 * 3 + l] + D[i * 3 + 1] * S[1 * 3 + l] + D[i * 3 + 2] * S[2 * 3 + l];
  // GW[j][i] = scale * sum_k GF[i][k] hinv[k][j]
  if constexpr (SIMPLE) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const T sj = scale * p.hd[j];
#pragma unroll
      for (int i = 0; i < 3; ++i) GW[j * 3 + i] = sj * GF[i * 3 + j];
    }
  } else {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      GW[j * 3 + i] = scale * (GF[i * 3 + 0] * p.hinv[0 * 3 + j] + GF[i * 3 + 1] * p.hinv[1 * 3 + j] + GF[i * 3 + 2] * p.hinv[2 * 3 + j]);
  }
}

template <typename T, bool SIMPLE = false, typename P = StateParams<T>>
__device__ __forceinline__ T state_energy_grad(const T* __restrict__ W, const P& p, T scale,
                                               T* __restrict__ GW) {
  T D[9], s[6];
  const T E = state_energy<T, SIMPLE, P>(W, p, scale, D, s);
  state_gradient<T, SIMPLE, P>(D, s, p, scale, GW);
  return E;
}

// Per-cell evaluation. du[b][c]: displacement of the corner with offset bits b.
// Returns the cell energy (multi-state -kT log-sum-exp, micmec/pes/mmff.py:377-398)
// and writes the corner gradient g[b][c] (bits order).
// MODEL 0: single averaged matrix (nanocell_original.py); MODEL 1: eight corner
// matrices (nanocell.py).
template <typename T, int MODEL>
__device__ __forceinline__ double cell_eval(const T (&du)[8][3], const TypeParams<T>& tp, T (&g)[8][3]) {
  // edge displacement differences along d for the 4 edges with lower-corner bits b (bit d clear)
  T ed[3][4][3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      // enumerate the 4 corners with bit d clear
      const int lo = (d == 0) ? (e << 1) : (d == 1 ? ((e & 1) | ((e >> 1) << 2)) : e);
      const int hi = lo | (1 << d);
#pragma unroll
      for (int c = 0; c < 3; ++c) ed[d][e][c] = du[hi][c] - du[lo][c];
    }
  }
  T gacc[8][3];
  double m = 0.0, wsum = 0.0;
  const int ns = tp.nstates;
  for (int s = 0; s < ns; ++s) {
    const StateParams<T>& p = tp.s[s];
    T gs[8][3];
#pragma unroll
    for (int b = 0; b < 8; ++b)
#pragma unroll
      for (int c = 0; c < 3; ++c) gs[b][c] = T(0);
    T Es;
    if (MODEL == 0) {
      T W[9], GW[9];
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          W[d * 3 + c] = p.B[d * 3 + c] + T(0.25) * ((ed[d][0][c] + ed[d][1][c]) + (ed[d][2][c] + ed[d][3][c]));
      Es = state_energy_grad<T>(W, p, p.v0, GW);
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int lo = (d == 0) ? (e << 1) : (d == 1 ? ((e & 1) | ((e >> 1) << 2)) : e);
          const int hi = lo | (1 << d);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const T q = T(0.25) * GW[d * 3 + c];
            gs[hi][c] += q;
            gs[lo][c] -= q;
          }
        }
    } else {
      Es = T(0);
      const T scale = T(0.125) * p.v0;
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        T W[9], GW[9];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int lo = a & ~(1 << d);
          // index of that edge among the 4 along d
          const int e = (d == 0) ? (lo >> 1) : (d == 1 ? ((lo & 1) | ((lo >> 2) << 1)) : (lo & 3));
#pragma unroll
          for (int c = 0; c < 3; ++c) W[d * 3 + c] = p.B[d * 3 + c] + ed[d][e][c];
        }
        Es += state_energy_grad<T>(W, p, scale, GW);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int lo = a & ~(1 << d);
          const int hi = lo | (1 << d);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            gs[hi][c] += GW[d * 3 + c];
            gs[lo][c] -= GW[d * 3 + c];
          }
        }
      }
    }
    const double E = (double)Es + (double)p.df;
    if (s == 0) {
      m = E;
      wsum = 1.0;
#pragma unroll
      for (int b = 0; b < 8; ++b)
#pragma unroll
        for (int c = 0; c < 3; ++c) gacc[b][c] = gs[b][c];
    } else {
      // online -kT log-sum-exp with running minimum m
      const T kT = tp.kT;
      if (E < m) {
        const T r = exp(-(T)(m - E) / kT);  // rescale old terms
        wsum = wsum * (double)r + 1.0;
#pragma unroll
        for (int b = 0; b < 8; ++b)
#pragma unroll
          for (int c = 0; c < 3; ++c) gacc[b][c] = gacc[b][c] * r + gs[b][c];
        m = E;
      } else {
        const T w = exp(-(T)(E - m) / kT);
        wsum += (double)w;
#pragma unroll
        for (int b = 0; b < 8; ++b)
#pragma unroll
          for (int c = 0; c < 3; ++c) gacc[b][c] += w * gs[b][c];
      }
    }
  }
  double Ecell = m;
  if (ns > 1) {
    const T inv = T(1) / (T)wsum;
#pragma unroll
    for (int b = 0; b < 8; ++b)
#pragma unroll
      for (int c = 0; c < 3; ++c) gacc[b][c] *= inv;
    Ecell = m - (double)tp.kT * (double)log((T)wsum);
  }
#pragma unroll
  for (int b = 0; b < 8; ++b)
#pragma unroll
    for (int c = 0; c < 3; ++c) g[b][c] = gacc[b][c];
  return Ecell;
}

// Compensated (error-free TwoSum) FP32 accumulation: a value is the unevaluated
// sum hi + lo. Used for warp-level sums of per-cell and per-node FP32 terms before
// the grid-level reduction continues in FP64.
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);
  return F2{s, err + a.lo + b.lo};
}
template <int NV>
__device__ __forceinline__ void warp_sum_f2(F2 (&v)[NV]) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      F2 o{__shfl_down_sync(0xffffffffu, v[i].hi, off), __shfl_down_sync(0xffffffffu, v[i].lo, off)};
      v[i] = f2_add(v[i], o);
    }
}

// Block sum: compensated FP32 within each warp and across the warps (warp 0 adds the
// warps' (hi, lo) pairs in fixed order). The totals are left in v of thread 0.
// smem must hold NV * (blockDim.x / 32) doubles. Ends without a barrier: a caller
// that reuses smem afterwards synchronises first.
template <int NV>
__device__ __forceinline__ void block_sum_f2_pairs(F2 (&v)[NV], double* smem) {
  warp_sum_f2<NV>(v);
  F2* s2 = reinterpret_cast<F2*>(smem);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) s2[i * nw + wid] = v[i];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = (lane < nw) ? s2[i * nw + lane] : F2{0.0f, 0.0f};
    for (int off = 16; off > 0; off >>= 1) {
      if (off >= nw) continue;
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        F2 o{__shfl_down_sync(0xffffffffu, v[i].hi, off), __shfl_down_sync(0xffffffffu, v[i].lo, off)};
        v[i] = f2_add(v[i], o);
      }
    }
  }
}
// Block sum of 8 compensated values as a reduce-scatter: at each of the first three
// exchanges a lane keeps half of its values and adds its partner's copy of them (4, 2, then
// 1 pair exchanged instead of 8 at every level), so lane l ends with value l >> 2 of its
// warp; then warp w adds the warps' totals of values w, w + nw, ... in warp order. Fixed
// order throughout. emit(i, total) runs on lane 0 of the warp that owns value i.
// smem must hold 8 * (blockDim.x / 32) doubles; blockDim.x is a multiple of 32.
template <typename Emit>
__device__ __forceinline__ void block_scatter_sum8(const F2 (&v)[8], double* smem, Emit emit) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  auto xchg = [](F2 keep, F2 send, int mask) {
    return f2_add(keep, F2{__shfl_xor_sync(0xffffffffu, send.hi, mask), __shfl_xor_sync(0xffffffffu, send.lo, mask)});
  };
  F2 a[4], b[2], c;
  const bool u16 = lane & 16, u8 = lane & 8, u4 = lane & 4;
#pragma unroll
  for (int i = 0; i < 4; ++i) a[i] = xchg(u16 ? v[i + 4] : v[i], u16 ? v[i] : v[i + 4], 16);  // value 4 b4 + i
#pragma unroll
  for (int i = 0; i < 2; ++i) b[i] = xchg(u8 ? a[i + 2] : a[i], u8 ? a[i] : a[i + 2], 8);  // 4 b4 + 2 b3 + i
  c = xchg(u4 ? b[1] : b[0], u4 ? b[0] : b[1], 4);                                          // lane >> 2
  c = xchg(c, c, 2);
  c = xchg(c, c, 1);
  F2* s2 = reinterpret_cast<F2*>(smem);
  if ((lane & 3) == 0) s2[(lane >> 2) * nw + wid] = c;
  __syncthreads();
  for (int i = wid; i < 8; i += nw) {
    F2 t = lane < nw ? s2[i * nw + lane] : F2{0.0f, 0.0f};
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      if (off >= nw) continue;  // the partners hold zeros
      t = f2_add(t, F2{__shfl_down_sync(0xffffffffu, t.hi, off), __shfl_down_sync(0xffffffffu, t.lo, off)});
    }
    if (lane == 0) emit(i, t);
  }
}

// The same with the totals converted to FP64 in thread 0 (one conversion per value).
template <int NV>
__device__ __forceinline__ void block_sum_f2(F2 (&v)[NV], double (&out)[NV], double* smem) {
  block_sum_f2_pairs<NV>(v, smem);
  if (threadIdx.x == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) out[i] = (double)v[i].hi + (double)v[i].lo;
}

// Per-block partial sums in global memory, one 8-byte slot per value, value-major
// (slot v * nblocks + block): FP64 kernels store doubles, FP32 kernels the compensated
// pair (hi, lo) as two floats. Readers of other blocks' slots (after a fence and a
// ticket) load through L2.
__device__ __forceinline__ void store_pair(double* slot, F2 v) {
  *reinterpret_cast<float2*>(slot) = make_float2(v.hi, v.lo);
}
__device__ __forceinline__ F2 load_pair(const double* slot) {
  const float2 p = __ldcg(reinterpret_cast<const float2*>(slot));
  return F2{p.x, p.y};
}

// Totals of per-block partials (value-major: slot v * na + k of a, v * nb + k of b, for
// block k, so the lanes of a warp read consecutive slots) summed by one
// block in a fixed order: warp w sums values w, w + nw, ...; its lanes stride over the
// blocks, then a fixed shuffle tree. PAIRS: the slots hold compensated FP32 pairs,
// summed in compensated FP32 and converted to FP64 once; else doubles summed in FP64.
// Results in out_s (shared, NA + NB doubles), valid for every thread after the closing
// barrier.
template <int NA, int NB, bool PAIRS>
__device__ __forceinline__ void sum_partials_by_warp(const double* a, int na, const double* b, int nb,
                                                     double* out_s) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int v = wid; v < NA + NB; v += nw) {
    const bool first = v < NA;
    const double* base = first ? a + (size_t)v * na : b + (size_t)(v - NA) * nb;
    const int n = first ? na : nb;
    if constexpr (PAIRS) {
      F2 acc{0.0f, 0.0f};
#pragma unroll 8
      for (int k = lane; k < n; k += 32) acc = f2_add(acc, load_pair(base + k));
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const F2 o{__shfl_down_sync(0xffffffffu, acc.hi, off), __shfl_down_sync(0xffffffffu, acc.lo, off)};
        acc = f2_add(acc, o);
      }
      if (lane == 0) out_s[v] = (double)acc.hi + (double)acc.lo;
    } else {
      double acc = 0.0;
#pragma unroll 8
      for (int k = lane; k < n; k += 32) acc += __ldcg(base + k);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
      if (lane == 0) out_s[v] = acc;
    }
  }
  __syncthreads();
}

// IEEE 754 binary64 <-> binary32 conversions built from the bit layouts with integer
// operations only (the FP64 pipe of this part is narrow and hardware conversions queue
// there). d2f_rn rounds to nearest, ties to even, including subnormal results and
// overflow to infinity; every NaN becomes the canonical NaN 0x7fffffff. f2d is exact.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const unsigned e = (hi >> 20) & 0x7FFu;  // binary32 exponent field = e - 896
  unsigned f;
  if (e - 897u <= 253u) {  // normal binary32 result (before rounding)
    f = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1FFFFFFFu, halfway = 0x10000000u;
    f += (unsigned)(rem > halfway) | ((unsigned)(rem == halfway) & (f & 1u));  // a carry bumps the exponent
  } else if (e >= 1151u) {  // too large, infinity or NaN
    f = (e == 2047u && (((hi & 0xFFFFFu) | lo) != 0u)) ? 0x7FFFFFFFu : 0x7F800000u;
    if (f == 0x7FFFFFFFu) return __uint_as_float(f);
  } else if (e < 873u) {  // below half the smallest subnormal: zero
    f = 0u;
  } else {  // subnormal binary32: value = m * 2^(e - 1075), bits = round(m >> (926 - e))
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const unsigned sh = 926u - e;  // 30 .. 53
    const unsigned long long q = m >> sh, rem = m & ((1ull << sh) - 1ull), halfway = 1ull << (sh - 1u);
    f = (unsigned)q + ((unsigned)(rem > halfway) | ((unsigned)(rem == halfway) & ((unsigned)q & 1u)));
  }
  return __uint_as_float(sign | f);
}
__device__ __forceinline__ double f2d(float x) {
  const unsigned f = __float_as_uint(x);
  const unsigned sign = f & 0x80000000u, e = (f >> 23) & 0xFFu, m = f & 0x7FFFFFu;
  unsigned hi, lo;
  if (e - 1u <= 253u) {  // normal
    hi = sign | ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  } else if (e == 255u) {  // infinity, NaN (payload kept)
    hi = sign | 0x7FF00000u | (m >> 3);
    lo = m << 29;
  } else if (m == 0u) {  // zero
    hi = sign;
    lo = 0u;
  } else {  // subnormal: m * 2^-149 with the leading bit at position p
    const int p = 31 - __clz((int)m);
    const unsigned long long frac = ((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull;
    hi = sign | ((unsigned)(p + 874) << 20) | (unsigned)(frac >> 32);
    lo = (unsigned)frac;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// exp(d / kT) for d <= 0 and log(w) of the state combination. FP32: exp2 of d log2(e)/kT
// (no division) and log2 times ln 2; FP64: exp and log.
template <typename T>
__device__ __forceinline__ T lse_weight(T d, T kT, T lkT) {
  if constexpr (sizeof(T) == 4) return exp2f(d * lkT);
  else return exp(d / kT);
}
template <typename T>
__device__ __forceinline__ T lse_log(T w) {
  if constexpr (sizeof(T) == 4) return log2f(w) * 0.69314718055994531f;
  else return log(w);
}

// n / d for 0 <= n < 2^31 by a multiply-high and a shift (Granlund and Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994, section 4):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(m, n) + n) >> l.
struct FastDiv {
  uint32_t m, l;
};
inline FastDiv make_fastdiv(uint32_t d) {
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  const unsigned long long m = ((1ull << 32) * ((1ull << l) - d)) / d + 1ull;
  return FastDiv{(uint32_t)m, l};
}
__device__ __forceinline__ int fdiv(int n, FastDiv f) { return (int)((__umulhi((uint32_t)n, f.m) + (uint32_t)n) >> f.l); }

// The part of StateParams the cubic form reads, loaded with four 16-byte shared-memory
// loads (FP32: B[9], v0, df, hd[3], cub[3] are the first 17 of 20 aligned floats).
template <typename T>
struct CubicView {
  T B[9];
  T v0, df;
  T hd[3];
  T cub[3];
};
__device__ __forceinline__ void load_cubic(const StateParams<float>& p, CubicView<float>& c) {
  const float4* q = reinterpret_cast<const float4*>(&p);
  const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
  const float q4 = p.cub[2];
  c.B[0] = q0.x; c.B[1] = q0.y; c.B[2] = q0.z; c.B[3] = q0.w;
  c.B[4] = q1.x; c.B[5] = q1.y; c.B[6] = q1.z; c.B[7] = q1.w;
  c.B[8] = q2.x; c.v0 = q2.y; c.df = q2.z; c.hd[0] = q2.w;
  c.hd[1] = q3.x; c.hd[2] = q3.y; c.cub[0] = q3.z; c.cub[1] = q3.w;
  c.cub[2] = q4;
}
static_assert(offsetof(StateParams<float>, B) == 0 && offsetof(StateParams<float>, v0) == 36 &&
                  offsetof(StateParams<float>, df) == 40 && offsetof(StateParams<float>, hd) == 44 &&
                  offsetof(StateParams<float>, cub) == 56,
              "load_cubic assumes this layout");

// Eight lanes per cell (eight-corner-matrix model). Lane a (corner offset bits) of an
// aligned 8-lane group holds the displacement du of vertex a; it evaluates corner
// matrix a for every state of the cell's type. Edges to the neighbours a^1, a^2,
// a^4 come from xor-shuffles; state energies are summed over the group; vertex a's
// gradient collects the row-d gradients of matrices a and a^(1<<d) (the same edge).
// All 32 lanes of the warp must call this together (the state loop runs to the
// warp's largest state count). Returns the cell energy (same in the 8 lanes) and
// the gradient g of vertex a.
template <typename T, bool SIMPLE = false>
__device__ __forceinline__ T cell8_eval(const T (&du)[3], int a, const TypeParams<T>& tpl, bool valid, T (&g)[3]) {
  // edge (vertex a -> neighbour a^(1<<d)) displacement differences, oriented lo -> hi
  T ed[3][3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const bool hi = (a >> d) & 1;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const T other = __shfl_xor_sync(0xffffffffu, du[x], 1 << d);
      ed[d][x] = hi ? du[x] - other : other - du[x];
    }
  }
  const int ns_lane = valid ? tpl.nstates : 1;
  const int ns = __reduce_max_sync(0xffffffffu, ns_lane);
  const T kT = tpl.kT;
  struct NoView {};
  typedef typename std::conditional<SIMPLE && sizeof(T) == 4, CubicView<float>, NoView>::type View;
  // energy part of state p: strain and stress of matrix a (Dm, sv), the cell's elastic
  // energy summed over the group, plus the state's free energy
  auto energy = [&](const StateParams<T>& p, View& cv, T (&Dm)[9], T (&sv)[6]) -> T {
    T W[9], Es, df;
    if constexpr (SIMPLE && sizeof(T) == 4) {
      load_cubic(p, cv);
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int x = 0; x < 3; ++x) W[d * 3 + x] = cv.B[d * 3 + x] + ed[d][x];
      Es = state_energy<T, true, CubicView<float>>(W, cv, T(0.125) * cv.v0, Dm, sv);
      df = cv.df;
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int x = 0; x < 3; ++x) W[d * 3 + x] = p.B[d * 3 + x] + ed[d][x];
      Es = state_energy<T, SIMPLE>(W, p, T(0.125) * p.v0, Dm, sv);
      df = p.df;
    }
    Es += __shfl_xor_sync(0xffffffffu, Es, 1);
    Es += __shfl_xor_sync(0xffffffffu, Es, 2);
    Es += __shfl_xor_sync(0xffffffffu, Es, 4);
    return Es + df;
  };
  // row gradients of matrix a in state p from the energy part's Dm, sv
  auto gradient = [&](const StateParams<T>& p, const View& cv, const T (&Dm)[9], const T (&sv)[6], T* GW) {
    if constexpr (SIMPLE && sizeof(T) == 4) state_gradient<T, true, CubicView<float>>(Dm, sv, cv, T(0.125) * cv.v0, GW);
    else state_gradient<T, SIMPLE>(Dm, sv, p, T(0.125) * p.v0, GW);
  };
  // state-weighted row gradients of matrix a (online -kT log-sum-exp weights); the
  // exchange with the neighbouring matrices happens once, after the state loop. The
  // first state (every lane has one) starts the running minimum m and the sums.
  T Gacc[9];
  T m, wsum = T(1);
  {
    View cv;
    T Dm[9], sv[6];
    m = energy(tpl.s[0], cv, Dm, sv);
    gradient(tpl.s[0], cv, Dm, sv, Gacc);
  }
  for (int s = 1; s < ns; ++s) {
    const bool active = s < ns_lane;
    const StateParams<T>& p = tpl.s[active ? s : 0];
    View cv;
    T Dm[9], sv[6];
    const T E = energy(p, cv, Dm, sv);
    // A state whose weight against the lowest energy so far is below e^-50 adds nothing
    // representable to the weighted gradient (nor to the weight sum): its gradient is not
    // formed. The lowest energy can only fall later, so the weight stays below e^-50.
    if (active && !(E - m >= T(50) * kT)) {
      T GW[9];
      gradient(p, cv, Dm, sv, GW);
      if (E < m) {
        const T r = lse_weight<T>(E - m, kT, tpl.lkT);
        wsum = wsum * r + T(1);
#pragma unroll
        for (int i = 0; i < 9; ++i) Gacc[i] = Gacc[i] * r + GW[i];
        m = E;
      } else {
        const T w = lse_weight<T>(m - E, kT, tpl.lkT);
        wsum += w;
#pragma unroll
        for (int i = 0; i < 9; ++i) Gacc[i] += w * GW[i];
      }
    }
  }
  // vertex a's gradient: row d of matrix a and of matrix a^(1<<d) (the same edge)
  g[0] = g[1] = g[2] = T(0);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const T sg = ((a >> d) & 1) ? T(1) : T(-1);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      const T mine = Gacc[d * 3 + x];
      g[x] += sg * (mine + __shfl_xor_sync(0xffffffffu, mine, 1 << d));
    }
  }
  T Ecell = m;
  if (ns_lane > 1) {
    T inv;
    if constexpr (sizeof(T) == 4) inv = __frcp_rn(wsum);
    else inv = T(1) / wsum;
#pragma unroll
    for (int x = 0; x < 3; ++x) g[x] *= inv;
    Ecell = m - kT * lse_log<T>(wsum);
  }
  return Ecell;
}

// ---------------------------------------------------------------- one thread per cell
// The eight-corner-matrix model evaluated by one thread for a whole cell: du[b][x] is the
// displacement of the corner with offset bits b. A state's energy sums the eight corner
// matrices; the gradient of corner matrix a adds its row d to vertex a | bit d and
// subtracts it from vertex a & ~bit d (the two ends of that row's edge). No lane exchanges
// are needed, and the cell's gradient and vertices stay in the thread's registers.

template <typename T, bool SIMPLE>
struct StateView;  // the part of a state's parameters the thread keeps in registers
template <>
struct StateView<float, true> {
  CubicView<float> v;
  __device__ __forceinline__ void load(const StateParams<float>& p) { load_cubic(p, v); }
  __device__ __forceinline__ const CubicView<float>& params(const StateParams<float>&) const { return v; }
  __device__ __forceinline__ float B(const StateParams<float>&, int i) const { return v.B[i]; }
  __device__ __forceinline__ float v0(const StateParams<float>&) const { return v.v0; }
  __device__ __forceinline__ float df(const StateParams<float>&) const { return v.df; }
};
template <typename T, bool SIMPLE>
struct StateView {  // parameters read from shared memory where they are used
  __device__ __forceinline__ void load(const StateParams<T>&) {}
  __device__ __forceinline__ const StateParams<T>& params(const StateParams<T>& p) const { return p; }
  __device__ __forceinline__ T B(const StateParams<T>& p, int i) const { return p.B[i]; }
  __device__ __forceinline__ T v0(const StateParams<T>& p) const { return p.v0; }
  __device__ __forceinline__ T df(const StateParams<T>& p) const { return p.df; }
};

// Corner matrix a of a cell minus the rest matrix: row d = B_d + du[a | bit d] - du[a & ~bit d].
template <typename T, bool SIMPLE>
__device__ __forceinline__ void corner_w(const T (&du)[8][3], int a, const StateView<T, SIMPLE>& sv,
                                         const StateParams<T>& p, T (&W)[9]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int hi = a | (1 << d), lo = a & ~(1 << d);
#pragma unroll
    for (int c = 0; c < 3; ++c) W[d * 3 + c] = sv.B(p, d * 3 + c) + (du[hi][c] - du[lo][c]);
  }
}

// Energy of one state summed over the eight corner matrices (scale det(h0) / 8), plus its
// free energy.
template <typename T, bool SIMPLE>
__device__ __forceinline__ T cell_state_energy(const T (&du)[8][3], const StateParams<T>& p) {
  StateView<T, SIMPLE> sv;
  sv.load(p);
  const T scale = T(0.125) * sv.v0(p);
  T E = T(0);
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    T W[9], D[9], st[6];
    corner_w<T, SIMPLE>(du, a, sv, p, W);
    E += state_energy<T, SIMPLE>(W, sv.params(p), scale, D, st);
  }
  return E + sv.df(p);
}

// The same, and the state's gradient times `weight` added to the vertex gradients g.
template <typename T, bool SIMPLE>
__device__ __forceinline__ T cell_state_energy_grad(const T (&du)[8][3], const StateParams<T>& p, T weight,
                                                    T (&g)[8][3]) {
  StateView<T, SIMPLE> sv;
  sv.load(p);
  const T scale = T(0.125) * sv.v0(p);
  const T gscale = scale * weight;
  T E = T(0);
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    T W[9], D[9], st[6], GW[9];
    corner_w<T, SIMPLE>(du, a, sv, p, W);
    E += state_energy<T, SIMPLE>(W, sv.params(p), scale, D, st);
    state_gradient<T, SIMPLE>(D, st, sv.params(p), gscale, GW);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int hi = a | (1 << d), lo = a & ~(1 << d);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        g[hi][c] += GW[d * 3 + c];
        g[lo][c] -= GW[d * 3 + c];
      }
    }
  }
  return E + sv.df(p);
}

// The averaged-matrix model (nanocell_original.py:46-132) by one thread: the cell matrix
// minus the rest matrix has rows W_d = B_d + (sum of the four edge vectors along d) / 4;
// the energy is that of one strain with scale det(h0), and row d of its gradient is spread
// over the four edges along d with weight 1/4.
template <typename T, bool SIMPLE>
__device__ __forceinline__ void average_w(const T (&du)[8][3], const StateView<T, SIMPLE>& sv, const StateParams<T>& p,
                                          T (&W)[9]) {
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T e = T(0);
#pragma unroll
      for (int lo = 0; lo < 8; ++lo)
        if (!((lo >> d) & 1)) e += du[lo | (1 << d)][c] - du[lo][c];
      W[d * 3 + c] = sv.B(p, d * 3 + c) + T(0.25) * e;
    }
}

template <typename T, bool SIMPLE>
__device__ __forceinline__ T avg_state_energy(const T (&du)[8][3], const StateParams<T>& p) {
  StateView<T, SIMPLE> sv;
  sv.load(p);
  T W[9], D[9], st[6];
  average_w<T, SIMPLE>(du, sv, p, W);
  return state_energy<T, SIMPLE>(W, sv.params(p), sv.v0(p), D, st) + sv.df(p);
}

template <typename T, bool SIMPLE>
__device__ __forceinline__ T avg_state_energy_grad(const T (&du)[8][3], const StateParams<T>& p, T weight,
                                                   T (&g)[8][3]) {
  StateView<T, SIMPLE> sv;
  sv.load(p);
  T W[9], D[9], st[6], GW[9];
  average_w<T, SIMPLE>(du, sv, p, W);
  const T E = state_energy<T, SIMPLE>(W, sv.params(p), sv.v0(p), D, st);
  state_gradient<T, SIMPLE>(D, st, sv.params(p), T(0.25) * sv.v0(p) * weight, GW);
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int lo = 0; lo < 8; ++lo)
      if (!((lo >> d) & 1))
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          g[lo | (1 << d)][c] += GW[d * 3 + c];
          g[lo][c] -= GW[d * 3 + c];
        }
  return E + sv.df(p);
}

// Energy (with free energy) of one state of a cell, MODEL 0 averaged matrix, 1 eight
// corner matrices; and the same with the state's gradient times `weight` added to g.
template <typename T, int MODEL, bool SIMPLE>
__device__ __forceinline__ T model_state_energy(const T (&du)[8][3], const StateParams<T>& p) {
  if constexpr (MODEL == 0) return avg_state_energy<T, SIMPLE>(du, p);
  else return cell_state_energy<T, SIMPLE>(du, p);
}
template <typename T, int MODEL, bool SIMPLE>
__device__ __forceinline__ T model_state_energy_grad(const T (&du)[8][3], const StateParams<T>& p, T weight,
                                                     T (&g)[8][3]) {
  if constexpr (MODEL == 0) return avg_state_energy_grad<T, SIMPLE>(du, p, weight, g);
  else return cell_state_energy_grad<T, SIMPLE>(du, p, weight, g);
}

// Cell energy (multi-state -kT log-sum-exp, micmec/pes/mmff.py:377-398) and vertex
// gradients g (offset-bits order) of one cell, evaluated by one thread. State 0's energy
// and gradient come from one pass over the corners, the other states' energies from one
// pass each. Then the weights: a state whose weight is below e^-50 forms no gradient (the
// lowest energy is known by then, and usually every state but one is that far up); state
// 0's gradient is rescaled by its weight, and the other states are evaluated again with
// their weight folded into the gradient scale.
template <typename T, bool SIMPLE, int MODEL = 1>
__device__ __forceinline__ T cell1_eval(const T (&du)[8][3], const TypeParams<T>& p, T (&g)[8][3]) {
#pragma unroll
  for (int b = 0; b < 8; ++b)
#pragma unroll
    for (int x = 0; x < 3; ++x) g[b][x] = T(0);
  T Ecell = model_state_energy_grad<T, MODEL, SIMPLE>(du, p.s[0], T(1), g);
  const int ns = p.nstates;
  if (ns > 1) {
    T E[MM_MAX_STATES];
    E[0] = Ecell;
    T m = Ecell;
    for (int s = 1; s < ns; ++s) {
      E[s] = model_state_energy<T, MODEL, SIMPLE>(du, p.s[s]);
      m = E[s] < m ? E[s] : m;
    }
    const T kT = p.kT;
    T wsum = T(0), w0 = T(0);
    for (int s = 0; s < ns; ++s) {
      const T w = (E[s] - m >= T(50) * kT) ? T(0) : lse_weight<T>(m - E[s], kT, p.lkT);
      wsum += w;
      if (s == 0) w0 = w;
    }
    T inv;
    if constexpr (sizeof(T) == 4) inv = __frcp_rn(wsum);
    else inv = T(1) / wsum;
    const T f0 = w0 * inv;
#pragma unroll
    for (int b = 0; b < 8; ++b)
#pragma unroll
      for (int x = 0; x < 3; ++x) g[b][x] *= f0;
    for (int s = 1; s < ns; ++s)
      if (E[s] - m < T(50) * kT)
        model_state_energy_grad<T, MODEL, SIMPLE>(du, p.s[s], lse_weight<T>(m - E[s], kT, p.lkT) * inv, g);
    Ecell = m - kT * lse_log<T>(wsum);
  }
  return Ecell;
}

// ---------------------------------------------------------------- reductions

template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV]) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
}

// Deterministic block sum of NV doubles; result valid in thread 0.
// smem must hold NV * (blockDim.x / 32) doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem) {
  warp_sum<NV>(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) smem[i * nw + wid] = v[i];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = (lane < nw) ? smem[i * nw + lane] : 0.0;
    warp_sum<NV>(v);
  }
  __syncthreads();
}

// ---------------------------------------------------------------- random numbers
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11),
// restated from the published round function and constants.
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    // both halves of each 32 x 32 -> 64-bit product from one wide multiply
    const uint64_t p0 = (uint64_t)M0 * ctr.x, p1 = (uint64_t)M1 * ctr.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    ctr = U4{hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Uniform in (0, 1) from the top 23 bits of a 32-bit word: 1 + m 2^-23 in [1, 2) built
// from its bit pattern, minus (1 - 2^-24) (exact), so u = (m + 1/2) 2^-23. Integer and
// FP32 add only (no conversion instruction).
__device__ __forceinline__ float uniform_open(uint32_t w) {
  return __uint_as_float(0x3f800000u | (w >> 9)) - 0.99999994f;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Three standard normals for (node, step, call) via Box-Muller on Philox output.
__device__ __forceinline__ void normal3(uint64_t seed, uint32_t node, uint32_t step, uint32_t call, float (&z)[3]) {
  U4 r = philox4x32_10(U4{node, step, call, 0x4d4d4543u}, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float u1 = uniform_open(r.x), u2 = uniform_open(r.y), u3 = uniform_open(r.z), u4 = uniform_open(r.w);
  // Box-Muller with the hardware approximations of log2, sqrt, sin and cos (absolute
  // errors ~1e-6 on these ranges, far below what the thermostat's statistics resolve);
  // angles 2 pi (u - 1/2) in [-pi, pi), where those approximations are most accurate; the
  // clamp keeps an approximate log of u ~ 1 from turning -2 log u negative. The radius is
  // at most sqrt(-2 ln 2^-24) = 5.8 (the normal's mass beyond it is 8e-9).
  const float r1 = sqrt_approx(fmaxf(-2.0f * __logf(u1), 0.0f)), r2 = sqrt_approx(fmaxf(-2.0f * __logf(u3), 0.0f));
  const float twopi = 6.2831853071795865f;
  float s1, c1;
  __sincosf(twopi * (u2 - 0.5f), &s1, &c1);
  z[0] = r1 * c1;
  z[1] = r1 * s1;
  z[2] = r2 * __cosf(twopi * (u4 - 0.5f));
}

}  // namespace mm
