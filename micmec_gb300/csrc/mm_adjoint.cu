// Adjoint of the force evaluation: parameter gradients, Hessian-vector products and
// their mixed derivatives, in FP64.
//
// One thread per cell evaluates, in forward-mode dual numbers (value + tangent along
// a caller-given node displacement field lam and lattice-matrix tangent dL):
//   * the cell energy, its corner gradient (value: forces; tangent: (H lam) terms),
//   * the gradient of the cell energy with respect to its type's parameters for every
//     state: the 6x6 stress map A (36), the rest matrix h0 (9) and the state free
//     energy (1). Value: dE/dtheta; tangent: d/dtheta (lam . dE/dx), the mixed
//     derivative a loss on forces needs.
// The energy model is the reference's (nanocell.py:40-132 / nanocell_original.py:46-132,
// multi-state combination mmff.py:377-398); derivatives with respect to h0 go through
// h0^-1 (dh0^-1 = -h0^-1 dh0 h0^-1), det h0 (ddet = det h0^-T) and B = L - h0.
// Node quantities are gathered in corner order (no atomics); parameter gradients are
// summed per (type, state) over cells in a fixed order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/micmec_gb300.h"
#include "mm_device.cuh"
#include "mm_handle.h"

using namespace mm;

namespace {

struct Dual {
  double v, d;
};
__device__ __forceinline__ Dual mk(double v, double d = 0.0) { return Dual{v, d}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual{-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator*(double s, Dual b) { return Dual{s * b.v, s * b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double s) { return Dual{s * a.v, s * a.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual{q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) {
  a.v += b.v;
  a.d += b.d;
  return a;
}
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) {
  a.v -= b.v;
  a.d -= b.d;
  return a;
}
__device__ __forceinline__ Dual dexp(Dual a) {
  const double e = exp(a.v);
  return Dual{e, e * a.d};
}
__device__ __forceinline__ Dual dlog(Dual a) { return Dual{log(a.v), a.d / a.v}; }

constexpr int kAdjThreads = 128;
constexpr int kPG = 46;  // per state: A (36), h0 (9), free energy (1)
constexpr int kAdjPart = 20;  // energy (2) + virial value/tangent (18)

// One state of one corner matrix (or of the averaged matrix): energy, dE/dW, and
// accumulation of dE/dA and dE/dhinv (all in duals).
__device__ __forceinline__ Dual state_adj(const Dual* W, const StateTable& p, double scale, Dual* GW, Dual* dA,
                                          Dual* dhinv) {
  Dual D[9];
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) D[i * 3 + k] = W[i] * p.hinv[k * 3] + W[3 + i] * p.hinv[k * 3 + 1] + W[6 + i] * p.hinv[k * 3 + 2];
  Dual e[6];
  e[0] = D[0] + 0.5 * (D[0] * D[0] + D[3] * D[3] + D[6] * D[6]);
  e[1] = D[4] + 0.5 * (D[1] * D[1] + D[4] * D[4] + D[7] * D[7]);
  e[2] = D[8] + 0.5 * (D[2] * D[2] + D[5] * D[5] + D[8] * D[8]);
  e[3] = 0.5 * (D[5] + D[7] + D[1] * D[2] + D[4] * D[5] + D[7] * D[8]);
  e[4] = 0.5 * (D[2] + D[6] + D[0] * D[2] + D[3] * D[5] + D[6] * D[8]);
  e[5] = 0.5 * (D[1] + D[3] + D[0] * D[1] + D[3] * D[4] + D[6] * D[7]);
  Dual s[6];
  for (int q = 0; q < 6; ++q) {
    Dual acc = mk(0.0);
    for (int r = 0; r < 6; ++r) acc += p.A[q * 6 + r] * e[r];
    s[q] = acc;
  }
  const double w[6] = {1, 1, 1, 2, 2, 2};
  Dual dens = mk(0.0);
  for (int q = 0; q < 6; ++q) dens += w[q] * (e[q] * s[q]);
  for (int q = 0; q < 6; ++q)
    for (int r = 0; r < 6; ++r) dA[q * 6 + r] += (0.5 * scale * w[q]) * (e[q] * e[r]);
  const Dual S[9] = {s[0], s[5], s[4], s[5], s[1], s[3], s[4], s[3], s[2]};
  Dual GF[9];
  for (int i = 0; i < 3; ++i)
    for (int l = 0; l < 3; ++l)
      GF[i * 3 + l] = S[i * 3 + l] + D[i * 3] * S[l] + D[i * 3 + 1] * S[3 + l] + D[i * 3 + 2] * S[6 + l];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i)
      GW[j * 3 + i] = scale * (GF[i * 3] * p.hinv[j] + GF[i * 3 + 1] * p.hinv[3 + j] + GF[i * 3 + 2] * p.hinv[6 + j]);
  // dE/dhinv[k][j] = scale * sum_i GF[i][k] W[j][i]
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      dhinv[k * 3 + j] += scale * (GF[k] * W[j * 3] + GF[3 + k] * W[j * 3 + 1] + GF[6 + k] * W[j * 3 + 2]);
  return (0.5 * scale) * dens;
}

struct AdjTopo {
  int N, M, structured, nx, ny, nz;
  const int32_t* cell_nodes;
  const int32_t* node_cells;
  const int32_t* node_lat;
  const uint8_t* cell_type;
};

template <int MODEL, bool STRUCT>
__global__ void __launch_bounds__(kAdjThreads) k_cells_adj(AdjTopo t, const TypeTable* __restrict__ tt,
                                                           const double* __restrict__ box, const double* __restrict__ dbox,
                                                           const double* __restrict__ u, const double* __restrict__ lam,
                                                           double* __restrict__ G, double* __restrict__ Gt,
                                                           double* __restrict__ P, double* __restrict__ cpart) {
  __shared__ double red[kAdjPart * (kAdjThreads / 32)];
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[kAdjPart];
  for (int i = 0; i < kAdjPart; ++i) acc[i] = 0.0;
  if (cell < t.M) {
    Dual du[8][3];
    for (int kc = 0; kc < 8; ++kc) {
      const int b = corner_to_bits(kc);
      int node;
      if (STRUCT) {
        const int nyz = t.ny * t.nz, i = cell / nyz, r = cell - i * nyz, j = r / t.nz, k = r - j * t.nz;
        int a0 = i + (b & 1), b0 = j + ((b >> 1) & 1), c0 = k + (b >> 2);
        a0 = a0 == t.nx ? 0 : a0;
        b0 = b0 == t.ny ? 0 : b0;
        c0 = c0 == t.nz ? 0 : c0;
        node = (a0 * t.ny + b0) * t.nz + c0;
      } else {
        node = t.cell_nodes[kc * t.M + cell];
      }
      for (int x = 0; x < 3; ++x) du[b][x] = mk(u[x * t.N + node], lam ? lam[3 * node + x] : 0.0);
    }
    Dual L[9];
    for (int i = 0; i < 9; ++i) L[i] = mk(box[i], dbox ? dbox[i] : 0.0);
    const int ty = t.cell_type[cell];
    const TypeTable& T = tt[ty];
    // edge differences
    Dual ed[3][4][3];
    for (int d = 0; d < 3; ++d)
      for (int e = 0; e < 4; ++e) {
        const int lo = (d == 0) ? (e << 1) : (d == 1 ? ((e & 1) | ((e >> 1) << 2)) : e);
        const int hi = lo | (1 << d);
        for (int x = 0; x < 3; ++x) ed[d][e][x] = du[hi][x] - du[lo][x];
      }
    Dual Es[MM_MAX_STATES];
    Dual gs[MM_MAX_STATES][8][3];
    Dual pg[MM_MAX_STATES][kPG];
    const int ns = T.nstates;
    for (int s = 0; s < ns; ++s) {
      const StateTable& p = T.s[s];
      for (int b = 0; b < 8; ++b)
        for (int x = 0; x < 3; ++x) gs[s][b][x] = mk(0.0);
      Dual dA[36], dhinv[9], dB[9];
      for (int i = 0; i < 36; ++i) dA[i] = mk(0.0);
      for (int i = 0; i < 9; ++i) dhinv[i] = dB[i] = mk(0.0);
      Dual B[9];
      for (int i = 0; i < 9; ++i) B[i] = L[i] - mk(p.h0[i]);
      Dual E = mk(0.0);
      if (MODEL == 0) {
        Dual W[9], GW[9];
        for (int d = 0; d < 3; ++d)
          for (int x = 0; x < 3; ++x)
            W[d * 3 + x] = B[d * 3 + x] + 0.25 * ((ed[d][0][x] + ed[d][1][x]) + (ed[d][2][x] + ed[d][3][x]));
        E = state_adj(W, p, p.v0, GW, dA, dhinv);
        for (int i = 0; i < 9; ++i) dB[i] += GW[i];
        for (int d = 0; d < 3; ++d)
          for (int e = 0; e < 4; ++e) {
            const int lo = (d == 0) ? (e << 1) : (d == 1 ? ((e & 1) | ((e >> 1) << 2)) : e);
            const int hi = lo | (1 << d);
            for (int x = 0; x < 3; ++x) {
              gs[s][hi][x] += 0.25 * GW[d * 3 + x];
              gs[s][lo][x] -= 0.25 * GW[d * 3 + x];
            }
          }
      } else {
        for (int a = 0; a < 8; ++a) {
          Dual W[9], GW[9];
          for (int d = 0; d < 3; ++d) {
            const int lo = a & ~(1 << d);
            const int e = (d == 0) ? (lo >> 1) : (d == 1 ? ((lo & 1) | ((lo >> 2) << 1)) : (lo & 3));
            for (int x = 0; x < 3; ++x) W[d * 3 + x] = B[d * 3 + x] + ed[d][e][x];
          }
          E += state_adj(W, p, 0.125 * p.v0, GW, dA, dhinv);
          for (int i = 0; i < 9; ++i) dB[i] += GW[i];
          for (int d = 0; d < 3; ++d) {
            const int lo = a & ~(1 << d), hi = lo | (1 << d);
            for (int x = 0; x < 3; ++x) {
              gs[s][hi][x] += GW[d * 3 + x];
              gs[s][lo][x] -= GW[d * 3 + x];
            }
          }
        }
      }
      // dE/dh0 = -dE/dB - hinv^T dE/dhinv hinv^T + E_elastic hinv^T
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          Dual acc2 = mk(0.0);
          for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) acc2 += (p.hinv[k * 3 + i] * p.hinv[j * 3 + l]) * dhinv[k * 3 + l];
          pg[s][36 + i * 3 + j] = -dB[i * 3 + j] - acc2 + E * p.hinv[j * 3 + i];
        }
      for (int i = 0; i < 36; ++i) pg[s][i] = dA[i];
      Es[s] = E + mk(p.df);
    }
    // -kT log-sum-exp over states (mmff.py:388-398), weights in duals
    Dual Emin = Es[0];
    for (int s = 1; s < ns; ++s)
      if (Es[s].v < Emin.v) Emin = Es[s];
    Dual wsum = mk(0.0), wts[MM_MAX_STATES];
    for (int s = 0; s < ns; ++s) {
      wts[s] = dexp(-(Es[s] - Emin) / mk(T.kT));
      wsum += wts[s];
    }
    Dual Ecell = Emin - mk(T.kT) * dlog(wsum);
    for (int s = 0; s < ns; ++s) wts[s] = wts[s] / wsum;
    Dual g[8][3];
    for (int b = 0; b < 8; ++b)
      for (int x = 0; x < 3; ++x) {
        Dual a0 = mk(0.0);
        for (int s = 0; s < ns; ++s) a0 += wts[s] * gs[s][b][x];
        g[b][x] = a0;
      }
    for (int kc = 0; kc < 8; ++kc) {
      const int b = corner_to_bits(kc);
      for (int x = 0; x < 3; ++x) {
        G[(kc * 3 + x) * (size_t)t.M + cell] = g[b][x].v;
        Gt[(kc * 3 + x) * (size_t)t.M + cell] = g[b][x].d;
      }
    }
    // parameter gradients of the cell energy: weights times state gradients; dE/d(free energy) = weight
    // (not stored when the caller asked for no parameter gradients, e.g. Hessian products)
    if (P)
    for (int s = 0; s < MM_MAX_STATES; ++s)
      for (int k = 0; k < kPG; ++k) {
        Dual val = mk(0.0);
        if (s < ns) val = (k == 45) ? wts[s] : wts[s] * pg[s][k];
        const size_t idx = ((size_t)(s * kPG + k) * 2) * t.M + cell;
        P[idx] = val.v;
        P[idx + t.M] = val.d;
      }
    acc[0] = Ecell.v;
    acc[1] = Ecell.d;
    // virial sum_b g_b (x) (offset(b) . L + du_b - du_0), value and tangent
    for (int b = 1; b < 8; ++b)
      for (int y = 0; y < 3; ++y) {
        Dual r = du[b][y] - du[0][y];
        if (b & 1) r += L[0 * 3 + y];
        if (b & 2) r += L[1 * 3 + y];
        if (b & 4) r += L[2 * 3 + y];
        for (int x = 0; x < 3; ++x) {
          const Dual vt = g[b][x] * r;
          acc[2 + x * 3 + y] += vt.v;
          acc[11 + x * 3 + y] += vt.d;
        }
      }
  }
  block_sum<kAdjPart>(acc, red);
  if (threadIdx.x == 0)
    for (int i = 0; i < kAdjPart; ++i) cpart[blockIdx.x * kAdjPart + i] = acc[i];
}

template <bool STRUCT>
__global__ void k_gather_adj(AdjTopo t, const double* __restrict__ G, const double* __restrict__ Gt,
                             double* __restrict__ gpos, double* __restrict__ hvp) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
  double s[3] = {0, 0, 0}, st[3] = {0, 0, 0};
  int i = 0, j = 0, k = 0;
  if (STRUCT) {
    const int nyz = t.ny * t.nz;
    i = n / nyz;
    const int r = n - i * nyz;
    j = r / t.nz;
    k = r - j * t.nz;
  }
  for (int kc = 0; kc < 8; ++kc) {
    int cell;
    if (STRUCT) {
      const int b = corner_to_bits(kc);
      int a0 = i - (b & 1), b0 = j - ((b >> 1) & 1), c0 = k - (b >> 2);
      a0 = a0 < 0 ? t.nx - 1 : a0;
      b0 = b0 < 0 ? t.ny - 1 : b0;
      c0 = c0 < 0 ? t.nz - 1 : c0;
      cell = (a0 * t.ny + b0) * t.nz + c0;
    } else {
      cell = t.node_cells[kc * t.N + n];
      if (cell < 0) continue;
    }
    for (int x = 0; x < 3; ++x) {
      s[x] += G[(kc * 3 + x) * (size_t)t.M + cell];
      st[x] += Gt[(kc * 3 + x) * (size_t)t.M + cell];
    }
  }
  for (int x = 0; x < 3; ++x) {
    if (gpos) gpos[3 * n + x] = s[x];
    if (hvp) hvp[3 * n + x] = st[x];
  }
}

// Sum per-cell parameter gradients over the cells of each type (fixed order).
// out[(ty * 4 + s) * 46 + k][2]
__global__ void k_param_reduce(int M, const uint8_t* __restrict__ ctype, const double* __restrict__ P, int ntypes,
                               double* __restrict__ out) {
  __shared__ double red[2 * 8];
  const int slot = blockIdx.x;  // ty * (4*46) + s*46 + k
  const int ty = slot / (MM_MAX_STATES * kPG);
  const int sk = slot % (MM_MAX_STATES * kPG);
  double acc[2] = {0.0, 0.0};
  for (int c = threadIdx.x; c < M; c += blockDim.x)
    if (ctype[c] == ty) {
      const size_t idx = ((size_t)sk * 2) * M + c;
      acc[0] += P[idx];
      acc[1] += P[idx + M];
    }
  block_sum<2>(acc, red);
  if (threadIdx.x == 0) {
    out[2 * slot] = acc[0];
    out[2 * slot + 1] = acc[1];
  }
}

__global__ void k_adj_finalize(const double* __restrict__ cpart, int nblk, double* __restrict__ energy,
                               double* __restrict__ vtens) {
  __shared__ double red[kAdjPart * 8];
  double acc[kAdjPart];
  for (int i = 0; i < kAdjPart; ++i) acc[i] = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x)
    for (int i = 0; i < kAdjPart; ++i) acc[i] += cpart[b * kAdjPart + i];
  block_sum<kAdjPart>(acc, red);
  if (threadIdx.x == 0) {
    if (energy) {
      energy[0] = acc[0];
      energy[1] = acc[1];
    }
    if (vtens)
      for (int i = 0; i < 18; ++i) vtens[i] = acc[2 + i];
  }
}

}  // namespace

extern "C" {

mm_status mm_set_params(mm_handle* h, const double* h0, const double* C, const double* free_energy,
                        const double* temp_eff) {
  if (!h || !h0 || !C || !free_energy || !temp_eff) return MM_ERR_ARG;
  const double kB = 1.3806505e-23 / 4.35974381e-18;
  const int P6[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
  for (int t = 0; t < h->ntypes; ++t) {
    TypeTable& tt = h->tt[t];
    tt.kT = kB * temp_eff[t];
    for (int s = 0; s < MM_MAX_STATES; ++s) {
      const int slot = t * MM_MAX_STATES + (s < tt.nstates ? s : 0);
      StateTable& st = tt.s[s];
      std::memcpy(st.h0, h0 + 9 * slot, 9 * sizeof(double));
      const double* a = st.h0;
      const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
      const double d = a[0] * c00 + a[1] * c01 + a[2] * c02;
      const double inv[9] = {c00 / d, (a[2] * a[7] - a[1] * a[8]) / d, (a[1] * a[5] - a[2] * a[4]) / d,
                             c01 / d, (a[0] * a[8] - a[2] * a[6]) / d, (a[2] * a[3] - a[0] * a[5]) / d,
                             c02 / d, (a[1] * a[6] - a[0] * a[7]) / d, (a[0] * a[4] - a[1] * a[3]) / d};
      std::memcpy(st.hinv, inv, sizeof(inv));
      st.v0 = d;
      const double* Cs = C + 81 * slot;
      for (int p = 0; p < 6; ++p)
        for (int q = 0; q < 6; ++q) {
          const int i = P6[p][0], j = P6[p][1], k = P6[q][0], l = P6[q][1];
          double v = 0.5 * (Cs[((i * 3 + j) * 3 + k) * 3 + l] + Cs[((j * 3 + i) * 3 + k) * 3 + l]);
          if (k != l) v += 0.5 * (Cs[((i * 3 + j) * 3 + l) * 3 + k] + Cs[((j * 3 + i) * 3 + l) * 3 + k]);
          st.A[p * 6 + q] = v;
        }
      st.df = free_energy[slot];
    }
  }
  h->simple = mm::tables_are_simple(h->tt, h->ntypes);
  const cudaError_t e = cudaMemcpy(h->d_tt, h->tt, sizeof(h->tt), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_set_params: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  return MM_OK;
}

mm_status mm_adjoint(mm_handle* h, const double* pos, const double* lam, const double* dlattice, double* energy,
                     double* gpos, double* hvp, double* vtens, double* pgrad, void* stream) {
  if (!h || !pos) return MM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t M = (size_t)h->M;
  const int nblk = (int)((M + kAdjThreads - 1) / kAdjThreads);
  // FP64 scratch (allocated on first use, kept with the handle)
  static_assert(sizeof(double) == 8, "");
  const size_t need = (24 * M) * 2 + (size_t)MM_MAX_STATES * kPG * 2 * M + (size_t)nblk * kAdjPart + 16;
  if (!h->d_adj || h->adj_len < need) {
    if (h->d_adj) cudaFree(h->d_adj);
    h->d_adj = nullptr;
    h->adj_len = 0;
    const cudaError_t e = cudaMalloc((void**)&h->d_adj, need * sizeof(double));
    if (e != cudaSuccess) {
      mm::set_error(std::string("mm_adjoint: cudaMalloc: ") + cudaGetErrorString(e));
      return MM_ERR_CUDA;
    }
    h->adj_len = need;
  }
  double* G = h->d_adj;
  double* Gt = G + 24 * M;
  double* P = Gt + 24 * M;
  double* cpart = P + (size_t)MM_MAX_STATES * kPG * 2 * M;
  double* dbox = cpart + (size_t)nblk * kAdjPart;
  if (dlattice) {
    const cudaError_t e = cudaMemcpyAsync(dbox, dlattice, 9 * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return MM_ERR_CUDA;
  }
  // displacements in FP64
  mm::launch_pos_to_state(h, pos, st);
  AdjTopo t{h->N, h->M, h->structured, h->nn[0], h->nn[1], h->nn[2], h->d_cell_nodes, h->d_node_cells, h->d_node_lat,
            h->d_cell_type};
  const double* db = dlattice ? dbox : nullptr;
  double* const Pw = pgrad ? P : nullptr;
  if (h->model == MM_MODEL_ORIGINAL) {
    if (h->structured) k_cells_adj<0, true><<<nblk, kAdjThreads, 0, st>>>(t, h->d_tt, h->d_box, db, h->d_u, lam, G, Gt, Pw, cpart);
    else k_cells_adj<0, false><<<nblk, kAdjThreads, 0, st>>>(t, h->d_tt, h->d_box, db, h->d_u, lam, G, Gt, Pw, cpart);
  } else {
    if (h->structured) k_cells_adj<1, true><<<nblk, kAdjThreads, 0, st>>>(t, h->d_tt, h->d_box, db, h->d_u, lam, G, Gt, Pw, cpart);
    else k_cells_adj<1, false><<<nblk, kAdjThreads, 0, st>>>(t, h->d_tt, h->d_box, db, h->d_u, lam, G, Gt, Pw, cpart);
  }
  if (gpos || hvp) {
    const int nb = (h->N + 255) / 256;
    if (h->structured) k_gather_adj<true><<<nb, 256, 0, st>>>(t, G, Gt, gpos, hvp);
    else k_gather_adj<false><<<nb, 256, 0, st>>>(t, G, Gt, gpos, hvp);
  }
  if (pgrad) k_param_reduce<<<h->ntypes * MM_MAX_STATES * kPG, 256, 0, st>>>(h->M, h->d_cell_type, P, h->ntypes, pgrad);
  k_adj_finalize<<<1, 256, 0, st>>>(cpart, nblk, energy, vtens);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_adjoint: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  return MM_OK;
}

}  // extern "C"
