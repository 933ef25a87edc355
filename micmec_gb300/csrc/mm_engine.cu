// MD with the reference's Nose-Hoover-chain thermostat and MTK barostat for one system
// spread over the whole GPU (the batch kernel keeps a system on one CTA; this engine is
// for lattices too large for that).
//
// A step is a sequence of grid-wide kernels on one stream, in the order of the
// reference's Verlet step with its hooks (micmec/sampling/verlet.py:140-166,
// TBCombination npt.py:99-148, MTKBarostat.baro npt.py:653-736, NHChain nvt.py:410-458,
// Langevin nvt.py:196-218): force evaluations (the lattice cell kernel and a
// fixed-order energy/virial reduction; FP64 cells also gather an FP64 gradient, FP32
// cells gather inside the kicks), node updates (kick, drift, scalings by a 3x3 matrix or
// a scalar, Langevin) that also reduce the kinetic energy and tensor, and one-thread
// controller kernels for the barostat and chain algebra in FP64. All totals use
// fixed-order reductions.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/micmec_gb300.h"
#include "mm_control.cuh"
#include "mm_device.cuh"
#include "mm_handle.h"

using namespace mm;
using namespace mmc;

namespace {

constexpr int kET = 256;
constexpr int kKin = 7;  // ekin + kinetic tensor (6)

struct ETopo {
  int N, M, structured, nx, ny, nz;
  const int32_t* node_cells;
};

template <typename T, bool STRUCT>
__global__ void k_eng_gather(ETopo t, const T* __restrict__ G, double* __restrict__ gs) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= t.N) return;
  T s[3] = {T(0), T(0), T(0)};
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
    for (int x = 0; x < 3; ++x) s[x] += G[(kc * 3 + x) * (size_t)t.M + cell];
  }
  for (int x = 0; x < 3; ++x) gs[x * (size_t)t.N + n] = (double)s[x];
}

// energy and virial of the last cell kernel (block partials, fixed order) into ctl
// (FP32 handles: the cell kernel's partials are compensated FP32 pairs)
template <bool PAIRS>
__global__ void k_eng_energy(const double* __restrict__ cpart, int nblk, double* __restrict__ ctl) {
  __shared__ double acc[10];
  sum_partials_by_warp<10, 0, PAIRS>(cpart, nblk, nullptr, 0, acc);
  if (threadIdx.x == 0) {
    ctl[C_EPOT] = acc[0];
    for (int i = 0; i < 9; ++i) ctl[C_VT + i] = acc[1 + i];
  }
}

enum { OP_KICK_DRIFT = 0, OP_KICK = 1, OP_SCALE_U = 2, OP_SCALE_V = 3, OP_SCALE_VS = 4, OP_LANGEVIN = 5,
       OP_KINETIC = 6 };

struct NodeOp {
  int op, kinetic;
  double dt, c1;
  unsigned long long seed;
  long long step, noise_step0;
  unsigned call;
};

template <typename T>
__global__ void __launch_bounds__(kET) k_eng_nodes(int N, NodeOp o, const double* __restrict__ gs, double* __restrict__ u,
                                                   double* __restrict__ v, T* __restrict__ disp,
                                                   const double* __restrict__ mass, const double* __restrict__ invm,
                                                   const double* __restrict__ mat, const double* __restrict__ c2,
                                                   const double* __restrict__ noise, double* __restrict__ npart,
                                                   unsigned* __restrict__ ticket, double* __restrict__ ctl) {
  __shared__ double red[kKin * (kET / 32)];
  __shared__ bool last;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[kKin];
  for (int i = 0; i < kKin; ++i) acc[i] = 0.0;
  if (n < N) {
    double vv[3];
    for (int x = 0; x < 3; ++x) vv[x] = v[x * (size_t)N + n];
    if (o.op == OP_KICK_DRIFT || o.op == OP_KICK) {
      const double im = invm[n];
      for (int x = 0; x < 3; ++x) vv[x] += 0.5 * (-gs[x * (size_t)N + n] * im) * o.dt;
      if (o.op == OP_KICK_DRIFT)
        for (int x = 0; x < 3; ++x) {
          const double un = u[x * (size_t)N + n] + o.dt * vv[x];
          u[x * (size_t)N + n] = un;
          disp[x * (size_t)N + n] = (T)un;
        }
    } else if (o.op == OP_SCALE_U) {
      const double a = u[n], b = u[(size_t)N + n], c = u[2 * (size_t)N + n];
      const double r[3] = {a * mat[0] + b * mat[3] + c * mat[6], a * mat[1] + b * mat[4] + c * mat[7],
                           a * mat[2] + b * mat[5] + c * mat[8]};
      for (int x = 0; x < 3; ++x) {
        u[x * (size_t)N + n] = r[x];
        disp[x * (size_t)N + n] = (T)r[x];
      }
    } else if (o.op == OP_SCALE_V) {
      const double a = vv[0], b = vv[1], c = vv[2];
      vv[0] = a * mat[0] + b * mat[3] + c * mat[6];
      vv[1] = a * mat[1] + b * mat[4] + c * mat[7];
      vv[2] = a * mat[2] + b * mat[5] + c * mat[8];
    } else if (o.op == OP_SCALE_VS) {
      for (int x = 0; x < 3; ++x) vv[x] *= mat[0];
    } else if (o.op == OP_LANGEVIN) {
      double z[3];
      if (noise) {
        const size_t base = ((size_t)(o.step - o.noise_step0) * 2 + o.call) * (size_t)N * 3;
        for (int x = 0; x < 3; ++x) z[x] = noise[base + 3 * n + x];
      } else {
        float zf[3];
        normal3(o.seed, (uint32_t)n, (uint32_t)o.step, o.call, zf);
        for (int x = 0; x < 3; ++x) z[x] = zf[x];
      }
      for (int x = 0; x < 3; ++x) vv[x] = o.c1 * vv[x] + c2[n] * z[x];
    }
    if (o.op != OP_SCALE_U && o.op != OP_KINETIC)
      for (int x = 0; x < 3; ++x) v[x * (size_t)N + n] = vv[x];
    if (o.kinetic) {
      const double m = mass[n];
      acc[0] = 0.5 * m * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
      acc[1] = m * vv[0] * vv[0];
      acc[2] = m * vv[1] * vv[1];
      acc[3] = m * vv[2] * vv[2];
      acc[4] = m * vv[1] * vv[2];
      acc[5] = m * vv[0] * vv[2];
      acc[6] = m * vv[0] * vv[1];
    }
  }
  if (!o.kinetic) return;
  block_sum<kKin>(acc, red);
  if (threadIdx.x == 0) {
    for (int i = 0; i < kKin; ++i) npart[blockIdx.x * kKin + i] = acc[i];
    __threadfence();
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot[kKin];
  for (int i = 0; i < kKin; ++i) tot[i] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
    for (int i = 0; i < kKin; ++i) tot[i] += ((volatile double*)npart)[b * kKin + i];
  block_sum<kKin>(tot, red);
  if (threadIdx.x == 0) {
    *ticket = 0u;
    ctl[C_EKIN] = tot[0];
    const double k[9] = {tot[1], tot[6], tot[5], tot[6], tot[2], tot[4], tot[5], tot[4], tot[3]};
    for (int i = 0; i < 9; ++i) ctl[C_KT + i] = k[i];
  }
}

// FP32 cells: one kernel per node operation with the corner-gradient gather fused into the
// kicks (no separate gradient array), the increments of v and u formed in FP32 and added to
// the FP64 state, and the kinetic sums in compensated FP32. 1024-thread blocks own equal
// contiguous node ranges; block partials (value-major compensated pairs) are summed by the
// block that arrives last, one warp per value.
constexpr int kEN = 1024;
constexpr int kKin6 = 6;  // kinetic tensor xx, yy, zz, yz, xz, xy (ekin = half the trace)

struct ETopo32 {
  int N, M, nx, ny, nz;
  FastDiv div_nyz, div_nz;
  const int32_t* node_cells;  // [8][N], or null for the implicit lattice
};

template <bool STRUCT>
__device__ __forceinline__ void gather32(const ETopo32& t, const float* __restrict__ G, int n, float (&s)[3]) {
  s[0] = s[1] = s[2] = 0.0f;
  int i = 0, j = 0, k = 0;
  if (STRUCT) {
    i = fdiv(n, t.div_nyz);
    const int r = n - i * (t.ny * t.nz);
    j = fdiv(r, t.div_nz);
    k = r - j * t.nz;
  }
#pragma unroll
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
#pragma unroll
    for (int x = 0; x < 3; ++x) s[x] += G[(kc * 3 + x) * (size_t)t.M + cell];
  }
}

template <bool STRUCT>
__global__ void __launch_bounds__(kEN, 1) k_eng_nodes32(ETopo32 t, NodeOp o, const float* __restrict__ G,
                                                        double* __restrict__ u, double* __restrict__ v,
                                                        float* __restrict__ disp, const float4* __restrict__ nodef,
                                                        const double* __restrict__ mat, const double* __restrict__ c2,
                                                        const double* __restrict__ noise, double* __restrict__ npart,
                                                        unsigned* __restrict__ ticket, double* __restrict__ ctl) {
  __shared__ double red[kKin6 * (kEN / 32)];
  __shared__ double tot[kKin6];
  __shared__ bool last;
  const int nb = gridDim.x;
  const size_t N = (size_t)t.N;
  F2 acc[kKin6];
#pragma unroll
  for (int i = 0; i < kKin6; ++i) acc[i] = F2{0.0f, 0.0f};
  // uniform factors in FP32 (increments), formed once
  const float hf = (float)(0.5 * o.dt), dtf = (float)o.dt;
  float rm[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) rm[i] = (float)(mat[i] - ((i % 4 == 0) ? 1.0 : 0.0));  // R - I (scalings)
  const float fm1 = (float)(mat[0] - 1.0);                                               // f - 1 (scalar scaling)
  const float c1m1 = (float)(o.c1 - 1.0);
  const int n_end = (int)(((long long)t.N * (blockIdx.x + 1)) / nb);
  for (int n = (int)(((long long)t.N * blockIdx.x) / nb) + threadIdx.x; n < n_end; n += blockDim.x) {
    if (o.op == OP_SCALE_U) {
      double w[3];
      float wf[3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        w[x] = u[x * N + n];
        wf[x] = d2f_rn(w[x]);
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double un = w[x] + f2d(wf[0] * rm[x] + wf[1] * rm[3 + x] + wf[2] * rm[6 + x]);
        u[x * N + n] = un;
        disp[x * N + n] = d2f_rn(un);
      }
      continue;
    }
    double vv[3];
    float vf[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      vv[x] = v[x * N + n];
      vf[x] = d2f_rn(vv[x]);
    }
    float q[3] = {0.0f, 0.0f, 0.0f};  // velocity increment
    if (o.op == OP_KICK_DRIFT || o.op == OP_KICK) {
      float s[3];
      gather32<STRUCT>(t, G, n, s);
      const float imf = nodef[n].y;
#pragma unroll
      for (int x = 0; x < 3; ++x) q[x] = hf * (-s[x] * imf);
    } else if (o.op == OP_SCALE_V) {
#pragma unroll
      for (int x = 0; x < 3; ++x) q[x] = vf[0] * rm[x] + vf[1] * rm[3 + x] + vf[2] * rm[6 + x];
    } else if (o.op == OP_SCALE_VS) {
#pragma unroll
      for (int x = 0; x < 3; ++x) q[x] = vf[x] * fm1;
    } else if (o.op == OP_LANGEVIN) {
      float z[3];
      if (noise) {
        const size_t base = ((size_t)(o.step - o.noise_step0) * 2 + o.call) * N * 3;
#pragma unroll
        for (int x = 0; x < 3; ++x) z[x] = d2f_rn(noise[base + 3 * n + x]);
      } else {
        normal3(o.seed, (uint32_t)n, (uint32_t)o.step, o.call, z);
      }
      const float amp = d2f_rn(c2[n]);
#pragma unroll
      for (int x = 0; x < 3; ++x) q[x] = c1m1 * vf[x] + amp * z[x];
    }
    if (o.op != OP_KINETIC) {
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        vv[x] += f2d(q[x]);
        v[x * N + n] = vv[x];
        vf[x] = d2f_rn(vv[x]);
      }
      if (o.op == OP_KICK_DRIFT)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const double un = u[x * N + n] + f2d(dtf * vf[x]);
          u[x * N + n] = un;
          disp[x * N + n] = d2f_rn(un);
        }
    }
    if (o.kinetic) {
      const float mf = nodef[n].x;
      acc[0] = f2_add(acc[0], F2{mf * vf[0] * vf[0], 0.0f});
      acc[1] = f2_add(acc[1], F2{mf * vf[1] * vf[1], 0.0f});
      acc[2] = f2_add(acc[2], F2{mf * vf[2] * vf[2], 0.0f});
      acc[3] = f2_add(acc[3], F2{mf * vf[1] * vf[2], 0.0f});
      acc[4] = f2_add(acc[4], F2{mf * vf[0] * vf[2], 0.0f});
      acc[5] = f2_add(acc[5], F2{mf * vf[0] * vf[1], 0.0f});
    }
  }
  if (!o.kinetic) return;
  block_sum_f2_pairs<kKin6>(acc, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < kKin6; ++i) store_pair(npart + (size_t)i * nb + blockIdx.x, acc[i]);
    __threadfence();
    last = (atomicAdd(ticket, 1u) == (unsigned)nb - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  sum_partials_by_warp<kKin6, 0, true>(npart, nb, nullptr, 0, tot);
  if (threadIdx.x == 0) {
    *ticket = 0u;
    ctl[C_EKIN] = 0.5 * (tot[0] + tot[1] + tot[2]);
    const double k[9] = {tot[0], tot[5], tot[4], tot[5], tot[1], tot[3], tot[4], tot[3], tot[2]};
#pragma unroll
    for (int i = 0; i < 9; ++i) ctl[C_KT + i] = k[i];
  }
}

enum { CT_CV0, CT_BARO_VEL, CT_BARO_POS, CT_BARO_VSCALE, CT_NHC, CT_NHC_ECONS, CT_SAVE_EKIN, CT_LANG_CORR, CT_ECB,
       CT_RECORD, CT_BER_T, CT_BER_T_CORR, CT_CSVR, CT_BBARO, CT_BBARO_CORR, CT_LBARO_SAVE, CT_LBARO_CORR, CT_BCHAIN };

// One-thread controller: barostat / chain algebra on the control block (FP64). `arg` is
// the G1 flag of CT_NHC and the draw index (0..3 within the step) of CT_BARO_VEL.
__global__ void k_eng_ctl(int op, BMD p, int arg, long long step, double* __restrict__ ctl, double* __restrict__ mat,
                          double* __restrict__ box, double* __restrict__ scal, double* __restrict__ rec) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* c = ctl;
  const double kT = kBoltzmannHa * p.temp;
  const bool chain = p.thermo == TH_NHC || (p.bflags & BF_CHAIN);
  switch (op) {
    case CT_CV0:  // the chain velocity the barostat velocity feels: its own chain's, else the thermostat's
      scal[0] = (p.bflags & BF_CHAIN) ? c[C_BCVEL + 0] : c[C_CVEL + 0];
      break;
    case CT_BARO_VEL: {
      double z6[6];
      const bool lang = p.baro == BA_LANGEVIN;
      if (lang) lbaro_draws(p, 0u, 1, step, arg, z6);
      update_baro_vel(c, p, chain, scal[0], lang ? z6 : nullptr);
      break;
    }
    case CT_BARO_POS:
      mtk_pos_scaling(c, p, mat);
      scale_domain(c, mat);
      for (int i = 0; i < 9; ++i) box[i] = c[C_L + i];
      break;
    case CT_BARO_VSCALE:
      mtk_vel_scaling(c, p, mat);
      break;
    case CT_BCHAIN:
      mtk_chain_step(c, p);
      break;
    case CT_NHC: {
      const double G1 = arg ? 2 * ekin_baro(c) - c[C_BNDOF] * kT : 0.0;
      mat[0] = nhc_call(c, p, arg != 0, G1, kT);
      break;
    }
    case CT_NHC_ECONS:
      c[C_ECT] = nhc_econs(c, p, kT);
      break;
    case CT_SAVE_EKIN:
      scal[1] = c[C_EKIN];
      break;
    case CT_LANG_CORR:
      c[C_ECT] += scal[1] - c[C_EKIN];
      break;
    case CT_ECB:
      c[C_ECB] = mtk_econs(c, p);
      break;
    case CT_BER_T:  // Berendsen thermostat factor; ekin before the scaling kept
      scal[1] = c[C_EKIN];
      mat[0] = berendsen_factor(c, p);
      break;
    case CT_BER_T_CORR:
      c[C_ECT] += (1 - mat[0] * mat[0]) * scal[1];
      break;
    case CT_CSVR:  // updates ekin, the kinetic tensor and the correction itself
      mat[0] = csvr_call(c, p, 0u, 1, step);
      break;
    case CT_BBARO:  // Berendsen barostat: scaling matrix and domain; epot before kept
      scal[2] = c[C_EPOT];
      berendsen_mu(c, p, mat);
      scale_domain(c, mat);
      for (int i = 0; i < 9; ++i) box[i] = c[C_L + i];
      break;
    case CT_BBARO_CORR:
      c[C_ECB] += scal[2] - c[C_EPOT];
      break;
    case CT_LBARO_SAVE:
      scal[3] = c[C_EPOT] + c[C_EKIN];
      break;
    case CT_LBARO_CORR:
      c[C_ECB] += scal[3] - c[C_EPOT] - c[C_EKIN];
      break;
    case CT_RECORD: {
      if (!rec) break;
      double corr = c[C_ECT] + c[C_ECB];
      if (p.thermo == TH_NHC && p.baro != BA_NONE && !(p.bflags & BF_CHAIN))
        corr += c[C_BNDOF] * kT * c[C_CPOS + 0];
      rec[BR_EPOT] = c[C_EPOT];
      rec[BR_EKIN] = c[C_EKIN];
      rec[BR_ECORR] = corr;
      rec[BR_VOL] = c[C_VOL];
      for (int i = 0; i < 9; ++i) {
        rec[BR_VT + i] = c[C_VT + i];
        rec[BR_KT + i] = c[C_KT + i];
        rec[BR_RV + i] = c[C_RV + i];
      }
      break;
    }
  }
}

struct Engine {
  mm_handle* h;
  cudaStream_t st;
  BMD p;
  ETopo t;
  double* ctl;
  double* mat;
  double* scal;
  double* gs;
  double* npart;
  unsigned* ticket;
  int nb;

  void ctlop(int op, int arg = 0, double* rec = nullptr, long long step = 0) {
    k_eng_ctl<<<1, 32, 0, st>>>(op, p, arg, step, ctl, mat, h->d_box, scal, rec);
  }
  template <typename T>
  void nodes_t(NodeOp o) {
    k_eng_nodes<T><<<nb, kET, 0, st>>>(h->N, o, gs, h->d_u, h->d_v, (T*)h->d_disp, h->d_mass, h->d_invm, mat, h->d_c2,
                                       p.noise, npart, ticket, ctl);
  }
  int nb32 = 0;  // node-update blocks of the FP32 kernel
  ETopo32 t32;
  void nodes(int op, int kinetic, long long step = 0, unsigned call = 0) {
    NodeOp o;
    o.op = op;
    o.kinetic = kinetic;
    o.dt = p.dt;
    o.c1 = std::exp(-p.dt / p.timecon / 2.0);
    o.seed = p.seed;
    o.step = step;
    o.noise_step0 = p.step0 + 1;
    o.call = call;
    if (h->prec == MM_PREC_FP32) {
      if (h->structured)
        k_eng_nodes32<true><<<nb32, kEN, 0, st>>>(t32, o, (const float*)h->d_G, h->d_u, h->d_v, (float*)h->d_disp,
                                                  h->d_nodef, mat, h->d_c2, p.noise, npart, ticket, ctl);
      else
        k_eng_nodes32<false><<<nb32, kEN, 0, st>>>(t32, o, (const float*)h->d_G, h->d_u, h->d_v, (float*)h->d_disp,
                                                   h->d_nodef, mat, h->d_c2, p.noise, npart, ticket, ctl);
    } else {
      nodes_t<double>(o);
    }
  }
  void forces() {
    launch_cells(h, st, nullptr);
    // FP32 cells: the kicks gather the corner gradients themselves
    if (h->prec != MM_PREC_FP32) {
      if (h->structured) k_eng_gather<double, true><<<nb, kET, 0, st>>>(t, (const double*)h->d_G, gs);
      else k_eng_gather<double, false><<<nb, kET, 0, st>>>(t, (const double*)h->d_G, gs);
    }
    if (h->prec == MM_PREC_FP32) k_eng_energy<true><<<1, kET, 0, st>>>(h->d_cpart, cell_grid(h), ctl);
    else k_eng_energy<false><<<1, kET, 0, st>>>(h->d_cpart, cell_grid(h), ctl);
  }
  // MTK / Langevin barostat half step (draws call0, call0 + 1 of the step)
  void baro_half(long long step, int call0) {
    ctlop(CT_BARO_VEL, call0, nullptr, step);
    ctlop(CT_BARO_POS);
    nodes(OP_SCALE_U, 0);
    forces();
    ctlop(CT_BARO_VSCALE);
    nodes(OP_SCALE_V, 1);
    ctlop(CT_BARO_VEL, call0 + 1, nullptr, step);
  }
  // barostat pre (call0 = 0) or post (call0 = 2) call of the MTK or Langevin barostat
  // (the MTK barostat's own chain: after the half step in pre, before it in post)
  void baro(long long step, int call0) {
    const bool bch = p.bflags & BF_CHAIN;
    if (bch && call0 != 0) ctlop(CT_BCHAIN);
    if (p.thermo == TH_NHC || bch) ctlop(CT_CV0);
    if (p.baro == BA_LANGEVIN) ctlop(CT_LBARO_SAVE);
    baro_half(step, call0);
    if (bch && call0 == 0) ctlop(CT_BCHAIN);
    if (p.baro == BA_LANGEVIN) ctlop(CT_LBARO_CORR);
    else if (call0 != 0) ctlop(CT_ECB);
  }
  void berendsen_baro() {
    ctlop(CT_BBARO);
    nodes(OP_SCALE_U, 0);
    forces();
    ctlop(CT_BBARO_CORR);
  }
  void thermo(long long step, unsigned call) {
    if (p.thermo == TH_LANGEVIN) {
      ctlop(CT_SAVE_EKIN);
      nodes(OP_LANGEVIN, 1, step, call);
      ctlop(CT_LANG_CORR);
    } else if (p.thermo == TH_NHC) {
      ctlop(CT_NHC, mtk_couples_chain(p));
      nodes(OP_SCALE_VS, 1);
      if (call == 1) ctlop(CT_NHC_ECONS);
    } else if (p.thermo == TH_BERENDSEN && call == 0) {
      ctlop(CT_BER_T);
      nodes(OP_SCALE_VS, 1);
      ctlop(CT_BER_T_CORR);
    } else if (p.thermo == TH_CSVR && call == 0) {
      ctlop(CT_CSVR, 0, nullptr, step);
      nodes(OP_SCALE_VS, 0);
    }
  }
};

}  // namespace

extern "C" mm_status mm_md_engine(mm_handle* h, double* pos, double* vel, int nsteps, double timestep, int thermo,
                                  double temp, double timecon, int baro, double press, int chain, uint64_t seed,
                                  const double* noise, const double* hook_noise, double* ctl_host, double* records,
                                  int64_t step0, void* stream) {
  if (!h || !pos || !vel || !ctl_host || nsteps < 0 || !(timestep > 0.0) || !hooks_valid(thermo, timecon, baro, chain) ||
      (thermo == TH_NHC && chain != 3) || (baro != BA_NONE && !h->pbc)) {
    mm::set_error("mm_md_engine: bad argument");
    return MM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  // scratch: control block, matrix, scalars, FP64 gradient, kinetic partials, ticket
  const int nb = (h->N + kET - 1) / kET;
  const size_t need = C_LEN + 16 + 8 + 3 * (size_t)h->N + (size_t)nb * kKin + 8;
  if (!h->d_eng || h->eng_len < need) {
    if (h->d_eng) cudaFree(h->d_eng);
    h->d_eng = nullptr;
    const cudaError_t e = cudaMalloc((void**)&h->d_eng, need * sizeof(double));
    if (e != cudaSuccess) {
      mm::set_error(std::string("mm_md_engine: cudaMalloc: ") + cudaGetErrorString(e));
      return MM_ERR_CUDA;
    }
    h->eng_len = need;
    cudaMemsetAsync(h->d_eng, 0, need * sizeof(double), st);
  }
  Engine E;
  E.h = h;
  E.st = st;
  E.ctl = h->d_eng;
  E.mat = E.ctl + C_LEN;
  E.scal = E.mat + 16;
  E.gs = E.scal + 8;
  E.npart = E.gs + 3 * (size_t)h->N;
  E.ticket = (unsigned*)(E.npart + (size_t)nb * kKin);
  E.nb = nb;
  E.t = ETopo{h->N, h->M, h->structured, h->nn[0], h->nn[1], h->nn[2], h->d_node_cells};
  {
    const int nsm = h->num_sms > 0 ? h->num_sms : 152;
    const int want = (h->N + kEN - 1) / kEN;
    E.nb32 = want < nsm ? want : nsm;
    E.t32.N = h->N;
    E.t32.M = h->M;
    E.t32.nx = h->nn[0];
    E.t32.ny = h->nn[1];
    E.t32.nz = h->nn[2];
    E.t32.div_nyz = make_fastdiv((uint32_t)(h->nn[1] * h->nn[2] > 0 ? h->nn[1] * h->nn[2] : 1));
    E.t32.div_nz = make_fastdiv((uint32_t)(h->nn[2] > 0 ? h->nn[2] : 1));
    E.t32.node_cells = h->structured ? nullptr : h->d_node_cells;
  }
  BMD& p = E.p;
  p.dt = timestep;
  p.temp = temp;
  p.timecon = timecon > 0 ? timecon : 1.0;
  p.press = press;
  p.nsteps = nsteps;
  p.thermo = thermo;
  parse_baro(baro, p);  // kind and MTK options
  p.chain = chain;
  p.seed = seed;
  p.step0 = step0;
  p.noise = noise;
  p.hnoise = hook_noise;
  p.rec = nullptr;
  // Langevin amplitudes (same cache as mm_md_run)
  if (thermo == 1) {
    const double c1 = std::exp(-timestep / timecon / 2.0);
    std::vector<double> c2(h->N);
    const double kB = 1.3806505e-23 / 4.35974381e-18;
    for (int i = 0; i < h->N; ++i) c2[i] = std::sqrt((1.0 - c1 * c1) * temp * kB / h->h_mass[i]);
    if (cudaMemcpyAsync(h->d_c2, c2.data(), h->N * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return MM_ERR_CUDA;
    h->md.c2_key[0] = -1.0;  // invalidate the mm_md_run cache (its FP32 copy was not refreshed)
  }
  // control block: lattice and domain from the handle, hook constants from the caller
  for (int i = 0; i < 9; ++i) {
    ctl_host[C_L + i] = h->L[i];
    ctl_host[C_RV + i] = h->rvecs[i];
  }
  ctl_host[C_VOL] = h->volume;
  if (cudaMemcpyAsync(E.ctl, ctl_host, C_LEN * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(E.ticket, 0, sizeof(unsigned), st) != cudaSuccess)
    return MM_ERR_CUDA;
  launch_pos_to_state(h, pos, st);
  launch_aos_to_soa(h->N, vel, h->d_v, st);
  E.forces();
  E.nodes(OP_KINETIC, 1);  // kinetic totals of the initial velocities
  for (int s = 1; s <= nsteps; ++s) {
    const long long step = step0 + s;
    if (p.baro == BA_MTK || p.baro == BA_LANGEVIN) E.baro(step, 0);
    E.thermo(step, 0);
    E.nodes(OP_KICK_DRIFT, 0);
    E.forces();
    E.nodes(OP_KICK, 1);
    E.thermo(step, 1);
    if (p.baro == BA_MTK || p.baro == BA_LANGEVIN) E.baro(step, 2);
    if (p.baro == BA_BERENDSEN) E.berendsen_baro();
    E.ctlop(CT_RECORD, 0, records ? records + (size_t)(s - 1) * BR_LEN : nullptr);
  }
  launch_state_to_pos(h, pos, st);
  launch_soa_to_aos(h->N, h->d_v, vel, st);
  if (cudaMemcpyAsync(ctl_host, E.ctl, C_LEN * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return MM_ERR_CUDA;
  // the handle's domain follows the barostat
  for (int i = 0; i < 9; ++i) {
    h->L[i] = ctl_host[C_L + i];
    h->rvecs[i] = ctl_host[C_RV + i];
  }
  h->volume = ctl_host[C_VOL];
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_md_engine: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  return MM_OK;
}
