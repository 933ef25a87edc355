// MD with the reference's Nose-Hoover-chain thermostat and MTK barostat for one system
// spread over the whole GPU (the batch kernel keeps a system on one CTA; this engine is
// for lattices too large for that).
//
// A step is a sequence of grid-wide kernels on one stream, in the order of the
// reference's Verlet step with its hooks (micmec/sampling/verlet.py:140-166,
// TBCombination npt.py:99-148, MTKBarostat.baro npt.py:653-736, NHChain nvt.py:410-458,
// Langevin nvt.py:196-218): force evaluations (the lattice cell kernel, a per-node
// gather into an FP64 gradient and a fixed-order energy/virial reduction), node
// updates (kick, drift, scalings by a 3x3 matrix or a scalar, Langevin) that also
// reduce the kinetic energy and tensor, and one-thread controller kernels for the
// barostat and chain algebra in FP64. All totals use fixed-order reductions.
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
  __shared__ double red[10 * (kET / 32)];
  double acc[10];
  if constexpr (PAIRS) {
    F2 f[10];
    for (int i = 0; i < 10; ++i) f[i] = F2{0.0f, 0.0f};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
      for (int i = 0; i < 10; ++i) {
        const float2 p = __ldcg(reinterpret_cast<const float2*>(cpart + i * nblk + b));
        f[i] = f2_add(f[i], F2{p.x, p.y});
      }
    block_sum_f2<10>(f, acc, red);
  } else {
    for (int i = 0; i < 10; ++i) acc[i] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
      for (int i = 0; i < 10; ++i) acc[i] += cpart[i * nblk + b];
    block_sum<10>(acc, red);
  }
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

enum { CT_CV0, CT_BARO_VEL, CT_BARO_POS, CT_BARO_VSCALE, CT_NHC, CT_NHC_ECONS, CT_SAVE_EKIN, CT_LANG_CORR, CT_ECB,
       CT_RECORD };

// One-thread controller: barostat / chain algebra on the control block (FP64).
__global__ void k_eng_ctl(int op, BMD p, int g1, double* __restrict__ ctl, double* __restrict__ mat,
                          double* __restrict__ box, double* __restrict__ scal, double* __restrict__ rec) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* c = ctl;
  const double kT = (1.3806505e-23 / 4.35974381e-18) * p.temp;
  const bool chain = p.thermo == 2;
  switch (op) {
    case CT_CV0:
      scal[0] = c[C_CVEL + 0];
      break;
    case CT_BARO_VEL:
      update_baro_vel(c, p, chain, scal[0]);
      break;
    case CT_BARO_POS: {
      sym_exp(c + C_VP, p.dt / 2, mat);
      double Ln[9], Rn[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double sl = 0.0, sr = 0.0;
          for (int k = 0; k < 3; ++k) {
            sl += c[C_L + i * 3 + k] * mat[k * 3 + j];
            sr += c[C_RV + i * 3 + k] * mat[k * 3 + j];
          }
          Ln[i * 3 + j] = sl;
          Rn[i * 3 + j] = sr;
        }
      for (int i = 0; i < 9; ++i) {
        c[C_L + i] = Ln[i];
        c[C_RV + i] = Rn[i];
        box[i] = Ln[i];
      }
      const double* r = c + C_RV;
      c[C_VOL] = fabs(r[0] * (r[4] * r[8] - r[5] * r[7]) + r[1] * (r[5] * r[6] - r[3] * r[8]) +
                      r[2] * (r[3] * r[7] - r[4] * r[6]));
      break;
    }
    case CT_BARO_VSCALE: {
      double S[9];
      const double tr = c[C_VP + 0] + c[C_VP + 4] + c[C_VP + 8];
      for (int i = 0; i < 9; ++i) S[i] = c[C_VP + i] + ((i % 4 == 0) ? tr / c[C_NDOF] : 0.0);
      sym_exp(S, -p.dt / 2, mat);
      break;
    }
    case CT_NHC: {
      const double G1 = g1 ? 2 * ekin_baro(c) - c[C_BNDOF] * kT : 0.0;
      mat[0] = nhc_call(c, p, g1 != 0, G1, kT);
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
      c[C_ECB] = ekin_baro(c) + p.press * c[C_VOL];
      break;
    case CT_RECORD: {
      if (!rec) break;
      double corr = c[C_ECT] + c[C_ECB];
      if (p.thermo == 2 && p.baro == 1) corr += c[C_BNDOF] * kT * c[C_CPOS + 0];
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

  void ctlop(int op, int g1 = 0, double* rec = nullptr) {
    k_eng_ctl<<<1, 32, 0, st>>>(op, p, g1, ctl, mat, h->d_box, scal, rec);
  }
  template <typename T>
  void nodes_t(NodeOp o) {
    k_eng_nodes<T><<<nb, kET, 0, st>>>(h->N, o, gs, h->d_u, h->d_v, (T*)h->d_disp, h->d_mass, h->d_invm, mat, h->d_c2,
                                       p.noise, npart, ticket, ctl);
  }
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
    if (h->prec == MM_PREC_FP32) nodes_t<float>(o);
    else nodes_t<double>(o);
  }
  void forces() {
    launch_cells(h, st, nullptr);
    if (h->prec == MM_PREC_FP32) {
      if (h->structured) k_eng_gather<float, true><<<nb, kET, 0, st>>>(t, (const float*)h->d_G, gs);
      else k_eng_gather<float, false><<<nb, kET, 0, st>>>(t, (const float*)h->d_G, gs);
    } else {
      if (h->structured) k_eng_gather<double, true><<<nb, kET, 0, st>>>(t, (const double*)h->d_G, gs);
      else k_eng_gather<double, false><<<nb, kET, 0, st>>>(t, (const double*)h->d_G, gs);
    }
    if (h->prec == MM_PREC_FP32) k_eng_energy<true><<<1, kET, 0, st>>>(h->d_cpart, cell_grid(h), ctl);
    else k_eng_energy<false><<<1, kET, 0, st>>>(h->d_cpart, cell_grid(h), ctl);
  }
  void baro_half() {
    ctlop(CT_BARO_VEL);
    ctlop(CT_BARO_POS);
    nodes(OP_SCALE_U, 0);
    forces();
    ctlop(CT_BARO_VSCALE);
    nodes(OP_SCALE_V, 1);
    ctlop(CT_BARO_VEL);
  }
  void thermo(long long step, unsigned call) {
    if (p.thermo == 1) {
      ctlop(CT_SAVE_EKIN);
      nodes(OP_LANGEVIN, 1, step, call);
      ctlop(CT_LANG_CORR);
    } else if (p.thermo == 2) {
      ctlop(CT_NHC, p.baro == 1);
      nodes(OP_SCALE_VS, 1);
      if (call == 1) ctlop(CT_NHC_ECONS);
    }
  }
};

}  // namespace

extern "C" mm_status mm_md_engine(mm_handle* h, double* pos, double* vel, int nsteps, double timestep, int thermo,
                                  double temp, double timecon, int baro, double press, int chain, uint64_t seed,
                                  const double* noise, double* ctl_host, double* records, int64_t step0,
                                  void* stream) {
  if (!h || !pos || !vel || !ctl_host || nsteps < 0 || !(timestep > 0.0) || thermo < 0 || thermo > 2 || baro < 0 ||
      baro > 1 || (thermo == 2 && chain != 3) || (thermo == 1 && !(timecon > 0.0)) || (baro == 1 && !h->pbc)) {
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
  BMD& p = E.p;
  p.dt = timestep;
  p.temp = temp;
  p.timecon = thermo == 1 ? timecon : (timecon > 0 ? timecon : 1.0);
  p.press = press;
  p.nsteps = nsteps;
  p.thermo = thermo;
  p.baro = baro;
  p.chain = chain;
  p.seed = seed;
  p.step0 = step0;
  p.noise = noise;
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
    if (baro) {
      if (thermo == 2) E.ctlop(CT_CV0);
      E.baro_half();
    }
    E.thermo(step, 0);
    E.nodes(OP_KICK_DRIFT, 0);
    E.forces();
    E.nodes(OP_KICK, 1);
    E.thermo(step, 1);
    if (baro) {
      if (thermo == 2) E.ctlop(CT_CV0);
      E.baro_half();
      E.ctlop(CT_ECB);
    }
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
