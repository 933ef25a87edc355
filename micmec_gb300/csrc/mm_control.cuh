// Controller state and one-thread FP64 algebra of the thermostat/barostat hooks,
// shared by the batch kernels and the lattice MD engine: the per-system control
// block layout, the MTK barostat velocity update (micmec/sampling/npt.py:654-681),
// symmetric 3x3 matrix exponentials for the MTK scalings (npt.py:686-720), and the
// Nose-Hoover chain (micmec/sampling/nvt.py:410-458).
#pragma once

#include <cuda_runtime.h>

namespace mmc {

// per-system controller state (FP64), layout of the `ctl` array
enum {
  C_L = 0,            // 9 lattice matrix
  C_RV = 9,           // 9 domain vectors
  C_VOL = 18,
  C_EPOT = 19,
  C_EKIN = 20,
  C_VT = 21,          // 9 virial
  C_KT = 30,          // 9 kinetic tensor
  C_VP = 39,          // 9 barostat velocity tensor
  C_CPOS = 48,        // 3 chain positions
  C_CVEL = 51,        // 3 chain velocities
  C_CMASS = 54,       // 3 chain masses
  C_NDOF = 57,
  C_MPRESS = 58,      // barostat mass
  C_BNDOF = 59,       // barostat degrees of freedom
  C_ECT = 60,         // thermostat conserved-energy correction
  C_ECB = 61,         // barostat conserved-energy correction
  C_GMAX = 62,        // relaxation: largest node gradient norm
  C_ITER = 63,        // relaxation: iterations used
  C_ALPHA = 64,       // relaxation: last step length
  C_LEN = 72
};
enum { BR_EPOT = 0, BR_EKIN = 1, BR_ECORR = 2, BR_VOL = 3, BR_VT = 4, BR_KT = 13, BR_RV = 22, BR_LEN = 31 };

struct BMD {
  double dt, temp, timecon, press;
  int nsteps, thermo, baro, chain;
  unsigned long long seed;
  long long step0;
  const double* noise;   // replay: [nsteps][2][Ntot][3] or null
  double* rec;           // [nsys][nsteps][BR_LEN] or null
};

// ------------------------------------------------------------ small 3x3 helpers (thread 0, FP64)

__device__ inline void jacobi3(const double* Ain, double* w, double* Q) {
  double A[9];
  for (int i = 0; i < 9; ++i) A[i] = Ain[i];
  for (int i = 0; i < 9; ++i) Q[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    const double diag = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const double apq = A[p * 3 + q];
        if (apq == 0.0) continue;
        const double app = A[p * 3 + p], aqq = A[q * 3 + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(tt * tt + 1.0), sn = tt * c;
        for (int k = 0; k < 3; ++k) {  // A <- J^T A J
          const double akp = A[k * 3 + p], akq = A[k * 3 + q];
          A[k * 3 + p] = c * akp - sn * akq;
          A[k * 3 + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = A[p * 3 + k], aqk = A[q * 3 + k];
          A[p * 3 + k] = c * apk - sn * aqk;
          A[q * 3 + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {  // Q <- Q J
          const double qkp = Q[k * 3 + p], qkq = Q[k * 3 + q];
          Q[k * 3 + p] = c * qkp - sn * qkq;
          Q[k * 3 + q] = sn * qkp + c * qkq;
        }
      }
  }
  w[0] = A[0];
  w[1] = A[4];
  w[2] = A[8];
}

// R = Q diag(exp(f * w)) Q^T for a symmetric S (eigenpairs w, Q)
__device__ inline void sym_exp(const double* S, double f, double* R) {
  double w[3], Q[9];
  jacobi3(S, w, Q);
  double e[3];
  for (int i = 0; i < 3; ++i) e[i] = exp(f * w[i]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i * 3 + j] = Q[i * 3 + 0] * e[0] * Q[j * 3 + 0] + Q[i * 3 + 1] * e[1] * Q[j * 3 + 1] +
                                              Q[i * 3 + 2] * e[2] * Q[j * 3 + 2];
}

// MTK: update of the barostat velocity tensor (npt.py:654-681), thread 0
__device__ inline void update_baro_vel(double* c, const BMD& p, bool chain, double cv0) {
  const double dt = p.dt;
  if (chain)
    for (int i = 0; i < 9; ++i) c[C_VP + i] *= exp(-dt * cv0 / 8);
  double pt[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) pt[i * 3 + j] = c[C_KT + i * 3 + j] - c[C_VT + i * 3 + j];
  double ps[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ps[i * 3 + j] = 0.5 * (pt[j * 3 + i] + pt[i * 3 + j]);
  const double diag = 2.0 * c[C_EKIN] / c[C_NDOF] - p.press * c[C_VOL];
  for (int i = 0; i < 9; ++i) {
    const double Gi = (ps[i] + ((i % 4 == 0) ? diag : 0.0)) / c[C_MPRESS];
    c[C_VP + i] += Gi * dt / 4;
  }
  if (chain)
    for (int i = 0; i < 9; ++i) c[C_VP + i] *= exp(-dt * cv0 / 8);
}

__device__ inline double ekin_baro(const double* c) {
  double s = 0.0;
  for (int i = 0; i < 9; ++i) s += c[C_VP + i] * c[C_VP + i];
  return 0.5 * c[C_MPRESS] * s;
}

// one bead update of the Nose-Hoover chain (nvt.py:411-435), thread 0
__device__ inline void nhc_bead(double* c, const BMD& p, int k, double ekin, bool g1, double G1_add, double kT) {
  const int L = p.chain;
  double g;
  if (k == 0) {
    g = 2 * ekin - c[C_NDOF] * kT;
    if (g1) g += G1_add;
  } else {
    g = c[C_CMASS + k - 1] * c[C_CVEL + k - 1] * c[C_CVEL + k - 1] - kT;
  }
  g /= c[C_CMASS + k];
  if (k == L - 1) {
    c[C_CVEL + k] += g * p.dt / 4;
  } else {
    c[C_CVEL + k] *= exp(-c[C_CVEL + k + 1] * p.dt / 8);
    c[C_CVEL + k] += g * p.dt / 4;
    c[C_CVEL + k] *= exp(-c[C_CVEL + k + 1] * p.dt / 8);
  }
}

// Full NHChain call (nvt.py:410-451): returns the velocity scale factor; updates ekin in c.
__device__ inline double nhc_call(double* c, const BMD& p, bool g1, double G1_add, double kT) {
  double ekin = c[C_EKIN];
  for (int k = p.chain - 1; k >= 0; --k) nhc_bead(c, p, k, ekin, g1, G1_add, kT);
  for (int k = 0; k < p.chain; ++k) c[C_CPOS + k] += c[C_CVEL + k] * p.dt / 2;
  const double factor = exp(-c[C_CVEL + 0] * p.dt / 2);
  ekin *= factor * factor;
  for (int k = 0; k < p.chain; ++k) nhc_bead(c, p, k, ekin, g1, G1_add, kT);
  c[C_EKIN] = ekin;
  return factor;
}

__device__ inline double nhc_econs(const double* c, const BMD& p, double kT) {
  double s = 0.0, sp = 0.0;
  for (int k = 0; k < p.chain; ++k) s += c[C_CVEL + k] * c[C_CVEL + k] * c[C_CMASS + k];
  for (int k = 1; k < p.chain; ++k) sp += c[C_CPOS + k];
  return 0.5 * s + kT * (c[C_NDOF] * c[C_CPOS + 0] + sp);
}


}  // namespace mmc
