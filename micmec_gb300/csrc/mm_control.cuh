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

__device__ inline double norm1_3(const double* A) {
  double m = 0.0;
  for (int j = 0; j < 3; ++j) {
    const double c = fabs(A[j]) + fabs(A[3 + j]) + fabs(A[6 + j]);
    m = c > m ? c : m;
  }
  return m;
}
__device__ inline void matmul3(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i * 3 + j] = A[i * 3] * B[j] + A[i * 3 + 1] * B[3 + j] + A[i * 3 + 2] * B[6 + j];
}

// R = exp(f S) for a symmetric 3x3 S: the matrix exponential the reference forms from
// an eigen-decomposition (np.linalg.eigh, npt.py:700-716), here by scaling and squaring
// of the Taylor series (Moler and Van Loan, "Nineteen dubious ways to compute the
// exponential of a matrix, twenty-five years later", SIAM Review 45, 2003): A = f S / 2^k
// with ||A||_1 <= 1/8, T = sum_n A^n / n! until a term falls below 1e-18 ||T||_1, then
// R = T^(2^k). The barostat's arguments are small (k = 0, a handful of terms), and the
// result agrees with the eigen-decomposition form to FP64 rounding.
__device__ inline void sym_exp(const double* S, double f, double* R) {
  double A[9];
  for (int i = 0; i < 9; ++i) A[i] = f * S[i];
  int k = 0;
  double nrm = norm1_3(A);
  while (nrm > 0.125 && k < 64) {
    for (int i = 0; i < 9; ++i) A[i] *= 0.5;
    nrm *= 0.5;
    ++k;
  }
  double term[9], tmp[9];
  for (int i = 0; i < 9; ++i) R[i] = term[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int n = 1; n <= 20; ++n) {
    matmul3(term, A, tmp);
    const double inv = 1.0 / n;
    for (int i = 0; i < 9; ++i) {
      term[i] = tmp[i] * inv;
      R[i] += term[i];
    }
    if (norm1_3(term) <= 1e-18 * norm1_3(R)) break;
  }
  for (int q = 0; q < k; ++q) {
    matmul3(R, R, tmp);
    for (int i = 0; i < 9; ++i) R[i] = tmp[i];
  }
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
