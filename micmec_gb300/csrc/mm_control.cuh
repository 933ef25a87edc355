// Controller state and one-thread FP64 algebra of the thermostat/barostat hooks,
// shared by the batch kernels and the lattice MD engine: the per-system control
// block layout, the MTK and Langevin barostat velocity updates
// (micmec/sampling/npt.py:654-681, 404-439), symmetric 3x3 matrix exponentials for
// their scalings (npt.py:686-720), the Berendsen barostat's scaling matrix
// (npt.py:266-282), the Nose-Hoover chain (micmec/sampling/nvt.py:410-458), the
// Berendsen thermostat's factor (nvt.py:152-159) and the CSVR thermostat's factor
// (nvt.py:257-270) with its random draws.
#pragma once

#include <cuda_runtime.h>

#include "mm_device.cuh"

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
  C_CNDOF = 65,       // degrees of freedom the chain thermostats (0: C_NDOF)
  C_BTAU = 66,        // Langevin barostat: time constant
  C_BTEMP = 67,       // Langevin barostat: temperature
  C_SAVE = 68,        // scratch of the hook bookkeeping (energy before a hook call)
  C_SRES = 69,        // cell relaxation: largest residual stress component
  C_BCPOS = 70,       // 3 MTK barostat's own chain (baro_thermo): positions
  C_BCVEL = 73,       // 3 velocities
  C_BCMASS = 76,      // 3 masses
  C_BCTEMP = 79,      // its temperature (kelvin)
  C_LEN = 80
};
// thermostat / barostat kinds
enum { TH_NONE = 0, TH_LANGEVIN = 1, TH_NHC = 2, TH_BERENDSEN = 3, TH_CSVR = 4 };
enum { BA_NONE = 0, BA_MTK = 1, BA_BERENDSEN = 2, BA_LANGEVIN = 3 };
// per-system replayed draws of one step (hook noise): the CSVR thermostat's normal R and
// chi-squared S, then the lower triangles (00, 10, 11, 20, 21, 22) of the Langevin
// barostat's four unit-normal tensors
enum { HN_R = 0, HN_S = 1, HN_B = 2, HN_LEN = 26 };
enum { BR_EPOT = 0, BR_EKIN = 1, BR_ECORR = 2, BR_VOL = 3, BR_VT = 4, BR_KT = 13, BR_RV = 22, BR_LEN = 31 };

// Barostat options: isotropic domain fluctuations (the MTK and Langevin barostat velocity is
// one number, kept in C_VP + 0; the Berendsen scaling a multiple of the identity), a volume
// constraint (a traceless barostat velocity or scaling increment), and for the MTK barostat
// a Nose-Hoover chain of its own on the barostat velocity (MTKBarostat, npt.py:513-757;
// BerendsenBarostat, npt.py:180-292; LangevinBarostat, npt.py:295-510).
enum { BF_ISO = 1, BF_VOLC = 2, BF_CHAIN = 4 };

struct BMD {
  double dt, temp, timecon, press;
  int nsteps, thermo, baro, chain;
  int bflags, bchain;  // barostat options (BF_*) and the length of the MTK barostat's own chain
  unsigned long long seed;
  long long step0;
  const double* noise;   // replay: [nsteps][2][Ntot][3] or null
  const double* hnoise;  // replay: [nsteps][nsys][HN_LEN] or null
  double* rec;           // [nsys][nsteps][BR_LEN] or null
};

constexpr double kBoltzmannHa = 1.3806505e-23 / 4.35974381e-18;  // Hartree / K

// Hook kinds the step kernels run: thermostats none / Langevin / NHC (chain 1..3) /
// Berendsen / CSVR, barostats none / MTK / Berendsen / Langevin; CSVR alone (the
// reference's TBCombination does not pair it with a barostat, npt.py:163-177).
// The barostat argument of the C ABI: the kind (BA_*) in bits 0-3, the options BF_* in bits
// 4-6 (BF_CHAIN for the MTK barostat only) and the length (1..3) of the MTK barostat's own
// chain in bits 8-11. Splits it into p.baro, p.bflags and p.bchain; false if the
// combination is not supported.
inline bool parse_baro(int code, BMD& p) {
  p.baro = code & 0xF;
  p.bflags = (code >> 4) & 0x7;
  p.bchain = (code >> 8) & 0xF;
  if (code & ~0xF7F) return false;
  if (p.bflags && p.baro == BA_NONE) return false;
  if ((p.bflags & BF_CHAIN) && p.baro != BA_MTK) return false;
  if ((p.bflags & BF_ISO) && (p.bflags & BF_VOLC)) return false;  // no degree of freedom left
  if ((p.bflags & BF_CHAIN) ? (p.bchain < 1 || p.bchain > 3) : (p.bchain != 0)) return false;
  return true;
}

inline bool hooks_valid(int thermo, double timecon, int baro_code, int chain) {
  BMD q{};
  if (!parse_baro(baro_code, q)) return false;
  const int baro = q.baro;
  if (thermo < TH_NONE || thermo > TH_CSVR || baro < BA_NONE || baro > BA_LANGEVIN) return false;
  if (thermo == TH_NHC && (chain < 1 || chain > 3)) return false;
  if ((thermo == TH_LANGEVIN || thermo == TH_BERENDSEN || thermo == TH_CSVR) && !(timecon > 0.0)) return false;
  if (thermo == TH_CSVR && baro != BA_NONE) return false;
  return true;
}

// ------------------------------------------------------------ per-system random draws
// Philox stream of the hook draws, keyed by (system, step, tag): disjoint from the
// per-node Langevin stream (whose last counter word is a different constant).
__device__ inline void hook_uniform4(unsigned long long seed, unsigned sys, long long step, unsigned tag,
                                     double (&u)[4]) {
  const mm::U4 r = mm::philox4x32_10(mm::U4{sys, (uint32_t)step, tag, 0x484f4f4bu}, (uint32_t)seed,
                                     (uint32_t)(seed >> 32));
  const double s = 2.3283064365386963e-10;  // 2^-32: uniforms in (0, 1)
  u[0] = ((double)r.x + 0.5) * s;
  u[1] = ((double)r.y + 0.5) * s;
  u[2] = ((double)r.z + 0.5) * s;
  u[3] = ((double)r.w + 0.5) * s;
}

// Two standard normals from two uniforms (Box-Muller, FP64).
__device__ inline void box_muller(double u1, double u2, double& z0, double& z1) {
  const double r = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  z0 = r * cs;
  z1 = r * sn;
}

// n standard normals for (system, step, tag): four per generator call.
__device__ inline void hook_normals(unsigned long long seed, unsigned sys, long long step, unsigned tag, int n,
                                    double* z) {
  for (int q = 0; 4 * q < n; ++q) {
    double u[4], v[4];
    hook_uniform4(seed, sys, step, (tag << 8) | (unsigned)q, u);
    box_muller(u[0], u[1], v[0], v[1]);
    box_muller(u[2], u[3], v[2], v[3]);
    for (int i = 0; i < 4 && 4 * q + i < n; ++i) z[4 * q + i] = v[i];
  }
}

// Gamma(a, 1) variate by Marsaglia and Tsang, "A simple method for generating gamma
// variables", ACM TOMS 26 (2000) 363-372: d = a - 1/3, c = 1 / sqrt(9 d); draw a normal
// x until v = (1 + c x)^3 > 0 and log(u) < x^2/2 + d - d v + d log v, return d v. For
// a < 1 the result for a + 1 is multiplied by u^(1/a). Each try accepts with probability
// above 0.95; the loop is bounded (64 tries) and returns d if every try was rejected.
__device__ inline double gamma_mt(double a, unsigned long long seed, unsigned sys, long long step, unsigned tag) {
  double boost = 1.0;
  if (a < 1.0) {
    double u[4];
    hook_uniform4(seed, sys, step, (tag << 8) | 255u, u);
    boost = pow(u[0], 1.0 / a);
    a += 1.0;
  }
  const double d = a - 1.0 / 3.0, cc = 1.0 / sqrt(9.0 * d);
  for (unsigned k = 0; k < 64; ++k) {
    double u[4];
    hook_uniform4(seed, sys, step, (tag << 8) | k, u);
    double x, unused;
    box_muller(u[0], u[1], x, unused);
    double v = 1.0 + cc * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    if (log(u[2]) < 0.5 * x * x + d - d * v + d * log(v)) return boost * d * v;
  }
  return boost * d;
}

// tags of the hook draws
enum { TAG_CSVR_R = 1, TAG_CSVR_S = 2, TAG_LBARO = 8 };

// ------------------------------------------------------------ FP64 scalar helpers
// On this part an FP64 instruction occupies its SM sub-partition for ~64 cycles, and the
// hook algebra below is a dependent chain of them on one thread or warp while the rest of
// the CTA waits: it avoids FP64 divisions (a Newton sequence each) where the reciprocal of
// a constant does, and evaluates the exponentials of the hooks' small arguments by a short
// Taylor series.

// 1 / n for n = 0..20 (entry 0 unused), each the correctly rounded double.
static __device__ __constant__ const double kInvN[21] = {
    0.0, 1.0 / 1, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8, 1.0 / 9, 1.0 / 10,
    1.0 / 11, 1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15, 1.0 / 16, 1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20};

// exp(x). For |x| < 2^-5 (the thermostat and barostat factors: x = -dt v / 8 and the like)
// the Taylor polynomial to x^9 in Horner form (truncation below x^10 / 10! < 2.5e-22, far
// under half an ulp of the result); otherwise the library exp. The range test reads the
// exponent field on the integer pipe.
__device__ inline double exp_small(double x) {
  const unsigned hi = (unsigned)(__double_as_longlong(x) >> 32);
  if (((hi >> 20) & 0x7FFu) >= 1023u - 5u) return exp(x);
  double r = 2.7557319223985893e-06;  // 1/9!
  r = fma(r, x, 2.48015873015873e-05);  // 1/8!
  r = fma(r, x, 0.0001984126984126984);  // 1/7!
  r = fma(r, x, 0.001388888888888889);  // 1/6!
  r = fma(r, x, 0.008333333333333333);  // 1/5!
  r = fma(r, x, 0.041666666666666664);  // 1/4!
  r = fma(r, x, 0.16666666666666666);  // 1/3!
  r = fma(r, x, 0.5);
  r = fma(r, x, 1.0);
  return fma(r, x, 1.0);
}

// ------------------------------------------------------------ small 3x3 helpers (thread 0, FP64)

__device__ inline double norm1_3(const double* A) {
  double m = 0.0;
  for (int j = 0; j < 3; ++j) {
    const double c = fabs(A[j]) + fabs(A[3 + j]) + fabs(A[6 + j]);
    m = c > m ? c : m;
  }
  return m;
}
// C = A B; each entry with explicitly fused steps (a0 b0, then + a1 b1, then + a2 b2), so
// that the one-entry-per-lane form of the batch kernels rounds identically.
__device__ inline void matmul3(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = fma(A[i * 3 + 2], B[6 + j], fma(A[i * 3 + 1], B[3 + j], __dmul_rn(A[i * 3], B[j])));
}

// R = exp(f S) for a symmetric 3x3 S: the matrix exponential the reference forms from
// an eigen-decomposition (np.linalg.eigh, npt.py:700-716), here by scaling and squaring
// of the Taylor series (Moler and Van Loan, "Nineteen dubious ways to compute the
// exponential of a matrix, twenty-five years later", SIAM Review 45, 2003): A = f S / 2^k
// with ||A||_1 <= 1/8, T = sum_n A^n / n!, then R = T^(2^k). Terms are added until the
// bound ||A||^n / n! of the last one falls below 5e-19 (||T||_1 >= 2 - e^(1/8) > 0.86, so
// every omitted term is below 1e-18 ||T||_1). The barostat's arguments are small (k = 0, a
// handful of terms), and the result agrees with the eigen-decomposition form to FP64
// rounding.
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
  double bound = 1.0;
  for (int n = 1; n <= 20; ++n) {
    matmul3(term, A, tmp);
    const double inv = kInvN[n];
    for (int i = 0; i < 9; ++i) {
      term[i] = __dmul_rn(tmp[i], inv);  // not fused with the sum below
      R[i] = __dadd_rn(R[i], term[i]);
    }
    bound = __dmul_rn(__dmul_rn(bound, nrm), inv);
    if (bound <= 5e-19) break;
  }
  for (int q = 0; q < k; ++q) {
    matmul3(R, R, tmp);
    for (int i = 0; i < 9; ++i) R[i] = tmp[i];
  }
}

// Update of the barostat velocity tensor, thread 0: MTK (npt.py:654-681) when z6 is null;
// Langevin barostat (npt.py:404-439) with z6 = the lower triangle (00, 10, 11, 20, 21, 22)
// of a unit-normal tensor: friction exp(-dt / (8 timecon)) before and after, and the
// random force R = z sqrt(2 W kT / (dt timecon)) (symmetric) in the update.
__device__ inline void update_baro_vel(double* c, const BMD& p, bool chain, double cv0, const double* z6 = nullptr) {
  const double dt = p.dt;
  const double fric = z6 ? exp_small(-dt / (8 * c[C_BTAU])) : 1.0;
  const double cfac = chain ? exp_small(-dt * cv0 / 8) : 1.0;
  const double inv_mass = 1.0 / c[C_MPRESS];
  if (z6)
    for (int i = 0; i < 9; ++i) c[C_VP + i] *= fric;
  if (chain)
    for (int i = 0; i < 9; ++i) c[C_VP + i] *= cfac;
  double pt[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) pt[i * 3 + j] = c[C_KT + i * 3 + j] - c[C_VT + i * 3 + j];
  double ps[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ps[i * 3 + j] = 0.5 * (pt[j * 3 + i] + pt[i * 3 + j]);
  const double diag = 2.0 * c[C_EKIN] / c[C_NDOF] - p.press * c[C_VOL];
  double R[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (z6) {
    const double sc = sqrt(2 * c[C_MPRESS] * kBoltzmannHa * c[C_BTEMP] / (dt * c[C_BTAU]));
    const int tri[9] = {0, 1, 3, 1, 2, 4, 3, 4, 5};  // (i, j) -> lower-triangle slot of (max, min)
    for (int i = 0; i < 9; ++i) R[i] = z6[tri[i]] * sc;
  }
  double G[9];
  for (int i = 0; i < 9; ++i) G[i] = (ps[i] + ((i % 4 == 0) ? diag : 0.0)) * inv_mass;
  if (p.bflags & BF_ISO) {  // one number: the trace of G, the first entry of R
    const double t = G[0] + G[4] + G[8];
    for (int i = 0; i < 9; ++i) {
      G[i] = (i == 0) ? t : 0.0;
      R[i] = (i == 0) ? R[0] : 0.0;
    }
  } else if (p.bflags & BF_VOLC) {  // traceless
    const double t3 = (G[0] + G[4] + G[8]) / 3, r3 = (R[0] + R[4] + R[8]) / 3;
    for (int i = 0; i < 9; i += 4) {
      G[i] -= t3;
      R[i] -= r3;
    }
  }
  for (int i = 0; i < 9; ++i) {
    if (z6) c[C_VP + i] += (G[i] - R[i] * inv_mass) * dt / 4;
    else c[C_VP + i] += G[i] * dt / 4;
  }
  if (z6)
    for (int i = 0; i < 9; ++i) c[C_VP + i] *= fric;
  if (chain)
    for (int i = 0; i < 9; ++i) c[C_VP + i] *= cfac;
}

// The six unit normals of Langevin-barostat call `call` (0..3) of step `step`, system `sys`.
__device__ inline void lbaro_draws(const BMD& p, unsigned sys, int nsys, long long step, int call, double* z6) {
  if (p.hnoise) {
    const double* h = p.hnoise + ((size_t)(step - p.step0 - 1) * nsys + sys) * HN_LEN + HN_B + 6 * call;
    for (int i = 0; i < 6; ++i) z6[i] = h[i];
  } else {
    hook_normals(p.seed, sys, step, TAG_LBARO + call, 6, z6);
  }
}

// Domain update of a barostat: L <- L M, domain vectors <- rv M, volume from them.
__device__ inline void scale_domain(double* c, const double* M) {
  double Ln[9], Rn[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double sl = 0.0, sr = 0.0;
      for (int k = 0; k < 3; ++k) {
        sl += c[C_L + i * 3 + k] * M[k * 3 + j];
        sr += c[C_RV + i * 3 + k] * M[k * 3 + j];
      }
      Ln[i * 3 + j] = sl;
      Rn[i * 3 + j] = sr;
    }
  for (int i = 0; i < 9; ++i) {
    c[C_L + i] = Ln[i];
    c[C_RV + i] = Rn[i];
  }
  const double* r = c + C_RV;
  c[C_VOL] = fabs(r[0] * (r[4] * r[8] - r[5] * r[7]) + r[1] * (r[5] * r[6] - r[3] * r[8]) +
                  r[2] * (r[3] * r[7] - r[4] * r[6]));
}

// Berendsen barostat scaling matrix (npt.py:266-277), anisotropic, no volume constraint:
// mu = sym(I - dt / W (P I - (K - V) / vol)), K = sum m v (x) v, V the virial.
__device__ inline void berendsen_mu(const double* c, const BMD& p, double* mu) {
  double dmu[9], m[9];
  for (int i = 0; i < 9; ++i) {
    const double ptens = (c[C_KT + i] - c[C_VT + i]) / c[C_VOL];
    dmu[i] = p.dt / c[C_MPRESS] * (((i % 4 == 0) ? p.press : 0.0) - ptens);
  }
  if (p.bflags & BF_VOLC) {  // traceless increment
    const double t3 = (dmu[0] + dmu[4] + dmu[8]) / 3;
    for (int i = 0; i < 9; i += 4) dmu[i] -= t3;
  }
  for (int i = 0; i < 9; ++i) m[i] = ((i % 4 == 0) ? 1.0 : 0.0) - dmu[i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) mu[i * 3 + j] = 0.5 * (m[i * 3 + j] + m[j * 3 + i]);
  if (p.bflags & BF_ISO) {  // the cube root of the mean diagonal, times the identity
    const double f = cbrt((mu[0] + mu[4] + mu[8]) / 3.0);
    for (int i = 0; i < 9; ++i) mu[i] = (i % 4 == 0) ? f : 0.0;
  }
}

// Berendsen thermostat factor (nvt.py:152-159): sqrt(1 + dt / timecon (T / T_inst - 1)).
__device__ inline double berendsen_factor(const double* c, const BMD& p) {
  const double temp_inst = 2.0 * c[C_EKIN] / (kBoltzmannHa * c[C_NDOF]);
  return sqrt(1 + p.dt / p.timecon * (p.temp / temp_inst - 1));
}

// CSVR thermostat (nvt.py:257-270), thread 0: draws R and S (replayed or generated),
// returns alpha and applies its effect on ekin, the kinetic tensor and the correction.
__device__ inline double csvr_call(double* c, const BMD& p, unsigned sys, int nsys, long long step) {
  double R, S;
  if (p.hnoise) {
    const double* h = p.hnoise + ((size_t)(step - p.step0 - 1) * nsys + sys) * HN_LEN;
    R = h[HN_R];
    S = h[HN_S];
  } else {
    double z[2];
    hook_normals(p.seed, sys, step, TAG_CSVR_R, 2, z);
    R = z[0];
    const double n1 = c[C_NDOF] - 1.0;
    S = n1 > 0.0 ? 2.0 * gamma_mt(0.5 * n1, p.seed, sys, step, TAG_CSVR_S) : 0.0;
  }
  const double cc = exp(-p.dt / p.timecon);
  const double kin = 0.5 * c[C_NDOF] * kBoltzmannHa * p.temp;
  const double ekin = c[C_EKIN];
  const double fact = (1 - cc) * kin / c[C_NDOF] / ekin;
  const double x = R + sqrt(cc / fact);
  const double sgn = (x > 0.0) - (x < 0.0);
  const double alpha = sgn * sqrt(cc + (S + R * R) * fact + 2 * R * sqrt(cc * fact));
  c[C_ECT] += (1 - alpha * alpha) * ekin;
  c[C_EKIN] = alpha * alpha * ekin;
  for (int i = 0; i < 9; ++i) c[C_KT + i] *= alpha * alpha;
  return alpha;
}

__device__ inline double ekin_baro(const double* c) {
  double s = 0.0;
  for (int i = 0; i < 9; ++i) s += c[C_VP + i] * c[C_VP + i];
  return 0.5 * c[C_MPRESS] * s;
}

// degrees of freedom the chain thermostats: those of the thermostat's own init, which
// differ from the integrator's when a Langevin barostat later widens them (npt.py:86-90)
__device__ inline double chain_ndof(const double* c) { return c[C_CNDOF] > 0.0 ? c[C_CNDOF] : c[C_NDOF]; }

// A Nose-Hoover chain in the control block: slots of its positions, velocities and masses,
// its length, degrees of freedom and kT.
struct ChainRef {
  int pos, vel, mass, len;
  double ndof, kT;
};
// the particle thermostat's chain
__device__ inline ChainRef particle_chain(const double* c, const BMD& p, double kT) {
  return ChainRef{C_CPOS, C_CVEL, C_CMASS, p.chain, chain_ndof(c), kT};
}
// the MTK barostat's own chain (its degrees of freedom are the barostat's, npt.py:579-583)
__device__ inline ChainRef baro_chain(const double* c, const BMD& p) {
  return ChainRef{C_BCPOS, C_BCVEL, C_BCMASS, p.bchain, c[C_BNDOF], kBoltzmannHa * c[C_BCTEMP]};
}

// one bead update of a Nose-Hoover chain (nvt.py:411-435), thread 0; inv_mass[k] = 1 /
// (mass of bead k). The friction factor of the next bead is the same before and after the
// force term, so it is formed once.
__device__ inline void nhc_bead(double* c, const BMD& p, const ChainRef& ch, int k, double ekin, bool g1,
                                double G1_add, const double (&inv_mass)[3]) {
  double g;
  if (k == 0) {
    g = 2 * ekin - ch.ndof * ch.kT;
    if (g1) g += G1_add;
  } else {
    g = c[ch.mass + k - 1] * c[ch.vel + k - 1] * c[ch.vel + k - 1] - ch.kT;
  }
  g *= inv_mass[k];
  if (k == ch.len - 1) {
    c[ch.vel + k] += g * p.dt / 4;
  } else {
    const double fr = exp_small(-c[ch.vel + k + 1] * p.dt / 8);
    c[ch.vel + k] *= fr;
    c[ch.vel + k] += g * p.dt / 4;
    c[ch.vel + k] *= fr;
  }
}

// Full NHChain call (nvt.py:410-451) on the kinetic energy ekin: returns the velocity scale
// factor, and ekin after the scaling in ekin_out.
__device__ inline double chain_call(double* c, const BMD& p, const ChainRef& ch, bool g1, double G1_add,
                                    double ekin, double& ekin_out) {
  double inv_mass[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < ch.len; ++k) inv_mass[k] = 1.0 / c[ch.mass + k];
  for (int k = ch.len - 1; k >= 0; --k) nhc_bead(c, p, ch, k, ekin, g1, G1_add, inv_mass);
  for (int k = 0; k < ch.len; ++k) c[ch.pos + k] += c[ch.vel + k] * p.dt / 2;
  const double factor = exp_small(-c[ch.vel + 0] * p.dt / 2);
  ekin *= factor * factor;
  for (int k = 0; k < ch.len; ++k) nhc_bead(c, p, ch, k, ekin, g1, G1_add, inv_mass);
  ekin_out = ekin;
  return factor;
}

// The particle thermostat's chain call: returns the velocity scale factor; updates ekin in c.
__device__ inline double nhc_call(double* c, const BMD& p, bool g1, double G1_add, double kT) {
  double ek;
  const double f = chain_call(c, p, particle_chain(c, p, kT), g1, G1_add, c[C_EKIN], ek);
  c[C_EKIN] = ek;
  return f;
}

// conserved-energy correction of a chain (NHChain.get_econs_correction, nvt.py:453-458)
__device__ inline double chain_econs(const double* c, const ChainRef& ch) {
  double s = 0.0, sp = 0.0;
  for (int k = 0; k < ch.len; ++k) s += c[ch.vel + k] * c[ch.vel + k] * c[ch.mass + k];
  for (int k = 1; k < ch.len; ++k) sp += c[ch.pos + k];
  return 0.5 * s + ch.kT * (ch.ndof * c[ch.pos + 0] + sp);
}
__device__ inline double nhc_econs(const double* c, const BMD& p, double kT) {
  return chain_econs(c, particle_chain(c, p, kT));
}

// MTK options. The barostat's own chain acts on its kinetic energy in the pre call after
// the half step and in the post call before it (npt.py:616-651); the scaled velocity it
// returns is not used (the chain couples through its velocity, chainvel0).
__device__ inline void mtk_chain_step(double* c, const BMD& p) {
  double unused;
  chain_call(c, p, baro_chain(c, p), false, 0.0, ekin_baro(c), unused);
}
// barostat correction of the conserved energy after its post call (npt.py:644-651)
__device__ inline double mtk_econs(const double* c, const BMD& p) {
  double e = ekin_baro(c);
  if (!(p.bflags & BF_VOLC)) e += p.press * c[C_VOL];
  if (p.bflags & BF_CHAIN) e += chain_econs(c, baro_chain(c, p));
  return e;
}
// the coupling term the particle chain receives from the MTK barostat (add_press_cont,
// npt.py:738-743): none when the barostat has its own chain
__host__ __device__ inline bool mtk_couples_chain(const BMD& p) { return p.baro == BA_MTK && !(p.bflags & BF_CHAIN); }

// Scaling of positions (and domain) and of velocities in an MTK half step, row-vector form
// x <- x M (npt.py:686-720): anisotropic exp(vp dt / 2) and exp(-(vp + tr(vp) / ndof) dt / 2)
// (without the trace term under the volume constraint); isotropic exp(vp dt / 2) I and
// exp(-(1 + 3 / ndof) vp dt / 2) I.
__device__ inline void mtk_pos_scaling(const double* c, const BMD& p, double* M) {
  if (p.bflags & BF_ISO) {
    const double f = exp_small(c[C_VP + 0] * p.dt / 2);
    for (int i = 0; i < 9; ++i) M[i] = (i % 4 == 0) ? f : 0.0;
  } else {
    sym_exp(c + C_VP, p.dt / 2, M);
  }
}
__device__ inline void mtk_vel_scaling(const double* c, const BMD& p, double* M) {
  if (p.bflags & BF_ISO) {
    const double f = exp_small(-((1.0 + 3.0 / c[C_NDOF]) * c[C_VP + 0]) * p.dt / 2);
    for (int i = 0; i < 9; ++i) M[i] = (i % 4 == 0) ? f : 0.0;
    return;
  }
  double S[9];
  const double tr = (p.bflags & BF_VOLC) ? 0.0 : c[C_VP + 0] + c[C_VP + 4] + c[C_VP + 8];
  for (int i = 0; i < 9; ++i) S[i] = c[C_VP + i] + ((i % 4 == 0) ? tr / c[C_NDOF] : 0.0);
  sym_exp(S, -p.dt / 2, M);
}


}  // namespace mmc
