// Batched systems: hundreds of independent periodic lattices of uneven size
// (defect configurations, strain-scan points, replicas) in one persistent launch.
//
// Each CTA owns a list of whole systems (longest-first, balanced on the host) and
// runs every step of a system before moving on, so a step needs only CTA-wide
// barriers: force evaluation (cells, then the per-node gather), kicks, drifts,
// Langevin / Nose-Hoover-chain thermostats and the MTK barostat. The barostat's
// 3x3 algebra (symmetric eigen-decompositions by cyclic Jacobi rotations) runs on
// one thread in FP64. The step order is that of the reference's Verlet step with
// its hooks (micmec/sampling/verlet.py:140-166; TBCombination, npt.py:99-148;
// MTKBarostat.baro, npt.py:653-736; NHChain, nvt.py:410-458; Langevin, nvt.py:196-218).
// A second persistent kernel relaxes every system with nonlinear conjugate
// gradients (Polak-Ribiere+, secant line search).
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

using namespace mm;
using namespace mmc;

namespace {

constexpr int kMaxBT = 256;  // largest CTA size; the kernels are instantiated for 128 and 256
constexpr int kMaxNW = kMaxBT / 32;

struct BSys {
  int nx, ny, nz, M;
  long long off;  // first node / cell in the concatenated arrays
};

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
  for (int idx = threadIdx.x; idx < ntypes * MM_MAX_STATES; idx += blockDim.x) {
    const int ty = idx / MM_MAX_STATES, s = idx % MM_MAX_STATES;
    fill_state_params<T>(sh.tp[ty].s[s], tt[ty].s[s], L);
    if (s == 0) fill_type_scalars<T>(sh.tp[ty], tt[ty]);
  }
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

// Energy, virial (into sh.ctl) and node gradient (a.gpos) of system sy.
template <typename T, int MODEL>
__device__ void forces(const BArgs& a, Shared<T>& sh, const BSys& sy) {
  const T* disp = (const T*)a.disp;
  T* G = (T*)a.G + 24 * sy.off;
  const long long N3 = a.Ntot;
  const int M = sy.M;
  double acc[10];
  for (int i = 0; i < 10; ++i) acc[i] = 0.0;
  if (MODEL >= 1) {  // eight corner matrices; MODEL 2: diagonal h0 and cubic stress maps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, av = threadIdx.x & 7;
    const int ngroups = (M + 3) / 4;
    const int nw = blockDim.x >> 5;
    for (int grp = warp; grp < ngroups; grp += nw) {
      const int cell = grp * 4 + (lane >> 3);
      const bool valid = cell < M;
      T du[3] = {T(0), T(0), T(0)};
      int ty = 0;
      if (valid) {
        const int nyz = sy.ny * sy.nz, i = cell / nyz, r = cell - i * nyz, j = r / sy.nz, k = r - j * sy.nz;
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
        if (av == 0) acc[0] += (double)E;
        for (int x = 0; x < 3; ++x)
          for (int y = 0; y < 3; ++y) acc[1 + x * 3 + y] += (double)(g[x] * rel[y]);
      }
    }
  } else {
    for (int cell = threadIdx.x; cell < M; cell += blockDim.x) {
      const int nyz = sy.ny * sy.nz, i = cell / nyz, r = cell - i * nyz, j = r / sy.nz, k = r - j * sy.nz;
      T du[8][3];
      for (int b = 0; b < 8; ++b) {
        const int node = wrap_node(sy, i + (b & 1), j + ((b >> 1) & 1), k + (b >> 2));
        for (int x = 0; x < 3; ++x) du[b][x] = disp[x * N3 + sy.off + node];
      }
      T g[8][3];
      const double E = cell_eval<T, 0>(du, sh.tp[a.ctype[sy.off + cell]], g);
      for (int kc = 0; kc < 8; ++kc)
        for (int x = 0; x < 3; ++x) G[(kc * 3 + x) * (size_t)M + cell] = g[corner_to_bits(kc)][x];
      acc[0] += E;
      for (int b = 1; b < 8; ++b)
        for (int y = 0; y < 3; ++y) {
          T rr = du[b][y] - du[0][y];
          if (b & 1) rr += sh.L[0 * 3 + y];
          if (b & 2) rr += sh.L[1 * 3 + y];
          if (b & 4) rr += sh.L[2 * 3 + y];
          for (int x = 0; x < 3; ++x) acc[1 + x * 3 + y] += (double)(g[b][x] * rr);
        }
    }
  }
  cta_sum<10>(acc, sh.red);
  if (threadIdx.x == 0) {
    sh.ctl[C_EPOT] = acc[0];
    for (int i = 0; i < 9; ++i) sh.ctl[C_VT + i] = acc[1 + i];
  }
  __syncthreads();  // G complete
  for (int n = threadIdx.x; n < M; n += blockDim.x) {
    const int nyz = sy.ny * sy.nz, i = n / nyz, r = n - i * nyz, j = r / sy.nz, k = r - j * sy.nz;
    T s[3] = {T(0), T(0), T(0)};
    for (int kc = 0; kc < 8; ++kc) {
      const int b = corner_to_bits(kc);
      const int cell = wrap_cell(sy, i - (b & 1), j - ((b >> 1) & 1), k - (b >> 2));
      for (int x = 0; x < 3; ++x) s[x] += G[(kc * 3 + x) * (size_t)M + cell];
    }
    for (int x = 0; x < 3; ++x) a.gpos[x * N3 + sy.off + n] = (double)s[x];
  }
  __syncthreads();
}

// ekin and kinetic tensor into sh.ctl
__device__ void kinetic(const BArgs& a, double* ctl, double* red, const BSys& sy) {
  double acc[7];
  for (int i = 0; i < 7; ++i) acc[i] = 0.0;
  const long long N3 = a.Ntot;
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    const double m = a.mass[g], v0 = a.v[g], v1 = a.v[N3 + g], v2 = a.v[2 * N3 + g];
    acc[0] += 0.5 * m * (v0 * v0 + v1 * v1 + v2 * v2);
    acc[1] += m * v0 * v0;
    acc[2] += m * v1 * v1;
    acc[3] += m * v2 * v2;
    acc[4] += m * v1 * v2;
    acc[5] += m * v0 * v2;
    acc[6] += m * v0 * v1;
  }
  block_sum<7>(acc, red);
  if (threadIdx.x == 0) {
    ctl[C_EKIN] = acc[0];
    const double k[9] = {acc[1], acc[6], acc[5], acc[6], acc[2], acc[4], acc[5], acc[4], acc[3]};
    for (int i = 0; i < 9; ++i) ctl[C_KT + i] = k[i];
  }
  __syncthreads();
}

// u <- u R (positions of all nodes times a 3x3 matrix, row-vector convention); same for v
__device__ void scale_rows(double* arr, long long N3, const BSys& sy, const double* R) {
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
    const long long g = sy.off + n;
    const double x = arr[g], y = arr[N3 + g], z = arr[2 * N3 + g];
    arr[g] = x * R[0] + y * R[3] + z * R[6];
    arr[N3 + g] = x * R[1] + y * R[4] + z * R[7];
    arr[2 * N3 + g] = x * R[2] + y * R[5] + z * R[8];
  }
}

template <typename T>
__device__ void write_disp(const BArgs& a, const BSys& sy) {
  T* disp = (T*)a.disp;
  const long long N3 = a.Ntot;
  for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
    for (int x = 0; x < 3; ++x) disp[x * N3 + sy.off + n] = (T)a.u[x * N3 + sy.off + n];
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

// thermostat pre/post (THERMO 1 = Langevin, 2 = NHC)
template <int THERMO>
__device__ void thermostat(const BArgs& a, double* c, double* red, const BSys& sy,
                           const BMD& p, long long step, unsigned call, bool g1, double kT) {
  const long long N3 = a.Ntot;
  if (THERMO == 1) {
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
    kinetic(a, c, red, sy);
    if (threadIdx.x == 0) c[C_ECT] += ekin0 - c[C_EKIN];
    __syncthreads();
  } else if (THERMO == 2) {
    __shared__ double factor;
    if (threadIdx.x == 0) {
      double G1 = 0.0;
      if (g1) G1 = 2 * ekin_baro(c) - c[C_BNDOF] * kT;
      factor = nhc_call(c, p, g1, G1, kT);
    }
    __syncthreads();
    const double f = factor;
    for (int n = threadIdx.x; n < sy.M; n += blockDim.x)
      for (int x = 0; x < 3; ++x) a.v[x * N3 + sy.off + n] *= f;
    __syncthreads();
    kinetic(a, c, red, sy);  // ktens for the barostat; ekin re-summed
    if (threadIdx.x == 0 && call == 1) c[C_ECT] = nhc_econs(c, p, kT);
    __syncthreads();
  }
}

// MTK half step (MTKBarostat.baro, npt.py:653-736): barostat velocity, position and
// domain scaling, force evaluation, velocity scaling, barostat velocity again.
template <typename T, int MODEL>
__device__ void baro_half(const BArgs& a, Shared<T>& sh, const BSys& sy, const BMD& p, bool chain, double* cv0p) {
  double* c = sh.ctl;
  const long long N3 = a.Ntot;
  if (threadIdx.x == 0) {
    update_baro_vel(c, p, chain, chain ? *cv0p : 0.0);
    sym_exp(c + C_VP, p.dt / 2, sh.mat);
    double Ln[9], Rn[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double sl = 0.0, sr = 0.0;
        for (int k = 0; k < 3; ++k) {
          sl += c[C_L + i * 3 + k] * sh.mat[k * 3 + j];
          sr += c[C_RV + i * 3 + k] * sh.mat[k * 3 + j];
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
  __syncthreads();
  scale_rows(a.u, N3, sy, sh.mat);
  refresh_B<T>(sh, a.tt, a.ntypes, c + C_L);
  __syncthreads();
  write_disp<T>(a, sy);
  __syncthreads();
  forces<T, MODEL>(a, sh, sy);
  if (threadIdx.x == 0) {
    double S[9];
    const double tr = c[C_VP + 0] + c[C_VP + 4] + c[C_VP + 8];
    for (int i = 0; i < 9; ++i) S[i] = c[C_VP + i] + ((i % 4 == 0) ? tr / c[C_NDOF] : 0.0);
    sym_exp(S, -p.dt / 2, sh.mat);
  }
  __syncthreads();
  scale_rows(a.v, N3, sy, sh.mat);
  __syncthreads();
  kinetic(a, c, sh.red, sy);
  if (threadIdx.x == 0) update_baro_vel(c, p, chain, chain ? *cv0p : 0.0);
  __syncthreads();
}

template <typename T, int MODEL, int BT>
__global__ void __launch_bounds__(BT) k_batch_md(BArgs a, BMD p) {
  const int THERMO = p.thermo, BARO = p.baro;
  __shared__ Shared<T> sh;
  __shared__ double cv0;
  const long long N3 = a.Ntot;
  for (int w = a.work_off[blockIdx.x]; w < a.work_off[blockIdx.x + 1]; ++w) {
    const int b = a.work[w];
    const BSys sy = a.sys[b];
    for (int i = threadIdx.x; i < C_LEN; i += blockDim.x) sh.ctl[i] = a.ctl[(size_t)b * C_LEN + i];
    __syncthreads();
    double* c = sh.ctl;
    load_tables<T>(sh, a.tt, a.ntypes, c + C_L);
    __syncthreads();
    const double kT = (1.3806505e-23 / 4.35974381e-18) * p.temp;  // boltzmann (Hartree / K) x T
    write_disp<T>(a, sy);
    __syncthreads();
    forces<T, MODEL>(a, sh, sy);
    kinetic(a, c, sh.red, sy);
    for (int st = 1; st <= p.nsteps; ++st) {
      const long long step = p.step0 + st;
      // ---- pre hooks: barostat, then thermostat (TBCombination.pre)
      if (BARO == 1) {
        if (threadIdx.x == 0) cv0 = c[C_CVEL + 0];
        __syncthreads();
        baro_half<T, MODEL>(a, sh, sy, p, THERMO == 2, &cv0);
      }
      if (THERMO == 1) thermostat<1>(a, c, sh.red, sy, p, step, 0u, BARO == 1, kT);
      if (THERMO == 2) thermostat<2>(a, c, sh.red, sy, p, step, 0u, BARO == 1, kT);
      // ---- velocity Verlet
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
        const long long g = sy.off + n;
        const double im = a.invm[g];
        for (int x = 0; x < 3; ++x) {
          const double vv = a.v[x * N3 + g] + 0.5 * (-a.gpos[x * N3 + g] * im) * p.dt;
          a.v[x * N3 + g] = vv;
          a.u[x * N3 + g] += p.dt * vv;
        }
      }
      __syncthreads();
      write_disp<T>(a, sy);
      __syncthreads();
      forces<T, MODEL>(a, sh, sy);
      for (int n = threadIdx.x; n < sy.M; n += blockDim.x) {
        const long long g = sy.off + n;
        const double im = a.invm[g];
        for (int x = 0; x < 3; ++x) a.v[x * N3 + g] += 0.5 * (-a.gpos[x * N3 + g] * im) * p.dt;
      }
      __syncthreads();
      kinetic(a, c, sh.red, sy);
      // ---- post hooks: thermostat, then barostat
      if (THERMO == 1) thermostat<1>(a, c, sh.red, sy, p, step, 1u, BARO == 1, kT);
      if (THERMO == 2) thermostat<2>(a, c, sh.red, sy, p, step, 1u, BARO == 1, kT);
      if (BARO == 1) {
        if (threadIdx.x == 0) cv0 = c[C_CVEL + 0];
        __syncthreads();
        baro_half<T, MODEL>(a, sh, sy, p, THERMO == 2, &cv0);
        if (threadIdx.x == 0) c[C_ECB] = ekin_baro(c) + p.press * c[C_VOL];
      }
      if (threadIdx.x == 0 && p.rec) {
        double* r = p.rec + ((size_t)b * p.nsteps + (st - 1)) * BR_LEN;
        double corr = c[C_ECT] + c[C_ECB];
        if (THERMO == 2 && BARO == 1) corr += c[C_BNDOF] * kT * c[C_CPOS + 0];
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

}  // namespace

// ------------------------------------------------------------------ host side

namespace {

const double kBoltz = 1.3806505e-23 / 4.35974381e-18;

bool bok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  mm::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}
#define BCUDA(call)                                 \
  do {                                              \
    if (!bok((call), #call)) return MM_ERR_CUDA;    \
  } while (0)

void binv3(const double* a, double* out, double* det) {
  const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
  const double d = a[0] * c00 + a[1] * c01 + a[2] * c02;
  out[0] = c00 / d;
  out[1] = (a[2] * a[7] - a[1] * a[8]) / d;
  out[2] = (a[1] * a[5] - a[2] * a[4]) / d;
  out[3] = c01 / d;
  out[4] = (a[0] * a[8] - a[2] * a[6]) / d;
  out[5] = (a[2] * a[3] - a[0] * a[5]) / d;
  out[6] = c02 / d;
  out[7] = (a[1] * a[6] - a[0] * a[7]) / d;
  out[8] = (a[0] * a[4] - a[1] * a[3]) / d;
  *det = d;
}

void bstress_map(const double* C, double* A) {
  const int P[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
  for (int p = 0; p < 6; ++p)
    for (int q = 0; q < 6; ++q) {
      const int i = P[p][0], j = P[p][1], k = P[q][0], l = P[q][1];
      double v = 0.5 * (C[((i * 3 + j) * 3 + k) * 3 + l] + C[((j * 3 + i) * 3 + k) * 3 + l]);
      if (k != l) v += 0.5 * (C[((i * 3 + j) * 3 + l) * 3 + k] + C[((j * 3 + i) * 3 + l) * 3 + k]);
      A[p * 6 + q] = v;
    }
}

}  // namespace

struct mm_batch {
  int nsys = 0, model = 1, prec = 0, ntypes = 0, num_sms = 0;
  int simple = 0;  // every rest matrix diagonal and every stress map cubic (exactly)
  long long Ntot = 0;
  int bt = 256;        // CTA size
  int nctas = 0;       // persistent CTAs
  std::vector<BSys> sys;
  std::vector<double> mass;
  mm::TypeTable tt[MM_MAX_TYPES];
  // device
  BSys* d_sys = nullptr;
  int* d_work = nullptr;
  int* d_work_off = nullptr;
  mm::TypeTable* d_tt = nullptr;
  uint8_t* d_ctype = nullptr;
  double *d_mass = nullptr, *d_invm = nullptr, *d_u = nullptr, *d_v = nullptr, *d_gpos = nullptr, *d_ctl = nullptr;
  double *d_cgd = nullptr, *d_cgu = nullptr, *d_cgg = nullptr;
  double *d_save = nullptr;  // autotuning: saved u, v, ctl
  void* d_disp = nullptr;
  void* d_G = nullptr;
  cudaGraphExec_t graph = nullptr;
  BMD graph_key;
  int graph_bt = 0, graph_nctas = 0;
};

namespace {

void batch_free(mm_batch* b) {
  if (!b) return;
  void* bufs[] = {b->d_sys, b->d_work, b->d_work_off, b->d_tt, b->d_ctype, b->d_mass, b->d_invm, b->d_u, b->d_v,
                  b->d_gpos, b->d_ctl, b->d_cgd, b->d_cgu, b->d_cgg, b->d_save, b->d_disp, b->d_G};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  delete b;
}

// longest-processing-time assignment of systems to CTAs
mm_status batch_partition(mm_batch* b, int nctas) {
  if (nctas < 1) nctas = 1;
  if (nctas > b->nsys) nctas = b->nsys;
  std::vector<int> order(b->nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->sys[x].M > b->sys[y].M; });
  std::vector<long long> load(nctas, 0);
  std::vector<std::vector<int>> lists(nctas);
  for (int s : order) {
    int best = 0;
    for (int c = 1; c < nctas; ++c)
      if (load[c] < load[best]) best = c;
    load[best] += b->sys[s].M;
    lists[best].push_back(s);
  }
  std::vector<int> work, off(1, 0);
  for (auto& l : lists) {
    work.insert(work.end(), l.begin(), l.end());
    off.push_back((int)work.size());
  }
  BCUDA(cudaMemcpy(b->d_work, work.data(), work.size() * sizeof(int), cudaMemcpyHostToDevice));
  BCUDA(cudaMemcpy(b->d_work_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
  b->nctas = nctas;
  return MM_OK;
}

BArgs batch_args(mm_batch* b) {
  BArgs a;
  a.sys = b->d_sys;
  a.nsys = b->nsys;
  a.work = b->d_work;
  a.work_off = b->d_work_off;
  a.tt = b->d_tt;
  a.ntypes = b->ntypes;
  a.ctype = b->d_ctype;
  a.mass = b->d_mass;
  a.invm = b->d_invm;
  a.u = b->d_u;
  a.v = b->d_v;
  a.disp = b->d_disp;
  a.G = b->d_G;
  a.gpos = b->d_gpos;
  a.ctl = b->d_ctl;
  a.cgd = b->d_cgd;
  a.cgu = b->d_cgu;
  a.cgg = b->d_cgg;
  a.Ntot = b->Ntot;
  return a;
}

template <typename T, int MODEL>
void launch_md_t(mm_batch* b, const BMD& p, cudaStream_t st) {
  BArgs a = batch_args(b);
  if (b->bt == 128) k_batch_md<T, MODEL, 128><<<b->nctas, 128, 0, st>>>(a, p);
  else k_batch_md<T, MODEL, 256><<<b->nctas, 256, 0, st>>>(a, p);
}

void launch_md(mm_batch* b, const BMD& p, cudaStream_t st) {
  if (b->prec == MM_PREC_FP32) {
    if (b->model == MM_MODEL_NANOCELL && b->simple) launch_md_t<float, 2>(b, p, st);
    else if (b->model == MM_MODEL_NANOCELL) launch_md_t<float, 1>(b, p, st);
    else launch_md_t<float, 0>(b, p, st);
  } else {
    if (b->model == MM_MODEL_NANOCELL) launch_md_t<double, 1>(b, p, st);
    else launch_md_t<double, 0>(b, p, st);
  }
}

template <typename T, int MODEL>
void launch_relax_t(mm_batch* b, int max_iter, double gtol, cudaStream_t st) {
  BArgs a = batch_args(b);
  if (b->bt == 128) k_batch_relax<T, MODEL, 128><<<b->nctas, 128, 0, st>>>(a, max_iter, gtol);
  else k_batch_relax<T, MODEL, 256><<<b->nctas, 256, 0, st>>>(a, max_iter, gtol);
}

void launch_relax(mm_batch* b, int max_iter, double gtol, cudaStream_t st) {
  if (b->prec == MM_PREC_FP32) {
    if (b->model == MM_MODEL_NANOCELL && b->simple) launch_relax_t<float, 2>(b, max_iter, gtol, st);
    else if (b->model == MM_MODEL_NANOCELL) launch_relax_t<float, 1>(b, max_iter, gtol, st);
    else launch_relax_t<float, 0>(b, max_iter, gtol, st);
  } else {
    if (b->model == MM_MODEL_NANOCELL) launch_relax_t<double, 1>(b, max_iter, gtol, st);
    else launch_relax_t<double, 0>(b, max_iter, gtol, st);
  }
}

bool same_key(const BMD& x, const BMD& y) {
  return x.dt == y.dt && x.temp == y.temp && x.timecon == y.timecon && x.press == y.press && x.nsteps == y.nsteps &&
         x.thermo == y.thermo && x.baro == y.baro && x.chain == y.chain && x.seed == y.seed && x.step0 == y.step0 &&
         x.noise == y.noise && x.rec == y.rec;
}

}  // namespace

extern "C" {

mm_status mm_batch_create(int nsys, const int32_t* shapes, const int32_t* cell_type, int ntypes,
                          const int32_t* nstates, const double* h0, const double* C, const double* free_energy,
                          const double* temp_eff, const double* masses, int model, int precision, mm_batch** out) {
  if (!out || nsys < 1 || !shapes || !cell_type || !nstates || !h0 || !C || !free_energy || !temp_eff || !masses ||
      ntypes < 1 || ntypes > MM_MAX_TYPES || (model != 0 && model != 1) || (precision != 0 && precision != 1)) {
    mm::set_error("mm_batch_create: bad argument");
    return MM_ERR_ARG;
  }
  mm_batch* b = new mm_batch();
  b->nsys = nsys;
  b->model = model;
  b->prec = precision;
  b->ntypes = ntypes;
  long long off = 0;
  for (int s = 0; s < nsys; ++s) {
    BSys y;
    y.nx = shapes[3 * s];
    y.ny = shapes[3 * s + 1];
    y.nz = shapes[3 * s + 2];
    if (y.nx < 2 || y.ny < 2 || y.nz < 2) {
      batch_free(b);
      mm::set_error("mm_batch_create: every lattice direction needs at least 2 cells");
      return MM_ERR_ARG;
    }
    y.M = y.nx * y.ny * y.nz;
    y.off = off;
    off += y.M;
    b->sys.push_back(y);
  }
  b->Ntot = off;
  for (long long i = 0; i < off; ++i)
    if (cell_type[i] < 0 || cell_type[i] >= ntypes) {
      batch_free(b);
      mm::set_error("mm_batch_create: cell type out of range");
      return MM_ERR_ARG;
    }
  for (int t = 0; t < ntypes; ++t) {
    if (nstates[t] < 1 || nstates[t] > MM_MAX_STATES) {
      batch_free(b);
      mm::set_error("mm_batch_create: nstates out of range");
      return MM_ERR_ARG;
    }
    mm::TypeTable& tt = b->tt[t];
    std::memset(&tt, 0, sizeof(tt));
    tt.nstates = nstates[t];
    tt.kT = kBoltz * temp_eff[t];
    for (int st = 0; st < MM_MAX_STATES; ++st) {
      const int slot = t * MM_MAX_STATES + (st < nstates[t] ? st : 0);
      std::memcpy(tt.s[st].h0, h0 + 9 * slot, 9 * sizeof(double));
      binv3(tt.s[st].h0, tt.s[st].hinv, &tt.s[st].v0);
      bstress_map(C + 81 * slot, tt.s[st].A);
      tt.s[st].df = free_energy[slot];
    }
  }
  b->simple = mm::tables_are_simple(b->tt, ntypes);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t N = (size_t)off, esz = precision == MM_PREC_FP32 ? 4 : 8;
  b->mass.assign(masses, masses + N);
  std::vector<double> invm(N);
  for (size_t i = 0; i < N; ++i) invm[i] = 1.0 / masses[i];
  std::vector<uint8_t> ct(N);
  for (size_t i = 0; i < N; ++i) ct[i] = (uint8_t)cell_type[i];
  bool ok = bok(cudaMalloc(&b->d_sys, nsys * sizeof(BSys)), "malloc") &&
            bok(cudaMalloc(&b->d_work, nsys * sizeof(int)), "malloc") &&
            bok(cudaMalloc(&b->d_work_off, (nsys + 1) * sizeof(int)), "malloc") &&
            bok(cudaMalloc(&b->d_tt, sizeof(b->tt)), "malloc") && bok(cudaMalloc(&b->d_ctype, N), "malloc") &&
            bok(cudaMalloc(&b->d_mass, N * 8), "malloc") && bok(cudaMalloc(&b->d_invm, N * 8), "malloc") &&
            bok(cudaMalloc(&b->d_u, 3 * N * 8), "malloc") && bok(cudaMalloc(&b->d_v, 3 * N * 8), "malloc") &&
            bok(cudaMalloc(&b->d_gpos, 3 * N * 8), "malloc") &&
            bok(cudaMalloc(&b->d_ctl, (size_t)nsys * C_LEN * 8), "malloc") &&
            bok(cudaMalloc(&b->d_cgd, 3 * N * 8), "malloc") && bok(cudaMalloc(&b->d_cgu, 3 * N * 8), "malloc") &&
            bok(cudaMalloc(&b->d_cgg, 3 * N * 8), "malloc") &&
            bok(cudaMalloc(&b->d_save, (6 * N + (size_t)nsys * C_LEN) * 8), "malloc") &&
            bok(cudaMalloc(&b->d_disp, 3 * N * esz), "malloc") && bok(cudaMalloc(&b->d_G, 24 * N * esz), "malloc");
  if (ok)
    ok = bok(cudaMemcpy(b->d_sys, b->sys.data(), nsys * sizeof(BSys), cudaMemcpyHostToDevice), "upload") &&
         bok(cudaMemcpy(b->d_tt, b->tt, sizeof(b->tt), cudaMemcpyHostToDevice), "upload") &&
         bok(cudaMemcpy(b->d_ctype, ct.data(), N, cudaMemcpyHostToDevice), "upload") &&
         bok(cudaMemcpy(b->d_mass, masses, N * 8, cudaMemcpyHostToDevice), "upload") &&
         bok(cudaMemcpy(b->d_invm, invm.data(), N * 8, cudaMemcpyHostToDevice), "upload") &&
         bok(cudaMemset(b->d_v, 0, 3 * N * 8), "memset") && bok(cudaMemset(b->d_u, 0, 3 * N * 8), "memset") &&
         bok(cudaMemset(b->d_ctl, 0, (size_t)nsys * C_LEN * 8), "memset");
  if (!ok || batch_partition(b, std::min(nsys, 2 * b->num_sms)) != MM_OK) {
    batch_free(b);
    return MM_ERR_CUDA;
  }
  *out = b;
  return MM_OK;
}

mm_status mm_batch_destroy(mm_batch* b) {
  batch_free(b);
  return MM_OK;
}

mm_status mm_batch_set_state(mm_batch* b, const double* pos, const double* vel, const double* rvecs) {
  if (!b || !pos || !rvecs) return MM_ERR_ARG;
  const size_t N = (size_t)b->Ntot;
  std::vector<double> u(3 * N), v(3 * N, 0.0), ctl((size_t)b->nsys * C_LEN);
  BCUDA(cudaMemcpy(ctl.data(), b->d_ctl, ctl.size() * 8, cudaMemcpyDeviceToHost));
  for (int s = 0; s < b->nsys; ++s) {
    const BSys& y = b->sys[s];
    double* c = ctl.data() + (size_t)s * C_LEN;
    const double* r = rvecs + 9 * s;
    const int n[3] = {y.nx, y.ny, y.nz};
    for (int d = 0; d < 3; ++d)
      for (int x = 0; x < 3; ++x) {
        c[C_L + 3 * d + x] = r[3 * d + x] / n[d];
        c[C_RV + 3 * d + x] = r[3 * d + x];
      }
    c[C_VOL] = std::fabs(r[0] * (r[4] * r[8] - r[5] * r[7]) + r[1] * (r[5] * r[6] - r[3] * r[8]) +
                         r[2] * (r[3] * r[7] - r[4] * r[6]));
    for (int node = 0; node < y.M; ++node) {
      const int i = node / (y.ny * y.nz), j = (node / y.nz) % y.ny, k = node % y.nz;
      const size_t g = (size_t)y.off + node;
      for (int x = 0; x < 3; ++x) {
        const double X = i * c[C_L + x] + j * c[C_L + 3 + x] + k * c[C_L + 6 + x];
        u[x * N + g] = pos[3 * g + x] - X;
        if (vel) v[x * N + g] = vel[3 * g + x];
      }
    }
  }
  BCUDA(cudaMemcpy(b->d_u, u.data(), u.size() * 8, cudaMemcpyHostToDevice));
  BCUDA(cudaMemcpy(b->d_v, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
  BCUDA(cudaMemcpy(b->d_ctl, ctl.data(), ctl.size() * 8, cudaMemcpyHostToDevice));
  return MM_OK;
}

mm_status mm_batch_get_state(mm_batch* b, double* pos, double* vel, double* rvecs) {
  if (!b) return MM_ERR_ARG;
  const size_t N = (size_t)b->Ntot;
  std::vector<double> u(3 * N), v(3 * N), ctl((size_t)b->nsys * C_LEN);
  BCUDA(cudaDeviceSynchronize());
  BCUDA(cudaMemcpy(u.data(), b->d_u, u.size() * 8, cudaMemcpyDeviceToHost));
  BCUDA(cudaMemcpy(v.data(), b->d_v, v.size() * 8, cudaMemcpyDeviceToHost));
  BCUDA(cudaMemcpy(ctl.data(), b->d_ctl, ctl.size() * 8, cudaMemcpyDeviceToHost));
  for (int s = 0; s < b->nsys; ++s) {
    const BSys& y = b->sys[s];
    const double* c = ctl.data() + (size_t)s * C_LEN;
    if (rvecs)
      for (int i = 0; i < 9; ++i) rvecs[9 * s + i] = c[C_RV + i];
    for (int node = 0; node < y.M; ++node) {
      const int i = node / (y.ny * y.nz), j = (node / y.nz) % y.ny, k = node % y.nz;
      const size_t g = (size_t)y.off + node;
      for (int x = 0; x < 3; ++x) {
        if (pos) pos[3 * g + x] = (i * c[C_L + x] + j * c[C_L + 3 + x] + k * c[C_L + 6 + x]) + u[x * N + g];
        if (vel) vel[3 * g + x] = v[x * N + g];
      }
    }
  }
  return MM_OK;
}

mm_status mm_batch_control(mm_batch* b, double* ctl_host, int write) {
  if (!b || !ctl_host) return MM_ERR_ARG;
  const size_t bytes = (size_t)b->nsys * C_LEN * 8;
  if (write) BCUDA(cudaMemcpy(b->d_ctl, ctl_host, bytes, cudaMemcpyHostToDevice));
  else {
    BCUDA(cudaDeviceSynchronize());
    BCUDA(cudaMemcpy(ctl_host, b->d_ctl, bytes, cudaMemcpyDeviceToHost));
  }
  return MM_OK;
}

mm_status mm_batch_md(mm_batch* b, int nsteps, double timestep, int thermo, double temp, double timecon, int baro,
                      double press, int chain, uint64_t seed, int64_t step0, const double* noise, double* records,
                      int use_graph, void* stream) {
  if (!b || nsteps < 0 || !(timestep > 0.0) || thermo < 0 || thermo > 2 || baro < 0 || baro > 1 ||
      (thermo == 2 && (chain < 1 || chain > 3)) || (thermo == 1 && !(timecon > 0.0))) {
    mm::set_error("mm_batch_md: bad argument");
    return MM_ERR_ARG;
  }
  if (nsteps == 0) return MM_OK;
  BMD p;
  p.dt = timestep;
  p.temp = temp;
  p.timecon = timecon;
  p.press = press;
  p.nsteps = nsteps;
  p.thermo = thermo;
  p.baro = baro;
  p.chain = chain;
  p.seed = seed;
  p.step0 = step0;
  p.noise = noise;
  p.rec = records;
  cudaStream_t st = (cudaStream_t)stream;
  if (!use_graph) {
    launch_md(b, p, st);
    BCUDA(cudaGetLastError());
    return MM_OK;
  }
  if (!b->graph || !same_key(p, b->graph_key) || b->graph_bt != b->bt || b->graph_nctas != b->nctas) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaStream_t cs;
    BCUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g;
    BCUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    launch_md(b, p, cs);
    BCUDA(cudaStreamEndCapture(cs, &g));
    BCUDA(cudaGraphInstantiate(&b->graph, g, 0));
    cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    b->graph_key = p;
    b->graph_bt = b->bt;
    b->graph_nctas = b->nctas;
  }
  BCUDA(cudaGraphLaunch(b->graph, st));
  return MM_OK;
}

mm_status mm_batch_relax(mm_batch* b, int max_iter, double gtol, void* stream) {
  if (!b || max_iter < 0 || !(gtol > 0.0)) return MM_ERR_ARG;
  launch_relax(b, max_iter, gtol, (cudaStream_t)stream);
  BCUDA(cudaGetLastError());
  return MM_OK;
}

// Autotuner: times `probe_steps` MD steps for each CTA size (128, 256) and number of
// persistent CTAs (1, 2, 4 per SM, capped by the system count), restoring the state
// after every probe, and keeps the fastest configuration.
mm_status mm_batch_autotune(mm_batch* b, int probe_steps, double timestep, int thermo, double temp, double timecon,
                            int baro, double press, int chain, double* best_ms) {
  if (!b || probe_steps < 1) return MM_ERR_ARG;
  const size_t N = (size_t)b->Ntot;
  const size_t cbytes = (size_t)b->nsys * C_LEN * 8;
  BCUDA(cudaDeviceSynchronize());
  BCUDA(cudaMemcpy(b->d_save, b->d_u, 3 * N * 8, cudaMemcpyDeviceToDevice));
  BCUDA(cudaMemcpy(b->d_save + 3 * N, b->d_v, 3 * N * 8, cudaMemcpyDeviceToDevice));
  BCUDA(cudaMemcpy(b->d_save + 6 * N, b->d_ctl, cbytes, cudaMemcpyDeviceToDevice));
  cudaEvent_t e0, e1;
  BCUDA(cudaEventCreate(&e0));
  BCUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_bt = b->bt, best_ctas = b->nctas;
  const int bts[2] = {128, 256};
  const int per_sm[3] = {1, 2, 4};
  for (int ib = 0; ib < 2; ++ib)
    for (int ip = 0; ip < 3; ++ip) {
      b->bt = bts[ib];
      mm_status s = batch_partition(b, std::min(b->nsys, per_sm[ip] * b->num_sms));
      if (s != MM_OK) return s;
      BMD p;
      p.dt = timestep;
      p.temp = temp;
      p.timecon = timecon;
      p.press = press;
      p.nsteps = probe_steps;
      p.thermo = thermo;
      p.baro = baro;
      p.chain = chain;
      p.seed = 12345u;
      p.step0 = 0;
      p.noise = nullptr;
      p.rec = nullptr;
      BCUDA(cudaEventRecord(e0, 0));
      launch_md(b, p, 0);
      BCUDA(cudaEventRecord(e1, 0));
      BCUDA(cudaEventSynchronize(e1));
      BCUDA(cudaGetLastError());
      float ms = 0.f;
      BCUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        best_bt = b->bt;
        best_ctas = b->nctas;
      }
      BCUDA(cudaMemcpy(b->d_u, b->d_save, 3 * N * 8, cudaMemcpyDeviceToDevice));
      BCUDA(cudaMemcpy(b->d_v, b->d_save + 3 * N, 3 * N * 8, cudaMemcpyDeviceToDevice));
      BCUDA(cudaMemcpy(b->d_ctl, b->d_save + 6 * N, cbytes, cudaMemcpyDeviceToDevice));
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->bt = best_bt;
  mm_status s = batch_partition(b, best_ctas);
  if (best_ms) *best_ms = best;
  return s;
}

mm_status mm_batch_config(mm_batch* b, int* cta_threads, int* nctas) {
  if (!b) return MM_ERR_ARG;
  if (cta_threads) *cta_threads = b->bt;
  if (nctas) *nctas = b->nctas;
  return MM_OK;
}

}  // extern "C"
