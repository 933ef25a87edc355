// Internal state of one mm_handle (a system living on the device) and the
// kernel launchers shared by the C-ABI translation unit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/micmec_gb300.h"
#include "mm_device.cuh"

struct mm_handle {
  int N = 0, M = 0;
  int structured = 0;  // implicit periodic lattice: node index == cell index
  int nn[3] = {0, 0, 0};
  int pbc = 1;
  int model = MM_MODEL_NANOCELL;
  int prec = MM_PREC_FP64;
  int ntypes = 0;
  int num_sms = 0;
  int simple = 0;  // all rest matrices diagonal and all stress maps cubic (exactly)
  int cell_kernel = 1;  // nanocell model: 1 = one thread per cell (k_cells1), 8 = eight lanes per cell (k_cells8)
  int cell_occ[2] = {0, 0};  // resident cell-kernel blocks per SM (general, simple); 0 = not queried
  int node_occ[2] = {0, 0};  // resident node-kernel blocks per SM (no thermostat, Langevin)
  mm::TypeTable tt[MM_MAX_TYPES];
  double rvecs[9] = {0};
  double L[9] = {0};
  double volume = 0.0;
  std::vector<double> h_mass;
  // device buffers
  mm::TypeTable* d_tt = nullptr;
  double* d_box = nullptr;            // lattice matrix L (9)
  int32_t* d_cell_nodes = nullptr;    // [8][M]
  int32_t* d_node_cells = nullptr;    // [8][N]
  int32_t* d_node_lat = nullptr;      // [3][N]
  uint8_t* d_cell_type = nullptr;     // [M]
  double* d_mass = nullptr;           // [N]
  double* d_invm = nullptr;           // [N]
  double* d_c2 = nullptr;             // [N] Langevin noise amplitude
  float4* d_nodef = nullptr;          // [N] FP32 copies: mass, 1/mass, Langevin amplitude
  double* d_u = nullptr;              // [3][N] displacement from lattice sites (FP64)
  double* d_v = nullptr;              // [3][N] velocities (FP64)
  void* d_disp = nullptr;             // [3][N] displacement in the cell precision
  void* d_G = nullptr;                // [24][M] corner gradients in the cell precision
  double* d_ecell = nullptr;          // [M] per-cell energies (last compute)
  double* d_cpart = nullptr;          // per cell-block partials
  double* d_npart = nullptr;          // per node-block partials
  unsigned* d_ticket = nullptr;       // last-block ticket
  double* d_carry = nullptr;          // values carried between MD kernels
  double* d_io = nullptr;             // staging: pos (3N), gpos (3N), energy+vtens (10)
  int* d_flag = nullptr;              // NaN flag
  double* d_adj = nullptr;            // adjoint scratch (allocated on first mm_adjoint call)
  size_t adj_len = 0;
  double* d_eng = nullptr;            // NHC/MTK engine scratch (allocated on first mm_md_engine call)
  cudaStream_t copy_st[2] = {nullptr, nullptr};  // host-buffer step: side streams for parallel copies
  cudaEvent_t copy_ev[3] = {nullptr, nullptr, nullptr};
  size_t eng_len = 0;
  // MD session
  struct {
    double dt = 0.0, c1 = 1.0, temp = 0.0, timecon = 0.0;
    int thermo = 0;
    uint64_t seed = 0;
    int64_t step = 0;          // last step whose first half has been applied
    int64_t noise_step0 = 0;   // step index of noise[0]
    const double* noise = nullptr;
    int mid = 0;               // 1: the next step has been started (x advanced)
    double c2_key[3] = {-1.0, -1.0, -1.0};
  } md;
};

namespace mm {
// 1 if every (type, state) has a diagonal h0 and a cubic-form stress map A.
inline int tables_are_simple(const TypeTable* tt, int ntypes) {
  for (int t = 0; t < ntypes; ++t)
    for (int s = 0; s < MM_MAX_STATES; ++s) {
      const StateTable& st = tt[t].s[s];
      const double* h = st.h0;
      if (h[1] != 0.0 || h[2] != 0.0 || h[3] != 0.0 || h[5] != 0.0 || h[6] != 0.0 || h[7] != 0.0) return 0;
      const double* A = st.A;
      const double a = A[0], b = A[1], c = A[21];
      for (int p = 0; p < 6; ++p)
        for (int q = 0; q < 6; ++q) {
          double want = 0.0;
          if (p < 3 && q < 3) want = (p == q) ? a : b;
          else if (p == q) want = c;
          if (A[p * 6 + q] != want) return 0;
        }
    }
  return 1;
}
void set_error(const std::string& s);
const char* last_error();
int cell_blocks(const mm_handle* h);  // upper bound of the cell grid (partials buffer size)
int node_blocks(const mm_handle* h);  // upper bound of the node grid (partials buffer size)
int cell_grid(mm_handle* h);          // cell grid of a launch: resident blocks x SMs, capped
int node_grid(mm_handle* h, int thermo);
void launch_cells(mm_handle* h, cudaStream_t st, double* ecell);
void launch_pos_to_state(mm_handle* h, const double* pos, cudaStream_t st);
void launch_state_to_pos(mm_handle* h, double* pos, cudaStream_t st);
void launch_gather(mm_handle* h, double* gpos, int* flag, cudaStream_t st);
void launch_finalize(mm_handle* h, double* energy, double* vtens, int* flag, cudaStream_t st);
void launch_aos_to_soa(int N, const double* a, double* s, cudaStream_t st);
void launch_selftest_convert(const double* din, float* dout, const float* fin, double* fout, int n, cudaStream_t st);
void launch_soa_to_aos(int N, const double* s, double* a, cudaStream_t st);
void launch_md_nodes(mm_handle* h, double dt, double c1, uint64_t seed, int64_t step, int64_t noise_step0, int finish,
                     int start, int thermo, const double* noise, double* record, double* gpos_out, cudaStream_t st);
void launch_md_host_begin(mm_handle* h, double dt, double c1, uint64_t seed, int64_t step, int thermo,
                          double* pos, const double* vel, const double* gpos, cudaStream_t st);
void launch_md_host_end(mm_handle* h, double* vel, cudaStream_t st);
}  // namespace mm
