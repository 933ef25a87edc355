// extern "C" entry points of libmicmec_gb300 (declared in include/micmec_gb300.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/micmec_gb300.h"
#include "mm_handle.h"

#define MM_VERSION "micmec_gb300 0.1 (sm_103a)"

namespace {

const double kBoltzmann = 1.3806505e-23 / 4.35974381e-18;  // Hartree / K (molmod value)

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  mm::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

#define MM_CUDA(call)                                   \
  do {                                                  \
    if (!cuda_ok((call), #call)) return MM_ERR_CUDA;    \
  } while (0)

void inv3(const double* a, double* out, double* det) {
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
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

// 6x6 map from the Voigt strain (00,11,22,12,02,01) to the symmetric part of
// sigma_ij = C_ijkl eps_kl; off-diagonal strain columns collect the kl and lk terms.
void voigt_stress_map(const double* C, double* A) {
  const int P[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
  auto c = [&](int i, int j, int k, int l) { return C[((i * 3 + j) * 3 + k) * 3 + l]; };
  for (int p = 0; p < 6; ++p) {
    const int i = P[p][0], j = P[p][1];
    for (int q = 0; q < 6; ++q) {
      const int k = P[q][0], l = P[q][1];
      double v = 0.5 * (c(i, j, k, l) + c(j, i, k, l));
      if (k != l) v += 0.5 * (c(i, j, l, k) + c(j, i, l, k));
      A[p * 6 + q] = v;
    }
  }
}

template <typename X>
bool dev_alloc(X** p, size_t count) {
  if (count == 0) count = 1;
  return cuda_ok(cudaMalloc((void**)p, count * sizeof(X)), "cudaMalloc");
}

void free_handle(mm_handle* h) {
  if (!h) return;
  for (int i = 0; i < 2; ++i)
    if (h->copy_st[i]) cudaStreamDestroy(h->copy_st[i]);
  for (int i = 0; i < 3; ++i)
    if (h->copy_ev[i]) cudaEventDestroy(h->copy_ev[i]);
  void* bufs[] = {h->d_tt, h->d_box, h->d_cell_nodes, h->d_node_cells, h->d_node_lat, h->d_cell_type,
                  h->d_mass, h->d_invm, h->d_c2, h->d_u, h->d_v, h->d_disp, h->d_G, h->d_ecell,
                  h->d_cpart, h->d_npart, h->d_ticket, h->d_carry, h->d_io, h->d_flag, h->d_adj, h->d_nodef, h->d_eng};
  for (void* b : bufs)
    if (b) cudaFree(b);
  delete h;
}

mm_status upload_box(mm_handle* h) {
  MM_CUDA(cudaMemcpy(h->d_box, h->L, 9 * sizeof(double), cudaMemcpyHostToDevice));
  return MM_OK;
}

}  // namespace

extern "C" {

const char* mm_last_error(void) { return mm::last_error(); }
const char* mm_version(void) { return MM_VERSION; }

mm_status mm_selftest_convert(const double* din, float* dout, const float* fin, double* fout, int n, void* stream) {
  if (n < 0 || (n > 0 && (!din || !dout || !fin || !fout))) {
    mm::set_error("mm_selftest_convert: bad arguments");
    return MM_ERR_ARG;
  }
  mm::launch_selftest_convert(din, dout, fin, fout, n, (cudaStream_t)stream);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_selftest_convert: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  return MM_OK;
}

mm_status mm_create(int nnodes, int ncells, const int32_t* node_coords, const int32_t* cell_nodes,
                    const int32_t* node_cells, const int32_t* cell_type, const int32_t* lattice_shape, int pbc,
                    int ntypes, const int32_t* nstates, const double* h0, const double* C,
                    const double* free_energy, const double* temp_eff, const double* masses, int model,
                    int precision, mm_handle** out) {
  if (!out || nnodes <= 0 || ncells <= 0 || !node_coords || !cell_nodes || !node_cells || !cell_type ||
      !lattice_shape || !nstates || !h0 || !C || !free_energy || !temp_eff || !masses) {
    mm::set_error("mm_create: missing argument");
    return MM_ERR_ARG;
  }
  if (ntypes < 1 || ntypes > MM_MAX_TYPES || (model != MM_MODEL_ORIGINAL && model != MM_MODEL_NANOCELL) ||
      (precision != MM_PREC_FP64 && precision != MM_PREC_FP32)) {
    mm::set_error("mm_create: bad ntypes/model/precision");
    return MM_ERR_ARG;
  }
  const int N = nnodes, M = ncells;
  for (int i = 0; i < M; ++i)
    if (cell_type[i] < 0 || cell_type[i] >= ntypes) {
      mm::set_error("mm_create: cell type out of range");
      return MM_ERR_ARG;
    }
  for (int i = 0; i < 8 * M; ++i)
    if (cell_nodes[i] < 0 || cell_nodes[i] >= N) {
      mm::set_error("mm_create: cell_nodes out of range");
      return MM_ERR_ARG;
    }
  for (int i = 0; i < 8 * N; ++i)
    if (node_cells[i] < -1 || node_cells[i] >= M) {
      mm::set_error("mm_create: node_cells out of range");
      return MM_ERR_ARG;
    }
  mm_handle* h = new mm_handle();
  h->N = N;
  h->M = M;
  h->pbc = pbc ? 1 : 0;
  h->model = model;
  h->prec = precision;
  h->ntypes = ntypes;
  for (int d = 0; d < 3; ++d) h->nn[d] = lattice_shape[d];
  {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
  }

  // parameter table
  for (int t = 0; t < ntypes; ++t) {
    if (nstates[t] < 1 || nstates[t] > MM_MAX_STATES) {
      free_handle(h);
      mm::set_error("mm_create: nstates out of range");
      return MM_ERR_ARG;
    }
    mm::TypeTable& tt = h->tt[t];
    std::memset(&tt, 0, sizeof(tt));
    tt.nstates = nstates[t];
    tt.kT = kBoltzmann * temp_eff[t];
    for (int s = 0; s < MM_MAX_STATES; ++s) {
      const int slot = t * MM_MAX_STATES + (s < nstates[t] ? s : 0);
      mm::StateTable& st = tt.s[s];
      std::memcpy(st.h0, h0 + 9 * slot, 9 * sizeof(double));
      inv3(st.h0, st.hinv, &st.v0);
      voigt_stress_map(C + 81 * slot, st.A);
      st.df = free_energy[slot];
    }
  }

  h->simple = mm::tables_are_simple(h->tt, ntypes);
  // cell kernel of the eight-corner-matrix model: one thread per cell unless the environment
  // asks for the eight-lane form (MICMEC_CELL_KERNEL=8); both give the same results
  if (const char* ck = std::getenv("MICMEC_CELL_KERNEL")) h->cell_kernel = (std::atoi(ck) == 8) ? 8 : 1;

  // structured lattice detection: periodic, every lattice site a node and a cell,
  // tables identical to the implicit ones
  bool structured = pbc && (N == M) && (N == lattice_shape[0] * lattice_shape[1] * lattice_shape[2]);
  if (structured) {
    const int nx = lattice_shape[0], ny = lattice_shape[1], nz = lattice_shape[2];
    const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    for (int c = 0; c < M && structured; ++c) {
      const int i = c / (ny * nz), j = (c / nz) % ny, k = c % nz;
      if (node_coords[3 * c] != i || node_coords[3 * c + 1] != j || node_coords[3 * c + 2] != k) structured = false;
      for (int q = 0; q < 8 && structured; ++q) {
        const int a = (i + corner[q][0]) % nx, b = (j + corner[q][1]) % ny, cc = (k + corner[q][2]) % nz;
        if (cell_nodes[8 * c + q] != (a * ny + b) * nz + cc) structured = false;
        const int ca = (i - corner[q][0] + nx) % nx, cb = (j - corner[q][1] + ny) % ny, ccc = (k - corner[q][2] + nz) % nz;
        if (node_cells[8 * c + q] != (ca * ny + cb) * nz + ccc) structured = false;
      }
    }
  }
  h->structured = structured ? 1 : 0;

  const size_t esz = (precision == MM_PREC_FP32) ? sizeof(float) : sizeof(double);
  const int ncb = mm::cell_blocks(h), nnb = mm::node_blocks(h);
  bool ok = dev_alloc(&h->d_tt, MM_MAX_TYPES) && dev_alloc(&h->d_box, 9) && dev_alloc(&h->d_cell_type, M) &&
            dev_alloc(&h->d_mass, N) && dev_alloc(&h->d_invm, N) && dev_alloc(&h->d_c2, N) &&
            dev_alloc(&h->d_u, 3 * (size_t)N) && dev_alloc(&h->d_v, 3 * (size_t)N) &&
            dev_alloc((char**)&h->d_disp, 3 * (size_t)N * esz) && dev_alloc((char**)&h->d_G, 24 * (size_t)M * esz) &&
            dev_alloc(&h->d_ecell, M) && dev_alloc(&h->d_cpart, (size_t)ncb * 10) &&
            dev_alloc(&h->d_npart, (size_t)nnb * 9 + 16) && dev_alloc(&h->d_ticket, 1) && dev_alloc(&h->d_carry, 4) &&
            dev_alloc(&h->d_io, 9 * (size_t)N + 64) && dev_alloc(&h->d_flag, 1) && dev_alloc(&h->d_nodef, N);
  if (ok && !structured)
    ok = dev_alloc(&h->d_cell_nodes, 8 * (size_t)M) && dev_alloc(&h->d_node_cells, 8 * (size_t)N) &&
         dev_alloc(&h->d_node_lat, 3 * (size_t)N);
  if (!ok) {
    free_handle(h);
    return MM_ERR_CUDA;
  }
  // uploads
  std::vector<uint8_t> ty(M);
  for (int i = 0; i < M; ++i) ty[i] = (uint8_t)cell_type[i];
  h->h_mass.assign(masses, masses + N);
  std::vector<double> invm(N);
  for (int i = 0; i < N; ++i) invm[i] = 1.0 / masses[i];
  std::vector<float4> nodef(N);
  for (int i = 0; i < N; ++i) nodef[i] = make_float4((float)masses[i], (float)invm[i], 0.0f, 0.0f);
  bool up = cuda_ok(cudaMemcpy(h->d_tt, h->tt, sizeof(h->tt), cudaMemcpyHostToDevice), "upload tt") &&
            cuda_ok(cudaMemcpy(h->d_cell_type, ty.data(), M, cudaMemcpyHostToDevice), "upload types") &&
            cuda_ok(cudaMemcpy(h->d_mass, masses, N * sizeof(double), cudaMemcpyHostToDevice), "upload mass") &&
            cuda_ok(cudaMemcpy(h->d_invm, invm.data(), N * sizeof(double), cudaMemcpyHostToDevice), "upload invm") &&
            cuda_ok(cudaMemcpy(h->d_nodef, nodef.data(), N * sizeof(float4), cudaMemcpyHostToDevice), "upload nodef") &&
            cuda_ok(cudaMemset(h->d_ticket, 0, sizeof(unsigned)), "memset") &&
            cuda_ok(cudaMemset(h->d_carry, 0, 4 * sizeof(double)), "memset") &&
            cuda_ok(cudaMemset(h->d_v, 0, 3 * (size_t)N * sizeof(double)), "memset") &&
            cuda_ok(cudaMemset(h->d_flag, 0, sizeof(int)), "memset");
  if (up && !structured) {
    std::vector<int32_t> cn(8 * (size_t)M), nc(8 * (size_t)N), nl(3 * (size_t)N);
    for (int c = 0; c < M; ++c)
      for (int q = 0; q < 8; ++q) cn[(size_t)q * M + c] = cell_nodes[8 * c + q];
    for (int n = 0; n < N; ++n) {
      for (int q = 0; q < 8; ++q) nc[(size_t)q * N + n] = node_cells[8 * n + q];
      for (int d = 0; d < 3; ++d) nl[(size_t)d * N + n] = node_coords[3 * n + d];
    }
    up = cuda_ok(cudaMemcpy(h->d_cell_nodes, cn.data(), cn.size() * 4, cudaMemcpyHostToDevice), "upload cn") &&
         cuda_ok(cudaMemcpy(h->d_node_cells, nc.data(), nc.size() * 4, cudaMemcpyHostToDevice), "upload nc") &&
         cuda_ok(cudaMemcpy(h->d_node_lat, nl.data(), nl.size() * 4, cudaMemcpyHostToDevice), "upload nl");
  }
  if (!up) {
    free_handle(h);
    return MM_ERR_CUDA;
  }
  // default lattice matrix: unit spacing until mm_set_domain is called
  for (int i = 0; i < 9; ++i) h->L[i] = (i % 4 == 0) ? 1.0 : 0.0;
  if (upload_box(h) != MM_OK) {
    free_handle(h);
    return MM_ERR_CUDA;
  }
  *out = h;
  return MM_OK;
}

mm_status mm_destroy(mm_handle* h) {
  free_handle(h);
  return MM_OK;
}

mm_status mm_set_domain(mm_handle* h, const double* rvecs, const double* lattice) {
  if (!h) return MM_ERR_ARG;
  if (h->pbc && !rvecs) {
    mm::set_error("mm_set_domain: periodic system needs rvecs");
    return MM_ERR_ARG;
  }
  if (!h->pbc && !lattice) {
    mm::set_error("mm_set_domain: isolated system needs a lattice matrix");
    return MM_ERR_ARG;
  }
  if (rvecs) {
    std::memcpy(h->rvecs, rvecs, 9 * sizeof(double));
    double inv[9], det;
    inv3(rvecs, inv, &det);
    h->volume = std::fabs(det);
  } else {
    std::memset(h->rvecs, 0, sizeof(h->rvecs));
    h->volume = 0.0;
  }
  if (lattice) {
    std::memcpy(h->L, lattice, 9 * sizeof(double));
  } else {
    for (int d = 0; d < 3; ++d)
      for (int x = 0; x < 3; ++x) h->L[3 * d + x] = rvecs[3 * d + x] / h->nn[d];
  }
  return upload_box(h);
}

mm_status mm_compute(mm_handle* h, const double* pos, double* gpos, double* vtens, double* energy, int* status_dev,
                     void* stream) {
  if (!h || !pos || !energy) return MM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  mm::launch_pos_to_state(h, pos, st);
  mm::launch_cells(h, st, h->d_ecell);
  if (gpos) mm::launch_gather(h, gpos, status_dev, st);
  mm::launch_finalize(h, energy, vtens, status_dev, st);
  MM_CUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_compute_host(mm_handle* h, const double* pos, double* gpos, double* vtens, double* energy) {
  if (!h || !pos || !energy) return MM_ERR_ARG;
  const size_t n3 = 3 * (size_t)h->N;
  double* d_pos = h->d_io;
  double* d_gpos = h->d_io + n3;
  double* d_out = h->d_io + 2 * n3;  // energy, vtens(9)
  cudaStream_t st = 0;
  MM_CUDA(cudaMemcpyAsync(d_pos, pos, n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  if (gpos) MM_CUDA(cudaMemcpyAsync(d_gpos, gpos, n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  if (vtens) MM_CUDA(cudaMemcpyAsync(d_out + 1, vtens, 9 * sizeof(double), cudaMemcpyHostToDevice, st));
  MM_CUDA(cudaMemsetAsync(h->d_flag, 0, sizeof(int), st));
  mm_status s = mm_compute(h, d_pos, gpos ? d_gpos : nullptr, vtens ? d_out + 1 : nullptr, d_out, h->d_flag, st);
  if (s != MM_OK) return s;
  int flag = 0;
  double out[10];
  if (gpos) MM_CUDA(cudaMemcpyAsync(gpos, d_gpos, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  MM_CUDA(cudaMemcpyAsync(out, d_out, 10 * sizeof(double), cudaMemcpyDeviceToHost, st));
  MM_CUDA(cudaMemcpyAsync(&flag, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  MM_CUDA(cudaStreamSynchronize(st));
  *energy = out[0];
  if (vtens) std::memcpy(vtens, out + 1, 9 * sizeof(double));
  if (flag || std::isnan(out[0])) {
    mm::set_error("NaN in energy, gradient or virial");
    return MM_ERR_NAN;
  }
  return MM_OK;
}

mm_status mm_cell_results(mm_handle* h, double* epot_cells, double* gpos_cells, void* stream) {
  if (!h) return MM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (epot_cells)
    MM_CUDA(cudaMemcpyAsync(epot_cells, h->d_ecell, h->M * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (gpos_cells) {
    // corner-major SoA [k][x][M] -> (M, 8, 3), converted to FP64 on the host side of torch;
    // here only the FP64 layout transform is offered for FP64 handles.
    if (h->prec != MM_PREC_FP64) {
      mm::set_error("mm_cell_results: gpos_cells is only available for FP64 handles");
      return MM_ERR_ARG;
    }
    // strided transpose: one 2-D copy per (corner, component)
    for (int q = 0; q < 24; ++q)
      MM_CUDA(cudaMemcpy2DAsync(gpos_cells + q, 24 * sizeof(double), (double*)h->d_G + (size_t)q * h->M,
                                sizeof(double), sizeof(double), h->M, cudaMemcpyDeviceToDevice, st));
  }
  return MM_OK;
}

static mm_status md_prepare(mm_handle* h, double timestep, int thermo, double temp, double timecon, uint64_t seed,
                            cudaStream_t st) {
  if (!(timestep > 0.0)) return MM_ERR_ARG;
  if (thermo != MM_THERMO_NONE && thermo != MM_THERMO_LANGEVIN) return MM_ERR_ARG;
  h->md.dt = timestep;
  h->md.thermo = thermo;
  h->md.temp = temp;
  h->md.timecon = timecon;
  h->md.seed = seed;
  h->md.c1 = 1.0;
  if (thermo == MM_THERMO_LANGEVIN) {
    if (!(timecon > 0.0) || !(temp >= 0.0)) return MM_ERR_ARG;
    h->md.c1 = std::exp(-timestep / timecon / 2.0);
    if (h->md.c2_key[0] != timestep || h->md.c2_key[1] != temp || h->md.c2_key[2] != timecon) {
      std::vector<double> c2(h->N);
      std::vector<float4> nodef(h->N);
      const double c1 = h->md.c1;
      for (int i = 0; i < h->N; ++i) {
        c2[i] = std::sqrt((1.0 - c1 * c1) * temp * kBoltzmann / h->h_mass[i]);
        nodef[i] = make_float4((float)h->h_mass[i], (float)(1.0 / h->h_mass[i]), (float)c2[i], 0.0f);
      }
      MM_CUDA(cudaMemcpyAsync(h->d_c2, c2.data(), h->N * sizeof(double), cudaMemcpyHostToDevice, st));
      MM_CUDA(cudaMemcpyAsync(h->d_nodef, nodef.data(), h->N * sizeof(float4), cudaMemcpyHostToDevice, st));
      MM_CUDA(cudaStreamSynchronize(st));
      h->md.c2_key[0] = timestep;
      h->md.c2_key[1] = temp;
      h->md.c2_key[2] = timecon;
    }
  }
  return MM_OK;
}

mm_status mm_md_begin(mm_handle* h, const double* pos, const double* vel, double timestep, int thermo, double temp,
                      double timecon, uint64_t seed, const double* noise, int64_t step0, void* stream) {
  if (!h || !pos || !vel) return MM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  mm_status s = md_prepare(h, timestep, thermo, temp, timecon, seed, st);
  if (s != MM_OK) return s;
  h->md.noise = noise;
  h->md.noise_step0 = step0 + 1;
  h->md.step = step0;
  mm::launch_pos_to_state(h, pos, st);
  mm::launch_aos_to_soa(h->N, vel, h->d_v, st);
  // forces at the initial positions, then the first half of step step0+1
  mm::launch_cells(h, st, nullptr);
  mm::launch_md_nodes(h, h->md.dt, h->md.c1, h->md.seed, h->md.step, h->md.noise_step0, 0, 1, h->md.thermo,
                      h->md.noise, nullptr, nullptr, st);
  h->md.mid = 1;
  MM_CUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_md_advance(mm_handle* h, int nsteps, double* records, int finish, void* stream) {
  if (!h || nsteps < 0) return MM_ERR_ARG;
  if (!h->md.mid) {
    mm::set_error("mm_md_advance: no step in progress (call mm_md_begin)");
    return MM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  for (int s = 1; s <= nsteps; ++s) {
    const int last = finish && (s == nsteps);
    mm::launch_cells(h, st, nullptr);
    mm::launch_md_nodes(h, h->md.dt, h->md.c1, h->md.seed, h->md.step + 1, h->md.noise_step0, 1, !last,
                        h->md.thermo, h->md.noise, records ? records + (size_t)(s - 1) * MM_REC_LEN : nullptr,
                        nullptr, st);
    h->md.step += 1;
    if (last) h->md.mid = 0;
  }
  MM_CUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_md_end(mm_handle* h, double* pos, double* vel, void* stream) {
  if (!h || !pos || !vel) return MM_ERR_ARG;
  if (h->md.mid) {
    mm::set_error("mm_md_end: a step is in progress (advance with finish=1 first)");
    return MM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  mm::launch_state_to_pos(h, pos, st);
  mm::launch_soa_to_aos(h->N, h->d_v, vel, st);
  MM_CUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_md_run(mm_handle* h, double* pos, double* vel, int nsteps, double timestep, int thermo, double temp,
                    double timecon, uint64_t seed, const double* noise, double* records, int64_t step0,
                    void* stream) {
  if (!h || !pos || !vel || nsteps < 0) return MM_ERR_ARG;
  if (nsteps == 0) return MM_OK;
  mm_status s = mm_md_begin(h, pos, vel, timestep, thermo, temp, timecon, seed, noise, step0, stream);
  if (s != MM_OK) return s;
  s = mm_md_advance(h, nsteps, records, 1, stream);
  if (s != MM_OK) return s;
  return mm_md_end(h, pos, vel, stream);
}

mm_status mm_md_time_kernels(mm_handle* h, int nsteps, void* flush_buf, size_t flush_bytes, double* ms_cells,
                              double* ms_nodes, void* stream) {
  if (!h || nsteps <= 0 || !ms_cells || !ms_nodes) return MM_ERR_ARG;
  if (!h->md.mid) {
    mm::set_error("mm_md_time_kernels: no step in progress (call mm_md_begin)");
    return MM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<cudaEvent_t> ev(3 * (size_t)nsteps);
  for (auto& e : ev) MM_CUDA(cudaEventCreate(&e));
  for (int s = 0; s < nsteps; ++s) {
    if (flush_buf && flush_bytes) MM_CUDA(cudaMemsetAsync(flush_buf, s & 0xff, flush_bytes, st));
    MM_CUDA(cudaEventRecord(ev[3 * s], st));
    mm::launch_cells(h, st, nullptr);
    MM_CUDA(cudaEventRecord(ev[3 * s + 1], st));
    mm::launch_md_nodes(h, h->md.dt, h->md.c1, h->md.seed, h->md.step + 1, h->md.noise_step0, 1, 1, h->md.thermo,
                        h->md.noise, nullptr, nullptr, st);
    MM_CUDA(cudaEventRecord(ev[3 * s + 2], st));
    h->md.step += 1;
  }
  MM_CUDA(cudaStreamSynchronize(st));
  double a = 0.0, b = 0.0;
  for (int s = 0; s < nsteps; ++s) {
    float t1 = 0.f, t2 = 0.f;
    MM_CUDA(cudaEventElapsedTime(&t1, ev[3 * s], ev[3 * s + 1]));
    MM_CUDA(cudaEventElapsedTime(&t2, ev[3 * s + 1], ev[3 * s + 2]));
    a += t1;
    b += t2;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  *ms_cells = a;
  *ms_nodes = b;
  return MM_OK;
}

// The host-buffer step moves pos, vel and the gradient (three arrays of 24 B per
// node) each way; one copy per array on its own stream lets several copy engines
// share the host link.
static mm_status ensure_copy_streams(mm_handle* h) {
  for (int i = 0; i < 2; ++i)
    if (!h->copy_st[i]) MM_CUDA(cudaStreamCreateWithFlags(&h->copy_st[i], cudaStreamNonBlocking));
  for (int i = 0; i < 3; ++i)
    if (!h->copy_ev[i]) MM_CUDA(cudaEventCreateWithFlags(&h->copy_ev[i], cudaEventDisableTiming));
  return MM_OK;
}

// dst[i] <- src[i] (n bytes each) for three arrays: array 0 on st, arrays 1 and 2 on the
// side streams; st waits for all three.
static mm_status copy3(mm_handle* h, void* const* dst, const void* const* src, size_t n, cudaMemcpyKind kind,
                       cudaStream_t st) {
  MM_CUDA(cudaEventRecord(h->copy_ev[0], st));
  for (int i = 0; i < 2; ++i) {
    MM_CUDA(cudaStreamWaitEvent(h->copy_st[i], h->copy_ev[0], 0));
    MM_CUDA(cudaMemcpyAsync(dst[1 + i], src[1 + i], n, kind, h->copy_st[i]));
    MM_CUDA(cudaEventRecord(h->copy_ev[1 + i], h->copy_st[i]));
  }
  MM_CUDA(cudaMemcpyAsync(dst[0], src[0], n, kind, st));
  for (int i = 0; i < 2; ++i) MM_CUDA(cudaStreamWaitEvent(st, h->copy_ev[1 + i], 0));
  return MM_OK;
}

mm_status mm_md_step_host(mm_handle* h, double* pos, double* vel, double* gpos, double* record, double timestep,
                          int thermo, double temp, double timecon, uint64_t seed, int64_t step) {
  if (!h || !pos || !vel || !gpos) return MM_ERR_ARG;
  cudaStream_t st = 0;
  mm_status s = md_prepare(h, timestep, thermo, temp, timecon, seed, st);
  if (s != MM_OK) return s;
  s = ensure_copy_streams(h);
  if (s != MM_OK) return s;
  const size_t n3 = 3 * (size_t)h->N, bytes = n3 * sizeof(double);
  double* d_pos = h->d_io;
  double* d_gpos = h->d_io + n3;
  double* d_vel = h->d_io + 2 * n3;
  double* d_rec = h->d_io + 3 * n3;
  // carry (pre-thermostat correction) is produced by the begin kernel only through ekin;
  // the host-buffer step reports the post-thermostat correction alone.
  MM_CUDA(cudaMemsetAsync(h->d_carry, 0, sizeof(double), st));
  {
    void* dst[3] = {d_pos, d_vel, d_gpos};
    const void* src[3] = {pos, vel, gpos};
    s = copy3(h, dst, src, bytes, cudaMemcpyHostToDevice, st);
    if (s != MM_OK) return s;
  }
  mm::launch_md_host_begin(h, h->md.dt, h->md.c1, seed, step, thermo, d_pos, d_vel, d_gpos, st);
  // the new positions are final after the drift: copy them back while the forces run
  MM_CUDA(cudaEventRecord(h->copy_ev[0], st));
  MM_CUDA(cudaStreamWaitEvent(h->copy_st[0], h->copy_ev[0], 0));
  MM_CUDA(cudaMemcpyAsync(pos, d_pos, bytes, cudaMemcpyDeviceToHost, h->copy_st[0]));
  MM_CUDA(cudaEventRecord(h->copy_ev[1], h->copy_st[0]));
  mm::launch_cells(h, st, nullptr);
  mm::launch_md_nodes(h, h->md.dt, h->md.c1, seed, step, step, 1, 0, thermo, nullptr, d_rec, d_gpos, st);
  mm::launch_md_host_end(h, d_vel, st);
  MM_CUDA(cudaGetLastError());
  // velocities and gradient on two streams; the step ends when all three copies are done
  MM_CUDA(cudaEventRecord(h->copy_ev[0], st));
  MM_CUDA(cudaStreamWaitEvent(h->copy_st[1], h->copy_ev[0], 0));
  MM_CUDA(cudaMemcpyAsync(gpos, d_gpos, bytes, cudaMemcpyDeviceToHost, h->copy_st[1]));
  MM_CUDA(cudaEventRecord(h->copy_ev[2], h->copy_st[1]));
  MM_CUDA(cudaMemcpyAsync(vel, d_vel, bytes, cudaMemcpyDeviceToHost, st));
  MM_CUDA(cudaStreamWaitEvent(st, h->copy_ev[1], 0));
  MM_CUDA(cudaStreamWaitEvent(st, h->copy_ev[2], 0));
  if (record) MM_CUDA(cudaMemcpyAsync(record, d_rec, MM_REC_LEN * sizeof(double), cudaMemcpyDeviceToHost, st));
  MM_CUDA(cudaStreamSynchronize(st));
  return MM_OK;
}

}  // extern "C"
