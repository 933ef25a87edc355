// mm_compute_noalloc: the force evaluation of mm_compute for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc at all: code that runs inside another
// framework's memory pool or a fixed-budget arena, plugins loaded into a host that
// owns every device allocation, or code paths where an allocation would
// synchronise the device at the wrong moment. mm_create allocates a handle's
// buffers, so those callers cannot use it. This entry point takes everything it
// needs from the caller's buffers and keeps its working memory (status words, node
// displacements, corner gradients, block partial sums, the parameter table) in
// one file-scope __device__ array, g_noalloc_scratch, of MM_NOALLOC_SCRATCH_BYTES
// bytes. Every GPU that loads the library holds that array until the process
// exits.
//
// Set-up: the first call on each device looks up the array's device address with
// cudaGetSymbolAddress while that device is current (the array's name in host code
// is only a host-side stand-in, not a device address). No call can be captured into a
// CUDA graph (each copies its parameters from host memory and synchronises the stream):
// a call on a stream that is being captured returns MM_ERR_ARG. The address is kept for
// the life of the process: after a cudaDeviceReset the module is loaded again and the kept
// address is stale, so a process that resets a device does not call this entry point
// afterwards.
//
// Every call shares the one array and leaves its contents behind; everything a call
// needs is rewritten or cleared by that call (the status words are cleared first).
// Calls whose work overlaps on the GPU (different streams or host threads, same
// device) race on the array and must be serialised by the caller.
//
// Checks on the device: cell types outside [0, ntypes) are found by the kernel that
// narrows them to bytes; the call reads that verdict back and returns MM_ERR_ARG
// before any kernel indexes the parameter table with them. A NaN in the energy,
// gradient or virial is returned as MM_ERR_NAN, as mm_compute_host does.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/micmec_gb300.h"
#include "mm_handle.h"

namespace {

constexpr size_t kAlign = 256;
constexpr size_t kScratchBytes = MM_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Device address of the scratch array on the current device (looked up once per device).
mm_status scratch_address(unsigned char** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_compute_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    mm::set_error("mm_compute_noalloc: device index " + std::to_string(dev) + " is beyond the " +
                  std::to_string(kMaxDevices) + " devices this entry point keeps addresses for");
    return MM_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      mm::set_error(std::string("mm_compute_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return MM_ERR_CUDA;
    }
    g_scratch_ptr[dev] = (unsigned char*)p;
  }
  *out = g_scratch_ptr[dev];
  return MM_OK;
}

void inverse3(const double* a, double* out, double* det) {
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

// Symmetric stress in Voigt order (00,11,22,12,02,01) as a linear map of the strain.
void stress_map(const double* C, double* A) {
  static const int P[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
  for (int p = 0; p < 6; ++p)
    for (int q = 0; q < 6; ++q) {
      const int i = P[p][0], j = P[p][1], k = P[q][0], l = P[q][1];
      double v = 0.5 * (C[((i * 3 + j) * 3 + k) * 3 + l] + C[((j * 3 + i) * 3 + k) * 3 + l]);
      if (k != l) v += 0.5 * (C[((i * 3 + j) * 3 + l) * 3 + k] + C[((j * 3 + i) * 3 + l) * 3 + k]);
      A[p * 6 + q] = v;
    }
}

// Status words at the start of the scratch array: [0] a cell type outside [0, ntypes)
// was seen, [1] a NaN was produced (set by the gather and finalize kernels).
constexpr int kStatusWords = 2;

// Cell types narrowed to bytes; an out-of-range type is stored as 0 (so nothing reads
// beyond the parameter table) and reported through bad[0].
__global__ void k_types_to_u8(int M, int ntypes, const int32_t* __restrict__ in, uint8_t* __restrict__ out,
                              int* __restrict__ bad) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M) return;
  const int32_t t = in[c];
  const bool ok = t >= 0 && t < ntypes;
  out[c] = ok ? (uint8_t)t : (uint8_t)0;
  if (!ok) atomicOr(bad, 1);
}

}  // namespace

extern "C" mm_status mm_compute_noalloc(const int32_t* lattice_shape, const int32_t* cell_type, int ntypes,
                                        const int32_t* nstates, const double* h0, const double* C,
                                        const double* free_energy, const double* temp_eff, const double* rvecs,
                                        int model, int precision, const double* pos, double* gpos, double* vtens,
                                        double* energy, void* stream) {
  if (!lattice_shape || !cell_type || !nstates || !h0 || !C || !free_energy || !temp_eff || !rvecs || !pos ||
      !energy) {
    mm::set_error("mm_compute_noalloc: missing argument");
    return MM_ERR_ARG;
  }
  if (ntypes < 1 || ntypes > MM_MAX_TYPES || (model != MM_MODEL_ORIGINAL && model != MM_MODEL_NANOCELL) ||
      (precision != MM_PREC_FP64 && precision != MM_PREC_FP32)) {
    mm::set_error("mm_compute_noalloc: bad ntypes/model/precision");
    return MM_ERR_ARG;
  }
  const long long ncells = (long long)lattice_shape[0] * lattice_shape[1] * lattice_shape[2];
  if (lattice_shape[0] < 2 || lattice_shape[1] < 2 || lattice_shape[2] < 2) {
    mm::set_error("mm_compute_noalloc: every lattice direction needs at least 2 cells");
    return MM_ERR_ARG;
  }
  if (ncells > MM_NOALLOC_MAX_CELLS) {
    mm::set_error("mm_compute_noalloc: lattice has " + std::to_string(ncells) + " cells; the static scratch holds " +
                  std::to_string(MM_NOALLOC_MAX_CELLS) + " at most");
    return MM_ERR_ARG;
  }
  for (int t = 0; t < ntypes; ++t)
    if (nstates[t] < 1 || nstates[t] > MM_MAX_STATES) {
      mm::set_error("mm_compute_noalloc: nstates out of range");
      return MM_ERR_ARG;
    }
  {
    // a call copies its parameters from host memory and synchronises the stream, neither of
    // which a stream capture allows
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t e = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
    if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
      (void)cudaGetLastError();
      mm::set_error("mm_compute_noalloc: the stream is being captured; calls cannot be captured");
      return MM_ERR_ARG;
    }
  }
  unsigned char* base = nullptr;
  mm_status s = scratch_address(&base);
  if (s != MM_OK) return s;

  // A stack-resident handle whose buffers are carved out of the scratch array.
  mm_handle h;
  h.N = h.M = (int)ncells;
  h.structured = 1;
  h.pbc = 1;
  h.model = model;
  h.prec = precision;
  h.ntypes = ntypes;
  for (int d = 0; d < 3; ++d) h.nn[d] = lattice_shape[d];
  {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&h.num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const size_t M = (size_t)ncells;
  const size_t esz = precision == MM_PREC_FP32 ? sizeof(float) : sizeof(double);
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += round_up(bytes);
    return p;
  };
  int* d_status = (int*)carve(kStatusWords * sizeof(int));
  h.d_u = (double*)carve(3 * M * sizeof(double));
  h.d_disp = carve(3 * M * esz);
  h.d_G = carve(24 * M * esz);
  h.d_cpart = (double*)carve((size_t)mm::cell_blocks(&h) * 10 * sizeof(double));
  h.d_cell_type = (uint8_t*)carve(M);
  h.d_tt = (mm::TypeTable*)carve(sizeof(mm::TypeTable) * MM_MAX_TYPES);
  h.d_box = (double*)carve(9 * sizeof(double));
  if (off > kScratchBytes) {  // cannot happen for ncells <= MM_NOALLOC_MAX_CELLS
    mm::set_error("mm_compute_noalloc: scratch layout exceeds the static array");
    return MM_ERR_ARG;
  }

  // parameter table and lattice matrix, built on the host stack
  mm::TypeTable tt[MM_MAX_TYPES];
  std::memset(tt, 0, sizeof(tt));
  const double kB = 1.3806505e-23 / 4.35974381e-18;
  for (int t = 0; t < ntypes; ++t) {
    tt[t].nstates = nstates[t];
    tt[t].kT = kB * temp_eff[t];
    for (int st = 0; st < MM_MAX_STATES; ++st) {
      const int slot = t * MM_MAX_STATES + (st < nstates[t] ? st : 0);
      std::memcpy(tt[t].s[st].h0, h0 + 9 * slot, 9 * sizeof(double));
      inverse3(tt[t].s[st].h0, tt[t].s[st].hinv, &tt[t].s[st].v0);
      stress_map(C + 81 * slot, tt[t].s[st].A);
      tt[t].s[st].df = free_energy[slot];
    }
  }
  h.simple = mm::tables_are_simple(tt, ntypes);
  double L[9];
  for (int d = 0; d < 3; ++d)
    for (int x = 0; x < 3; ++x) L[3 * d + x] = rvecs[3 * d + x] / lattice_shape[d];

  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(h.d_tt, tt, sizeof(tt), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.d_box, L, sizeof(L), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_compute_noalloc: parameter upload: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, kStatusWords * sizeof(int), st);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_compute_noalloc: parameter upload: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  // Types first: their verdict is read back before any kernel indexes the parameter table.
  k_types_to_u8<<<(int)((M + 255) / 256), 256, 0, st>>>((int)M, ntypes, cell_type, h.d_cell_type, d_status);
  int status[kStatusWords] = {0, 0};
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(status, d_status, sizeof(status), cudaMemcpyDeviceToHost, st);
  // This also waits for the parameter copies, which read host stack memory.
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_compute_noalloc: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  if (status[0]) {
    mm::set_error("mm_compute_noalloc: a cell type is outside [0, ntypes)");
    return MM_ERR_ARG;
  }
  mm::launch_pos_to_state(&h, pos, st);
  mm::launch_cells(&h, st, nullptr);
  if (gpos) mm::launch_gather(&h, gpos, d_status + 1, st);
  mm::launch_finalize(&h, energy, vtens, d_status + 1, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_compute_noalloc: launch: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  e = cudaMemcpyAsync(status, d_status, sizeof(status), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    mm::set_error(std::string("mm_compute_noalloc: ") + cudaGetErrorString(e));
    return MM_ERR_CUDA;
  }
  if (status[1]) {
    mm::set_error("mm_compute_noalloc: NaN in energy, gradient or virial");
    return MM_ERR_NAN;
  }
  return MM_OK;
}
