// Batched systems: host API (mm_batch_*). The persistent kernels live in
// mm_batch_dev.cuh (device code), mm_batch_md.cu and mm_batch_relax.cu.
#include "mm_batch_dev.cuh"

using namespace mmb;

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

mmb::BatchLaunch batch_launch(mm_batch* b) {
  mmb::BatchLaunch L;
  L.a = batch_args(b);
  L.bt = b->bt;
  L.nctas = b->nctas;
  L.prec = b->prec;
  L.model = b->model;
  L.simple = b->simple;
  return L;
}
void launch_md(mm_batch* b, const BMD& p, cudaStream_t st) { mmb::launch_md(batch_launch(b), p, st); }
void launch_relax(mm_batch* b, int max_iter, double gtol, cudaStream_t st) {
  mmb::launch_relax(batch_launch(b), max_iter, gtol, st);
}
void launch_relax_cell(mm_batch* b, const CellRelax& r, cudaStream_t st) {
  mmb::launch_relax_cell(batch_launch(b), r, st);
}

// Per-type parameter tables (rest matrices and their inverses, stress maps, free
// energies, kT) in b->tt, and the cubic-specialisation flag.
void fill_type_tables(mm_batch* b, const int32_t* nstates, const double* h0, const double* C,
                      const double* free_energy, const double* temp_eff) {
  for (int t = 0; t < b->ntypes; ++t) {
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
  b->simple = mm::tables_are_simple(b->tt, b->ntypes);
}

bool same_key(const BMD& x, const BMD& y) {
  return x.dt == y.dt && x.temp == y.temp && x.timecon == y.timecon && x.press == y.press && x.nsteps == y.nsteps &&
         x.thermo == y.thermo && x.baro == y.baro && x.bflags == y.bflags && x.bchain == y.bchain &&
         x.chain == y.chain && x.seed == y.seed && x.step0 == y.step0 && x.noise == y.noise && x.hnoise == y.hnoise &&
         x.rec == y.rec;
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
    y.div_nyz = mm::make_fastdiv((uint32_t)(y.ny * y.nz));
    y.div_nz = mm::make_fastdiv((uint32_t)y.nz);
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
  for (int t = 0; t < ntypes; ++t)
    if (nstates[t] < 1 || nstates[t] > MM_MAX_STATES) {
      batch_free(b);
      mm::set_error("mm_batch_create: nstates out of range");
      return MM_ERR_ARG;
    }
  fill_type_tables(b, nstates, h0, C, free_energy, temp_eff);
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
  // default: one system per CTA, longest first; the CTA scheduler then starts each
  // system as soon as a slot frees, which balances uneven step costs better than a
  // fixed assignment of several systems to each resident CTA
  if (!ok || batch_partition(b, nsys) != MM_OK) {
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
                      double press, int chain, uint64_t seed, int64_t step0, const double* noise,
                      const double* hook_noise, double* records, int use_graph, void* stream) {
  if (!b || nsteps < 0 || !(timestep > 0.0) || !hooks_valid(thermo, timecon, baro, chain)) {
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
  parse_baro(baro, p);  // kind and MTK options
  p.chain = chain;
  p.seed = seed;
  p.step0 = step0;
  p.noise = noise;
  p.hnoise = hook_noise;
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

mm_status mm_batch_set_params(mm_batch* b, const int32_t* nstates, const double* h0, const double* C,
                               const double* free_energy, const double* temp_eff) {
  if (!b || !nstates || !h0 || !C || !free_energy || !temp_eff) return MM_ERR_ARG;
  for (int t = 0; t < b->ntypes; ++t)
    if (nstates[t] < 1 || nstates[t] > MM_MAX_STATES) {
      mm::set_error("mm_batch_set_params: nstates out of range");
      return MM_ERR_ARG;
    }
  BCUDA(cudaDeviceSynchronize());
  fill_type_tables(b, nstates, h0, C, free_energy, temp_eff);
  BCUDA(cudaMemcpy(b->d_tt, b->tt, sizeof(b->tt), cudaMemcpyHostToDevice));
  if (b->graph) {  // a captured launch may have been built for the other specialisation
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return MM_OK;
}

mm_status mm_batch_relax(mm_batch* b, int max_iter, double gtol, void* stream) {
  if (!b || max_iter < 0 || !(gtol > 0.0)) return MM_ERR_ARG;
  launch_relax(b, max_iter, gtol, (cudaStream_t)stream);
  BCUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_batch_relax_cell(mm_batch* b, int max_iter, double gtol, double stol, double press, int full,
                              void* stream) {
  if (!b || max_iter < 0 || !(gtol > 0.0) || !(stol > 0.0) || !(press == press) || (full != 0 && full != 1)) {
    mm::set_error("mm_batch_relax_cell: bad argument");
    return MM_ERR_ARG;
  }
  CellRelax r;
  r.max_iter = max_iter;
  r.gtol = gtol;
  r.stol = stol;
  r.press = press;
  r.full = full;
  launch_relax_cell(b, r, (cudaStream_t)stream);
  BCUDA(cudaGetLastError());
  return MM_OK;
}

// Autotuner: times `probe_steps` MD steps for each CTA size (128, 256) and number of
// CTAs (1, 2, 4 per SM, or one per system; capped by the system count), restoring the
// state after every probe, and keeps the fastest configuration.
mm_status mm_batch_autotune(mm_batch* b, int probe_steps, double timestep, int thermo, double temp, double timecon,
                            int baro, double press, int chain, double* best_ms) {
  if (!b || probe_steps < 1 || !(timestep > 0.0) || !hooks_valid(thermo, timecon, baro, chain)) return MM_ERR_ARG;
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
  const int ctas[4] = {b->num_sms, 2 * b->num_sms, 4 * b->num_sms, b->nsys};
  for (int ib = 0; ib < 2; ++ib)
    for (int ip = 0; ip < 4; ++ip) {
      if (ip > 0 && std::min(b->nsys, ctas[ip]) == std::min(b->nsys, ctas[ip - 1])) continue;
      b->bt = bts[ib];
      mm_status s = batch_partition(b, std::min(b->nsys, ctas[ip]));
      if (s != MM_OK) return s;
      BMD p;
      p.dt = timestep;
      p.temp = temp;
      p.timecon = timecon;
      p.press = press;
      p.nsteps = probe_steps;
      p.thermo = thermo;
      parse_baro(baro, p);  // kind and MTK options
      p.chain = chain;
      p.seed = 12345u;
      p.step0 = 0;
      p.noise = nullptr;
      p.hnoise = nullptr;
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

mm_status mm_selftest_sym_exp(const double* S, int n, double f, double* r_thread, double* r_warp, void* stream) {
  if (n < 0 || (n > 0 && (!S || !r_thread || !r_warp))) {
    mm::set_error("mm_selftest_sym_exp: bad arguments");
    return MM_ERR_ARG;
  }
  if (n > 0) mmb::k_selftest_sym_exp<<<n, 32, 0, (cudaStream_t)stream>>>(S, n, f, r_thread, r_warp);
  BCUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_selftest_exp_small(const double* x, double* out, int n, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out))) {
    mm::set_error("mm_selftest_exp_small: bad arguments");
    return MM_ERR_ARG;
  }
  if (n > 0) mmb::k_selftest_exp_small<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(x, out, n);
  BCUDA(cudaGetLastError());
  return MM_OK;
}

mm_status mm_batch_config(mm_batch* b, int* cta_threads, int* nctas) {
  if (!b) return MM_ERR_ARG;
  if (cta_threads) *cta_threads = b->bt;
  if (nctas) *nctas = b->nctas;
  return MM_OK;
}

}  // extern "C"
