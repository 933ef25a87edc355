/*
 * micmec_gb300 — C ABI of the GB300-native MicMec force-evaluation and
 * integration path (one GPU, sm_103a).
 *
 * The reference (molmod/micmec) is a Python package; its force path is the
 * `ForcePart.compute(gpos, vtens)` call of micmec/pes/mmff.py:87-149 and the
 * Verlet loop of micmec/sampling/verlet.py:140-166. This library is what a
 * binding of that path calls (the package's micmec_gb300/_native.py binds it with
 * ctypes).
 *
 * Conventions
 *  - All quantities are in atomic units and FP64 at the boundary.
 *  - Arrays are C-contiguous; (N,3) means node-major xyz triples.
 *  - Pointers marked "device" are CUDA device pointers (e.g. torch tensors);
 *    "host" pointers are ordinary CPU memory.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Every call returns an mm_status. Calls that take a stream only enqueue
 *    work; results are valid after the stream is synchronised.
 *  - A handle is used from one host thread at a time.
 */
#ifndef MICMEC_GB300_H
#define MICMEC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MM_OK = 0,
  MM_ERR_NAN = 1,     /* NaN in energy, gradient or virial (reference: ValueError, mmff.py:135-148) */
  MM_ERR_ARG = 2,     /* invalid argument */
  MM_ERR_CUDA = 3,    /* CUDA runtime error */
  MM_ERR_TIMEOUT = 4, /* a bounded device-side wait ran out */
} mm_status;

enum { MM_MODEL_ORIGINAL = 0, MM_MODEL_NANOCELL = 1 };
enum { MM_PREC_FP64 = 0, MM_PREC_FP32 = 1 };
enum { MM_THERMO_NONE = 0, MM_THERMO_LANGEVIN = 1 };

/* Per-step MD record, MM_REC_LEN doubles per step (see mm_md_run). */
enum {
  MM_REC_EPOT = 0,      /* potential energy after the step */
  MM_REC_EKIN = 1,      /* kinetic energy after the step (after the "post" thermostat) */
  MM_REC_DECONS = 2,    /* change of the thermostat's conserved-energy correction during the step */
  MM_REC_VTENS = 3,     /* 9: virial tensor, row-major */
  MM_REC_KTENS = 12,    /* 9: kinetic tensor sum_i m_i v_i (x) v_i */
  MM_REC_LEN = 21
};

typedef struct mm_handle mm_handle;

/*
 * Create a system.
 *  nnodes, ncells      : N and M.
 *  node_coords (N,3)   : host, integer lattice coordinates (kk,ll,mm) of every node,
 *                        the reference's Grid.nodes (micmec/utils.py:113-136).
 *  cell_nodes  (M,8)   : host, reference `surrounding_nodes` (corner order of utils.py:43-52).
 *  node_cells  (N,8)   : host, reference `surrounding_cells` (-1 = no cell).
 *  cell_type   (M)     : host, 0-based index into the type table.
 *  lattice_shape[3]    : nodes per lattice direction (Grid.n?_nodes).
 *  pbc                 : 1 = 3-D periodic, 0 = isolated.
 *  ntypes, nstates[ntypes]
 *  h0 [ntypes*4][9], C [ntypes*4][81], free_energy [ntypes*4], temp_eff [ntypes]:
 *                        host, per (type, state) rest cell matrix (rows = cell vectors),
 *                        3x3x3x3 elasticity tensor, state free energy; per type the
 *                        effective temperature (kelvin). Slot (t, s) is t*4+s.
 *  masses (N)          : host, node masses.
 *  model               : MM_MODEL_*.  precision : MM_PREC_*.
 * Replaces: ForcePartMechanical.__init__ (micmec/pes/mmff.py:207-245), which reads
 * the same system arrays and type{k}/... parameters and builds a dense
 * minimum-image table (mmff.py:258-286); here the image shift is implicit in the
 * lattice coordinates.
 */
mm_status mm_create(int nnodes, int ncells, const int32_t* node_coords, const int32_t* cell_nodes,
                    const int32_t* node_cells, const int32_t* cell_type, const int32_t* lattice_shape,
                    int pbc, int ntypes, const int32_t* nstates, const double* h0, const double* C,
                    const double* free_energy, const double* temp_eff, const double* masses, int model,
                    int precision, mm_handle** out);

/* Release all device memory of a handle (no reference counterpart: Python frees the
   ForcePartMechanical's arrays). */
mm_status mm_destroy(mm_handle* h);

/*
 * Set the domain. rvecs (3,3) host, rows = domain vectors (periodic systems), or
 * NULL for an isolated system. `lattice` (3,3) host: the lattice matrix whose rows
 * are the node spacings along the three lattice directions; NULL = rvecs[d]/n_d.
 * Replaces: MicMecForceField.update_rvecs -> Domain.update_rvecs
 * (micmec/pes/mmff.py:191-193, micmec/pes/ext.pyx:52-72).
 */
mm_status mm_set_domain(mm_handle* h, const double* rvecs, const double* lattice);

/*
 * Energy, gradient and virial at positions pos (N,3).
 *  pos         : device (N,3).
 *  gpos        : device (N,3) or NULL; the gradient is ADDED to its contents.
 *  vtens       : device (3,3) or NULL; the virial is ADDED to its contents.
 *  energy      : device double[1]; the energy is WRITTEN.
 *  status_dev  : device int[1] or NULL; set to 1 if a NaN was produced.
 * Replaces: ForcePart.compute(gpos, vtens) for the "micmec" part
 * (micmec/pes/mmff.py:87-149, 288-323; the add-into semantics of mmff.py:143-148).
 */
mm_status mm_compute(mm_handle* h, const double* pos, double* gpos, double* vtens, double* energy,
                     int* status_dev, void* stream);

/*
 * Same as mm_compute with host buffers: copies pos in, runs, copies results back and
 * synchronises. gpos/vtens may be NULL. Returns MM_ERR_NAN if energy, gradient or
 * virial contain a NaN (the reference raises ValueError, mmff.py:135-148).
 */
mm_status mm_compute_host(mm_handle* h, const double* pos, double* gpos, double* vtens, double* energy);

/* Per-cell energies (M) and corner gradients (M,8,3) of the last compute: device outputs.
   The reference keeps the same arrays as ForcePartMechanical.epot_cells / gpos_cells
   (micmec/pes/mmff.py:243-244, 288-301). */
mm_status mm_cell_results(mm_handle* h, double* epot_cells, double* gpos_cells, void* stream);

/*
 * Velocity-Verlet MD on the device (micmec/sampling/verlet.py:119-166), optionally with
 * the Langevin thermostat applied before and after every step (nvt.py:196-218).
 *  pos, vel  : device (N,3); read at the start, overwritten with the final state.
 *  nsteps    : number of steps.
 *  timestep  : dt.   thermo : MM_THERMO_*.   temp, timecon : Langevin parameters.
 *  seed      : Philox seed for the Langevin noise.
 *  noise     : device (nsteps, 2, N, 3) standard normals to use instead of the
 *              generator (index 0 = "pre", 1 = "post"), or NULL.
 *  records   : device (nsteps, MM_REC_LEN) per-step observables, or NULL.
 *  step0     : index of the first step (counter0), used as the noise counter.
 */
mm_status mm_md_run(mm_handle* h, double* pos, double* vel, int nsteps, double timestep, int thermo,
                    double temp, double timecon, uint64_t seed, const double* noise, double* records,
                    int64_t step0, void* stream);

/*
 * MD session for step-by-step control (what mm_md_run does in one call):
 *  mm_md_begin   : load pos/vel (device (N,3)), evaluate the forces and start the
 *                  first step (step0 + 1). Parameters as mm_md_run.
 *  mm_md_advance : run nsteps steps; records as mm_md_run. With finish = 1 the last
 *                  step is completed without starting the next one (the state is
 *                  then a clean end-of-step state); with finish = 0 the next step is
 *                  already started, so further mm_md_advance calls continue seamlessly.
 *  mm_md_end     : write the end-of-step state to pos/vel (device (N,3)).
 * Replaces VerletIntegrator.initialize / propagate / the state read-back of a run
 * (micmec/sampling/verlet.py:119-166, iterative.py:74-100) when they are driven step by step.
 */
mm_status mm_md_begin(mm_handle* h, const double* pos, const double* vel, double timestep, int thermo, double temp,
                      double timecon, uint64_t seed, const double* noise, int64_t step0, void* stream);
mm_status mm_md_advance(mm_handle* h, int nsteps, double* records, int finish, void* stream);
mm_status mm_md_end(mm_handle* h, double* pos, double* vel, void* stream);

/*
 * MD with the hooks of mm_batch_md (thermo 0..4; the barostat codes of mm_batch_md, MTK
 * options included; the particle NHC with chain length 3)
 * for a system of any size spread over the whole GPU: the step of
 * VerletIntegrator.propagate (micmec/sampling/verlet.py:140-166) with TBCombination and
 * the thermostats and barostats (micmec/sampling/npt.py:52-757; nvt.py:110-274,
 * 361-532) as grid-wide kernels and one-thread controller kernels.
 *  pos, vel (N,3) device: in/out.   ctl_host double[MM_BATCH_CTL] host: hook constants
 *  and state in the layout of mm_batch_control (ndof, chain masses/positions/velocities,
 *  barostat mass/velocity/dof, conserved-energy corrections); returned updated. The
 *  lattice/domain part is taken from the handle and returned after the barostat moved it.
 *  records device (nsteps, MM_BATCH_REC) or NULL.  noise: as mm_md_run, or NULL.
 *  hook_noise: device (nsteps, 1, MM_HOOK_NOISE) as mm_batch_md, or NULL.
 */
mm_status mm_md_engine(mm_handle* h, double* pos, double* vel, int nsteps, double timestep, int thermo, double temp,
                       double timecon, int baro, double press, int chain, uint64_t seed, const double* noise,
                       const double* hook_noise, double* ctl_host, double* records, int64_t step0, void* stream);

/*
 * Measurement helper: run nsteps steps of the session like mm_md_advance(finish = 0),
 * with CUDA events around the cell kernel and the node kernel of every step, and
 * return the summed durations (ms). If flush_buf is given, flush_bytes of it are
 * overwritten before every step (outside the timed spans) to evict L2.
 * No reference counterpart (measurement only).
 */
mm_status mm_md_time_kernels(mm_handle* h, int nsteps, void* flush_buf, size_t flush_bytes, double* ms_cells,
                             double* ms_nodes, void* stream);

/*
 * One velocity-Verlet step with host buffers, the step of
 * VerletIntegrator.propagate (micmec/sampling/verlet.py:140-166) with an optional
 * Langevin thermostat before and after it (nvt.py:196-208):
 *  pos, vel (N,3) host : in/out.   gpos (N,3) host : in = gradient at pos, out = new gradient.
 *  record host double[MM_REC_LEN] or NULL; MM_REC_DECONS holds the "post" correction only.
 * Copies in, runs one force evaluation and the fused updates, copies out, synchronises.
 */
mm_status mm_md_step_host(mm_handle* h, double* pos, double* vel, double* gpos, double* record, double timestep,
                          int thermo, double temp, double timecon, uint64_t seed, int64_t step);

/*
 * Allocation-free force evaluation. No counterpart in the reference: it exists for
 * callers that cannot allocate device memory (code running inside another
 * framework's memory pool or a fixed-budget arena, plugins whose host owns every
 * device allocation, paths where an allocation would synchronise the device at the
 * wrong time), since mm_create allocates. It computes what mm_compute computes, for
 * a fully periodic lattice (every lattice site a node and a cell, nodes and cells
 * numbered as the reference's Grid does), and calls no cudaMalloc/cudaFree.
 *  lattice_shape[3]  : host, cells per direction (each >= 2), at most
 *                      MM_NOALLOC_MAX_CELLS cells in total (larger lattices: MM_ERR_ARG).
 *  cell_type (M)     : device int32, 0-based type index per cell; a type outside
 *                      [0, ntypes) is found on the device and returned as MM_ERR_ARG
 *                      before any energy is evaluated.
 *  ntypes, nstates, h0, C, free_energy, temp_eff : host, as mm_create.
 *  rvecs (3,3)       : host domain vectors.
 *  pos (N,3)         : device.  gpos (N,3), vtens (3,3): device or NULL, ADDED to.
 *  energy            : device double[1], written.
 * Working memory is one static device array of MM_NOALLOC_SCRATCH_BYTES bytes per
 * GPU, held until the process exits. The first call on a device looks up the
 * array's address; the address is kept for the process's life, so a process that calls
 * cudaDeviceReset does not use this entry point afterwards. Calls cannot be captured into
 * a CUDA graph (each copies its parameters from host memory and synchronises `stream`): a
 * call on a stream that is being captured returns MM_ERR_ARG. Calls share the array: calls that overlap on the GPU race. The
 * call synchronises `stream` before it returns. Returns MM_ERR_NAN when the energy,
 * gradient or virial holds a NaN (as mm_compute_host).
 */
#define MM_NOALLOC_MAX_CELLS 32768
#define MM_NOALLOC_SCRATCH_BYTES (8u << 20)
mm_status mm_compute_noalloc(const int32_t* lattice_shape, const int32_t* cell_type, int ntypes,
                             const int32_t* nstates, const double* h0, const double* C, const double* free_energy,
                             const double* temp_eff, const double* rvecs, int model, int precision,
                             const double* pos, double* gpos, double* vtens, double* energy, void* stream);

/*
 * Topology of a system from its grid of cell types, built on the device (the tables of
 * build_system, micmec/utils.py:164-263, with the reference's orderings: cells and nodes
 * lexicographic over grid coordinates, corner k = neighbor_nodes[k], node masses summed
 * in increasing cell order).
 *  grid      : device int32 (nx, ny, nz), last index fastest; 0 = vacancy, else a type id
 *              below ntype_ids (others: MM_ERR_ARG).
 *  pbc       : host int32[3].  type_mass : host double[ntype_ids] (index = type id).
 *  cell_size : host double[3], node spacing along x, y, z.
 *  Outputs (device), sized for every grid point; the first counts[0] cells and
 *  counts[1] nodes are valid: surrounding_nodes int64 (cells, 8), surrounding_cells
 *  int64 (nodes, 8; -1 = no cell) (both 16-byte aligned), masses double (nodes), pos double (nodes, 3),
 *  types int32 (cells), boundary uint8 (nodes; 1 on the node grid's faces).
 *  counts    : host int64[2] = (number of cells, number of nodes).
 */
mm_status mm_build_topology(const int32_t* grid, int nx, int ny, int nz, const int32_t* pbc, const double* type_mass,
                            int ntype_ids, const double* cell_size, int64_t* surrounding_nodes,
                            int64_t* surrounding_cells, double* masses, double* pos, int32_t* types,
                            uint8_t* boundary, int64_t* counts, void* stream);

/*
 * Batched systems: nsys independent, fully periodic lattices (every lattice site a
 * node and a cell) of uneven size, evaluated and integrated in one persistent launch
 * (one CTA runs whole systems). No single reference function corresponds: the
 * reference runs one System per Python process; this replaces many independent
 * runs of VerletIntegrator (micmec/sampling/verlet.py:140-166) with
 * TBCombination / LangevinThermostat / NHCThermostat / MTKBarostat hooks
 * (npt.py:52-177, 513-757; nvt.py:165-218, 361-532) and of an optimiser
 * (micmec/sampling/opt.py) over those systems.
 *  shapes (nsys,3)   : host, cells per direction of each system (each >= 2).
 *  cell_type (sum M) : host, 0-based type per cell, systems concatenated.
 *  masses (sum N)    : host, node masses, concatenated.
 *  Other parameters as mm_create.
 */
typedef struct mm_batch mm_batch;
mm_status mm_batch_create(int nsys, const int32_t* shapes, const int32_t* cell_type, int ntypes,
                          const int32_t* nstates, const double* h0, const double* C, const double* free_energy,
                          const double* temp_eff, const double* masses, int model, int precision, mm_batch** out);
mm_status mm_batch_destroy(mm_batch* b);
/* Host (sum N,3) positions, velocities (or NULL: zero) and (nsys,3,3) domain vectors: the
   System.pos / VerletIntegrator vel / Domain rvecs of each system (micmec/system.py). */
mm_status mm_batch_set_state(mm_batch* b, const double* pos, const double* vel, const double* rvecs);
mm_status mm_batch_get_state(mm_batch* b, double* pos, double* vel, double* rvecs);
/*
 * Per-system controller block, MM_BATCH_CTL doubles per system (host; write = 1 uploads,
 * 0 downloads): lattice matrix (0..8), domain vectors (9..17), volume (18), energy (19),
 * kinetic energy (20), virial (21..29), kinetic tensor (30..38), barostat velocity
 * tensor (39..47), chain positions (48..50), velocities (51..53), masses (54..56),
 * ndof (57), barostat mass (58), barostat dof (59), thermostat / barostat
 * conserved-energy corrections (60, 61), relaxation: largest gradient (62), iterations (63),
 * chain ndof (65; 0 = ndof), Langevin barostat time constant (66) and temperature (67),
 * the MTK barostat's own chain: positions (70..72), velocities (73..75), masses (76..78),
 * temperature (79).
 */
#define MM_BATCH_CTL 80
#define MM_BATCH_REC 31
mm_status mm_batch_control(mm_batch* b, double* ctl, int write);
/*
 * nsteps MD steps of every system. thermo: 0 none, 1 Langevin, 2 Nose-Hoover chain of
 * length `chain`, 3 Berendsen, 4 CSVR (no barostat); baro: 0 none, 1 MTK,
 * 2 Berendsen, 3 Langevin barostat, at pressure `press`, anisotropic unless baro |
 * MM_BARO_ISO (isotropic: the MTK and Langevin barostat velocity is the scalar at control
 * slot 39, the rest of the tensor zero; the Berendsen scaling a multiple of the identity) or
 * | MM_BARO_VOLC (volume constraint); for the MTK barostat also | MM_MTK_CHAIN |
 * (length << 8) (a Nose-Hoover chain of its own on the barostat velocity, length 1..3, state
 * at control slots 70..79; MTKBarostat(baro_thermo=...); micmec/sampling/npt.py:180-757). The
 * controller block must hold ndof, chain masses/state and ndof, barostat mass,
 * velocity, dof, and for the Langevin barostat its time constant and temperature (as
 * the reference's hook init sets them). noise (device, (nsteps, 2, sum N, 3)) replays
 * the Langevin thermostat's normals instead of the generator; hook_noise (device,
 * (nsteps, nsys, MM_HOOK_NOISE)) replays the CSVR thermostat's R and S and the Langevin
 * barostat's four unit-normal tensors per step (lower triangles 00, 10, 11, 20, 21,
 * 22); records (device, (nsys, nsteps, MM_BATCH_REC)): energy, kinetic energy,
 * conserved-energy correction, volume, virial(9), kinetic tensor(9), domain
 * vectors(9). use_graph: launch through a cached CUDA graph.
 * Replaces the loop of VerletIntegrator.run with its hooks (micmec/sampling/verlet.py:
 * 140-166; nvt.py:110-274, 361-532; npt.py:52-757).
 */
#define MM_HOOK_NOISE 26
#define MM_BARO_ISO 0x10
#define MM_BARO_VOLC 0x20
#define MM_MTK_CHAIN 0x40
mm_status mm_batch_md(mm_batch* b, int nsteps, double timestep, int thermo, double temp, double timecon, int baro,
                      double press, int chain, uint64_t seed, int64_t step0, const double* noise,
                      const double* hook_noise, double* records, int use_graph, void* stream);
/*
 * Replace the parameter tables of a batch (same layout as mm_batch_create): used by
 * parameter fits that relax or run many systems per parameter value. No reference
 * counterpart (the reference builds a new ForcePartMechanical, micmec/pes/mmff.py:207-245).
 */
mm_status mm_batch_set_params(mm_batch* b, const int32_t* nstates, const double* h0, const double* C,
                              const double* free_energy, const double* temp_eff);
/* Relax node positions of every system (domain fixed) until max |gradient| < gtol: the
   reference's CartesianDOF with an optimiser (micmec/sampling/opt.py:147-443), here
   Polak-Ribiere+ conjugate gradients with a secant line search. */
mm_status mm_batch_relax(mm_batch* b, int max_iter, double gtol, void* stream);
/*
 * Relax node positions and domain of every system together (the reference's
 * BaseCellDOF with CG/QN, micmec/sampling/dof.py:199-697, opt.py:147-443): full = 0
 * StrainCellDOF (rvecs = A rvecs0, A symmetric), full = 1 FullCellDOF (all nine domain
 * components); external pressure `press` adds E = P V (ForcePartPressure). Stops when
 * max |node gradient| < gtol and max |vtens / V + P I| < stol, or after max_iter
 * iterations; the controller block then holds the domain, energy, virial, the largest
 * gradient (62), iterations (63) and the largest residual stress (69).
 */
mm_status mm_batch_relax_cell(mm_batch* b, int max_iter, double gtol, double stol, double press, int full,
                              void* stream);
/* Choose the CTA size (128/256) and the CTA count (1, 2, 4 per SM or one per system; the default
   after mm_batch_create is one per system) by timing probe_steps MD steps (state restored).
   mm_batch_config reports the choice. No reference counterpart (launch configuration). */
mm_status mm_batch_autotune(mm_batch* b, int probe_steps, double timestep, int thermo, double temp, double timecon,
                            int baro, double press, int chain, double* best_ms);
mm_status mm_batch_config(mm_batch* b, int* cta_threads, int* nctas);

/*
 * Replace the parameters of a handle (same layout as mm_create): used by
 * differentiable parameter fits. No reference counterpart (the reference builds a
 * new ForcePartMechanical for new parameters, mmff.py:207-245).
 */
mm_status mm_set_params(mm_handle* h, const double* h0, const double* C, const double* free_energy,
                        const double* temp_eff);

/*
 * Adjoint evaluation in FP64 (forward-mode tangent along a node displacement field
 * lam and a lattice-matrix tangent dlattice, on top of the energy, gradient and
 * parameter gradient). Derivatives of the reference's energy model
 * (micmec/pes/nanocell.py:40-132, nanocell_original.py:46-132, mmff.py:377-398).
 *  pos (N,3) device; lam (N,3) device or NULL (zero); dlattice (3,3) host or NULL.
 *  energy  device double[2] : E, dE/dt along (lam, dlattice).
 *  gpos    device (N,3) or NULL : dE/dx.
 *  hvp     device (N,3) or NULL : d(dE/dx)/dt = H lam (+ lattice coupling).
 *  vtens   device double[18] or NULL : virial and its tangent.
 *  pgrad   device double[ntypes*4*46*2] or NULL : per (type, state) slot, 46 values
 *          [dE/dA (36, the 6x6 stress map of mm_create), dE/dh0 (9), dE/d(free energy)],
 *          each as (value, tangent): the tangent is d/dtheta (lam . dE/dx).
 */
mm_status mm_adjoint(mm_handle* h, const double* pos, const double* lam, const double* dlattice, double* energy,
                     double* gpos, double* hvp, double* vtens, double* pgrad, void* stream);

/* Last CUDA error string of the calling thread's last failing call (the reference raises
   Python exceptions instead; no counterpart). */
const char* mm_last_error(void);

/* Library version string (no reference counterpart). */
const char* mm_version(void);

/*
 * Self-test of the device-side FP64 <-> FP32 conversions the FP32 node update uses
 * (integer-pipe restatements of IEEE 754 round-to-nearest-even and exact widening):
 * dout[i] = (float)din[i], fout[i] = (double)fin[i] for i < n. All pointers device.
 * No reference counterpart (test support).
 */
mm_status mm_selftest_convert(const double* din, float* dout, const float* fin, double* fout, int n, void* stream);

/*
 * Self-test of the batch kernels' warp-parallel 3x3 algebra: the matrix exponential
 * R = exp(f S) of n row-major 3x3 matrices S (9 doubles each) by the one-thread form
 * (r_thread) and by the form with lane e of a warp forming entry e (r_warp); the two are
 * the same expressions in the same order and agree bit for bit. All pointers device.
 * No reference counterpart (test support).
 */
mm_status mm_selftest_sym_exp(const double* S, int n, double f, double* r_thread, double* r_warp, void* stream);

/*
 * Self-test of the exponential the hook algebra uses for its small arguments (a Taylor
 * polynomial to x^9 for |x| < 2^-5, the library exp otherwise): out[i] = exp(x[i]) for
 * i < n. All pointers device. No reference counterpart (test support).
 */
mm_status mm_selftest_exp_small(const double* x, double* out, int n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MICMEC_GB300_H */
