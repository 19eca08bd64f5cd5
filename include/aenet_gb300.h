/*
 * aenet_gb300.h -- extensions of the libaenet C API for whole structures
 * and batches, served by the same library (libaenet_gb300.so) and the same
 * potential state as aenet.h.
 *
 * The reference evaluates one atom per call (src/aenet.f90:410-486) inside
 * predict.x's per-atom loop (src/predict.F90:574-706), with its own
 * linked-cell neighbour list (src/ext/lclist.f90).  These entry points take
 * whole structures instead: the neighbour search, descriptors, networks,
 * forces, virial and energy reduction all run on the GPU.
 *
 * Precision: AENET_GPU_FP64 evaluates everything in FP64 (the plain path,
 * parity with the reference to 1e-10 eV/atom); AENET_GPU_MIXED evaluates
 * descriptors, networks and forces in FP32 with the normalisation and the
 * per-structure energy sums in FP64.
 *
 * All arrays are plain C arrays; no function aborts the process.
 */
#ifndef AENET_GB300_H_INCLUDED
#define AENET_GB300_H_INCLUDED

#ifdef __cplusplus
extern "C" {
#endif

#define AENET_GPU_FP64 0
#define AENET_GPU_MIXED 1

/* additional status codes (the reference's 0..4 keep their meaning) */
#define AENET_ERR_CUDA 5       /* a CUDA call failed */
#define AENET_ERR_INPUT 6      /* invalid argument or non-finite coordinate */

/* run flags */
#define AENET_GPU_FORCES 1u
#define AENET_GPU_VIRIAL 2u

/* Options of the evaluator.  Keys:
 *   "angular_domain" = "current" | "legacy"
 *       current: T_n(cos theta) (src/ext/sfbasis.f90:825, 832);
 *       legacy : T_n((2 cos theta - pi)/pi), the mapping the Chebyshev
 *                potentials shipped with aenet were trained with.
 *   "cell_div" = "1" | "2" | "3"   cells per cut-off length in the
 *       neighbour search grid (performance only).
 *   "z_refine" = "1" .. "4"   the search cells are that many times narrower
 *       along the third lattice axis: the same stencil rows, each cut more
 *       finely to the cut-off sphere (performance only).
 *   "lanes_per_atom" = "8" | "16" | "32"   descriptor kernels' lanes per
 *       atom (performance only).
 *   "adjoint_lanes_per_atom" = "0" | "8" | "16" | "32"   the same for the
 *       adjoint kernels; 0 follows lanes_per_atom (performance only).
 *   "neighbour_kernel" = "atom" | "cell" | "stream" | "half" | "struct" |
 *       "struct_half"   neighbour
 *       search with one warp per atom (pruned per atom), one warp per home
 *       cell with a lane per home atom (dense cells of large structures),
 *       one warp per home cell with a lane per candidate, each batch of
 *       candidates tested against every home atom (few atoms per cell), or
 *       one warp per atom over half the stencil, each pair found once and
 *       written to both rows (the order inside a row then varies from run
 *       to run), or one block per structure with the structure's cell
 *       lists built in shared memory and warps taking its atoms in turn,
 *       over the full stencil (struct) or the half stencil with both rows
 *       written (struct_half; row order then varies from run to run)
 *       (batches of small structures; plans with fewer structures than
 *       twice the SMs, or whose largest structure does not fit a block,
 *       use the warp-per-atom search); same neighbour sets (performance
 *       only).
 *   "networks" = "tensor" | "simt"   mixed-path networks on the tcgen05
 *       tensor cores (split BF16, FP32 accumulation; networks with two
 *       hidden layers and widths up to 64) or on FP32 SIMT.
 *   "angular_terms" = "moments" | "pairs"   mixed-path angular Chebyshev
 *       terms from per-atom moments of real spherical harmonics (the pair
 *       sum rewritten by the addition theorem; cost linear in the angular
 *       neighbours, angular orders up to 6) or from the pair sum itself.
 *       Same values up to FP32 rounding; the FP64 path always sums pairs.
 *   "angular_spin" = "own" | "stale"   spin weights of the Chebyshev
 *       angular pairs (species-weighted bases).  own: s_j s_k.  stale: as
 *       sfb_eval forms them (src/ext/sfbasis.f90:514, 556), where s_j is
 *       refreshed only for neighbours inside the radial cut-off, so that
 *       with a_Rc > r_Rc a neighbour beyond r_Rc carries the spin of the
 *       last earlier neighbour inside it (1 before any).  The order is the
 *       caller's for aenet_atomic_energy(_and_forces) and
 *       aenet_gpu_neighbor_list_energy_forces, and for whole structures the
 *       order of the reference's lcl_nbdist_cart (the atom's own images,
 *       then the other atoms in ascending index, home copy before images).
 *       Pair form only (the moment form is skipped); applies to plans
 *       created afterwards; the force term of the training loss and the
 *       descriptor Jacobians need "own" (AENET_ERR_INPUT otherwise).
 *   "per_atom_kernel" = "fused" | "cluster" | "block" | "graph"
 *       aenet_atomic_energy(_and_forces) on Chebyshev potentials (orders up
 *       to 24 radial, 16 angular; up to 512 neighbours; angular_spin own):
 *       one launch evaluates the call, the row read from and the results
 *       written to mapped host memory, on a cluster of eight blocks that
 *       split the rows and pairs (cluster), on one block (block), or on
 *       one block for rows under 96 neighbours with at most 160 angular
 *       pairs and on a cluster otherwise (fused, the default); or the batch kernels run on a one-row table
 *       from a captured graph (graph; also what Behler potentials, stale
 *       spins and longer rows always take).  Same results to FP64
 *       rounding.
 * Returns AENET_OK or AENET_ERR_INPUT.  "cell_div" and "z_refine" apply to
 * plans created afterwards, "angular_domain" from the next evaluation (the
 * device tables are rebuilt), the others from the next launch. */
int aenet_gpu_set_option(const char* key, const char* value);

/* Energy and forces of one structure from HOST arrays.  Replaces the atom
 * loop of predict.x's get_energy (src/predict.F90:574-706): coords[3*natoms]
 * Cartesian, type_ids[natoms] 1-based, lattice[9] rows = lattice vectors
 * (ignored when pbc == 0: an isolated structure), precision
 * AENET_GPU_FP64 | AENET_GPU_MIXED.  Outputs (any may be NULL): *E_total
 * (sum of atomic energies including free-atom energies), *E_coh (minus the
 * free-atom energies), E_atoms[natoms], F[3*natoms] (overwritten),
 * virial[9] (W_ab = -dE/d(strain_ab), eV). */
void aenet_gpu_structure_energy_forces(int natoms, const double* coords,
                                       const int* type_ids,
                                       const double* lattice, int pbc,
                                       int precision, double* E_total,
                                       double* E_coh, double* E_atoms,
                                       double* F, double* virial, int* stat);

/* Batched evaluation with HOST arrays: nstruc structures packed
 * back-to-back (natoms[s] atoms each), lattices[9*nstruc], pbc[nstruc].
 * E[nstruc] total energies, F[3*sum natoms], virial[9*nstruc] (optional). */
void aenet_gpu_batch_energy_forces(int nstruc, const int* natoms,
                                   const double* coords, const int* type_ids,
                                   const double* lattices, const int* pbc,
                                   int precision, double* E, double* F,
                                   double* virial, int* stat);

/* ---- device-resident plans (stream ordered, no allocation per run) ----
 * A plan fixes the batch layout (structure sizes, cells, pbc) and owns the
 * device workspace.  Runs read positions and write results in DEVICE
 * memory on the given CUDA stream and may be captured in a CUDA graph. */
typedef struct aenet_gpu_plan aenet_gpu_plan;

/* coords0 (host, may be NULL for periodic batches) gives the initial
 * positions used to size the binning boxes of isolated structures. */
aenet_gpu_plan* aenet_gpu_plan_create(int nstruc, const int* natoms,
                                      const double* lattices, const int* pbc,
                                      const double* coords0, int precision,
                                      int* stat);
void aenet_gpu_plan_destroy(aenet_gpu_plan* plan);
int aenet_gpu_plan_natoms(const aenet_gpu_plan* plan);
/* Replace the lattice of every structure (host array, 9*nstruc); the cell
 * grids must stay within the capacities chosen at creation. */
int aenet_gpu_plan_set_lattices(aenet_gpu_plan* plan, const double* lattices);

/* Full pass: neighbours, descriptors, networks, energies and (flags)
 * forces / virial.  d_coords[3*N] (double), d_types[N] (int, 1-based);
 * outputs in device memory, any may be NULL: d_E[nstruc], d_E_atoms[N],
 * d_F[3*N] (double, overwritten), d_virial[9*nstruc]. */
int aenet_gpu_plan_run(aenet_gpu_plan* plan, const double* d_coords,
                       const int* d_types, double* d_E, double* d_E_atoms,
                       double* d_F, double* d_virial, unsigned flags,
                       void* stream);

/* Split pass for automatic differentiation: forward computes energies and
 * keeps dE/dG; backward then writes d_grad[3*N] = sum_s w[s] dE_s/dR
 * (w = d_weights[nstruc], device, NULL = all ones) and optionally the
 * virial of the weighted energy. */
int aenet_gpu_plan_forward(aenet_gpu_plan* plan, const double* d_coords,
                           const int* d_types, double* d_E,
                           double* d_E_atoms, void* stream);
int aenet_gpu_plan_backward(aenet_gpu_plan* plan, const double* d_weights,
                            double* d_grad, double* d_virial, void* stream);

/* The full pass with forces, with CUDA events recorded on `stream` between
 * the stages; ms[8] receives the stage durations in milliseconds: type
 * check, neighbour search (cell lists and search), descriptor, networks,
 * energy reduction, adjoint, force output, and last the search kernel
 * alone (part of the second entry).  Synchronises the stream. */
int aenet_gpu_plan_profile(aenet_gpu_plan* plan, const double* d_coords,
                           const int* d_types, double* d_E, double* d_F,
                           float* ms, void* stream);

/* Measured FP32 FMA throughput of the current device in TFLOP/s (a
 * dependent-chain-free FMA loop over every SM); the denominator of the
 * FP32 roofline of the descriptor kernels. */
int aenet_gpu_measure_fp32_peak(double* tflops, void* stream);

/* Device status word of a plan: 0, or the AENET_GPU_ST_* bits raised by
 * its runs since it was created (the word is not cleared between
 * aenet_gpu_plan_run calls, so one read after several runs covers them
 * all; create a new plan, or use the host-buffer entry points, which clear
 * it per call, for a per-run status). */
#define AENET_GPU_ST_NB_OVERFLOW 1u
#define AENET_GPU_ST_BAD_COORD 2u
#define AENET_GPU_ST_BAD_TYPE 4u
#define AENET_GPU_ST_CELL_OVERFLOW 8u
#define AENET_GPU_ST_TC_TIMEOUT 16u   /* a tensor-core wait gave up (results invalid) */
unsigned aenet_gpu_plan_status(aenet_gpu_plan* plan, void* stream);

/* Neighbour table of the last run (device pointers, for inspection and
 * tests): cap slots per atom, counts[N], packed index|species<<26, and
 * (x, y, z, distance) vectors as double4 (FP64 plans) or float4. */
int aenet_gpu_plan_neighbors(aenet_gpu_plan* plan, int* cap,
                             const int** d_counts, const int** d_jt,
                             const void** d_vec);

/* Descriptor of the last forward (device, [N][nsf_pad], double for FP64
 * plans, float for mixed) and its row stride. */
int aenet_gpu_plan_descriptors(aenet_gpu_plan* plan, const void** d_G,
                               int* nsf_pad);

/* ---- training ---------------------------------------------------------
 * Loss of a batch against target energies (and forces) and its gradient
 * with respect to every network weight, in one stream-ordered pass.
 * Replaces eval_next_structure / eval_net (src/train.f90:799-916) with
 * ff_wderiv (src/ext/feedforward.f90:763-860) and the accumulation of
 * src/optimize.f90:698-734.
 *
 * mode AENET_GPU_LOSS_ENERGY: the reference's loss,
 *     SSE = sum_s dE_s^2 / 2,  dE_s = (E_target,s - E_s) / (E_scale N_s),
 *     gradient sum_s dE_s Dw_s, Dw_s = -sum_{i in s} dy_i/dw / N_s
 *     (y: network output in normalised units; w_E, w_F ignored; every
 *     species must share E_scale, as potentials trained together do).
 * mode AENET_GPU_LOSS_ENERGY_FORCES (no counterpart in the reference,
 *     whose force training is not implemented, train.f90:812-813):
 *     L = w_E sum_s (E_s - E_target,s)^2 / N_s^2
 *       + w_F sum_i |F_i - F_target,i|^2   (eV, Angstrom);
 *     the force term is differentiated exactly (Chebyshev bases only).
 * Device arrays: d_E_target[nstruc] total energies, d_F_target[3N] (mode
 * 2 with w_F != 0), *d_loss, d_grad[sum over species of Wsize] ordered
 * like aenet_gpu_get_weights; d_E[nstruc] and d_F[3N] (optional) receive
 * the energies and forces of the same pass. */
#define AENET_GPU_LOSS_ENERGY 1
#define AENET_GPU_LOSS_ENERGY_FORCES 2
int aenet_gpu_plan_loss_gradient(aenet_gpu_plan* plan, const double* d_coords,
                                 const int* d_types, const double* d_E_target,
                                 const double* d_F_target, int mode, double w_E,
                                 double w_F, double* d_loss, double* d_grad,
                                 double* d_E, double* d_F, void* stream);

/* Training from stored descriptors (aenet training-set files hold the
 * normalised descriptors of every atom, src/trainset.f90): load them into a
 * plan (HOST G[N][ld], ld >= aenet_nsf_max, atom order of the plan), then
 * evaluate the reference's energy loss and gradient from them
 * (AENET_GPU_LOSS_ENERGY semantics; d_E_target are total energies in eV)
 * without positions or a neighbour search. */
int aenet_gpu_plan_load_descriptors(aenet_gpu_plan* plan, const double* G, int ld);

/* Descriptor Jacobians for generate.x's PyTorch export (sfderiv_i and
 * sfderiv_j of stp_eval, written by pyo_write_atom_sf_info,
 * src/pytorchoutput.f90:104-138): raw (unnormalised) FP64 derivatives of
 * the Chebyshev descriptors of atoms [atom0, atom0 + count) with respect to
 * the central atom, d_dG_i[count][nsf_max][3], and to each neighbour slot,
 * d_dG_j[count][cap][nsf_max][3]; d_nbl[count][cap] the neighbours' 0-based
 * atom indices in the batch (periodic images repeat an index), d_nnb[count]
 * the neighbour counts.  Reads the neighbour table of the plan's last run
 * (aenet_gpu_plan_run or _forward), so call it after one; FP64 plans only
 * (AENET_ERR_INPUT otherwise), Chebyshev or Behler bases.  nsf_max is
 * aenet_nsf_max, cap the value of aenet_gpu_plan_neighbour_capacity. */
int aenet_gpu_plan_neighbour_capacity(const aenet_gpu_plan* plan);
int aenet_gpu_plan_descriptor_jacobian(aenet_gpu_plan* plan, int atom0, int count,
                                       double* d_dG_i, double* d_dG_j, int* d_nbl,
                                       int* d_nnb, void* stream);
int aenet_gpu_plan_descriptor_loss_gradient(aenet_gpu_plan* plan, const int* d_types,
                                            const double* d_E_target, double* d_loss,
                                            double* d_grad, double* d_E, void* stream);

/* Network weights of all species, concatenated in type order, each the
 * reference's W(1:Wsize) (src/ext/feedforward.f90:55-89, the order
 * opt_bfgs_weights flattens them in, src/optimize.f90:1731-1737).
 * aenet_gpu_network_nweights returns Wsize of one species (-1 if not
 * loaded).  aenet_gpu_set_weights updates the device copies in place:
 * existing plans and captured graphs use the new weights. */
int aenet_gpu_network_nweights(int type_id);
int aenet_gpu_get_weights(double* W);
int aenet_gpu_set_weights(const double* W);
/* Write one species' potential with its current weights (.nn, the record
 * layout it was read with). */
int aenet_gpu_save_potential(int type_id, const char* filename);

/* ---- caller's neighbour lists (MD engines) --------------------------------
 * Energy and forces from the caller's full neighbour list, the interface an
 * MD engine with its own domain decomposition (LAMMPS-style local + ghost
 * atoms) needs: the engine keeps its neighbour lists, this evaluates the
 * potential on the GPU.  HOST arrays:
 *   x[3*nall]          positions of the nlocal local atoms, then the ghosts
 *   type_ids[nall]     1-based type ids
 *   neigh_offset[nlocal+1], neighbors[neigh_offset[nlocal]]
 *                      CSR lists of each local atom's neighbours (indices
 *                      into 0 .. nall-1, the atom itself excluded); pairs
 *                      beyond Rc_max + 1e-3 are ignored, so lists built
 *                      with a skin work as they are
 * Outputs (may be NULL): *E_total (local atoms), E_atoms[nlocal],
 * F[3*nall] forces on local AND ghost atoms (the engine adds the ghost
 * forces to their owners), virial[9] of the local atoms' energy.
 * Synchronous; returns an AENET status. */
int aenet_gpu_neighbor_list_energy_forces(int nlocal, int nall, const double* x,
                                          const int* type_ids,
                                          const int* neigh_offset,
                                          const int* neighbors, int precision,
                                          double* E_total, double* E_atoms,
                                          double* F, double* virial);

/* ---- molecular dynamics -------------------------------------------------
 * Velocity-Verlet NVE dynamics of one periodic structure with the loaded
 * potentials, every step on the GPU (the integration ASE's VelocityVerlet
 * performs in python3/scripts/aenet-md.py:72-97, here without ASE and
 * without a host round trip per step).  Units: coords A, velocities A/fs,
 * masses[ntypes] amu by type id, dt fs; forces eV/A, energies eV.
 * Neighbour lists use a Verlet skin: built with Rc + skin and rebuilt when
 * an atom has moved more than skin/2 (skin 0: rebuilt every step).
 * precision AENET_GPU_MIXED or AENET_GPU_FP64 (the integration itself is
 * FP64 in both).  Not thread-safe per object. */
typedef struct aenet_gpu_md aenet_gpu_md;
aenet_gpu_md* aenet_gpu_md_create(int natoms, const double* lattice,
                                  const double* coords, const double* velocities,
                                  const int* type_ids, const double* masses,
                                  double dt, double skin, int precision,
                                  int* stat);
void aenet_gpu_md_destroy(aenet_gpu_md* md);
/* nsteps steps; *E_pot, *E_kin (may be NULL) after the last one */
int aenet_gpu_md_run(aenet_gpu_md* md, int nsteps, double* E_pot, double* E_kin);
/* host copies of the current state (any may be NULL) */
int aenet_gpu_md_get(aenet_gpu_md* md, double* coords, double* velocities,
                     double* forces);
/* device time (ms) of the force part of the steps so far, split into
 * steps that rebuilt the neighbour table and steps that refreshed the
 * stored pair vectors (each includes descriptors, networks and forces) */
int aenet_gpu_md_phase_times(aenet_gpu_md* md, double* build_ms, long long* build_steps,
                             double* refresh_ms, long long* refresh_steps);
/* steps taken and neighbour-table builds so far */
int aenet_gpu_md_counters(aenet_gpu_md* md, long long* steps, int* builds);
/* plain FP64 energy of the current positions (the mixed run's monitor) */
int aenet_gpu_md_energy_fp64(aenet_gpu_md* md, double* E);

/* ---- evaluation without device memory allocation ---------------------
 * No counterpart in the reference (aenet runs on the CPU and allocates its
 * work arrays per call).  For callers that cannot allocate device memory
 * while they run -- MD engines that reserve all GPU memory at start-up and
 * forbid cudaMalloc in the time loop, plugins whose host application owns
 * the memory pool -- this computes the energy and forces of ONE periodic
 * structure using only the caller's device buffers plus a fixed scratch
 * array compiled into the library (about 19.3 MiB per GPU, held until the
 * process exits).
 *
 * Inputs (device): d_coords[3*natoms] Cartesian, d_types[natoms] 1-based;
 * lattice[9] (HOST) rows = lattice vectors.  Outputs (device, any may be
 * NULL): *d_E total energy, d_F[3*natoms], d_virial[9], *d_status (the
 * AENET_GPU_ST_* word of this run).  Work is queued on `stream`; the call
 * returns without synchronising.
 *
 * Limits: natoms <= AENET_NOALLOC_MAX_ATOMS, at most
 * AENET_NOALLOC_MAX_NEIGHBORS neighbours per atom (more sets
 * AENET_GPU_ST_NB_OVERFLOW in *d_status), at most AENET_NOALLOC_MAX_CELLS
 * neighbour-grid cells; larger inputs return AENET_ERR_MALLOC at once.
 * The potentials must be loaded and one allocating evaluation must have
 * run first (it builds the device tables): otherwise AENET_ERR_INIT.
 * The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the one scratch array: calls that overlap on the GPU
 * (different streams, threads) race and give wrong results.  The call
 * reads the loaded potentials' device tables: do not load, reload or
 * release potentials while calls are queued or running.
 * Kernels: the one-warp-per-atom neighbour search on the unrefined grid,
 * the pair form of the angular terms and the SIMT networks (the options
 * neighbour_kernel, z_refine, angular_terms, angular_spin and networks do
 * not apply; mixed results differ from aenet_gpu_structure_energy_forces
 * by FP32 rounding).  Angular neighbours are staged up to a count sized
 * from the structure's density (at most AENET_NOALLOC_MAX_NEIGHBORS);
 * more set AENET_GPU_ST_NB_OVERFLOW. */
#define AENET_NOALLOC_MAX_ATOMS 2048
#define AENET_NOALLOC_MAX_NEIGHBORS 192
#define AENET_NOALLOC_MAX_CELLS 65536
int aenet_gpu_structure_energy_forces_noalloc(int natoms, const double* d_coords,
                                              const int* d_types,
                                              const double* lattice,
                                              int precision, double* d_E,
                                              double* d_F, double* d_virial,
                                              unsigned* d_status, void* stream);

#ifdef __cplusplus
}
#endif

#endif
