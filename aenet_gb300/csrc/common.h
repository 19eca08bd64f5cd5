// Shared definitions of the GB300 evaluator: device-side tables of the
// loaded potentials, per-structure geometry records and kernel launchers.
//
// Layout conventions (all device memory):
//   positions      double [N][3]   Cartesian, Angstrom
//   types          int    [N]      0-based global species index
//   neighbour table ELL with `cap` slots per atom:
//       nb_jt  int    [N*cap]  neighbour atom index | (species << AE_TYPE_SHIFT)
//       nb_vec T4     [N*cap]  (R_ij.x, R_ij.y, R_ij.z, |R_ij|), T = float|double
//       nb_cnt int    [N]      number of valid slots
//   descriptors    T      [N][nsf_pad]  normalised features
//   dE/dG          T      [N][nsf_pad]  scaled by E_scale and the
//                                       normalisation scale, so that the
//                                       adjoint contracts raw descriptor
//                                       derivatives with it
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define AE_MAXT 8            // species per potential set
#define AE_MAXNSF 160        // descriptor length
#define AE_MAXLAYERS 8       // network layers including input and output
#define AE_MAXNODES 64       // nodes per hidden layer
#define AE_MAXCHEB 32        // Chebyshev order + 1
#define AE_TYPE_SHIFT 26
#define AE_INDEX_MASK ((1 << AE_TYPE_SHIFT) - 1)
#define AE_MAXG4 64          // Behler angular functions per triple type
#define AE_MAXG2 64          // Behler radial functions per pair type
#define AE_MOMA 7            // angular functions (order + 1) of the moment form
// static shared memory a kernel may add to its dynamic allocation; the
// launchers opt in to large dynamic shared memory once the sum passes 48 KB
#define AE_STATIC_SMEM 1024

// status bits written by kernels into a device word
#define AE_ST_NB_OVERFLOW 1u
#define AE_ST_BAD_COORD 2u
#define AE_ST_BAD_TYPE 4u
#define AE_ST_CELL_OVERFLOW 8u
#define AE_ST_TC_TIMEOUT 16u     // a tensor-core wait ran out of iterations

enum { AE_SF_CHEBYSHEV = 1, AE_SF_BEHLER = 2 };

// ----------------------------------------------------------------------
// Potential tables
// ----------------------------------------------------------------------
struct ChebTable {
  double r_Rc, a_Rc;
  int r_N, a_N;     // number of radial / angular functions (order + 1)
  int multi;        // spin-weighted copy present
  int nsf;
  // feature offsets: [radial r_N][angular a_N][radial spin][angular spin]
  int r_i1, a_i1, r_i2, a_i2;
  float spin[AE_MAXT];          // typespin of each GLOBAL neighbour species
  int angular_legacy;           // T_n((2cos - pi)/pi) instead of T_n(cos)
};

struct BehlerFn {     // one radial (G1..G3) or angular (G4, G5) function
  double Rc, p1, p2, p3;  // G2: Rs, eta; G3: kappa; G4/G5: lambda, zeta, eta
  float fRc, fp1, fp2, fp3;   // the same parameters rounded to float
  int kind;               // 1..5
  int out;                // feature index (reference order)
  int izeta;              // zeta as an integer in [1, 64] when it is one, else 0
  int pad;
};

// The angular functions of one neighbour-species pair when they form a
// product grid: one kind (G4 or G5), one Rc, lambda = +-1, and every
// combination of nl (lambda, zeta) pairs with ne eta values present once.
// The kernels then evaluate per neighbour pair one exponential per eta and
// one power per (lambda, zeta) instead of one of each per function.
#define AE_BG_NL 16
#define AE_BG_NE 8
struct BehlerGrid {
  int kind;                           // 4 or 5
  int nl, ne;
  int pad;
  double Rc;
  double lam[AE_BG_NL], zeta[AE_BG_NL], eta[AE_BG_NE];
  float fRc;
  float flam[AE_BG_NL], fzeta[AE_BG_NL], feta[AE_BG_NE];
  int izeta[AE_BG_NL];                // zeta as an integer in [1, 64], else 0
  int out[AE_BG_NL * AE_BG_NE];       // feature index of (l, e): out[l * AE_BG_NE + e]
};

// Per central species: functions grouped by neighbour species (radial) and
// neighbour species pair (angular), with the feature index each feeds.
struct BehlerTable {
  int nsf;
  double rc_max;                      // largest Rc of any function
  int rad_off[AE_MAXT + 1];           // into fn[] by neighbour species
  int ang_off[AE_MAXT * AE_MAXT + 1]; // by (tj, tk) with tj <= tk
  int grid_of[AE_MAXT * AE_MAXT];     // index of the pair's BehlerGrid, or -1
  int grid_off;                       // byte offset of the BehlerGrid array
  int nfn;
  BehlerFn fn[1];                     // variable length (allocated larger)
};

struct NetTable {
  int nlayers;
  int nnodes[AE_MAXLAYERS];
  int f_a[AE_MAXLAYERS];              // activation of layer l (l >= 1)
  int w_off[AE_MAXLAYERS];            // offset of layer l -> l+1 weights
  int pitch[AE_MAXLAYERS];            // row pitch (odd) of layer l weights
  int wtotal;                         // padded weight count
};

struct SpeciesTable {
  int sftype;
  int nsf;
  double E_scale, E_shift, E_atom;
  ChebTable cheb;
  NetTable net;
  int behler_off;                     // byte offset of BehlerTable in blob
};

struct PotDevice {
  int ntypes;
  int nsf_max;
  int nsf_pad;                        // row stride of descriptor arrays
  double Rc_max;                      // neighbour cut-off (before +1e-3)
  SpeciesTable sp[AE_MAXT];
  // device pointers
  const double* shift;                // [ntypes][nsf_pad] normalisation
  const double* scale;                // [ntypes][nsf_pad]
  // the same constants for FP32 kernels: shift as an unevaluated sum
  // hi + lo of two floats (FP64 precision), scale rounded to float
  const float2* shift2;               // [ntypes][nsf_pad]
  const float* scale32;               // [ntypes][nsf_pad]
  const double* w64;                  // weights, row-major W[o][k], pitch
  const float* w32;
  const unsigned char* behler_blob;   // BehlerTable per species
  int behler_grid_only;               // every non-empty angular list is a BehlerGrid
  // tensor-core networks of the mixed path (two hidden layers): per species
  // an image of split-BF16 operand tiles and FP32 vectors (TcLayout)
  int tc_ok;                          // every species fits the tensor-core kernel
  int tc_kin, tc_h;                   // padded input and hidden widths (32 or 64)
  int tc_tanh;                        // every species: tanh hidden layers, linear output
  const unsigned char* tc_img;        // [ntypes][TcLayout::bytes]
  // angular terms in moment form (FP32 path): per species the Legendre
  // expansion T_n(x(c)) = sum_l q[n][l] P_l(c) of the angular basis in
  // c = cos(theta), [ntypes][AE_MOMA][AE_MOMA]; null when unavailable
  const float* qleg;
};

// Per-species image for the tensor-core networks.  Operand tiles are
// K-major in the canonical no-swizzle layout of the MMA shared-memory
// descriptor: 8 x 8 (rows x BF16) core matrices of 128 contiguous bytes,
// core matrices along K adjacent (leading byte offset 128), row blocks
// (K/8) * 128 bytes apart (stride byte offset).  Each operand is stored as
// a high part and a low part (x = hi + lo, both BF16), hi first.
//   B1  [h][kin]   layer-1 weights W1[o][k]
//   B2  [h][h]     layer-2 weights W2[o][k]
//   B2T [h][h]     W2 transposed (rows k, columns o) for the backward pass
//   B1T [kin][h]   W1 transposed
//   vec (FP32)     b1[h] b2[h] w3[h] nsc[kin] {b3, f_a1, f_a2, f_a3}
// Padded rows and columns are zero.
struct TcLayout {
  int kin, h;
  int b1, b2, b2t, b1t, vec, bytes;
};
__host__ __device__ inline TcLayout tc_layout(int kin, int h) {
  TcLayout L;
  L.kin = kin;
  L.h = h;
  L.b1 = 0;
  L.b2 = L.b1 + 4 * h * kin;
  L.b2t = L.b2 + 4 * h * h;
  L.b1t = L.b2t + 4 * h * h;
  L.vec = L.b1t + 4 * kin * h;
  L.bytes = L.vec + 4 * (3 * h + kin + 4);
  L.bytes = (L.bytes + 127) & ~127;
  return L;
}
// byte offset of element (r, k) of a K-major operand with K columns
__host__ __device__ inline int tc_core_offset(int r, int k, int K) {
  return ((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// ----------------------------------------------------------------------
// Structures of a batch
// ----------------------------------------------------------------------
struct StructGeom {
  double L[9];        // lattice vectors as rows: L[3*v + c]
  double B[9];        // reciprocal rows incl. 2 pi: s_v = (B[v].r)/(2 pi)
  double origin[3];   // isolated structures: corner of the binning box
  double box[3];      // isolated structures: edge lengths of the box
  float Lf[9];
  float hf[3];        // heights of the cell (periodic) or box edges
  float inv_nc[3];    // 1 / nc and 1 / hf, so the search kernels multiply
  float inv_hf[3];
  double rc2;         // (Rc + 1e-3)^2, the neighbour predicate
  float rc2_lo, rc2_hi;   // FP32 distances in [lo, hi] are decided in FP64
  float rcf;          // Rc + 1e-3 (pruning of the cell stencil)
  int pbc;
  int ortho;          // lattice vectors along x, y, z: stencil rows are pruned
  int frac_mode;      // 0: s = (B r)/(2 pi) (predict.x), 1: s = (B r)/(2 pi)
                      // with B without 2 pi (aenet_nbl_init), 2: input is s
  int nc[3];          // cell grid
  int kr[3];          // stencil half width per axis
  int cell_off;       // first cell of this structure in the global grid
  int atom_off, natoms;
  int chunk_off;      // first energy-reduction chunk (AE_ECHUNK atoms each)
};

#define AE_ECHUNK 2048      // atoms per chunk of the per-structure energy sum

// ----------------------------------------------------------------------
// launchers (defined in the .cu files)
// ----------------------------------------------------------------------
struct NbBuffers {
  const StructGeom* geom;
  const int* atom_struct;     // [N]
  double* s_wrap;             // [N][3] wrapped lattice coordinates
  double* r_wrap;             // [N][3] Cartesian of the wrapped coordinates
  float4* r_f32;              // [N] (x, y, z, species as int bits)
  int* cell_of;               // [N] packed cell coordinates cx|cy<<10|cz<<20
  int* slot_of;               // [N] rank of the atom inside its cell
  int* cell_count;            // [ncells_total]
  int* cell_start;            // [ncells_total + 1] exclusive prefix of counts
  int* scan_tmp;              // [scan blocks + 1]
  int* cell_atoms;            // [N] atoms in cell order
  float4* cell_pos;           // [N] r_f32 in cell order
  int ncells_total;
  int nstruc;
  int cap;                    // neighbour slots per atom
  int* nb_cnt;
  int* nb_jt;
  void* nb_vec;               // float4 or double4_32a
  int* nb_img;                // optional: image T packed 3 x 10-bit signed
  unsigned* status;
  cudaEvent_t ev_search;      // optional: recorded right before the search kernel
  // per-structure search (cell_kernel 4): structures largest first, and the
  // shared-memory capacity of one block (atoms, cells); null = unavailable
  const int* struct_order;
  int smem_atoms, smem_cells;
  // optional, per-structure search only: the search reads the caller's
  // 1-based type ids and writes the checked 0-based ones here (no separate
  // type kernel)
  int* types0_out;
  int ntypes;
  int cell_kernel;            // 0: warp per atom; warp per home cell with a lane per
                              // home atom (1) or a lane per candidate (2); 3: warp per
                              // atom over the half stencil, each pair written to both rows;
                              // 4: block per structure, cell lists in shared memory
};

int ae_launch_neighbors(int natoms, const double* pos, const int* types,
                        const NbBuffers& nb, int fp64, cudaStream_t s);
// ELL table from a caller's CSR neighbour list (local atoms, indices into
// local + ghost atoms)
int ae_launch_ell_from_csr(int nlocal, int nall, const double* x, const int* types1, int ntypes,
                           const int* offs, const int* nbr, double rc2, int cap, int* nb_cnt,
                           int* nb_jt, void* nb_vec, int fp64, unsigned* status, cudaStream_t s);

struct DescBuffers {
  int natoms;
  const int* types;
  const int* nb_cnt;
  const int* nb_jt;
  const void* nb_vec;
  int cap;
  int cap_a;                   // staged angular neighbours per atom
  int lpa;                     // lanes per atom of the descriptor kernels
  void* G;                     // [N][nsf_pad] (T)
  void* dEdG;                  // [N][nsf_pad] (T)
  double* E_atom;              // [N]
  void* F;                     // [N][4] (T) force accumulator (T=float: float4)
  double* virial;             // [nstruc][9] or null
  const int* atom_struct;
  const double* grad_scale;    // per structure factor on dE (or null = 1)
  unsigned* status;
  const void* U;               // [N] T4 per-atom directions of the tangent pass
  void* V;                     // [N][nsf_pad] (T) normalised descriptor tangents
  float* M;                    // [N][mom_pad] angular moments (FP32 moment form) or null
  int mom_pad;
  // angular spin weights as sfb_eval forms them (sfbasis.f90:514, 556):
  // the pair (j, k) of a row, j first in the reference's neighbour order,
  // weighs s_eff(j) s(k), where s_eff(j) is the spin of the last neighbour
  // up to j in that order inside the radial cut-off (1 before any).  Per
  // table slot: the rank in that order and s_eff; null = s(j) s(k).
  const int* nb_rank;          // [N*cap]
  const float* nb_seff;        // [N*cap]
};

// rank and stale spin of every slot of the neighbour table in the
// reference's lcl_nbdist_cart order (self images first, then atoms in
// ascending index, each with its home copy first and then the images in
// the order i3, i2, i1 with i1 fastest), or with caller_order in slot
// order (rows built from a caller's list); Chebyshev bases only.  geom,
// atom_struct and r_wrap are read only without caller_order.
int ae_launch_stale_order(int natoms, const StructGeom* geom, const int* atom_struct,
                          const double* r_wrap, const PotDevice& pd, const DescBuffers& b,
                          int fp64, int caller_order, int* rank, float* seff, cudaStream_t s);

int ae_launch_chebyshev_forward(const PotDevice& pd, const DescBuffers& b,
                                int fp64, cudaStream_t s);
// One FP64 Chebyshev atom per launch (the per-atom entry points): one
// block, or (cluster != 0) a cluster of eight blocks; the header comes as
// a launch argument, rows and outputs in mapped host memory.  Input: the
// header (also kept at the start of the block), then at
// AE_ATOM_IN_VEC the neighbour vectors (R_ij, |R_ij|) as double4[n] and
// their species (0-based) as int[n].  Output: E_i (double), status
// (unsigned), then at AE_ATOM_OUT_F the forces double[n + 1][3] (central
// atom first).  Returns AE_ATOM_NA when the potential or the row does not
// fit the kernel (Behler functions, larger orders, more than AE_ATOM_NMAX
// neighbours).
struct AtomCallHeader {
  int n;        // neighbours
  int ti;       // central species (0-based)
  int forces;   // 1: energy and forces, 0: energy only
  int pad;
};
#define AE_ATOM_IN_VEC 32
#define AE_ATOM_OUT_F 16
#define AE_ATOM_NMAX 512
#define AE_ATOM_NA (-2)
#define AE_ATOM_CLUSTER_ROWS 96   // rows from which the fused per-atom call takes the cluster
#define AE_ATOM_BLOCK_PAIRS 160   // angular pairs beyond which it takes the cluster (one
                                  // round of the one-block form's pair threads)
int ae_launch_atom(const PotDevice& pd, const AtomCallHeader& hd, const void* in, void* out,
                   int cluster, cudaStream_t s);
int ae_launch_chebyshev_adjoint(const PotDevice& pd, const DescBuffers& b,
                                int fp64, cudaStream_t s);
int ae_launch_chebyshev_tangent(const PotDevice& pd, const DescBuffers& b,
                                int fp64, cudaStream_t s);
// FP64 descriptor Jacobians of atoms [atom0, atom0 + count): dG/dR of the
// central atom [count][nsf_max][3] and of every neighbour slot
// [count][cap][nsf_max][3], the neighbours' atom indices [count][cap] and
// counts [count]
int ae_launch_chebyshev_jacobian(const PotDevice& pd, const DescBuffers& b, int atom0, int count,
                                 int nsf_max, double* Ji, double* Jj, int* nbl, int* nnb,
                                 cudaStream_t s);
int ae_launch_behler_jacobian(const PotDevice& pd, const DescBuffers& b, int atom0, int count,
                              int nsf_max, double* Ji, double* Jj, int* nbl, int* nnb,
                              cudaStream_t s);
int ae_launch_behler_forward(const PotDevice& pd, const DescBuffers& b,
                             int fp64, cudaStream_t s);
int ae_launch_behler_adjoint(const PotDevice& pd, const DescBuffers& b,
                             int fp64, cudaStream_t s);
int ae_launch_mlp(const PotDevice& pd, const DescBuffers& b, int fp64,
                  cudaStream_t s);
// tensor-core networks (mixed path); atoms grouped by species in `order`
int ae_launch_mlp_tc(const PotDevice& pd, const DescBuffers& b, const int* order,
                     const int* spec_off, cudaStream_t s);
int ae_fma_peak(double* tflops, cudaStream_t s);
int ae_launch_types(int natoms, const int* types1, int* types0, int ntypes,
                    unsigned* status, cudaStream_t s);
// per-structure energies: FP64 sums over chunks of AE_ECHUNK atoms (one
// warp each; chunk_struct[c] = structure of chunk c), then over each
// structure's chunks, in pairwise order
// one_chunk_each: every structure has 1 .. AE_ECHUNK atoms (the chunk pass
// then writes every total and the combining pass is skipped)
int ae_launch_energy_reduce_chunked(int nstruc, int nchunks, const StructGeom* geom,
                                    const int* chunk_struct, const double* E_atom, double2* part,
                                    double* E_struct, int one_chunk_each, cudaStream_t s);
int ae_launch_energy_reduce(int nstruc, const StructGeom* geom,
                            const double* E_atom, double* E_struct,
                            cudaStream_t s);
int ae_launch_forces_out(int natoms, const void* Facc, int fp64, double* F,
                         double sign, cudaStream_t s);

// training: species partition, loss, weight gradients (k_train.cu)
int ae_part_scratch_ints(int natoms);
int ae_launch_partition(int natoms, int ntypes, const int* types0, int* scratch, int* order,
                        int* spec_off, cudaStream_t s);
int ae_launch_loss(int nstruc, const StructGeom* geom, const double* E_struct, const double* E_tgt,
                   const void* Facc, const double* F_tgt, int mode, double wE, double wF,
                   double E_scale, double* cE, void* U, double* loss_s, double* loss, int fp64,
                   cudaStream_t s);
int ae_wgrad_wcap(const PotDevice& pd);
int ae_wgrad_nblk(int ntypes);
int ae_launch_mlp_wgrad(const PotDevice& pd, const int* order, const int* spec_off, const void* G,
                        const void* V, const int* atom_struct, const double* cE, double cF,
                        int physical, double* partial, double* grad, int fp64, cudaStream_t s);

// molecular dynamics (k_md.cu)
int ae_md_kick_drift(int n, double* pos, double* vel, const double* F, const double* invm,
                     double half_dt_acc, double dt, cudaStream_t s);
int ae_md_kick(int n, double* vel, const double* F, const double* invm, double half_dt_acc,
               cudaStream_t s);
int ae_md_displacement(int n, const double* pos, const double* rb, double lim2, int* flag,
                       cudaStream_t s);
int ae_md_after_build(int n, const double* pos, const double* r_wrap, double* S, double* rb,
                      cudaStream_t s);
int ae_md_refresh(int n, const StructGeom* geom, const int* atom_struct, const double* pos,
                  const double* S, int cap, const int* nb_cnt, const int* nb_jt, const int* nb_img,
                  void* nb_vec, int fp64, cudaStream_t s);
int ae_md_refresh_f32(int n, const StructGeom* geom, const int* atom_struct, const double* pos,
                      const double* S, float4* p32, int cap, const int* nb_cnt, const int* nb_jt,
                      const int* nb_img, void* nb_vec, cudaStream_t s);
int ae_md_ekin_blocks();
int ae_md_ekin(int n, const double* vel, const double* invm, double* part, double half_mass_unit,
               double* out, cudaStream_t s);
