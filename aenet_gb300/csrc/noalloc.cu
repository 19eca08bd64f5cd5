// Energy and forces of one periodic structure without any device memory
// allocation.
//
// Who needs this: codes that must not call cudaMalloc once they run --
// molecular-dynamics engines that set up all device memory at start-up and
// forbid allocation inside the time loop (allocation can synchronise the
// device or fail after fragmentation), and plugin environments whose host
// application owns the device memory pool.  They pass device buffers for
// the inputs and outputs; everything else the pass needs lives in one
// file-scope __device__ array of fixed size that every GPU loading this
// library holds until the process exits.
//
// Limits: AENET_NOALLOC_MAX_ATOMS atoms, AENET_NOALLOC_MAX_NEIGHBORS
// neighbours per atom, AENET_NOALLOC_MAX_CELLS cells of the neighbour
// grid; larger inputs are rejected with AENET_ERR_MALLOC before anything
// is launched.
//
// Kernels: the neighbour search with one warp per atom on the unrefined
// grid, the pair form of the angular terms, the SIMT networks; the options
// neighbour_kernel, z_refine, angular_terms, angular_spin and networks do
// not apply (each neighbour carries its own spin), so mixed-precision
// results differ from aenet_gpu_structure_energy_forces by FP32 rounding
// only.  The staged angular neighbours per atom follow the structure's
// density (as the plans do, at most the neighbour limit) and the lanes per
// atom of the descriptor kernels are raised when their shared memory would
// not fit.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "../../include/aenet_gb300.h"
#include "common.h"

int ae_device_tables(PotDevice* out, double* rc, int* cell_div);
int ae_lanes_per_atom();
int ae_periodic_geom(StructGeom* G, const double* lattice, int natoms, double rc, int cell_div);

namespace {

// status codes of include/aenet.h (exported there as variables)
constexpr int ST_OK = 0;
constexpr int ST_ERR_MALLOC = 2;

constexpr size_t NA_ATOMS = AENET_NOALLOC_MAX_ATOMS;
constexpr size_t NA_NB = AENET_NOALLOC_MAX_NEIGHBORS;
constexpr size_t NA_CELLS = AENET_NOALLOC_MAX_CELLS;

constexpr size_t up(size_t x) { return (x + 255) & ~size_t(255); }

// fixed layout of the scratch array (sizes for the largest precision)
constexpr size_t O_GEOM = 0;
constexpr size_t O_AS = O_GEOM + up(sizeof(StructGeom));
constexpr size_t O_T0 = O_AS + up(4 * NA_ATOMS);
constexpr size_t O_S = O_T0 + up(4 * NA_ATOMS);
constexpr size_t O_R = O_S + up(24 * NA_ATOMS);
constexpr size_t O_RF = O_R + up(24 * NA_ATOMS);
constexpr size_t O_CO = O_RF + up(16 * NA_ATOMS);
constexpr size_t O_SO = O_CO + up(4 * NA_ATOMS);
constexpr size_t O_CC = O_SO + up(4 * NA_ATOMS);
constexpr size_t O_CS = O_CC + up(4 * NA_CELLS);
constexpr size_t O_SC = O_CS + up(4 * (NA_CELLS + 1));
constexpr size_t O_CA = O_SC + up(4 * (NA_CELLS / 1024 + 2));
constexpr size_t O_CP = O_CA + up(4 * NA_ATOMS);
constexpr size_t O_NC = O_CP + up(16 * NA_ATOMS);
constexpr size_t O_JT = O_NC + up(4 * NA_ATOMS);
constexpr size_t O_VEC = O_JT + up(4 * NA_ATOMS * NA_NB);
constexpr size_t O_G = O_VEC + up(32 * NA_ATOMS * NA_NB);
constexpr size_t O_DG = O_G + up(8 * AE_MAXNSF * NA_ATOMS);
constexpr size_t O_EA = O_DG + up(8 * AE_MAXNSF * NA_ATOMS);
constexpr size_t O_F = O_EA + up(8 * NA_ATOMS);
constexpr size_t O_ES = O_F + up(32 * NA_ATOMS);
constexpr size_t O_V = O_ES + up(8);
constexpr size_t O_ST = O_V + up(72);
constexpr size_t SCRATCH_BYTES = O_ST + up(16);

// The scratch itself.  Host code must not take its address directly (on
// the host the name refers to a stand-in, not device memory): the device
// address comes from cudaGetSymbolAddress, once per device.
__device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_na_mu;
void* g_na_ptr[MAX_DEVICES] = {nullptr};

__global__ void k_store_geom(StructGeom* dst, StructGeom g) { *dst = g; }

}  // namespace

extern "C" __attribute__((visibility("default"))) int aenet_gpu_structure_energy_forces_noalloc(
    int natoms, const double* d_coords, const int* d_types, const double* lattice, int precision,
    double* d_E, double* d_F, double* d_virial, unsigned* d_status, void* stream) {
  if (natoms < 1 || !d_coords || !d_types || !lattice) return AENET_ERR_INPUT;
  if ((size_t)natoms > NA_ATOMS) return ST_ERR_MALLOC;
  PotDevice pd;
  double rc = 0.0;
  int cell_div = 2;
  int st = ae_device_tables(&pd, &rc, &cell_div);
  if (st) return st;
  if (pd.nsf_pad > AE_MAXNSF) return ST_ERR_MALLOC;
  // per-device set-up: the device address of the scratch array
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return AENET_ERR_CUDA;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return AENET_ERR_CUDA;
      g_na_ptr[dev] = p;
    }
    base = g_na_ptr[dev];
  }
  StructGeom G;
  st = ae_periodic_geom(&G, lattice, natoms, rc, cell_div);
  if (st) return st;
  const size_t ncells = (size_t)G.nc[0] * G.nc[1] * G.nc[2];
  if (ncells > NA_CELLS) return ST_ERR_MALLOC;
  G.cell_off = 0;
  G.atom_off = 0;
  const int fp64 = precision == AENET_GPU_FP64 ? 1 : 0;
  const size_t tsz = fp64 ? 8 : 4;
  cudaStream_t s = (cudaStream_t)stream;
  char* b = (char*)base;
  StructGeom* geom = (StructGeom*)(b + O_GEOM);
  int* atom_struct = (int*)(b + O_AS);
  int* types0 = (int*)(b + O_T0);
  unsigned* status = (unsigned*)(b + O_ST);
  double* E_struct = (double*)(b + O_ES);
  double* virial = (double*)(b + O_V);
  void* Facc = b + O_F;
  // what must start at zero: the previous call's contents stay in the array
  k_store_geom<<<1, 1, 0, s>>>(geom, G);
  if (cudaMemsetAsync(atom_struct, 0, 4 * (size_t)natoms, s) != cudaSuccess) return AENET_ERR_CUDA;
  if (cudaMemsetAsync(status, 0, 4, s) != cudaSuccess) return AENET_ERR_CUDA;
  int e = ae_launch_types(natoms, d_types, types0, pd.ntypes, status, s);
  NbBuffers nb{};
  nb.geom = geom;
  nb.atom_struct = atom_struct;
  nb.s_wrap = (double*)(b + O_S);
  nb.r_wrap = (double*)(b + O_R);
  nb.r_f32 = (float4*)(b + O_RF);
  nb.cell_of = (int*)(b + O_CO);
  nb.slot_of = (int*)(b + O_SO);
  nb.cell_count = (int*)(b + O_CC);
  nb.cell_start = (int*)(b + O_CS);
  nb.scan_tmp = (int*)(b + O_SC);
  nb.cell_atoms = (int*)(b + O_CA);
  nb.cell_pos = (float4*)(b + O_CP);
  nb.ncells_total = (int)ncells;
  nb.nstruc = 1;
  nb.cap = (int)NA_NB;
  nb.nb_cnt = (int*)(b + O_NC);
  nb.nb_jt = (int*)(b + O_JT);
  nb.nb_vec = b + O_VEC;
  nb.nb_img = nullptr;
  nb.status = status;
  if (!e) e = ae_launch_neighbors(natoms, d_coords, types0, nb, fp64, s);
  DescBuffers d{};
  d.natoms = natoms;
  d.types = types0;
  d.nb_cnt = nb.nb_cnt;
  d.nb_jt = nb.nb_jt;
  d.nb_vec = nb.nb_vec;
  d.cap = (int)NA_NB;
  // staged angular neighbours: the expected count inside the largest
  // angular cut-off with half again as many and 16 spare (as the plans size
  // them), at most the neighbour limit
  {
    const double* a = lattice;
    const double c0 = a[4] * a[8] - a[5] * a[7], c1 = a[5] * a[6] - a[3] * a[8],
                 c2 = a[3] * a[7] - a[4] * a[6];
    const double vol = std::fabs(a[0] * c0 + a[1] * c1 + a[2] * c2);
    double arc = 0.0;
    for (int t = 0; t < pd.ntypes; ++t)
      arc = std::max(arc, pd.sp[t].sftype == AE_SF_CHEBYSHEV ? pd.sp[t].cheb.a_Rc : rc);
    const double ra = arc + 1e-3;
    const double nexp = vol > 0 ? 4.18879020478639 * ra * ra * ra * natoms / vol : (double)NA_NB;
    int ca = (int)std::ceil(1.5 * nexp + 16.0);
    ca = (ca + 7) & ~7;
    d.cap_a = std::min(std::max(ca, 8), (int)NA_NB);
  }
  // lanes per atom: as set, raised while the descriptor kernels' shared
  // memory per block (4 warps of 32 / lpa atoms) would exceed 200 KB
  d.lpa = ae_lanes_per_atom();
  {
    const size_t t4 = fp64 ? 32 : 16;
    const size_t group = (2 * t4 + 3 * tsz) * (size_t)d.cap_a + tsz * (size_t)pd.nsf_pad + 32;
    while (d.lpa < 32 && group * (size_t)(4 * 32 / d.lpa) > 200 * 1024) d.lpa *= 2;
  }
  d.G = b + O_G;
  d.dEdG = b + O_DG;
  d.E_atom = (double*)(b + O_EA);
  d.F = Facc;
  d.virial = d_virial ? virial : nullptr;
  d.atom_struct = atom_struct;
  d.grad_scale = nullptr;
  d.status = status;
  const bool behler = pd.sp[0].sftype == AE_SF_BEHLER;
  if (!e) e = behler ? ae_launch_behler_forward(pd, d, fp64, s) : ae_launch_chebyshev_forward(pd, d, fp64, s);
  if (!e) e = ae_launch_mlp(pd, d, fp64, s);
  if (!e) e = ae_launch_energy_reduce(1, geom, d.E_atom, E_struct, s);
  if (!e && d_E) e = (int)cudaMemcpyAsync(d_E, E_struct, 8, cudaMemcpyDeviceToDevice, s);
  if (!e && (d_F || d_virial)) {
    e = (int)cudaMemsetAsync(Facc, 0, 4 * tsz * (size_t)natoms, s);
    if (!e && d_virial) e = (int)cudaMemsetAsync(virial, 0, 72, s);
    if (!e) e = behler ? ae_launch_behler_adjoint(pd, d, fp64, s) : ae_launch_chebyshev_adjoint(pd, d, fp64, s);
    if (!e && d_F) e = ae_launch_forces_out(natoms, Facc, fp64, d_F, 1.0, s);
    if (!e && d_virial) e = (int)cudaMemcpyAsync(d_virial, virial, 72, cudaMemcpyDeviceToDevice, s);
  }
  if (!e && d_status) e = (int)cudaMemcpyAsync(d_status, status, 4, cudaMemcpyDeviceToDevice, s);
  return e ? AENET_ERR_CUDA : ST_OK;
}
