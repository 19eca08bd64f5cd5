// C-ABI of libaenet_gb300.so: the drop-in libaenet API (include/aenet.h,
// replacing src/aenet.f90) and the batched GPU extensions
// (include/aenet_gb300.h).
//
// Host state mirrors the reference's module globals (aenet.f90:115-132):
// one set of potentials per process, loaded from .nn files; when the last
// potential is loaded the device tables (normalisation, network weights in
// FP64 and FP32, descriptor parameters) are built once.
//
// Evaluation always runs on the GPU.  There is no CPU path: if no CUDA
// device is usable the entry points return AENET_ERR_CUDA.
//
// Compiled with -ffp-contract=off: the reciprocal lattice is computed with
// the unfused operations of geo_recip_lattice (geometry.f90:491-516) so
// that lattice coordinates, and therefore neighbour sets, match the
// reference bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/aenet.h"
#include "../../include/aenet_gb300.h"
#include "common.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

// ---------------------------------------------------------------------
// exported data (aenet.f90:101-118)
// ---------------------------------------------------------------------
EXPORT int AENET_OK = 0;
EXPORT int AENET_ERR_INIT = 1;
EXPORT int AENET_ERR_MALLOC = 2;
EXPORT int AENET_ERR_IO = 3;
EXPORT int AENET_ERR_TYPE = 4;
EXPORT int AENET_TYPELEN = 2;
EXPORT int AENET_PATHLEN = 1024;
EXPORT bool AENET_TRUE = true;
EXPORT bool AENET_FALSE = false;
EXPORT int aenet_nsf_max = 0;
EXPORT int aenet_nnb_max = 0;
EXPORT double aenet_Rc_min = 0.0;
EXPORT double aenet_Rc_max = 0.0;

namespace {

constexpr double CONST_PI = 3.141592653589793;  // constants.f90

// ---------------------------------------------------------------------
// .nn potential files (potential.f90:111-157)
// ---------------------------------------------------------------------
struct HostNet {
  int nlayers = 0, nnodes_max = 0, Wsize = 0, nvalues = 0;
  std::vector<int> nnodes, f_a, iw, iv;
  std::vector<double> W;
};
struct HostSetup {
  std::string description, atomtype, sftype;
  std::vector<std::string> envtypes;
  int nenv = 0, nsf = 0, nsfparam = 0, neval = 0;
  double Rc_min = 0, Rc_max = 0;
  std::vector<int> sf, sfenv;
  std::vector<double> sfparam, vmin, vmax, vavg, vcov;
  bool legacy = false;
};
struct HostTs {
  std::string file;
  bool normalized = false;
  double scale = 1, shift = 0;
  std::vector<std::string> typeName;
  std::vector<double> E_atom;
};
struct HostPot {
  bool init = false;
  HostNet net;
  HostSetup stp;
  HostTs ts;
  double E_scale = 1, E_shift = 0, E_atom = 0;
  std::string path;
  std::vector<std::string> recs;     // the file's records (W is record 9)
};

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)tolower((unsigned char)c);
  return s;
}

// Fortran unformatted sequential records: [int32 n][payload][int32 n]
bool read_records(const char* path, std::vector<std::string>& recs) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  std::string data;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) data.append(buf, n);
  fclose(f);
  size_t i = 0;
  while (i < data.size()) {
    if (i + 4 > data.size()) return false;
    int32_t len;
    memcpy(&len, data.data() + i, 4);
    if (len < 0 || i + 8 + (size_t)len > data.size()) return false;
    int32_t len2;
    memcpy(&len2, data.data() + i + 4 + len, 4);
    if (len2 != len) return false;
    recs.emplace_back(data.data() + i + 4, (size_t)len);
    i += 8 + (size_t)len;
  }
  return true;
}

template <typename T>
bool rec_vec(const std::string& r, std::vector<T>& out, size_t count) {
  if (r.size() != count * sizeof(T)) return false;
  out.resize(count);
  if (count) memcpy(out.data(), r.data(), r.size());
  return true;
}

template <typename T>
bool rec_one(const std::string& r, T& out) {
  if (r.size() != sizeof(T)) return false;
  memcpy(&out, r.data(), sizeof(T));
  return true;
}

std::vector<std::string> split_names(const std::string& r, int n) {
  std::vector<std::string> v;
  for (int k = 0; k < n; ++k) v.push_back(trim(r.substr(2 * k, 2)));
  return v;
}

// load_Network (feedforward.f90:291-306), load_Setup (sfsetup.f90:585-609),
// load_TrnSet_info (trainset.f90:432-441).  Returns an AENET status.
int load_nn(const char* path, const std::vector<std::string>& global_types, HostPot& pot) {
  std::vector<std::string> r;
  if (!read_records(path, r)) return 3;
  if (r.size() != 35 && r.size() != 36) return 3;
  const bool legacy = r.size() == 35;
  size_t k = 0;
  HostNet& net = pot.net;
  int32_t v;
  if (!rec_one(r[k++], v)) return 3;
  net.nlayers = v;
  if (net.nlayers < 2 || net.nlayers > AE_MAXLAYERS) return 3;
  if (!rec_one(r[k++], v)) return 3;
  net.nnodes_max = v;
  if (!rec_one(r[k++], v)) return 3;
  net.Wsize = v;
  if (!rec_one(r[k++], v)) return 3;
  net.nvalues = v;
  if (!rec_vec(r[k++], net.nnodes, net.nlayers)) return 3;
  if (!rec_vec(r[k++], net.f_a, net.nlayers - 1)) return 3;
  if (!rec_vec(r[k++], net.iw, net.nlayers)) return 3;
  if (!rec_vec(r[k++], net.iv, net.nlayers)) return 3;
  if (net.Wsize <= 0 || !rec_vec(r[k++], net.W, net.Wsize)) return 3;
  // consistency with new_Network's bookkeeping
  int ws = 0;
  for (int l = 0; l + 1 < net.nlayers; ++l) ws += (net.nnodes[l] + 1) * net.nnodes[l + 1];
  if (ws != net.Wsize || net.nnodes[net.nlayers - 1] != 1) return 3;
  HostSetup& s = pot.stp;
  s.legacy = legacy;
  s.description = trim(r[k++]);
  s.atomtype = trim(r[k++]);
  if (!rec_one(r[k++], v)) return 3;
  s.nenv = v;
  if (s.nenv < 1 || (int)r[k].size() != 2 * s.nenv) return 3;
  s.envtypes = split_names(r[k++], s.nenv);
  if (!rec_one(r[k++], s.Rc_min)) return 3;
  if (!rec_one(r[k++], s.Rc_max)) return 3;
  s.sftype = trim(r[k++]);
  if (!rec_one(r[k++], v)) return 3;
  s.nsf = v;
  if (!rec_one(r[k++], v)) return 3;
  s.nsfparam = v;
  if (s.nsf < 1 || s.nsfparam < 1) return 3;
  if (!rec_vec(r[k++], s.sf, s.nsf)) return 3;
  if (!rec_vec(r[k++], s.sfparam, (size_t)s.nsfparam * s.nsf)) return 3;
  if (r[k].size() % (4 * (size_t)s.nsf) != 0) return 3;
  {
    size_t nenvmax = r[k].size() / (4 * (size_t)s.nsf);
    std::vector<int> raw;
    rec_vec(r[k++], raw, nenvmax * s.nsf);
    s.sfenv.assign(2 * (size_t)s.nsf, 0);
    for (int f = 0; f < s.nsf; ++f)
      for (size_t q = 0; q < nenvmax && q < 2; ++q) s.sfenv[2 * f + q] = raw[f * nenvmax + q];
  }
  if (!rec_one(r[k++], v)) return 3;
  s.neval = v;
  if (!rec_vec(r[k++], s.vmin, s.nsf)) return 3;
  if (!rec_vec(r[k++], s.vmax, s.nsf)) return 3;
  if (!rec_vec(r[k++], s.vavg, s.nsf)) return 3;
  if (!legacy) {
    if (!rec_vec(r[k++], s.vcov, s.nsf)) return 3;
  }
  HostTs& ts = pot.ts;
  ts.file = trim(r[k++]);
  if (!rec_one(r[k++], v)) return 3;
  ts.normalized = v != 0;
  if (!rec_one(r[k++], ts.scale)) return 3;
  if (!rec_one(r[k++], ts.shift)) return 3;
  if (!rec_one(r[k++], v)) return 3;
  int nt = v;
  if (nt < 1 || (int)r[k].size() != 2 * nt) return 3;
  ts.typeName = split_names(r[k++], nt);
  if (!rec_vec(r[k++], ts.E_atom, nt)) return 3;
  // potential.f90:145-151
  pot.E_scale = 1.0 / ts.scale;
  pot.E_shift = ts.shift;
  int it = -1;
  for (int q = 0; q < nt; ++q)
    if (ts.typeName[q] == s.atomtype) {
      it = q;
      break;
    }
  if (it < 0) return 3;
  pot.E_atom = ts.E_atom[it];
  pot.path = path;
  pot.recs = std::move(r);
  (void)global_types;
  pot.init = true;
  return 0;
}

// save_Network / save_Setup / save_TrnSet_info in the layout the file was
// read with, with the current weights in record 9
bool write_records(const char* path, const std::vector<std::string>& recs) {
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  bool ok = true;
  for (const auto& r : recs) {
    int32_t n = (int32_t)r.size();
    ok = ok && fwrite(&n, 4, 1, f) == 1;
    ok = ok && (r.empty() || fwrite(r.data(), 1, r.size(), f) == r.size());
    ok = ok && fwrite(&n, 4, 1, f) == 1;
  }
  return fclose(f) == 0 && ok;
}

// ---------------------------------------------------------------------
// global state
// ---------------------------------------------------------------------
struct DevBlob {
  void* p = nullptr;
  ~DevBlob() {
    if (p) cudaFree(p);
  }
};

struct State {
  bool init = false, loaded = false;
  int ntypes = 0;
  std::vector<std::string> types;
  std::vector<HostPot> pots;
  int angular_legacy = 0;
  int cell_div = 2;
  int z_refine = 1;          // search cells along the third axis per cell_div cell
  int lpa_default = 16;
  int lpa_adjoint = 0;        // lanes per atom of the adjoint (0: as the forward)
  int networks_tc = 1;       // tensor-core networks on the mixed path when eligible
  int nb_cell = 0;           // neighbour search: warp per atom (0), per home cell with a lane
                             // per home atom (1), per home cell with a lane per candidate (2),
                             // warp per atom over the half stencil (3)
  int angular_moments = 1;   // FP32 angular terms in moment form where instantiated
  int angular_spin_stale = 0;  // Chebyshev spin block with sfb_eval's stale s_j
  int atom_fused = 2;          // per-atom calls: one fused launch, on a cluster of blocks for
                               // rows of AE_ATOM_CLUSTER_ROWS neighbours or more and on one
                               // block below (2), always on a cluster (3), always on one
                               // block (1); or the graph of the batch kernels (0)
  std::vector<double> scale_host;   // 1/s per [type][nsf_pad] of the loaded tables
  // device tables
  bool dev_ready = false;
  int gen = 0;                // bumped by every option change and table build: captured
                              // graphs of the host-buffer path are redone after it
  PotDevice pd{};
  std::unique_ptr<DevBlob> blob;
  std::vector<std::vector<unsigned char>> behler_host;
  // stand-alone Chebyshev basis (aenet_sfb_*)
  bool sfb_init = false;
  int sfb_ntypes = 0, sfb_rorder = 0, sfb_aorder = 0;
  double sfb_rRc = 0, sfb_aRc = 0;
  PotDevice sfb_pd{};
  std::unique_ptr<DevBlob> sfb_blob;
  // neighbour list API (aenet_nbl_*)
  bool nbl_init = false;
  int nbl_natoms = 0;
  std::vector<int> nbl_cnt, nbl_jt, nbl_img;
  std::vector<double> nbl_vec, nbl_cart, nbl_s;
  std::vector<int> nbl_types;
  int nbl_cap = 0;
  double nbl_L[9];
  int nbl_pbc = 1;
};

State g;
std::mutex g_mu;

int cuda_ok() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return 0;
  return 1;
}

// typespin of new_SFBasis (sfbasis.f90:142-147) for local type index l
// (1-based) of a basis with num_types species
float typespin(int num_types, int l) {
  int s = -num_types / 2;
  for (int i = 1; i <= num_types; ++i) {
    if (s == 0 && (num_types % 2) == 0) s = s + 1;
    if (i == l) return (float)s;
    s = s + 1;
  }
  return 0.f;
}

// Legendre expansion of the angular basis: T_n(x(c)) = sum_l q[n][l] P_l(c)
// for n < a_N <= AE_MOMA, x(c) = c or the legacy (2c - pi)/pi of
// sfbasis.f90's PI.  Monomial coefficients in c, peeled from the top degree.
std::vector<float> legendre_table(int a_N, int legacy) {
  const int D = AE_MOMA;
  std::vector<float> q(D * D, 0.f);
  if (a_N > D) return q;
  const double pi = 3.14159265358979;
  const double al = legacy ? 2.0 / pi : 1.0, be = legacy ? -1.0 : 0.0;
  std::vector<std::vector<double>> Tn(D, std::vector<double>(D, 0.0)), Pl = Tn;
  Tn[0][0] = 1.0;
  if (D > 1) {
    Tn[1][0] = be;
    Tn[1][1] = al;
  }
  for (int k = 1; k + 1 < D; ++k)
    for (int e = 0; e < D; ++e) {
      double v = 2.0 * be * Tn[k][e] - Tn[k - 1][e];
      if (e > 0) v += 2.0 * al * Tn[k][e - 1];
      Tn[k + 1][e] = v;
    }
  Pl[0][0] = 1.0;
  if (D > 1) Pl[1][1] = 1.0;
  for (int k = 1; k + 1 < D; ++k)
    for (int e = 0; e < D; ++e) {
      double v = -k * Pl[k - 1][e];
      if (e > 0) v += (2.0 * k + 1.0) * Pl[k][e - 1];
      Pl[k + 1][e] = v / (k + 1.0);
    }
  for (int n = 0; n < a_N; ++n) {
    std::vector<double> rem = Tn[n];
    for (int l = n; l >= 0; --l) {
      const double c = rem[l] / Pl[l][l];
      q[n * D + l] = (float)c;
      for (int e = 0; e <= l; ++e) rem[e] -= c * Pl[l][e];
    }
  }
  return q;
}

int local_type(const HostSetup& s, const std::string& name) {
  for (int j = 0; j < s.nenv; ++j)
    if (s.envtypes[j] == name) return j + 1;
  return 0;
}

// lcl_nmax_nbdist (lclist.f90:229-245)
int nmax_nbdist(double rmin, double rmax) {
  double V_atom = std::pow(0.5 * rmin, 3);
  double V_cut = std::pow(rmax + 0.5 * rmin, 3);
  return (int)std::ceil(V_cut / V_atom * 0.7405);
}

int odd_pitch(int n) { return (n % 2) ? n : n + 1; }

// BF16 round to nearest even from the FP32 value of v, and back
uint16_t bf16_rn(double v) {
  float f = (float)v;
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return (uint16_t)(u >> 16);   // inf / nan
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
double bf16_to_double(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// Device layout of one network's weights appended to w64: layer l as rows
// W[o][k] (bias in column nin) with an odd row pitch.  The Fortran slice
// W(iw+1 : iw+(nin+1)*nout) is column-major (nout, nin+1).
void device_weights(const HostNet& net, NetTable& nt, std::vector<double>& w64) {
  int iw = 0;
  for (int l = 0; l + 1 < net.nlayers; ++l) {
    int nin = net.nnodes[l], nout = net.nnodes[l + 1];
    int pitch = odd_pitch(nin + 1);
    nt.pitch[l] = pitch;
    nt.w_off[l] = (int)w64.size();
    size_t base = w64.size();
    w64.resize(base + (size_t)pitch * nout, 0.0);
    for (int o = 0; o < nout; ++o)
      for (int c = 0; c <= nin; ++c) w64[base + (size_t)o * pitch + c] = net.W[iw + o + c * nout];
    iw += (nin + 1) * nout;
  }
}

// Behler tables: registration under the GLOBAL type index and evaluation
// with the LOCAL (env) index of the central atom's setup, as in
// setup_symmfunc_Behler2011 (sfsetup.f90:1298) and stp_eval
// (sfsetup.f90:925-944); the per-species table below is what
// sf_fingerprint evaluates for a central atom of that species.
int build_behler(std::vector<std::vector<unsigned char>>& out, std::vector<double>& rc_max_out,
                 int* grid_only);

// Split-BF16 images of every species' network for the tensor-core kernel
// (two hidden layers, input and hidden widths up to 64; TcLayout in
// common.h).  Sets pd.tc_ok / tc_kin / tc_h; empty when not eligible.
std::vector<unsigned char> make_tc_image(PotDevice& pd, const std::vector<double>& scale) {
  std::vector<unsigned char> tc_img;
  pd.tc_ok = 0;
  pd.tc_tanh = 0;
  {
    bool ok = true;
    int kin = 0, h = 0;
    for (int t = 0; t < g.ntypes; ++t) {
      const HostNet& net = g.pots[t].net;
      if (net.nlayers != 4 || net.nnodes[3] != 1 || net.nnodes[0] > 64 || net.nnodes[1] > 64 ||
          net.nnodes[2] > 64)
        ok = false;
      else {
        kin = std::max(kin, net.nnodes[0]);
        h = std::max(h, std::max(net.nnodes[1], net.nnodes[2]));
      }
    }
    if (ok) {
      kin = kin <= 32 ? 32 : 64;
      h = h <= 32 ? 32 : 64;
      const TcLayout L = tc_layout(kin, h);
      tc_img.assign((size_t)g.ntypes * L.bytes, 0);
      for (int t = 0; t < g.ntypes; ++t) {
        const HostNet& net = g.pots[t].net;
        unsigned char* base = tc_img.data() + (size_t)t * L.bytes;
        const int n0 = net.nnodes[0], n1 = net.nnodes[1], n2 = net.nnodes[2];
        const int iw1 = 0, iw2 = (n0 + 1) * n1, iw3 = iw2 + (n1 + 1) * n2;
        // Fortran W slices are column-major (nout, nin+1), bias in column nin
        auto W1 = [&](int o, int k) { return net.W[iw1 + o + k * n1]; };
        auto W2 = [&](int o, int k) { return net.W[iw2 + o + k * n2]; };
        auto put = [&](int off, int R, int K, int r, int k, double v) {
          uint16_t hi = bf16_rn(v);
          uint16_t lo = bf16_rn(v - bf16_to_double(hi));
          int o = tc_core_offset(r, k, K);
          memcpy(base + off + o, &hi, 2);
          memcpy(base + off + 2 * R * K + o, &lo, 2);
        };
        for (int o = 0; o < n1; ++o)
          for (int k = 0; k < n0; ++k) {
            put(L.b1, h, kin, o, k, W1(o, k));
            put(L.b1t, kin, h, k, o, W1(o, k));
          }
        for (int o = 0; o < n2; ++o)
          for (int k = 0; k < n1; ++k) {
            put(L.b2, h, h, o, k, W2(o, k));
            put(L.b2t, h, h, k, o, W2(o, k));
          }
        float* vec = reinterpret_cast<float*>(base + L.vec);
        for (int o = 0; o < n1; ++o) vec[o] = (float)W1(o, n0);
        for (int o = 0; o < n2; ++o) vec[h + o] = (float)W2(o, n1);
        for (int k = 0; k < n2; ++k) vec[2 * h + k] = (float)net.W[iw3 + k];
        for (int k = 0; k < n0; ++k)
          vec[3 * h + k] = (float)(pd.sp[t].E_scale * scale[(size_t)t * pd.nsf_pad + k]);
        vec[3 * h + kin] = (float)net.W[iw3 + n2];
        vec[3 * h + kin + 1] = (float)net.f_a[0];
        vec[3 * h + kin + 2] = (float)net.f_a[1];
        vec[3 * h + kin + 3] = (float)net.f_a[2];
      }
      pd.tc_ok = 1;
      pd.tc_kin = kin;
      pd.tc_h = h;
      pd.tc_tanh = 1;
      for (int t = 0; t < g.ntypes; ++t) {
        const HostNet& net = g.pots[t].net;
        if (net.f_a[0] != 1 || net.f_a[1] != 1 || net.f_a[2] != 0) pd.tc_tanh = 0;
      }
    }
  }
  return tc_img;
}

int build_device_tables() {
  ++g.gen;
  if (!cuda_ok()) return AENET_ERR_CUDA;
  PotDevice pd{};
  pd.ntypes = g.ntypes;
  int nsf_max = 0;
  for (auto& p : g.pots) nsf_max = std::max(nsf_max, p.stp.nsf);
  if (nsf_max > AE_MAXNSF) return AENET_ERR_INPUT;
  pd.nsf_max = nsf_max;
  pd.nsf_pad = (nsf_max + 3) & ~3;
  pd.Rc_max = aenet_Rc_max;
  std::string sftype = lower(g.pots[0].stp.sftype);
  for (auto& p : g.pots)
    if (lower(p.stp.sftype) != sftype) return AENET_ERR_INPUT;
  std::vector<double> shift((size_t)g.ntypes * pd.nsf_pad, 0.0), scale(shift.size(), 0.0);
  std::vector<double> w64;
  for (int t = 0; t < g.ntypes; ++t) {
    const HostPot& p = g.pots[t];
    SpeciesTable& sp = pd.sp[t];
    sp.nsf = p.stp.nsf;
    sp.E_scale = p.E_scale;
    sp.E_shift = p.E_shift;
    sp.E_atom = p.E_atom;
    // normalisation (sfsetup.f90:985-1035; legacy 16-record setups use
    // max(avg - min, max - avg), sfsetup.f90:118-123)
    for (int k = 0; k < p.stp.nsf; ++k) {
      double sh = p.stp.vavg[k], s;
      if (p.stp.legacy) {
        double a = p.stp.vavg[k] - p.stp.vmin[k], b = p.stp.vmax[k] - p.stp.vavg[k];
        s = a > b ? a : b;
      } else {
        s = std::sqrt(p.stp.vcov[k] - sh * sh);
      }
      shift[(size_t)t * pd.nsf_pad + k] = sh;
      scale[(size_t)t * pd.nsf_pad + k] = (s <= 1.0e-10) ? 0.0 : 1.0 / s;
    }
    // network
    NetTable& nt = sp.net;
    const HostNet& net = p.net;
    nt.nlayers = net.nlayers;
    for (int l = 0; l < net.nlayers; ++l) {
      nt.nnodes[l] = net.nnodes[l];
      if (net.nnodes[l] > AE_MAXNODES && l > 0) return AENET_ERR_INPUT;
    }
    if (net.nnodes[0] != p.stp.nsf) return AENET_ERR_INPUT;
    nt.f_a[0] = 0;
    for (int l = 1; l < net.nlayers; ++l) nt.f_a[l] = net.f_a[l - 1];
    device_weights(net, nt, w64);
    // Chebyshev (setup_basis_chebyshev, sfsetup.f90:1162-1179)
    if (sftype == "chebyshev") {
      sp.sftype = AE_SF_CHEBYSHEV;
      ChebTable& ct = sp.cheb;
      ct.r_Rc = p.stp.sfparam[0];
      int r_order = (int)std::lround(p.stp.sfparam[1]);
      ct.a_Rc = p.stp.sfparam[2];
      int a_order = (int)std::lround(p.stp.sfparam[3]);
      ct.r_N = r_order + 1;
      ct.a_N = a_order + 1;
      if (ct.r_N < 1 || ct.a_N < 1 || ct.r_N > AE_MAXCHEB || ct.a_N > AE_MAXCHEB)
        return AENET_ERR_INPUT;
      ct.multi = p.stp.nenv > 1 ? 1 : 0;
      ct.nsf = (ct.r_N + ct.a_N) * (ct.multi ? 2 : 1);
      if (ct.nsf != p.stp.nsf) return AENET_ERR_INPUT;
      ct.r_i1 = 0;
      ct.a_i1 = ct.r_N;
      ct.r_i2 = ct.r_N + ct.a_N;
      ct.a_i2 = 2 * ct.r_N + ct.a_N;
      ct.angular_legacy = g.angular_legacy;
      for (int gt = 0; gt < AE_MAXT; ++gt) ct.spin[gt] = 0.f;
      for (int gt = 0; gt < g.ntypes; ++gt) {
        int l = local_type(p.stp, g.types[gt]);
        ct.spin[gt] = l > 0 ? typespin(p.stp.nenv, l) : 0.f;
      }
    } else if (sftype == "behler2011") {
      sp.sftype = AE_SF_BEHLER;
    } else {
      return AENET_ERR_INPUT;
    }
  }
  int wtotal = (int)w64.size();
  for (int t = 0; t < g.ntypes; ++t) pd.sp[t].net.wtotal = wtotal;
  std::vector<float> w32(w64.begin(), w64.end());
  std::vector<float> shift2(2 * shift.size()), scale32(scale.size());
  for (size_t q = 0; q < shift.size(); ++q) {
    float hi = (float)shift[q];
    shift2[2 * q] = hi;
    shift2[2 * q + 1] = (float)(shift[q] - (double)hi);
    scale32[q] = (float)scale[q];
  }
  // split-BF16 images for the tensor-core networks
  std::vector<unsigned char> tc_img = make_tc_image(pd, scale);
  // Legendre tables of the moment form (Chebyshev species)
  std::vector<float> qleg((size_t)g.ntypes * AE_MOMA * AE_MOMA, 0.f);
  for (int t = 0; t < g.ntypes; ++t)
    if (pd.sp[t].sftype == AE_SF_CHEBYSHEV) {
      std::vector<float> qt = legendre_table(pd.sp[t].cheb.a_N, pd.sp[t].cheb.angular_legacy);
      std::copy(qt.begin(), qt.end(), qleg.begin() + (size_t)t * AE_MOMA * AE_MOMA);
    }
  g.scale_host = scale;
  // Behler tables
  std::vector<std::vector<unsigned char>> bt;
  std::vector<double> bt_rc;
  if (sftype == "behler2011") {
    int st = build_behler(bt, bt_rc, &pd.behler_grid_only);
    if (st) return st;
  }
  size_t blob_bytes = 0;
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off_shift = blob_bytes;
  blob_bytes = align(blob_bytes + shift.size() * 8);
  size_t off_scale = blob_bytes;
  blob_bytes = align(blob_bytes + scale.size() * 8);
  size_t off_w64 = blob_bytes;
  blob_bytes = align(blob_bytes + w64.size() * 8);
  size_t off_w32 = blob_bytes;
  blob_bytes = align(blob_bytes + w32.size() * 4);
  size_t off_sh2 = blob_bytes;
  blob_bytes = align(blob_bytes + shift2.size() * 4);
  size_t off_sc32 = blob_bytes;
  blob_bytes = align(blob_bytes + scale32.size() * 4);
  size_t off_tc = blob_bytes;
  blob_bytes = align(blob_bytes + tc_img.size());
  size_t off_q = blob_bytes;
  blob_bytes = align(blob_bytes + qleg.size() * 4);
  size_t off_beh = blob_bytes;
  std::vector<size_t> beh_off;
  for (auto& b : bt) {
    beh_off.push_back(blob_bytes - off_beh);
    blob_bytes = align(blob_bytes + b.size());
  }
  auto blob = std::make_unique<DevBlob>();
  if (cudaMalloc(&blob->p, blob_bytes + 256) != cudaSuccess) return AENET_ERR_CUDA;
  char* base = (char*)blob->p;
  cudaMemcpy(base + off_shift, shift.data(), shift.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(base + off_scale, scale.data(), scale.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(base + off_w64, w64.data(), w64.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(base + off_w32, w32.data(), w32.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(base + off_sh2, shift2.data(), shift2.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(base + off_sc32, scale32.data(), scale32.size() * 4, cudaMemcpyHostToDevice);
  for (size_t q = 0; q < bt.size(); ++q)
    cudaMemcpy(base + off_beh + beh_off[q], bt[q].data(), bt[q].size(), cudaMemcpyHostToDevice);
  if (!tc_img.empty()) cudaMemcpy(base + off_tc, tc_img.data(), tc_img.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(base + off_q, qleg.data(), qleg.size() * 4, cudaMemcpyHostToDevice);
  if (cudaDeviceSynchronize() != cudaSuccess) return AENET_ERR_CUDA;
  pd.shift = (const double*)(base + off_shift);
  pd.scale = (const double*)(base + off_scale);
  pd.w64 = (const double*)(base + off_w64);
  pd.w32 = (const float*)(base + off_w32);
  pd.shift2 = (const float2*)(base + off_sh2);
  pd.scale32 = (const float*)(base + off_sc32);
  pd.behler_blob = (const unsigned char*)(base + off_beh);
  pd.tc_img = tc_img.empty() ? nullptr : (const unsigned char*)(base + off_tc);
  pd.qleg = (const float*)(base + off_q);
  for (size_t q = 0; q < bt.size(); ++q) pd.sp[q].behler_off = (int)beh_off[q];
  g.pd = pd;
  g.blob = std::move(blob);
  g.behler_host = bt;
  g.dev_ready = true;
  return 0;
}

int ensure_device() {
  if (!g.loaded) return AENET_ERR_INIT;
  if (g.dev_ready) return 0;
  return build_device_tables();
}

}  // namespace

// ---------------------------------------------------------------------
// Behler tables (defined after the anonymous namespace helpers)
// ---------------------------------------------------------------------
namespace {
BehlerFn make_fn(double Rc, double p1, double p2, double p3, int kind, int out) {
  BehlerFn b{};
  b.Rc = Rc;
  b.p1 = p1;
  b.p2 = p2;
  b.p3 = p3;
  b.fRc = (float)Rc;
  b.fp1 = (float)p1;
  b.fp2 = (float)p2;
  b.fp3 = (float)p3;
  b.kind = kind;
  b.out = out;
  // G4/G5 zeta (p2) evaluated by repeated squaring when it is a small integer
  b.izeta = 0;
  if ((kind == 4 || kind == 5) && p2 >= 1.0 && p2 <= 64.0 && p2 == std::floor(p2)) b.izeta = (int)p2;
  return b;
}

// Whether the angular functions fns[f0, f1) form a product grid (one kind,
// one Rc, lambda = +-1, every (lambda, zeta) x eta combination once); fills
// `gr` when they do.
bool angular_grid(const std::vector<BehlerFn>& fns, int f0, int f1, BehlerGrid& gr) {
  if (f1 - f0 < 2) return false;
  memset(&gr, 0, sizeof(gr));
  const BehlerFn& a = fns[f0];
  if (a.kind != 4 && a.kind != 5) return false;
  gr.kind = a.kind;
  gr.Rc = a.Rc;
  std::vector<std::pair<double, double>> lz;
  std::vector<double> et;
  for (int f = f0; f < f1; ++f) {
    const BehlerFn& b = fns[f];
    if (b.kind != a.kind || b.Rc != a.Rc || (b.p1 != 1.0 && b.p1 != -1.0) || !(b.p2 > 0.0))
      return false;
    auto key = std::make_pair(b.p1, b.p2);
    if (std::find(lz.begin(), lz.end(), key) == lz.end()) lz.push_back(key);
    if (std::find(et.begin(), et.end(), b.p3) == et.end()) et.push_back(b.p3);
  }
  if ((int)lz.size() > AE_BG_NL || (int)et.size() > AE_BG_NE) return false;
  if ((int)(lz.size() * et.size()) != f1 - f0) return false;
  gr.nl = (int)lz.size();
  gr.ne = (int)et.size();
  for (int q = 0; q < AE_BG_NL * AE_BG_NE; ++q) gr.out[q] = -1;
  for (int f = f0; f < f1; ++f) {
    const BehlerFn& b = fns[f];
    int l = (int)(std::find(lz.begin(), lz.end(), std::make_pair(b.p1, b.p2)) - lz.begin());
    int e = (int)(std::find(et.begin(), et.end(), b.p3) - et.begin());
    if (gr.out[l * AE_BG_NE + e] >= 0) return false;
    gr.out[l * AE_BG_NE + e] = b.out;
  }
  gr.fRc = (float)gr.Rc;
  for (int l = 0; l < gr.nl; ++l) {
    gr.lam[l] = lz[l].first;
    gr.zeta[l] = lz[l].second;
    gr.flam[l] = (float)gr.lam[l];
    gr.fzeta[l] = (float)gr.zeta[l];
    const double z = gr.zeta[l];
    gr.izeta[l] = (z >= 1.0 && z <= 64.0 && z == std::floor(z)) ? (int)z : 0;
  }
  for (int e = 0; e < gr.ne; ++e) {
    gr.eta[e] = et[e];
    gr.feta[e] = (float)et[e];
  }
  return true;
}

int build_behler(std::vector<std::vector<unsigned char>>& out, std::vector<double>& rc_max_out,
                 int* grid_only) {
  // sf_init over the global types (sfsetup.f90:800-808, symmfunc.f90:91-140)
  const int nt = g.ntypes;
  *grid_only = 1;
  int nGmax = 0;
  for (auto& p : g.pots) nGmax = std::max(nGmax, p.stp.nsf);
  // registered functions: by (type1 global, pair/triple of LOCAL env
  // indices of that potential's setup), in registration order, per kind
  struct Fn {
    int kind;
    double Rc, p1, p2, p3;
  };
  // idx2/idx3 of symmfunc.f90:105-120 over nt types
  auto idx2 = [&](int i, int j) { return (i - 1) * nt + j; };  // 1-based pair id
  std::vector<int> idx3((size_t)(nt + 1) * (nt + 1) * (nt + 1), 0);
  int n3 = 0;
  for (int i = 1; i <= nt; ++i)
    for (int j = 1; j <= nt; ++j) {
      idx3[((size_t)i * (nt + 1) + j) * (nt + 1) + j] = ++n3;
      for (int k = j + 1; k <= nt; ++k) {
        ++n3;
        idx3[((size_t)i * (nt + 1) + j) * (nt + 1) + k] = n3;
        idx3[((size_t)i * (nt + 1) + k) * (nt + 1) + j] = n3;
      }
    }
  auto IDX3 = [&](int i, int j, int k) { return idx3[((size_t)i * (nt + 1) + j) * (nt + 1) + k]; };
  int npairs = nt * nt;
  std::vector<std::vector<std::vector<Fn>>> rad(npairs + 1, std::vector<std::vector<Fn>>(6));
  std::vector<std::vector<std::vector<Fn>>> ang(n3 + 1, std::vector<std::vector<Fn>>(6));
  std::vector<int> nG_type(nt + 1, 0);
  for (int t = 1; t <= nt; ++t) {
    const HostSetup& s = g.pots[t - 1].stp;
    for (int f = 0; f < s.nsf; ++f) {
      int kind = s.sf[f];
      const double* p = &s.sfparam[(size_t)f * s.nsfparam];
      int t2 = s.sfenv[2 * f], t3 = s.sfenv[2 * f + 1];
      double P[4] = {0, 0, 0, 0};
      for (int q = 0; q < std::min(4, s.nsfparam); ++q) P[q] = p[q];
      if (kind >= 1 && kind <= 3) {
        if (t2 < 1 || t2 > nt) return AENET_ERR_INPUT;
        auto& L = rad[idx2(t, t2)][kind];
        if ((int)L.size() >= nGmax) return AENET_ERR_INPUT;
        Fn fn{kind, P[0], 0, 0, 0};
        if (kind == 2) { fn.p1 = P[1]; fn.p2 = P[2]; }
        if (kind == 3) { fn.p1 = P[1]; }
        L.push_back(fn);
      } else if (kind == 4 || kind == 5) {
        if (t2 < 1 || t2 > nt || t3 < 1 || t3 > nt) return AENET_ERR_INPUT;
        auto& L = ang[IDX3(t, t2, t3)][kind];
        if ((int)L.size() >= nGmax) return AENET_ERR_INPUT;
        // sf_pG4: Rc, lambda, zeta, eta
        L.push_back(Fn{kind, P[0], P[1], P[2], P[3]});
      } else {
        return AENET_ERR_INPUT;
      }
      nG_type[t] += 1;
    }
  }
  // per central GLOBAL species: the table evaluated with type1 = ltype of
  // the central species in its own setup, neighbour species mapped through
  // the same setup's ltype.
  out.clear();
  rc_max_out.clear();
  for (int c = 0; c < nt; ++c) {
    const HostSetup& s = g.pots[c].stp;
    int type1 = local_type(s, g.types[c]);
    if (type1 < 1 || type1 > nt) return AENET_ERR_INPUT;
    if (s.nsf < nG_type[type1]) return AENET_ERR_INPUT;
    // feature offsets, sf_build_index (symmfunc.f90:284-305)
    std::vector<int> iG02(npairs + 1, 0), iG03(n3 + 1, 0);
    {
      int i = 0;
      for (int t2 = 1; t2 <= nt; ++t2) {
        int pij = idx2(type1, t2);
        iG02[pij] = i;
        for (int kd = 1; kd <= 5; ++kd) i += (int)rad[pij][kd].size();
        for (int t3 = t2; t3 <= nt; ++t3) {
          int tijk = IDX3(type1, t2, t3);
          iG03[tijk] = i;
          for (int kd = 1; kd <= 5; ++kd) i += (int)ang[tijk][kd].size();
        }
      }
    }
    std::vector<BehlerFn> fns;
    BehlerTable hdr{};
    hdr.nsf = s.nsf;
    double rcm = 0;
    // radial functions for each GLOBAL neighbour species gj
    for (int gj = 0; gj <= nt; ++gj) {
      hdr.rad_off[gj] = (int)fns.size();
      if (gj == nt) break;
      int lj = local_type(s, g.types[gj]);
      if (lj < 1 || lj > nt) continue;
      int pij = idx2(type1, lj);
      int iG = iG02[pij];
      for (int kd = 1; kd <= 3; ++kd)
        for (auto& f : rad[pij][kd]) {
          fns.push_back(make_fn(f.Rc, f.p1, f.p2, f.p3, kd, iG++));
          rcm = std::max(rcm, f.Rc);
        }
    }
    for (int gj = 0; gj < nt; ++gj)
      for (int gk = 0; gk < nt; ++gk) {
        hdr.ang_off[gj * nt + gk] = (int)fns.size();
        int lj = local_type(s, g.types[gj]), lk = local_type(s, g.types[gk]);
        if (lj < 1 || lj > nt || lk < 1 || lk > nt) continue;
        int tijk = IDX3(type1, lj, lk);
        int iG = iG03[tijk];
        for (int kd = 4; kd <= 5; ++kd)
          for (auto& f : ang[tijk][kd]) {
            fns.push_back(make_fn(f.Rc, f.p1, f.p2, f.p3, kd, iG++));
            rcm = std::max(rcm, f.Rc);
          }
      }
    hdr.ang_off[nt * nt] = (int)fns.size();
    hdr.nfn = (int)fns.size();
    hdr.rc_max = rcm;
    // product grids of the angular lists (evaluation order only; the
    // functions and their feature indices are the ones listed above)
    std::vector<BehlerGrid> grids;
    for (int q = 0; q < nt * nt; ++q) {
      hdr.grid_of[q] = -1;
      BehlerGrid gr;
      if (angular_grid(fns, hdr.ang_off[q], hdr.ang_off[q + 1], gr)) {
        hdr.grid_of[q] = (int)grids.size();
        grids.push_back(gr);
      } else if (hdr.ang_off[q + 1] > hdr.ang_off[q]) {
        *grid_only = 0;
      }
    }
    size_t fbytes = sizeof(BehlerTable) + sizeof(BehlerFn) * (fns.size() + 1);
    fbytes = (fbytes + 15) & ~size_t(15);
    hdr.grid_off = grids.empty() ? 0 : (int)fbytes;
    size_t bytes = fbytes + sizeof(BehlerGrid) * grids.size();
    std::vector<unsigned char> buf(bytes, 0);
    memcpy(buf.data(), &hdr, sizeof(BehlerTable));
    BehlerTable* bt = reinterpret_cast<BehlerTable*>(buf.data());
    if (!fns.empty()) memcpy(bt->fn, fns.data(), sizeof(BehlerFn) * fns.size());
    if (!grids.empty()) memcpy(buf.data() + fbytes, grids.data(), sizeof(BehlerGrid) * grids.size());
    out.push_back(std::move(buf));
    rc_max_out.push_back(rcm);
  }
  return 0;
}
}  // namespace

// ---------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------
struct aenet_gpu_plan {
  int nstruc = 0, natoms = 0, fp64 = 1;
  bool keep_images = false;
  std::vector<StructGeom> geom_h;
  std::vector<int> natoms_h;
  std::vector<int> pbc_h;
  const PotDevice* pd = nullptr;   // tables used by this plan
  int cell_div = 2;
  int z_refine = 1;
  double rc = 0;
  // device memory
  void* mem = nullptr;
  size_t mem_bytes = 0;
  StructGeom* geom_d = nullptr;
  int* atom_struct = nullptr;
  int* types0 = nullptr;
  double* s_wrap = nullptr;
  double* r_wrap = nullptr;
  float4* r_f32 = nullptr;
  int* cell_of = nullptr;
  int* slot_of = nullptr;
  int* cell_count = nullptr;
  int* cell_start = nullptr;
  int* scan_tmp = nullptr;
  int* cell_atoms = nullptr;
  float4* cell_pos = nullptr;
  int ncells = 0;
  int cap = 0;
  int cap_a = 0;      // staged angular neighbours per atom
  int lpa = 0;        // lanes per atom in the descriptor kernels (0 = default)
  int* nb_cnt = nullptr;
  int* nb_jt = nullptr;
  void* nb_vec = nullptr;
  int* nb_img = nullptr;
  float* M = nullptr;         // angular moments of the FP32 moment form
  int mom_pad = 0;
  int* nb_rank = nullptr;     // stale-spin order of the table slots (option angular_spin)
  float* nb_seff = nullptr;
  int stale_caller_order = 0; // table rows hold a caller's lists (rank = slot)
  int* struct_order = nullptr;  // structures by decreasing size (per-structure search)
  int smem_atoms = 0, smem_cells = 0;
  void* G = nullptr;
  void* dEdG = nullptr;
  double* E_atom = nullptr;
  void* Facc = nullptr;
  double* E_struct = nullptr;
  double* virial = nullptr;
  unsigned* status = nullptr;
  int nchunks = 0;            // energy-reduction chunks over all structures
  int one_chunk_each = 0;     // every structure has 1 .. AE_ECHUNK atoms
  double2* e_part = nullptr;
  int* chunk_struct = nullptr;  // [nchunks] structure of each energy chunk
  int* order = nullptr;       // atoms grouped by species (tensor-core networks, training)
  int* spec_off = nullptr;    // [AE_MAXT + 1]
  int* part_scratch = nullptr;
  // training workspace, allocated by the first loss/gradient call
  void* tmem = nullptr;
  double* cE = nullptr;       // [nstruc] dL/dE coefficients
  double* loss_s = nullptr;   // [nstruc]
  void* U = nullptr;          // [N] T4 dL/dF
  double* partial = nullptr;  // per-block weight-gradient rows
  ~aenet_gpu_plan() {
    if (mem) cudaFree(mem);
    if (tmem) cudaFree(tmem);
  }
};

namespace {
// One cached plan (with its I/O staging buffers) for the host-buffer entry
// points: a call with the same batch layout (structure sizes, lattices,
// pbc, precision) reuses the device workspace instead of reallocating it.
struct HostPlanCache {
  std::unique_ptr<aenet_gpu_plan> plan;
  std::vector<int> natoms, pbc;
  std::vector<double> lattices;
  int precision = -1;
  bool isolated = false;
  char* io = nullptr;
  size_t io_bytes = 0;
  cudaStream_t stream = nullptr;
  unsigned* status_h = nullptr;   // pinned: the status read back stays asynchronous
  // the plan's run captured as a CUDA graph (device pointers of the cached
  // buffers are fixed), with the outputs it was captured for and g.gen
  cudaGraphExec_t graph = nullptr;
  unsigned graph_key = 0;
  int graph_gen = -1;
  ~HostPlanCache() {
    drop_graph();
    if (io) cudaFree(io);
    if (stream) cudaStreamDestroy(stream);
    if (status_h) cudaFreeHost(status_h);
  }
  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
  void reset() {
    drop_graph();
    plan.reset();
    if (io) cudaFree(io);
    io = nullptr;
    io_bytes = 0;
  }
};
// Large host-buffer batches run as up to AE_HOST_CHUNKS chunks of whole
// structures, each with its own cached plan and stream, so that one
// chunk's copies overlap the others' kernels.
constexpr int AE_HOST_CHUNKS = 4;
constexpr long long AE_CHUNK_ATOMS = 131072;   // atoms per chunk at least
HostPlanCache g_cache[AE_HOST_CHUNKS];
void host_cache_reset() {
  for (auto& c : g_cache) c.reset();
}
void nlist_release();   // drops the neighbour-list entry point's workspace
}  // namespace

namespace {

void cross(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// geometry of one structure
// Cells of the search grid are rcp/cell_div wide along the first two axes
// and z_refine times narrower along the third: stencil rows keep their
// number while the cut of each row to the cut-off sphere gets finer.
int make_geom(StructGeom& G, const double* lat, int pbc, const double* coords, int natoms,
              double rc, int cell_div, int frac_mode, const int* force_nc = nullptr,
              int z_refine = 1) {
  memset(&G, 0, sizeof(G));
  G.pbc = pbc;
  G.frac_mode = frac_mode;
  const double rcp = rc + 1.0e-3;
  G.rc2 = rcp * rcp;   // (Rc + EPS)*(Rc + EPS), lclist.f90:572
  const double w = rcp / cell_div;
  double ext = rcp;
  G.rcf = (float)rcp;
  if (pbc) {
    for (int q = 0; q < 9; ++q) G.L[q] = lat[q];
    G.ortho = (lat[1] == 0.0 && lat[2] == 0.0 && lat[3] == 0.0 && lat[5] == 0.0 &&
               lat[6] == 0.0 && lat[7] == 0.0 && lat[0] > 0.0 && lat[4] > 0.0 && lat[8] > 0.0)
                  ? 1 : 0;
    const double* a1 = lat;
    const double* a2 = lat + 3;
    const double* a3 = lat + 6;
    // geo_cell_volume with avec(i,j) = component i of vector j
    double V = a1[0] * a2[1] * a3[2] + a1[1] * a2[2] * a3[0] + a1[2] * a2[0] * a3[1] -
               a1[2] * a2[1] * a3[0] - a1[0] * a2[2] * a3[1] - a1[1] * a2[0] * a3[2];
    if (!(std::fabs(V) > 0.0) || !std::isfinite(V)) return AENET_ERR_INPUT;
    double b1[3], b2[3], b3[3];
    cross(a2, a3, b1);
    cross(a1, a3, b2);
    cross(a1, a2, b3);
    for (int c = 0; c < 3; ++c) {
      if (frac_mode == 0) {
        G.B[c] = (b1[c] / V) * 2.0 * CONST_PI;
        G.B[3 + c] = (-b2[c] / V) * 2.0 * CONST_PI;
        G.B[6 + c] = (b3[c] / V) * 2.0 * CONST_PI;
      } else {
        G.B[c] = b1[c] / V;
        G.B[3 + c] = -b2[c] / V;
        G.B[6 + c] = b3[c] / V;
      }
    }
    const double* bb[3] = {b1, b2, b3};
    for (int a = 0; a < 3; ++a) {
      double bl = std::sqrt(bb[a][0] * bb[a][0] + bb[a][1] * bb[a][1] + bb[a][2] * bb[a][2]);
      double h = std::fabs(V) / bl;   // height of the cell along axis a
      G.hf[a] = (float)h;
      int nc = (int)std::floor(h / (a == 2 ? w / z_refine : w));
      if (nc < 1) nc = 1;
      if (nc > 1000) nc = 1000;
      if (force_nc) nc = force_nc[a];
      G.nc[a] = nc;
      G.kr[a] = (int)std::ceil(rcp * nc / h * (1.0 + 1e-12));
      if (G.kr[a] < 1) G.kr[a] = 1;
      ext += std::sqrt(lat[3 * a] * lat[3 * a] + lat[3 * a + 1] * lat[3 * a + 1] +
                       lat[3 * a + 2] * lat[3 * a + 2]);
    }
  } else {
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    for (int i = 0; i < natoms; ++i)
      for (int c = 0; c < 3; ++c) {
        double x = coords ? coords[3 * i + c] : 0.0;
        if (i == 0 || x < mn[c]) mn[c] = x;
        if (i == 0 || x > mx[c]) mx[c] = x;
      }
    // atoms of an isolated structure may leave this box later; their cells
    // are clamped, which keeps every pair within reach of the full stencil
    // but not of a pruned one, so no pruning here
    G.ortho = 0;
    for (int c = 0; c < 3; ++c) {
      G.origin[c] = mn[c] - 0.5 * rcp;
      G.box[c] = (mx[c] - mn[c]) + rcp;
      G.hf[c] = (float)G.box[c];
      G.L[4 * c] = G.box[c];
      int nc = (int)std::floor(G.box[c] / (c == 2 ? w / z_refine : w));
      if (nc < 1) nc = 1;
      if (nc > 1000) nc = 1000;
      G.nc[c] = nc;
      G.kr[c] = (int)std::ceil(rcp * nc / G.box[c] * (1.0 + 1e-12));
      if (G.kr[c] < 1) G.kr[c] = 1;
      ext += std::fabs(G.origin[c]) + G.box[c];
    }
  }
  for (int q = 0; q < 9; ++q) G.Lf[q] = (float)G.L[q];
  for (int c = 0; c < 3; ++c) {
    G.inv_nc[c] = 1.0f / (float)G.nc[c];
    G.inv_hf[c] = 1.0f / G.hf[c];
  }
  // FP32 distances carry an error below ~1e-6 ext per component; the band
  // is four times the resulting bound on d^2
  double err = 4.0 * (2.0 * rcp * 4.0e-7 * ext + 1.0e-6 * G.rc2);
  G.rc2_lo = std::nextafter((float)(G.rc2 - err), 0.0f);
  G.rc2_hi = std::nextafter((float)(G.rc2 + err), 1e30f);
  G.natoms = natoms;
  return 0;
}

// the loaded potentials are Chebyshev bases with a spin block and the
// stale-spin option is on
bool stale_spin_wanted() {
  if (!g.angular_spin_stale || !g.dev_ready) return false;
  for (int t = 0; t < g.pd.ntypes; ++t)
    if (g.pd.sp[t].sftype == AE_SF_CHEBYSHEV && g.pd.sp[t].cheb.multi) return true;
  return false;
}

int plan_alloc(aenet_gpu_plan* P, const double* coords0, const double* lattices) {
  const double rc = P->rc;
  int cell_off = 0, atom_off = 0, nchunks = 0;
  size_t natoms = 0;
  double dens_max = 0;
  for (int s = 0; s < P->nstruc; ++s) {
    StructGeom& G = P->geom_h[s];
    const double* c0 = coords0 ? coords0 + 3 * (size_t)atom_off : nullptr;
    int st = make_geom(G, lattices ? lattices + 9 * (size_t)s : nullptr, P->pbc_h[s], c0,
                       P->natoms_h[s], rc, P->cell_div, 0, nullptr, P->z_refine);
    if (st) return st;
    int nc = G.nc[0] * G.nc[1] * G.nc[2];
    G.cell_off = cell_off;
    G.atom_off = atom_off;
    G.chunk_off = nchunks;
    nchunks += (P->natoms_h[s] + AE_ECHUNK - 1) / AE_ECHUNK;
    cell_off += nc;
    atom_off += P->natoms_h[s];
    natoms += P->natoms_h[s];
    double vol;
    if (G.pbc) {
      const double* a = G.L;
      double c[3];
      cross(a + 3, a + 6, c);
      vol = std::fabs(a[0] * c[0] + a[1] * c[1] + a[2] * c[2]);
    } else {
      vol = G.box[0] * G.box[1] * G.box[2];
    }
    double rcp = rc + 1e-3;
    double nbexp = 4.18879020478639 * rcp * rcp * rcp * P->natoms_h[s] / vol;
    if (!G.pbc) nbexp = std::min(nbexp, (double)P->natoms_h[s]);
    dens_max = std::max(dens_max, nbexp);
  }
  P->natoms = (int)natoms;
  P->ncells = cell_off;
  P->nchunks = nchunks;
  P->one_chunk_each = 1;
  for (int s = 0; s < P->nstruc; ++s)
    if (P->natoms_h[s] < 1 || P->natoms_h[s] > AE_ECHUNK) P->one_chunk_each = 0;
  if (P->cap <= 0) {
    int cap = (int)std::ceil(1.5 * dens_max + 32.0);
    P->cap = (cap + 31) & ~31;
  }
  if (P->cap_a <= 0) {
    // angular cut-off of the loaded potentials
    double arc = 0.0;
    if (P->pd)
      for (int t = 0; t < P->pd->ntypes; ++t)
        arc = std::max(arc, P->pd->sp[t].sftype == AE_SF_CHEBYSHEV ? P->pd->sp[t].cheb.a_Rc : rc);
    double frac = arc > 0 ? std::pow(std::min(1.0, (arc + 1e-3) / (rc + 1e-3)), 3) : 1.0;
    int ca = (int)std::ceil(1.5 * dens_max * frac + 16.0);
    ca = (ca + 7) & ~7;
    P->cap_a = std::min(ca, P->cap);
  }
  // layout
  const int N = P->natoms;
  const size_t tsz = P->fp64 ? 8 : 4;
  const size_t nsf_pad = P->pd ? (size_t)P->pd->nsf_pad : 4;
  const size_t npairs = (size_t)N * P->cap;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = (off + bytes + 255) & ~(size_t)255;
    return o;
  };
  size_t o_geom = take(sizeof(StructGeom) * P->nstruc);
  size_t o_as = take(4 * (size_t)N);
  size_t o_t0 = take(4 * (size_t)N);
  size_t o_s = take(24 * (size_t)N);
  size_t o_r = take(24 * (size_t)N);
  size_t o_rf = take(16 * (size_t)N);
  size_t o_co = take(4 * (size_t)N);
  size_t o_so = take(4 * (size_t)N);
  size_t o_cc = take(4 * (size_t)P->ncells);
  size_t o_cs = take(4 * ((size_t)P->ncells + 1));
  size_t o_sc = take(4 * ((size_t)P->ncells / 1024 + 2));
  size_t o_ca = take(4 * (size_t)N);
  size_t o_cp = take(16 * (size_t)N);
  size_t o_nc = take(4 * (size_t)N);
  size_t o_jt = take(4 * npairs);
  size_t o_vec = take((P->fp64 ? 32 : 16) * npairs);
  size_t o_img = P->keep_images ? take(4 * npairs) : 0;
  // moment buffer of the FP32 path: both blocks' moments per atom
  P->mom_pad = 0;
  if (!P->fp64 && P->pd && P->pd->qleg) {
    int aN = 0;
    for (int t = 0; t < P->pd->ntypes; ++t) aN = std::max(aN, P->pd->sp[t].cheb.a_N);
    if (aN <= AE_MOMA) P->mom_pad = (2 * aN * aN + 3) & ~3;
  }
  size_t o_M = P->mom_pad ? take(4 * (size_t)P->mom_pad * N) : 0;
  const bool stale = stale_spin_wanted();
  size_t o_rk = stale ? take(4 * npairs) : 0;
  size_t o_se = stale ? take(4 * npairs) : 0;
  size_t o_G = take(tsz * nsf_pad * N);
  size_t o_dG = take(tsz * nsf_pad * N);
  size_t o_E = take(8 * (size_t)N);
  size_t o_F = take(4 * tsz * (size_t)N);
  size_t o_Es = take(8 * (size_t)P->nstruc);
  size_t o_V = take(72 * (size_t)P->nstruc);
  size_t o_st = take(16);
  size_t o_ep = take(16 * (size_t)(P->nchunks + 1));
  size_t o_chs = take(4 * (size_t)(P->nchunks + 1));
  size_t o_ord = take(4 * (size_t)N);
  size_t o_spo = take(4 * (AE_MAXT + 1));
  size_t o_ps = take(4 * (size_t)ae_part_scratch_ints(N));
  // per-structure search: every structure's cell lists and row counters
  // (28 B per atom, 4 B per cell) fit one block's shared memory (at most 48 KB with the unit
  // tables)
  int max_n = 0, max_c = 0;
  for (int s = 0; s < P->nstruc; ++s) {
    max_n = std::max(max_n, P->natoms_h[s]);
    max_c = std::max(max_c, P->geom_h[s].nc[0] * P->geom_h[s].nc[1] * P->geom_h[s].nc[2]);
  }
  // and there are enough structures to give every SM a few blocks (fewer,
  // larger structures spread better one warp per atom)
  int nsm = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    nsm = 0;
  const bool per_struct = nsm > 0 && P->nstruc >= 2 * nsm &&
                          28 * (size_t)max_n + 4 * ((size_t)max_c + 1) + 24576 <= 48 * 1024;
  size_t o_so2 = per_struct ? take(4 * (size_t)P->nstruc) : 0;
  if (cudaMalloc(&P->mem, off) != cudaSuccess) return AENET_ERR_CUDA;
  P->mem_bytes = off;
  char* b = (char*)P->mem;
  P->geom_d = (StructGeom*)(b + o_geom);
  P->atom_struct = (int*)(b + o_as);
  P->types0 = (int*)(b + o_t0);
  P->s_wrap = (double*)(b + o_s);
  P->r_wrap = (double*)(b + o_r);
  P->r_f32 = (float4*)(b + o_rf);
  P->cell_of = (int*)(b + o_co);
  P->slot_of = (int*)(b + o_so);
  P->cell_count = (int*)(b + o_cc);
  P->cell_start = (int*)(b + o_cs);
  P->scan_tmp = (int*)(b + o_sc);
  P->cell_atoms = (int*)(b + o_ca);
  P->cell_pos = (float4*)(b + o_cp);
  P->nb_cnt = (int*)(b + o_nc);
  P->nb_jt = (int*)(b + o_jt);
  P->nb_vec = (void*)(b + o_vec);
  P->nb_img = P->keep_images ? (int*)(b + o_img) : nullptr;
  P->M = P->mom_pad ? (float*)(b + o_M) : nullptr;
  P->nb_rank = stale ? (int*)(b + o_rk) : nullptr;
  P->nb_seff = stale ? (float*)(b + o_se) : nullptr;
  P->G = (void*)(b + o_G);
  P->dEdG = (void*)(b + o_dG);
  P->E_atom = (double*)(b + o_E);
  P->Facc = (void*)(b + o_F);
  P->E_struct = (double*)(b + o_Es);
  P->virial = (double*)(b + o_V);
  P->status = (unsigned*)(b + o_st);
  P->e_part = (double2*)(b + o_ep);
  P->chunk_struct = (int*)(b + o_chs);
  P->order = (int*)(b + o_ord);
  P->spec_off = (int*)(b + o_spo);
  P->part_scratch = (int*)(b + o_ps);
  P->struct_order = per_struct ? (int*)(b + o_so2) : nullptr;
  P->smem_atoms = max_n;
  P->smem_cells = max_c;
  if (per_struct) {
    std::vector<int> ord(P->nstruc);
    for (int s = 0; s < P->nstruc; ++s) ord[s] = s;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int c) { return P->natoms_h[a] > P->natoms_h[c]; });
    cudaMemcpy(P->struct_order, ord.data(), 4 * (size_t)P->nstruc, cudaMemcpyHostToDevice);
  }
  std::vector<int> as(N);
  for (int s = 0, a = 0; s < P->nstruc; ++s)
    for (int q = 0; q < P->natoms_h[s]; ++q) as[a++] = s;
  cudaMemcpy(P->geom_d, P->geom_h.data(), sizeof(StructGeom) * P->nstruc, cudaMemcpyHostToDevice);
  if (N) cudaMemcpy(P->atom_struct, as.data(), 4 * (size_t)N, cudaMemcpyHostToDevice);
  std::vector<int> cs;
  cs.reserve(P->nchunks);
  for (int s = 0; s < P->nstruc; ++s)
    for (int c = 0; c < (P->natoms_h[s] + AE_ECHUNK - 1) / AE_ECHUNK; ++c) cs.push_back(s);
  if (!cs.empty())
    cudaMemcpy(P->chunk_struct, cs.data(), 4 * cs.size(), cudaMemcpyHostToDevice);
  cudaMemset(P->status, 0, 16);
  if (cudaDeviceSynchronize() != cudaSuccess) return AENET_ERR_CUDA;
  return 0;
}

aenet_gpu_plan* plan_new(int nstruc, const int* natoms, const double* lattices, const int* pbc,
                         const double* coords0, int precision, const PotDevice* pd, double rc,
                         int cap, bool keep_images, int* stat) {
  auto P = std::make_unique<aenet_gpu_plan>();
  P->nstruc = nstruc;
  P->fp64 = precision == AENET_GPU_FP64 ? 1 : 0;
  P->natoms_h.assign(natoms, natoms + nstruc);
  P->pbc_h.assign(nstruc, 1);
  if (pbc)
    for (int s = 0; s < nstruc; ++s) P->pbc_h[s] = pbc[s] ? 1 : 0;
  for (int s = 0; s < nstruc; ++s)
    if (natoms[s] < 0 || (P->pbc_h[s] && !lattices)) {
      *stat = AENET_ERR_INPUT;
      return nullptr;
    }
  P->geom_h.resize(nstruc);
  P->pd = pd;
  P->rc = rc;
  P->cell_div = g.cell_div;
  P->z_refine = g.z_refine;
  P->cap = cap;
  P->cap_a = cap > 0 ? cap : 0;   // an explicit capacity (a retry) stages every neighbour
  P->keep_images = keep_images;
  int st = plan_alloc(P.get(), coords0, lattices);
  if (st) {
    *stat = st;
    return nullptr;
  }
  *stat = 0;
  return P.release();
}

DescBuffers desc_buffers(aenet_gpu_plan* P, const double* grad_scale, bool virial) {
  DescBuffers d{};
  d.natoms = P->natoms;
  d.types = P->types0;
  d.nb_cnt = P->nb_cnt;
  d.nb_jt = P->nb_jt;
  d.nb_vec = P->nb_vec;
  d.cap = P->cap;
  d.cap_a = P->cap_a;
  d.lpa = P->lpa ? P->lpa : g.lpa_default;
  d.G = P->G;
  d.dEdG = P->dEdG;
  d.E_atom = P->E_atom;
  d.F = P->Facc;
  d.virial = virial ? P->virial : nullptr;
  d.atom_struct = P->atom_struct;
  d.grad_scale = grad_scale;
  d.status = P->status;
  if (g.angular_moments && P->M) {
    d.M = P->M;
    d.mom_pad = P->mom_pad;
  }
  if (P->nb_rank) {
    d.nb_rank = P->nb_rank;
    d.nb_seff = P->nb_seff;
    d.M = nullptr;    // ordered spin weights need the pair form
  }
  return d;
}

NbBuffers nb_buffers(aenet_gpu_plan* P) {
  NbBuffers nb{};
  nb.geom = P->geom_d;
  nb.atom_struct = P->atom_struct;
  nb.s_wrap = P->s_wrap;
  nb.r_wrap = P->r_wrap;
  nb.r_f32 = P->r_f32;
  nb.cell_of = P->cell_of;
  nb.slot_of = P->slot_of;
  nb.cell_count = P->cell_count;
  nb.cell_start = P->cell_start;
  nb.scan_tmp = P->scan_tmp;
  nb.cell_atoms = P->cell_atoms;
  nb.cell_pos = P->cell_pos;
  nb.ncells_total = P->ncells;
  nb.nstruc = P->nstruc;
  nb.cap = P->cap;
  nb.nb_cnt = P->nb_cnt;
  nb.nb_jt = P->nb_jt;
  nb.nb_vec = P->nb_vec;
  nb.nb_img = P->nb_img;
  nb.status = P->status;
  nb.cell_kernel = g.nb_cell;
  nb.struct_order = P->struct_order;
  nb.smem_atoms = P->smem_atoms;
  nb.smem_cells = P->smem_cells;
  return nb;
}

int ck(int e) { return e ? AENET_ERR_CUDA : 0; }

// The types the neighbour search reads: the per-structure searches take
// the caller's 1-based ids and write the checked 0-based ones themselves;
// the other searches read the 0-based ids of the type kernel, launched
// here.  Null on a launch error.
const int* search_types(aenet_gpu_plan* P, NbBuffers& nb, const int* d_types, cudaStream_t s) {
  if ((nb.cell_kernel == 4 || nb.cell_kernel == 5) && nb.struct_order) {
    nb.types0_out = P->types0;
    nb.ntypes = P->pd->ntypes;
    return d_types;
  }
  if (ae_launch_types(P->natoms, d_types, P->types0, P->pd->ntypes, P->status, s)) return nullptr;
  return P->types0;
}

int plan_eval(aenet_gpu_plan* P, double* d_E, double* d_E_atoms, cudaStream_t s);

// neighbours + descriptors + networks + energies
int plan_forward(aenet_gpu_plan* P, const double* d_coords, const int* d_types, double* d_E,
                 double* d_E_atoms, cudaStream_t s) {
  NbBuffers nb = nb_buffers(P);
  const int* t_in = search_types(P, nb, d_types, s);
  if (!t_in) return AENET_ERR_CUDA;
  if (ck(ae_launch_neighbors(P->natoms, d_coords, t_in, nb, P->fp64, s))) return AENET_ERR_CUDA;
  return plan_eval(P, d_E, d_E_atoms, s);
}

// networks: tensor-core kernel on the mixed path when the networks fit it
// (atoms grouped by species first), the SIMT kernel otherwise
int plan_networks(aenet_gpu_plan* P, const DescBuffers& d, cudaStream_t s) {
  const PotDevice& pd = *P->pd;
  if (!P->fp64 && pd.tc_ok && g.networks_tc) {
    if (ck(ae_launch_partition(P->natoms, pd.ntypes, P->types0, P->part_scratch, P->order,
                               P->spec_off, s)))
      return AENET_ERR_CUDA;
    return ck(ae_launch_mlp_tc(pd, d, P->order, P->spec_off, s));
  }
  return ck(ae_launch_mlp(pd, d, P->fp64, s));
}

// descriptors + networks + energies on the current neighbour table
int plan_eval(aenet_gpu_plan* P, double* d_E, double* d_E_atoms, cudaStream_t s) {
  const PotDevice& pd = *P->pd;
  DescBuffers d = desc_buffers(P, nullptr, false);
  if (d.nb_rank &&
      ck(ae_launch_stale_order(P->natoms, P->geom_d, P->atom_struct, P->r_wrap, pd, d, P->fp64,
                               P->stale_caller_order, P->nb_rank, P->nb_seff, s)))
    return AENET_ERR_CUDA;
  int e = (pd.sp[0].sftype == AE_SF_BEHLER) ? ae_launch_behler_forward(pd, d, P->fp64, s)
                                             : ae_launch_chebyshev_forward(pd, d, P->fp64, s);
  if (ck(e)) return AENET_ERR_CUDA;
  if (plan_networks(P, d, s)) return AENET_ERR_CUDA;
  if (ck(ae_launch_energy_reduce_chunked(P->nstruc, P->nchunks, P->geom_d, P->chunk_struct,
                                         P->E_atom, P->e_part, P->E_struct, P->one_chunk_each, s)))
    return AENET_ERR_CUDA;
  if (d_E && cudaMemcpyAsync(d_E, P->E_struct, 8 * (size_t)P->nstruc, cudaMemcpyDeviceToDevice, s))
    return AENET_ERR_CUDA;
  if (d_E_atoms &&
      cudaMemcpyAsync(d_E_atoms, P->E_atom, 8 * (size_t)P->natoms, cudaMemcpyDeviceToDevice, s))
    return AENET_ERR_CUDA;
  return 0;
}

int plan_adjoint(aenet_gpu_plan* P, const double* grad_scale, double* d_out, double out_sign,
                 double* d_virial, cudaStream_t s) {
  const PotDevice& pd = *P->pd;
  const size_t tsz = P->fp64 ? 8 : 4;
  if (cudaMemsetAsync(P->Facc, 0, 4 * tsz * (size_t)P->natoms, s)) return AENET_ERR_CUDA;
  if (d_virial && cudaMemsetAsync(P->virial, 0, 72 * (size_t)P->nstruc, s)) return AENET_ERR_CUDA;
  DescBuffers d = desc_buffers(P, grad_scale, d_virial != nullptr);
  if (g.lpa_adjoint) d.lpa = g.lpa_adjoint;
  int e = (pd.sp[0].sftype == AE_SF_BEHLER) ? ae_launch_behler_adjoint(pd, d, P->fp64, s)
                                             : ae_launch_chebyshev_adjoint(pd, d, P->fp64, s);
  if (ck(e)) return AENET_ERR_CUDA;
  if (d_out && ck(ae_launch_forces_out(P->natoms, P->Facc, P->fp64, d_out, out_sign, s)))
    return AENET_ERR_CUDA;
  if (d_virial &&
      cudaMemcpyAsync(d_virial, P->virial, 72 * (size_t)P->nstruc, cudaMemcpyDeviceToDevice, s))
    return AENET_ERR_CUDA;
  return 0;
}

}  // namespace

// =====================================================================
//                     libaenet API (include/aenet.h)
// =====================================================================

EXPORT void aenet_init(int ntypes, char* atom_types[], int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g.init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  if (ntypes < 1 || ntypes > AE_MAXT || !atom_types) {
    *stat = AENET_ERR_MALLOC;
    return;
  }
  g.pots.clear();
  g.types.clear();
  g.blob.reset();
  g.dev_ready = false;
  g.loaded = false;
  g.ntypes = ntypes;
  for (int i = 0; i < ntypes; ++i) {
    char buf[3] = {0, 0, 0};
    if (atom_types[i]) strncpy(buf, atom_types[i], 2);
    g.types.push_back(trim(buf));
  }
  g.pots.assign(ntypes, HostPot());
  g.init = true;
  *stat = AENET_OK;
}

EXPORT void aenet_final(int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  *stat = AENET_OK;
  if (g.init) {
    host_cache_reset();
    nlist_release();
    g.blob.reset();
    g.pots.clear();
    g.types.clear();
    g.init = false;
    g.loaded = false;
    g.dev_ready = false;
    g.ntypes = 0;
  }
}

EXPORT void aenet_print_info(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init) {
    printf(" Nothing to print. AenetLib is not initialized.\n");
    return;
  }
  for (int t = 0; t < g.ntypes; ++t) {
    const HostPot& p = g.pots[t];
    if (!p.init) continue;
    printf(" Atomic species : %s\n File name      : %s\n\n", p.stp.atomtype.c_str(), p.path.c_str());
    printf(" Network        :");
    for (int l = 0; l < p.net.nlayers; ++l) printf(" %d", p.net.nnodes[l]);
    printf("\n Descriptor     : %s, %d functions, Rc = %.3f\n", p.stp.sftype.c_str(), p.stp.nsf,
           p.stp.Rc_max);
    printf(" E_scale, E_shift, E_atom : %.10g %.10g %.10g\n\n", p.E_scale, p.E_shift, p.E_atom);
  }
}

EXPORT void aenet_load_potential(int type_id, char* filename, int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!filename) {
    *stat = AENET_ERR_IO;
    return;
  }
  if (strlen(filename) > 1024) {   // aenet.f90:303-307
    *stat = AENET_ERR_MALLOC;
    return;
  }
  if (!g.init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  if (type_id <= 0 || type_id > g.ntypes) {
    *stat = AENET_ERR_TYPE;
    return;
  }
  std::string path = trim(filename);
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    *stat = AENET_ERR_IO;
    return;
  }
  fclose(f);
  HostPot pot;
  int st = load_nn(path.c_str(), g.types, pot);
  if (st) {
    *stat = AENET_ERR_IO;
    return;
  }
  g.pots[type_id - 1] = std::move(pot);
  g.dev_ready = false;
  bool all = true;
  for (auto& p : g.pots) all = all && p.init;
  if (all) {
    // pot_get_range (potential.f90:244-266), lcl_nmax_nbdist, stp_nsf_max
    double rmin = g.pots[0].stp.Rc_min, rmax = g.pots[0].stp.Rc_max;
    int nsf = 0;
    for (auto& p : g.pots) {
      rmin = std::min(rmin, p.stp.Rc_min);
      rmax = std::max(rmax, p.stp.Rc_max);
      nsf = std::max(nsf, p.stp.nsf);
    }
    aenet_Rc_min = rmin;
    aenet_Rc_max = rmax;
    aenet_nnb_max = nmax_nbdist(rmin, rmax);
    aenet_nsf_max = nsf;
    g.loaded = true;
  }
  *stat = AENET_OK;
}

EXPORT bool aenet_all_loaded(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init) return true;   // empty loop over zero potentials
  for (auto& p : g.pots)
    if (!p.init) return false;
  return true;
}

EXPORT double aenet_free_atom_energy(int type_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init || type_id < 1 || type_id > g.ntypes) return 0.0;
  return g.pots[type_id - 1].E_atom;
}

namespace {

// Workspace of the per-atom calls: device scratch and a pinned staging
// block that grow to the largest call seen and are then reused, and a
// library stream.  A call copies its inputs in with one transfer and its
// energy, status and forces out with one; nothing is allocated once the
// buffers are large enough.  The sequence of one call (copy in, kernels,
// copy out) is captured once per row capacity as a CUDA graph and then
// replayed, one launch per call.  The buffers live until the process exits.
struct AtomGraph {
  int cap, forces, stale, gen;
  cudaGraphExec_t exec;
};
struct AtomScratch {
  char* dev = nullptr;
  size_t dev_bytes = 0;
  char* host = nullptr;
  size_t host_bytes = 0;
  cudaStream_t stream = nullptr;
  std::vector<AtomGraph> graphs;
  char* mhost = nullptr;   // mapped pinned block of the fused per-atom launch
  char* mdev = nullptr;    // its device address
  size_t mbytes = 0;
  void drop_graphs() {
    for (auto& q : graphs) cudaGraphExecDestroy(q.exec);
    graphs.clear();
  }
};
AtomScratch g_atom;

int atom_scratch_reserve(size_t dev_bytes, size_t host_bytes) {
  if (!g_atom.stream && cudaStreamCreateWithFlags(&g_atom.stream, cudaStreamNonBlocking))
    return AENET_ERR_CUDA;
  if (g_atom.dev_bytes < dev_bytes || g_atom.host_bytes < host_bytes) g_atom.drop_graphs();
  if (g_atom.dev_bytes < dev_bytes) {
    if (g_atom.dev) cudaFree(g_atom.dev);
    g_atom.dev = nullptr;
    g_atom.dev_bytes = 0;
    const size_t want = std::max(dev_bytes, (size_t)1 << 20);
    if (cudaMalloc((void**)&g_atom.dev, want) != cudaSuccess) {
      g_atom.dev = nullptr;
      return AENET_ERR_MALLOC;
    }
    g_atom.dev_bytes = want;
  }
  if (g_atom.host_bytes < host_bytes) {
    if (g_atom.host) cudaFreeHost(g_atom.host);
    g_atom.host = nullptr;
    g_atom.host_bytes = 0;
    const size_t want = std::max(host_bytes, (size_t)1 << 18);
    if (cudaMallocHost((void**)&g_atom.host, want) != cudaSuccess) {
      g_atom.host = nullptr;
      return AENET_ERR_MALLOC;
    }
    g_atom.host_bytes = want;
  }
  return 0;
}

int atom_mapped_reserve(size_t bytes) {
  if (!g_atom.stream && cudaStreamCreateWithFlags(&g_atom.stream, cudaStreamNonBlocking))
    return AENET_ERR_CUDA;
  if (g_atom.mbytes >= bytes) return 0;
  if (g_atom.mhost) cudaFreeHost(g_atom.mhost);
  g_atom.mhost = g_atom.mdev = nullptr;
  g_atom.mbytes = 0;
  const size_t want = std::max(bytes, (size_t)1 << 16);
  if (cudaHostAlloc((void**)&g_atom.mhost, want, cudaHostAllocMapped) != cudaSuccess) {
    g_atom.mhost = nullptr;
    return AENET_ERR_MALLOC;
  }
  if (cudaHostGetDevicePointer((void**)&g_atom.mdev, g_atom.mhost, 0) != cudaSuccess) {
    cudaFreeHost(g_atom.mhost);
    g_atom.mhost = g_atom.mdev = nullptr;
    return AENET_ERR_CUDA;
  }
  g_atom.mbytes = want;
  return 0;
}

// One FP64 Chebyshev atom in one launch of the fused per-atom kernel (a
// cluster of blocks, or one block), the row and the results in mapped host
// memory; AE_ATOM_NA when the potential or the row does not fit that
// kernel.
int atomic_eval_fused(const double* coo_i, int type_i, int n_j, const double* coo_j,
                      const int* type_j, double* E_i, double* F_local) {
  const size_t in_bytes =
      ((size_t)AE_ATOM_IN_VEC + 36 * (size_t)n_j + 255) & ~(size_t)255;
  const size_t out_bytes = AE_ATOM_OUT_F + 24 * (size_t)(n_j + 1);
  int st = atom_mapped_reserve(in_bytes + out_bytes);
  if (st) return st;
  char* h = g_atom.mhost;
  AtomCallHeader* hd = reinterpret_cast<AtomCallHeader*>(h);
  hd->n = n_j;
  hd->ti = type_i - 1;
  hd->forces = F_local ? 1 : 0;
  hd->pad = 0;
  // R_ij = coo_j - coo_i (sfbasis.f90:488) and its length
  double* vec = reinterpret_cast<double*>(h + AE_ATOM_IN_VEC);
  int* ty = reinterpret_cast<int*>(h + AE_ATOM_IN_VEC + 32 * (size_t)n_j);
  const double a_Rc = g.pd.sp[type_i - 1].cheb.a_Rc;
  long long na = 0;   // angular neighbours
  for (int j = 0; j < n_j; ++j) {
    double R[3];
    for (int c = 0; c < 3; ++c) R[c] = coo_j[3 * j + c] - coo_i[c];
    vec[4 * j] = R[0];
    vec[4 * j + 1] = R[1];
    vec[4 * j + 2] = R[2];
    vec[4 * j + 3] = std::sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
    ty[j] = type_j[j] - 1;
    if (vec[4 * j + 3] <= a_Rc) ++na;
  }
  const char* ho = h + in_bytes;
  // one block is as fast for short rows whose pairs fit one round of its
  // pair threads (a cluster's launch and barriers cost a few
  // microseconds); the cluster is faster from there (measured on GB300:
  // 45 vs 53 us at 78 neighbours and 250 pairs, 114 vs 552 us at 300
  // neighbours)
  const bool cluster =
      g.atom_fused == 3 ||
      (g.atom_fused == 2 && (n_j >= AE_ATOM_CLUSTER_ROWS || na * (na - 1) / 2 > AE_ATOM_BLOCK_PAIRS));
  const int e = ae_launch_atom(g.pd, *hd, g_atom.mdev, g_atom.mdev + in_bytes, cluster,
                               g_atom.stream);
  if (e == AE_ATOM_NA) return AE_ATOM_NA;
  if (e || cudaStreamSynchronize(g_atom.stream) != cudaSuccess) return AENET_ERR_CUDA;
  if (*reinterpret_cast<const unsigned*>(ho + 8)) return AENET_ERR_CUDA;
  *E_i = *reinterpret_cast<const double*>(ho);
  if (F_local) memcpy(F_local, ho + AE_ATOM_OUT_F, 24 * (size_t)(n_j + 1));
  return 0;
}

// One atom with caller-supplied neighbours, evaluated on the GPU as a
// one-row neighbour table (aenet.f90:359-486).  F_local[(n_j+1)*3]
// receives the forces on the central atom (row 0) and on each neighbour.
// With the option angular_spin = stale the spin weights follow the
// caller's neighbour order, as sfb_eval's do.
int atomic_eval(const double* coo_i, int type_i, int n_j, const double* coo_j, const int* type_j,
                double* E_i, double* F_local) {
  if (!(g.init && g.loaded)) return AENET_ERR_INIT;
  if (type_i < 1 || type_i > g.ntypes || n_j < 0) return AENET_ERR_TYPE;
  for (int j = 0; j < n_j; ++j)
    if (type_j[j] < 1 || type_j[j] > g.ntypes) return AENET_ERR_TYPE;
  int st = ensure_device();
  if (st) return st;
  const PotDevice& pd = g.pd;
  const int cap = std::max(32, (n_j + 31) & ~31);
  const bool fp64 = true;
  const bool stale = stale_spin_wanted();
  if (g.atom_fused && !stale && n_j <= AE_ATOM_NMAX) {
    st = atomic_eval_fused(coo_i, type_i, n_j, coo_j, type_j, E_i, F_local);
    if (st != AE_ATOM_NA) return st;
  }
  const size_t nsf_pad = pd.nsf_pad;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = (off + bytes + 255) & ~(size_t)255;
    return o;
  };
  // inputs (one upload), device-only work arrays, outputs (one download)
  const size_t o_vec = take(32 * (size_t)cap), o_jt = take(4 * (size_t)cap), o_hdr = take(16);
  const size_t up_bytes = off;
  const size_t o_rk = stale ? take(4 * (size_t)cap) : 0, o_se = stale ? take(4 * (size_t)cap) : 0;
  const size_t o_G = take(8 * nsf_pad), o_dG = take(8 * nsf_pad);
  const size_t o_out = take(0);
  const size_t out_bytes = 32 + 32 * (size_t)(cap + 1);   // E, status, pad, force rows
  take(out_bytes);
  st = atom_scratch_reserve(off, std::max(up_bytes, out_bytes));
  if (st) return st;
  // host neighbour row: R_ij = coo_j - coo_i (sfbasis.f90:488)
  char* h = g_atom.host;
  double* vec = (double*)(h + o_vec);
  int* jt = (int*)(h + o_jt);
  memset(h, 0, up_bytes);
  for (int j = 0; j < n_j; ++j) {
    double R[3];
    for (int c = 0; c < 3; ++c) R[c] = coo_j[3 * j + c] - coo_i[c];
    vec[4 * j] = R[0];
    vec[4 * j + 1] = R[1];
    vec[4 * j + 2] = R[2];
    vec[4 * j + 3] = std::sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
    jt[j] = (j + 1) | ((type_j[j] - 1) << AE_TYPE_SHIFT);
  }
  int* hdr = (int*)(h + o_hdr);
  hdr[0] = n_j;         // neighbour count
  hdr[1] = type_i - 1;  // central species (0-based)
  hdr[2] = 0;           // structure of the atom
  char* b = g_atom.dev;
  cudaStream_t s = g_atom.stream;
  DescBuffers d{};
  d.natoms = 1;
  d.types = (const int*)(b + o_hdr + 4);
  d.nb_cnt = (const int*)(b + o_hdr);
  d.nb_jt = (const int*)(b + o_jt);
  d.nb_vec = b + o_vec;
  d.cap = cap;
  d.cap_a = cap;
  d.lpa = 32;
  d.G = b + o_G;
  d.dEdG = b + o_dG;
  d.E_atom = (double*)(b + o_out);
  d.status = (unsigned*)(b + o_out + 8);
  d.F = b + o_out + 32;
  d.virial = nullptr;
  d.atom_struct = (const int*)(b + o_hdr + 8);
  d.grad_scale = nullptr;
  const bool behler = pd.sp[0].sftype == AE_SF_BEHLER;
  const bool use_stale = stale && !behler;
  if (use_stale) {
    d.nb_rank = (const int*)(b + o_rk);
    d.nb_seff = (const float*)(b + o_se);
  }
  const size_t down = F_local ? out_bytes : 16;
  // the whole call on the stream: copy in, clear outputs, kernels, copy out
  auto enqueue = [&]() -> int {
    int e = (int)cudaMemcpyAsync(b, h, up_bytes, cudaMemcpyHostToDevice, s);
    if (!e) e = (int)cudaMemsetAsync(b + o_out, 0, out_bytes, s);
    if (!e && use_stale)
      e = ae_launch_stale_order(1, nullptr, nullptr, nullptr, pd, d, 1, 1, (int*)(b + o_rk),
                                (float*)(b + o_se), s);
    if (!e) e = behler ? ae_launch_behler_forward(pd, d, fp64, s) : ae_launch_chebyshev_forward(pd, d, fp64, s);
    if (!e) e = ae_launch_mlp(pd, d, fp64, s);
    if (!e && F_local)
      e = behler ? ae_launch_behler_adjoint(pd, d, fp64, s) : ae_launch_chebyshev_adjoint(pd, d, fp64, s);
    if (!e) e = (int)cudaMemcpyAsync(h, b + o_out, down, cudaMemcpyDeviceToHost, s);
    return e;
  };
  const int fkey = F_local ? 1 : 0, skey = use_stale ? 1 : 0;
  cudaGraphExec_t exec = nullptr;
  for (auto& q : g_atom.graphs)
    if (q.cap == cap && q.forces == fkey && q.stale == skey && q.gen == g.gen) exec = q.exec;
  if (!exec) {
    // capture this call's sequence once for the row capacity
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int e = enqueue();
      const cudaError_t ee = cudaStreamEndCapture(s, &graph);
      if (!e && ee == cudaSuccess && graph &&
          cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
        std::vector<AtomGraph> keep;
        for (auto& q : g_atom.graphs) {
          if (q.gen == g.gen) keep.push_back(q);
          else cudaGraphExecDestroy(q.exec);
        }
        g_atom.graphs.swap(keep);
        g_atom.graphs.push_back(AtomGraph{cap, fkey, skey, g.gen, exec});
      } else {
        exec = nullptr;
      }
      if (graph) cudaGraphDestroy(graph);
    }
    cudaGetLastError();   // a failed capture leaves nothing behind: run directly
  }
  int e = exec ? (int)cudaGraphLaunch(exec, s) : enqueue();
  if (!e) e = (int)cudaStreamSynchronize(s);
  if (e) return AENET_ERR_CUDA;
  const unsigned status = *(const unsigned*)(h + 8);
  if (status) return AENET_ERR_CUDA;
  *E_i = *(const double*)h;
  if (F_local) {
    const double* f4 = (const double*)(h + 32);
    for (int q = 0; q <= n_j; ++q)
      for (int c = 0; c < 3; ++c) F_local[3 * q + c] = f4[4 * q + c];
  }
  return 0;
}

}  // namespace

EXPORT void aenet_atomic_energy(double coo_i[3], int type_i, int n_j, double coo_j[],
                                int type_j[], double* E_i, int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  *stat = atomic_eval(coo_i, type_i, n_j, coo_j, type_j, E_i, nullptr);
}

EXPORT void aenet_atomic_energy_and_forces(double coo_i[3], int type_i, int index_i, int n_j,
                                           double coo_j[], int type_j[], int index_j[],
                                           int natoms, double* E_i, double F[], int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (index_i < 1 || index_i > natoms) {
    *stat = AENET_ERR_INPUT;
    return;
  }
  for (int j = 0; j < n_j; ++j)
    if (index_j[j] < 1 || index_j[j] > natoms) {
      *stat = AENET_ERR_INPUT;
      return;
    }
  std::vector<double> Fl(3 * (size_t)(n_j + 1));
  int st = atomic_eval(coo_i, type_i, n_j, coo_j, type_j, E_i, Fl.data());
  if (st) {
    *stat = st;
    return;
  }
  // accumulate into the caller's F (aenet.f90:471-477)
  for (int c = 0; c < 3; ++c) F[3 * (index_i - 1) + c] += Fl[c];
  for (int j = 0; j < n_j; ++j)
    for (int c = 0; c < 3; ++c) F[3 * (index_j[j] - 1) + c] += Fl[3 * (j + 1) + c];
  *stat = AENET_OK;
}

EXPORT void aenet_convert_atom_types(int ntypes_in, char* atom_types[], int natoms_in,
                                     int type_id_in[], int type_id_out[], int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  // geo_type_conv: map by name from the input type list to the library's
  for (int i = 0; i < natoms_in; ++i) {
    int t = type_id_in[i];
    if (t < 1 || t > ntypes_in || !atom_types[t - 1]) {
      *stat = AENET_ERR_TYPE;
      return;
    }
    char buf[3] = {0, 0, 0};
    strncpy(buf, atom_types[t - 1], 2);
    std::string name = trim(buf);
    int out = 0;
    for (int q = 0; q < g.ntypes; ++q)
      if (g.types[q] == name) {
        out = q + 1;
        break;
      }
    if (!out) {
      *stat = AENET_ERR_TYPE;
      return;
    }
    type_id_out[i] = out;
  }
  *stat = AENET_OK;
}

// ---- stand-alone Chebyshev basis (aenet.f90:652-799) ----------------

EXPORT void aenet_sfb_init(int ntypes, char* atom_types[], int radial_order, int angular_order,
                           double radial_Rc, double angular_Rc, int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  (void)atom_types;
  if (g.sfb_init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  if (ntypes < 1 || ntypes > AE_MAXT || radial_order < 0 || angular_order < 0 ||
      radial_order + 1 > AE_MAXCHEB || angular_order + 1 > AE_MAXCHEB) {
    *stat = AENET_ERR_INPUT;
    return;
  }
  if (!cuda_ok()) {
    *stat = AENET_ERR_CUDA;
    return;
  }
  PotDevice pd{};
  pd.ntypes = 1;
  ChebTable& ct = pd.sp[0].cheb;
  pd.sp[0].sftype = AE_SF_CHEBYSHEV;
  ct.r_Rc = radial_Rc;
  ct.a_Rc = angular_Rc;
  ct.r_N = radial_order + 1;
  ct.a_N = angular_order + 1;
  ct.multi = ntypes > 1;
  ct.nsf = (ct.r_N + ct.a_N) * (ct.multi ? 2 : 1);
  ct.r_i1 = 0;
  ct.a_i1 = ct.r_N;
  ct.r_i2 = ct.r_N + ct.a_N;
  ct.a_i2 = 2 * ct.r_N + ct.a_N;
  ct.angular_legacy = g.angular_legacy;
  for (int t = 0; t < ntypes; ++t) ct.spin[t] = typespin(ntypes, t + 1);
  pd.sp[0].nsf = ct.nsf;
  pd.nsf_max = ct.nsf;
  pd.nsf_pad = (ct.nsf + 3) & ~3;
  std::vector<double> shift(pd.nsf_pad, 0.0), scale(pd.nsf_pad, 1.0);
  std::vector<float> shift2(2 * (size_t)pd.nsf_pad, 0.f), scale32(pd.nsf_pad, 1.f);
  auto blob = std::make_unique<DevBlob>();
  if (cudaMalloc(&blob->p, 28 * (size_t)pd.nsf_pad) != cudaSuccess) {
    *stat = AENET_ERR_CUDA;
    return;
  }
  cudaMemcpy(blob->p, shift.data(), 8 * (size_t)pd.nsf_pad, cudaMemcpyHostToDevice);
  cudaMemcpy((char*)blob->p + 8 * (size_t)pd.nsf_pad, scale.data(), 8 * (size_t)pd.nsf_pad,
             cudaMemcpyHostToDevice);
  cudaMemcpy((char*)blob->p + 16 * (size_t)pd.nsf_pad, shift2.data(), 8 * (size_t)pd.nsf_pad,
             cudaMemcpyHostToDevice);
  cudaMemcpy((char*)blob->p + 24 * (size_t)pd.nsf_pad, scale32.data(), 4 * (size_t)pd.nsf_pad,
             cudaMemcpyHostToDevice);
  pd.shift = (const double*)blob->p;
  pd.scale = (const double*)((char*)blob->p + 8 * (size_t)pd.nsf_pad);
  pd.shift2 = (const float2*)((char*)blob->p + 16 * (size_t)pd.nsf_pad);
  pd.scale32 = (const float*)((char*)blob->p + 24 * (size_t)pd.nsf_pad);
  g.sfb_pd = pd;
  g.sfb_blob = std::move(blob);
  g.sfb_ntypes = ntypes;
  g.sfb_rorder = radial_order;
  g.sfb_aorder = angular_order;
  g.sfb_rRc = radial_Rc;
  g.sfb_aRc = angular_Rc;
  g.sfb_init = true;
  *stat = AENET_OK;
}

EXPORT void aenet_sfb_final(int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.sfb_init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  g.sfb_blob.reset();
  g.sfb_init = false;
  *stat = AENET_OK;
}

EXPORT int aenet_sfb_nvalues(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g.sfb_init ? g.sfb_pd.sp[0].cheb.nsf : 0;
}

EXPORT void aenet_sfb_eval(int itype0, double coo0[3], int nat, int itype1[], double coo1[], int nv,
                           double values[], int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  (void)itype0;
  if (!g.sfb_init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  const PotDevice& pd = g.sfb_pd;
  if (nv != pd.sp[0].cheb.nsf || nat < 0) {
    *stat = AENET_ERR_INPUT;
    return;
  }
  for (int j = 0; j < nat; ++j)
    if (itype1[j] < 1 || itype1[j] > g.sfb_ntypes) {
      *stat = AENET_ERR_TYPE;
      return;
    }
  const int cap = std::max(32, (nat + 31) & ~31);
  std::vector<double> vec(4 * (size_t)cap, 0.0);
  std::vector<int> jt(cap, 0);
  for (int j = 0; j < nat; ++j) {
    double R[3];
    for (int c = 0; c < 3; ++c) R[c] = coo1[3 * j + c] - coo0[c];
    for (int c = 0; c < 3; ++c) vec[4 * j + c] = R[c];
    vec[4 * j + 3] = std::sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
    jt[j] = (j + 1) | ((itype1[j] - 1) << AE_TYPE_SHIFT);
  }
  size_t nsf_pad = pd.nsf_pad;
  void* mem = nullptr;
  size_t bytes = 32 * (size_t)cap + 4 * (size_t)cap + 64 + 16 * nsf_pad + 1024;
  if (cudaMalloc(&mem, bytes) != cudaSuccess) {
    *stat = AENET_ERR_CUDA;
    return;
  }
  char* b = (char*)mem;
  char* p_vec = b;
  char* p_jt = p_vec + 32 * (size_t)cap;
  char* p_small = p_jt + 4 * (size_t)cap;  // cnt, type, struct
  char* p_G = p_small + 256;
  int small[3] = {nat, 0, 0};
  cudaMemcpy(p_vec, vec.data(), 32 * (size_t)cap, cudaMemcpyHostToDevice);
  cudaMemcpy(p_jt, jt.data(), 4 * (size_t)cap, cudaMemcpyHostToDevice);
  cudaMemcpy(p_small, small, 12, cudaMemcpyHostToDevice);
  DescBuffers d{};
  d.natoms = 1;
  d.nb_cnt = (const int*)p_small;
  d.types = (const int*)(p_small + 4);
  d.atom_struct = (const int*)(p_small + 8);
  d.nb_jt = (const int*)p_jt;
  d.nb_vec = p_vec;
  d.cap = cap;
  d.cap_a = cap;
  d.lpa = 32;
  d.G = p_G;
  int e = ae_launch_chebyshev_forward(pd, d, 1, 0);
  std::vector<double> out(nsf_pad);
  if (!e) e = (int)cudaMemcpy(out.data(), p_G, 8 * nsf_pad, cudaMemcpyDeviceToHost);
  cudaFree(mem);
  if (e) {
    *stat = AENET_ERR_CUDA;
    return;
  }
  for (int k = 0; k < nv; ++k) values[k] = out[k];
  *stat = AENET_OK;
}

// sfb_reconstruct_radial (sfbasis.f90:581-637): a host-side utility of
// the descriptor basis, not part of the energy/force path.
EXPORT void aenet_sfb_reconstruct_radial(int nv, double values[], int nx, double x[], double y[],
                                         int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.sfb_init) {
    *stat = AENET_ERR_INIT;
    return;
  }
  const double PI = 3.14159265358979;
  const int rN = g.sfb_rorder + 1;
  if (nv < rN || nx < 2) {
    *stat = AENET_ERR_INPUT;
    return;
  }
  const double Rc = g.sfb_rRc;
  double dx = Rc / (double)(nx - 1);
  for (int ix = 0; ix < nx; ++ix) x[ix] = (double)ix * dx;
  std::vector<double> f(rN);
  for (int ix = 0; ix < nx - 1; ++ix) {
    double xx = (2.0 * x[ix] - 0.0 - Rc) / (Rc - 0.0);
    f[0] = 1.0;
    if (rN > 1) f[1] = xx;
    for (int i = 2; i < rN; ++i) f[i] = 2.0 * xx * f[i - 1] - f[i - 2];
    double r = x[ix] / Rc;
    double w = 0.5 / std::sqrt(r - r * r);
    for (int i = 0; i < rN; ++i) f[i] = f[i] * w * (1.0 / PI);
    f[0] = 0.5 * f[0];
    y[ix] = 0.0;
    for (int ic = rN - 1; ic >= 0; --ic) y[ix] = y[ix] + values[ic] * f[ic];
  }
  y[nx - 1] = 0.0;
  *stat = AENET_OK;
}

// ---- neighbour list API (aenet.f90:571-639) --------------------------

EXPORT void aenet_nbl_init(double latt_vec[9], int natoms, int atom_types[], double coords[],
                           bool cartesian, bool pbc) {
  std::lock_guard<std::mutex> lk(g_mu);
  g.nbl_init = false;
  if (natoms < 1 || !g.loaded || !cuda_ok()) return;
  int nat = natoms;
  int pbcv = pbc ? 1 : 0;
  // latt_vec is Fortran latticeVec(3,3): columns are vectors == rows here
  aenet_gpu_plan* P = nullptr;
  {
    auto Pn = std::make_unique<aenet_gpu_plan>();
    Pn->nstruc = 1;
    Pn->fp64 = 1;
    Pn->natoms_h = {nat};
    Pn->pbc_h = {pbcv};
    Pn->geom_h.resize(1);
    Pn->pd = nullptr;
    Pn->rc = aenet_Rc_max;
    Pn->cell_div = g.cell_div;
    Pn->z_refine = g.z_refine;
    Pn->keep_images = true;
    // isolated structures are binned on the Cartesian input
    int st = make_geom(Pn->geom_h[0], latt_vec, pbcv, coords, nat, aenet_Rc_max, g.cell_div,
                       cartesian ? 1 : 2, nullptr, g.z_refine);
    if (st) return;
    // plan_alloc recomputes the geometry with frac_mode 0; redo with the
    // nbl convention afterwards
    StructGeom keep = Pn->geom_h[0];
    if (plan_alloc(Pn.get(), coords, latt_vec)) return;
    keep.cell_off = 0;
    keep.atom_off = 0;
    Pn->geom_h[0] = keep;
    if (cudaMemcpy(Pn->geom_d, &keep, sizeof(StructGeom), cudaMemcpyHostToDevice) != cudaSuccess)
      return;
    P = Pn.release();
  }
  std::unique_ptr<aenet_gpu_plan> hold(P);
  // coordinates and types on the device; every failure leaves the list
  // uninitialised (aenet_nbl_neighbors then returns no neighbours)
  struct DevFree {
    void* p = nullptr;
    ~DevFree() {
      if (p) cudaFree(p);
    }
  } io;
  if (cudaMalloc(&io.p, 28 * (size_t)nat) != cudaSuccess) {
    io.p = nullptr;
    return;
  }
  double* d_c = (double*)io.p;
  int* d_t = (int*)(d_c + 3 * (size_t)nat);
  if (cudaMemcpy(d_c, coords, 24 * (size_t)nat, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_t, atom_types, 4 * (size_t)nat, cudaMemcpyHostToDevice) != cudaSuccess)
    return;
  int ntmax = g.ntypes;
  if (ae_launch_types(nat, d_t, P->types0, ntmax, P->status, 0)) return;
  NbBuffers nb = nb_buffers(P);
  if (ae_launch_neighbors(nat, d_c, P->types0, nb, 1, 0)) return;
  g.nbl_cnt.resize(nat);
  g.nbl_jt.resize((size_t)nat * P->cap);
  g.nbl_img.resize((size_t)nat * P->cap);
  g.nbl_vec.resize((size_t)nat * P->cap * 4);
  g.nbl_s.resize(3 * (size_t)nat);
  g.nbl_cart.resize(3 * (size_t)nat);
  unsigned status = 0;
  if (cudaMemcpy(g.nbl_cnt.data(), P->nb_cnt, 4 * (size_t)nat, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(g.nbl_jt.data(), P->nb_jt, 4 * (size_t)nat * P->cap, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(g.nbl_img.data(), P->nb_img, 4 * (size_t)nat * P->cap, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(g.nbl_vec.data(), P->nb_vec, 32 * (size_t)nat * P->cap, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(g.nbl_s.data(), P->s_wrap, 24 * (size_t)nat, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(g.nbl_cart.data(), P->r_wrap, 24 * (size_t)nat, cudaMemcpyDeviceToHost) ||
      cudaMemcpy(&status, P->status, 4, cudaMemcpyDeviceToHost))
    return;
  if (cudaDeviceSynchronize() != cudaSuccess || status) return;
  g.nbl_natoms = nat;
  g.nbl_types.assign(atom_types, atom_types + nat);
  memcpy(g.nbl_L, latt_vec, sizeof(g.nbl_L));
  g.nbl_pbc = pbcv;
  // coords = matmul(latt_vec, coo_latt) (aenet.f90:605)
  for (size_t q = 0; q < 3 * (size_t)nat; ++q) coords[q] = g.nbl_cart[q];
  g.nbl_cap = P->cap;
  g.nbl_init = true;
}

EXPORT void aenet_nbl_final(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g.nbl_init = false;
  g.nbl_cnt.clear();
  g.nbl_jt.clear();
  g.nbl_img.clear();
  g.nbl_vec.clear();
}

EXPORT void aenet_nbl_neighbors(int iatom, int* nnb, double nbcoo[], double nbdist[], int nblist[],
                                int nbtype[]) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.nbl_init || iatom < 1 || iatom > g.nbl_natoms) {
    *nnb = 0;
    return;
  }
  const int cap = g.nbl_cap;
  const int i = iatom - 1;
  const int n = g.nbl_cnt[i];
  const int lim = std::min(n, *nnb);
  for (int k = 0; k < lim; ++k) {
    size_t q = (size_t)i * cap + k;
    int j = g.nbl_jt[q] & AE_INDEX_MASK;
    int img = g.nbl_img[q];
    int T[3];
    for (int c = 0; c < 3; ++c) {
      int v = (img >> (10 * c)) & 1023;
      T[c] = v >= 512 ? v - 1024 : v;
    }
    // nbcoo = latticeVec (s_j + T) (lclist.f90:606-611, 646-650)
    for (int c = 0; c < 3; ++c) {
      if (g.nbl_pbc) {
        double u0 = g.nbl_s[3 * j] + (double)T[0], u1 = g.nbl_s[3 * j + 1] + (double)T[1],
               u2 = g.nbl_s[3 * j + 2] + (double)T[2];
        double t = g.nbl_L[c] * u0;
        t = t + g.nbl_L[3 + c] * u1;
        t = t + g.nbl_L[6 + c] * u2;
        nbcoo[3 * k + c] = t;
      } else {
        nbcoo[3 * k + c] = g.nbl_cart[3 * j + c];
      }
    }
    nbdist[k] = g.nbl_vec[4 * q + 3];
    nblist[k] = j + 1;
    nbtype[k] = g.nbl_types[j];
  }
  *nnb = lim;
}

// =====================================================================
//                 batched extensions (include/aenet_gb300.h)
// =====================================================================

EXPORT int aenet_gpu_set_option(const char* key, const char* value) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!key || !value) return AENET_ERR_INPUT;
  ++g.gen;
  std::string k = key, v = value;
  if (k == "angular_domain") {
    if (v == "legacy") g.angular_legacy = 1;
    else if (v == "current") g.angular_legacy = 0;
    else return AENET_ERR_INPUT;
    g.dev_ready = false;
    return AENET_OK;
  }
  if (k == "adjoint_lanes_per_atom") {
    int d = atoi(v.c_str());
    if (d != 0 && d != 8 && d != 16 && d != 32) return AENET_ERR_INPUT;
    g.lpa_adjoint = d;
    return AENET_OK;
  }
  if (k == "lanes_per_atom") {
    int d = atoi(v.c_str());
    if (d != 8 && d != 16 && d != 32) return AENET_ERR_INPUT;
    g.lpa_default = d;
    return AENET_OK;
  }
  if (k == "z_refine") {
    int d = atoi(v.c_str());
    if (d < 1 || d > 4) return AENET_ERR_INPUT;
    g.z_refine = d;
    return AENET_OK;
  }
  if (k == "cell_div") {
    int d = atoi(v.c_str());
    if (d < 1 || d > 3) return AENET_ERR_INPUT;
    g.cell_div = d;
    return AENET_OK;
  }
  if (k == "neighbour_kernel") {
    if (v == "cell") g.nb_cell = 1;
    else if (v == "stream") g.nb_cell = 2;
    else if (v == "half") g.nb_cell = 3;
    else if (v == "struct") g.nb_cell = 4;
    else if (v == "struct_half") g.nb_cell = 5;
    else if (v == "atom") g.nb_cell = 0;
    else return AENET_ERR_INPUT;
    return AENET_OK;
  }
  if (k == "angular_terms") {
    if (v == "moments") g.angular_moments = 1;
    else if (v == "pairs") g.angular_moments = 0;
    else return AENET_ERR_INPUT;
    return AENET_OK;
  }
  if (k == "per_atom_kernel") {
    if (v == "fused") g.atom_fused = 2;
    else if (v == "cluster") g.atom_fused = 3;
    else if (v == "block") g.atom_fused = 1;
    else if (v == "graph") g.atom_fused = 0;
    else return AENET_ERR_INPUT;
    return AENET_OK;
  }
  if (k == "angular_spin") {
    if (v == "stale") g.angular_spin_stale = 1;
    else if (v == "own") g.angular_spin_stale = 0;
    else return AENET_ERR_INPUT;
    return AENET_OK;
  }
  if (k == "networks") {
    if (v == "tensor") g.networks_tc = 1;
    else if (v == "simt") g.networks_tc = 0;
    else return AENET_ERR_INPUT;
    return AENET_OK;
  }
  return AENET_ERR_INPUT;
}

EXPORT aenet_gpu_plan* aenet_gpu_plan_create(int nstruc, const int* natoms, const double* lattices,
                                             const int* pbc, const double* coords0, int precision,
                                             int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (nstruc < 1 || !natoms) {
    *stat = AENET_ERR_INPUT;
    return nullptr;
  }
  int st = ensure_device();
  if (st) {
    *stat = st;
    return nullptr;
  }
  return plan_new(nstruc, natoms, lattices, pbc, coords0, precision, &g.pd, aenet_Rc_max, 0, false,
                  stat);
}

EXPORT void aenet_gpu_plan_destroy(aenet_gpu_plan* plan) {
  std::lock_guard<std::mutex> lk(g_mu);
  delete plan;
}

EXPORT int aenet_gpu_plan_natoms(const aenet_gpu_plan* plan) { return plan ? plan->natoms : 0; }

EXPORT int aenet_gpu_plan_set_lattices(aenet_gpu_plan* P, const double* lattices) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!P || !lattices) return AENET_ERR_INPUT;
  for (int s = 0; s < P->nstruc; ++s) {
    StructGeom G;
    if (!P->pbc_h[s]) continue;
    StructGeom& O = P->geom_h[s];
    // the cell grid keeps its dimensions (the slot layout depends on them);
    // the stencil half widths follow the new heights
    int st = make_geom(G, lattices + 9 * (size_t)s, 1, nullptr, P->natoms_h[s], P->rc, P->cell_div,
                       O.frac_mode, O.nc, P->z_refine);
    if (st) return st;
    G.cell_off = O.cell_off;
    G.atom_off = O.atom_off;
    G.chunk_off = O.chunk_off;
    O = G;
  }
  if (cudaMemcpy(P->geom_d, P->geom_h.data(), sizeof(StructGeom) * P->nstruc, cudaMemcpyHostToDevice))
    return AENET_ERR_CUDA;
  return 0;
}

EXPORT int aenet_gpu_plan_run(aenet_gpu_plan* P, const double* d_coords, const int* d_types,
                              double* d_E, double* d_E_atoms, double* d_F, double* d_virial,
                              unsigned flags, void* stream) {
  if (!P) return AENET_ERR_INPUT;
  cudaStream_t s = (cudaStream_t)stream;
  int st = plan_forward(P, d_coords, d_types, d_E, d_E_atoms, s);
  if (st) return st;
  if ((flags & (AENET_GPU_FORCES | AENET_GPU_VIRIAL)) || d_F || d_virial)
    return plan_adjoint(P, nullptr, d_F, 1.0, (flags & AENET_GPU_VIRIAL) ? d_virial : nullptr, s);
  return 0;
}

EXPORT int aenet_gpu_plan_forward(aenet_gpu_plan* P, const double* d_coords, const int* d_types,
                                  double* d_E, double* d_E_atoms, void* stream) {
  if (!P) return AENET_ERR_INPUT;
  return plan_forward(P, d_coords, d_types, d_E, d_E_atoms, (cudaStream_t)stream);
}

EXPORT int aenet_gpu_plan_backward(aenet_gpu_plan* P, const double* d_weights, double* d_grad,
                                   double* d_virial, void* stream) {
  if (!P) return AENET_ERR_INPUT;
  // the adjoint accumulates forces -dE/dR; the output is their negative
  return plan_adjoint(P, d_weights, d_grad, -1.0, d_virial, (cudaStream_t)stream);
}

namespace {
int plan_train_alloc(aenet_gpu_plan* P) {
  if (P->tmem) return 0;
  const PotDevice& pd = *P->pd;
  const size_t N = (size_t)P->natoms, tsz = P->fp64 ? 8 : 4;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = (off + bytes + 255) & ~(size_t)255;
    return o;
  };
  size_t o_ce = take(8 * (size_t)P->nstruc);
  size_t o_ls = take(8 * (size_t)P->nstruc);
  size_t o_u = take(4 * tsz * N);
  size_t o_p = take(8 * (size_t)pd.ntypes * ae_wgrad_nblk(pd.ntypes) * ae_wgrad_wcap(pd));
  if (cudaMalloc(&P->tmem, off) != cudaSuccess) {
    P->tmem = nullptr;
    return AENET_ERR_CUDA;
  }
  char* b = (char*)P->tmem;
  P->cE = (double*)(b + o_ce);
  P->loss_s = (double*)(b + o_ls);
  P->U = (void*)(b + o_u);
  P->partial = (double*)(b + o_p);
  if (cudaMemset(P->tmem, 0, off) != cudaSuccess) return AENET_ERR_CUDA;
  return 0;
}
}  // namespace

// Loss and gradient with respect to every network weight (training).
EXPORT int aenet_gpu_plan_loss_gradient(aenet_gpu_plan* P, const double* d_coords,
                                        const int* d_types, const double* d_E_target,
                                        const double* d_F_target, int mode, double w_E,
                                        double w_F, double* d_loss, double* d_grad, double* d_E,
                                        double* d_F, void* stream) {
  if (!P || !d_coords || !d_types || !d_E_target || !d_loss || !d_grad) return AENET_ERR_INPUT;
  if (mode != AENET_GPU_LOSS_ENERGY && mode != AENET_GPU_LOSS_ENERGY_FORCES) return AENET_ERR_INPUT;
  const PotDevice& pd = *P->pd;
  const bool force_term = mode == AENET_GPU_LOSS_ENERGY_FORCES && w_F != 0.0;
  if (force_term && !d_F_target) return AENET_ERR_INPUT;
  // the force term needs the descriptor tangent, written for Chebyshev bases
  if (force_term && pd.sp[0].sftype != AE_SF_CHEBYSHEV) return AENET_ERR_INPUT;
  // ... with each neighbour's own spin (angular_spin = own)
  if (force_term && P->nb_rank) return AENET_ERR_INPUT;
  if (mode == AENET_GPU_LOSS_ENERGY)
    for (int t = 1; t < pd.ntypes; ++t)
      if (std::fabs(pd.sp[t].E_scale - pd.sp[0].E_scale) > 1e-12 * std::fabs(pd.sp[0].E_scale))
        return AENET_ERR_INPUT;   // one normalisation for the whole training set
  int st = plan_train_alloc(P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  st = plan_forward(P, d_coords, d_types, d_E, nullptr, s);
  if (st) return st;
  if (force_term || d_F) {
    st = plan_adjoint(P, nullptr, d_F, 1.0, nullptr, s);
    if (st) return st;
  }
  if (ck(ae_launch_loss(P->nstruc, P->geom_d, P->E_struct, d_E_target, P->Facc,
                        force_term ? d_F_target : nullptr, mode == AENET_GPU_LOSS_ENERGY ? 0 : 1, w_E, w_F, pd.sp[0].E_scale, P->cE,
                        P->U, P->loss_s, d_loss, P->fp64, s)))
    return AENET_ERR_CUDA;
  if (force_term) {
    DescBuffers d = desc_buffers(P, nullptr, false);
    d.U = P->U;
    d.V = P->dEdG;   // dE/dG is not needed any more in this pass
    if (ck(ae_launch_chebyshev_tangent(pd, d, P->fp64, s))) return AENET_ERR_CUDA;
  }
  if (ck(ae_launch_partition(P->natoms, pd.ntypes, P->types0, P->part_scratch, P->order,
                             P->spec_off, s)))
    return AENET_ERR_CUDA;
  if (ck(ae_launch_mlp_wgrad(pd, P->order, P->spec_off, P->G, force_term ? P->dEdG : nullptr,
                             P->atom_struct, P->cE, force_term ? -1.0 : 0.0,
                             mode == AENET_GPU_LOSS_ENERGY_FORCES, P->partial, d_grad, P->fp64, s)))
    return AENET_ERR_CUDA;
  return 0;
}

// ---- molecular dynamics ---------------------------------------------

// amu A^2 / fs^2 in eV: 1.66053906660e-27 kg * 1e10 m^2/s^2 / 1.602176634e-19 J
static const double MD_MASS_UNIT = 1.66053906660e-17 / 1.602176634e-19;

struct aenet_gpu_md {
  std::unique_ptr<aenet_gpu_plan> P;
  std::unique_ptr<aenet_gpu_plan> P64;   // FP64 re-evaluation, created on first use
  int n = 0, precision = AENET_GPU_MIXED, cap = 0;
  double dt = 1.0, skin = 0.0;
  double lattice[9];
  cudaStream_t stream = nullptr;
  void* mem = nullptr;
  double *pos = nullptr, *vel = nullptr, *F = nullptr, *S = nullptr, *rb = nullptr,
         *invm = nullptr, *part = nullptr, *scal = nullptr;   // scal: E, E_kin, E_fp64
  float4* p32 = nullptr;      // positions in the frame of the last build (mixed path)
  int *types = nullptr, *flag = nullptr;
  long long steps = 0;
  int builds = 0;
  // device time of the force part of each step (table build or refresh,
  // descriptors, networks, adjoint), by kind of step; events of the last
  // step are read at the next synchronisation
  double ms_build = 0.0, ms_refresh = 0.0;
  long long n_build = 0, n_refresh = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int pending = -1;           // -1 none, 0 refresh step, 1 build step
  ~aenet_gpu_md() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (mem) cudaFree(mem);
    if (stream) cudaStreamDestroy(stream);
  }
  void collect() {
    if (pending < 0) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess) {
      if (pending) {
        ms_build += ms;
        ++n_build;
      } else {
        ms_refresh += ms;
        ++n_refresh;
      }
    }
    pending = -1;
  }
};

namespace {
int md_plan(aenet_gpu_md* M, int cap) {
  int st = 0;
  const int pbc = 1;
  M->P.reset(plan_new(1, &M->n, M->lattice, &pbc, nullptr, M->precision, &g.pd,
                      aenet_Rc_max + M->skin, cap, true, &st));
  if (!M->P) return st ? st : AENET_ERR_CUDA;
  M->cap = M->P->cap;
  return 0;
}

// full neighbour search at the current positions, then energies and forces
int md_build(aenet_gpu_md* M) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    aenet_gpu_plan* P = M->P.get();
    cudaStream_t s = M->stream;
    if (cudaMemsetAsync(P->status, 0, 4, s)) return AENET_ERR_CUDA;
    int st = plan_forward(P, M->pos, M->types, nullptr, nullptr, s);
    if (st) return st;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, P->status, 4, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
      return AENET_ERR_CUDA;
    if (h & (AE_ST_BAD_COORD | AE_ST_BAD_TYPE | AE_ST_CELL_OVERFLOW)) return AENET_ERR_INPUT;
    if (h & AE_ST_TC_TIMEOUT) return AENET_ERR_CUDA;
    if (h & AE_ST_NB_OVERFLOW) {
      st = md_plan(M, ((M->cap * 3 / 2) + 31) & ~31);
      if (st) return st;
      continue;
    }
    ++M->builds;
    if (ck(ae_md_after_build(M->n, M->pos, P->r_wrap, M->S, M->rb, s))) return AENET_ERR_CUDA;
    return plan_adjoint(P, nullptr, M->F, 1.0, nullptr, s);
  }
  return AENET_ERR_MALLOC;
}
}  // namespace

// Velocity-Verlet MD of one periodic structure (see include/aenet_gb300.h).
EXPORT aenet_gpu_md* aenet_gpu_md_create(int natoms, const double* lattice, const double* coords,
                                         const double* velocities, const int* type_ids,
                                         const double* masses, double dt, double skin,
                                         int precision, int* stat) {
  int dummy;
  if (!stat) stat = &dummy;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init || !g.loaded) {
    *stat = AENET_ERR_INIT;
    return nullptr;
  }
  if (natoms < 1 || !lattice || !coords || !type_ids || !masses || !(dt > 0.0) || !(skin >= 0.0) ||
      (precision != AENET_GPU_FP64 && precision != AENET_GPU_MIXED)) {
    *stat = AENET_ERR_INPUT;
    return nullptr;
  }
  for (int t = 0; t < g.ntypes; ++t)
    if (!(masses[t] > 0.0)) {
      *stat = AENET_ERR_INPUT;
      return nullptr;
    }
  int st = ensure_device();
  if (st) {
    *stat = st;
    return nullptr;
  }
  auto M = std::make_unique<aenet_gpu_md>();
  M->n = natoms;
  M->dt = dt;
  M->skin = skin;
  M->precision = precision;
  memcpy(M->lattice, lattice, sizeof(M->lattice));
  if (cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking)) {
    *stat = AENET_ERR_CUDA;
    return nullptr;
  }
  const size_t N = natoms;
  const size_t bytes = 8 * (3 * N * 5 + N + ae_md_ekin_blocks() + 4) + 4 * (N + 4) + 16 * N + 256 * 11;
  if (cudaMalloc(&M->mem, bytes)) {
    M->mem = nullptr;
    *stat = AENET_ERR_CUDA;
    return nullptr;
  }
  char* b = (char*)M->mem;
  size_t off = 0;
  auto take = [&](size_t n) {
    char* p = b + off;
    off = (off + n + 255) & ~(size_t)255;
    return p;
  };
  M->pos = (double*)take(24 * N);
  M->vel = (double*)take(24 * N);
  M->F = (double*)take(24 * N);
  M->S = (double*)take(24 * N);
  M->rb = (double*)take(24 * N);
  M->invm = (double*)take(8 * N);
  M->part = (double*)take(8 * (size_t)ae_md_ekin_blocks());
  M->scal = (double*)take(32);
  M->types = (int*)take(4 * N);
  M->flag = (int*)take(16);
  M->p32 = (float4*)take(16 * N);
  std::vector<double> invm(N), v0(3 * N, 0.0);
  for (size_t i = 0; i < N; ++i) {
    const int t = type_ids[i];
    if (t < 1 || t > g.ntypes) {
      *stat = AENET_ERR_TYPE;
      return nullptr;
    }
    invm[i] = 1.0 / masses[t - 1];
  }
  if (velocities) std::copy(velocities, velocities + 3 * N, v0.begin());
  if (cudaMemcpy(M->pos, coords, 24 * N, cudaMemcpyHostToDevice) ||
      cudaMemcpy(M->vel, v0.data(), 24 * N, cudaMemcpyHostToDevice) ||
      cudaMemcpy(M->invm, invm.data(), 8 * N, cudaMemcpyHostToDevice) ||
      cudaMemcpy(M->types, type_ids, 4 * N, cudaMemcpyHostToDevice)) {
    *stat = AENET_ERR_CUDA;
    return nullptr;
  }
  st = md_plan(M.get(), 0);
  if (!st) st = md_build(M.get());
  if (!st && cudaStreamSynchronize(M->stream)) st = AENET_ERR_CUDA;
  if (st) {
    *stat = st;
    return nullptr;
  }
  *stat = AENET_OK;
  return M.release();
}

EXPORT void aenet_gpu_md_destroy(aenet_gpu_md* M) { delete M; }

EXPORT int aenet_gpu_md_run(aenet_gpu_md* M, int nsteps, double* E_pot, double* E_kin) {
  if (!M || nsteps < 0) return AENET_ERR_INPUT;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s = M->stream;
  aenet_gpu_plan* P = M->P.get();
  const double half_dt_acc = 0.5 * M->dt / MD_MASS_UNIT;
  const double lim2 = 0.25 * M->skin * M->skin;
  for (int k = 0; k < nsteps; ++k) {
    if (ck(ae_md_kick_drift(M->n, M->pos, M->vel, M->F, M->invm, half_dt_acc, M->dt, s)))
      return AENET_ERR_CUDA;
    bool rebuild = M->skin <= 0.0;
    if (!rebuild) {
      int h = 0;
      if (ck(ae_md_displacement(M->n, M->pos, M->rb, lim2, M->flag, s)) ||
          cudaMemcpyAsync(&h, M->flag, 4, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
        return AENET_ERR_CUDA;
      rebuild = h != 0;
    }
    M->collect();   // the previous step's events are complete after the sync
    if (!M->ev0 && (cudaEventCreate(&M->ev0) || cudaEventCreate(&M->ev1))) return AENET_ERR_CUDA;
    if (cudaEventRecord(M->ev0, s)) return AENET_ERR_CUDA;
    int st;
    if (rebuild) {
      st = md_build(M);
      P = M->P.get();
    } else {
      const int e = P->fp64 ? ae_md_refresh(M->n, P->geom_d, P->atom_struct, M->pos, M->S, P->cap,
                                            P->nb_cnt, P->nb_jt, P->nb_img, P->nb_vec, 1, s)
                            : ae_md_refresh_f32(M->n, P->geom_d, P->atom_struct, M->pos, M->S,
                                                M->p32, P->cap, P->nb_cnt, P->nb_jt, P->nb_img,
                                                P->nb_vec, s);
      if (ck(e)) return AENET_ERR_CUDA;
      st = plan_eval(P, nullptr, nullptr, s);
      if (!st) st = plan_adjoint(P, nullptr, M->F, 1.0, nullptr, s);
    }
    if (st) return st;
    if (cudaEventRecord(M->ev1, s)) return AENET_ERR_CUDA;
    M->pending = rebuild ? 1 : 0;
    if (ck(ae_md_kick(M->n, M->vel, M->F, M->invm, half_dt_acc, s))) return AENET_ERR_CUDA;
    ++M->steps;
  }
  if (ck(ae_md_ekin(M->n, M->vel, M->invm, M->part, 0.5 * MD_MASS_UNIT, M->scal + 1, s)) ||
      cudaMemcpyAsync(M->scal, P->E_struct, 8, cudaMemcpyDeviceToDevice, s))
    return AENET_ERR_CUDA;
  double h[2];
  if (cudaMemcpyAsync(h, M->scal, 16, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
    return AENET_ERR_CUDA;
  M->collect();
  if (E_pot) *E_pot = h[0];
  if (E_kin) *E_kin = h[1];
  return AENET_OK;
}

EXPORT int aenet_gpu_md_get(aenet_gpu_md* M, double* coords, double* velocities, double* forces) {
  if (!M) return AENET_ERR_INPUT;
  const size_t b = 24 * (size_t)M->n;
  cudaStream_t s = M->stream;
  if ((coords && cudaMemcpyAsync(coords, M->pos, b, cudaMemcpyDeviceToHost, s)) ||
      (velocities && cudaMemcpyAsync(velocities, M->vel, b, cudaMemcpyDeviceToHost, s)) ||
      (forces && cudaMemcpyAsync(forces, M->F, b, cudaMemcpyDeviceToHost, s)) ||
      cudaStreamSynchronize(s))
    return AENET_ERR_CUDA;
  return AENET_OK;
}

EXPORT int aenet_gpu_md_phase_times(aenet_gpu_md* M, double* build_ms, long long* build_steps,
                                    double* refresh_ms, long long* refresh_steps) {
  if (!M) return AENET_ERR_INPUT;
  if (build_ms) *build_ms = M->ms_build;
  if (build_steps) *build_steps = M->n_build;
  if (refresh_ms) *refresh_ms = M->ms_refresh;
  if (refresh_steps) *refresh_steps = M->n_refresh;
  return AENET_OK;
}

EXPORT int aenet_gpu_md_counters(aenet_gpu_md* M, long long* steps, int* builds) {
  if (!M) return AENET_ERR_INPUT;
  if (steps) *steps = M->steps;
  if (builds) *builds = M->builds;
  return AENET_OK;
}

// FP64 energy of the current positions (its own plan without skin)
EXPORT int aenet_gpu_md_energy_fp64(aenet_gpu_md* M, double* E) {
  if (!M || !E) return AENET_ERR_INPUT;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s = M->stream;
  if (!M->P64) {
    int st = 0;
    const int pbc = 1;
    M->P64.reset(plan_new(1, &M->n, M->lattice, &pbc, nullptr, AENET_GPU_FP64, &g.pd, aenet_Rc_max,
                          0, false, &st));
    if (!M->P64) return st ? st : AENET_ERR_CUDA;
  }
  int st = plan_forward(M->P64.get(), M->pos, M->types, M->scal + 2, nullptr, s);
  if (st) return st;
  if (cudaMemcpyAsync(E, M->scal + 2, 8, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
    return AENET_ERR_CUDA;
  return AENET_OK;
}

// ---- caller's neighbour lists (MD engines) ---------------------------

namespace {
struct NlistCtx {
  std::unique_ptr<aenet_gpu_plan> P;
  int nlocal = -1, nall = -1, cap = 0, cap_a = 0, precision = -1;
  size_t nnz_cap = 0;
  void* io = nullptr;
  size_t io_bytes = 0;
  double* x = nullptr;
  int* types = nullptr;
  int* offs = nullptr;
  int* nbr = nullptr;
  void* Facc = nullptr;
  double* F = nullptr;
  double* E = nullptr;
  double* Ea = nullptr;
  double* V = nullptr;
  cudaStream_t stream = nullptr;
  ~NlistCtx() {
    if (io) cudaFree(io);
    if (stream) cudaStreamDestroy(stream);
  }
};
std::unique_ptr<NlistCtx> g_nlist;
void nlist_release() { g_nlist.reset(); }

int nlist_setup(NlistCtx& c, int nlocal, int nall, const double* x, size_t nnz, int cap, int cap_a,
                int precision) {
  if (!c.stream && cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking)) return AENET_ERR_CUDA;
  if (!c.P || c.nlocal != nlocal || c.precision != precision || cap > c.cap || cap_a != c.cap_a ||
      (c.P->nb_rank != nullptr) != stale_spin_wanted()) {
    int st = 0;
    const int pbc = 0;
    c.P.reset(plan_new(1, &nlocal, nullptr, &pbc, x, precision, &g.pd, aenet_Rc_max, cap, false, &st));
    if (!c.P) return st ? st : AENET_ERR_CUDA;
    c.P->cap_a = std::min(cap_a, c.P->cap);
    c.P->stale_caller_order = 1;   // the rows keep the engine's list order
    c.nlocal = nlocal;
    c.precision = precision;
    c.cap = c.P->cap;
    c.cap_a = cap_a;
    c.nall = -1;
  }
  const size_t tsz = precision == AENET_GPU_FP64 ? 8 : 4;
  if (c.nall != nall || nnz > c.nnz_cap) {
    if (c.io) cudaFree(c.io);
    c.io = nullptr;
    size_t off = 0;
    auto take = [&](size_t b) {
      size_t o = off;
      off = (off + b + 255) & ~(size_t)255;
      return o;
    };
    const size_t NA = nall, NL = nlocal;
    size_t o_x = take(24 * NA), o_t = take(4 * NA), o_o = take(4 * (NL + 1)), o_n = take(4 * nnz + 4);
    size_t o_fa = take(4 * tsz * NA), o_f = take(24 * NA), o_e = take(8), o_ea = take(8 * NL + 8),
           o_v = take(72);
    if (cudaMalloc(&c.io, off)) {
      c.io = nullptr;
      return AENET_ERR_CUDA;
    }
    char* b = (char*)c.io;
    c.x = (double*)(b + o_x);
    c.types = (int*)(b + o_t);
    c.offs = (int*)(b + o_o);
    c.nbr = (int*)(b + o_n);
    c.Facc = (void*)(b + o_fa);
    c.F = (double*)(b + o_f);
    c.E = (double*)(b + o_e);
    c.Ea = (double*)(b + o_ea);
    c.V = (double*)(b + o_v);
    c.nall = nall;
    c.nnz_cap = nnz;
  }
  return 0;
}
}  // namespace

// Energy and forces from the caller's neighbour list (see aenet_gb300.h).
EXPORT int aenet_gpu_neighbor_list_energy_forces(int nlocal, int nall, const double* x,
                                                 const int* type_ids, const int* neigh_offset,
                                                 const int* neighbors, int precision,
                                                 double* E_total, double* E_atoms, double* F,
                                                 double* virial) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init || !g.loaded) return AENET_ERR_INIT;
  if (nlocal < 1 || nall < nlocal || !x || !type_ids || !neigh_offset ||
      (precision != AENET_GPU_FP64 && precision != AENET_GPU_MIXED))
    return AENET_ERR_INPUT;
  int st = ensure_device();
  if (st) return st;
  const size_t nnz = (size_t)neigh_offset[nlocal];
  if (neigh_offset[0] != 0 || (nnz && !neighbors)) return AENET_ERR_INPUT;
  int cap = 0;
  for (int i = 0; i < nlocal; ++i) {
    const int n = neigh_offset[i + 1] - neigh_offset[i];
    if (n < 0) return AENET_ERR_INPUT;
    cap = std::max(cap, n);
  }
  cap = ((cap + 31) & ~31) + 32;
  // staged angular neighbours: the share of the cut-off sphere inside the
  // largest angular cut-off, with room to spare; all of them on a retry
  double arc = 0.0;
  for (int t = 0; t < g.pd.ntypes; ++t)
    arc = std::max(arc, g.pd.sp[t].sftype == AE_SF_CHEBYSHEV ? g.pd.sp[t].cheb.a_Rc : aenet_Rc_max);
  const double frac = std::pow(std::min(1.0, (arc + 1e-3) / (aenet_Rc_max + 1e-3)), 3);
  int cap_a = std::min(cap, (((int)std::ceil(1.5 * frac * cap) + 16) + 7) & ~7);
  if (!g_nlist) g_nlist = std::make_unique<NlistCtx>();
  NlistCtx& c = *g_nlist;
  for (int attempt = 0; attempt < 2; ++attempt) {
    st = nlist_setup(c, nlocal, nall, x, nnz, cap, cap_a, precision);
    if (st) {
      g_nlist.reset();
      return st;
    }
    aenet_gpu_plan* P = c.P.get();
    cudaStream_t s = c.stream;
    const size_t tsz = P->fp64 ? 8 : 4;
    const double rcp = aenet_Rc_max + 1.0e-3;
    if (cudaMemcpyAsync(c.x, x, 24 * (size_t)nall, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(c.types, type_ids, 4 * (size_t)nall, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(c.offs, neigh_offset, 4 * ((size_t)nlocal + 1), cudaMemcpyHostToDevice, s) ||
        (nnz && cudaMemcpyAsync(c.nbr, neighbors, 4 * nnz, cudaMemcpyHostToDevice, s)) ||
        cudaMemsetAsync(P->status, 0, 4, s))
      return AENET_ERR_CUDA;
    const PotDevice& pd = *P->pd;
    if (ck(ae_launch_types(nlocal, c.types, P->types0, pd.ntypes, P->status, s)) ||
        ck(ae_launch_ell_from_csr(nlocal, nall, c.x, c.types, pd.ntypes, c.offs, c.nbr, rcp * rcp,
                                  P->cap, P->nb_cnt, P->nb_jt, P->nb_vec, P->fp64, P->status, s)))
      return AENET_ERR_CUDA;
    st = plan_eval(P, c.E, c.Ea, s);
    if (st) return st;
    if (cudaMemsetAsync(c.Facc, 0, 4 * tsz * (size_t)nall, s) ||
        cudaMemsetAsync(P->virial, 0, 72, s))
      return AENET_ERR_CUDA;
    DescBuffers d = desc_buffers(P, nullptr, true);
    d.F = c.Facc;
    if (g.lpa_adjoint) d.lpa = g.lpa_adjoint;
    int e = (pd.sp[0].sftype == AE_SF_BEHLER) ? ae_launch_behler_adjoint(pd, d, P->fp64, s)
                                               : ae_launch_chebyshev_adjoint(pd, d, P->fp64, s);
    if (ck(e) || ck(ae_launch_forces_out(nall, c.Facc, P->fp64, c.F, 1.0, s))) return AENET_ERR_CUDA;
    unsigned status = 0;
    double Et = 0.0;
    if (cudaMemcpyAsync(&status, P->status, 4, cudaMemcpyDeviceToHost, s) ||
        cudaMemcpyAsync(&Et, c.E, 8, cudaMemcpyDeviceToHost, s) ||
        (E_atoms && cudaMemcpyAsync(E_atoms, c.Ea, 8 * (size_t)nlocal, cudaMemcpyDeviceToHost, s)) ||
        (F && cudaMemcpyAsync(F, c.F, 24 * (size_t)nall, cudaMemcpyDeviceToHost, s)) ||
        (virial && cudaMemcpyAsync(virial, P->virial, 72, cudaMemcpyDeviceToHost, s)) ||
        cudaStreamSynchronize(s))
      return AENET_ERR_CUDA;
    if (status & AE_ST_BAD_TYPE) return AENET_ERR_TYPE;
    if (status & AE_ST_TC_TIMEOUT) return AENET_ERR_CUDA;
    if (status & AE_ST_NB_OVERFLOW) {
      cap_a = cap;   // stage every neighbour
      continue;
    }
    if (E_total) *E_total = Et;
    return AENET_OK;
  }
  return AENET_ERR_MALLOC;
}

// ---- training from stored descriptors (training-set files) -----------

// Copy externally computed, normalised descriptors into the plan.
EXPORT int aenet_gpu_plan_load_descriptors(aenet_gpu_plan* P, const double* G, int ld) {
  if (!P || !G || !P->pd) return AENET_ERR_INPUT;
  const int nsf_pad = P->pd->nsf_pad, N = P->natoms;
  if (ld < P->pd->nsf_max || ld < 1) return AENET_ERR_INPUT;
  const int cols = std::min(ld, nsf_pad);
  if (P->fp64) {
    std::vector<double> h((size_t)N * nsf_pad, 0.0);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < cols; ++k) h[(size_t)i * nsf_pad + k] = G[(size_t)i * ld + k];
    if (cudaMemcpy(P->G, h.data(), 8 * h.size(), cudaMemcpyHostToDevice)) return AENET_ERR_CUDA;
  } else {
    std::vector<float> h((size_t)N * nsf_pad, 0.0f);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < cols; ++k) h[(size_t)i * nsf_pad + k] = (float)G[(size_t)i * ld + k];
    if (cudaMemcpy(P->G, h.data(), 4 * h.size(), cudaMemcpyHostToDevice)) return AENET_ERR_CUDA;
  }
  return AENET_OK;
}

// Descriptor Jacobians (raw, FP64) of atoms [atom0, atom0 + count) from the
// neighbour table of the plan's last run: generate.x's PyTorch export.
EXPORT int aenet_gpu_plan_neighbour_capacity(const aenet_gpu_plan* P) { return P ? P->cap : -1; }

EXPORT int aenet_gpu_plan_descriptor_jacobian(aenet_gpu_plan* P, int atom0, int count,
                                              double* d_dG_i, double* d_dG_j, int* d_nbl,
                                              int* d_nnb, void* stream) {
  if (!P || !P->pd || !P->fp64 || !d_dG_i || !d_dG_j || !d_nbl || !d_nnb) return AENET_ERR_INPUT;
  if (P->nb_rank) return AENET_ERR_INPUT;   // Jacobians with each neighbour's own spin only
  if (atom0 < 0 || count < 0 || atom0 + count > P->natoms) return AENET_ERR_INPUT;
  const PotDevice& pd = *P->pd;
  const int sft = pd.sp[0].sftype;
  for (int t = 1; t < pd.ntypes; ++t)
    if (pd.sp[t].sftype != sft) return AENET_ERR_INPUT;
  DescBuffers d = desc_buffers(P, nullptr, false);
  const int e = sft == AE_SF_BEHLER
                    ? ae_launch_behler_jacobian(pd, d, atom0, count, pd.nsf_max, d_dG_i, d_dG_j,
                                                d_nbl, d_nnb, (cudaStream_t)stream)
                    : ae_launch_chebyshev_jacobian(pd, d, atom0, count, pd.nsf_max, d_dG_i, d_dG_j,
                                                   d_nbl, d_nnb, (cudaStream_t)stream);
  if (ck(e)) return AENET_ERR_CUDA;
  return AENET_OK;
}

// The reference's energy loss and weight gradient from the loaded
// descriptors (no positions, no neighbour search): networks, per-structure
// energies, SSE = sum_s dE_s^2/2 and sum_s dE_s Dw_s.
EXPORT int aenet_gpu_plan_descriptor_loss_gradient(aenet_gpu_plan* P, const int* d_types,
                                                   const double* d_E_target, double* d_loss,
                                                   double* d_grad, double* d_E, void* stream) {
  if (!P || !d_types || !d_E_target || !d_loss || !d_grad) return AENET_ERR_INPUT;
  const PotDevice& pd = *P->pd;
  for (int t = 1; t < pd.ntypes; ++t)
    if (std::fabs(pd.sp[t].E_scale - pd.sp[0].E_scale) > 1e-12 * std::fabs(pd.sp[0].E_scale))
      return AENET_ERR_INPUT;
  int st = plan_train_alloc(P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (ck(ae_launch_types(P->natoms, d_types, P->types0, pd.ntypes, P->status, s))) return AENET_ERR_CUDA;
  DescBuffers d = desc_buffers(P, nullptr, false);
  if (plan_networks(P, d, s)) return AENET_ERR_CUDA;
  if (ck(ae_launch_energy_reduce_chunked(P->nstruc, P->nchunks, P->geom_d, P->chunk_struct,
                                         P->E_atom, P->e_part, P->E_struct, P->one_chunk_each, s)))
    return AENET_ERR_CUDA;
  if (d_E && cudaMemcpyAsync(d_E, P->E_struct, 8 * (size_t)P->nstruc, cudaMemcpyDeviceToDevice, s))
    return AENET_ERR_CUDA;
  if (ck(ae_launch_loss(P->nstruc, P->geom_d, P->E_struct, d_E_target, P->Facc, nullptr, 0, 1.0, 0.0,
                        pd.sp[0].E_scale, P->cE, P->U, P->loss_s, d_loss, P->fp64, s)) ||
      ck(ae_launch_partition(P->natoms, pd.ntypes, P->types0, P->part_scratch, P->order,
                             P->spec_off, s)) ||
      ck(ae_launch_mlp_wgrad(pd, P->order, P->spec_off, P->G, nullptr, P->atom_struct, P->cE, 0.0, 0,
                             P->partial, d_grad, P->fp64, s)))
    return AENET_ERR_CUDA;
  return AENET_OK;
}

// ---- network weights ------------------------------------------------

EXPORT int aenet_gpu_network_nweights(int type_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init || type_id < 1 || type_id > g.ntypes || !g.pots[type_id - 1].init) return -1;
  return g.pots[type_id - 1].net.Wsize;
}

EXPORT int aenet_gpu_get_weights(double* W) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init || !g.loaded) return AENET_ERR_INIT;
  if (!W) return AENET_ERR_INPUT;
  size_t o = 0;
  for (auto& p : g.pots) {
    std::copy(p.net.W.begin(), p.net.W.end(), W + o);
    o += p.net.W.size();
  }
  return AENET_OK;
}

// Replace every species' weights (type order, each W(1:Wsize)).  The device
// copies are overwritten in place, so plans and captured graphs stay valid.
EXPORT int aenet_gpu_set_weights(const double* W) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init || !g.loaded) return AENET_ERR_INIT;
  if (!W) return AENET_ERR_INPUT;
  size_t total = 0;
  for (auto& p : g.pots) total += p.net.W.size();
  for (size_t q = 0; q < total; ++q)
    if (!std::isfinite(W[q])) return AENET_ERR_INPUT;
  size_t o = 0;
  for (auto& p : g.pots) {
    std::copy(W + o, W + o + p.net.W.size(), p.net.W.begin());
    if (p.recs.size() > 8 && p.recs[8].size() == 8 * p.net.W.size())
      memcpy(&p.recs[8][0], p.net.W.data(), 8 * p.net.W.size());
    o += p.net.W.size();
  }
  if (g.dev_ready) {
    std::vector<double> w64;
    for (int t = 0; t < g.ntypes; ++t) {
      NetTable nt{};
      device_weights(g.pots[t].net, nt, w64);
    }
    std::vector<float> w32(w64.begin(), w64.end());
    if (cudaMemcpy(const_cast<double*>(g.pd.w64), w64.data(), 8 * w64.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(const_cast<float*>(g.pd.w32), w32.data(), 4 * w32.size(), cudaMemcpyHostToDevice))
      return AENET_ERR_CUDA;
    if (g.pd.tc_ok && g.pd.tc_img) {
      PotDevice tmp = g.pd;
      std::vector<unsigned char> img = make_tc_image(tmp, g.scale_host);
      if (img.empty() || cudaMemcpy(const_cast<unsigned char*>(g.pd.tc_img), img.data(), img.size(),
                                    cudaMemcpyHostToDevice))
        return AENET_ERR_CUDA;
    }
  }
  return AENET_OK;
}

// Write the potential of one species with its current weights, in the
// record layout it was read with (save_Network / save_Setup /
// save_TrnSet_info, feedforward.f90:291-306, sfsetup.f90:585-609,
// trainset.f90:432-441).
EXPORT int aenet_gpu_save_potential(int type_id, const char* filename) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.init) return AENET_ERR_INIT;
  if (type_id < 1 || type_id > g.ntypes || !g.pots[type_id - 1].init) return AENET_ERR_TYPE;
  if (!filename || strlen(filename) > 1024) return AENET_ERR_MALLOC;
  return write_records(filename, g.pots[type_id - 1].recs) ? AENET_OK : AENET_ERR_IO;
}

// Same pipeline as aenet_gpu_plan_run(..., AENET_GPU_FORCES) with CUDA
// events recorded on `stream` between the stages; ms[0..6] receive the
// durations of: type check, neighbour search, descriptor, networks,
// energy reduction, adjoint (forces), force output.  Synchronises.
EXPORT int aenet_gpu_plan_profile(aenet_gpu_plan* P, const double* d_coords, const int* d_types,
                                  double* d_E, double* d_F, float* ms, void* stream) {
  if (!P || !ms) return AENET_ERR_INPUT;
  cudaStream_t s = (cudaStream_t)stream;
  const PotDevice& pd = *P->pd;
  cudaEvent_t ev[9];
  for (int q = 0; q < 9; ++q) cudaEventCreate(&ev[q]);
  int e = 0;
  cudaEventRecord(ev[0], s);
  NbBuffers nb = nb_buffers(P);
  const int* t_in = search_types(P, nb, d_types, s);
  if (!t_in) e = 1;
  cudaEventRecord(ev[1], s);
  nb.ev_search = ev[8];
  if (t_in) e |= ae_launch_neighbors(P->natoms, d_coords, t_in, nb, P->fp64, s);
  cudaEventRecord(ev[2], s);
  DescBuffers d = desc_buffers(P, nullptr, false);
  if (d.nb_rank)
    e |= ae_launch_stale_order(P->natoms, P->geom_d, P->atom_struct, P->r_wrap, pd, d, P->fp64,
                               P->stale_caller_order, P->nb_rank, P->nb_seff, s);
  e |= (pd.sp[0].sftype == AE_SF_BEHLER) ? ae_launch_behler_forward(pd, d, P->fp64, s)
                                          : ae_launch_chebyshev_forward(pd, d, P->fp64, s);
  cudaEventRecord(ev[3], s);
  e |= plan_networks(P, d, s);
  cudaEventRecord(ev[4], s);
  e |= ae_launch_energy_reduce_chunked(P->nstruc, P->nchunks, P->geom_d, P->chunk_struct,
                                       P->E_atom, P->e_part, P->E_struct, P->one_chunk_each, s);
  if (d_E) cudaMemcpyAsync(d_E, P->E_struct, 8 * (size_t)P->nstruc, cudaMemcpyDeviceToDevice, s);
  cudaEventRecord(ev[5], s);
  const size_t tsz = P->fp64 ? 8 : 4;
  cudaMemsetAsync(P->Facc, 0, 4 * tsz * (size_t)P->natoms, s);
  if (g.lpa_adjoint) d.lpa = g.lpa_adjoint;
  e |= (pd.sp[0].sftype == AE_SF_BEHLER) ? ae_launch_behler_adjoint(pd, d, P->fp64, s)
                                          : ae_launch_chebyshev_adjoint(pd, d, P->fp64, s);
  cudaEventRecord(ev[6], s);
  if (d_F) e |= ae_launch_forces_out(P->natoms, P->Facc, P->fp64, d_F, 1.0, s);
  cudaEventRecord(ev[7], s);
  if (cudaEventSynchronize(ev[7]) != cudaSuccess) e = 1;
  for (int q = 0; q < 7; ++q) cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]);
  cudaEventElapsedTime(&ms[7], ev[8], ev[2]);
  for (int q = 0; q < 9; ++q) cudaEventDestroy(ev[q]);
  return e ? AENET_ERR_CUDA : 0;
}

EXPORT int aenet_gpu_measure_fp32_peak(double* tflops, void* stream) {
  if (!tflops) return AENET_ERR_INPUT;
  if (!cuda_ok()) return AENET_ERR_CUDA;
  return ae_fma_peak(tflops, (cudaStream_t)stream) ? AENET_ERR_CUDA : 0;
}

EXPORT unsigned aenet_gpu_plan_status(aenet_gpu_plan* P, void* stream) {
  if (!P) return 0;
  unsigned v = 0;
  cudaMemcpyAsync(&v, P->status, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  cudaStreamSynchronize((cudaStream_t)stream);
  return v;
}

EXPORT int aenet_gpu_plan_neighbors(aenet_gpu_plan* P, int* cap, const int** d_counts,
                                    const int** d_jt, const void** d_vec) {
  if (!P) return AENET_ERR_INPUT;
  *cap = P->cap;
  *d_counts = P->nb_cnt;
  *d_jt = P->nb_jt;
  *d_vec = P->nb_vec;
  return 0;
}

EXPORT int aenet_gpu_plan_descriptors(aenet_gpu_plan* P, const void** d_G, int* nsf_pad) {
  if (!P) return AENET_ERR_INPUT;
  *d_G = P->G;
  *nsf_pad = P->pd->nsf_pad;
  return 0;
}

// ---- internal accessors used by noalloc.cu ----------------------------

// Copy of the device tables of the loaded potentials and the neighbour
// cut-off; returns 0 when the tables exist (they are built by the first
// evaluation after loading), AENET_ERR_INIT otherwise.  Never allocates.
int ae_device_tables(PotDevice* out, double* rc, int* cell_div) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!(g.init && g.loaded && g.dev_ready)) return AENET_ERR_INIT;
  *out = g.pd;
  *rc = aenet_Rc_max;
  *cell_div = g.cell_div;
  return 0;
}

int ae_lanes_per_atom() { return g.lpa_default; }

// Geometry of one periodic structure (host arithmetic only).
int ae_periodic_geom(StructGeom* G, const double* lattice, int natoms, double rc, int cell_div) {
  return make_geom(*G, lattice, 1, nullptr, natoms, rc, cell_div, 0);
}

// ---- host-buffer entry points ----------------------------------------

namespace {


bool cache_matches(const HostPlanCache& c, int nstruc, const int* natoms, const double* lattices,
                   const int* pbc, int precision) {
  if (!c.plan || c.precision != precision || (int)c.natoms.size() != nstruc || c.isolated) return false;
  if ((c.plan->nb_rank != nullptr) != stale_spin_wanted()) return false;
  if (memcmp(c.natoms.data(), natoms, 4 * (size_t)nstruc)) return false;
  for (int s = 0; s < nstruc; ++s)
    if (c.pbc[s] != (pbc ? (pbc[s] ? 1 : 0) : 1)) return false;
  if (lattices && memcmp(c.lattices.data(), lattices, 72 * (size_t)nstruc)) return false;
  return true;
}

// One chunk: (re)build its plan when the layout changed or cap > 0 asks
// for a larger capacity, then enqueue on its stream the copies in, the run
// and the status read back.  Nothing waits here.
int chunk_submit(HostPlanCache& c, int nstruc, const int* natoms, const double* coords,
                 const int* type_ids, const double* lattices, const int* pbc, int precision,
                 bool want_E_atoms, bool want_virial, bool want_forces, int cap) {
  int st = 0;
  if (cap > 0 || !cache_matches(c, nstruc, natoms, lattices, pbc, precision)) {
    c.reset();
    c.plan.reset(plan_new(nstruc, natoms, lattices, pbc, coords, precision, &g.pd, aenet_Rc_max,
                          cap, false, &st));
    if (!c.plan) return st ? st : AENET_ERR_CUDA;
    c.natoms.assign(natoms, natoms + nstruc);
    c.pbc.assign(nstruc, 1);
    c.isolated = false;
    for (int q = 0; q < nstruc; ++q) {
      c.pbc[q] = pbc ? (pbc[q] ? 1 : 0) : 1;
      if (!c.pbc[q]) c.isolated = true;   // binning box follows the coordinates
    }
    c.lattices.assign(lattices ? lattices : nullptr, lattices ? lattices + 9 * (size_t)nstruc : nullptr);
    c.precision = precision;
  }
  if (!c.stream && cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess)
    return AENET_ERR_CUDA;
  if (!c.status_h && cudaHostAlloc(&c.status_h, 16, cudaHostAllocDefault) != cudaSuccess) {
    c.status_h = nullptr;
    return AENET_ERR_CUDA;
  }
  aenet_gpu_plan* P = c.plan.get();
  const int N = P->natoms;
  const size_t bytes = 24 * (size_t)N + 4 * (size_t)N + 8 * (size_t)nstruc + 8 * (size_t)N +
                       24 * (size_t)N + 72 * (size_t)nstruc + 1024;
  if (c.io_bytes < bytes) {
    if (c.io) cudaFree(c.io);
    c.io = nullptr;
    if (cudaMalloc(&c.io, bytes) != cudaSuccess) return AENET_ERR_CUDA;
    c.io_bytes = bytes;
  }
  double* d_c = (double*)c.io;
  double* d_F = d_c + 3 * (size_t)N;
  double* d_Ea = d_F + 3 * (size_t)N;
  double* d_E = d_Ea + N;
  double* d_V = d_E + nstruc;
  int* d_t = (int*)(d_V + 9 * (size_t)nstruc);
  cudaStream_t s = c.stream;
  *c.status_h = 0;
  if (cudaMemsetAsync(P->status, 0, 4, s) ||
      cudaMemcpyAsync(d_c, coords, 24 * (size_t)N, cudaMemcpyHostToDevice, s) ||
      cudaMemcpyAsync(d_t, type_ids, 4 * (size_t)N, cudaMemcpyHostToDevice, s))
    return AENET_ERR_CUDA;
  const unsigned flags =
      (want_forces ? AENET_GPU_FORCES : 0u) | (want_virial ? AENET_GPU_VIRIAL : 0u);
  const unsigned key = flags | (want_E_atoms ? 4u : 0u);
  if (!c.graph || c.graph_key != key || c.graph_gen != g.gen) {
    // capture the run once per plan, outputs and settings; replays then
    // cost one launch
    c.drop_graph();
    cudaGraph_t gr = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return AENET_ERR_CUDA;
    st = aenet_gpu_plan_run(P, d_c, d_t, d_E, want_E_atoms ? d_Ea : nullptr,
                            (want_forces || want_virial) ? d_F : nullptr,
                            want_virial ? d_V : nullptr, flags, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &gr);
    if (st || ce != cudaSuccess || !gr) {
      if (gr) cudaGraphDestroy(gr);
      cudaGetLastError();
      return st ? st : AENET_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&c.graph, gr, 0);
    cudaGraphDestroy(gr);
    if (ie != cudaSuccess) {
      c.graph = nullptr;
      return AENET_ERR_CUDA;
    }
    c.graph_key = key;
    c.graph_gen = g.gen;
  }
  if (cudaGraphLaunch(c.graph, s) != cudaSuccess) return AENET_ERR_CUDA;
  return cudaMemcpyAsync(c.status_h, P->status, 4, cudaMemcpyDeviceToHost, s) ? AENET_ERR_CUDA : 0;
}

// The chunk's results back to the caller's arrays (enqueued after every
// chunk's run, so that a pageable destination, which makes the copy wait
// for its data, holds up no other chunk's kernels).
int chunk_collect(HostPlanCache& c, int nstruc, double* E, double* E_atoms, double* F,
                  double* virial, bool want_forces) {
  aenet_gpu_plan* P = c.plan.get();
  const int N = P->natoms;
  double* d_c = (double*)c.io;
  double* d_F = d_c + 3 * (size_t)N;
  double* d_Ea = d_F + 3 * (size_t)N;
  double* d_E = d_Ea + N;
  double* d_V = d_E + nstruc;
  cudaStream_t s = c.stream;
  if (E && cudaMemcpyAsync(E, d_E, 8 * (size_t)nstruc, cudaMemcpyDeviceToHost, s))
    return AENET_ERR_CUDA;
  if (E_atoms && cudaMemcpyAsync(E_atoms, d_Ea, 8 * (size_t)N, cudaMemcpyDeviceToHost, s))
    return AENET_ERR_CUDA;
  if (F && want_forces && cudaMemcpyAsync(F, d_F, 24 * (size_t)N, cudaMemcpyDeviceToHost, s))
    return AENET_ERR_CUDA;
  if (virial && cudaMemcpyAsync(virial, d_V, 72 * (size_t)nstruc, cudaMemcpyDeviceToHost, s))
    return AENET_ERR_CUDA;
  return 0;
}

// after a failure: let every chunk's queued work finish, then drop the plans
int drain_and_reset(int st) {
  for (auto& c : g_cache)
    if (c.stream) cudaStreamSynchronize(c.stream);
  host_cache_reset();
  return st;
}

int batch_host(int nstruc, const int* natoms, const double* coords, const int* type_ids,
               const double* lattices, const int* pbc, int precision, double* E,
               double* E_atoms, double* F, double* virial, bool want_forces) {
  int st = ensure_device();
  if (st) return st;
  // chunks of whole structures with about equal atom counts
  long long Ntot = 0;
  for (int q = 0; q < nstruc; ++q) Ntot += natoms[q];
  int C = (int)std::min<long long>(AE_HOST_CHUNKS, std::max<long long>(1, Ntot / AE_CHUNK_ATOMS));
  C = std::min(C, nstruc);
  int sb[AE_HOST_CHUNKS + 1];
  long long ab[AE_HOST_CHUNKS + 1];
  sb[0] = 0;
  ab[0] = 0;
  {
    long long acc = 0;
    int k = 1;
    for (int q = 0; q < nstruc && k < C; ++q) {
      acc += natoms[q];
      if (acc * C >= Ntot * k) {
        sb[k] = q + 1;
        ab[k] = acc;
        ++k;
      }
    }
    for (; k < C; ++k) {   // fewer structures than cut points: empty chunks are dropped below
      sb[k] = nstruc;
      ab[k] = Ntot;
    }
    sb[C] = nstruc;
    ab[C] = Ntot;
  }
  int caps[AE_HOST_CHUNKS] = {0, 0, 0, 0};
  bool pending[AE_HOST_CHUNKS];
  for (int k = 0; k < C; ++k) pending[k] = sb[k + 1] > sb[k];
  for (int k = C; k < AE_HOST_CHUNKS; ++k) g_cache[k].reset();   // the layout changed
  for (int attempt = 0; attempt < 4; ++attempt) {
    for (int k = 0; k < C; ++k) {
      if (!pending[k]) continue;
      const int s0 = sb[k], ns = sb[k + 1] - s0;
      const size_t a0 = (size_t)ab[k];
      st = chunk_submit(g_cache[k], ns, natoms + s0, coords + 3 * a0, type_ids + a0,
                        lattices ? lattices + 9 * (size_t)s0 : nullptr, pbc ? pbc + s0 : nullptr,
                        precision, E_atoms != nullptr, virial != nullptr, want_forces, caps[k]);
      if (st) return drain_and_reset(st);
    }
    for (int k = 0; k < C; ++k) {
      if (!pending[k]) continue;
      const int s0 = sb[k], ns = sb[k + 1] - s0;
      const size_t a0 = (size_t)ab[k];
      st = chunk_collect(g_cache[k], ns, E ? E + s0 : nullptr, E_atoms ? E_atoms + a0 : nullptr,
                         F ? F + 3 * a0 : nullptr, virial ? virial + 9 * (size_t)s0 : nullptr,
                         want_forces);
      if (st) return drain_and_reset(st);
    }
    bool again = false;
    int err = 0;
    for (int k = 0; k < C; ++k) {
      if (!pending[k]) continue;
      HostPlanCache& c = g_cache[k];
      if (cudaStreamSynchronize(c.stream) != cudaSuccess) return drain_and_reset(AENET_ERR_CUDA);
      const unsigned status = *c.status_h;
      pending[k] = false;
      if (status & AE_ST_TC_TIMEOUT) {
        c.reset();
        err = AENET_ERR_CUDA;
      } else if (status & AE_ST_BAD_COORD) {
        err = err ? err : AENET_ERR_INPUT;
      } else if (status & AE_ST_BAD_TYPE) {
        err = err ? err : AENET_ERR_TYPE;
      } else if (status & (AE_ST_NB_OVERFLOW | AE_ST_CELL_OVERFLOW)) {
        // retry with larger capacities (the angular capacity follows cap)
        caps[k] = c.plan->cap * 2;
        pending[k] = true;
        again = true;
      }
    }
    if (err) return err;
    if (!again) return 0;
  }
  return AENET_ERR_MALLOC;
}

}  // namespace

EXPORT void aenet_gpu_structure_energy_forces(int natoms, const double* coords, const int* type_ids,
                                              const double* lattice, int pbc, int precision,
                                              double* E_total, double* E_coh, double* E_atoms,
                                              double* F, double* virial, int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!(g.init && g.loaded)) {
    *stat = AENET_ERR_INIT;
    return;
  }
  if (natoms < 1 || !coords || !type_ids) {
    *stat = AENET_ERR_INPUT;
    return;
  }
  std::vector<double> Ea(natoms);
  double E = 0;
  int st = batch_host(1, &natoms, coords, type_ids, lattice, &pbc, precision, &E, Ea.data(), F,
                      virial, F != nullptr);
  if (st) {
    *stat = st;
    return;
  }
  if (E_total) *E_total = E;
  if (E_atoms) memcpy(E_atoms, Ea.data(), 8 * (size_t)natoms);
  if (E_coh) {
    double c = E;
    for (int i = 0; i < natoms; ++i) c -= g.pots[type_ids[i] - 1].E_atom;
    *E_coh = c;
  }
  *stat = AENET_OK;
}

EXPORT void aenet_gpu_batch_energy_forces(int nstruc, const int* natoms, const double* coords,
                                          const int* type_ids, const double* lattices, const int* pbc,
                                          int precision, double* E, double* F, double* virial,
                                          int* stat) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!(g.init && g.loaded)) {
    *stat = AENET_ERR_INIT;
    return;
  }
  if (nstruc < 1 || !natoms || !coords || !type_ids) {
    *stat = AENET_ERR_INPUT;
    return;
  }
  *stat = batch_host(nstruc, natoms, coords, type_ids, lattices, pbc, precision, E, nullptr, F,
                     virial, F != nullptr);
}
