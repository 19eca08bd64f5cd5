// Descriptor Jacobians of the Chebyshev basis in FP64, for the PyTorch
// export of generate.x (sfderiv_i / sfderiv_j of stp_eval, written by
// pyo_write_atom_sf_info, src/pytorchoutput.f90:104-138).
//
// One warp per central atom, one lane per neighbour slot.  Radial terms
// (sfb_radial, src/ext/sfbasis.f90:762-793): dG_n/dR_j = (R_ij/d)(fc' T_n +
// fc T_n').  Angular terms (sfb_angular, sfbasis.f90:797-858): the lane of
// slot a walks every partner b and adds d(w T_n(cos))/dR_a to its own row,
// so each pair is evaluated from both ends and no two lanes write the same
// row.  The central atom's row is minus the sum over the neighbours (the
// descriptor depends on R_ij = r_j - r_i only).  Raw, unnormalised values,
// as stp_eval returns them without `scaled`.
#include "k_cheb_impl.cuh"

namespace {

using cheb::SFB_EPS;
using cheb::SFB_PI;

__global__ void __launch_bounds__(128) k_jacobian(PotDevice pd, DescBuffers b, int atom0, int count,
                                                  int nsf_max, double* __restrict__ Ji,
                                                  double* __restrict__ Jj, int* __restrict__ nbl,
                                                  int* __restrict__ nnb) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;   // row of the output
  if (r >= count) return;
  const int i = atom0 + r;
  const int n = b.nb_cnt[i];
  const ChebTable& ct = pd.sp[b.types[i]].cheb;
  const double4_32a* __restrict__ vec =
      reinterpret_cast<const double4_32a*>(b.nb_vec) + (size_t)i * b.cap;
  const int* __restrict__ jt = b.nb_jt + (size_t)i * b.cap;
  const size_t rs = (size_t)nsf_max * 3;
  double* __restrict__ Jrow = Jj + (size_t)r * b.cap * rs;
  const bool multi = ct.multi;
  const double r_Rc = ct.r_Rc, a_Rc = ct.a_Rc;
  if (lane == 0) nnb[r] = n;

  // ---- zero the rows, radial terms
  for (int a = lane; a < n; a += 32) {
    double* Ja = Jrow + (size_t)a * rs;
    for (size_t q = 0; q < rs; ++q) Ja[q] = 0.0;
    nbl[(size_t)r * b.cap + a] = jt[a] & AE_INDEX_MASK;
    const double4_32a v = vec[a];
    const double d = v.w;
    const double s = multi ? (double)ct.spin[jt[a] >> AE_TYPE_SHIFT] : 0.0;
    if (d <= r_Rc && d > SFB_EPS) {
      double fc, dfc;
      cheb::cutoff(d, r_Rc, fc, dfc);
      const double x = (2.0 * d - r_Rc) / r_Rc, x2 = x + x, dxdd = 2.0 / r_Rc;
      double tm1 = 1.0, t0 = x, um1 = 1.0, u0 = x2;   // T_q and U_{q-1}
      for (int q = 0; q < ct.r_N; ++q) {
        double Tq, dTq;
        if (q == 0) {
          Tq = 1.0;
          dTq = 0.0;
        } else {
          Tq = t0;
          dTq = q * um1 * dxdd;
          const double tn = x2 * t0 - tm1;
          tm1 = t0;
          t0 = tn;
          const double un = x2 * u0 - um1;
          um1 = u0;
          u0 = un;
        }
        const double g = (dfc * Tq + fc * dTq) / d;
        for (int c = 0; c < 3; ++c) {
          const double Rc = c == 0 ? v.x : (c == 1 ? v.y : v.z);
          Ja[(ct.r_i1 + q) * 3 + c] = g * Rc;
          if (multi) Ja[(ct.r_i2 + q) * 3 + c] = s * g * Rc;
        }
      }
    }
  }
  __syncwarp();

  // ---- angular terms: the lane of slot a over all partners b
  for (int a = lane; a < n; a += 32) {
    const double4_32a va = vec[a];
    const double da = va.w;
    if (!(da <= a_Rc && da >= SFB_EPS)) continue;
    double fa, dfa;
    cheb::cutoff(da, a_Rc, fa, dfa);
    const double sa = multi ? (double)ct.spin[jt[a] >> AE_TYPE_SHIFT] : 0.0;
    const double id_a2 = 1.0 / (da * da);
    double* Ja = Jrow + (size_t)a * rs;
    for (int bb = 0; bb < n; ++bb) {
      if (bb == a) continue;
      const double4_32a vb = vec[bb];
      const double db = vb.w;
      if (!(db <= a_Rc && db >= SFB_EPS)) continue;
      double fb, dfb;
      cheb::cutoff(db, a_Rc, fb, dfb);
      const double sb = multi ? (double)ct.spin[jt[bb] >> AE_TYPE_SHIFT] : 0.0;
      const double id_ab = 1.0 / (da * db);
      const double cosv = (va.x * vb.x + va.y * vb.y + va.z * vb.z) / (da * db);
      double x, dxdc;
      cheb::angular_arg(cosv, ct.angular_legacy, x, dxdc);
      const double w = fa * fb;
      // d cos / dR_a and d w / dR_a
      double dcos[3], dw[3];
      const double Ra[3] = {va.x, va.y, va.z}, Rb[3] = {vb.x, vb.y, vb.z};
      for (int c = 0; c < 3; ++c) {
        dcos[c] = -cosv * Ra[c] * id_a2 + Rb[c] * id_ab;
        dw[c] = dfa * fb * Ra[c] / da;
      }
      const double x2 = x + x;
      double tm1 = 1.0, t0 = x, um1 = 1.0, u0 = x2;
      const double ss = sa * sb;
      for (int q = 0; q < ct.a_N; ++q) {
        double Tq, dTq;
        if (q == 0) {
          Tq = 1.0;
          dTq = 0.0;
        } else {
          Tq = t0;
          dTq = q * um1 * dxdc;
          const double tn = x2 * t0 - tm1;
          tm1 = t0;
          t0 = tn;
          const double un = x2 * u0 - um1;
          um1 = u0;
          u0 = un;
        }
        for (int c = 0; c < 3; ++c) {
          const double val = dw[c] * Tq + w * dTq * dcos[c];
          Ja[(ct.a_i1 + q) * 3 + c] += val;
          if (multi) Ja[(ct.a_i2 + q) * 3 + c] += ss * val;
        }
      }
    }
  }
  __syncwarp();

  // ---- the central atom: minus the neighbours' sum
  const int nq = ct.nsf * 3;
  for (int q = lane; q < (int)rs; q += 32) {
    double acc = 0.0;
    if (q < nq)
      for (int a = 0; a < n; ++a) acc -= Jrow[(size_t)a * rs + q];
    Ji[(size_t)r * rs + q] = acc;
  }
}

}  // namespace

int ae_launch_chebyshev_jacobian(const PotDevice& pd, const DescBuffers& b, int atom0, int count,
                                 int nsf_max, double* Ji, double* Jj, int* nbl, int* nnb,
                                 cudaStream_t s) {
  if (count <= 0) return 0;
  const int blocks = (count + 3) / 4;
  k_jacobian<<<blocks, 128, 0, s>>>(pd, b, atom0, count, nsf_max, Ji, Jj, nbl, nnb);
  return (int)cudaGetLastError();
}
