/*
 * aenet_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C FP64 restatement of aenet's energy-and-force path, used as the
 * parity oracle for the GPU evaluator and as the timed CPU baseline.  It is
 * never linked into, loaded by, or called from the product library; only the
 * test suite, the smoke check and the benchmark's CPU-baseline leg use it.
 *
 * Every routine follows the reference Fortran statement by statement where
 * the arithmetic matters (constants, evaluation order, loop order) and cites
 * the file:line it restates (paths relative to the aenet source tree):
 *
 *   neighbour list ....... src/ext/lclist.f90      (lcl_init, lcl_nblist,
 *                                                   lcl_nbdist_cart, cell
 *                                                   multiples, T vectors)
 *   Chebyshev basis ...... src/ext/chebyshev.f90, src/ext/sfbasis.f90
 *   Behler functions ..... src/ext/symmfunc.f90
 *   setup/normalisation .. src/sfsetup.f90
 *   network .............. src/ext/feedforward.f90
 *   energy/forces ........ src/aenet.f90:359-486
 *   structure driver ..... src/predict.F90:574-706, src/geometry.f90:491-739
 *
 * Compile with -ffp-contract=off so that a*b+c is never fused: the neighbour
 * predicate is defined on unfused IEEE arithmetic (the GPU kernel uses the
 * same unfused operations), which makes neighbour sets bit-comparable.
 *
 * Switches beyond the current reference semantics (all default off):
 *   angular domain "legacy"  : T_n((2cos - pi)/pi) angular basis used by the
 *                              potentials shipped with the reference.
 *   normaliser "legacy"      : (G - avg)/max(avg - min, max - avg), the
 *                              scaling of 16-record setups (no sfval_cov).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

#define MAXT 16
#define MAXL 16
#define NG 5

/* sfbasis.f90:72-75 (note the truncated PI) */
static const double SFB_PI = 3.14159265358979;
static const double SFB_EPS = 1.0e-12;
/* symmfunc.f90:38 */
static const double SF_PI = 3.14159265358979;
/* constants.f90 */
static const double CONST_PI = 3.141592653589793;

enum { ORC_OK = 0, ORC_ERR_INIT = 1, ORC_ERR_MALLOC = 2, ORC_ERR_IO = 3,
       ORC_ERR_TYPE = 4, ORC_ERR_ARG = 5 };

/* ------------------------------------------------------------------ */
/*  data model: Network (feedforward.f90:55-89), Setup                */
/*  (sfsetup.f90:81-154), NNPot (potential.f90:68-103)                */
/* ------------------------------------------------------------------ */

typedef struct {
    int init;
    int nlayers;
    int nnodes[MAXL + 1];   /* 1-based */
    int f_a[MAXL + 1];      /* 2..nlayers */
    int iw[MAXL + 1];       /* 1-based */
    int iv[MAXL + 1];       /* 1-based */
    int nnodes_max, Wsize, nvalues;
    double *W;              /* W(1:Wsize) stored 0-based */
} orc_net;

typedef struct {
    int init;
    int sftype;             /* 1 Chebyshev, 2 Behler2011 */
    int nenv;
    int env_global[MAXT + 1];   /* gtype(1:nenv)   sfsetup.f90:740-750 */
    int ltype[MAXT + 1];        /* ltype(1:ntypes) sfsetup.f90:729-737 */
    double Rc_min, Rc_max;
    int nsf;
    int *sf;                /* sf(nsf) */
    double *sfparam;        /* sfparam(4, nsf) column-major */
    int *sfenv;             /* sfenv(2, nsf) column-major */
    double *vmin, *vmax, *vavg, *vcov;
    int normalizer;         /* 0 = avg/cov (current), 1 = legacy min/max */
} orc_setup;

typedef struct {
    int init;
    orc_net net;
    orc_setup stp;
    double E_scale, E_shift, E_atom;
} orc_pot;

/* FingerprintBasis (sfbasis.f90:51-70) */
typedef struct {
    int init;
    int r_order, a_order, r_N, a_N;
    double r_Rc, a_Rc;
    int r_i1, r_f1, r_i2, r_f2, a_i1, a_f1, a_i2, a_f2;
    int N, num_types, multi, num_values;
    double typespin[MAXT + 1];  /* 1-based by local type */
} orc_sfb;

static int g_init = 0;
static int g_loaded = 0;
static int g_ntypes = 0;
static orc_pot g_pot[MAXT + 1];
static orc_sfb g_sfb[MAXT + 1];
static int g_angular_legacy = 0;
static double g_Rc_min = 0.0, g_Rc_max = 0.0;
/* Candidate mode of the neighbour list.  0: the linked-cell candidate
 * search of lclist.f90 as written (it can miss neighbours in thin cells,
 * see orc_set_complete_candidates).  1: every atom is a candidate and the
 * image box is sized from the true reciprocal lattice, which yields every
 * (atom, image) pair within the cut-off. */
static int g_complete = 1;
static int g_nnb_max = 0, g_nsf_max = 0;

/* ------------------------------------------------------------------ */
/* Behler tables: symmfunc.f90:63-79 (module variables)               */
/* ------------------------------------------------------------------ */
static int sf_isInit = 0;
static int sf_nTypes, sf_nPairs, sf_nTriples, sf_nGMax;
static int *sf_idx2;   /* (nTypes, nTypes) */
static int *sf_idx3;   /* (nTypes, nTypes, nTypes) */
static int *sf_iG02, *sf_iG03;
static int *sf_nG2, *sf_nG3;   /* (NG, nPairs) / (NG, nTriples) */
static int *sf_nG_type;
static double *sf_pG1, *sf_pG2, *sf_pG3, *sf_pG4, *sf_pG5;

#define IDX2(i, j) sf_idx2[((j) - 1) * sf_nTypes + ((i) - 1)]
#define IDX3(i, j, k) sf_idx3[(((k) - 1) * sf_nTypes + ((j) - 1)) * sf_nTypes + ((i) - 1)]
#define NG2(f, p) sf_nG2[((p) - 1) * NG + ((f) - 1)]
#define NG3(f, t) sf_nG3[((t) - 1) * NG + ((f) - 1)]
#define PG1(g, p) sf_pG1[((p) - 1) * sf_nGMax + ((g) - 1)]
#define PG2(a, g, p) sf_pG2[(((p) - 1) * sf_nGMax + ((g) - 1)) * 3 + ((a) - 1)]
#define PG3(a, g, p) sf_pG3[(((p) - 1) * sf_nGMax + ((g) - 1)) * 2 + ((a) - 1)]
#define PG4(a, g, t) sf_pG4[(((t) - 1) * sf_nGMax + ((g) - 1)) * 4 + ((a) - 1)]
#define PG5(a, g, t) sf_pG5[(((t) - 1) * sf_nGMax + ((g) - 1)) * 4 + ((a) - 1)]

/* ================================================================== */
/*                         small vector helpers                       */
/* ================================================================== */

/* Fortran matmul(A(3,3), v(3)) with column-major A: sum over columns in
 * ascending order. */
static inline void matvec3(const double *A, const double *v, double *out)
{
    for (int r = 0; r < 3; ++r) {
        double s = A[0 * 3 + r] * v[0];
        s = s + A[1 * 3 + r] * v[1];
        s = s + A[2 * 3 + r] * v[2];
        out[r] = s;
    }
}

static inline double dot3(const double *a, const double *b)
{
    double s = a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}

/* lclist.f90:1058-1068 / geometry.f90:521-531 */
static inline void vproduct(const double *a, const double *b, double *c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* ================================================================== */
/*                      Chebyshev polynomials                         */
/*                 chebyshev.f90:41-75 and 81-128                     */
/* ================================================================== */

static void cheb_T(double r, double r0, double r1, int n, double *T)
{
    double x = (2.0 * r - r0 - r1) / (r1 - r0);
    T[0] = 1.0;
    if (n > 0) {
        T[1] = x;
        for (int i = 2; i <= n; ++i) T[i] = 2.0 * x * T[i - 1] - T[i - 2];
    }
}

static void cheb_dT(double r, double r0, double r1, int n, double *dT)
{
    double x = (2.0 * r - r0 - r1) / (r1 - r0);
    dT[0] = 0.0;
    if (n > 0) {
        double U1 = 1.0, U2, U3;
        dT[1] = U1;
        U2 = 2.0 * x;
        for (int i = 2; i <= n; ++i) {
            dT[i] = U2 * (double)i;
            U3 = 2.0 * x * U2 - U1;
            U1 = U2;
            U2 = U3;
        }
    }
    for (int i = 0; i <= n; ++i) dT[i] = dT[i] * 2.0 / (r1 - r0);
}

/* ================================================================== */
/*                    Chebyshev descriptor (sfbasis)                  */
/* ================================================================== */

/* new_SFBasis, sfbasis.f90:83-151 */
static void new_sfb(orc_sfb *sfb, int num_types, int r_order, int a_order,
                    double r_Rc, double a_Rc)
{
    memset(sfb, 0, sizeof(*sfb));
    sfb->num_types = num_types;
    sfb->r_order = r_order;
    sfb->a_order = a_order;
    sfb->r_Rc = r_Rc;
    sfb->a_Rc = a_Rc;
    sfb->r_N = r_order + 1;
    sfb->a_N = a_order + 1;
    sfb->num_values = sfb->r_N > sfb->a_N ? sfb->r_N : sfb->a_N;
    sfb->N = sfb->r_N + sfb->a_N;
    sfb->r_i1 = 1;
    sfb->r_f1 = sfb->r_i1 + sfb->r_N - 1;
    sfb->a_i1 = sfb->r_f1 + 1;
    sfb->a_f1 = sfb->a_i1 + sfb->a_N - 1;
    sfb->r_i2 = sfb->a_f1 + 1;
    sfb->r_f2 = sfb->r_i2 + sfb->r_N - 1;
    sfb->a_i2 = sfb->r_f2 + 1;
    sfb->a_f2 = sfb->a_i2 + sfb->a_N - 1;
    if (num_types > 1) {
        sfb->multi = 1;
        sfb->N = 2 * sfb->N;
    }
    /* typespin: sfbasis.f90:142-147 */
    int s = -num_types / 2;
    for (int i = 1; i <= num_types; ++i) {
        if (s == 0 && (num_types % 2) == 0) s = s + 1;
        sfb->typespin[i] = (double)s;
        s = s + 1;
    }
    sfb->init = 1;
}

/* sfb_fc, sfb_fc_d1: sfbasis.f90:719-752 */
static inline double sfb_fc(double Rij, double Rc)
{
    if (Rij >= Rc) return 0.0;
    return 0.5 * (cos(SFB_PI / Rc * Rij) + 1.0);
}

static inline double sfb_fc_d1(double Rij, double Rc)
{
    if (Rij >= Rc) return 0.0;
    double a = SFB_PI / Rc;
    return -0.5 * a * sin(a * Rij);
}

/* sfb_radial: sfbasis.f90:762-793 */
static void sfb_radial(const orc_sfb *sfb, const double *R_ij, double d_ij,
                       double *values, double *deriv_i, double *deriv_j)
{
    double f[64], df[64];
    double w_ij = sfb_fc(d_ij, sfb->r_Rc);
    cheb_T(d_ij, 0.0, sfb->r_Rc, sfb->r_order, f);
    for (int i = 0; i < sfb->r_N; ++i) values[i] = w_ij * f[i];
    if (deriv_i && deriv_j) {
        double dw_ij = sfb_fc_d1(d_ij, sfb->r_Rc);
        cheb_dT(d_ij, 0.0, sfb->r_Rc, sfb->r_order, df);
        for (int i = 0; i < sfb->r_N; ++i) {
            double t = dw_ij * f[i] + w_ij * df[i];
            for (int c = 0; c < 3; ++c) {
                deriv_i[i * 3 + c] = -(R_ij[c] / d_ij * t);
                deriv_j[i * 3 + c] = -deriv_i[i * 3 + c];
            }
        }
    }
}

/* sfb_angular: sfbasis.f90:797-858; the legacy switch replaces the
 * interval [-1,1] of line 825/832 by [0,PI]. */
static void sfb_angular(const orc_sfb *sfb, const double *R_ij,
                        const double *R_ik, double d_ij, double d_ik,
                        double cos_ijk, double *values, double *deriv_i,
                        double *deriv_j, double *deriv_k)
{
    double f[64], df[64];
    double r0 = g_angular_legacy ? 0.0 : -1.0;
    double r1 = g_angular_legacy ? SFB_PI : 1.0;
    double fc_j = sfb_fc(d_ij, sfb->a_Rc);
    double fc_k = sfb_fc(d_ik, sfb->a_Rc);
    double w_ijk = fc_j * fc_k;
    cheb_T(cos_ijk, r0, r1, sfb->a_order, f);
    for (int i = 0; i < sfb->a_N; ++i) values[i] = w_ijk * f[i];
    if (deriv_i && deriv_j && deriv_k) {
        double dfc_j = sfb_fc_d1(d_ij, sfb->a_Rc);
        double dfc_k = sfb_fc_d1(d_ik, sfb->a_Rc);
        cheb_dT(cos_ijk, r0, r1, sfb->a_order, df);
        double id_ij2 = 1.0 / (d_ij * d_ij);
        double id_ik2 = 1.0 / (d_ik * d_ik);
        double id_ij_ik = 1.0 / (d_ij * d_ik);
        double di_cos[3], dj_cos[3], dk_cos[3], di_w[3], dj_w[3], dk_w[3];
        for (int c = 0; c < 3; ++c) {
            di_cos[c] = cos_ijk * (R_ij[c] * id_ij2 + R_ik[c] * id_ik2)
                        - (R_ij[c] + R_ik[c]) * id_ij_ik;
            dj_cos[c] = -cos_ijk * R_ij[c] * id_ij2 + R_ik[c] * id_ij_ik;
            dk_cos[c] = -cos_ijk * R_ik[c] * id_ik2 + R_ij[c] * id_ij_ik;
            di_w[c] = -(dfc_j * fc_k * R_ij[c] / d_ij + fc_j * dfc_k * R_ik[c] / d_ik);
            dj_w[c] = dfc_j * fc_k * R_ij[c] / d_ij;
            dk_w[c] = fc_j * dfc_k * R_ik[c] / d_ik;
        }
        for (int i = 0; i < sfb->a_N; ++i) {
            for (int c = 0; c < 3; ++c) {
                deriv_i[i * 3 + c] = di_w[c] * f[i] + w_ijk * df[i] * di_cos[c];
                deriv_j[i * 3 + c] = dj_w[c] * f[i] + w_ijk * df[i] * dj_cos[c];
                deriv_k[i * 3 + c] = dk_w[c] * f[i] + w_ijk * df[i] * dk_cos[c];
            }
        }
    }
}

/* sfb_eval: sfbasis.f90:440-571.  deriv0(3,nv), deriv1(3,nv,nat) in
 * column-major order; either both or neither derivative array is given. */
static int sfb_eval(const orc_sfb *sfb, const double *coo0, int nat,
                    const int *itype1, const double *coo1, int nv,
                    double *values, double *deriv0, double *deriv1)
{
    if (!sfb->init) return ORC_ERR_INIT;
    if (nv != sfb->N) return ORC_ERR_ARG;
    int do_deriv = (deriv0 != NULL && deriv1 != NULL);
    double sv[64], sdi[3 * 64], sdj[3 * 64], sdk[3 * 64];
    if (do_deriv) {
        memset(deriv0, 0, sizeof(double) * 3 * nv);
        memset(deriv1, 0, sizeof(double) * 3 * nv * (size_t)nat);
    }
    for (int i = 0; i < sfb->N; ++i) values[i] = 0.0;
    double s_j = 1.0, s_k;
    for (int j = 0; j < nat; ++j) {
        double R_ij[3];
        for (int c = 0; c < 3; ++c) R_ij[c] = coo1[3 * j + c] - coo0[c];
        double d_ij = sqrt(dot3(R_ij, R_ij));
        if (d_ij <= sfb->r_Rc && d_ij > SFB_EPS) {
            int i1 = sfb->r_i1 - 1, N = sfb->r_N;
            double *d1j = deriv1 ? deriv1 + (size_t)3 * nv * j : NULL;
            if (do_deriv) {
                sfb_radial(sfb, R_ij, d_ij, sv, sdi, sdj);
                for (int n = 0; n < N; ++n) {
                    values[i1 + n] = values[i1 + n] + sv[n];
                    for (int c = 0; c < 3; ++c) {
                        deriv0[3 * (i1 + n) + c] += sdi[3 * n + c];
                        d1j[3 * (i1 + n) + c] += sdj[3 * n + c];
                    }
                }
            } else {
                sfb_radial(sfb, R_ij, d_ij, sv, NULL, NULL);
                for (int n = 0; n < N; ++n) values[i1 + n] = values[i1 + n] + sv[n];
            }
            if (sfb->multi) {
                int t = itype1[j];
                if (t < 1 || t > sfb->num_types) return ORC_ERR_TYPE;
                s_j = sfb->typespin[t];
                i1 = sfb->r_i2 - 1;
                for (int n = 0; n < N; ++n) {
                    values[i1 + n] = values[i1 + n] + s_j * sv[n];
                    if (do_deriv) {
                        for (int c = 0; c < 3; ++c) {
                            deriv0[3 * (i1 + n) + c] += s_j * sdi[3 * n + c];
                            d1j[3 * (i1 + n) + c] += s_j * sdj[3 * n + c];
                        }
                    }
                }
            }
        }
        if (d_ij > sfb->a_Rc) continue;
        for (int k = j + 1; k < nat; ++k) {
            double R_ik[3];
            for (int c = 0; c < 3; ++c) R_ik[c] = coo1[3 * k + c] - coo0[c];
            double d_ik = sqrt(dot3(R_ik, R_ik));
            if (d_ik > sfb->a_Rc || d_ik < SFB_EPS) continue;
            double cos_ijk = dot3(R_ij, R_ik) / (d_ij * d_ik);
            int i1 = sfb->a_i1 - 1, N = sfb->a_N;
            double *d1j = deriv1 ? deriv1 + (size_t)3 * nv * j : NULL;
            double *d1k = deriv1 ? deriv1 + (size_t)3 * nv * k : NULL;
            if (do_deriv) {
                sfb_angular(sfb, R_ij, R_ik, d_ij, d_ik, cos_ijk, sv, sdi, sdj, sdk);
                for (int n = 0; n < N; ++n) {
                    values[i1 + n] = values[i1 + n] + sv[n];
                    for (int c = 0; c < 3; ++c) {
                        deriv0[3 * (i1 + n) + c] += sdi[3 * n + c];
                        d1j[3 * (i1 + n) + c] += sdj[3 * n + c];
                        d1k[3 * (i1 + n) + c] += sdk[3 * n + c];
                    }
                }
            } else {
                sfb_angular(sfb, R_ij, R_ik, d_ij, d_ik, cos_ijk, sv, NULL, NULL, NULL);
                for (int n = 0; n < N; ++n) values[i1 + n] = values[i1 + n] + sv[n];
            }
            if (sfb->multi) {
                int t = itype1[k];
                if (t < 1 || t > sfb->num_types) return ORC_ERR_TYPE;
                s_k = sfb->typespin[t];
                i1 = sfb->a_i2 - 1;
                double sjk = s_j * s_k;
                for (int n = 0; n < N; ++n) {
                    values[i1 + n] = values[i1 + n] + sjk * sv[n];
                    if (do_deriv) {
                        for (int c = 0; c < 3; ++c) {
                            deriv0[3 * (i1 + n) + c] += sjk * sdi[3 * n + c];
                            d1j[3 * (i1 + n) + c] += sjk * sdj[3 * n + c];
                            d1k[3 * (i1 + n) + c] += sjk * sdk[3 * n + c];
                        }
                    }
                }
            }
        }
    }
    return ORC_OK;
}

/* ================================================================== */
/*                 Behler symmetry functions (symmfunc)               */
/* ================================================================== */

static void sf_final(void)
{
    if (!sf_isInit) return;
    free(sf_idx2); free(sf_idx3); free(sf_iG02); free(sf_iG03);
    free(sf_nG2); free(sf_nG3); free(sf_nG_type);
    free(sf_pG1); free(sf_pG2); free(sf_pG3); free(sf_pG4); free(sf_pG5);
    sf_isInit = 0;
}

/* sf_init: symmfunc.f90:91-140 */
static int sf_init(int ntypes, int nGmax)
{
    sf_final();
    sf_nTypes = ntypes;
    sf_nGMax = nGmax;
    sf_idx2 = calloc((size_t)ntypes * ntypes, sizeof(int));
    sf_idx3 = calloc((size_t)ntypes * ntypes * ntypes, sizeof(int));
    int idx2 = 0, idx3 = 0;
    for (int i = 1; i <= ntypes; ++i)
        for (int j = 1; j <= ntypes; ++j) {
            idx2 = idx2 + 1;
            IDX2(i, j) = idx2;
            idx3 = idx3 + 1;
            IDX3(i, j, j) = idx3;
            for (int k = j + 1; k <= ntypes; ++k) {
                idx3 = idx3 + 1;
                IDX3(i, j, k) = idx3;
                IDX3(i, k, j) = idx3;
            }
        }
    sf_nPairs = idx2;
    sf_nTriples = idx3;
    sf_nG_type = calloc(ntypes + 1, sizeof(int));
    sf_nG2 = calloc((size_t)NG * sf_nPairs, sizeof(int));
    sf_nG3 = calloc((size_t)NG * sf_nTriples, sizeof(int));
    sf_iG02 = calloc(sf_nPairs + 1, sizeof(int));
    sf_iG03 = calloc(sf_nTriples + 1, sizeof(int));
    sf_pG1 = calloc((size_t)nGmax * sf_nPairs, sizeof(double));
    sf_pG2 = calloc((size_t)3 * nGmax * sf_nPairs, sizeof(double));
    sf_pG3 = calloc((size_t)2 * nGmax * sf_nPairs, sizeof(double));
    sf_pG4 = calloc((size_t)4 * nGmax * sf_nTriples, sizeof(double));
    sf_pG5 = calloc((size_t)4 * nGmax * sf_nTriples, sizeof(double));
    if (!sf_idx2 || !sf_idx3 || !sf_nG_type || !sf_nG2 || !sf_nG3 || !sf_iG02
        || !sf_iG03 || !sf_pG1 || !sf_pG2 || !sf_pG3 || !sf_pG4 || !sf_pG5)
        return ORC_ERR_MALLOC;
    sf_isInit = 1;
    return ORC_OK;
}

/* sf_build_index: symmfunc.f90:284-305 */
static void sf_build_index(void)
{
    for (int t1 = 1; t1 <= sf_nTypes; ++t1) {
        int i = 0;
        for (int t2 = 1; t2 <= sf_nTypes; ++t2) {
            int pij = IDX2(t1, t2);
            sf_iG02[pij] = i;
            for (int f = 1; f <= NG; ++f) i += NG2(f, pij);
            for (int t3 = t2; t3 <= sf_nTypes; ++t3) {
                int tijk = IDX3(t1, t2, t3);
                sf_iG03[tijk] = i;
                for (int f = 1; f <= NG; ++f) i += NG3(f, tijk);
            }
        }
    }
}

/* sf_add_rad: symmfunc.f90:160-215 */
static int sf_add_rad(int funct, int type1, int type2, double Rc, double Rs,
                      double eta, double kappa)
{
    if (type1 < 1 || type1 > sf_nTypes || type2 < 1 || type2 > sf_nTypes)
        return ORC_ERR_TYPE;
    int pij = IDX2(type1, type2);
    if (NG2(funct, pij) >= sf_nGMax) return ORC_ERR_MALLOC;
    int iG = NG2(funct, pij) + 1;
    switch (funct) {
    case 1: PG1(iG, pij) = Rc; break;
    case 2: PG2(1, iG, pij) = Rc; PG2(2, iG, pij) = Rs; PG2(3, iG, pij) = eta; break;
    case 3: PG3(1, iG, pij) = Rc; PG3(2, iG, pij) = kappa; break;
    default: return ORC_ERR_ARG;
    }
    sf_nG_type[type1] += 1;
    NG2(funct, pij) = iG;
    sf_build_index();
    return ORC_OK;
}

/* sf_add_ang: symmfunc.f90:219-275 */
static int sf_add_ang(int funct, int type1, int type2, int type3, double Rc,
                      double eta, double lambda, double zeta)
{
    if (type1 < 1 || type1 > sf_nTypes || type2 < 1 || type2 > sf_nTypes
        || type3 < 1 || type3 > sf_nTypes)
        return ORC_ERR_TYPE;
    int tijk = IDX3(type1, type2, type3);
    if (NG3(funct, tijk) >= sf_nGMax) return ORC_ERR_MALLOC;
    int iG = NG3(funct, tijk) + 1;
    switch (funct) {
    case 4: PG4(1, iG, tijk) = Rc; PG4(2, iG, tijk) = lambda;
            PG4(3, iG, tijk) = zeta; PG4(4, iG, tijk) = eta; break;
    case 5: PG5(1, iG, tijk) = Rc; PG5(2, iG, tijk) = lambda;
            PG5(3, iG, tijk) = zeta; PG5(4, iG, tijk) = eta; break;
    default: return ORC_ERR_ARG;
    }
    sf_nG_type[type1] += 1;
    NG3(funct, tijk) = iG;
    sf_build_index();
    return ORC_OK;
}

/* sf_cut: symmfunc.f90:823-838 */
static inline void sf_cut(double Rij, double Rc, double *fc, double *dfc)
{
    if (Rij >= Rc) { *fc = 0.0; *dfc = 0.0; }
    else {
        *fc = 0.5 * (cos(SF_PI * Rij / Rc) + 1.0);
        *dfc = -0.5 * SF_PI / Rc * sin(SF_PI * Rij / Rc);
    }
}

/* G1/G2/G3 updates: symmfunc.f90:445-610 */
static void sf_rad_update(int pij, const double *v, double Rij, double *G,
                          int *iG, double *dGi, double *dGj)
{
    for (int g = 1; g <= NG2(1, pij); ++g) {
        *iG += 1;
        double fc, dfc;
        sf_cut(Rij, PG1(g, pij), &fc, &dfc);
        G[*iG - 1] += fc;
        if (dGi) for (int c = 0; c < 3; ++c) dGi[3 * (*iG - 1) + c] -= dfc * v[c];
        if (dGj) for (int c = 0; c < 3; ++c) dGj[3 * (*iG - 1) + c] += dfc * v[c];
    }
    for (int g = 1; g <= NG2(2, pij); ++g) {
        *iG += 1;
        double Rc = PG2(1, g, pij), Rs = PG2(2, g, pij), eta = PG2(3, g, pij);
        double fc, dfc;
        sf_cut(Rij, Rc, &fc, &dfc);
        double arg = Rij - Rs;
        double fexp = exp(-eta * arg * arg);
        double G2 = fexp * fc;
        double dG2 = fexp * (dfc - 2.0 * eta * arg * fc);
        G[*iG - 1] += G2;
        if (dGi) for (int c = 0; c < 3; ++c) dGi[3 * (*iG - 1) + c] -= dG2 * v[c];
        if (dGj) for (int c = 0; c < 3; ++c) dGj[3 * (*iG - 1) + c] += dG2 * v[c];
    }
    for (int g = 1; g <= NG2(3, pij); ++g) {
        *iG += 1;
        double Rc = PG3(1, g, pij), kappa = PG3(2, g, pij);
        double fc, dfc;
        sf_cut(Rij, Rc, &fc, &dfc);
        double arg = kappa * Rij;
        double fcos = cos(arg), fsin = sin(arg);
        double G3 = fcos * fc;
        double dG3 = fcos * dfc - kappa * fsin * fc;
        G[*iG - 1] += G3;
        if (dGi) for (int c = 0; c < 3; ++c) dGi[3 * (*iG - 1) + c] -= dG3 * v[c];
        if (dGj) for (int c = 0; c < 3; ++c) dGj[3 * (*iG - 1) + c] += dG3 * v[c];
    }
}

/* sf_F1_ijk: symmfunc.f90:625-654 */
static void sf_F1(const double *vij, const double *vik, double Rij, double Rik,
                  double cost, double lambda, double zeta, double *F,
                  double *dFj, double *dFk)
{
    double arg = 0.5 * (1.0 + lambda * cost);
    double prefactor = 0.5 * zeta * lambda * pow(arg, zeta - 1.0);
    *F = pow(arg, zeta);
    for (int c = 0; c < 3; ++c) {
        dFj[c] = prefactor * (-cost * (vij[c] / Rij) + vik[c] / Rij);
        dFk[c] = prefactor * (-cost * (vik[c] / Rik) + vij[c] / Rik);
    }
}

/* sf_F2_ij: symmfunc.f90:662-682 */
static inline void sf_F2(double Rij, double Rc, double eta, double *F, double *dF)
{
    double fc, dfc;
    sf_cut(Rij, Rc, &fc, &dfc);
    double fexp = exp(-eta * Rij * Rij);
    *F = fexp * fc;
    *dF = fexp * (dfc - 2.0 * eta * Rij * fc);
}

/* G4/G5 updates: symmfunc.f90:686-811 */
static void sf_ang_update(int tijk, const double *v1, const double *v2,
                          const double *v3, double Rij, double Rik, double Rjk,
                          double cost, double *G, int *iG, double *dGi,
                          double *dGj, double *dGk)
{
    double F1, dF1j[3], dF1k[3], F2ij, dF2ij, F2ik, dF2ik, F2jk, dF2jk, d[3];
    for (int g = 1; g <= NG3(4, tijk); ++g) {
        *iG += 1;
        double Rc = PG4(1, g, tijk), lambda = PG4(2, g, tijk);
        double zeta = PG4(3, g, tijk), eta = PG4(4, g, tijk);
        sf_F1(v1, v2, Rij, Rik, cost, lambda, zeta, &F1, dF1j, dF1k);
        sf_F2(Rij, Rc, eta, &F2ij, &dF2ij);
        sf_F2(Rik, Rc, eta, &F2ik, &dF2ik);
        sf_F2(Rjk, Rc, eta, &F2jk, &dF2jk);
        double G4 = F1 * F2ij * F2ik * F2jk;
        G[*iG - 1] += 2.0 * G4;
        int o = 3 * (*iG - 1);
        if (dGi) {
            for (int c = 0; c < 3; ++c)
                d[c] = F2jk * (-(dF1j[c] + dF1k[c]) * F2ij * F2ik
                               - v1[c] * F1 * dF2ij * F2ik
                               - v2[c] * F1 * F2ij * dF2ik);
            for (int c = 0; c < 3; ++c) dGi[o + c] += 2.0 * d[c];
        }
        if (dGj) {
            for (int c = 0; c < 3; ++c)
                d[c] = dF1j[c] * F2ij * F2ik * F2jk
                       + v1[c] * F1 * dF2ij * F2ik * F2jk
                       - v3[c] * F1 * F2ij * F2ik * dF2jk;
            for (int c = 0; c < 3; ++c) dGj[o + c] += 2.0 * d[c];
        }
        if (dGk) {
            for (int c = 0; c < 3; ++c)
                d[c] = dF1k[c] * F2ij * F2ik * F2jk
                       + v2[c] * F1 * F2ij * dF2ik * F2jk
                       + v3[c] * F1 * F2ij * F2ik * dF2jk;
            for (int c = 0; c < 3; ++c) dGk[o + c] += 2.0 * d[c];
        }
    }
    for (int g = 1; g <= NG3(5, tijk); ++g) {
        *iG += 1;
        double Rc = PG5(1, g, tijk), lambda = PG5(2, g, tijk);
        double zeta = PG5(3, g, tijk), eta = PG5(4, g, tijk);
        sf_F1(v1, v2, Rij, Rik, cost, lambda, zeta, &F1, dF1j, dF1k);
        sf_F2(Rij, Rc, eta, &F2ij, &dF2ij);
        sf_F2(Rik, Rc, eta, &F2ik, &dF2ik);
        double G5 = F1 * F2ij * F2ik;
        G[*iG - 1] += 2.0 * G5;
        int o = 3 * (*iG - 1);
        if (dGi) {
            for (int c = 0; c < 3; ++c)
                d[c] = -(dF1j[c] + dF1k[c]) * F2ij * F2ik
                       - v1[c] * F1 * dF2ij * F2ik - v2[c] * F1 * F2ij * dF2ik;
            for (int c = 0; c < 3; ++c) dGi[o + c] += 2.0 * d[c];
        }
        if (dGj) {
            for (int c = 0; c < 3; ++c)
                d[c] = dF1j[c] * F2ij * F2ik + v1[c] * F1 * dF2ij * F2ik;
            for (int c = 0; c < 3; ++c) dGj[o + c] += 2.0 * d[c];
        }
        if (dGk) {
            for (int c = 0; c < 3; ++c)
                d[c] = dF1k[c] * F2ij * F2ik + v2[c] * F1 * F2ij * dF2ik;
            for (int c = 0; c < 3; ++c) dGk[o + c] += 2.0 * d[c];
        }
    }
}

/* sf_fingerprint: symmfunc.f90:311-431 */
static int sf_fingerprint(int type1, const double *Xi, int nx, const double *X,
                          const int *typej, int n, double *G, double *dGi,
                          double *dGj)
{
    int deriv = (dGi != NULL && dGj != NULL);
    if (!sf_isInit) return ORC_ERR_INIT;
    if (type1 < 1 || type1 > sf_nTypes) return ORC_ERR_TYPE;
    if (n < sf_nG_type[type1]) return ORC_ERR_ARG;
    for (int i = 0; i < n; ++i) G[i] = 0.0;
    if (deriv) {
        memset(dGi, 0, sizeof(double) * 3 * n);
        memset(dGj, 0, sizeof(double) * 3 * n * (size_t)nx);
    }
    for (int j = 0; j < nx; ++j) {
        if (typej[j] < 1 || typej[j] > sf_nTypes) return ORC_ERR_TYPE;
        int pij = IDX2(type1, typej[j]);
        double R1[3];
        for (int c = 0; c < 3; ++c) R1[c] = X[3 * j + c] - Xi[c];
        double Rij = sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2]);
        for (int c = 0; c < 3; ++c) R1[c] = R1[c] / Rij;
        int iG = sf_iG02[pij];
        sf_rad_update(pij, R1, Rij, G, &iG, dGi, deriv ? dGj + (size_t)3 * n * j : NULL);
        for (int k = j + 1; k < nx; ++k) {
            if (typej[k] < 1 || typej[k] > sf_nTypes) return ORC_ERR_TYPE;
            int tijk = IDX3(type1, typej[j], typej[k]);
            double R2[3], R3[3];
            for (int c = 0; c < 3; ++c) R2[c] = X[3 * k + c] - Xi[c];
            double Rik = sqrt(R2[0] * R2[0] + R2[1] * R2[1] + R2[2] * R2[2]);
            if (!(Rik <= 1.0e-8)) for (int c = 0; c < 3; ++c) R2[c] = R2[c] / Rik;
            for (int c = 0; c < 3; ++c) R3[c] = X[3 * k + c] - X[3 * j + c];
            double Rjk = sqrt(R3[0] * R3[0] + R3[1] * R3[1] + R3[2] * R3[2]);
            if (!(Rjk <= 1.0e-8)) for (int c = 0; c < 3; ++c) R3[c] = R3[c] / Rjk;
            double cost = R1[0] * R2[0] + R1[1] * R2[1] + R1[2] * R2[2];
            if (cost < -1.0) cost = -1.0;
            if (cost > 1.0) cost = 1.0;
            iG = sf_iG03[tijk];
            sf_ang_update(tijk, R1, R2, R3, Rij, Rik, Rjk, cost, G, &iG, dGi,
                          deriv ? dGj + (size_t)3 * n * j : NULL,
                          deriv ? dGj + (size_t)3 * n * k : NULL);
        }
    }
    return ORC_OK;
}

/* ================================================================== */
/*                 setup evaluation and normalisation                 */
/* ================================================================== */

/* stp_normalize: sfsetup.f90:985-1035; legacy scaling documented at
 * sfsetup.f90:118-123 for setups without sfval_cov. */
static void stp_normalize(const orc_setup *stp, double *sfval, double *di,
                          double *dj, int n, int nsf_stride)
{
    for (int isf = 0; isf < stp->nsf; ++isf) {
        double shift = stp->vavg[isf], s, scale;
        if (stp->normalizer == 1) {
            double a = stp->vavg[isf] - stp->vmin[isf];
            double b = stp->vmax[isf] - stp->vavg[isf];
            s = a > b ? a : b;
        } else {
            s = sqrt(stp->vcov[isf] - shift * shift);
        }
        scale = (s <= 1.0e-10) ? 0.0 : 1.0 / s;
        sfval[isf] = scale * (sfval[isf] - shift);
        if (di && dj) {
            for (int c = 0; c < 3; ++c) di[3 * isf + c] = scale * di[3 * isf + c];
            for (int j = 0; j < n; ++j)
                for (int c = 0; c < 3; ++c)
                    dj[((size_t)j * nsf_stride + isf) * 3 + c] =
                        scale * dj[((size_t)j * nsf_stride + isf) * 3 + c];
        }
    }
}

/* stp_eval: sfsetup.f90:887-979 (scaled evaluation; the unscaled branch
 * that updates the running statistics is orc_stp_stats below).  di(3,nsf),
 * dj(3,nsf,n) with an nsf stride equal to nsf. */
static int stp_eval(int itype0, const double *coo0, int n, const double *coo1,
                    const int *type1, double *sfval, double *di, double *dj,
                    int scaled)
{
    orc_pot *pot = &g_pot[itype0];
    orc_setup *stp = &pot->stp;
    int type0_loc = stp->ltype[itype0];
    int *type1_loc = malloc(sizeof(int) * (n > 0 ? n : 1));
    if (!type1_loc) return ORC_ERR_MALLOC;
    for (int i = 0; i < n; ++i) {
        if (type1[i] < 1 || type1[i] > g_ntypes) { free(type1_loc); return ORC_ERR_TYPE; }
        type1_loc[i] = stp->ltype[type1[i]];
    }
    int st;
    if (stp->sftype == 1) {
        st = sfb_eval(&g_sfb[itype0], coo0, n, type1_loc, coo1, stp->nsf,
                      sfval, di, dj);
    } else {
        st = sf_fingerprint(type0_loc, coo0, n, coo1, type1_loc, stp->nsf,
                            sfval, di, dj);
    }
    free(type1_loc);
    if (st) return st;
    if (scaled) stp_normalize(stp, sfval, di, dj, n, stp->nsf);
    return ORC_OK;
}

/* ================================================================== */
/*                      feed-forward network                          */
/* ================================================================== */

/* ff_activate: feedforward.f90:932-969 */
static inline void ff_activate(int t, double x, double *y, double *dy)
{
    const double a = 1.7159, b = 0.666666666666667, c = 0.1;
    double tb;
    switch (t) {
    case 0: *y = x; *dy = 1.0; break;
    case 1: *y = tanh(x); *dy = 1.0 - (*y) * (*y); break;
    case 2: *y = 1.0 / (1.0 + exp(-x)); *dy = (*y) * (1.0 - *y); break;
    case 3: tb = tanh(b * x); *y = a * tb; *dy = a * (1.0 - tb * tb) * b; break;
    case 4: tb = tanh(b * x); *y = a * tb + c * x; *dy = a * (1.0 - tb * tb) * b + c; break;
    default: *y = 0.0; *dy = 0.0;
    }
}

/* ff_eval: feedforward.f90:586-655.  values/derivs are 1-based arrays of
 * length nvalues+1. */
static void ff_eval(const orc_net *net, const double *x, double *values,
                    double *derivs, double *y)
{
    double work[1024];
    int n1 = net->nnodes[1];
    for (int i = 1; i <= n1; ++i) values[i] = x[i - 1];
    int iw1 = 1, iv1 = 1, n2 = 1;
    for (int l = 1; l <= net->nlayers - 1; ++l) {
        int iw2 = net->iw[l + 1], iv2 = net->iv[l + 1];
        values[iv2] = 1.0;
        n2 = net->nnodes[l + 1];
        for (int r = 0; r < n2; ++r) {
            double s = 0.0;
            for (int c = 0; c <= n1; ++c)
                s = s + net->W[(iw1 - 1) + r + c * n2] * values[iv1 + c];
            work[r] = s;
        }
        iv1 = iv2 + 1;
        iw1 = iw2 + 1;
        for (int r = 0; r < n2; ++r)
            ff_activate(net->f_a[l + 1], work[r], &values[iv1 + r], &derivs[iv1 + r]);
        n1 = n2;
    }
    *y = values[iv1];
}

/* ff_deriv: feedforward.f90:661-757, including its dense work arrays of
 * size (nmax+1)x(nmax+1)^2 that are cleared on every call.  dy(1:nx);
 * jacobian(1:Wsize) 0-based. */
static void ff_deriv(const orc_net *net, const double *derivs,
                     double *jacobian, double *dy)
{
    int m = net->nnodes_max + 1;
    double *work2 = malloc(sizeof(double) * m * m);
    double *work3 = malloc(sizeof(double) * m * m);
    double *work4 = malloc(sizeof(double) * (size_t)m * m * m);
    double *tmp = malloc(sizeof(double) * m * m);
#define W2(i, j) work2[((j) - 1) * m + (i) - 1]
#define W3(i, j) work3[((j) - 1) * m + (i) - 1]
#define W4(i, j) work4[((size_t)(j) - 1) * m + (i) - 1]
    for (int i = 0; i < net->Wsize; ++i) jacobian[i] = 0.0;
    memset(work4, 0, sizeof(double) * (size_t)m * m * m);
    for (int i = 1; i <= m; ++i) W4(i, i) = 1.0;
    int iw1 = 1, iv1 = 1, n2 = 1, n1 = net->nnodes[1], n0 = n1;
    for (int l = 1; l <= net->nlayers - 1; ++l) {
        int iw2 = net->iw[l + 1], iv2 = net->iv[l + 1];
        n2 = net->nnodes[l + 1];
        for (int j = 1; j <= n2; ++j)
            for (int i = 1; i <= n2; ++i) W2(i, j) = 0.0;
        for (int i = 1; i <= n2; ++i) W2(i, i) = derivs[iv2 + i];
        /* work3 = work2 * reshape(W(iw1:iw2-n2), (n2, n1)) */
        for (int c = 1; c <= n1; ++c)
            for (int r = 1; r <= n2; ++r) {
                double s = 0.0;
                for (int k = 1; k <= n2; ++k)
                    s = s + W2(r, k) * net->W[(iw1 - 1) + (k - 1) + (c - 1) * n2];
                W3(r, c) = s;
            }
        for (int c = 1; c <= n1; ++c)
            for (int r = 1; r <= n2; ++r)
                jacobian[(iw1 - 1) + (r - 1) + (c - 1) * n2] = W3(r, c);
        /* work4(1:n2,1:n0) = work3(1:n2,1:n1) * work4(1:n1,1:n0) */
        for (int c = 1; c <= n0; ++c)
            for (int r = 1; r <= n2; ++r) {
                double s = 0.0;
                for (int k = 1; k <= n1; ++k) s = s + W3(r, k) * W4(k, c);
                tmp[(c - 1) * m + (r - 1)] = s;
            }
        for (int c = 1; c <= n0; ++c)
            for (int r = 1; r <= n2; ++r) W4(r, c) = tmp[(c - 1) * m + (r - 1)];
        iv1 = iv2 + 1;
        iw1 = iw2 + 1;
        n1 = n2;
    }
    (void)iv1;
    for (int c = 1; c <= n0; ++c) dy[c - 1] = W4(1, c);
#undef W2
#undef W3
#undef W4
    free(work2); free(work3); free(work4); free(tmp);
}

/* ff_wderiv: feedforward.f90:763-860 for a single output node.
 * dy_dw(1:Wsize) 0-based. */
static void ff_wderiv(const orc_net *net, const double *values,
                      const double *derivs, const double *jacobian,
                      double *dy_dw)
{
    int m = net->nnodes_max + 1;
    double *work2 = malloc(sizeof(double) * m * m);
    double *work3 = calloc((size_t)m * m, sizeof(double));
    double *work4 = malloc(sizeof(double) * (size_t)m * m * m);
    double *tmp = malloc(sizeof(double) * m * m);
#define W2(i, j) work2[((j) - 1) * m + (i) - 1]
#define W3(i, j) work3[((j) - 1) * m + (i) - 1]
#define W4(i, j) work4[((size_t)(j) - 1) * m + (i) - 1]
    for (int i = 1; i <= m; ++i) W3(i, i) = 1.0;
    int iv2 = net->iv[net->nlayers];
    int n2 = net->nnodes[net->nlayers], n3 = net->nnodes[net->nlayers];
    for (int l = net->nlayers - 1; l >= 1; --l) {
        int iw1 = net->iw[l] + 1, iv1 = net->iv[l] + 1;
        int n1 = net->nnodes[l];
        for (int c = 1; c <= n1 + 1; ++c)
            for (int r = 1; r <= n2; ++r)
                W2(r, c) = derivs[iv2 + r] * values[iv1 + c - 1];
        int n12 = (n1 + 1) * n2;
        for (int c = 1; c <= n12; ++c)
            for (int r = 1; r <= n2; ++r) W4(r, c) = 0.0;
        int in0 = 1;
        for (int in1 = 1; in1 <= n1 + 1; ++in1)
            for (int in2 = 1; in2 <= n2; ++in2) {
                W4(in2, in0) = W2(in2, in1);
                in0 = in0 + 1;
            }
        /* dy_dw(1:n3, iw1:iw2) = work3(1:n3,1:n2) * work4(1:n2,1:n12) */
        for (int c = 1; c <= n12; ++c) {
            double s = 0.0;
            for (int k = 1; k <= n2; ++k) s = s + W3(1, k) * W4(k, c);
            dy_dw[iw1 - 1 + c - 1] = s;
        }
        (void)n3;
        /* work3(1:n3,1:n1) = work3(1:n3,1:n2) * reshape(jacobian(iw1:iw2-n2),(n2,n1)) */
        for (int c = 1; c <= n1; ++c) {
            double s = 0.0;
            for (int k = 1; k <= n2; ++k)
                s = s + W3(1, k) * jacobian[(iw1 - 1) + (k - 1) + (c - 1) * n2];
            tmp[c - 1] = s;
        }
        for (int c = 1; c <= n1; ++c) W3(1, c) = tmp[c - 1];
        iv2 = iv1 - 1;
        n2 = n1;
    }
#undef W2
#undef W3
#undef W4
    free(work2); free(work3); free(work4); free(tmp);
}

/* ================================================================== */
/*                       public oracle interface                      */
/* ================================================================== */

ORC_EXPORT int orc_init(int ntypes)
{
    if (g_init) return ORC_ERR_INIT;
    if (ntypes < 1 || ntypes > MAXT) return ORC_ERR_ARG;
    memset(g_pot, 0, sizeof(g_pot));
    memset(g_sfb, 0, sizeof(g_sfb));
    g_ntypes = ntypes;
    g_init = 1;
    g_loaded = 0;
    g_angular_legacy = 0;
    return ORC_OK;
}

ORC_EXPORT void orc_final(void)
{
    for (int t = 1; t <= MAXT; ++t) {
        orc_pot *p = &g_pot[t];
        free(p->net.W);
        free(p->stp.sf); free(p->stp.sfparam); free(p->stp.sfenv);
        free(p->stp.vmin); free(p->stp.vmax); free(p->stp.vavg); free(p->stp.vcov);
    }
    memset(g_pot, 0, sizeof(g_pot));
    sf_final();
    g_init = 0;
    g_loaded = 0;
}

/* new_Network index bookkeeping: feedforward.f90:97-149 */
ORC_EXPORT int orc_set_network(int itype, int nlayers, const int *nnodes,
                               const int *f_a, const double *W, int Wsize)
{
    if (!g_init) return ORC_ERR_INIT;
    if (itype < 1 || itype > g_ntypes) return ORC_ERR_TYPE;
    if (nlayers < 2 || nlayers > MAXL) return ORC_ERR_ARG;
    orc_net *net = &g_pot[itype].net;
    free(net->W);
    memset(net, 0, sizeof(*net));
    net->nlayers = nlayers;
    net->nnodes_max = 0;
    for (int l = 1; l <= nlayers; ++l) {
        net->nnodes[l] = nnodes[l - 1];
        if (nnodes[l - 1] > net->nnodes_max) net->nnodes_max = nnodes[l - 1];
    }
    for (int l = 2; l <= nlayers; ++l) net->f_a[l] = f_a[l - 2];
    net->Wsize = 0;
    net->iw[1] = 0;
    for (int l = 1; l <= nlayers - 1; ++l) {
        net->Wsize += (net->nnodes[l] + 1) * net->nnodes[l + 1];
        net->iw[l + 1] = net->Wsize;
    }
    net->nvalues = 0;
    net->iv[1] = 0;
    for (int l = 1; l <= nlayers - 1; ++l) {
        net->nvalues += net->nnodes[l] + 1;
        net->iv[l + 1] = net->nvalues;
    }
    net->nvalues += net->nnodes[nlayers];
    if (Wsize != net->Wsize) return ORC_ERR_ARG;
    net->W = malloc(sizeof(double) * Wsize);
    if (!net->W) return ORC_ERR_MALLOC;
    memcpy(net->W, W, sizeof(double) * Wsize);
    if (net->nnodes[nlayers] != 1) return ORC_ERR_ARG;
    net->init = 1;
    return ORC_OK;
}

/* Setup fields (sfsetup.f90:560-621) with the type maps of
 * stp_set_global_types (sfsetup.f90:721-755): env_global[j] is the global
 * type id (1-based) whose name equals envtypes(j), or 0. */
ORC_EXPORT int orc_set_setup(int itype, int sftype, int nenv,
                             const int *env_global, double Rc_min,
                             double Rc_max, int nsf, const int *sf,
                             const double *sfparam, const int *sfenv,
                             const double *vmin, const double *vmax,
                             const double *vavg, const double *vcov,
                             int normalizer)
{
    if (!g_init) return ORC_ERR_INIT;
    if (itype < 1 || itype > g_ntypes) return ORC_ERR_TYPE;
    if (nenv < 1 || nenv > MAXT || nsf < 1) return ORC_ERR_ARG;
    orc_setup *s = &g_pot[itype].stp;
    s->sftype = sftype;
    s->nenv = nenv;
    for (int j = 1; j <= nenv; ++j) s->env_global[j] = env_global[j - 1];
    for (int g = 1; g <= g_ntypes; ++g) {
        s->ltype[g] = 0;
        for (int j = 1; j <= nenv; ++j)
            if (env_global[j - 1] == g) { s->ltype[g] = j; break; }
    }
    s->Rc_min = Rc_min;
    s->Rc_max = Rc_max;
    s->nsf = nsf;
    s->sf = malloc(sizeof(int) * nsf);
    s->sfparam = malloc(sizeof(double) * 4 * nsf);
    s->sfenv = malloc(sizeof(int) * 2 * nsf);
    s->vmin = malloc(sizeof(double) * nsf);
    s->vmax = malloc(sizeof(double) * nsf);
    s->vavg = malloc(sizeof(double) * nsf);
    s->vcov = malloc(sizeof(double) * nsf);
    memcpy(s->sf, sf, sizeof(int) * nsf);
    memcpy(s->sfparam, sfparam, sizeof(double) * 4 * nsf);
    memcpy(s->sfenv, sfenv, sizeof(int) * 2 * nsf);
    memcpy(s->vmin, vmin, sizeof(double) * nsf);
    memcpy(s->vmax, vmax, sizeof(double) * nsf);
    memcpy(s->vavg, vavg, sizeof(double) * nsf);
    if (vcov) memcpy(s->vcov, vcov, sizeof(double) * nsf);
    else memset(s->vcov, 0, sizeof(double) * nsf);
    s->normalizer = normalizer;
    s->init = 1;
    return ORC_OK;
}

/* load_NNPot: potential.f90:145-151 */
ORC_EXPORT int orc_set_energy(int itype, double scale, double shift, double E_atom)
{
    if (!g_init) return ORC_ERR_INIT;
    if (itype < 1 || itype > g_ntypes) return ORC_ERR_TYPE;
    g_pot[itype].E_scale = 1.0 / scale;
    g_pot[itype].E_shift = shift;
    g_pot[itype].E_atom = E_atom;
    g_pot[itype].init = 1;
    return ORC_OK;
}

/* lcl_nmax_nbdist: lclist.f90:229-245 */
static int lcl_nmax_nbdist(double rmin, double rmax)
{
    double V_atom = pow(0.5 * rmin, 3);
    double V_cut = pow(rmax + 0.5 * rmin, 3);
    return (int)ceil(V_cut / V_atom * 0.7405);
}

/* aenet_load_potential (aenet.f90:281-289) once all are loaded, i.e.
 * pot_get_range + stp_init (sfsetup.f90:771-826). */
ORC_EXPORT int orc_finalize(int angular_legacy)
{
    if (!g_init) return ORC_ERR_INIT;
    for (int t = 1; t <= g_ntypes; ++t)
        if (!g_pot[t].init || !g_pot[t].net.init || !g_pot[t].stp.init)
            return ORC_ERR_INIT;
    g_angular_legacy = angular_legacy;
    g_Rc_min = g_pot[1].stp.Rc_min;
    g_Rc_max = g_pot[1].stp.Rc_max;
    for (int t = 1; t <= g_ntypes; ++t) {
        if (g_pot[t].stp.Rc_min < g_Rc_min) g_Rc_min = g_pot[t].stp.Rc_min;
        if (g_pot[t].stp.Rc_max > g_Rc_max) g_Rc_max = g_pot[t].stp.Rc_max;
    }
    g_nnb_max = lcl_nmax_nbdist(g_Rc_min, g_Rc_max);
    int sftype = g_pot[1].stp.sftype;
    g_nsf_max = 0;
    for (int t = 1; t <= g_ntypes; ++t) {
        if (g_pot[t].stp.sftype != sftype) return ORC_ERR_ARG;
        if (g_pot[t].stp.nsf > g_nsf_max) g_nsf_max = g_pot[t].stp.nsf;
    }
    if (sftype == 1) {
        /* setup_basis_chebyshev: sfsetup.f90:1162-1179 */
        for (int t = 1; t <= g_ntypes; ++t) {
            orc_setup *s = &g_pot[t].stp;
            double r_Rc = s->sfparam[0];
            int r_N = (int)lround(s->sfparam[1]);
            double a_Rc = s->sfparam[2];
            int a_N = (int)lround(s->sfparam[3]);
            new_sfb(&g_sfb[t], s->nenv, r_N, a_N, r_Rc, a_Rc);
            if (g_sfb[t].N != s->nsf) return ORC_ERR_ARG;
            if (g_sfb[t].num_values > 63) return ORC_ERR_ARG;
        }
    } else {
        /* setup_symmfunc_Behler2011: sfsetup.f90:1287-1347 */
        int st = sf_init(g_ntypes, g_nsf_max);
        if (st) return st;
        for (int t = 1; t <= g_ntypes; ++t) {
            orc_setup *s = &g_pot[t].stp;
            for (int isf = 0; isf < s->nsf; ++isf) {
                int f = s->sf[isf];
                const double *p = s->sfparam + 4 * isf;
                int t2 = s->sfenv[2 * isf], t3 = s->sfenv[2 * isf + 1];
                if (f >= 1 && f <= 3) {
                    st = sf_add_rad(f, t, t2, p[0], f == 2 ? p[1] : 0.0,
                                    f == 2 ? p[2] : 0.0, f == 3 ? p[1] : 0.0);
                } else if (f == 4 || f == 5) {
                    st = sf_add_ang(f, t, t2, t3, p[0], p[3], p[1], p[2]);
                } else {
                    st = ORC_ERR_ARG;
                }
                if (st) return st;
            }
        }
    }
    g_loaded = 1;
    return ORC_OK;
}

ORC_EXPORT double orc_Rc_min(void) { return g_Rc_min; }
ORC_EXPORT double orc_Rc_max(void) { return g_Rc_max; }
ORC_EXPORT int orc_nnb_max(void) { return g_nnb_max; }
ORC_EXPORT int orc_nsf_max(void) { return g_nsf_max; }
ORC_EXPORT int orc_nsf(int itype) { return g_pot[itype].stp.nsf; }

/* Descriptor of one atom (stp_eval); di(3,nsf), dj(3,nsf,n) optional. */
ORC_EXPORT int orc_descriptor(const double *coo_i, int type_i, int n_j,
                              const double *coo_j, const int *type_j,
                              int scaled, double *sfval, double *di, double *dj)
{
    if (!g_loaded) return ORC_ERR_INIT;
    if (type_i < 1 || type_i > g_ntypes) return ORC_ERR_TYPE;
    return stp_eval(type_i, coo_i, n_j, coo_j, type_j, sfval, di, dj, scaled);
}

/* Running statistics of the unscaled branch of stp_eval (sfsetup.f90:
 * 960-977) accumulated over a set of descriptor vectors; used to write
 * potential files whose normalisation matches a given structure. */
ORC_EXPORT void orc_stp_stats(int nsf, int nvec, const double *vecs,
                              double *vmin, double *vmax, double *vavg,
                              double *vcov)
{
    for (int e = 0; e < nvec; ++e) {
        const double *v = vecs + (size_t)e * nsf;
        if (e == 0) {
            for (int i = 0; i < nsf; ++i) {
                vmin[i] = v[i]; vmax[i] = v[i]; vavg[i] = v[i]; vcov[i] = v[i] * v[i];
            }
        } else {
            for (int i = 0; i < nsf; ++i) {
                if (v[i] < vmin[i]) vmin[i] = v[i];
                if (v[i] > vmax[i]) vmax[i] = v[i];
                vavg[i] = ((double)e * vavg[i] + v[i]) / (double)(e + 1);
                vcov[i] = ((double)e * vcov[i] + v[i] * v[i]) / (double)(e + 1);
            }
        }
    }
}

/* aenet_atomic_energy: aenet.f90:359-408 */
ORC_EXPORT int orc_atomic_energy(const double *coo_i, int type_i, int n_j,
                                 const double *coo_j, const int *type_j,
                                 double *E_i)
{
    if (!g_loaded) return ORC_ERR_INIT;
    if (type_i < 1 || type_i > g_ntypes) return ORC_ERR_TYPE;
    orc_pot *pot = &g_pot[type_i];
    int nvalues = pot->net.nvalues;
    double *sfval = malloc(sizeof(double) * g_nsf_max);
    double *values = malloc(sizeof(double) * (nvalues + 1));
    double *derivs = malloc(sizeof(double) * (nvalues + 1));
    if (!sfval || !values || !derivs) { free(sfval); free(values); free(derivs); return ORC_ERR_MALLOC; }
    int st = stp_eval(type_i, coo_i, n_j, coo_j, type_j, sfval, NULL, NULL, 1);
    if (!st) {
        double y;
        ff_eval(&pot->net, sfval, values, derivs, &y);
        *E_i = pot->E_scale * y + pot->E_shift;
        *E_i = *E_i + pot->E_atom;
    }
    free(sfval); free(values); free(derivs);
    return st;
}

/* aenet_atomic_energy_and_forces: aenet.f90:410-486.  F(3,natoms) is
 * accumulated; index_i and index_j are 1-based. */
ORC_EXPORT int orc_atomic_energy_and_forces(const double *coo_i, int type_i,
                                            int index_i, int n_j,
                                            const double *coo_j,
                                            const int *type_j,
                                            const int *index_j, int natoms,
                                            double *E_i, double *F)
{
    if (!g_loaded) return ORC_ERR_INIT;
    if (type_i < 1 || type_i > g_ntypes) return ORC_ERR_TYPE;
    if (n_j > g_nnb_max) return ORC_ERR_MALLOC;
    orc_pot *pot = &g_pot[type_i];
    int nvalues = pot->net.nvalues, nweights = pot->net.Wsize;
    int nsf = pot->stp.nsf;
    double *dE_dG = malloc(sizeof(double) * g_nsf_max);
    double *sfval = malloc(sizeof(double) * g_nsf_max);
    double *sfderiv_i = malloc(sizeof(double) * 3 * g_nsf_max);
    double *sfderiv_j = malloc(sizeof(double) * 3 * (size_t)g_nsf_max * g_nnb_max);
    double *values = malloc(sizeof(double) * (nvalues + 1));
    double *derivs = malloc(sizeof(double) * (nvalues + 1));
    double *jacobian = malloc(sizeof(double) * nweights);
    int st = ORC_OK;
    if (!dE_dG || !sfval || !sfderiv_i || !sfderiv_j || !values || !derivs || !jacobian) {
        st = ORC_ERR_MALLOC;
        goto done;
    }
    st = stp_eval(type_i, coo_i, n_j, coo_j, type_j, sfval, sfderiv_i, sfderiv_j, 1);
    if (st) goto done;
    double y;
    ff_eval(&pot->net, sfval, values, derivs, &y);
    ff_deriv(&pot->net, derivs, jacobian, dE_dG);
    *E_i = pot->E_scale * y + pot->E_shift;
    *E_i = *E_i + pot->E_atom;
    {
        double m[3];
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < nsf; ++k) s = s + sfderiv_i[3 * k + c] * dE_dG[k];
            m[c] = s;
        }
        for (int c = 0; c < 3; ++c)
            F[3 * (index_i - 1) + c] = F[3 * (index_i - 1) + c] - pot->E_scale * m[c];
        for (int j = 0; j < n_j; ++j) {
            const double *dj = sfderiv_j + (size_t)3 * nsf * j;
            for (int c = 0; c < 3; ++c) {
                double s = 0.0;
                for (int k = 0; k < nsf; ++k) s = s + dj[3 * k + c] * dE_dG[k];
                m[c] = s;
            }
            int idx = index_j[j];
            if (idx < 1 || idx > natoms) { st = ORC_ERR_ARG; goto done; }
            for (int c = 0; c < 3; ++c)
                F[3 * (idx - 1) + c] = F[3 * (idx - 1) + c] - pot->E_scale * m[c];
        }
    }
done:
    free(dE_dG); free(sfval); free(sfderiv_i); free(sfderiv_j);
    free(values); free(derivs); free(jacobian);
    return st;
}

/* Per-atom energy and its weight derivative dE_i/dw (train.f90:893-916:
 * ff_eval, ff_deriv, ff_wderiv), scaled by E_scale. */
ORC_EXPORT int orc_atomic_energy_wgrad(const double *coo_i, int type_i,
                                       int n_j, const double *coo_j,
                                       const int *type_j, double *E_i,
                                       double *dE_dw)
{
    if (!g_loaded) return ORC_ERR_INIT;
    if (type_i < 1 || type_i > g_ntypes) return ORC_ERR_TYPE;
    orc_pot *pot = &g_pot[type_i];
    int nvalues = pot->net.nvalues, nw = pot->net.Wsize;
    double *sfval = malloc(sizeof(double) * g_nsf_max);
    double *values = malloc(sizeof(double) * (nvalues + 1));
    double *derivs = malloc(sizeof(double) * (nvalues + 1));
    double *jac = malloc(sizeof(double) * nw);
    double *dy = malloc(sizeof(double) * g_nsf_max);
    int st = stp_eval(type_i, coo_i, n_j, coo_j, type_j, sfval, NULL, NULL, 1);
    if (!st) {
        double y;
        ff_eval(&pot->net, sfval, values, derivs, &y);
        ff_deriv(&pot->net, derivs, jac, dy);
        ff_wderiv(&pot->net, values, derivs, jac, dE_dw);
        for (int i = 0; i < nw; ++i) dE_dw[i] = pot->E_scale * dE_dw[i];
        *E_i = pot->E_scale * y + pot->E_shift + pot->E_atom;
    }
    free(sfval); free(values); free(derivs); free(jac); free(dy);
    return st;
}

/* ================================================================== */
/*                  linked-cell neighbour list (lclist)               */
/* ================================================================== */

typedef struct {
    int init, natoms, pbc;
    double r_min, r_max;
    double L[9];            /* latticeVec(3,3) column-major */
    double gridVec[9];
    int nCells[3];
    int *cell;              /* head atom per cell, 1-based atom ids, 0 = none */
    int *atomList;          /* next atom in the same cell */
    int *cellList;          /* (3, natoms) */
    int nCvecs, nTvecs;
    int *Cvec, *Tvec;       /* (3, n) */
    double *cooLatt;        /* (3, natoms), wrapped in place */
    const int *atomType;
} orc_lcl;

/* cell volume (lclist.f90:990-1008) */
static double cell_volume(const double *a)
{
#define A(i, j) a[((j) - 1) * 3 + (i) - 1]
    double V = A(1, 1) * A(2, 2) * A(3, 3) + A(2, 1) * A(3, 2) * A(1, 3)
               + A(3, 1) * A(1, 2) * A(2, 3) - A(3, 1) * A(2, 2) * A(1, 3)
               - A(1, 1) * A(3, 2) * A(2, 3) - A(2, 1) * A(1, 2) * A(3, 3);
#undef A
    return fabs(V);
}

/* heights of the cell spanned by the columns of avec: lclist.f90:743-756 */
static void cell_heights(const double *avec, double *h)
{
    double v[3], n;
    vproduct(avec + 0, avec + 3, v);
    n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) v[c] = v[c] / n;
    h[2] = fabs(v[0] * avec[6] + v[1] * avec[7] + v[2] * avec[8]);
    vproduct(avec + 0, avec + 6, v);
    n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) v[c] = v[c] / n;
    h[1] = fabs(v[0] * avec[3] + v[1] * avec[4] + v[2] * avec[5]);
    vproduct(avec + 3, avec + 6, v);
    n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) v[c] = v[c] / n;
    h[0] = fabs(v[0] * avec[0] + v[1] * avec[1] + v[2] * avec[2]);
}

/* inner_sphere: lclist.f90:1014-1048 */
static double inner_sphere(const double *avec)
{
    double h[3];
    cell_heights(avec, h);
    double r = h[2];
    if (h[1] < r) r = h[1];
    if (h[0] < r) r = h[0];
    return 0.5 * r;
}

/* cell_multiples: lclist.f90:725-782 */
static void cell_multiples(double r_max, const double *L, double *gridVec, int *nCells)
{
    double h[3];
    cell_heights(L, h);
    double h_min = h[0];
    if (h[1] < h_min) h_min = h[1];
    if (h[2] < h_min) h_min = h[2];
    if (h_min < 0.5) h_min = 0.5;
    for (int d = 0; d < 3; ++d) {
        int n = (int)floor(h[d] / h_min);
        nCells[d] = n > 1 ? n : 1;
    }
    for (int d = 0; d < 3; ++d)
        for (int c = 0; c < 3; ++c) gridVec[3 * d + c] = L[3 * d + c] / (double)nCells[d];
    double r = inner_sphere(gridVec);
    if (r > 0.5 * r_max) {
        for (int d = 0; d < 3; ++d) nCells[d] = (int)floor(nCells[d] * (2.0 * r / r_max));
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < 3; ++c) gridVec[3 * d + c] = L[3 * d + c] / (double)nCells[d];
    }
}

/* sphere_supercell: lclist.f90:1074-1101 */
static void sphere_supercell(const double *avec, double r, int *n)
{
    const double EPS = 0.001;
    double V = cell_volume(avec);
    double b[3][3];
    /* avec(i,:) rows are taken in the Fortran; row i = (avec(i,1..3)) */
    double r1[3] = {avec[0], avec[3], avec[6]};
    double r2[3] = {avec[1], avec[4], avec[7]};
    double r3[3] = {avec[2], avec[5], avec[8]};
    vproduct(r2, r3, b[0]);
    vproduct(r1, r3, b[1]);
    vproduct(r1, r2, b[2]);
    for (int c = 0; c < 3; ++c) {
        b[0][c] = b[0][c] / V;
        b[1][c] = -b[1][c] / V;
        b[2][c] = b[2][c] / V;
    }
    for (int d = 0; d < 3; ++d) {
        double blen = sqrt(b[d][0] * b[d][0] + b[d][1] * b[d][1] + b[d][2] * b[d][2]);
        n[d] = (int)ceil(r * blen + EPS);
    }
}

static int imodulo(int a, int n) { int m = a % n; return m < 0 ? m + n : m; }

/* cell_from_Cvec: lclist.f90:854-887 (returns 0 in ic[0] if outside) */
static void cell_from_Cvec(const int *ref, const int *cv, const int *nc, int pbc, int *ic)
{
    if (pbc) {
        for (int d = 0; d < 3; ++d) ic[d] = imodulo(ref[d] + cv[d] - 1, nc[d]) + 1;
    } else {
        int out = 0;
        for (int d = 0; d < 3; ++d) {
            ic[d] = ref[d] + cv[d];
            if (ic[d] > nc[d] || ic[d] < 1) out = 1;
        }
        if (out) ic[0] = ic[1] = ic[2] = 0;
    }
}

/* translation_vectors: lclist.f90:1235-1386 */
static int translation_vectors(double Rc, const double *avec, int *nT, int **T,
                               const int *nc, int pbc)
{
    const double EPS = 1.0e-3;
    int n[3];
    sphere_supercell(avec, Rc + EPS, n);
    for (int d = 0; d < 3; ++d) n[d] = (n[d] / 2 + 1) + 1;
    if (nc)
        for (int d = 0; d < 3; ++d) if (nc[d] - 1 < n[d]) n[d] = nc[d] - 1;
    int cap = (2 * n[0] + 1) * (2 * n[1] + 1) * (2 * n[2] + 1);
    if (cap < 1) cap = 1;
    int *T1 = malloc(sizeof(int) * 3 * cap);
    int *cells = malloc(sizeof(int) * 3 * cap);
    if (!T1 || !cells) { free(T1); free(cells); return ORC_ERR_MALLOC; }
    int iT = 0;
    for (int i3 = -n[2]; i3 <= n[2]; ++i3)
        for (int i2 = -n[1]; i2 <= n[1]; ++i2)
            for (int i1 = -n[0]; i1 <= n[0]; ++i1) {
                if (i1 == 0 && i2 == 0 && i3 == 0) continue;
                int Tn[3] = {i1, i2, i3}, ic[3] = {0, 0, 0};
                int redundant = 0;
                if (nc && pbc) {
                    static const int one[3] = {1, 1, 1};
                    cell_from_Cvec(one, Tn, nc, 1, ic);
                    for (int q = 0; q < iT; ++q)
                        if (cells[3 * q] == ic[0] && cells[3 * q + 1] == ic[1]
                            && cells[3 * q + 2] == ic[2]) { redundant = 1; break; }
                }
                if (!redundant) {
                    T1[3 * iT] = i1; T1[3 * iT + 1] = i2; T1[3 * iT + 2] = i3;
                    cells[3 * iT] = ic[0]; cells[3 * iT + 1] = ic[1]; cells[3 * iT + 2] = ic[2];
                    iT++;
                }
            }
    free(cells);
    *nT = iT;
    *T = T1;
    return ORC_OK;
}

/* Image box that provably contains every image within Rc: |T_a| <=
 * ceil(Rc * |b_a|) + 1 with b_a the reciprocal vectors of the columns of
 * L (no 2 PI); same loop order as translation_vectors. */
static int complete_translation_vectors(double Rc, const double *L, int *nT, int **T)
{
    double b[3][3];
    vproduct(L + 3, L + 6, b[0]);
    vproduct(L + 6, L + 0, b[1]);
    vproduct(L + 0, L + 3, b[2]);
    double V = fabs(dot3(L + 0, b[0]));
    int n[3];
    for (int d = 0; d < 3; ++d) {
        double bl = sqrt(dot3(b[d], b[d])) / V;
        n[d] = (int)ceil(Rc * bl) + 1;
    }
    int cap = (2 * n[0] + 1) * (2 * n[1] + 1) * (2 * n[2] + 1);
    int *T1 = malloc(sizeof(int) * 3 * cap);
    if (!T1) return ORC_ERR_MALLOC;
    int iT = 0;
    for (int i3 = -n[2]; i3 <= n[2]; ++i3)
        for (int i2 = -n[1]; i2 <= n[1]; ++i2)
            for (int i1 = -n[0]; i1 <= n[0]; ++i1) {
                if (i1 == 0 && i2 == 0 && i3 == 0) continue;
                T1[3 * iT] = i1; T1[3 * iT + 1] = i2; T1[3 * iT + 2] = i3;
                iT++;
            }
    *nT = iT;
    *T = T1;
    return ORC_OK;
}

ORC_EXPORT void orc_set_complete_candidates(int complete) { g_complete = complete; }

/* wrap_cooLatt: lclist.f90:953-987 */
static void wrap_cooLatt(double *coo, int pbc)
{
    if (!pbc) return;
    for (int d = 0; d < 3; ++d) {
        while (coo[d] < 0.0) coo[d] = coo[d] + 1.0;
        while (coo[d] >= 1.0) coo[d] = coo[d] - 1.0;
    }
}

static void lcl_free(orc_lcl *l)
{
    free(l->cell); free(l->atomList); free(l->cellList);
    free(l->Cvec); free(l->Tvec);
    memset(l, 0, sizeof(*l));
}

#define CELL(l, i1, i2, i3) (l)->cell[(((i1) - 1) * (l)->nCells[1] + ((i2) - 1)) * (l)->nCells[2] + ((i3) - 1)]

/* lcl_init: lclist.f90:99-159 (cooLatt wrapped in place) */
static int lcl_init(orc_lcl *l, double r_min, double r_max, const double *L,
                    int natoms, const int *atomType, double *cooLatt, int pbc)
{
    memset(l, 0, sizeof(*l));
    l->r_min = r_min; l->r_max = r_max; l->natoms = natoms; l->pbc = pbc;
    memcpy(l->L, L, sizeof(double) * 9);
    l->atomType = atomType;
    l->cooLatt = cooLatt;
    cell_multiples(r_max, L, l->gridVec, l->nCells);
    size_t nc = (size_t)l->nCells[0] * l->nCells[1] * l->nCells[2];
    l->cell = calloc(nc, sizeof(int));
    l->atomList = calloc(natoms + 1, sizeof(int));
    l->cellList = calloc((size_t)3 * (natoms + 1), sizeof(int));
    if (!l->cell || !l->atomList || !l->cellList) { lcl_free(l); return ORC_ERR_MALLOC; }
    /* cell_assign_atoms: lclist.f90:692-719; cell_get 833-845; cell_add 893-909 */
    for (int ia = 1; ia <= natoms; ++ia) {
        double *c = cooLatt + 3 * (ia - 1);
        wrap_cooLatt(c, pbc);
        int ic[3];
        for (int d = 0; d < 3; ++d) {
            double x = c[d] * (double)l->nCells[d] + 0.5;
            int v = (int)lround(x);
            ic[d] = v < l->nCells[d] ? v : l->nCells[d];
            if (ic[d] < 1) ic[d] = 1;   /* isolated structures outside the box */
        }
        l->atomList[ia] = CELL(l, ic[0], ic[1], ic[2]);
        CELL(l, ic[0], ic[1], ic[2]) = ia;
        for (int d = 0; d < 3; ++d) l->cellList[3 * ia + d] = ic[d];
    }
    int st = translation_vectors(r_max, l->gridVec, &l->nCvecs, &l->Cvec, l->nCells, pbc);
    if (st) { lcl_free(l); return st; }
    if (pbc) {
        if (g_complete)
            st = complete_translation_vectors(r_max + 1.0e-3, L, &l->nTvecs, &l->Tvec);
        else
            st = translation_vectors(r_max, L, &l->nTvecs, &l->Tvec, NULL, 1);
        if (st) { lcl_free(l); return st; }
    }
    l->init = 1;
    return ORC_OK;
}

/* lcl_nblist: lclist.f90:281-376 (without a capacity limit) */
static int lcl_nblist(const orc_lcl *l, int iatom, int *nblist)
{
    if (g_complete) {
        int inb = 0;
        for (int ia = 1; ia <= l->natoms; ++ia)
            if (ia != iatom) nblist[inb++] = ia;
        return inb;
    }
    int ic0[3] = {l->cellList[3 * iatom], l->cellList[3 * iatom + 1], l->cellList[3 * iatom + 2]};
    int inb = 0;
    int iat = CELL(l, ic0[0], ic0[1], ic0[2]);
    if (iat != 0) {
        if (iat != iatom) nblist[inb++] = iat;
        while (l->atomList[iat] != 0) {
            iat = l->atomList[iat];
            if (iat == iatom) continue;
            nblist[inb++] = iat;
        }
    }
    for (int iv = 0; iv < l->nCvecs; ++iv) {
        int ic[3];
        cell_from_Cvec(ic0, l->Cvec + 3 * iv, l->nCells, l->pbc, ic);
        if (ic[0] < 1 || ic[1] < 1 || ic[2] < 1) continue;
        iat = CELL(l, ic[0], ic[1], ic[2]);
        if (iat != 0) {
            int dup = 0;
            for (int q = 0; q < inb; ++q) if (nblist[q] == iat) { dup = 1; break; }
            if (!dup) nblist[inb++] = iat;
            while (l->atomList[iat] != 0) {
                iat = l->atomList[iat];
                dup = 0;
                for (int q = 0; q < inb; ++q) if (nblist[q] == iat) { dup = 1; break; }
                if (!dup) nblist[inb++] = iat;
            }
        }
    }
    return inb;
}

/* lcl_nbdist_cart: lclist.f90:520-677.  Output arrays are sized by the
 * caller with capacity cap; returns the neighbour count or -1 on overflow. */
static int lcl_nbdist_cart(const orc_lcl *l, int iatom, int cap, int *cand,
                           double *nbcoo, double *nbdist, int *nblist,
                           int *nbtype, double Rc)
{
    const double EPS = 1.0e-3;
    double Rc2 = (Rc + EPS) * (Rc + EPS);
    int nc = lcl_nblist(l, iatom, cand);
    int nnb = 0;
    const double *si = l->cooLatt + 3 * (iatom - 1);
    for (int iT = 0; iT < l->nTvecs; ++iT) {
        double Td[3] = {(double)l->Tvec[3 * iT], (double)l->Tvec[3 * iT + 1], (double)l->Tvec[3 * iT + 2]};
        double cart[3];
        matvec3(l->L, Td, cart);
        double dist2 = dot3(cart, cart);
        if (dist2 <= Rc2) {
            if (nnb >= cap) return -1;
            nblist[nnb] = iatom;
            nbtype[nnb] = l->atomType[iatom - 1];
            double s[3] = {si[0] + Td[0], si[1] + Td[1], si[2] + Td[2]};
            matvec3(l->L, s, nbcoo + 3 * nnb);
            nbdist[nnb] = sqrt(dist2);
            nnb++;
        }
    }
    double coo1[3];
    matvec3(l->L, si, coo1);
    for (int q = 0; q < nc; ++q) {
        int iat = cand[q];
        const double *sj = l->cooLatt + 3 * (iat - 1);
        double coo2[3], cart[3];
        matvec3(l->L, sj, coo2);
        for (int c = 0; c < 3; ++c) cart[c] = coo2[c] - coo1[c];
        double dist2 = dot3(cart, cart);
        if (dist2 <= Rc2) {
            if (nnb >= cap) return -1;
            nblist[nnb] = iat;
            nbtype[nnb] = l->atomType[iat - 1];
            memcpy(nbcoo + 3 * nnb, coo2, sizeof(coo2));
            nbdist[nnb] = sqrt(dist2);
            nnb++;
        }
        for (int iT = 0; iT < l->nTvecs; ++iT) {
            double s[3];
            for (int c = 0; c < 3; ++c) s[c] = sj[c] + (double)l->Tvec[3 * iT + c];
            matvec3(l->L, s, coo2);
            for (int c = 0; c < 3; ++c) cart[c] = coo2[c] - coo1[c];
            dist2 = dot3(cart, cart);
            if (dist2 <= Rc2) {
                if (nnb >= cap) return -1;
                nblist[nnb] = iat;
                nbtype[nnb] = l->atomType[iat - 1];
                memcpy(nbcoo + 3 * nnb, coo2, sizeof(coo2));
                nbdist[nnb] = sqrt(dist2);
                nnb++;
            }
        }
    }
    return nnb;
}

/* The neighbour-list API of aenet.f90:571-639 (aenet_nbl_init/neighbors):
 * lattice coordinates in, wrapped in place. */
static orc_lcl g_lcl;
static double *g_lcl_coo = NULL;
static int *g_lcl_types = NULL;
static int *g_lcl_cand = NULL;

ORC_EXPORT int orc_nbl_init(const double *L, int natoms, const int *types,
                            const double *cooLatt, int pbc, double r_min,
                            double r_max)
{
    if (g_lcl.init) lcl_free(&g_lcl);
    free(g_lcl_coo); free(g_lcl_types); free(g_lcl_cand);
    g_lcl_coo = malloc(sizeof(double) * 3 * natoms);
    g_lcl_types = malloc(sizeof(int) * natoms);
    g_lcl_cand = malloc(sizeof(int) * (natoms + 1));
    if (!g_lcl_coo || !g_lcl_types || !g_lcl_cand) return ORC_ERR_MALLOC;
    memcpy(g_lcl_coo, cooLatt, sizeof(double) * 3 * natoms);
    memcpy(g_lcl_types, types, sizeof(int) * natoms);
    return lcl_init(&g_lcl, r_min, r_max, L, natoms, g_lcl_types, g_lcl_coo, pbc);
}

ORC_EXPORT int orc_nbl_neighbors(int iatom, int cap, double *nbcoo,
                                 double *nbdist, int *nblist, int *nbtype,
                                 double Rc)
{
    if (!g_lcl.init) return -2;
    return lcl_nbdist_cart(&g_lcl, iatom, cap, g_lcl_cand, nbcoo, nbdist,
                           nblist, nbtype, Rc);
}

ORC_EXPORT void orc_nbl_wrapped(double *cooLatt)
{
    if (g_lcl.init) memcpy(cooLatt, g_lcl_coo, sizeof(double) * 3 * g_lcl.natoms);
}

ORC_EXPORT void orc_nbl_final(void)
{
    if (g_lcl.init) lcl_free(&g_lcl);
    free(g_lcl_coo); free(g_lcl_types); free(g_lcl_cand);
    g_lcl_coo = NULL; g_lcl_types = NULL; g_lcl_cand = NULL;
}

/* ================================================================== */
/*                 structure driver (predict.x get_energy)            */
/* ================================================================== */

/* geo_recip_lattice (geometry.f90:491-516) and the conversion of
 * geo_init_xsf (geometry.f90:697-712): cooLatt = (B cart)/(2 PI) with B
 * the reciprocal lattice including the factor 2 PI. */
ORC_EXPORT void orc_cart_to_latt(const double *L, int natoms, const double *cart,
                                 double *cooLatt)
{
#define A(i, j) L[((j) - 1) * 3 + (i) - 1]
    double a1[3] = {A(1, 1), A(2, 1), A(3, 1)};
    double a2[3] = {A(1, 2), A(2, 2), A(3, 2)};
    double a3[3] = {A(1, 3), A(2, 3), A(3, 3)};
    double V = A(1, 1) * A(2, 2) * A(3, 3) + A(2, 1) * A(3, 2) * A(1, 3)
               + A(3, 1) * A(1, 2) * A(2, 3) - A(3, 1) * A(2, 2) * A(1, 3)
               - A(1, 1) * A(3, 2) * A(2, 3) - A(2, 1) * A(1, 2) * A(3, 3);
#undef A
    double b1[3], b2[3], b3[3];
    vproduct(a2, a3, b1);
    vproduct(a1, a3, b2);
    vproduct(a1, a2, b3);
    double B[9]; /* bvec(3,3) column-major: bvec(i,:) = row i */
    for (int c = 0; c < 3; ++c) {
        B[c * 3 + 0] = (b1[c] / V) * 2.0 * CONST_PI;
        B[c * 3 + 1] = (-b2[c] / V) * 2.0 * CONST_PI;
        B[c * 3 + 2] = (b3[c] / V) * 2.0 * CONST_PI;
    }
    for (int i = 0; i < natoms; ++i) {
        double s[3];
        matvec3(B, cart + 3 * i, s);
        for (int c = 0; c < 3; ++c) cooLatt[3 * i + c] = s[c] / (2.0 * CONST_PI);
    }
}

/* geo_get_bounds (geometry.f90:538-582): bounding box of an isolated
 * structure; cart is shifted in place, L receives the box. */
ORC_EXPORT void orc_bounding_box(int natoms, double *cart, double *L)
{
    const double EPS = 2.0e-6;
    double mn[3], mx[3];
    for (int c = 0; c < 3; ++c) { mn[c] = cart[c]; mx[c] = cart[c]; }
    for (int i = 1; i < natoms; ++i)
        for (int c = 0; c < 3; ++c) {
            if (cart[3 * i + c] < mn[c]) mn[c] = cart[3 * i + c];
            if (cart[3 * i + c] > mx[c]) mx[c] = cart[3 * i + c];
        }
    memset(L, 0, sizeof(double) * 9);
    for (int c = 0; c < 3; ++c) L[c * 3 + c] = mx[c] - mn[c] + EPS;
    for (int i = 0; i < natoms; ++i)
        for (int c = 0; c < 3; ++c) cart[3 * i + c] = cart[3 * i + c] - (mn[c] - 0.5 * EPS);
}

/* get_energy: predict.F90:574-706.  L(3,3) column-major lattice vectors,
 * cart(3,natoms) Cartesian input (periodic) or any Cartesian frame
 * (isolated: a bounding box is built as geo_init_xsf does).  F(3,natoms)
 * and E_atoms(natoms) optional.  nthreads > 1 splits the atom loop over
 * OpenMP threads with per-thread force buffers (the MPI split of
 * predict.F90:632 done with threads). */
ORC_EXPORT int orc_structure_energy_forces(const double *L_in, int natoms,
                                           const double *cart_in,
                                           const int *types, int pbc,
                                           int nthreads, int atom_limit,
                                           double *Ecoh, double *Etot,
                                           double *F, double *E_atoms)
{
    if (!g_loaded) return ORC_ERR_INIT;
    double L[9];
    double *cart = malloc(sizeof(double) * 3 * natoms);
    double *cooLatt = malloc(sizeof(double) * 3 * natoms);
    if (!cart || !cooLatt) { free(cart); free(cooLatt); return ORC_ERR_MALLOC; }
    memcpy(cart, cart_in, sizeof(double) * 3 * natoms);
    if (pbc) memcpy(L, L_in, sizeof(double) * 9);
    else orc_bounding_box(natoms, cart, L);
    orc_cart_to_latt(L, natoms, cart, cooLatt);
    orc_lcl l;
    int st = lcl_init(&l, g_Rc_min, g_Rc_max, L, natoms, types, cooLatt, pbc);
    if (st) { free(cart); free(cooLatt); return st; }
    int nat_eval = (atom_limit > 0 && atom_limit < natoms) ? atom_limit : natoms;
    double ecoh = 0.0, etot = 0.0;
    if (F) memset(F, 0, sizeof(double) * 3 * natoms);
    if (nthreads < 1) nthreads = 1;
    int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+:ecoh, etot)
#endif
    {
        int cap = g_nnb_max;
        int *cand = malloc(sizeof(int) * (natoms + 1));
        int *nblist = malloc(sizeof(int) * cap);
        int *nbtype = malloc(sizeof(int) * cap);
        double *nbcoo = malloc(sizeof(double) * 3 * cap);
        double *nbdist = malloc(sizeof(double) * cap);
        double *Floc = F ? calloc((size_t)3 * natoms, sizeof(double)) : NULL;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int ia = 1; ia <= nat_eval; ++ia) {
            int type_i = types[ia - 1];
            double coo_i[3];
            matvec3(L, cooLatt + 3 * (ia - 1), coo_i);
            int nnb = lcl_nbdist_cart(&l, ia, cap, cand, nbcoo, nbdist, nblist, nbtype, g_Rc_max);
            if (nnb < 0) { err = ORC_ERR_MALLOC; continue; }
            double E_i = 0.0;
            int s;
            if (F) s = orc_atomic_energy_and_forces(coo_i, type_i, ia, nnb, nbcoo, nbtype, nblist, natoms, &E_i, Floc);
            else s = orc_atomic_energy(coo_i, type_i, nnb, nbcoo, nbtype, &E_i);
            if (s) { err = s; continue; }
            etot = etot + E_i;
            ecoh = ecoh + E_i - g_pot[type_i].E_atom;
            if (E_atoms) E_atoms[ia - 1] = E_i;
        }
        if (F) {
#ifdef _OPENMP
#pragma omp critical
#endif
            for (size_t q = 0; q < (size_t)3 * natoms; ++q) F[q] += Floc[q];
        }
        free(cand); free(nblist); free(nbtype); free(nbcoo); free(nbdist); free(Floc);
    }
    lcl_free(&l);
    free(cart); free(cooLatt);
    *Ecoh = ecoh;
    *Etot = etot;
    return err;
}

/* Chebyshev basis without potentials: aenet_sfb_init / aenet_sfb_eval
 * (aenet.f90:652-771) and aenet_sfb_reconstruct_radial (773-799,
 * sfbasis.f90:581-637). */
static orc_sfb g_sfb_free;

ORC_EXPORT int orc_sfb_init(int ntypes, int radial_order, int angular_order,
                            double radial_Rc, double angular_Rc)
{
    if (g_sfb_free.init) return ORC_ERR_INIT;
    if (ntypes < 1 || ntypes > MAXT) return ORC_ERR_ARG;
    new_sfb(&g_sfb_free, ntypes, radial_order, angular_order, radial_Rc, angular_Rc);
    return ORC_OK;
}

ORC_EXPORT int orc_sfb_final(void)
{
    if (!g_sfb_free.init) return ORC_ERR_INIT;
    g_sfb_free.init = 0;
    return ORC_OK;
}

ORC_EXPORT int orc_sfb_nvalues(void) { return g_sfb_free.init ? g_sfb_free.N : 0; }

ORC_EXPORT int orc_sfb_eval(int itype0, const double *coo0, int nat,
                            const int *itype1, const double *coo1, int nv,
                            double *values, double *deriv0, double *deriv1)
{
    (void)itype0;
    if (!g_sfb_free.init) return ORC_ERR_INIT;
    return sfb_eval(&g_sfb_free, coo0, nat, itype1, coo1, nv, values, deriv0, deriv1);
}

ORC_EXPORT int orc_sfb_reconstruct_radial(const double *coeff, int nx, double *x, double *y)
{
    if (!g_sfb_free.init) return ORC_ERR_INIT;
    const orc_sfb *sfb = &g_sfb_free;
    double f[64];
    double dx = sfb->r_Rc / (double)(nx - 1);
    for (int ix = 0; ix < nx; ++ix) x[ix] = (double)ix * dx;
    for (int ix = 0; ix < nx - 1; ++ix) {
        cheb_T(x[ix], 0.0, sfb->r_Rc, sfb->r_order, f);
        double r = x[ix] / sfb->r_Rc;
        double w = 0.5 / sqrt(r - r * r);
        for (int i = 0; i < sfb->r_N; ++i) f[i] = f[i] * w * (1.0 / SFB_PI);
        f[0] = 0.5f * f[0];
        y[ix] = 0.0;
        for (int ic = sfb->r_N - 1; ic >= 0; --ic) y[ix] = y[ix] + coeff[ic] * f[ic];
    }
    y[nx - 1] = 0.0;
    return ORC_OK;
}
