/*
 * aenet.h -- drop-in replacement of aenet's libaenet C API.
 *
 * Same symbols, signatures, status codes and semantics as the reference
 * header src/aenet.h:1-52 (implementation src/aenet.f90), served by
 * libaenet_gb300.so whose evaluation runs on the GPU.  Type ids are 1-based
 * in aenet_init order, forces are accumulated into the caller's array,
 * energies include the free-atom energy, coordinates are Cartesian
 * Angstrom, energies eV.  No function aborts the process: every failure is
 * reported through *stat.
 */
#ifndef AENET_H_INCLUDED
#define AENET_H_INCLUDED

#ifdef __cplusplus
#ifndef _Bool
#define _Bool bool
#endif
extern "C" {
#endif

/* src/aenet.h:4, src/aenet.f90:171-193 -- AENET_ERR_INIT if already
 * initialised; type names are at most AENET_TYPELEN characters. */
void aenet_init(int ntypes, char* atom_types[], int* stat);

/* src/aenet.h:5, src/aenet.f90:197-222 -- releases host and device state. */
void aenet_final(int* stat);

/* src/aenet.h:6, src/aenet.f90:228-244 */
void aenet_print_info(void);

/* src/aenet.h:7, src/aenet.f90:250-314 -- loads a .nn file (same format)
 * for 1-based type_id; when the last one is loaded, Rc_min/Rc_max,
 * nnb_max and nsf_max are set and the device tables are built. */
void aenet_load_potential(int type_id, char* filename, int* stat);

/* src/aenet.h:8, src/aenet.f90:316-331 */
_Bool aenet_all_loaded(void);

/* src/aenet.h:10, src/aenet.f90:337-346 (by value, as the header states) */
double aenet_free_atom_energy(int type_id);

/* src/aenet.h:12-14, src/aenet.f90:359-408 -- energy of one atom from its
 * neighbours (Cartesian coo_j[3*n_j], 1-based type_j).  FP64 on the GPU;
 * on Chebyshev potentials one kernel launch per call (the row read from
 * and the results written to mapped host memory), otherwise the batch
 * kernels on a one-row table (option "per_atom_kernel",
 * include/aenet_gb300.h).  Calls are serialised by a library lock. */
void aenet_atomic_energy(double coo_i[3], int type_i, int n_j,
                         double coo_j[], int type_j[], double* E_i,
                         int* stat);

/* src/aenet.h:16-19, src/aenet.f90:410-486 -- energy of one atom and the
 * force contributions of that energy, accumulated into F[natoms][3] at the
 * 1-based indices index_i and index_j[]. */
void aenet_atomic_energy_and_forces(double coo_i[3], int type_i, int index_i,
                                    int n_j, double coo_j[], int type_j[],
                                    int index_j[], int natoms, double* E_i,
                                    double F[], int* stat);

/* src/aenet.h:21-23, src/aenet.f90:492-553 */
void aenet_convert_atom_types(int ntypes_in, char* atom_types[],
                              int natoms_in, int type_id_in[],
                              int type_id_out[], int* stat);

/* src/aenet.h:25-37, src/aenet.f90:652-799 -- stand-alone Chebyshev basis */
void aenet_sfb_init(int ntypes, char* atom_types[], int radial_order,
                    int angular_order, double radial_Rc, double angular_Rc,
                    int* stat);
void aenet_sfb_final(int* stat);
int aenet_sfb_nvalues(void);
void aenet_sfb_eval(int itype0, double coo0[3], int nat, int itype1[],
                    double coo1[], int nv, double values[], int* stat);
void aenet_sfb_reconstruct_radial(int nv, double values[], int nx,
                                  double x[], double y[], int* stat);

/* src/aenet.f90:571-639 (exported without a prototype in the reference
 * header) -- linked-cell neighbour list; aenet_nbl_init overwrites coords
 * with the Cartesian coordinates of the wrapped lattice coordinates. */
void aenet_nbl_init(double latt_vec[9], int natoms, int atom_types[],
                    double coords[], _Bool cartesian, _Bool pbc);
void aenet_nbl_final(void);
void aenet_nbl_neighbors(int iatom, int* nnb, double nbcoo[],
                         double nbdist[], int nblist[], int nbtype[]);

/* src/aenet.f90:101-118, src/aenet.h:39-50 */
extern int AENET_OK;
extern int AENET_ERR_INIT;
extern int AENET_ERR_MALLOC;
extern int AENET_ERR_IO;
extern int AENET_ERR_TYPE;
extern int AENET_TYPELEN;
extern int AENET_PATHLEN;
extern _Bool AENET_TRUE;
extern _Bool AENET_FALSE;

extern int aenet_nsf_max;
extern int aenet_nnb_max;
extern double aenet_Rc_min;
extern double aenet_Rc_max;

#ifdef __cplusplus
}
#endif

#endif
