/*
 * nmmodel.h -- synthetic planet models and the continuous-Galerkin FEM
 * assembly that produces the CSR operators consumed by the eigensolver.
 *
 * This is the input side of the eigensolve path: it plays the role of the
 * reference's geometry / model / assembly layers and hands the eigensolver
 * exactly the matrices the reference hands pEVSL:
 *
 *   solid-only model   : A, B            (src/mod_cg_create_matrix.f90:980-1266,
 *                                          structure :1269-1455)
 *   fluid-solid model  : Ad, B, Ap, E, ET (src/mod_cg_create_matrix.f90:103-977,
 *                                          structure :1458-2033)
 *
 * All CSR arrays are 0-based (int32 row pointers and columns, float64 values),
 * rows sorted by column, i.e. the layout `setupmatvec` passes to
 * PEVSL_PARCSRCREATE_F90 after `col-1` (src/mod_matvec.f90:59,112,136,189,215,239).
 * Ap is returned with the reference's sign (negative definite); the solver
 * negates it itself as src/mod_matvec.f90:137 does.
 *
 * Every entry point returns 0 on success and a negative NMM_ERR_* code on
 * failure; nmm_last_error() gives the message.
 */
#ifndef NMMODEL_H
#define NMMODEL_H

#ifdef __cplusplus
extern "C" {
#endif

#define NMM_OK 0
#define NMM_ERR_ARG (-1)
#define NMM_ERR_MESH (-2)
#define NMM_ERR_IO (-3)
#define NMM_ERR_STATE (-4)

/* Matrix selectors for nmm_get_csr. */
#define NMM_MAT_A 0  /* solid-only stiffness (CGM%A)             */
#define NMM_MAT_B 1  /* mass (CGM%B)                              */
#define NMM_MAT_AD 2 /* displacement stiffness, fluid-solid path  */
#define NMM_MAT_AP 3 /* pressure block (negative), fluid-solid    */
#define NMM_MAT_E 4  /* displacement x pressure coupling          */
#define NMM_MAT_ET 5 /* pressure x displacement coupling          */

typedef struct nmm_model nmm_model;

/* Layered-ball generator options.  Radii in km, velocities in km/s, density
 * in g/cm^3 (the reference's model units, src/mod_cg_models.f90:49-51). */
typedef struct {
  int n_cells;           /* cube cells per axis, even (ball from n^3*6 tets) */
  int porder;            /* 1 or 2 (pOrder in global_conf)                  */
  double radius;         /* outer radius, default 6371                      */
  double r_icb;          /* inner-core boundary radius, default 1221        */
  double r_cmb;          /* core-mantle boundary radius, default 3480       */
  double jitter;         /* interior-node jitter, fraction of local edge    */
  unsigned long long seed;
  int fluid_core;        /* 1: outer core fluid (Vs = 0); 0: all solid      */
  int homogeneous;       /* 1: constant vp0/vs0/rho0 everywhere             */
  double vp0, vs0, rho0; /* used when homogeneous                           */
  double lateral_pert;   /* e.g. 0.02 for +-2 % lateral perturbation        */
  int lateral_lmax;      /* spherical-harmonic degree of the perturbation   */
} nmm_ball_opts;

typedef struct {
  int porder, pnp, nfp;
  int nvert, ntet, nnode; /* nnode = vertices (+ edge nodes for P2)        */
  int n_fluid_tets;
  int fsexist, purefluid; /* src/mod_geometry.f90:329-341                   */
  int n;                  /* displacement DOFs (B%Gsiz)                     */
  int np;                 /* pressure DOFs (Ap%Gsiz), 0 if no fluid         */
  long long nnz[6];       /* per NMM_MAT_*, 0 if absent                     */
  int assembled;
} nmm_info_t;

/* Fill defaults: 6371/1221/3480 km, jitter 0.1, fluid core, PREM-like
 * piecewise-linear profile, no lateral perturbation. */
void nmm_ball_default_opts(nmm_ball_opts* o);

/* Build the layered ball mesh and per-element nodal material. */
int nmm_ball_create(const nmm_ball_opts* o, nmm_model** out);

/* Load a model in the reference's binary input format: <base>_mesh.header
 * (text "Ntet Nvert"), <base>_ele.dat (int32 Ntet x 4, 1-based),
 * <base>_node.dat (float64 Nvert x 3), <base>_{vp,vs,rho}_pod_<p>_true.dat
 * (float64 Ntet x pNp) -- src/mod_geometry.f90:83-425,
 * src/mod_cg_models.f90:301-364. */
int nmm_load_files(const char* base_path, int porder, nmm_model** out);

/* Assemble the CSR operators: JOB = 1 without gravity, JOB = 2 (reference
 * gravity, src/mod_para.f90:133-138) once a gravity field is set. */
int nmm_assemble(nmm_model* m);

/* Reference gravity (JOB = 2): the gravitational acceleration at every
 * element node, float64 Ntet x pNp x 3 in m/s^2 (pointing inwards), the
 * layout of <base>_pod_<p>_potential_acceleration_true.dat
 * (src/mod_cg_models.f90:366-429).  Copied; NULL switches gravity off
 * (JOB = 1).  Either way the model is marked for re-assembly. */
int nmm_set_gravity(nmm_model* m, const double* g0);

/* Read <base>_pod_<p>_potential_acceleration_true.dat and set it. */
int nmm_load_gravity(nmm_model* m, const char* base_path);

/* Reference gravity of a generated ball from its radial density profile
 * (the lateral perturbation has zero mean on every sphere):
 * g = -G M(r) x / r^3, G in m^3 kg^-1 s^-2 (6.6723e-11 reproduces the
 * reference's demo gravity files).  NMM_ERR_STATE for loaded models. */
int nmm_ball_gravity(nmm_model* m, double G);

/* Write the model in the reference's input files under base_path (the files
 * nmm_load_files and nmm_load_gravity read): _mesh.header, _ele.dat,
 * _node.dat, _neigh.dat (int32 Ntet x 4, the tetrahedron opposite each
 * vertex, 1-based, -1 on the boundary), _{vp,vs,rho}_pod_<p>_true.dat and,
 * when set, the gravity file.  Vertices are numbered by increasing node id
 * among the vertex nodes (the model's own numbering for P1). */
int nmm_write_model_files(const nmm_model* m, const char* base_path);

/* The gravity field (borrowed, 3 pNp Ntet values) or NULL when off. */
int nmm_get_gravity(const nmm_model* m, const double** g0);

int nmm_info(const nmm_model* m, nmm_info_t* info);

/* Borrowed pointers into the model (valid until nmm_destroy). */
int nmm_get_csr(const nmm_model* m, int which, const int** rowptr, const int** col,
                const double** val, int* nrows, int* ncols, long long* nnz);

/* Mesh arrays (borrowed): node xyz (3*nnode), tet node lists (pnp*ntet, local
 * node order of the reference element), fluid flags (ntet), node status
 * (nnode, vstat codes 0..5 of src/mod_geometry.f90:301-310,672-680),
 * per-node first displacement DOF (vstt), DOF count (rnum 3|6), first
 * pressure DOF (pstt, -1 if none), and per-element nodal material
 * (pnp*ntet each). */
int nmm_mesh_arrays(const nmm_model* m, const double** xyz, const int** tets,
                    const unsigned char** fluid, const int** vstat, const int** vstt,
                    const int** rnum, const int** pstt, const double** vp,
                    const double** vs, const double** rho);

/* Replace the per-element nodal material (pnp*ntet values each, copied) and
 * mark the model for re-assembly.  The solid / fluid classification of every
 * element must stay as it is (NMM_ERR_ARG otherwise). */
int nmm_set_material(nmm_model* m, const double* vp, const double* vs, const double* rho);

/* Element matrices of tet k exactly as the assembly scatters them:
 * solid: TM, MM are (3 pnp)^2 row-major; fluid: FT, FM are (3 pnp + pnp)^2.
 * *dim receives the matrix dimension. */
int nmm_element_matrices(const nmm_model* m, int k, double* T, double* M, int* dim);

/* Reference element (borrowed, row-major pnp x pnp; drst is 3 x pnp x pnp;
 * massf is 4 x nfp x nfp; fmask 4 x nfp 0-based). */
int nmm_reference(const nmm_model* m, const double** nodes_rst, const double** massm,
                  const double** drst, const double** massf, const int** fmask);

/* Write eigenvectors / vertex lists in the reference's output formats
 * (src/mod_pevsl.f90:188-201,225-247): raw float64 per vector. */
int nmm_write_vector(const char* path, const double* x, long long n);

/* The reference's result files (src/mod_pevsl.f90:188-247, names of
 * src/mod_para.f90:269-288):
 *   <outputdir><basename>_JOB<job>_pod<p>_np<nproc>_<low>_<up>_<i>.dat
 *       eigenvector i (1-based), raw float64, n values in DOF order;
 *   <outputdir><basename>_pod<p>_np<nproc>_vlist.dat
 *       int32 per node in DOF order: its 1-based id in the input numbering
 *       (vertices of _node.dat, then P2 edge nodes);
 *   <outputdir><basename>_pod<p>_np<nproc>_vstat.dat (fluid-solid models)
 *       int32 node status (vstat codes 0..5).
 * <low>/<up> are the frequencies as the reference writes REAL(4) values
 * (gfortran list-directed).  X is n x nev column-major with leading
 * dimension ldx (unscaled eigenvectors).  The eigenvector file prefix is
 * copied to prefix_out (may be NULL). */
int nmm_write_results(const nmm_model* m, const char* outputdir, const char* basename, int job, int nproc,
                      double lowfreq, double upfreq, int nev, const double* X, long long ldx, char* prefix_out,
                      int prefix_len);

const char* nmm_last_error(void);
void nmm_destroy(nmm_model* m);

#ifdef __cplusplus
}
#endif
#endif
