/*
 * atomistica_gb300 — C-ABI of the GB300-native per-step force path.
 *
 * Drop-in replacement for the ISO_C_BINDING shims that Atomistica generates
 * for every potential (src/python/gen_factory.py:98-356, C prototypes
 * :380-401, function table src/python/c/factory.template.h:36-52) and for the
 * particles / neighbour-list objects they operate on
 * (src/python/f90/particles_wrap.f90, src/python/f90/neighbors_wrap.f90).
 *
 * Conventions kept from the reference:
 *   - every call returns an int error code; 0 = ERROR_NONE, negative = error
 *     (src/support/error.f90:81-86); the message is available from
 *     gb_get_error() (the reference pushes it on its error stack and converts
 *     it with error_to_py, src/python/c/py_f.c:36);
 *   - `epot` is set (zeroed, then accumulated; gen_factory.py:283), while `f`,
 *     `wpot` and every optional per-atom / per-bond output are ACCUMULATED into
 *     (the caller zeroes them, src/python/c/potential.c:468-479);
 *   - array layouts are those the Python extension hands to Fortran:
 *     positions and forces (nat,3) C-order (= Fortran (3,nat)); cell rows are
 *     the lattice vectors (particles.c:436-461); wpot is Fortran (3,3)
 *     (element (a,c) at wpot[a + 3c]); wpot_per_at / wpot_per_bond are Fortran
 *     (3,3,n) (element (a,c,i) at [a + 3c + 9i]); f_per_bond is (n,3);
 *   - optional outputs are NULL when not requested; a potential that does not
 *     support one (EAM: per-bond) returns an error (gen_factory.py:302-351);
 *   - per-bond arrays are indexed by the compact neighbour-list entry, in the
 *     order of gb_neighbors_get (the reference's f_pack_per_bond_* order,
 *     neighbors_wrap.f90:498-547).
 *
 * Pointers may be host or device (CUDA) memory; device pointers are used in
 * place, host pointers are staged through pinned buffers.  All device work
 * of one object runs on its CUDA stream (gb_*_set_stream).  Calls on one
 * handle are not re-entrant (as in the reference, tls.f90:45-49).
 *
 * There is no CPU fallback: without a CUDA device every compute entry point
 * returns GB_ERROR_CUDA.
 */
#ifndef ATOMISTICA_GB300_H
#define ATOMISTICA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes (src/support/error.f90:81-86 plus this library's own). */
#define GB_ERROR_NONE 0
#define GB_ERROR_UNSPECIFIED (-1)
#define GB_ERROR_FILE_NOT_FOUND (-2)
#define GB_ERROR_IO (-3)
#define GB_ERROR_IO_EOF (-4)
#define GB_ERROR_CUDA (-10)
#define GB_ERROR_ARGUMENT (-11)
#define GB_ERROR_CAPACITY (-12)
#define GB_ERROR_DOMAIN (-13)

/* Precision forms of the BOP kernels. */
#define GB_PRECISION_FP64 0  /* drop-in: FP64 throughout */
#define GB_PRECISION_MIXED 1 /* FP32 bond arithmetic, FP64 accumulation */

/* Flags of gb_potential_energy_and_forces_flags. */
#define GB_FORCES_SET 1 /* f is set to the forces instead of accumulated into */

typedef struct gb_particles gb_particles_t;
typedef struct gb_neighbors gb_neighbors_t;
typedef struct gb_potential gb_potential_t;
typedef struct gb_batch gb_batch_t;

/* Last error message of the calling thread ("" if none). */
const char *gb_get_error(void);
/* Library version string. */
const char *gb_version(void);
/* Number of CUDA devices visible (0 without a GPU). */
int gb_device_count(void);

/* ------------------------------------------------------------------------
 * Particles — replaces particles_t (src/python/f90/python_particles.f90:85-140)
 * and its Python binding (src/python/c/particles.c).
 * ---------------------------------------------------------------------- */
/* particles_new (particles_wrap.f90) */
int gb_particles_new(gb_particles_t **p);
void gb_particles_free(gb_particles_t *p);
/* particles_allocate (python_particles.f90:524-555) */
int gb_particles_allocate(gb_particles_t *p, int nat);
int gb_particles_get_nat(const gb_particles_t *p);
/* particles_set_cell (python_particles.f90:286-346): cell rows = lattice
 * vectors (3x3 row-major), pbc[3] nonzero = periodic. */
int gb_particles_set_cell(gb_particles_t *p, const double *cell, const int *pbc);
/* Writes the coordinates (nat,3) and marks positions changed
 * (I_changed_positions, python_particles.f90:768-777). */
int gb_particles_set_positions(gb_particles_t *p, const double *r);
/* Atomic numbers (nat); update_elements (python_particles.f90:617-658). */
int gb_particles_set_Z(gb_particles_t *p, const int *Z);
/* Stream used for the particles' uploads (NULL = a stream owned by p). */
int gb_particles_set_stream(gb_particles_t *p, void *cuda_stream);

/* ------------------------------------------------------------------------
 * Neighbour list — replaces neighbors_t (python_neighbors.f90:51-139).
 * ---------------------------------------------------------------------- */
/* neighbors_new(avgn) (neighbors_wrap.f90) */
int gb_neighbors_new(gb_neighbors_t **nl, int avgn);
void gb_neighbors_free(gb_neighbors_t *nl);
/* request_interaction_range (python_neighbors.f90:381-403) */
int gb_neighbors_request_interaction_range(gb_neighbors_t *nl, double cutoff);
double gb_neighbors_get_interaction_range(const gb_neighbors_t *nl);
/* neighbors_update (python_neighbors.f90:430-456): rebuilds the full
 * directed list if positions or cell changed. */
int gb_neighbors_update(gb_neighbors_t *nl, gb_particles_t *p);
/* Number of list entries after the last update (get_number_of_all_neighbors). */
int64_t gb_neighbors_get_size(const gb_neighbors_t *nl);
/* Copies the list (f_get_all_neighbors, neighbors_wrap.f90:425-455):
 * seed (nat+1 CSR offsets, int64), j (n, 0-based) and integer image shifts
 * dc (n,3) such that r_i - r_j + cell^T dc is the pair vector.  Any pointer
 * may be NULL; host or device memory. */
int gb_neighbors_get(gb_neighbors_t *nl, gb_particles_t *p, int64_t *seed, int *j,
                     int *dc);
int gb_neighbors_set_stream(gb_neighbors_t *nl, void *cuda_stream);

/* ------------------------------------------------------------------------
 * Potentials — replace the generated shims python_<mod>_{new, free,
 * init_without_parameters, bind_to, energy_and_forces}
 * (gen_factory.py:98-356; prototypes :380-401).
 * ---------------------------------------------------------------------- */

/* Tersoff parameter set: layout of BOP_DB_TYPE
 * (src/potentials/bop/tersoff/tersoff_params.f90:27-97), 0-based element and
 * symmetric pair indices (src/macros.inc:123). */
typedef struct gb_tersoff_params {
  int nel;
  int Z[3];
  double A[6], B[6], xi[6], lambda[6], mu[6], omega[6], mubo[6];
  int m[6];
  double beta[3], n[3], c[3], d[3], h[3];
  double r1[6], r2[6];
} gb_tersoff_params_t;

/* Kumagai parameter set (src/potentials/bop/kumagai/kumagai_params.f90:27-96). */
typedef struct gb_kumagai_params {
  int nel;
  int Z[1];
  double A[1], B[1], lambda1[1], lambda2[1];
  double eta[1], delta[1], alpha[1];
  int beta[1];
  double c1[1], c2[1], c3[1], c4[1], c5[1], h[1];
  double r1[1], r2[1];
} gb_kumagai_params_t;

/* Brenner (Albe-Erhart form) parameter set: layout of BOP_DB_TYPE
 * (src/potentials/bop/brenner/brenner_params.f90:27-65), every array per
 * symmetric element pair (0-based, src/macros.inc:123): dimer energy D0,
 * dimer length r0, Pauling slope S, stiffness beta, angular gamma, c, d, h,
 * bond-order exponents mu, n, m and the cutoff r1 < r2. */
typedef struct gb_brenner_params {
  int nel;
  int Z[3];
  double D0[6], r0[6], S[6], beta[6], gamma[6], c[6], d[6], h[6], mu[6], n[6];
  int m[6];
  double r1[6], r2[6];
} gb_brenner_params_t;

/* Juslin parameter set: layout of BOP_DB_TYPE
 * (src/potentials/bop/juslin/juslin_params.f90:31-70).  Pair arrays are per
 * ORDERED element pair, entry j + i*nel (0-based, src/macros.inc:139); an
 * entry with r0 < 0 takes the constants of its mirror pair (j, i) as the
 * reference's bind_to does (juslin_module.f90:273-300).  The h(dr) constants
 * alpha, omega, m are per element triplet (i, j, k), entry k + nel*(j + nel*i)
 * (src/macros.inc:146): h = omega exp((alpha dr)^m). */
typedef struct gb_juslin_params {
  int nel;
  int Z[3];
  double D0[9], r0[9], S[9], beta[9], gamma[9], c[9], d[9], h[9], n[9];
  double alpha[27], omega[27];
  int m[27];
  double r1[9], r2[9];
} gb_juslin_params_t;

/* Extra parameters of the screened variants TersoffScr / KumagaiScr /
 * BrennerScr / JuslinScr (tersoff_params.f90:81-90 under SCREENING), per
 * element pair entry (the first nel(nel+1)/2 symmetric entries; JuslinScr:
 * nel^2 ordered entries): outer (attractive/repulsive) cutoff or1 < or2,
 * bond-order cutoff bor1 < bor2 and the screening window Cmin < Cmax.  The
 * inner cutoff is r1 < r2 of the base parameter set (exp_cutoff form,
 * cutoff.f90:232-293). */
typedef struct gb_screening_params {
  double or1[9], or2[9], bor1[9], bor2[9], Cmin[9], Cmax[9];
} gb_screening_params_t;

/* python_tersoff_new + register (parameters set through a struct instead of
 * the ptrdict config tree, tersoff_registry.f90:22-115). params may be NULL
 * for the default Tersoff_PRB_39_5566_SiC set (tersoff_params.f90:99-138). */
int gb_tersoff_new(gb_potential_t **pot, const gb_tersoff_params_t *params);
/* python_kumagai_new; NULL = Kumagai_CompMaterSci_39_457_Si
 * (kumagai_params.f90:97-132). */
int gb_kumagai_new(gb_potential_t **pot, const gb_kumagai_params_t *params);
/* python_tersoff_scr_new (tersoff_scr.f90): NULL params / scr = the
 * Tersoff_PRB_39_5566_SiC__Scr set (m = 3, mubo = 1 / dimer length,
 * tersoff_params.f90:99-138 under SCREENING).  FP64 only. */
int gb_tersoff_scr_new(gb_potential_t **pot, const gb_tersoff_params_t *params,
                       const gb_screening_params_t *scr);
/* python_kumagai_scr_new (kumagai_scr.f90): NULL = the
 * Kumagai_CompMaterSci_39_457_Si__Scr set.  FP64 only. */
int gb_kumagai_scr_new(gb_potential_t **pot, const gb_kumagai_params_t *params,
                       const gb_screening_params_t *scr);
/* python_brenner_new (brenner.f90, brenner_module.f90:26-246): NULL params =
 * the Erhart_PRB_71_035211_SiC set (brenner_params.f90:67-117).  Rejects
 * d = 0 and S <= 1 as the reference's bind_to does. */
int gb_brenner_new(gb_potential_t **pot, const gb_brenner_params_t *params);
/* python_brenner_scr_new (brenner_scr.f90): NULL params / scr = the
 * Erhart_PRB_71_035211_SiC__Scr set.  FP64 only. */
int gb_brenner_scr_new(gb_potential_t **pot, const gb_brenner_params_t *params,
                       const gb_screening_params_t *scr);
/* python_juslin_new (juslin.f90, juslin_module.f90:27-406): NULL params =
 * the Juslin_J_Appl_Phys_98_123520_WCH set (juslin_params.f90:75-108).
 * Rejects d = 0 and S <= 1 as the reference's bind_to does. */
int gb_juslin_new(gb_potential_t **pot, const gb_juslin_params_t *params);
/* python_juslin_scr_new (juslin_scr.f90): NULL params / scr = the compiled-in
 * screened W-C-H set (juslin_params.f90:95-103 under SCREENING: Cmin = 1,
 * Cmax = 3).  C_dr_cut = Cmax^2 / (4 (Cmax - 1)) for every pair
 * (juslin_module.f90:305-307).  FP64 only. */
int gb_juslin_scr_new(gb_potential_t **pot, const gb_juslin_params_t *params,
                      const gb_screening_params_t *scr);
/* python_tabulated_alloy_eam_new + init(fn=...) (tabulated_alloy_eam.f90:147-259):
 * reads a DYNAMO setfl file of 1 to 10 elements (MAX_EAM_ELS, :60); each
 * element's atomic number must match its name in the header (:206-213). */
int gb_tabulated_alloy_eam_new(gb_potential_t **pot, const char *fn);
/* python_tabulated_eam_new + init(fn=...) (tabulated_eam.f90:147-200): a
 * single-element DYNAMO funcfl file; every atom is of its element
 * (elements = "*"); no mask; wpot_per_at is left untouched, as by the
 * reference kernel. */
int gb_tabulated_eam_new(gb_potential_t **pot, const char *fn);
/* python_<mod>_free */
void gb_potential_free(gb_potential_t *pot);
/* GB_PRECISION_FP64 (default) or GB_PRECISION_MIXED (BOP only). */
int gb_potential_set_precision(gb_potential_t *pot, int precision);
int gb_potential_set_stream(gb_potential_t *pot, void *cuda_stream);
/* Interaction cutoff the potential requests for the pair (Z1, Z2). */
double gb_potential_get_cutoff(const gb_potential_t *pot);

/* python_<mod>_bind_to (gen_factory.py:219-237 -> BIND_TO_FUNC,
 * default_bind_to_func.f90:25-146; tabulated_alloy_eam.f90:297-350):
 * maps elements and requests the interaction range on nl. */
int gb_potential_bind_to(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                         int *ierror);

/* The LAMMPS contract (pair_atomistica.cpp:386-545, bop_kernel.f90:577-597
 * under LAMMPS) for the bond-order potentials: nat = local + ghost atoms with
 * explicit positions r (nat,3) and atomic numbers Z (nat), a full symmetric
 * neighbour list over all of them without image shifts as 0-based CSR
 * (seed[nat+1], nbr[seed[nat]]), bonds computed for the first natloc atoms.
 * f (nat,3), wpot and the optional epot_per_at (nat) / wpot_per_at (nat,3,3)
 * are accumulated into for all nat atoms (the caller sums ghost
 * contributions back onto their owners); epot is set to the local atoms'
 * share.  Host or device pointers. */
int gb_potential_energy_and_forces_ghost(gb_potential_t *pot, int nat, int natloc,
                                         const double *r, const int *Z, const int *seed,
                                         const int *nbr, double *epot, double *f, double *wpot,
                                         const int *mask, double *epot_per_at,
                                         double *wpot_per_at, int *ierror);
/* lammps_<mod>_energy_and_forces (src/lammps/gen_factory.py:175-226): as
 * gb_potential_energy_and_forces_ghost, with the per-atom virial in the
 * layout the reference's LAMMPS build writes: vatom (nat,6) (= Fortran
 * (6,nat)), accumulated into with the LAMMPS sign, vatom[6i + k] -= w_k(i)
 * for k = xx, yy, zz, yx, zx, zy of atom i's virial (SUM_VIRIAL under
 * LAMMPS, macros.inc:202). */
int gb_potential_energy_and_forces_lammps(gb_potential_t *pot, int nat, int natloc,
                                          const double *r, const int *Z, const int *seed,
                                          const int *nbr, double *epot, double *f, double *wpot,
                                          const int *mask, double *epot_per_at, double *vatom,
                                          int *ierror);
/* python_<mod>_energy_and_forces (gen_factory.py:239-356 -> COMPUTE_FUNC,
 * default_compute_func.f90:25-100; tabulated_alloy_eam.f90:360-415).
 * q (charges) is accepted and ignored, as by these potentials. */
/* As gb_potential_energy_and_forces; flags = GB_FORCES_SET writes f (the
 * reference's own Python call without a forces argument returns a fresh
 * zeroed array, potential.c:468): no upload of the caller's f. */
int gb_potential_energy_and_forces_flags(gb_potential_t *pot, gb_particles_t *p,
                                         gb_neighbors_t *nl, const double *q, double *epot,
                                         double *f, double *wpot, const int *mask,
                                         double *epot_per_at, double *epot_per_bond,
                                         double *f_per_bond, double *wpot_per_at,
                                         double *wpot_per_bond, int flags, int *ierror);
int gb_potential_energy_and_forces(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                                   const double *q, double *epot, double *f, double *wpot,
                                   const int *mask, double *epot_per_at, double *epot_per_bond,
                                   double *f_per_bond, double *wpot_per_at,
                                   double *wpot_per_bond, int *ierror);

/* Per-class aliases with the reference's shim names' shape. */
int gb_tersoff_bind_to(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                       int *ierror);
int gb_tersoff_energy_and_forces(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                                 const double *q, double *epot, double *f, double *wpot,
                                 const int *mask, double *epot_per_at, double *epot_per_bond,
                                 double *f_per_bond, double *wpot_per_at,
                                 double *wpot_per_bond, int *ierror);
int gb_kumagai_bind_to(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                       int *ierror);
int gb_kumagai_energy_and_forces(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                                 const double *q, double *epot, double *f, double *wpot,
                                 const int *mask, double *epot_per_at, double *epot_per_bond,
                                 double *f_per_bond, double *wpot_per_at,
                                 double *wpot_per_bond, int *ierror);
int gb_brenner_bind_to(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                       int *ierror);
int gb_brenner_energy_and_forces(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                                 const double *q, double *epot, double *f, double *wpot,
                                 const int *mask, double *epot_per_at, double *epot_per_bond,
                                 double *f_per_bond, double *wpot_per_at,
                                 double *wpot_per_bond, int *ierror);
int gb_juslin_bind_to(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                      int *ierror);
int gb_juslin_energy_and_forces(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                                const double *q, double *epot, double *f, double *wpot,
                                const int *mask, double *epot_per_at, double *epot_per_bond,
                                double *f_per_bond, double *wpot_per_at,
                                double *wpot_per_bond, int *ierror);
/* The EAM classes keep the uniform 14-argument shim type of
 * python_<mod>_energy_and_forces (factory.template.h:48-50), so they fit
 * the same function table; arguments outside a class's features (per-bond
 * outputs; for TabulatedEAM also mask) are refused with GB_ERROR_ARGUMENT
 * and the shim's message (gen_factory.py:302-351). */
int gb_tabulated_alloy_eam_bind_to(gb_potential_t *pot, gb_particles_t *p,
                                   gb_neighbors_t *nl, int *ierror);
int gb_tabulated_alloy_eam_energy_and_forces(gb_potential_t *pot, gb_particles_t *p,
                                             gb_neighbors_t *nl, const double *q, double *epot,
                                             double *f, double *wpot, const int *mask,
                                             double *epot_per_at, double *epot_per_bond,
                                             double *f_per_bond, double *wpot_per_at,
                                             double *wpot_per_bond, int *ierror);
int gb_tabulated_eam_bind_to(gb_potential_t *pot, gb_particles_t *p, gb_neighbors_t *nl,
                             int *ierror);
int gb_tabulated_eam_energy_and_forces(gb_potential_t *pot, gb_particles_t *p,
                                       gb_neighbors_t *nl, const double *q, double *epot,
                                       double *f, double *wpot, const int *mask,
                                       double *epot_per_at, double *epot_per_bond,
                                       double *f_per_bond, double *wpot_per_at,
                                       double *wpot_per_bond, int *ierror);

/* The `elements` property of TabulatedAlloyEAM / TabulatedEAM
 * (tabulated_alloy_eam.f90:72, filter_from_string in src/core/filter.f90:
 * 55-120): "*" (default) = every element; otherwise comma-separated element
 * symbols or atomic numbers, each read into two characters.  Atoms of other
 * elements are skipped as centre and as neighbour (:316-335).  An unknown
 * symbol returns GB_ERROR_ARGUMENT ("Unknown element 'X'.").  Takes effect
 * on the next evaluation. */
int gb_potential_set_elements(gb_potential_t *pot, const char *elements);

/* Spline table export of an EAM potential (for parity checks of the host
 * setfl reader and spline builder against simple_spline_init,
 * simple_spline.f90:127-195): which = 0 F(rho), 1 rho(r), 2 phi(r) (index
 * i*nel+j).  Returns the number of points n; x0dx = {x0, dx, cut}; coef is
 * (8, n): y, d2y, c1, c2, c3, d1, d2, d3 (last column of the 6 interval
 * arrays is 0).  coef may be NULL. */
int gb_tabulated_alloy_eam_table(const gb_potential_t *pot, int which, int idx, double *x0dx,
                                 double *coef);

/* ------------------------------------------------------------------------
 * Allocation-free evaluation.  This entry point has no counterpart in the
 * reference.  It is meant for callers that cannot call cudaMalloc: codes
 * embedded in a host framework that has already reserved the device memory
 * for its own pool (so a cudaMalloc would fail or fragment that pool), and MD
 * loops that must not allocate during a time step.  It evaluates a Tersoff,
 * Kumagai or Brenner potential (non-screened; FP64 or mixed, as set on `pot`)
 * on a neighbour list the caller supplies and allocates nothing: all
 * intermediate buffers live in one static device array of 12,976,896 bytes
 * (about 13 MB) that every GPU loading this library holds until the process
 * exits.
 *
 *   limits: nat <= 16384 atoms and at most 262144 list entries; larger
 *           inputs are rejected with GB_ERROR_CAPACITY and a message.
 *   device memory: r (nat,3), Z (nat), seed (nat+1, int64), j (n), dc (n,3)
 *           — the full symmetric list in the layout of gb_neighbors_get —
 *           and the outputs epot (1 double, set), f (nat,3) and wpot (9,
 *           Fortran order), both accumulated into, as in
 *           gb_potential_energy_and_forces.
 *   host memory: cell (3x3, rows = lattice vectors).
 *   stream: the CUDA stream all work is issued on (NULL = default stream).
 *           The call blocks the host: it waits for the stream several times
 *           (to read the list size, the list checks and the tile plan) and
 *           returns after the stream has finished its work.
 *   checks: seed[0] = 0, non-decreasing offsets up to seed[nat], neighbour
 *           indices in [0, nat), image shifts within +-511 and a symmetric
 *           list are verified before any kernel walks the list; a violation
 *           returns GB_ERROR_ARGUMENT with a message.
 *   set-up: the first call on a device looks up the device address of the
 *           static array (cudaGetSymbolAddress); make that first call before
 *           any stream capture.
 *   sharing: every call uses the same array and finds it holding the
 *           previous call's data (the call clears what must start at zero);
 *           calls that overlap on the GPU — from several host threads or
 *           streams — race on it and must be serialised by the caller.
 * ---------------------------------------------------------------------- */
int gb_bop_energy_and_forces_noalloc(gb_potential_t *pot, int nat, const double *r,
                                     const double *cell, const int *Z, const int64_t *seed,
                                     const int *j, const int *dc, double *epot, double *f,
                                     double *wpot, void *cuda_stream);

/* ------------------------------------------------------------------------
 * Batches of independent structures (no counterpart in the reference: it
 * evaluates one particles object per call).  One neighbour build and one
 * bond-order tile launch cover all structures; per structure the results
 * equal a separate energy_and_forces call on that structure (same list, same
 * kernels).  Tersoff, Kumagai and Brenner, FP64 or mixed precision.
 * ---------------------------------------------------------------------- */
int gb_batch_new(gb_batch_t **batch);
void gb_batch_free(gb_batch_t *batch);
int gb_batch_set_stream(gb_batch_t *batch, void *cuda_stream);
/* nstruct structures; nat[s] atoms each (atoms of structure s follow those of
 * s-1); cells: nstruct x 3 x 3, rows = lattice vectors; pbc: nstruct x 3 (NULL:
 * periodic in all directions); Z: atomic numbers of all atoms. */
int gb_batch_set_structures(gb_batch_t *batch, int nstruct, const int *nat,
                            const double *cells, const int *pbc, const int *Z);
/* Positions of all atoms, (total atoms, 3); host or device memory. */
int gb_batch_set_positions(gb_batch_t *batch, const double *r);
int gb_batch_get_nat(const gb_batch_t *batch);
/* use_graph: after an evaluation, capture the whole evaluation (list build,
 * tiles, gather, sums) in a CUDA graph and replay it while structures,
 * potential and buffer sizes are unchanged (a replay whose list or tiles
 * overflow the captured sizes is discarded and the evaluation redone
 * eagerly).  autotune: time 64/32/16 atoms per tile on the first evaluation
 * of a geometry and keep the fastest.  Both off by default. */
int gb_batch_set_options(gb_batch_t *batch, int use_graph, int autotune);
/* Last evaluation: info[0] 1 if it was a graph replay, info[1] atoms per
 * tile, info[2] kernels in the captured graph (0: none), info[3] tile sizes
 * timed by the autotuner. */
int gb_batch_last_info(const gb_batch_t *batch, int64_t *info);
/* Velocity Verlet on the batch (src/standalone/verlet.f90:100-235):
 * md_set_state sets velocities v (total atoms, 3) and masses m (total atoms;
 * m <= 0 freezes an atom, the reference's group filter); md_run advances
 * nsteps steps of dt (v += f dt / 2m; r += v dt; forces; v += f dt / 2m, in
 * the caller's consistent units), writing epot[nstruct] / wpot (optional) of
 * the last step; with use_graph a whole step (both kicks, the drift, the list
 * build and the forces) is replayed as one CUDA graph.  md_get_state reads
 * positions, velocities and the forces at the current positions (any may be
 * NULL).  Host or device memory. */
int gb_batch_md_set_state(gb_batch_t *batch, const double *v, const double *m);
int gb_batch_md_run(gb_batch_t *batch, gb_potential_t *pot, double dt, int nsteps, double *epot,
                    double *wpot);
int gb_batch_md_get_state(gb_batch_t *batch, double *r, double *v, double *f);
/* epot[nstruct] set; f (total atoms, 3) and wpot[nstruct][3][3] (each in the
 * layout of energy_and_forces' wpot) accumulated.  Host or device memory. */
int gb_batch_energy_and_forces(gb_batch_t *batch, gb_potential_t *pot, double *epot, double *f,
                               double *wpot);

/* Tangent evaluation for parameter fitting (no counterpart in the
 * reference): single-element Tersoff (atoms of atomic number Z; others are
 * skipped) with the 14 continuous parameters params = {A, B, lambda, mu, beta,
 * n, c, d, h, R, S, xi, omega, mubo} and integer m.  Along the direction
 * (dparams, dr) — dparams[14] (NULL: 0) and a position direction dr
 * (total atoms, 3; NULL: 0) — returns epot[nstruct], f (total atoms, 3) and
 * their directional derivatives depot, df (all set, not accumulated; host or
 * device memory).  With dr = v and dparams = NULL, df = -H v (H the Hessian
 * of the energy).  The neighbour list is built for the cutoff S. */
int gb_batch_tersoff_tangent(gb_batch_t *batch, int Z, int m, const double *params,
                             const double *dparams, const double *dr, double *epot,
                             double *depot, double *f, double *df);
/* The reverse-mode (adjoint) counterpart for loss gradients, in one pass: the
 * hand-written gradient of each structure's energy with respect to the 14
 * parameters, dE_dparams (nstruct,14), evaluated in dual numbers along a
 * position direction v (total atoms,3; NULL: 0), which also gives
 * dv_dE_dparams (nstruct,14) = v . d(dE_s/dparams)/dr = d(v . dE_s/dr)/dparams
 * (the parameter gradient of a force-matching term with v = dL/dF, up to
 * sign) and hv (total atoms,3) = derivative of the forces along v = -H v,
 * recomputed from bond-order intermediates without per-triplet storage.
 * epot (nstruct) and f (total atoms,3) are the values.  mubo is
 * differentiated also at 0 (h = exp((2 mubo dr)^m)).  hv and dv_dE_dparams
 * may be NULL.  Host or device output pointers; all set, not accumulated.
 * No counterpart in the reference. */
int gb_batch_tersoff_adjoint(gb_batch_t *batch, int Z, int m, const double *params,
                             const double *v, double *epot, double *f, double *hv,
                             double *dE_dparams, double *dv_dE_dparams);

/* ------------------------------------------------------------------------
 * Diagnostics (no counterpart in the reference; used by the benchmark).
 * ---------------------------------------------------------------------- */
/* Timing of the last energy_and_forces call in milliseconds (CUDA events on
 * the potential's stream): [0] neighbour-list update, [1] force evaluation,
 * [2] total, [3] the dominant force kernel alone (bond-order tile kernel or
 * EAM pair kernel).  ms must hold 4 doubles. */
int gb_potential_last_timing(const gb_potential_t *pot, double *ms);
/* Work counts of the last energy_and_forces call: stats[0] directed bonds
 * (bond-order potentials), stats[1] bonds of the mixed form whose estimated
 * FP32 error sent them through the float-float recomputation, stats[2] atoms
 * per bond-order tile, stats[3] 1 when the call was a CUDA-graph replay
 * (gb_potential_set_graph), else 0.  stats must hold 4 int64_t. */
int gb_potential_last_stats(const gb_potential_t *pot, int64_t *stats);
/* CUDA-graph replay of whole evaluations (on != 0; off by default) for the
 * non-screened bond-order potentials and the EAM classes: an evaluation with
 * only epot, f and
 * wpot requested (no mask, no per-atom or per-bond outputs) that follows an
 * eager one on the same particles, neighbour list, cell and force array is
 * captured — neighbour build (single staged pass, no host decision), tile
 * kernel, gather, sums, the copies of status words and results — and the
 * next such evaluations replay it with one host synchronisation.  The
 * captured list has a per-atom capacity (1.25 x the largest coordination of
 * the eager build + 4) and the captured tile plan head room; a replay that
 * exceeded either leaves the forces untouched (set to zero with
 * GB_FORCES_SET) and is redone eagerly, then captured again.  Results equal
 * the eager path's bit for bit. */
int gb_potential_set_graph(gb_potential_t *pot, int on);
/* Atoms per bond-order tile (a power of two <= 64, reduced until the worst
 * tile fits in shared memory); 0 restores the automatic choice.  A tuning
 * knob: results do not depend on it beyond FP rounding of the tile sums. */
int gb_potential_set_tile_atoms(gb_potential_t *pot, int atoms);
/* Number of kernel launches this library has issued since it was loaded. */
uint64_t gb_kernel_launches(void);
/* FMA-chain microbenchmark on the current device: sustained FP64 (fp64=1)
 * or FP32 (fp64=0) throughput in TFLOP/s (2 flops per FMA). */
int gb_bench_fma_peak(int fp64, double *tflops);
/* Device check of the square root the EAM density pass derives from its
 * refined reciprocal square root: *mismatches = how many of n arguments,
 * drawn uniformly from [lo, hi] (lo > 0), differ from the correctly rounded
 * sqrt.  Diagnostic; no counterpart in the reference. */
int gb_diag_sqrt_check(int64_t n, double lo, double hi, int64_t *mismatches);
/* Host-only generator of the random workload structures: nat uniform
 * positions (pos: nat x 3, Cartesian) in the cell (rows = lattice vectors)
 * with every pair, over all periodic images, at least dmin apart (random
 * sequential addition, xoshiro256** stream of the given seed; at most
 * max_tries candidates).  Same result on every host. */
int gb_random_packing(int nat, const double *cell, double dmin, uint64_t seed,
                      int64_t max_tries, double *pos);

#ifdef __cplusplus
}
#endif

#endif /* ATOMISTICA_GB300_H */
