/* CPU oracle for the photon-propagation path: a plain-C restatement of the
 * reference's octree gather, RK4 geodesic integrator, infinitesimal lensing
 * Jacobian and per-pixel map reduction.
 *
 * TEST INFRASTRUCTURE ONLY.  It is the checker the CUDA path is compared
 * against (tests/, __graft_entry__.smoke) and the timed CPU baseline of
 * bench.py; the product never links or calls it.  It is itself pinned
 * bit-for-bit to the reference's own code (oracle/ref_harness.cpp) by
 * the committed golden fixtures (tests/test_keys_and_oracle.py,
 * tests/test_oracle_whole_rays.py, tests/test_oracle_velocity.py,
 * tests/test_oracle_cells.py).
 *
 * Every floating-point expression keeps the reference's operation order and
 * must be compiled without FMA contraction (-ffp-contract=off), as the
 * reference's x86-64 build is. */
#ifndef MPF_ORACLE_H
#define MPF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Velocity field of the octree (the reference built with -DVELOCITYFIELD):
 * per-cell velocities (gravity2.h:45) and the observer velocity the rays are
 * traced with (hmaps.h:80-84). */
typedef struct {
    const float* v;         /* n x 3 */
    double vobs[3];
} mpfo_velocity;

/* Sorted octree: n keys (128-bit, as hi/lo pairs) and 7 float fields per cell
 * in the order rho, phi, dphidx, dphidy, dphidz, a, dphidt; vel: NULL, or a
 * velocity field (the gathers then carry it, and every redshift takes the
 * ISW, Doppler and observer terms, integrator.h:765-767). */
typedef struct {
    int64_t n;
    const uint64_t* keys;   /* n x 2: hi, lo */
    const float* fields;    /* n x 7 */
    const mpfo_velocity* vel;
} mpfo_tree;

typedef struct {
    int64_t n;
    const double* t;
    const double* a;
    const double* dadt;
} mpfo_cosmo;

enum { MPFO_STOP_REDSHIFT = 0, MPFO_STOP_R = 1, MPFO_STOP_LAMBDA = 2, MPFO_STOP_T = 3,
       MPFO_STOP_A = 4, MPFO_STOP_PLANE = 5, MPFO_STOP_S = 6 };

/* Photon record (28 doubles): a t x y z dtdl dxdl dydl dzdl level ah rho phi
 * dphidx dphidy dphidz dphidt dphidl laplacian redshift dsdl2 error isw iswold
 * chi lambda s index.
 * Plane record (20 doubles): firstid f x y z distance A11 A12 A22 t a redshift
 * chi lambda s isw rho phi rho_max valid. */
#define MPFO_PHOTON 28
#define MPFO_PLANE 20

void mpfo_key_compute(unsigned level, double x, double y, double z, uint64_t* out);
unsigned mpfo_key_level(uint64_t hi, uint64_t lo);
int64_t mpfo_locate(const mpfo_tree* T, double x, double y, double z);
void mpfo_cic(const mpfo_tree* T, double x, double y, double z, float* out7);
void mpfo_tsc(const mpfo_tree* T, double x, double y, double z, float* out7);
void mpfo_ngp(const mpfo_tree* T, double x, double y, double z, float* out7);
double mpfo_interpolate(double x0, const double* x, const double* y, int64_t n);

/* Batch of rays.  launch: n x 6 (start xyz, end xyz, the 6-argument
 * Integrator::launch).  planes: values of the stop quantity at which map
 * planes are read (the last one is also the stop value); nplanes may be 0,
 * then stop_ref is used.  jacobian != 0 computes the infinitesimal Jacobian
 * at each plane's distance.  Outputs: steps[n], final[n x 28],
 * plane_out[n x nplanes x 20].  Returns 0, or a negative error. */
int mpfo_propagate(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                   int stop_kind, double stop_ref, const double* ki_target,
                   int64_t n, const double* launch, int nplanes, const double* planes, int jacobian,
                   int64_t* steps, double* final_out, double* plane_out, int nthreads);

/* Whole trajectory of one ray; returns the number of records (may exceed cap). */
int64_t mpfo_trajectory(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                        int stop_kind, double stop_ref, const double* launch, double* out, int64_t cap);

/* Catalogue root-finder (Catalogues::iterateNewtonMethod, infinitesimal
 * Jacobian, at most max_iterations + 1 rays per source).  src: n x 6 (x y z
 * vx vy vz in octree units and RAMSES velocity units), rotm1: 3x3 row-major
 * rotation to the octree frame or NULL (full sky), vobs: observer velocity.
 * out: n x 16 catalog rows: comoving phi theta, observed phi theta, miss,
 * iterations (42: rejected; with phi = theta = 42: failed, then firstid),
 * z_flrw z_pot z_dopp z_tdopp z_isw z_gr, a11 a12 a21 a22. */
int mpfo_catalogue(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                   int64_t n, const double* src, const double* rotm1, const double* vobs, double cat_accuracy,
                   double h, double mpc, int max_iterations, double* out, int nthreads);
/* Same with the Jacobian type: bundle = 1 is jacobiantype = "bundle" (the
 * four-ray Lensing::dbetadtheta from iteration 5 and at convergence), with
 * plane_sachs (1: "sachs", 0: "normal"), stop_bundle (MPFO_STOP_*) and
 * openingmin (radians); bundle = 2 is "infinitesimal_born" (the converged
 * source's Jacobian along its Order = -1 ray). */
int mpfo_catalogue_jac(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                       int64_t n, const double* src, const double* rotm1, const double* vobs, double cat_accuracy,
                       double h, double mpc, int max_iterations, int bundle, int plane_sachs, int stop_bundle,
                       double openingmin, double* out, int nthreads);

/* FillMap's lensing_born rays (hmaps.h:706-712): the Order = -1 ray of each
 * 6-argument launch to stop_ref, and the infinitesimal Jacobian along it at
 * the nd distances dist; size[n], A[n x nd x 3] (a11 a12 a22). */
int mpfo_born(const mpfo_tree* T, const mpfo_cosmo* C, double length, unsigned nsteps, int stop_kind, double stop_ref,
              int64_t n, const double* launch, int nd, const double* dist, int64_t* size, double* A);

/* Hmaps::FillMap with jacobiantype = "bundle": the central rays' surfaces
 * (plane_out, n x np x 20 as mpfo_propagate, without the infinitesimal
 * Jacobian) and Lensing::dbetadtheta's 2x2 Jacobian at each surface (jac_out,
 * n x np x 4: a11 a12 a21 a22).  plane_sachs: kiTarget = interpolated
 * direction (1) or position (0); stop_bundle: an MPFO_STOP_* value. */
/* Integrator::propagate (integrator.h:861-1015): the photon (start xyz,
 * direction as launched) and `count` photons at `angle` around it, integrated
 * without a stop criterion, the bundle checks and the central ray's angular
 * diameter distance; kind: the reference parameter (an MPFO_STOP_ value).
 * out: m x 29 in the trajectory file's column order.  Returns the central
 * trajectory's size, 0 when the bundle is rejected. */
int64_t mpfo_propagate_bundle(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps,
                              const double* photon, unsigned count, double angle, double rotation, int kind, double amin,
                              double* out, int64_t cap);

int mpfo_bundle(const mpfo_tree* T, const mpfo_cosmo* C, int order, double length, unsigned nsteps, int stop_kind,
                int64_t n, const double* launch, int np, const double* planes, int plane_sachs, int stop_bundle,
                double openingmin, double* plane_out, double* jac_out, int nthreads);

/* Hmaps::CreateOctreeVelocityWithCIC (scheme 1, hmaps.h:439-485) / WithTSC
 * (scheme 2, :501-550) on one thread: npart particles (pos, vel: npart x 3
 * floats) deposited at every level lmin..lmax on the cells with the exact key
 * of each vertex; rho (fields[7i], n x 7, the tree's keys) and v (n x 3)
 * accumulate in float.  flags: 1 = zero rho and v first (hmaps.cpp:395-396),
 * 2 = then v /= rho (zero read as 1) and, level by level, cells whose rho is
 * not normal take the parent's v (hmaps.cpp:424-441). */
int mpfo_velocity_deposit(const mpfo_tree* T, float* fields, float* v, int scheme, int64_t npart, const float* pos,
                          const float* pv, int flags);

/* Create_octree::PreparationASCII's per-cone body (create_octree.h:544-580):
 * Input::importascii of the cell rows (n x 10 floats: level x y z rho phi
 * fx fy fz a) with the cone / microsphere filter, then correctOctree
 * (sistemize, update, Input::correct, dphidt * da/dt).  records: capacity x
 * 48-byte cone records sorted by key; returns the cell count (records beyond
 * capacity are not written), -1 for bad arguments, -2 without memory.
 * completion_waves: 0 fills the completed octs' children one after the
 * other, as the reference's loop does; k > 0 fills them as the device does,
 * in at most k waves of gathers that read only children of earlier waves,
 * then the rest in order.  info (may be NULL): incomplete cells, children
 * filled in waves, waves, children filled in order after them. */
typedef struct {
    double cone_vertex[3], cone_base[3], cone_angle;
    double sphere_center[3], sphere_radius;
    const double* rotm1;       /* 3x3 row-major, or NULL (full sky) */
    double h, lboxmpch, mpc;
    int coarseonly, ncoarse, correction, coarsecorrection, acorrection, order;
    int completion_waves;
} mpfo_cells_params;
int64_t mpfo_cells_build(const float* rows, int64_t n, const mpfo_cells_params* P, const mpfo_cosmo* C, void* records,
                         int64_t capacity, double* amin, int64_t* info);
/* The reference's ASCII cell reads (stream >> unsigned >> 9 floats): rows
 * (capacity x 10 at most); returns the row count, -1 on a malformed row. */
int64_t mpfo_cells_parse(const char* text, int64_t length, float* rows, int64_t capacity);

void mpfo_batch_locate(const mpfo_tree* T, int64_t n, const double* xyz, int64_t* out, int nthreads);
void mpfo_batch_cic(const mpfo_tree* T, int64_t n, const double* xyz, float* out, int nthreads);
void mpfo_batch_tsc(const mpfo_tree* T, int64_t n, const double* xyz, float* out, int nthreads);
void mpfo_batch_ngp(const mpfo_tree* T, int64_t n, const double* xyz, float* out, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
