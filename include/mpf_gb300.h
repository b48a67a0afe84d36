/* mpf_gb300: GB300 (sm_103a) photon-propagation path of Magrathea-Pathfinder.
 *
 * C ABI: plain pointers and sizes, no C++ or CUDA types.  Every entry point
 * returns an mpf_status (0 = success, < 0 = error, > 0 = completed with a
 * warning); mpf_last_error() gives a message for the calling thread.
 *
 * Handles (mpf_octree, mpf_cosmology) own device memory on the device that
 * was current when they were created and are read-only afterwards: calls
 * from several host threads on different streams may share them.  An
 * mpf_surrogate changes when it is trained: one host thread at a time.  Buffers passed to the mpf_* calls below are
 * HOST memory unless the name ends in _device.
 *
 * Each entry point names the reference interface it stands in for
 * (paths within the reference source tree).
 */
#ifndef MPF_GB300_H
#define MPF_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MPF_OK = 0,
    MPF_WARN_MAX_STEPS = 1,      /* at least one ray hit params.max_steps */
    MPF_BAD_INPUT = -1,
    MPF_OUT_OF_MEMORY = -2,
    MPF_CUDA_ERROR = -3,
    MPF_NOT_SORTED = -4,         /* cone records must be sorted by key */
    MPF_NO_DEVICE = -5,
    MPF_IO_ERROR = -6,
    MPF_DEVICE_TIMEOUT = -7      /* a bounded device wait ran out; the context stays usable */
} mpf_status;

typedef enum {                    /* stop_ray / stop criterion, src/integrator.h:779-811 */
    MPF_STOP_REDSHIFT = 0,
    MPF_STOP_RADIUS = 1,          /* "r" / "radius": comoving distance in octree units */
    MPF_STOP_LAMBDA = 2,
    MPF_STOP_T = 3,               /* "t" / "eta": conformal time */
    MPF_STOP_A = 4,
    MPF_STOP_PLANE = 5,           /* x . plane_normal > stop_value */
    MPF_STOP_S = 6
} mpf_stop;

typedef struct mpf_octree mpf_octree;
typedef struct mpf_cosmology mpf_cosmology;

typedef struct {
    int64_t cells;
    int64_t nodes;
    int level_min, level_max;
    int top_level;
    int grid[3];
    int64_t device_bytes;
} mpf_octree_info;

/* Ray-tracing parameters (the parameter-file keys of the rays / hmaps /
 * catalogues executables, src/hmaps.h:148-199). */
typedef struct {
    double length;             /* lbox * mpc / h in metres (hmaps.cpp:165) */
    double stop_value;         /* interpRef; ignored when nplanes > 0 (last plane is used) */
    double plane_normal[3];    /* kiTarget for MPF_STOP_PLANE */
    const double* planes;      /* surfaces (values of the stop quantity), ascending; host memory */
    int nplanes;               /* <= MPF_MAX_PLANES */
    unsigned nsteps;           /* steps per cell */
    int order;                 /* 0 = NGP, 1 = CIC, 2 = TSC (the reference's ORDER); NGP runs the
                                  float64 kernel whatever `exact` says (no interpolation arithmetic) */
    int stop;                  /* mpf_stop */
    int jacobian;              /* infinitesimal Jacobian at each surface */
    int exact;                 /* 1: the reference's float64 gather arithmetic, bit-exact
                                  trajectories; 0: FP32 gather arithmetic (faster) */
    int64_t max_steps;         /* per ray; <= 0 means 1e8 */
    double vobs[3];            /* observer velocity (parameters v0x v0y v0z, hmaps.h:80-84, in the
                                  units of the octree's velocity field); read only when the octree
                                  carries a velocity field (mpf_octree_set_velocity /
                                  mpf_velocity_deposit) */
} mpf_params;

#define MPF_MAX_PLANES 16
#define MPF_PHOTON_FIELDS 28
#define MPF_PLANE_FIELDS 20

/* Photon record (28 doubles), the reference's Photon<double,3>:
 *   a t x y z dtdl dxdl dydl dzdl level ah rho phi dphidx dphidy dphidz dphidt
 *   dphidl laplacian redshift dsdl2 error isw iswold chi lambda s index
 * Surface record (20 doubles), what FillMap reads at each surface
 * (src/hmaps.h:612-676):
 *   firstid f x y z distance A11 A12 A22 t a redshift chi lambda s isw rho phi
 *   rho_max valid
 * A = the infinitesimal Jacobian (src/lensing.h:459-469), A21 = A12. */

int mpf_version(void);
const char* mpf_last_error(void);
int mpf_device_count(void);

/* Octree upload from cone records (48 bytes each, sorted by key): the
 * in-memory image the reference reads with Input::load (src/input.h:1297-1313)
 * and searches with SimpleHyperOctree::locate/cic/tsc
 * (src/magrathea/simplehyperoctree.h:874-899, 1410-1644). */
int mpf_octree_upload(const void* records, int64_t n, mpf_octree** out);
/* Same, reading a cone .bin file (Miscellaneous::loadOctree, src/miscellaneous.h:422-449). */
int mpf_octree_load(const char* path, mpf_octree** out);
int mpf_octree_get_info(const mpf_octree* o, mpf_octree_info* info);
void mpf_octree_destroy(mpf_octree* o);

/* Velocity field: the velocity slots of the reference's velocity-field octree
 * (src/gravity2.h:45, the build with -DVELOCITYFIELD).  An octree that carries
 * one is traced as that build does: the slots are interpolated with the other
 * fields, count in the emptiness test of each step, and every redshift is
 *   a0 / a (1 + phi0/c^2 - phi/c^2 + isw + v.k / (c k0) - v0n) - 1
 * (src/integrator.h:537-538, 594, 707-708, 765-767), v0n = vobs.k0 / (c k0_0)
 * with the params' vobs and the launch direction.  The catalogue root-finder
 * and the learned surrogate reject such an octree (the reference's catalogues
 * executable stops in that build, catalogues.cpp:290-293).  Changing the
 * field is not safe while another call uses the octree. */
/* v3: n x 3 floats (vx vy vz per cell, in the records' order); rho: n floats
 * that replace the cells' rho, or NULL to keep them.  v3 = NULL removes the
 * field (rho must then be NULL). */
int mpf_octree_set_velocity(mpf_octree* o, const float* v3, const float* rho);
/* The cells' velocities (zeros when the octree has none) and rho; either
 * pointer may be NULL. */
int mpf_octree_get_velocity(const mpf_octree* o, float* v3, float* rho);

#define MPF_VELOCITY_BEGIN 1     /* zero every cell's rho and velocity first (hmaps.cpp:395-396) */
#define MPF_VELOCITY_FINISH 2    /* then v /= rho (a zero rho read as 1) and, level by level, a cell
                                    whose rho is not a normal float takes its parent's velocity
                                    (hmaps.cpp:424-441) */
/* Hmaps::CreateOctreeVelocityWithCIC (scheme 1, src/hmaps.h:439-485) /
 * WithTSC (scheme 2, :501-550): n particles (pos n x 3 in octree units, vel
 * n x 3) deposited at every level of the octree on the cells that hold the
 * exact key of each of their 8 (27) vertices: rho += w, v += v_p w, in float,
 * in particle order, as the reference computes them on one thread.  Calls
 * with flags = 0 between a BEGIN and a FINISH accumulate further particle
 * files, as the reference's loop over shell files does (hmaps.cpp:399-420). */
int mpf_velocity_deposit(mpf_octree* o, int scheme, int64_t n, const float* pos, const float* vel, int flags);
/* Same with the particles in device memory, on `stream` (a cudaStream_t, or
 * NULL for the legacy default stream); returns when the deposit is complete. */
int mpf_velocity_deposit_device(mpf_octree* o, int scheme, int64_t n, const float* pos_device, const float* vel_device,
                                int flags, void* stream);
/* (cell, particle, vertex) pairs the last deposit call on the octree sorted:
 * the work measure of its passes.  No counterpart in the reference. */
int mpf_velocity_deposit_pairs(const mpf_octree* o, int64_t* pairs);

/* Cosmology table: conformal time, a, da/dt, d2a/dt2 rows as returned by
 * Input::acquire + Input::correct (src/input.h:1090-1224, 1329-1360). */
int mpf_cosmology_upload(const double* t, const double* a, const double* dadt, const double* d2adt2, int64_t n,
                         mpf_cosmology** out);
void mpf_cosmology_destroy(mpf_cosmology* c);

/* SimpleHyperOctree::locate: index of the cell (position in the sorted
 * records) or -1, for n positions xyz[3n]. */
int mpf_locate(const mpf_octree* o, int64_t n, const double* xyz, int64_t* cell);

/* SimpleHyperOctree::ngp (order 0) / cic (order 1) / tsc (order 2): 7 floats per position in
 * the order rho phi dphidx dphidy dphidz a dphidt. */
int mpf_interpolate(const mpf_octree* o, int order, int exact, int64_t n, const double* xyz, float* out7);

/* Integrator::launch (6-argument form) + Integrator::integrate with a stop
 * criterion (src/integrator.h:648-824) + Lensing::dbetadtheta_infinitesimal
 * (src/lensing.h:399-472) at each surface, for n rays; the per-pixel body of
 * Hmaps::FillMap (src/hmaps.h:583-700) and of the catalogue Newton step.
 * launch[6n]: start x y z, end x y z (direction = end - start).
 * Outputs (host, each may be NULL): steps[n] = trajectory size,
 * final_rec[28n] = last trajectory point, plane_rec[20 * nplanes * n]. */
int mpf_propagate(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n, const double* launch,
                  int64_t* steps, double* final_rec, double* plane_rec);

/* Errors of the FP32-gather kernel (exact = 0) against the float64 kernel,
 * which runs the reference's operation order and gives its own build's
 * outputs bit for bit: `sample` rays of the batch (launch records k * n /
 * sample) traced by both, compared output by output.  Deflection (the angle
 * between the launch direction and the ray's last position) and redshift:
 * relative to the float64 run, per ray; kappa, gamma1, gamma2, 1/mu at each
 * surface both runs reached: absolute, with the float64 run's largest |value|
 * as the scale.  p as for mpf_propagate (its `exact` is not read).  No
 * counterpart in the reference, whose every output is its own float64 run. */
typedef struct {
    int64_t rays;
    int64_t step_count_differs;     /* rays whose trajectory size differs */
    int64_t max_step_diff;
    double deflection_rel_max, deflection_rel_median;
    double redshift_rel_max, redshift_rel_median;
    int64_t surface_valid_differs;  /* (ray, surface) pairs usable in one run only */
    double lensing_abs_max[4];      /* kappa gamma1 gamma2 1/mu */
    double lensing_scale[4];
} mpf_accuracy;
int mpf_propagate_accuracy(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n,
                           const double* launch, int64_t sample, mpf_accuracy* out);

/* Same with device buffers, asynchronous on `stream` (a cudaStream_t, or NULL
 * for the legacy default stream).  status_device: one uint32 in device memory
 * that receives warning bits (bit 0: max_steps reached). */
int mpf_propagate_device(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n,
                         const double* launch_device, int64_t* steps_device, double* final_device,
                         double* plane_device, uint32_t* status_device, void* stream);

/* mpf_propagate with HOST buffers but without any device allocation: for
 * callers that cannot call cudaMalloc/cudaFree while they run (a pooling
 * allocator owns the GPU's memory, a hard per-process memory cap, or a loop
 * that cannot afford the device synchronisation of an allocation).  It has no
 * counterpart in the reference (which has no device code).  Launch records,
 * outputs, the work-queue counter and the status word are staged through one
 * static device array of MPF_NOALLOC_SCRATCH_BYTES per GPU, kept until the
 * process exits; a batch that does not fit is rejected with MPF_BAD_INPUT.
 * All calls share that array: calls that overlap on the GPU race, so
 * serialise them.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress): make it before any stream capture.  That address is
 * kept for the process's life, so it does not survive a cudaDeviceReset of
 * the device.  Arguments as for mpf_propagate (order 0 runs the float64
 * kernel; steps, final_rec and plane_rec may each be NULL).  Message of a
 * failed call: mpf_noalloc_last_error(). */
#define MPF_NOALLOC_SCRATCH_BYTES (16u << 20)
int mpf_propagate_noalloc(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n, const double* launch,
                          int64_t* steps, double* final_rec, double* plane_rec);
const char* mpf_noalloc_last_error(void);

/* Launch shape chosen by the library's autotuner for an octree on the
 * current device: kind 0 = the propagation kernel (mpf_propagate*,
 * mpf_hmaps_fill; the first batch of at least 2^17 rays is traced in four
 * slices with 128 x 1, 64 x 1, 32 x 1 and 128 x 2 threads per block x rays
 * per lane and work-queue claim, and the fastest in photon-steps/s is kept);
 * kind 1 = the catalogue's persistent kernel (its first three calls of at
 * least 2^16 sources run 128, 64 and 32 threads per block).  order: 1 (CIC)
 * or 2 (TSC).  *threads_per_block = 0 when not tuned yet; rates[4] (may be
 * NULL): the candidates' photon-steps/s.  No counterpart in the reference,
 * which has no device launches to tune.  MPF_AUTOTUNE=0 in the environment
 * keeps the default shape (128 threads, one ray per lane). */
int mpf_autotune_info(const mpf_octree* o, int kind, int order, int* threads_per_block, int* claim_depth, double* rates);

/* ------------------------------------------------------------------------ */
/* Catalogue root-finder                                                     */
/* ------------------------------------------------------------------------ */
/* Parameters of the catalogues executable that the root-finder reads
 * (src/catalogues.h:61-97; the observer is at the origin, catalogues.cpp:196-199). */
typedef struct {
    double length;             /* lbox * mpc / h in metres (catalogues.cpp:163) */
    double h;                  /* dimensionless Hubble parameter (Input::acquire) */
    double mpc;                /* metres per Mpc: parameters.mpc */
    double cat_accuracy;       /* stop when |x_s - x_ray| / |x_s| <= cat_accuracy */
    double vobs[3];            /* observer velocity: parameters.v0x, v0y, v0z */
    const double* rotm1;       /* 3x3 row-major rotation into the octree frame (narrow cones,
                                  relCat catalogues.h:818-826), or NULL (isfullsky) */
    unsigned nsteps;           /* RK4 steps per cell */
    int order;                 /* 0 = NGP, 1 = CIC, 2 = TSC */
    int exact;                 /* 1: reference float64 order; 0: FP32 gathers */
    int max_iterations;        /* 10 in the reference (use_previous_catalogues = 0) */
    /* jacobiantype (catalogues.h:505-529, 660-676): 0 = "infinitesimal";
     * 1 = "bundle", the four-ray Lensing::dbetadtheta from the sixth ray on and
     * at convergence, with the screen normal plane_sachs (1: "sachs", 0:
     * "normal"), the stop criterion stop_bundle (an mpf_stop: redshift, r,
     * lambda, t, a, or plane: the plane through the ray's end point normal to
     * the screen normal, catalogues.h:486-487) and the opening openingmin
     * (radians) */
    int jacobian_bundle;
    int plane_sachs;
    int stop_bundle;
    double openingmin;
    /* 1 = "infinitesimal_born" (catalogues.h:515, 670-673): the Newton steps
     * as "infinitesimal", the converged source's Jacobian along the FLRW (Born)
     * ray of its observed direction to its radius; exclusive with
     * jacobian_bundle */
    int jacobian_born;
} mpf_catalogue_params;

#define MPF_CATALOGUE_FIELDS 16

typedef struct {
    int64_t rays;              /* rays integrated, Jacobian re-traces included */
    int64_t photon_steps;      /* accepted RK4 steps over all of them */
    int64_t photon_steps_jacobian;  /* the part traced with the lensing Jacobian */
    int iterations;            /* Newton rounds run (at most max_iterations + 1) */
    int kernel_launches;       /* kernels this call launched */
} mpf_catalogue_stats;

/* Replaces Catalogues::relCat's per-source loop body (src/catalogues.h:811-856)
 * with Catalogues::iterateNewtonMethod / newtonMethod2d (catalogues.h:410-783)
 * and jacobiantype = "infinitesimal": for each source, rays launched at
 * (phi, theta) are integrated to the source radius, the miss is measured in
 * the screen basis and a Newton step updates (phi, theta), up to
 * max_iterations + 1 rays.  sources: n rows of `stride` doubles (>= 6: x y z
 * in octree units, vx vy vz in RAMSES units, then anything, e.g. id and npart
 * as in the reference's 8-column rows).  rows: n x 16, relCat's catalog row:
 * comoving phi theta, observed phi theta, miss, rays used (42 = rejected),
 * z_FLRW z_pot z_Doppler z_transverse z_ISW z_GR, a11 a12 a21 a22.  A source
 * the rays cannot reach has observed phi = theta = 42, miss 0 and the
 * reference's firstid in column 5 (catalogues.h:436-442).  stats may be NULL. */
int mpf_catalogue_newton(const mpf_octree* o, const mpf_cosmology* c, const mpf_catalogue_params* p, int64_t n,
                         const double* sources, int64_t stride, double* rows, mpf_catalogue_stats* stats);
/* Same, with sources and rows in device memory, on `stream` (a cudaStream_t;
 * NULL = the legacy default stream); returns when the rows are complete.
 * With the FP32-gather kernel and the infinitesimal Jacobian the call is one
 * CUDA graph launch: the sources' set-up and sort, then one persistent kernel
 * that takes sources from a device work queue and puts back those needing
 * another ray; the graph and its scratch are kept per stream and reused by
 * later calls with at most as many sources.  Otherwise (exact mode, bundle or
 * Born Jacobians) the call runs one batched ray launch per Newton round and
 * synchronises the stream between rounds. */
int mpf_catalogue_newton_device(const mpf_octree* o, const mpf_cosmology* c, const mpf_catalogue_params* p, int64_t n,
                                const double* sources_device, int64_t stride, double* rows_device,
                                mpf_catalogue_stats* stats, void* stream);

/* ------------------------------------------------------------------------ */
/* HEALPix maps                                                              */
/* ------------------------------------------------------------------------ */
/* Map components, the reference's index_components (src/hmaps.cpp:196-269,
 * hmaps.h:716-829): rows per surface in the order given; lensing gives 4
 * rows (kappa, gamma1, gamma2, 1/mu; 5 with the bundle Jacobian: w before
 * 1/mu), lensing_born 4 (the same from the Jacobian along the pixel's FLRW
 * ray, hmaps.h:706-712, 771-785), deflection 2 (phi - beta1, theta - beta2),
 * the others 1. */
typedef enum {
    MPF_MAP_LENSING = 0,
    MPF_MAP_LENSING_BORN = 1,     /* kappa gamma1 gamma2 1/mu along the FLRW (Born) ray of the pixel */
    MPF_MAP_DR = 2, MPF_MAP_DL = 3, MPF_MAP_DT = 4, MPF_MAP_DA = 5, MPF_MAP_DZ = 6, MPF_MAP_DS = 7,
    MPF_MAP_ISW = 8, MPF_MAP_DENS = 9, MPF_MAP_DENS_MAX = 10, MPF_MAP_STEPS = 11, MPF_MAP_PHI = 12,
    MPF_MAP_DEFLECTION = 13
} mpf_map_component;
#define MPF_MAX_MAP_COMPONENTS 16

/* Replaces Hmaps::FillMap (src/hmaps.h:583-832, jacobiantype = "infinitesimal")
 * for npix RING pixels of an nside map: pixel centre (pix2vec_ring), one ray
 * per pixel from the origin integrated to the last surface (p->planes, the
 * stop quantity p->stop: interpRefvec), the Jacobian and per-surface values,
 * and the float map rows.  homogeneous: nplanes x 5 (t, chi, lambda, a, z of
 * the FLRW reference ray at each surface, hmaps.cpp:302-333; the dr / dl /
 * dt / da / dz / ds rows are relative to them).  maps: nmaps * nplanes rows of
 * npix floats, row nmaps * iz + r for surface iz (the reference's map vector
 * order, columns in the order of `pixels`).  A pixel whose surface crossing
 * is unusable has 0 in every row of that surface, as in the reference. */
int mpf_hmaps_fill(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t nside, int64_t npix,
                   const int64_t* pixels, int ncomp, const int* components, const double* homogeneous, float* maps);

/* Same with jacobiantype = "bundle" (Lensing::dbetadtheta, src/lensing.h:148-336;
 * FillMap hmaps.h:653-695, 725-747): four extra rays per pixel on a screen at
 * +-tan(openingmin) (radians) around the pixel direction, integrated with the
 * stop criterion stop_bundle (an mpf_stop other than MPF_STOP_S, which the
 * reference's dbetadtheta does not accept either) to the central ray's value
 * of that quantity at each surface; the screen normal is the central ray's
 * direction (plane_sachs = 1, the reference's plane = "sachs") or position
 * (0, "normal").  With MPF_STOP_PLANE each surface stops the four rays on the
 * plane through the central ray's crossing point normal to that screen normal
 * (lensing.h:201, 281-294: kiTarget . position = kiTarget . posTarget).  Lensing gives 5
 * rows per surface: kappa, gamma1, gamma2, w (image rotation), 1/mu. */
int mpf_hmaps_fill_bundle(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t nside, int64_t npix,
                          const int64_t* pixels, int ncomp, const int* components, const double* homogeneous,
                          int plane_sachs, int stop_bundle, double openingmin, float* maps);

/* RING pixel centres computed on the device (the directions mpf_hmaps_fill
 * launches): vec[3n]. */
int mpf_pix2vec_ring(int64_t nside, int64_t n, const int64_t* pixels, double* vec);

/* ------------------------------------------------------------------------ */
/* Cone octree construction from simulation cells (create_octree, ASCII)     */
/* ------------------------------------------------------------------------ */
typedef struct {
    double cone_vertex[3], cone_base[3], cone_angle;   /* the cone the cells are kept in (Input::collide) */
    double sphere_center[3], sphere_radius;            /* the microsphere around the observer */
    const double* rotm1;       /* 3x3 row-major rotation of a narrow cone's cells, or NULL (full sky) */
    double h, omegam, lboxmpch, mpc;
    int coarseonly;            /* keep only the cells of file level ncoarse */
    int ncoarse;
    int correction;            /* 1: refined non-normal dphidt / rho from the parents, incomplete octs
                                  completed; 0: the parents of refined cells with a non-normal rho and
                                  the incomplete octs coarsened (input.h:1413-1482) */
    int coarsecorrection;      /* coarse non-normal densities from their neighbours */
    int acorrection;           /* 1: each cell's a snapped to the next lower value of the table of the
                                  cells' distinct scale factors, extended one shell below (Full Universe
                                  Run outputs, input.h:1485-1506) */
    int order;                 /* gather of the completed children: 0 NGP, 1 CIC, 2 TSC (the reference's ORDER) */
    double* amin;              /* acorrection: receives the table's first value (Input::correct's amin);
                                  may be NULL, left unchanged otherwise */
} mpf_cells_params;

/* Create_octree::PreparationASCII's per-cone body (src/create_octree.h:544-580):
 * Input::importascii (src/input.h:996-1067) of the cell rows with the cone /
 * sphere filter, Miscellaneous::correctOctree (src/miscellaneous.h:467-479:
 * Input::sistemize, SimpleHyperOctree::update, Input::correct, dphidt * da/dt)
 * on the device.  rows: n x 10 floats (level, x, y, z, rho, phi, force x y z,
 * a) as the reference reads them; records: capacity x 48-byte cone records,
 * sorted by key (what Input::save writes); count: the cells produced. */
int mpf_cells_build(const float* rows, int64_t n, const mpf_cells_params* cp, const mpf_cosmology* c, void* records,
                    int64_t capacity, int64_t* count);
/* The completion of incomplete octs in the calling thread's last
 * mpf_cells_build (Input::correct's sequential appends, src/input.h:1451-1482,
 * run as waves of independent gathers): info[0] incomplete cells, info[1]
 * children filled in waves, info[2] waves run, info[3] children filled in
 * order on one thread after them (MPF_COMPLETION_WAVES in the environment
 * caps the waves, default 32; 0 fills every child in order).  No counterpart
 * in the reference. */
int mpf_cells_completion_info(int64_t* info);
/* The reference's ASCII cell reads (stream >> unsigned >> 9 floats): text of
 * length bytes -> rows[count x 10] (capacity rows at most). */
int mpf_cells_parse(const char* text, int64_t length, float* rows, int64_t capacity, int64_t* count);

/* ------------------------------------------------------------------------ */
/* Ray bundles (the rays driver)                                             */
/* ------------------------------------------------------------------------ */
typedef struct {
    int count;                 /* nbundle: photons on the circle around each central photon */
    double angle;              /* opening: half-angle of the bundle's cone (radians) */
    int interpolation;         /* stop_ray, the reference parameter the bundle rays are compared at:
                                  MPF_STOP_REDSHIFT, _A (1/a - 1), _T, _LAMBDA or _RADIUS (distance from
                                  the start); any other value is read as redshift, as the reference does */
    double amin;               /* 0, or the scale factor (of the data) every ray must reach */
    int64_t capacity;          /* trajectory points kept per ray; a longer ray is an error */
    int homogeneous_level;     /* -1: the octree's field; >= 0: the FLRW reference of the rays driver
                                  (Order = -1 on a uniform octree of this level, rays.cpp:246-249,
                                  integrator.h:497-500), always with the reference float64 order */
} mpf_bundle_params;

#define MPF_TRAJECTORY_FIELDS 29

/* Integrator::propagate (src/integrator.h:861-1015), the per-photon body of
 * the rays driver (src/rays.cpp:278, 322), for n central photons:
 * photons[6n] = start x y z and direction dtdl-normalised as launched (dxdl
 * dydl dzdl, not renormalised); rotation[n] (may be NULL: 0) the circle's
 * rotation.  Each bundle (the photon and `count` photons at `angle` around it,
 * Integrator::launch integrator.h:346-380) is integrated without a stop
 * criterion (integrator.h:477-618), checked, and the central ray's angular
 * diameter distance computed.  Outputs: sizes[n] = central trajectory size (0
 * when the bundle is rejected), central[n x capacity x 29] = its points in the
 * trajectory file's column order (index a t x y z dtdl dxdl dydl dzdl level ah
 * rho phi dphidx dphidy dphidz dphidl laplacian redshift dsdl2 error distance
 * isw iswold chi lambda dphidt s; src/output.h:200-211, README 6.3).
 * p: length, nsteps, order, exact, max_steps (stop, planes, Jacobian unused). */
int mpf_rays_propagate(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, const mpf_bundle_params* bp,
                       int64_t n, const double* photons, const double* rotation, int64_t* sizes, double* central);

/* ------------------------------------------------------------------------ */
/* Learned field surrogate                                                   */
/* ------------------------------------------------------------------------ */
/* A per-cone neural field that stands in for the octree gather
 * (SimpleHyperOctree::tsc / cic, src/magrathea/simplehyperoctree.h:1410-1644)
 * inside the RK4 stages of Integrator::integrate (src/integrator.h:648-824).
 * It has no counterpart in the reference; the octree path stays its check and
 * fallback.  Network: (x, y, z, a) normalised to [-1, 1]^4 -> 64 Fourier
 * frequencies (sin, cos: 128 features) -> 4 hidden layers of 128 with SiLU ->
 * 5 outputs (phi, dphidx, dphidy, dphidz, dphidt), BF16 weights and FP32
 * accumulation on the tensor cores at inference, FP32 training. */
typedef struct mpf_surrogate mpf_surrogate;

#define MPF_SURROGATE_PARAMS 68112   /* W1 b1 W2 b2 W3 b3 W4 b4 (128x128, 128) W5 (16x128) b5 (16); W row-major [out][in] */
#define MPF_SURROGATE_NORM 274       /* lo[4] sc[4] freq[64][4] mean[5] std[5]: u = (p - lo) * sc - 1, s_j = freq_j . u */

typedef struct {
    double tan_half[2];        /* tangents of the cone's half-openings about +x, in y and z */
    double r_min, r_max;       /* radial range of the training samples (octree units) */
    double a_min, a_max;       /* range of the scale-factor input */
    double freq_sigma[4];      /* standard deviation of the Fourier frequencies (cycles over the
                                  normalised range [-1, 1]) for x, y, z, a */
    uint64_t seed;             /* frequencies, initial weights and the sample stream */
} mpf_surrogate_domain;

typedef struct {
    int64_t samples;           /* training samples (a fresh batch per step, samples / batch steps) */
    int64_t batch;             /* >= 256 */
    double lr;                 /* Adam learning rate, cosine decay to lr / 100 */
    int64_t stat_samples;      /* samples for the output normalisation (mean / std) */
} mpf_surrogate_train_params;

typedef struct {
    double loss_first, loss_last;   /* mean normalised loss over the first / last 1% of the steps */
    int64_t steps;
    double seconds;
    double samples_per_second;
    int kernel_launches_per_step;   /* kernels in the captured training step */
} mpf_surrogate_train_stats;

typedef struct {
    double tolerance;          /* relative drift of the checkpointed deflection that flags a photon */
    int check_every;           /* octree re-check period in RK4 steps (>= 1) */
    int fallback;              /* 1: flagged photons are re-run on the plain octree path in the call */
} mpf_surrogate_prop_params;

typedef struct {
    int64_t photon_steps;      /* RK4 steps taken with the surrogate */
    int64_t flagged_photons;
    int64_t fallback_photons;  /* re-run on the octree */
    int64_t fallback_steps;
    double surrogate_seconds;  /* device time of the surrogate launch */
    double fallback_seconds;
} mpf_surrogate_prop_stats;

int mpf_surrogate_create(const mpf_surrogate_domain* d, mpf_surrogate** out);
void mpf_surrogate_destroy(mpf_surrogate* s);
/* Draw `samples` points uniform in the cone and fit the network to the
 * octree's TSC field there (MSE on outputs normalised by their mean / std). */
int mpf_surrogate_train(mpf_surrogate* s, const mpf_octree* o, const mpf_surrogate_train_params* p,
                        mpf_surrogate_train_stats* stats);
/* n training samples of the stream from index `first`: inputs n x 4 (x y z a),
 * targets n x 5 (phi dphidx dphidy dphidz dphidt from the octree's TSC). */
int mpf_surrogate_sample(const mpf_surrogate* s, const mpf_octree* o, uint64_t first, int64_t n, float* inputs,
                         float* targets);
/* Parameters (MPF_SURROGATE_PARAMS floats) and normalisation (MPF_SURROGATE_NORM
 * floats); either pointer may be NULL. */
int mpf_surrogate_get_params(const mpf_surrogate* s, float* params, float* norm);
int mpf_surrogate_set_params(mpf_surrogate* s, const float* params, const float* norm);
/* Training loss and its gradient (MPF_SURROGATE_PARAMS floats) on a given
 * batch, through the training kernels. */
int mpf_surrogate_loss_grad(mpf_surrogate* s, int64_t n, const float* inputs, const float* targets, double* loss,
                            float* grad);
/* Network outputs (n x 5) through the tensor-core inference path. */
int mpf_surrogate_eval(mpf_surrogate* s, int64_t n, const float* inputs, float* out);
/* Integrator::integrate with the surrogate in the RK4 stages (no surfaces, no
 * Jacobian): p gives length, nsteps, order (of the octree re-checks), stop and
 * stop_value, max_steps; launch[6n] as mpf_propagate.  Outputs (host):
 * steps[n], final_rec[28n] (may be NULL; rho and ah are 0 for surrogate
 * photons), flags[n] (bit 0: drift above tolerance, bit 1: max_steps),
 * drift[n] (may be NULL).  With sp->fallback, flagged photons' steps and
 * records come from the plain octree path (mpf_propagate, FP32 gathers). */
int mpf_surrogate_propagate(mpf_surrogate* s, const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p,
                            const mpf_surrogate_prop_params* sp, int64_t n, const double* launch, int64_t* steps,
                            double* final_rec, uint8_t* flags, float* drift, mpf_surrogate_prop_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
