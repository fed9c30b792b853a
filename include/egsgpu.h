/*
 * egsgpu -- C ABI of the GB300 voxel-dose transport engine.
 *
 * This is the drop-in boundary for EGSnrc's particle-history loop on the
 * egs++ EGS_XYZGeometry / DOSXYZnrc path.  Each entry point names the
 * reference interface it replaces (paths relative to HEN_HOUSE).  Every
 * function returns an int status (0 = ok, >0 = error class, see
 * EGSGPU_ERR_*); nothing calls exit().  The library owns all device
 * buffers; the caller owns every host array passed in (copied on entry).
 * One handle per host thread; handles are independent.
 */
#ifndef EGSGPU_H
#define EGSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EGSGPU_OK 0
#define EGSGPU_ERR_ARG 1       /* bad argument / unsupported option            */
#define EGSGPU_ERR_DATA 2      /* data file missing or malformed                */
#define EGSGPU_ERR_MEDIUM 3    /* medium not found / inconsistent PEGS4 block   */
#define EGSGPU_ERR_CUDA 4      /* CUDA runtime error                            */
#define EGSGPU_ERR_CAPACITY 5  /* particle queue capacity exceeded              */
#define EGSGPU_ERR_LOOP 6      /* a device loop hit its iteration cap           */
#define EGSGPU_ERR_STATE 7     /* call order violated (e.g. run before media)   */

typedef struct egsgpu_handle egsgpu_handle;

/* Transport parameters: the egs++ ":start MC transport parameter:" block
 * (egs++/egs_advanced_application.cpp:482-562) restricted to the physics
 * profile this engine implements (PRESTA-II, EXACT or PRESTA-I BCA, spin off,
 * bound Compton norej, Rayleigh on, EADL relaxation, Sauter photo-electrons,
 * BH brems with KM angles, BH pair with simple angles). */
typedef struct {
    double ecut;          /* global electron cut-off, total energy (MeV)   */
    double pcut;          /* global photon cut-off (MeV)                    */
    double estepe;        /* max fractional energy loss per step (0.25)     */
    double ximax;         /* max first GS moment per step (0.5)             */
    double skindepth;     /* skin depth for BCA in elastic MFPs (3)         */
    int precision;        /* 32: FP32 transport (FP64 tallies); 64: FP64    */
    int block_size;       /* threads per CTA for the transport kernels; 0 = default */
    int ctas_per_sm;      /* resident CTAs per SM; 0 = default                       */
    long long chunk;      /* histories per wavefront chunk; 0 = automatic   */
    long long capacity;   /* particle-queue capacity per queue; 0 = automatic: the largest power of two
                             up to 2^27 whose four queues fit in a sixth of the free device memory */
    int requeue_lanes;    /* a warp whose queue is empty parks its particles for the
                             next round once this few lanes are busy; <= 0 = never
                             (default; results are identical either way) */
    int use_graph;        /* 1: replay the wavefront rounds from a CUDA graph, four
                             rounds per host check of the queues; 2: one graph
                             launch per chunk whose conditional WHILE node repeats
                             the rounds on the device until the queues drain (no
                             host round trips inside a chunk); 0: direct launches
                             with CUDA events around every kernel.  Graphs give
                             no per-kernel timing; results are identical */
    int inter_batch;      /* lanes of a warp due to interact before their interactions
                             are sampled together; 0 = default (8 electron, 12 photon
                             lanes), -1 = immediately (results are identical either way) */
    int howfarless;       /* 1: DOSXYZnrc HOWFARLESS transport (ihowfarless,
                             user_codes/dosxyznrc/dosxyznrc.mortran:425-455) for a
                             homogeneous phantom: particles see only its outer
                             faces, charged-particle steps deposit along a two-segment
                             hinge path, step limits floored at half the smallest
                             voxel size.  Refused for inhomogeneous phantoms, several
                             phantoms and the adjoint. */
    double smax;          /* maximum charged-particle step (cm): egs++ "Global Smax"
                             (egs++/egs_advanced_application.cpp:487), the smaxir
                             limit on tmxs in ELECTR (src/egsnrc.mortran:1179);
                             <= 0 = no limit (1e10 cm, src/egsnrc.macros:2269) */
    int bca_algorithm;    /* boundary crossing: 0 EXACT (default), 1 PRESTA-I: egs++
                             "Boundary crossing algorithm" (bca_algorithm,
                             src/egsnrc.mortran:2782-2783, 1247-1345).  With
                             PRESTA-I a skindepth <= 1e-4 selects the old PRESTA
                             default from the lowest ECUT (:2794-2815).  PRESTA-I
                             is for egsgpu_run and egsgpu_run_phantoms (not with
                             HOWFARLESS, the adjoint or egsgpu_run_noalloc). */
    int loop_cap;         /* iterations after which a device rejection loop is
                             abandoned; 0 = default (100000).  The reference's
                             analogues: the 100000-try limit of
                             simulateSingleShower (egs++/egs_application.cpp:
                             925-930) and loopMax (egs++/egs_functions.h:96) */
    int step_cap;         /* transport steps after which a particle is abandoned;
                             0 = default (2^22).  Either cap, once reached, makes
                             the run return EGSGPU_ERR_LOOP (the caps are set on
                             the device before each run: handles on one device
                             whose runs overlap share the last caps set) */
    int fp64_near_faces;  /* FP32 transport only: 1 computes the electron steps
                             that start within 2^-12 cm of a voxel face or may end
                             the range in FP64 (distances to the faces, residual
                             range, energy loss), in a kernel of its own; 0 =
                             default (FP32 throughout; FP64 dose tallies either
                             way).  For EXACT voxel transport (egsgpu_run,
                             egsgpu_run_phantoms): PRESTA-I, HOWFARLESS and the
                             adjoint ignore it, egsgpu_run_noalloc refuses it */
} egsgpu_config;

/* Source: egs++ EGS_ParallelBeam (sources/egs_parallel_beam) with a point
 * or rectangle shape (shapes/egs_rectangle) and a monoenergetic or
 * histogram spectrum (egs_spectra.cpp:491-740), or (shape 2) a phase-space
 * source: egs++ EGS_PhspSource / DOSXYZnrc isource 2
 * (sources/egs_phsp_source/egs_phsp_source.cpp:284-440). */
typedef struct {
    int charge;           /* -1 e-, 0 photon, +1 e+                          */
    int shape;            /* 0 point, 1 rectangle in the plane z = pos[2]    */
    double pos[3];        /* point position / plane z                        */
    double xmin, xmax, ymin, ymax;   /* rectangle extent                     */
    double dir[3];        /* beam direction (normalised on entry)            */
    int spectrum;         /* 0 monoenergetic, 1 histogram (counts per MeV)   */
    double energy;        /* kinetic energy for spectrum 0 (MeV)             */
    int nbins;            /* spectrum 1: number of bins                       */
    const double *edges;  /* spectrum 1: nbins+1 bin edges (MeV)              */
    const double *weights;/* spectrum 1: nbins values, counts per MeV         */
    /* shape 2: nphsp particles of 7 floats {charge, kinetic energy (MeV),
     * x, y, u, v, weight}, as in an .egsphsp file: a negative weight means a
     * negative w.  Particle i starts at (x + pos[0], y + pos[1], pos[2]) with
     * direction (u, v, +-sqrt(1 - u^2 - v^2)); history h uses particle
     * (h / (recycle + 1)) mod nphsp with weight |weight| / (recycle + 1).
     * dir, spectrum and energy are ignored. */
    long long nphsp;
    const float *phsp;
    int recycle;
    /* shape 2: a rotation R (row-major) applied to every particle before pos
     * is added, as egs++ EGS_TransformedSource applies its affine transform
     * (egs++/sources/egs_transformed_source, egs++/egs_transformations.h:
     * 480-540): the particle at (x, y, 0) with direction (u, v, w) starts at
     * R (x, y, 0) + pos with direction R (u, v, w).  All nine zero: no
     * rotation.  Must be zero for shapes 0 and 1. */
    double rot[9];
} egsgpu_source;

/* Default configuration (the egs_set_defaults profile, FP32 transport). */
void egsgpu_default_config(egsgpu_config *cfg);

/* Creates a handle on the current CUDA device.
 * Replaces egsInit + egs_set_defaults (interface/egs_interface2.h:712-740,
 * src/egs_utilities.mortran:896). */
int egsgpu_create(const egsgpu_config *cfg, egsgpu_handle **out);

/* Reads the PEGS4 blocks of the named media and builds every table
 * (XCOM photon cross sections, MS surface, Compton shells, photo edges).
 * Replaces egsAddMedium + egsHatch (interface/egs_interface2.h:760-790;
 * src/egsnrc.mortran:1828 HATCH). Medium k of `names` is medium index k. */
int egsgpu_load_media(egsgpu_handle *h, const char *data_dir, const char *pegs_file,
                      const char *const *names, int n);

/* Properties of loaded medium `index`: out[4] = {PEGS4 density (g/cm^3),
 * AE, AP (MeV), number of elements}. Replaces reading the MEDIA/THRESH
 * COMMON blocks (interface/egs_interface2.h:108-692: the_media, the_thresh). */
int egsgpu_get_medium(egsgpu_handle *h, int index, double *out);

/* Voxel phantom: plane positions (nx+1, ny+1, nz+1, cm), medium index and
 * relative density per voxel, voxel index ix + iy*nx + iz*nx*ny.
 * Replaces EGS_XYZGeometry construction and the egsHowfar/egsHownear/
 * egsStartParticle callbacks (egs++/geometry/egs_nd_geometry/egs_nd_geometry.h:769-1379,
 * egs++/egs_advanced_application.cpp:1351-1442). */
int egsgpu_set_xyz_geometry(egsgpu_handle *h, int nx, int ny, int nz, const double *xb,
                            const double *yb, const double *zb, const int32_t *med,
                            const double *rhor);

/* Replaces EGS_BaseSource::getNextParticle for the parallel-beam source
 * (egs++/egs_base_source.h:684, sources/egs_parallel_beam/egs_parallel_beam.h:150). */
int egsgpu_set_source(egsgpu_handle *h, const egsgpu_source *src);

/* Transports histories [first, first+n) in n_batch statistical batches with
 * Philox streams keyed by (seed, history index); results are independent
 * of chunking. Accumulates into the handle's tallies (call egsgpu_reset to
 * clear). `stream` is a cudaStream_t or NULL for the default stream; the
 * call returns after the work on it has completed.
 * Replaces EGS_Application::runSimulation / simulateSingleShower / egsShower
 * (egs++/egs_application.cpp:839-959, interface/egs_interface2.c:92-99). */
int egsgpu_run(egsgpu_handle *h, long long first, long long n, int n_batch, uint32_t seed,
               void *stream);

/* Clears tallies and counters. */
int egsgpu_reset(egsgpu_handle *h);

/* Per-voxel tallies over all batches run so far: sum of batch energy
 * deposits and sum of their squares (MeV, FP64), plus totals[8] =
 * {histories, batches, deposited, escaped, steps, photon steps, electron steps, pushes}.
 * Any pointer may be NULL. Replaces EGS_ScoringArray / DOSXYZ endep,endep2
 * (egs++/egs_scoring.h:219-390, user_codes/dosxyznrc/dosxyznrc.mortran:1229-1235). */
int egsgpu_get_tallies(egsgpu_handle *h, double *edep_sum, double *edep2_sum, double *totals);

/* Dose per source particle (Gy) and its 1-sigma uncertainty (Gy) from the
 * batch tallies: D = E*1.602e-10/(rho*V*N). Replaces
 * EGS_DoseScoring::reportResults/outputDoseFile
 * (ausgab_objects/egs_dose_scoring/egs_dose_scoring.cpp:309-480). */
int egsgpu_get_dose(egsgpu_handle *h, double *dose, double *sigma);

/* Several independent dose problems transported together.  The reference
 * runs one problem per process (an egs++ application with one geometry and
 * one source, egs++/egs_application.cpp:839-959; parallel jobs are separate
 * processes combined afterwards, egs_application.cpp:624).  Here every
 * phantom keeps its own geometry, source, Philox seed and history count, and
 * all phantoms share each wavefront, so small problems fill the GPU together.
 * Phantom k's results equal those of runs of its own with the same seed,
 * history ranges and batch count. */
typedef struct {
    int nx, ny, nz;
    const double *xb, *yb, *zb;     /* nx+1, ny+1, nz+1 plane positions (cm) */
    const int32_t *med;             /* medium index per voxel (x fastest)   */
    const double *rhor;             /* relative density per voxel           */
    egsgpu_source source;
    uint32_t seed;                  /* Philox seed of this phantom          */
    long long histories;            /* histories per egsgpu_run_phantoms   */
} egsgpu_phantom;

/* Replaces the single geometry and source by n phantoms (host arrays are
 * copied).  Until the next egsgpu_set_xyz_geometry, egsgpu_run and
 * egsgpu_get_dose return EGSGPU_ERR_STATE, and egsgpu_get_tallies returns
 * the phantoms' voxels laid end to end (offsets from egsgpu_get_phantom_info). */
int egsgpu_set_phantoms(egsgpu_handle *h, int n, const egsgpu_phantom *phantoms);
/* Transports every phantom's next `histories` histories in n_batch batches,
 * all phantoms in the same wavefronts (each batch: the same history split as
 * egsgpu_run).  The first call runs histories [0, n_k) of phantom k, the
 * second [n_k, 2 n_k), and so on. */
int egsgpu_run_phantoms(egsgpu_handle *h, int n_batch, void *stream);
/* Dose (Gy per source particle) and 1-sigma of phantom k. */
int egsgpu_get_phantom_dose(egsgpu_handle *h, int k, double *dose, double *sigma);
/* out[3] = {first global voxel index, voxels, histories run so far} of phantom k. */
int egsgpu_get_phantom_info(egsgpu_handle *h, int k, long long *out);

/* Gradient of a loss of the dose with respect to the voxels' relative
 * densities (rhor; the mass density is rhor times the medium's PEGS4
 * density).  The handle's tallies must hold exactly the run being
 * differentiated: histories [first, first+n) with `seed`, since the last
 * reset.  dL_dD[nvox] is the loss's derivative with respect to that run's dose
 * (Gy per particle, as from egsgpu_get_dose); dL_drhor[nvox] receives
 * dL/d(rhor).  The histories are replayed from their seeds twice (no paths
 * are stored): first to weigh each history's deposits by dL/dE, then with
 * adjoint kernels that add the photon path scores (attenuation and
 * interaction likelihoods scale with rhor) and the pathwise term of the
 * electrons' continuous energy loss; the dose's explicit 1/rhor factor is
 * added on the host.  No counterpart in the reference (which has no
 * derivatives); the density scaling it differentiates is the reference's
 * RHOF (src/egsnrc.mortran PHOTON GMFP = GMFPR0/RHOF, ELECTR tstep/rhof,
 * interface/egs_c_interface2.macros:398). */
int egsgpu_adjoint(egsgpu_handle *h, long long first, long long n, uint32_t seed, const double *dL_dD,
                   double *dL_drhor);

/* Optional per-history deposited energy (MeV) for histories
 * [first, first+n) of the next egsgpu_run call (n <= 2^24); pass NULL to
 * disable. A checking aid with no counterpart in the reference API. */
int egsgpu_set_history_tally(egsgpu_handle *h, long long first, long long n);
int egsgpu_get_history_tally(egsgpu_handle *h, double *out);

/* Geometry queries on the handle's phantom (set by egsgpu_set_xyz_geometry),
 * computed on the GPU by the transport kernels' own geometry functions in the
 * handle's precision.  A checking aid: each op is the EGS_XYZGeometry method
 * it replaces (egs++/geometry/egs_nd_geometry/egs_nd_geometry.h):
 *   op 0  isWhere (:791-805): inew[i] = region of point x[3i..3i+2], -1 outside;
 *   op 1  howfar (:963-1104), or howfarFromOut (:1281-1379) when ireg[i] < 0:
 *         from region ireg[i] at x along unit direction u[3i..3i+2] within
 *         t[i]; inew[i] = region entered (ireg[i] when no face is within t[i],
 *         -1 when leaving), t[i] = the distance (in/out);
 *   op 2  hownear (:1106-1122): t[i] = distance from x to the nearest face of
 *         region ireg[i] (>= 0).
 * Arrays of the ops that do not use them may be NULL; region indices beyond
 * the phantom are EGSGPU_ERR_ARG. */
int egsgpu_geometry_query(egsgpu_handle *h, int op, long long n, const int32_t *ireg, const double *x,
                          const double *u, double *t, int32_t *inew);

/* Device-side profile of the runs since the last reset: out[20] =
 * {ms source, ms photon, ms electron, ms batch, launches of each (4),
 *  photon steps, electron steps, photon-kernel pushes, electron-kernel pushes,
 *  photon interactions, electron interactions, autotuned chunk, graph in use
 *  (0 none, 1 round replay, 2 device-side loop),
 *  mean busy lanes per warp iteration in the photon and electron kernels,
 *  electron steps of the FP32 build computed in FP64 near a voxel face or
 *  the end of the range, launch shape chosen by the autotuner (-1: none yet;
 *  0..5 = threads per CTA / resident CTAs per SM of the photon and electron
 *  kernels relative to the most that fit: 128/0/0, 64/0/0, 96/0/0, 128/0/-1,
 *  128/-2/0, 64/0/-2)};
 * times are CUDA-event
 * durations on the launch stream.  No counterpart in the reference API
 * (the reference reports CPU time per batch, egs++/egs_timer.cpp). */
int egsgpu_get_profile(egsgpu_handle *h, double *out);

/* Checkpoint / restore of the run state (tallies, counters, next history
 * index). Replaces the .egsdat output/readData pair
 * (egs++/egs_application.cpp:482-560). `size` is in/out. */
int egsgpu_checkpoint(egsgpu_handle *h, void *buf, size_t *size);
int egsgpu_restore(egsgpu_handle *h, const void *buf, size_t size);

/* Combines the checkpoints of two shards of one problem (same phantom,
 * disjoint history ranges or seeds) into the checkpoint of their union:
 * histories, batches, energy totals, counters and the per-voxel batch sums
 * and sums of squares add, as the reference sums parallel jobs' .egsdat files
 * (egs++/egs_application.cpp:624-660, combineResults/addState).  Host only:
 * needs no GPU and no handle.  Shards with different histories per batch are
 * EGSGPU_ERR_ARG (batch-wise uncertainties need equal batches).  out may be
 * NULL to query *nout; `out` may alias `a`.  Restore the result with
 * egsgpu_restore to read doses. */
int egsgpu_combine_checkpoints(const void *a, size_t na, const void *b, size_t nb, void *out, size_t *nout);

/* No-allocation transport, for callers that may not allocate device memory
 * while they run: a real-time loop that must not block on the allocator, or a
 * host framework that owns every allocation (its memory pool) and forbids
 * others.  This entry point has no counterpart in the reference API.
 *
 * Transports histories [first, first+n) exactly as egsgpu_run would (same
 * random-number streams, same physics) and writes this call's deposited
 * energy per voxel (MeV, FP64) into `dose`, a caller-owned device array of
 * nx*ny*nz doubles on the current device, overwriting it.  The handle's
 * tallies are not touched.  The particle queues live in a fixed file-scope
 * device array of EGSGPU_NOALLOC_SCRATCH_MIB MiB that every GPU loading the
 * library holds until the process exits; the call makes no cudaMalloc or
 * cudaFree and creates no stream or event.  At most
 * EGSGPU_NOALLOC_MAX_HISTORIES histories per call (larger n is rejected with
 * EGSGPU_ERR_ARG); a chunk whose secondaries overflow the queues returns
 * EGSGPU_ERR_CAPACITY.  All work is ordered on `stream` (NULL = default
 * stream); the call synchronises that stream once per wavefront round, to
 * learn whether the queues have drained, and returns after the work
 * completes.  Block size, CTAs per SM and interaction batching are taken
 * from the handle's configuration as egsgpu_run takes them; the HOWFARLESS
 * and PRESTA-I options are refused (EGSGPU_ERR_ARG).  The call cannot be
 * recorded into a CUDA graph: on a stream that is capturing it returns
 * EGSGPU_ERR_STATE at once, before any other CUDA call, and the capture stays
 * valid.  The first call on each device looks up the array's device address
 * with cudaGetSymbolAddress.  Every call shares the
 * one array: calls that overlap on the GPU (from several threads, streams
 * or handles) race and must be serialised by the caller.  The handle's
 * media, geometry and source must have been set (those calls allocate). */
#define EGSGPU_NOALLOC_SCRATCH_MIB 40
#define EGSGPU_NOALLOC_MAX_HISTORIES 2048
int egsgpu_run_noalloc(egsgpu_handle *h, long long first, long long n, uint32_t seed, double *dose,
                       void *stream);

/* Phase-space files, the particle input of egs++ EGS_PhspSource and
 * IAEA_PhspSource and of DOSXYZnrc isource 2 (host only: needs no GPU and no
 * handle).  Reads the header, and records [first, first+count), of
 *   - a BEAMnrc .egsphsp file, MODE0 or MODE2
 *     (egs++/sources/egs_phsp_source/egs_phsp_source.cpp:77-160 header,
 *     :364-423 records), or
 *   - an IAEA phase-space pair <name>.IAEAheader + <name>.IAEAphsp
 *     (egs++/sources/iaea_phsp_source/iaea_phsp_source.cpp:77-224, :310-417;
 *     HEN_HOUSE/iaea_phsp/iaea_header.cpp:60-330, iaea_record.cpp:145-230);
 *     `path` is <name>, with or without either extension.
 * Each particle becomes the 7 floats egsgpu_source.phsp takes: charge,
 * kinetic energy (MeV), x, y, u, v, weight (negative when w < 0).
 * `particles` (7*count floats), `latch` (count; 0 where the file stores no
 * LATCH) and `new_history` (count; 1 for the first particle of an incident
 * history) may each be NULL; count = 0 reads the header only.  Files written
 * with the other byte order are read.  A file whose size disagrees with its
 * header, or an IAEA record of a neutron or proton, is EGSGPU_ERR_DATA.  The
 * message of a failed call is egsgpu_last_error(NULL) on the same thread. */
typedef struct egsgpu_phsp_info {
    int format;          /* 0 egsphsp MODE0, 1 egsphsp MODE2, 2 IAEA             */
    int has_latch;       /* the records carry an EGS LATCH                       */
    long long n;         /* particles in the file                                */
    long long photons;   /* photons in the file                                  */
    double incident;     /* incident histories that made the file                */
    double ekmax;        /* maximum kinetic energy (MeV); 0 if the header has none */
    double zmin, zmax;   /* z of the records read: 0 for egsphsp (the scoring
                            plane); for IAEA the constant Z, or the range of the
                            stored Z (NaN when only the header was read)       */
} egsgpu_phsp_info;
int egsgpu_read_phsp(const char *path, long long first, long long count, egsgpu_phsp_info *info,
                     float *particles, uint32_t *latch, unsigned char *new_history);

/* Last error message of the handle (never NULL); with a NULL handle, the
 * last error of a host-only call (egsgpu_read_phsp) on this thread. */
const char *egsgpu_last_error(egsgpu_handle *h);

void egsgpu_destroy(egsgpu_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* EGSGPU_H */
