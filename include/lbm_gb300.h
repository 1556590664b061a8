/*
 * lbm_gb300 -- C ABI of the GB300 lattice-Boltzmann engine (liblbm_gb300.so).
 *
 * The reference has no plugin interface: its API is the C++ class surface
 * Geometry(file, velSet, spacing, raydir) -> SubDomain(Geometry&) ->
 * Simulation(SubDomain&, tau, pressure, dt) with public step methods
 * (Simulation.h:26-50), Boundary::ApplyBc(double&) (Boundary.h:22) and
 * ConfigReader (ConfigReader.h:9-12).  Each entry point below names the
 * reference code it replaces.  The C++ classes in the package's host layer
 * keep the reference names and call these functions.
 *
 * Conventions
 *   - Every call returns lbm_status: 0 on success, a negative code on error.
 *     lbm_last_error(h) describes the last failure of a handle;
 *     lbm_last_global_error() the last failure of a call without a handle.
 *   - Host buffers are caller-owned; the library copies in and out.
 *   - Lattice point n = (k*ny + j)*nx + i (x fastest).  Arrays "per active
 *     node" list the non-solid points in increasing n.
 *   - One CUDA stream per handle.  A handle is not thread-safe; distinct
 *     handles may be driven from distinct threads.  No C++ exception crosses
 *     this interface.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int lbm_status;

#define LBM_OK 0
#define LBM_ERR_ARG (-1)       /* invalid argument */
#define LBM_ERR_CUDA (-2)      /* CUDA runtime error (message names the call) */
#define LBM_ERR_STATE (-3)     /* call out of order (e.g. step before geometry) */
#define LBM_ERR_NONFINITE (-4) /* a density became NaN/Inf: the run diverged */
#define LBM_ERR_ALLOC (-5)     /* device or host allocation failed */
#define LBM_ERR_IO (-6)        /* checkpoint / file error */
#define LBM_ERR_UNSUPPORTED (-7)

/* Lattices and precisions. */
#define LBM_D3Q19 19
#define LBM_D3Q27 27
#define LBM_F64 0   /* FP64 storage and arithmetic (oracle-grade) */
#define LBM_F32 1   /* FP32 storage and arithmetic */
#define LBM_F16 2   /* FP16 offsets (f - w)/w * 1024, FP32 arithmetic */
#define LBM_BF16 3  /* BF16 offsets (f - w)/w, FP32 arithmetic */

/* Semantics.
 * LBM_PARITY reproduces the reference step exactly (Simulation.cpp:569-601):
 *   collision on every non-solid node; push streaming that keeps a
 *   destination's previous value when the link comes from solid or the
 *   post-collision value is exactly zero (Simulation.cpp:211-237); Zou-He
 *   formulas of Boundary.cpp:129-157 and Simulation.cpp:628-838; the in-place
 *   wall rule of Simulation.cpp:843-863; wall shear stress from the
 *   post-boundary f and the same step's equilibrium, without the
 *   (1 - 1/2tau) factor (Simulation.cpp:880-898).
 * LBM_PHYSICS: half-way bounce-back for links from solid, Zou-He on any
 *   axis-aligned face, and wall shear stress from -(1 - 1/2tau) sum f_neq c c. */
#define LBM_PARITY 0
#define LBM_PHYSICS 1

/* Boundary condition kinds. */
#define LBM_BC_REF_INLET 1        /* Boundary::ApplyBc: x-min face, u = (v, 0, 0) */
#define LBM_BC_REF_OUTLET_YMAX 2  /* ApplyOutletBc outlet 1: y-max face, rho = 1 */
#define LBM_BC_REF_OUTLET_ZMIN 3  /* ApplyOutletBc outlets 2/3: z-min face, rho = 1 */
#define LBM_BC_VELOCITY 4         /* Zou-He velocity, normal inflow, any face */
#define LBM_BC_PRESSURE 5         /* Zou-He pressure (density = value), any face */

/* Faces: the boundary sits on this side of the fluid. */
#define LBM_FACE_XMIN 0
#define LBM_FACE_XMAX 1
#define LBM_FACE_YMIN 2
#define LBM_FACE_YMAX 3
#define LBM_FACE_ZMIN 4
#define LBM_FACE_ZMAX 5

/* Boundary-condition rules per handle (an ensemble packs one inlet and one
 * outlet rule per member into one lattice). */
#define LBM_MAX_BC 256

#define LBM_COLLISION_BGK 0
#define LBM_COLLISION_REGULARIZED 1
/* Inlet waveforms per handle (lbm_set_waveform). */
#define LBM_MAX_WAVES 256

typedef struct lbm_handle lbm_handle;

/* ---------------------------------------------------------------------
 * Voxelization.  Replaces Geometry::GetSubBoundingBox + generatePointsInSubBox
 * + labelPoints (ComplexGeometry.cpp:133-214, 318-351, 978-1053).
 */
typedef struct {
    double spacing;
    /* 1: bbox, origin and dims follow the reference rule from the triangles
     *    (outputs); 0: bbox (used by the ray adjustment), origin and dims are
     *    inputs. */
    int reference_bbox;
    double bbox[6];   /* min_x, max_x, min_y, max_y, min_z, max_z */
    double origin[3]; /* coordinates of point (0,0,0) */
    int dims[3];      /* nx, ny, nz */
    int64_t fluid_count; /* output */
    int64_t ray_tests;   /* output: ray-triangle tests performed */
} lbm_vox_desc;

/* tri12: ntri rows of x1 y1 z1 x2 y2 z2 x3 y3 z3 nx ny nz (the STL's own facet
 * normal, Struct.h:117-125).  mask_out (nx*ny*nz bytes, 1 = Fluid) may be NULL
 * to query dims only.  The mask is bit-identical to the reference's. */
lbm_status lbm_voxelize(const double* tri12, int64_t ntri, lbm_vox_desc* desc, uint8_t* mask_out);

/* Parse an ASCII STL (GeometryReader.cpp:33-117).  With tri12 == NULL only
 * *ntri is set; otherwise up to *ntri rows are written. */
lbm_status lbm_read_stl_ascii(const char* path, double* tri12, int64_t* ntri);

/* ---------------------------------------------------------------------
 * Solver handle.  Replaces SubDomain + Simulation construction
 * (Subdomain.cpp:3-32, Simulation.cpp:3-15).
 */
typedef struct {
    int Q;             /* LBM_D3Q19 or LBM_D3Q27 */
    int precision;     /* LBM_F64 / LBM_F32 / LBM_F16 / LBM_BF16 */
    int mode;          /* LBM_PARITY or LBM_PHYSICS */
    double tau;        /* relaxation time, > 0.5 */
    double spacing;    /* lattice spacing (geometry units) */
    double origin[3];  /* coordinates of lattice point (0,0,0) */
    double wss_scale;  /* C of the wall shear stress (reference: 1060*dt^2/(s^2*1e-6)) */
    double tawss_div;  /* TAWSS = accumulated |tau| / tawss_div (reference: 0.9) */
    int device;        /* CUDA device ordinal */
    /* Physics mode: LBM_COLLISION_BGK (the reference's, Simulation.cpp:43-208)
     * or LBM_COLLISION_REGULARIZED (no reference counterpart: the
     * non-equilibrium part is projected on its second moment before
     * relaxing, which keeps flows stable at tau near 1/2 where BGK diverges).
     * Parity mode is always BGK. */
    int collision;
} lbm_desc;

lbm_status lbm_create(const lbm_desc* desc, lbm_handle** out);
lbm_status lbm_destroy(lbm_handle* h);
const char* lbm_last_error(const lbm_handle* h);
const char* lbm_last_global_error(void);

/* Boundary specification.  Boundary points (Fluid points with a neighbour
 * that is NotFluid or outside the box, ComplexGeometry.cpp:1259-1300) lying
 * on lattice plane `plane` of the face's axis get this condition; the first
 * matching entry wins; the remaining boundary points are walls.  plane = -1
 * selects the extreme fluid layer on that face. */
typedef struct {
    int kind;      /* LBM_BC_* */
    int face;      /* LBM_FACE_* (REF kinds imply their face) */
    int plane;     /* lattice index on the face axis, or -1 */
    double value;  /* velocity scale (velocity kinds) or density (pressure) */
    int profile;   /* 0 uniform, 1 parabolic 1 - (d1^2 + d2^2)/R^2 */
    double c1, c2; /* profile centre on the two transverse axes (x<y<z order) */
    double R;      /* profile radius */
    /* Region rule (the form of ComplexGeometry.cpp:1369-1409): when region
     * != 0 a boundary point matches if |its coordinate on the face axis -
     * coord| <= tol and lo[t] < coordinate < hi[t] on the two transverse axes
     * (x<y<z order); `plane` is then unused.  Coordinates are origin +
     * index * spacing. */
    int region;
    double coord, tol;
    double lo[2], hi[2];
    /* Velocity kinds: the waveform (lbm_set_waveform) whose amplitude scales
     * the velocity each step; 0 is the table of lbm_set_inlet_table. */
    int wave;
} lbm_bc_spec;

/* mask: nx*ny*nz bytes (nonzero = Fluid).  Builds classes, boundary lists,
 * next-to-wall nodes and per-link masks on the device
 * (Subdomain.cpp:91-218), then initialises f = w (Node.cpp:30-37). */
lbm_status lbm_set_geometry(lbm_handle* h, const uint8_t* mask, const int dims[3],
                            const lbm_bc_spec* bc, int nbc);

/* Wall / next-to-wall normals from the surface (Subdomain.cpp:224-370). */
lbm_status lbm_set_normals_from_surface(lbm_handle* h, const double* tri12, int64_t ntri);
/* The same for the next-to-wall nodes whose coordinates lie in the box
 * lo <= x < hi only (one member of a packed ensemble and its own surface).
 * No reference counterpart (the reference holds one vessel). */
lbm_status lbm_set_normals_from_surface_box(lbm_handle* h, const double* tri12, int64_t ntri, const double lo[3],
                                            const double hi[3]);

/* Interpolated bounce-back (physics mode; the reference computes the wall
 * distances, Geometry::CalculateWallDistances, ComplexGeometry.cpp:550-608,
 * but never uses them).  For every missing link of the boundary list, the
 * fraction q in [0, 1] of the link at which it meets the surface (segment-
 * triangle intersection; the reference divides by the spacing instead of
 * the link length, which exceeds 1 on diagonal links) replaces half-way
 * bounce-back by the rule of Bouzidi, Firdaouss and Lallemand (2001):
 *   q < 1/2:  f_q(x) = 2q f*_i(x) + (1 - 2q) f*_i(x + c_q)
 *   q >= 1/2: f_q(x) = f*_i(x) / (2q) + (1 - 1/(2q)) f*_q(x)
 * (i = opp q, the link x -> x + c_i crossing the wall; a link without a
 * triangle, or with q < 1/2 and no fluid node at x + c_q, keeps half-way
 * bounce-back).  ntri == 0 returns to half-way bounce-back. */
lbm_status lbm_set_wall_distances(lbm_handle* h, const double* tri12, int64_t ntri);
/* Boundary-list points (pt[nsp], may be NULL) and their wall distances
 * q[nsp * Q] (entry-major; 0.5 where no link is missing or none is set). */
lbm_status lbm_get_wall_distances(lbm_handle* h, int64_t* pt, float* q);
/* Inlet amplitude per step: step s uses amp[s % n] (times the node's
 * profile factor and the spec's value).  Replaces InletVelocity_ =
 * getInletVelocity(t, 0.9) (Simulation.cpp:580). */
lbm_status lbm_set_inlet_table(lbm_handle* h, const double* amp, int64_t n);
/* Waveform `wave` (0 <= wave < LBM_MAX_WAVES; 0 is the inlet table above):
 * a velocity rule with this wave uses amp[s % n] at step s.  No reference
 * counterpart (the reference has one inlet waveform). */
lbm_status lbm_set_waveform(lbm_handle* h, int wave, const double* amp, int64_t n);

/* f = w_i, accumulators cleared, step counter 0 (Node.cpp:30-37,
 * Simulation.cpp:32-38). */
lbm_status lbm_init_equilibrium(lbm_handle* h);
/* f = f_eq(rho, u) + regularised non-equilibrium part (regularized != 0) or
 * f_eq only; rho and u (3 per node) per active node, FP32. */
lbm_status lbm_init_from_macro(lbm_handle* h, const float* rho, const float* u, int regularized);
/* The same from DEVICE arrays (nact and 3 * nact floats) written on
 * `stream` (a cudaStream_t, NULL = the default stream): the handle's stream
 * waits for `stream`, then builds the state; returns when it is built. */
lbm_status lbm_init_from_macro_device(lbm_handle* h, const float* rho, const float* u, int regularized,
                                      void* stream);

/* Advance nsteps full reference steps: collide, stream, inlet, outlets,
 * wall rule, wall shear stress, OSI/TAWSS (Simulation.cpp:577-586). */
lbm_status lbm_step(lbm_handle* h, int nsteps);
/* Same, without waiting: the launches are queued on the handle's stream and
 * the call returns; lbm_check_status (or any read-out) reports divergence. */
lbm_status lbm_step_async(lbm_handle* h, int nsteps);
/* Wait for the handle's stream and report LBM_ERR_NONFINITE if any density
 * became NaN/Inf since the last start. */
lbm_status lbm_check_status(lbm_handle* h);
lbm_status lbm_sync(lbm_handle* h);

typedef struct {
    int64_t points;   /* nx*ny*nz */
    int64_t active;   /* non-solid nodes */
    int64_t fluid;    /* interior fluid nodes */
    int64_t wall;     /* wall boundary nodes */
    int64_t bc[LBM_MAX_BC]; /* nodes per boundary condition */
    int64_t next_to_wall;
    int64_t special;  /* boundary + next-to-wall nodes (the boundary list) */
    int64_t segments; /* pull segments (stretches of active nodes sharing neighbour offsets) */
    int64_t steps;    /* steps taken */
    int64_t device_bytes; /* device memory held by the handle */
} lbm_counts;

lbm_status lbm_get_counts(lbm_handle* h, lbm_counts* out);
/* Per lattice point: 0 solid, 1 fluid, 2 wall, 3+b boundary condition b;
 * bit 7 set on next-to-wall nodes. */
lbm_status lbm_get_classes(lbm_handle* h, uint8_t* cls);

/* Post-boundary distributions of every active node, [a*Q + q] (the
 * reference's m_distributions after the last step). */
lbm_status lbm_get_distributions(lbm_handle* h, double* f);
lbm_status lbm_set_distributions(lbm_handle* h, const double* f);
/* rho and u of the post-boundary distributions per active node
 * (Collision's moment formulas, Simulation.cpp:52-175). */
lbm_status lbm_get_macro(lbm_handle* h, double* rho, double* u3);
/* Next-to-wall nodes in increasing n (Simulation.cpp:880-905). Any pointer
 * may be NULL. */
lbm_status lbm_get_wss(lbm_handle* h, int64_t* pt, double* normal3, double* wss, double* acc3,
                       double* acc_mag, double* osi, double* tawss);
/* Surface read-out (the reference's commented-out design,
 * OutputFile.cpp:431-488, FindClosestLatticePoint /
 * InterpolateAttributesToSTLVertices): for each of nv points xyz (physical
 * coordinates, 3 per point, e.g. STL vertices) the index into lbm_get_wss's
 * arrays of the nearest next-to-wall node (the nodes that carry WSS, OSI
 * and TAWSS here; the reference searched its wall-node list, whose WSS it
 * never sets), by Euclidean distance between lattice point coordinates,
 * ties to the lower index; -1 when none lies within max_radius lattice
 * spacings.  distance (may be NULL) receives the physical distance. */
lbm_status lbm_nearest_next_to_wall(lbm_handle* h, const double* xyz, int64_t nv, int max_radius, int64_t* nw_index,
                                    double* distance);
/* The same read-outs without waiting: the read-out launches are queued on
 * the handle's stream behind the steps already queued, and the copies into
 * the caller's buffers run on a second stream while later steps proceed
 * (pinned buffers, e.g. cudaHostAlloc, make the copies truly asynchronous).
 * The buffers hold the results once lbm_wait_outputs returns; a later
 * read-out of the same kind waits on the device for the earlier copies.
 * No reference counterpart (its output blocks the time loop). */
lbm_status lbm_get_macro_async(lbm_handle* h, double* rho, double* u3);
lbm_status lbm_get_wss_async(lbm_handle* h, int64_t* pt, double* normal3, double* wss, double* acc3,
                             double* acc_mag, double* osi, double* tawss);
lbm_status lbm_wait_outputs(lbm_handle* h);
/* FP64 sums over the post-boundary distributions: total mass, momentum, and
 * per boundary condition the momentum along its face axis (flux). */
lbm_status lbm_get_conservation(lbm_handle* h, double* mass, double* mom3, double* flux);

/* Checkpoint (versioned binary: header, distributions, accumulators). */
lbm_status lbm_save(lbm_handle* h, const char* path);
lbm_status lbm_load(lbm_handle* h, const char* path);

/* The handle's CUDA stream (cudaStream_t) for event timing by the caller. */
lbm_status lbm_get_stream(lbm_handle* h, void** stream);
/* Number of this library's kernels launched so far by the handle. */
lbm_status lbm_get_launch_count(lbm_handle* h, int64_t* launches);
/* Steps per captured CUDA graph (0 = launch kernels directly). */
lbm_status lbm_set_graph_steps(lbm_handle* h, int steps_per_graph);
/* Persistent stepping: each launch of the step kernel runs steps_per_launch
 * (even, >= 2) steps, one cooperative grid of at most as many blocks as fit
 * on the GPU at once, threads walking the active nodes with a grid stride
 * and a grid barrier between steps (0 = one launch per step, the default).
 * Results are bit-identical to one launch per step.  With graph steps set,
 * steps_per_graph must be a multiple of steps_per_launch and the graph
 * replays steps_per_graph / steps_per_launch persistent launches.  For
 * lattices whose step is shorter than a launch (single small vessels,
 * ensembles of small vessels); lattices beyond 32-bit population offsets
 * (Q * stride >= 2^31) are refused (LBM_ERR_UNSUPPORTED) at the next step.
 * Each barrier wait is bounded (~0.25 s): a wait that gives up ends the
 * launch and the next lbm_step / lbm_check_status returns LBM_ERR_CUDA.
 * New interface: the reference has one host loop iteration per step
 * (Simulation.cpp:575-599). */
lbm_status lbm_set_persistent(lbm_handle* h, int steps_per_launch);
/* Testing the bounded barrier: extra arrivals every barrier of the next
 * persistent launches waits for (0 in normal use).  A count far above any
 * grid size (e.g. 0x40000000) makes the next persistent launch's first
 * barrier unreachable: every block's wait gives up (well under a second),
 * the launch ends, and the next lbm_step / lbm_check_status returns
 * LBM_ERR_CUDA and clears the barrier; the state is then undefined until the
 * next lbm_init_*. */
lbm_status lbm_preset_barrier(lbm_handle* h, unsigned extra_arrivals);
/* Testing the error path of the step kernels' flags: sets the handle's flag
 * word as a kernel would raise it, so that the next lbm_step /
 * lbm_check_status reports it (and clears LBM_FLAG_BOUNDS).
 * LBM_FLAG_BOUNDS is raised for real only by the bounds-checked build
 * (pv_dec_original_gb300.build with checked=True, compiled with
 * -DLBM_CHECK), whose step kernels test every population, pull-row and
 * boundary-list index against its array and skip an access outside it.  No
 * reference counterpart (the reference has no error checks). */
#define LBM_FLAG_NONFINITE 1
#define LBM_FLAG_BOUNDS 4
lbm_status lbm_preset_flags(lbm_handle* h, unsigned flags);

/* Launch-shape variants of the step kernel: one node per thread with
 * (block size, minimum resident blocks per SM) = (128,12) (128,10) (128,8)
 * (256,3) (256,1); variant 5, the tiled kernel (bulk copies stage each
 * 256-node tile's sources in shared memory; physics mode, FP32 / FP16 /
 * BF16; elsewhere it runs variant 0, or 4 for FP64); variants 6 (128,10)
 * and 7 (128,12), the compact kernel (32 bytes of node metadata per warp of
 * 32 nodes instead of 12 bytes a node; physics mode, FP32 / FP16 / BF16,
 * half-way bounce-back; elsewhere variant 0).  A new handle starts on
 * variant 0, FP64 on variant 4.  lbm_autotune times each variant for
 * trial_steps steps on a snapshot of the current state, restores the
 * state, keeps the fastest and reports it (and, if ms_per_step is not NULL,
 * the time of every variant: LBM_NUM_VARIANTS floats).  No reference
 * counterpart (the reference has a single serial loop). */
#define LBM_NUM_VARIANTS 8
lbm_status lbm_autotune(lbm_handle* h, int trial_steps, int* best, float* ms_per_step);
lbm_status lbm_set_variant(lbm_handle* h, int variant);

/* ---------------------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (code running during CUDA graph capture, real-time loops with
 * memory fixed up-front, frameworks whose pool allocator owns the device):
 * FP64 sums over caller-owned device memory with no allocation at all.
 *   d_f:   device array of nact*Q doubles, distributions per node [a*Q + q]
 *   d_out: device array of 4 doubles <- mass, momentum x, y, z
 * Runs on `stream` (a cudaStream_t, NULL = default stream) and returns
 * without waiting.  The per-block scratch is a fixed 512 KiB device array
 * inside the library (held by every GPU that loads it until exit), so nact
 * is limited to 4,194,304; larger inputs get LBM_ERR_ARG.  The first call on
 * a device looks the array up with that device current: make it before any
 * stream capture; a device reset between calls is not supported (the
 * looked-up address is kept for the process).  All calls share the array:
 * calls that overlap on the GPU race; serialise them.  A CUDA error left
 * pending by earlier work is returned as LBM_ERR_CUDA, named as earlier,
 * with nothing launched.  Errors: lbm_last_global_error(). */
lbm_status lbm_moment_sums_noalloc(const double* d_f, int64_t nact, int Q, double* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
