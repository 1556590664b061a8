/*
 * CPU restatement of the reference's hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This oracle is the checker for the CUDA library: tests, the smoke check and
 * the CPU-baseline leg of the benchmark call it; the product never does.
 * Every function follows the reference's arithmetic in its operation order
 * (build with -ffp-contract=off) and cites the reference lines it restates.
 * It is pinned bit-for-bit against the reference's own sources compiled
 * unchanged (oracle/Makefile target `ref`) through golden vectors.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- lattice tables (LatticeModel.cpp:51-151 D3Q19, :208-334 D3Q27) ---- */
int oracle_lattice(int Q, int* c /*Q*3*/, double* w /*Q*/, int* opp /*Q*/);

/* ---- geometry ---- */
/* Bounding box (min_x,max_x,min_y,max_y,min_z,max_z) and lattice size by the
 * reference rule, quirks included (ComplexGeometry.cpp:145-165). */
void oracle_bbox_dims(const double* tri12, int64_t ntri, double spacing, double* bbox6, int* dims3);

/* +z ray-parity voxelization (ComplexGeometry.cpp:978-1053 with :853-884,
 * :803-848, :620-674).  mask[(k*ny+j)*nx+i] = 1 (Fluid) / 0 (NotFluid).
 * origin3/dims3 give the lattice (the reference: origin = bbox min); the ray
 * adjustment compares against bbox6.  culled=0 tests every triangle for
 * every point exactly as the reference; culled=1 skips triangles whose
 * (margin-widened) xy extent misses the column -- same answers, used to pin
 * the device binning at sizes the brute force cannot reach. */
int64_t oracle_voxelize(const double* tri12, int64_t ntri, const double* bbox6, const double* origin3,
                        double spacing, const int* dims3, uint8_t* mask, int culled, int nthreads);

/* Conservative xy margin of one triangle for column culling (<0: the
 * triangle can never pass isPointInsideTriangle; >1e29: never cull). */
double oracle_cull_margin(const double* tri12_row, double zspan);

/* Boundary points: Fluid points with a lattice neighbour that is NotFluid or
 * outside the box (ComplexGeometry.cpp:1259-1300).  out[n] = 1 for boundary. */
int64_t oracle_find_boundary(const uint8_t* mask, const int* dims3, int Q, uint8_t* out);

/* ---- solver ---- */
enum { ORC_PARITY = 0, ORC_PHYSICS = 1 };
enum { ORC_BC_REF_INLET = 1, ORC_BC_REF_OUTLET_YMAX = 2, ORC_BC_REF_OUTLET_ZMIN = 3,
       ORC_BC_VELOCITY = 4, ORC_BC_PRESSURE = 5 };

typedef struct {
    int kind;        /* ORC_BC_* */
    int face;        /* 0 x-min, 1 x-max, 2 y-min, 3 y-max, 4 z-min, 5 z-max */
    double value;    /* density for pressure faces; velocity scale for velocity faces */
    int profile;     /* 0 uniform, 1 parabolic 1 - (d1^2+d2^2)/R^2 on the two transverse axes */
    double c1, c2, R;
} oracle_bc;

typedef struct oracle_sim oracle_sim;

/* cls[n] per lattice point: 0 solid, 1 fluid, 2 wall, 3+b boundary of bc[b]. */
oracle_sim* oracle_sim_create(int Q, int mode, const int* dims3, const uint8_t* cls,
                              const double* origin3, double spacing, double tau,
                              const oracle_bc* bc, int nbc);
void oracle_sim_destroy(oracle_sim* s);
/* Per-step inlet amplitude table (step s uses amp[s % n]). */
void oracle_sim_set_amplitude(oracle_sim* s, const double* amp, int64_t n);
/* WSS scale C (reference: 1060*dt^2/(spacing^2*1e-6), Simulation.cpp:880-881)
 * and the TAWSS divisor (reference: Pulsatile period 0.9, Simulation.cpp:901). */
void oracle_sim_set_wss(oracle_sim* s, double C, double tawss_div);
/* Wall and next-to-wall normals from the surface (Subdomain.cpp:224-370). */
void oracle_sim_compute_normals(oracle_sim* s, const double* tri12, int64_t ntri, int nthreads);
void oracle_sim_step(oracle_sim* s, int nsteps, int nthreads);
/* Physics mode: regularized collision (1) instead of BGK (0, default). */
void oracle_sim_set_collision(oracle_sim* s, int regularized);
/* physics mode: interpolated bounce-back with wall distances from the
 * triangles (ntri = 0: half-way); distances per (active node, arriving q) */
void oracle_sim_set_wall_distances(oracle_sim* s, const double* tri12, int64_t ntri);
void oracle_sim_get_wall_distances(const oracle_sim* s, float* q);

int64_t oracle_sim_nactive(const oracle_sim* s);
int64_t oracle_sim_nnw(const oracle_sim* s);
/* Active points in increasing linear index; f/fnew/feq as [a*Q+q]. */
void oracle_sim_get_active(const oracle_sim* s, int64_t* pt, uint8_t* cls);
void oracle_sim_get_f(const oracle_sim* s, double* f, double* fnew, double* feq);
void oracle_sim_set_f(oracle_sim* s, const double* f);
void oracle_sim_get_macro(const oracle_sim* s, double* rho, double* u3);
/* Next-to-wall nodes in increasing linear index. */
void oracle_sim_get_nw(const oracle_sim* s, int64_t* pt, double* normal3, double* wss, double* acc3,
                       double* acc_mag, double* osi, double* tawss);
void oracle_sim_get_wall_normals(const oracle_sim* s, int64_t* pt, double* normal3);
/* FP64 conservation sums of the current post-boundary distributions:
 * mass, momentum[3], and per boundary condition the momentum along its face axis. */
void oracle_sim_conservation(const oracle_sim* s, double* mass, double* mom3, double* flux /*nbc*/);

#ifdef __cplusplus
}
#endif
#endif
