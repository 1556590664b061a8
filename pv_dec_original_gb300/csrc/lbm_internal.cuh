// Internal device structures shared by the library's translation units.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "lbm_lattice.cuh"
#include "../../include/lbm_gb300.h"

namespace lbm {

// Class byte per lattice point.
enum : uint8_t { CLS_SOLID = 0, CLS_FLUID = 1, CLS_WALL = 2, CLS_BC0 = 3, CLS_NW_BIT = 0x80, CLS_MASK = 0x7f };

// Error flags raised by kernels (polled by the host after each batch).
// FLAG_BOUNDS is raised only by the bounds-checked build (LBM_CHECK), whose
// step kernels test every index against its array before the access and
// skip the access when it falls outside.
enum : unsigned { FLAG_NONFINITE = 1u, FLAG_EXACT_ZERO = 2u, FLAG_BOUNDS = 4u, FLAG_TIMEOUT = 8u };

#ifdef LBM_CHECK
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

// Bounds-checked build: true when 0 <= i < n; otherwise raises FLAG_BOUNDS
// and the caller skips the access.  Compiles to `true` elsewhere.
__device__ __forceinline__ bool in_bounds(int64_t i, int64_t n, unsigned* flags) {
    if constexpr (!kChecked) {
        return true;
    } else {
        if (i >= 0 && i < n) return true;
        atomicOr(flags, FLAG_BOUNDS);
        return false;
    }
}

// Tiled step: tiles of kTileNodes consecutive active nodes whose sources
// are staged in shared memory by bulk copies.  Per-tile plan (int32):
// [0, Q) source-window start per population plane (element index, 16-byte
// aligned), [Q, 2Q) window length (elements, a multiple of 16 bytes), then
// the tile's first pull segment, its segment count (capped at segcap), the
// start of its next-to-wall entries (a multiple of 4) and their count (a
// multiple of 4).
constexpr int kTileNodes = 256;
constexpr int kTilePlanExtra = 4;

// Shared-memory layout of one pipeline stage (byte offsets) and the caps
// the plan guarantees.
struct TileGeom {
    int64_t ntiles;      // 0: no plan (the tiled variant falls back)
    int wcap;            // elements per plane of a source window
    int segcap;          // delta rows per tile
    int nwcap;           // next-to-wall entries per tile (per normal plane)
    int nstage;          // pipeline depth (2 or 3)
    int ctas_per_sm;
    int stage_bytes, smem_bytes;
    int off_pull, off_own, off_word, off_sp, off_delta, off_nrm, off_hdr;
};

struct BCDev {
    int kind;
    int face;
    double value;
    int profile;
    double c1, c2, R;
    int wave;        // inlet waveform of a velocity rule
    float value_m1;  // pressure rules: value - 1 (density offset) for the FP32-arithmetic formats
};

// Everything one stream-collide launch needs (passed by value).
struct StepParams {
    const void* fin;
    void* fout;
    int64_t stride;            // elements per population plane (active nodes, padded)
    const int32_t* seg_delta;  // per pull segment, Q source offsets in active-index space (rows of kDeltaRow<Q>)
    // compact step kernel (physics, FP32-arithmetic formats, 32-bit offsets):
    // per pull segment the Q offsets q * stride + delta_q from the node's own
    // entry of plane 0 (rows of kDeltaRow<Q>), and per warp of 32
    // consecutive active nodes kWarpBlockWords words of lane masks and first
    // boundary-list entries (step_kernels.cuh); null where not built
    const int32_t* seg_abs;
    const uint32_t* warp_block;
    int64_t nseg;              // pull segments (rows of seg_delta / seg_abs)
    // one thread per active node; packed word layout in step_kernels.cuh
    int64_t nact;
    const uint64_t* act_word;
    const int32_t* sp_of_act;  // boundary-list entry of an active node (or -1)
    // boundary list ("special": boundary + next-to-wall nodes)
    int64_t nsp;
    const uint32_t* sp_miss;  // bit q: lattice point x + c_q is not active
    const uint8_t* sp_cls;
    const int32_t* sp_nw;     // next-to-wall index or -1
    const double* sp_prof;    // inlet profile factor
    const int32_t* sp_bc;     // boundary-condition rule of a boundary-list entry (-1: none)
    double* sp_flux;          // read-out: momentum along the rule's face axis, per entry
    const float* sp_q;        // physics: wall distance of each missing link, [Q][nsp] (null: half-way bounce-back)
    void* stale;              // parity: previous post-boundary f, [q][nsp] in the arithmetic type
    // next-to-wall accumulators
    int64_t nnw;
    const double* nw_n;       // [3][nnw]
    double* nw_wss;
    double* nw_acc;           // [3][nnw]
    double* nw_accm;
    // FP32-arithmetic formats keep their next-to-wall data in FP32 (GB300's
    // FP64 rate is a small fraction of FP32): normals, a ring of the last
    // kRingSlots steps' stresses (one 16-byte store per node and step), and
    // compensated two-float accumulators (hi, lo) of tau_x, tau_y, tau_z,
    // |tau|.  The ring has two halves of kFoldEvery slots: while a step whose
    // index is a multiple of kFoldEvery writes one half, the first
    // fold_blocks blocks of its launch fold the other (the previous
    // kFoldEvery steps, in step order) into the accumulators
    const float* nw_nf;       // [3][nw_stride]
    int64_t nw_stride;        // plane stride of nw_nf (nnw + 1 rounded up to 4)
    float* nw_ring;           // float4 [kRingSlots][nnw]: step s in slot s % kRingSlots
    int64_t fold_blocks;      // leading blocks of a step launch that fold the ring (set by the launcher)
    int pdl_early;            // step launch: let the next launch begin at block start (else at block end)
    float2* nw_accf;          // [4][nnw]
    void* nw_prev;            // parity: rho, ux, uy, uz of the previous collision, [4][nnw]
    double tau;
    int collision;             // LBM_COLLISION_* (physics mode)
    double wss_C;
    // scalars derived on the host: FP64 arithmetic is slow on GB300, so no
    // thread recomputes them
    double inv_tau;            // 1/tau (the reference's (1.0 / m_relaxation))
    float inv_tau_f;
    float wss_C_f;             // C in FP32 (parity stress)
    float wss_phys_f;          // -(1 - 1/(2 tau)) C in FP32 (physics stress)
    double wss_phys;           // the same in FP64
    // inlet waveforms, concatenated: waveform w holds wave_len[w] entries
    // from amp + wave_off[w]; step index = *step_base + step_off
    const double* amp;
    const int64_t* wave_off;
    const int64_t* wave_len;
    const int64_t* step_base;  // step counter slot read by this launch
    int64_t* step_next;        // the other slot: written with *step_base + 1
    int step_off;
    int direct;                // read-out of the initial state: no pull, no boundary rules
    const int32_t* tile_plan;  // per tile: 2 Q + kTilePlanExtra int32
    TileGeom tile;
    const BCDev* bct;  // boundary-condition rules (device table)
    int nbc;
    unsigned* flags;
    // readout (materialize) outputs
    double* out_f;            // [a*Q + q] FP64, or null
    double* out_rho;          // rho per node (FP64 moments of the full f), or null
    double* out_u;            // u per node, 3 per node, or null
    const int32_t* act_idx;   // per point active index (readout only)
    double* partials;         // per block: mass - nact, mom3
};

constexpr int kPartialStride = 4;
constexpr int kStepThreads = 256;

// Launchers (one per translation unit family).  kind: 0 step, 1 prologue
// (collide the initial state), 2 materialize (post-boundary f + sums).
constexpr int kRingSlots = 32;  // FP32 stress ring: two halves of kFoldEvery steps
constexpr int kFoldEvery = 16;  // steps between folds of the FP32 stress ring
constexpr int kNumVariants = LBM_NUM_VARIANTS;  // launch-shape variants of the step kernel (step_kernels.cuh)
cudaError_t launch_step_f64(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t s);
cudaError_t launch_step_f32(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t s);
cudaError_t launch_step_f16(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t s);
cudaError_t launch_step_bf16(int Q, int mode, int kind, int variant, const StepParams& p, cudaStream_t s);
// Persistent launch of nsteps steps (even / odd step parameters, grid
// barrier word bar[2], zero between launches; nsteps = 0: the kernel's
// occupancy query only); 32-bit population offsets.
cudaError_t launch_multi_f64(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                             unsigned* bar, cudaStream_t s);
cudaError_t launch_multi_f32(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                             unsigned* bar, cudaStream_t s);
cudaError_t launch_multi_f16(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                             unsigned* bar, cudaStream_t s);
cudaError_t launch_multi_bf16(int Q, int mode, const StepParams& even, const StepParams& odd, int nsteps,
                              unsigned* bar, cudaStream_t s);

// Warp blocks of the compact step kernel (built by step_fast.cu): words of
// lane masks and first entries per warp of 32 active nodes, and the number
// of warps covered (whole blocks of 256 nodes plus one, zero past the last
// node).
constexpr int kWarpBlockWords = 8;
inline int64_t block_warps(int64_t nact) { return (nact + 255) / 256 * 8 + 8; }
cudaError_t build_compact_meta(int Q, const uint64_t* act_word, const int32_t* sp_of_act, int64_t nact, int64_t nnw,
                               const int32_t* seg_delta, int64_t nseg, int64_t stride, uint32_t* warp_block,
                               int32_t* seg_abs, cudaStream_t s);

// State initialisation: what = 0 fills f = w on every active node, what = 1
// stores fa[a*Q + q] (FP64, per active node) into the planes.
cudaError_t init_state(int precision, int Q, int what, void* f, int64_t stride, const double* fa, int64_t nact,
                       cudaStream_t s);
cudaError_t init_state_f64(int Q, int what, void* f, int64_t stride, const double* fa, int64_t nact, cudaStream_t s);
cudaError_t init_state_fast(int precision, int Q, int what, void* f, int64_t stride, const double* fa, int64_t nact,
                            cudaStream_t s);

// Read-out helpers (step_f64.cu): ordered FP64 sum of per-block partials;
// next-to-wall outputs [wss | normal n x 3 | acc n x 3 | acc_mag | osi | tawss].
cudaError_t wss_outputs(const double* w, const double* a, const double* am, const double* nrm, int64_t n,
                        double tawss_div, double* out, cudaStream_t st);
cudaError_t reduce_partials(const double* partials, int64_t nblocks, double* out, cudaStream_t s);
// Warm start: f = f_eq(rho, u) (+ regularised non-equilibrium part from
// finite-difference velocity gradients), FP64 per active node.
cudaError_t warm_start_f(int Q, const float* rho, const float* u, const int32_t* act_idx, const int64_t* act_pt,
                         int64_t nact, int nx, int ny, int nz, double tau, int regularized, double* fa,
                         cudaStream_t s);

// Voxelizer (voxelize.cu).
struct VoxResult {
    int64_t fluid;
    int64_t tests;
};
cudaError_t voxelize_device(const double* d_tri, int64_t ntri, const double bbox[6], const double origin[3],
                            double spacing, const int dims[3], uint8_t* d_mask, VoxResult* res, cudaStream_t s,
                            std::string* err);

// Exclusive scan of int64 counts (scan.cu); returns the total.
cudaError_t exclusive_scan_i64(const int64_t* d_in, int64_t* d_out, int64_t n, int64_t* total, cudaStream_t s);

// Normals: for each listed point, the area / distance^2 weighted surface
// normal (Subdomain.cpp:224-370).  out is [3][npts].
cudaError_t surface_normals(const double* d_tri, int64_t ntri, const int64_t* d_pts, int64_t npts, int nx, int ny,
                            const double origin[3], double spacing, double* d_out, cudaStream_t s);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Entries per pull-segment row of the delta table: Q offsets padded to a
// multiple of 4 (one 16-byte load per 4 offsets).
template <int Q>
constexpr int kDeltaRow = (Q + 3) / 4 * 4;

// Next-to-wall read-out of the FP32 formats into doubles [5][nnw]: |tau| of
// step `last` (ring slot; -1: none, wss_ckpt: restored values), then the
// accumulators of tau_x, tau_y, tau_z, |tau| plus ring slots 0 .. pending-1.
cudaError_t nw_readout_f32(const float2* accf, const float* ring, int64_t nnw, int first, int pending, int last,
                           const float* wss_ckpt, double* out, cudaStream_t st);

// 3x3x3 convolutions of the warm-start network on tcgen05 tensor cores
// (conv_tc.cu): the shapes they take (channels 16 / 32 / 64; input grid D x
// H x W with, at stride 1, D % 4, H % 16, W % 8 == 0, at stride 2 even
// dimensions and H / 2 % 16, W / 2 % 8 == 0), the forward convolution, the
// flipped-transposed weights that turn a stride-1 input gradient into a
// forward convolution, and the flag of a bounded wait that gave up (read
// and cleared).
bool conv3_tc_applies(int D, int H, int W, int ci, int co, int stride);
cudaError_t conv3_tc(const void* x, int D, int H, int W, int ci, const void* w, const float* bias, int co, int relu,
                     void* y, float* y32, int stride, cudaStream_t st);
cudaError_t conv3_flip_transpose(const void* w, void* wt, int co, int ci, cudaStream_t st);
// Weight gradient dw += dL/dw of a 3x3x3 convolution (stride 1 or 2) on
// tcgen05, for output grids whose x extent is a multiple of 16.
bool conv3_wgrad_tc_applies(int D, int H, int W, int ci, int co, int stride);
cudaError_t conv3_wgrad_tc(const void* x, int D, int H, int W, int ci, const void* dy, int co, int stride, float* dw,
                           cudaStream_t st);
cudaError_t conv_tc_status(unsigned* flags);

// Message returned by lbm_last_global_error() (capi.cu).
void set_last_global_error(const char* msg);

}  // namespace lbm
