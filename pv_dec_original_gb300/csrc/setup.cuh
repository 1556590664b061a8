// Device geometry lists built by setup.cu.
#pragma once
#include <string>
#include "lbm_internal.cuh"

namespace lbm {

struct ProfileSpec {
    int n;
    double s;
    double org[3];
    int profile[LBM_MAX_BC];
    int axis[LBM_MAX_BC];
    double c1[LBM_MAX_BC], c2[LBM_MAX_BC], R[LBM_MAX_BC];
};

struct GeometryLists {
    int64_t npts = 0;
    uint8_t* cls = nullptr;      // per point
    int64_t nsp = 0;             // boundary + next-to-wall nodes; next-to-wall first (entry s < nnw is
                                 // next-to-wall node s)
    int64_t* sp_pt = nullptr;
    uint32_t* sp_miss = nullptr;
    uint8_t* sp_cls = nullptr;
    int32_t* sp_nw = nullptr;
    int32_t* sp_bc = nullptr;    // boundary-condition rule of the entry, or -1
    int16_t* bcidx = nullptr;    // per point: boundary-condition rule (valid where cls >= CLS_BC0)
    double* sp_prof = nullptr;
    int64_t nnw = 0;
    int64_t* nw_pt = nullptr;
    int64_t nact = 0;
    uint64_t* act_word = nullptr;  // per active node: packed word (see step_kernels.cuh)
    int32_t* sp_of_act = nullptr;  // per active node: boundary-list entry or -1
    int32_t* act_idx = nullptr;  // per point
    int64_t* act_pt = nullptr;
    int plane[LBM_MAX_BC] = {0};
};

// d_seg_of_act: per active node, its pull segment (see capi.cu build_segments).
cudaError_t build_geometry(int Q, const uint8_t* d_mask, int nx, int ny, int nz, const lbm_bc_spec* bc, int nbc,
                           const double origin[3], double spacing, const int32_t* d_seg_of_act, GeometryLists& out,
                           cudaStream_t st, std::string& err);

// Nearest next-to-wall node (index into the next-to-wall list, -1 if none
// within rmax lattice spacings) and its distance of each of nv points xyz
// (physical coordinates, 3 per point).
cudaError_t nearest_next_to_wall(const double* d_xyz, int64_t nv, const GeometryLists& g, int nx, int ny, int nz,
                                 const double origin[3], double spacing, int rmax, int64_t* d_idx, double* d_dist,
                                 cudaStream_t st);

// Wall distances of the boundary list's missing links (interpolated
// bounce-back): d_q [Q][nsp], see k_wall_q.
cudaError_t wall_distances(int Q, const double* d_tri, int64_t ntri, const GeometryLists& g, int nx, int ny,
                           const double origin[3], double spacing, float* d_q, cudaStream_t st);

}  // namespace lbm
